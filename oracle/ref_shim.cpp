// ref_shim.cpp -- extern "C" entry points over the reference's own code,
// compiled for the host from the reference sources where they lie
// (oracle/build.py).  TEST INFRASTRUCTURE ONLY: it lets the tests compare
// the C restatement in fim_oracle.c, and the product's I/O, with the
// reference's code on the same inputs.  Nothing here is product code.
//
// The reference's solver functions are CUDA __device__ functions
// (src/eikonal/cuda_fim.h:1256-1411); the host compiler treats the CUDA
// execution-space annotations as ignored attributes, so they compile as host
// functions unchanged.
#include "src/eikonal/cuda_fim.h"
#include "src/io/vtk.h"
#include "src/io/io_json.h"

#include <cstring>
#include <cstdint>

using namespace tw;

extern "C" {

double ref_solve_tri(double e12, double e13, double e23, double p1, double p2)
{
  return solve_tri_cu(e12, e13, e23, p1, p2);
}

double ref_solve_tet(double e13, double e23, double e34, double e12, double e14, double e24,
                     double p1, double p2, double p3)
{
  return solve_tet_cu(e13, e23, e34, e12, e14, e24, p1, p2, p3);
}

// The constant gray-code tables (cuda_fim.h:41-48) as the host sees them.
void ref_gray_tables(int64_t *adf, int64_t *bce, int64_t *phi)
{
  for (int i = 0; i < 12; ++i) {
    adf[i] = d_gray_mappings.adf[i];
    bce[i] = d_gray_mappings.bce[i];
    phi[i] = d_gray_mappings.phi[i];
  }
}

// update_per_element on a one-tet submesh with slots 0..3 = vertices 0..3.
// state[s] and phi[s] are the slot states/times; t is the target slot.
double ref_update_corner(const double *geo6, int t, const int32_t *state, const double *phi,
                         double phi_start, double front_width)
{
  cnt_t e2n_cnt[1] = {4};
  idx_t e2n_dsp[1] = {0};
  idx_t e2n_con[4] = {0, 1, 2, 3};
  dbl_t geo[6];
  for (int k = 0; k < 6; ++k) geo[k] = geo6[k];
  smsh_t m;
  std::memset(&m, 0, sizeof(m));
  m.Nn = 4; m.Ne = 1; m.Nenc = 4;
  m.e2n_cnt = e2n_cnt; m.e2n_dsp = e2n_dsp; m.e2n_con = e2n_con; m.geo = geo;
  dbl_t ph[4]; int st[4];
  for (int s = 0; s < 4; ++s) { ph[s] = phi[s]; st[s] = state[s]; }
  eksv_t sv;
  sv.nNodes = 4; sv.Nenc = 4; sv.agg_state = ek_far;
  sv.phi_ms = ph; sv.states = st; sv.tmp_state = nullptr; sv.tmp_phi_ms = nullptr;
  return update_per_element(&m, &sv, (idx_t)t, 0, ek_narrow, phi_start, front_width);
}

// Runs the reference preprocessing on a global tet mesh:
// compute_base_connectivity (types.cpp:43-225) on the global mesh, then
// extract_submeshes2 (types.cpp:306-570), which also runs compute_geo per
// submesh with the hard-coded speeds 0.6 and fibre (1,0,0) of load_vtk.
// Outputs per global tet: its vertex ids in the submesh slot order (mapped
// back to global ids) and the six geo values; returns #aggregates.
int ref_extract(int64_t nV, int64_t nT, const double *xyz, const int64_t *tets, const int32_t *atags,
                int64_t *tet_slots, double *geo_out, int32_t *agg_of_tet)
{
  mesh_t mesh;
  mesh.n_points = nV; mesh.n_cells = nT;
  mesh.xyz.assign(xyz, xyz + 3 * nV);
  mesh.e2n_cnt.assign(nT, 4);
  mesh.e2n_dsp.resize(nT);
  mesh.e2n_con.assign(tets, tets + 4 * nT);
  for (int64_t e = 0; e < nT; ++e) mesh.e2n_dsp[e] = 4 * e;
  mesh.etype.assign(nT, Tetra);
  mesh.etags.assign(nT, 1);
  mesh.atags.assign(atags, atags + nT);
  mesh.lon.assign(3 * nT, 0.0);
  for (int64_t e = 0; e < nT; ++e) mesh.lon[3 * e] = 1.0;
  mesh.compute_base_connectivity(false);

  std::vector<mesh_t> subs;
  std::vector<std::vector<idx_t>> l2g, n2a, a2a;
  std::vector<idx_t> g2l;
  std::vector<std::map<idx_t, idx_t>> a2n;
  std::vector<std::map<idx_t, std::vector<idx_t>>> a2i;
  std::vector<std::vector<ipair_t>> n2i;
  const int na = extract_submeshes2(mesh, mesh.atags, subs, l2g, g2l, n2a, a2n, a2a, a2i, n2i);

  // walk each aggregate's tets in the same order extract_submeshes2 did
  std::vector<int64_t> next(na, 0);
  std::map<tag_t, int> tag2a;
  int cnt = 0;
  for (int64_t e = 0; e < nT; ++e) {
    auto it = tag2a.find(atags[e]);
    if (it == tag2a.end()) tag2a[atags[e]] = cnt++;
  }
  for (int64_t e = 0; e < nT; ++e) {
    const int a = tag2a[atags[e]];
    const int64_t k = next[a]++;
    const mesh_t &s = subs[a];
    for (int j = 0; j < 4; ++j) tet_slots[4 * e + j] = l2g[a][s.e2n_con[s.e2n_dsp[k] + j]];
    for (int j = 0; j < 6; ++j) geo_out[6 * e + j] = s.geo[6 * k + j];
    if (agg_of_tet) agg_of_tet[e] = a;
  }
  return na;
}

// load_vtk (src/io/vtk.cpp:11-106).  Two calls: sizes first (xyz == nullptr).
int ref_load_vtk(const char *path, int64_t *nV, int64_t *nT, double *xyz, int64_t *tets, int32_t *etags)
{
  mesh_t mesh;
  load_vtk(path, mesh);
  *nV = (int64_t)(mesh.xyz.size() / 3);
  *nT = (int64_t)mesh.e2n_cnt.size();
  if (xyz) std::memcpy(xyz, mesh.xyz.data(), sizeof(double) * mesh.xyz.size());
  if (tets) for (size_t i = 0; i < mesh.e2n_con.size(); ++i) tets[i] = mesh.e2n_con[i];
  if (etags) for (size_t i = 0; i < mesh.etags.size(); ++i) etags[i] = mesh.etags[i];
  return 0;
}

// save_vtk (src/io/vtk.cpp:109-211) with point data {phi, states}.
int ref_save_vtk(const char *path, int64_t nV, int64_t nT, const double *xyz, const int64_t *tets,
                 const int32_t *etags, const double *phi, const double *states)
{
  mesh_t mesh;
  mesh.xyz.assign(xyz, xyz + 3 * nV);
  mesh.e2n_cnt.assign(nT, 4);
  mesh.e2n_dsp.resize(nT);
  mesh.e2n_con.assign(tets, tets + 4 * nT);
  for (int64_t e = 0; e < nT; ++e) mesh.e2n_dsp[e] = 4 * e;
  mesh.etags.assign(etags, etags + nT);
  std::vector<std::vector<dbl_t>> data;
  std::vector<std::string> names;
  if (phi) { data.emplace_back(phi, phi + nV); names.push_back("phi"); }
  if (states) { data.emplace_back(states, states + nV); names.push_back("states"); }
  save_vtk(path, mesh, data, names, {}, {});
  return 0;
}

// load_options (src/io/io_json.cpp:228-296) + load_plan (:299-317).
// Outputs dt (us), n_steps, the first event's vertices and tstart.
int ref_load_plan(const char *cfg, const char *plan, double *dt, int64_t *n_steps,
                  int64_t *n_events, int64_t *vtx, int64_t *nvtx, double *tstart, double *cv3)
{
  mesh_t mesh;
  ek_data ek(mesh);
  load_options(cfg, ek.opts);
  load_plan(plan, ek);
  *dt = ek.opts.dt;
  *n_steps = (int64_t)ek.opts.n_steps;
  *n_events = (int64_t)ek.events.size();
  int64_t k = 0;
  for (const auto &ev : ek.events)
    for (auto v : ev.vtx) { if (vtx) vtx[k] = v; k++; }
  *nvtx = k;
  if (tstart && !ek.events.empty()) *tstart = ek.events[0].tstart;
  if (cv3 && !ek.rprops.empty()) { cv3[0] = ek.rprops[0].velo.x; cv3[1] = ek.rprops[0].velo.y; cv3[2] = ek.rprops[0].velo.z; }
  return 0;
}

}  // extern "C"
