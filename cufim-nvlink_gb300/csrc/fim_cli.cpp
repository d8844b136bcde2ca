// fim_cli.cpp -- command line front end with the reference's flags
// (src/main.cpp:170-237): --mesh --part --plan --odir --reps --info --test
// --num_threads, plus --cfg (the reference reads data/default.cfg from the
// working directory, src/main.cpp:95).  Runs the reference's pipeline
// (tw::run, src/main.cpp:84-104): load the VTK mesh and the partition tags,
// sort every tet's vertex ids (compute_base_connectivity, types.cpp:63-67),
// read config + plan, solve with tw::CudaSolverFIM and write the VTK result.
#include "cuda_solver_fim.h"

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include <cuda_runtime.h>

namespace {

// Minimal stand-ins with the member names tw::CudaSolverFIM reads.
struct Velo { double x = 0.6, y = 0.6, z = 0.6; };
struct RegionProp { Velo velo; };
struct Event { int active = 1; double tstart = 0.0; std::vector<int64_t> vtx; };
struct Opts { double dt = 1.0; size_t n_steps = 1; };
struct Mesh {
  std::vector<double> xyz, lon;
  std::vector<int64_t> e2n_con;
  std::vector<int32_t> atags, etags;
};
struct EkData {
  const Mesh &mesh;
  Opts opts;
  std::vector<Event> events;
  std::vector<RegionProp> rprops;
  explicit EkData(const Mesh &m) : mesh(m) {}
};

void fail(const std::string &msg)
{
  throw std::runtime_error(msg);
}

double run(const std::string &mesh_path, const std::string &part_path, const std::string &plan_path,
           const std::string &out_path, const std::string &cfg_path, int reps)
{
  Mesh mesh;
  int64_t nV = 0, nT = 0;
  if (fim_vtk_read(mesh_path.c_str(), &nV, &nT, nullptr, nullptr, nullptr) != FIM_OK) fail(fim_last_error(nullptr));
  mesh.xyz.resize(3 * nV);
  mesh.e2n_con.resize(4 * nT);
  mesh.etags.assign(nT, 0);
  if (fim_vtk_read(mesh_path.c_str(), &nV, &nT, mesh.xyz.data(), mesh.e2n_con.data(), mesh.etags.data()) != FIM_OK)
    fail(fim_last_error(nullptr));
  for (int64_t e = 0; e < nT; ++e) std::sort(mesh.e2n_con.begin() + 4 * e, mesh.e2n_con.begin() + 4 * e + 4);
  mesh.lon.assign(3 * nT, 0.0);  // load_vtk assigns fibre (1,0,0) to every tet (vtk.cpp:99-101)
  for (int64_t e = 0; e < nT; ++e) mesh.lon[3 * e] = 1.0;
  if (!part_path.empty()) {
    int64_t n = 0;
    if (fim_read_tags(part_path.c_str(), &n, nullptr) != FIM_OK) fail(fim_last_error(nullptr));
    if (n != nT) fail("partition file has " + std::to_string(n) + " tags for " + std::to_string(nT) + " tets");
    mesh.atags.resize(n);
    if (fim_read_tags(part_path.c_str(), &n, mesh.atags.data()) != FIM_OK) fail(fim_last_error(nullptr));
  }
  EkData ek(mesh);
  fim_plan_info info{};
  if (fim_load_plan(cfg_path.empty() ? nullptr : cfg_path.c_str(), plan_path.c_str(), &info, nullptr) != FIM_OK)
    fail(fim_last_error(nullptr));
  std::vector<int64_t> stim(info.n_stim_vertices);
  if (fim_load_plan(cfg_path.empty() ? nullptr : cfg_path.c_str(), plan_path.c_str(), &info, stim.data()) != FIM_OK)
    fail(fim_last_error(nullptr));
  ek.opts.dt = info.dt;
  ek.opts.n_steps = (size_t)info.n_steps;
  Event ev;
  ev.tstart = info.tstart;
  ev.vtx = stim;
  if (info.n_events > 0) ek.events.push_back(ev);
  if (info.has_cv) {
    RegionProp rp;
    rp.velo.x = info.cv[0]; rp.velo.y = info.cv[1]; rp.velo.z = info.cv[2];
    ek.rprops.push_back(rp);
  }
  std::vector<std::vector<double>> act, apd;
  tw::CudaSolverFIM solver(ek);
  return solver.solve(act, apd, out_path, reps);
}

void print_info()
{
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) n = 0;
  std::printf("CUDA devices: %d\n", n);
  for (int d = 0; d < n; ++d) {
    cudaDeviceProp p;
    cudaGetDeviceProperties(&p, d);
    std::printf("  %d: %s, sm_%d%d, %d SMs, %.1f GiB, L2 %.1f MiB, smem/block opt-in %zu KiB\n", d, p.name,
                p.major, p.minor, p.multiProcessorCount, p.totalGlobalMem / 1073741824.0, p.l2CacheSize / 1048576.0,
                p.sharedMemPerBlockOptin / 1024);
    for (int e = 0; e < n; ++e) {
      if (e == d) continue;
      int ok = 0;
      cudaDeviceCanAccessPeer(&ok, d, e);
      std::printf("     peer access %d -> %d: %s\n", d, e, ok ? "yes" : "no");
    }
  }
}

void usage()
{
  std::printf("usage: fim_cli --mesh=FILE --part=FILE --plan=FILE --odir=FILE [--reps=N] [--cfg=FILE]\n"
              "       fim_cli --test | --info\n");
}

}  // namespace

int main(int argc, char **argv)
{
  std::map<std::string, std::string> a;
  const std::map<std::string, std::string> alias = {{"-m", "--mesh"}, {"-p", "--part"}, {"-s", "--plan"},
                                                    {"-o", "--odir"}, {"-i", "--info"}, {"-t", "--test"},
                                                    {"-r", "--reps"}, {"-np", "--num_threads"}, {"-h", "--help"}};
  for (int i = 1; i < argc; ++i) {
    std::string k = argv[i], v;
    const size_t eq = k.find('=');
    if (eq != std::string::npos) { v = k.substr(eq + 1); k = k.substr(0, eq); }
    auto al = alias.find(k);
    if (al != alias.end()) k = al->second;
    const bool flag = (k == "--info" || k == "--test" || k == "--help");
    if (!flag && v.empty() && i + 1 < argc) v = argv[++i];
    a[k] = flag ? "1" : v;
  }
  int rc = 0;
  try {
    const int reps = a.count("--reps") ? std::atoi(a["--reps"].c_str()) : 1;
    const std::string cfg = a.count("--cfg") ? a["--cfg"] : "data/default.cfg";
    if (a.count("--help")) usage();
    else if (a.count("--info")) print_info();
    else if (a.count("--test"))
      run("data/ut_mesh/ut_mesh.vtk", "data/ut_mesh/ut_mesh.tags", "data/ut_mesh/ut_mesh.plan.json",
          "data/output/cufim-ut_mesh-out.vtk", cfg, 1);
    else if (reps < 1) std::printf("invalid number of reps!\n");
    else if (a.count("--mesh") && a.count("--part") && a.count("--plan") && a.count("--odir")) {
      const double t = run(a["--mesh"], a["--part"], a["--plan"], a["--odir"], cfg, reps);
      std::printf("Average execution time for %d runs: %f s\n", reps, t);
    } else usage();
  } catch (const std::exception &e) {
    std::fprintf(stderr, "%s\n", e.what());
    rc = 1;
  }
  return rc;
}
