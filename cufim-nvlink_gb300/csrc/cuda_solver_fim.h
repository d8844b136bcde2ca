// cuda_solver_fim.h -- drop-in replacement of the reference's solver class
// tw::CudaSolverFIM (src/eikonal/cuda_fim.h:1443-1577), built on the C ABI of
// include/fim.h.
//
// The constructor takes the reference's ek_data (src/core/types.h:382-406)
// -- or any type with the same member names -- and stages it on the GPU; the
// reference used to do this in its constructor (src/eikonal/cuda_fim.cu:
// 1218-1501).  solve() keeps the reference's signature and output: it runs
// num_reps solves, writes {phi, states} to the VTK file `file` with the
// reference's writer format, and returns the mean solve time in seconds
// (src/eikonal/cuda_fim.cu:2386-2503).  act_ms / apd_ms are accepted and left
// untouched, as in the reference.
//
// Members read from ek_data: mesh.xyz, mesh.e2n_con (4 ids per tet),
// mesh.atags (submesh tags, may be empty), mesh.etags, mesh.lon (fibre per
// tet), opts.dt, opts.n_steps, events[].{active,tstart,vtx}, rprops[].velo.
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/fim.h"

namespace tw {

struct fim_run_input {
  std::vector<double> xyz;         // 3 per vertex
  std::vector<int64_t> tets;       // 4 per tet, as written to the output file
  std::vector<int32_t> atags;      // submesh tags (empty: one submesh)
  std::vector<int32_t> etags;      // element tags written to the output file
  std::vector<double> fib, cf, ct; // conduction per tet
  std::vector<int64_t> stim;       // stimulated vertices (seeded at time 0)
  double dt = 0.0;
  int64_t n_steps = 1;
  double apd = 3e5;                // hard-coded APD of the reference (us)
  int device = 0;
};

class CudaSolverFIM {
 public:
  template <class EkData>
  explicit CudaSolverFIM(const EkData &ek)
  {
    init(stage(ek));
  }

  // What the constructor stages from ek_data, without touching the GPU.
  template <class EkData>
  static fim_run_input stage(const EkData &ek)
  {
    fim_run_input in;
    const auto &mesh = ek.mesh;
    in.xyz.assign(mesh.xyz.begin(), mesh.xyz.end());
    in.tets.assign(mesh.e2n_con.begin(), mesh.e2n_con.end());
    in.atags.assign(mesh.atags.begin(), mesh.atags.end());
    in.etags.assign(mesh.etags.begin(), mesh.etags.end());
    const size_t nT = in.tets.size() / 4;
    in.fib.assign(3 * nT, 0.0);
    for (size_t e = 0; e < nT; ++e) in.fib[3 * e] = 1.0;
    if (mesh.lon.size() >= 3 * nT) in.fib.assign(mesh.lon.begin(), mesh.lon.begin() + 3 * nT);
    // speeds: the reference hard-codes 0.6 (types.cpp:231); a plan's CVref
    // (read_funcs_from_json) is honoured when present.
    double vf = 0.6, vs = 0.6;
    if (!ek.rprops.empty()) { vf = ek.rprops[0].velo.x; vs = ek.rprops[0].velo.y; }
    in.cf.assign(nT, vf);
    in.ct.assign(nT, vs);
    // update_events_gpu (cuda_fim.cu:632-683) seeds events in order with
    // phi = 0 and stops at the first event that is inactive or starts
    // before time 0.
    for (const auto &ev : ek.events) {
      if (!(ev.tstart >= 0.0 && ev.active)) break;
      for (auto v : ev.vtx) in.stim.push_back((int64_t)v);
    }
    in.dt = ek.opts.dt;
    in.n_steps = (int64_t)ek.opts.n_steps;
    return in;
  }
  ~CudaSolverFIM();
  CudaSolverFIM(const CudaSolverFIM &) = delete;
  CudaSolverFIM &operator=(const CudaSolverFIM &) = delete;

  double solve(std::vector<std::vector<double>> &act_ms, std::vector<std::vector<double>> &apd_ms,
               const std::string file, const int num_reps = 1);
  double operator()(std::vector<std::vector<double>> &act_ms, std::vector<std::vector<double>> &apd_ms,
                    const std::string file, const int num_reps = 1)
  {
    return solve(act_ms, apd_ms, file, num_reps);
  }

  const std::vector<double> &phi() const { return phi_; }
  const std::vector<int32_t> &states() const { return states_; }
  fim_solver *handle() const { return s_; }

 private:
  void init(const fim_run_input &in);
  fim_solver *s_ = nullptr;
  fim_run_input in_;
  std::vector<double> phi_;
  std::vector<int32_t> states_;
};

}  // namespace tw
