// cuda_solver_fim.cpp -- non-template part of the tw::CudaSolverFIM drop-in.
#include "cuda_solver_fim.h"

#include <chrono>
#include <cstdio>

namespace tw {

static void check(int rc, fim_solver *s, const char *what)
{
  if (rc != FIM_OK) throw std::runtime_error(std::string(what) + ": " + fim_last_error(s));
}

void CudaSolverFIM::init(const fim_run_input &in)
{
  in_ = in;
  fim_opts o;
  fim_default_opts(&o);
  o.device = in.device;
  o.dt = in.dt;
  o.n_steps = (int)(in.n_steps < 1 ? 1 : in.n_steps);
  o.apd = in.apd;
  check(fim_create(&o, &s_), nullptr, "fim_create");
  const int64_t nV = (int64_t)(in.xyz.size() / 3), nT = (int64_t)(in.tets.size() / 4);
  check(fim_set_mesh(s_, nV, in.xyz.data(), nT, in.tets.data(), in.atags.empty() ? nullptr : in.atags.data()),
        s_, "fim_set_mesh");
  check(fim_set_conduction(s_, in.fib.data(), in.cf.data(), in.ct.data()), s_, "fim_set_conduction");
  std::vector<double> t0(in.stim.size(), 0.0);
  check(fim_set_stimuli(s_, (int64_t)in.stim.size(), in.stim.data(), t0.data()), s_, "fim_set_stimuli");
}

CudaSolverFIM::~CudaSolverFIM()
{
  if (s_) fim_destroy(s_);
}

double CudaSolverFIM::solve(std::vector<std::vector<double>> &, std::vector<std::vector<double>> &,
                            const std::string file, const int num_reps)
{
  double sum = 0.0;
  for (int r = 0; r < num_reps; ++r) {
    const auto t0 = std::chrono::steady_clock::now();
    check(fim_solve(s_, nullptr), s_, "fim_solve");
    const double sec = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    sum += sec;
    std::printf("run %2d took %.5f s.\n", r + 1, sec);
  }
  const int64_t nV = (int64_t)(in_.xyz.size() / 3), nT = (int64_t)(in_.tets.size() / 4);
  phi_.assign(nV, 0.0);
  states_.assign(nV, 0);
  check(fim_get_times(s_, phi_.data(), states_.data()), s_, "fim_get_times");
  if (!file.empty()) {
    std::vector<double> sd(states_.begin(), states_.end());
    check(fim_vtk_write(file.c_str(), nV, nT, in_.xyz.data(), in_.tets.data(),
                        in_.etags.empty() ? nullptr : in_.etags.data(), phi_.data(), sd.data()),
          nullptr, "fim_vtk_write");
  }
  return num_reps > 0 ? sum / num_reps : 0.0;
}

}  // namespace tw
