// ref_types_driver.cpp -- the reference's own pipeline (tw::run,
// src/main.cpp:84-104) on the reference's real types and readers, with the
// solver replaced by this repository's drop-in tw::CudaSolverFIM
// (cufim-nvlink_gb300/csrc/cuda_solver_fim.h).  Test infrastructure: built
// by oracle/build.py from the reference's sources where they lie, never
// shipped.
//
//   ref_types_driver stage MESH PART CFG PLAN DUMP   -- stage only: write what
//       the shim extracts from the reference's ek_data to DUMP (no GPU)
//   ref_types_driver solve MESH PART CFG PLAN OUT    -- the full run: solve
//       on the GPU and write the reference's result file OUT
//
// DUMP layout (native endian): int64 nV, nT, n_atags, n_etags, n_stim,
// n_steps; double dt; then xyz[3 nV], tets[4 nT] (int64), atags (int32),
// etags (int32), fib[3 nT], cf[nT], ct[nT] (double), stim (int64).
#include "core/types.h"
#include "io/io_base.h"
#include "io/io_json.h"
#include "io/vtk.h"

#include "cufim-nvlink_gb300/csrc/cuda_solver_fim.h"

#include <cstdio>
#include <exception>
#include <string>

namespace {

template <class T>
void put(std::FILE *f, const T *p, size_t n)
{
  if (n && std::fwrite(p, sizeof(T), n, f) != n) throw std::runtime_error("short write");
}

}  // namespace

int main(int argc, char **argv)
{
  if (argc != 7) {
    std::fprintf(stderr, "usage: %s stage|solve MESH PART CFG PLAN OUT\n", argv[0]);
    return 2;
  }
  const std::string mode = argv[1];
  try {
    // tw::run (src/main.cpp:84-104), with the config path as an argument
    tw::mesh_t mesh;
    tw::load_vtk(argv[2], mesh);
    tw::read_vector_txt(argv[3], mesh.atags);
    mesh.compute_base_connectivity(true);
    tw::ek_data ekdata(mesh);
    tw::load_options(argv[4], ekdata.opts);
    tw::load_plan(argv[5], ekdata);
    if (mode == "stage") {
      const tw::fim_run_input in = tw::CudaSolverFIM::stage(ekdata);
      std::FILE *f = std::fopen(argv[6], "wb");
      if (!f) throw std::runtime_error(std::string("cannot write ") + argv[6]);
      const int64_t hdr[6] = {(int64_t)(in.xyz.size() / 3), (int64_t)(in.tets.size() / 4), (int64_t)in.atags.size(),
                              (int64_t)in.etags.size(), (int64_t)in.stim.size(), in.n_steps};
      put(f, hdr, 6);
      put(f, &in.dt, 1);
      put(f, in.xyz.data(), in.xyz.size());
      put(f, in.tets.data(), in.tets.size());
      put(f, in.atags.data(), in.atags.size());
      put(f, in.etags.data(), in.etags.size());
      put(f, in.fib.data(), in.fib.size());
      put(f, in.cf.data(), in.cf.size());
      put(f, in.ct.data(), in.ct.size());
      put(f, in.stim.data(), in.stim.size());
      std::fclose(f);
      return 0;
    }
    std::vector<std::vector<double>> act_ms, apd_ms;
    tw::CudaSolverFIM solver(ekdata);
    const double t = solver.solve(act_ms, apd_ms, argv[6], 1);
    std::printf("Average execution time for %d runs: %f s\n", 1, t);
    return 0;
  } catch (const std::exception &e) {
    std::fprintf(stderr, "ref_types_driver: %s\n", e.what());
    return 1;
  }
}
