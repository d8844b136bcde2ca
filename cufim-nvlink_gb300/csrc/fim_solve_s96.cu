// fim_solve_s96.cu -- the persistent solve kernel for batches of up to
// 96 vertices / 2048 corners (one compiled batch shape; see fim_solve.cuh).
#define FIM_SLOTS 96
#define FIM_CORNER_CAP 2048
#define FIM_SHAPE_NS shape_s96
#include "fim_solve.cuh"

namespace fimgb {

cudaError_t solve_prepare_s96(int device, int block, int *max_grid)
{
  return shape_s96::prepare(device, block, max_grid);
}

cudaError_t solve_launch_s96(const FimDev &d, const FimParams &p, int grid, int block, cudaStream_t stream)
{
  return shape_s96::launch(d, p, grid, block, stream);
}

}  // namespace fimgb
