// fim_solve_s192.cu -- the persistent solve kernel for batches of up to
// 192 vertices / 4096 corners (one compiled batch shape; see fim_solve.cuh).
#define FIM_SLOTS 192
#define FIM_CORNER_CAP 4096
#define FIM_SHAPE_NS shape_s192
#include "fim_solve.cuh"

namespace fimgb {

cudaError_t solve_prepare_s192(int device, int block, int *max_grid)
{
  return shape_s192::prepare(device, block, max_grid);
}

cudaError_t solve_launch_s192(const FimDev &d, const FimParams &p, int grid, int block, cudaStream_t stream)
{
  return shape_s192::launch(d, p, grid, block, stream);
}

}  // namespace fimgb
