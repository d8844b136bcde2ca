// fim_solve_s160.cu -- the persistent solve kernel for batches of up to
// 160 vertices / 3072 corners (one compiled batch shape; see fim_solve.cuh).
#define FIM_SLOTS 160
#define FIM_CORNER_CAP 3072
#define FIM_SHAPE_NS shape_s160
#include "fim_solve.cuh"

namespace fimgb {

cudaError_t solve_prepare_s160(int device, int block, int *max_grid)
{
  return shape_s160::prepare(device, block, max_grid);
}

cudaError_t solve_launch_s160(const FimDev &d, const FimParams &p, int grid, int block, cudaStream_t stream)
{
  return shape_s160::launch(d, p, grid, block, stream);
}

}  // namespace fimgb
