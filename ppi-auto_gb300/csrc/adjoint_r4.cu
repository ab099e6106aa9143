// adjoint_r4.cu -- the constant adjoint's kernels at 4 records per thread
// (a separate translation unit so that the build compiles them in parallel).
#include "adjoint_impl.cuh"

namespace ppi {
cudaError_t launch_adjoint_r4(int math, int opset, const AdjointArgs& a, int block, int grid, size_t smem,
                              cudaStream_t s) {
   return adj::launch<4>(math, opset, a, block, grid, smem, s);
}
cudaError_t adjoint_occupancy_r4(int math, int opset, int block, size_t smem, int* per_sm) {
   return adj::occupancy<4>(math, opset, block, smem, per_sm);
}
}  // namespace ppi
