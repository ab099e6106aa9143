// evaluate_fast.cu -- evaluator kernels instantiated for one math mode
// (separate translation units so that the build compiles them in parallel);
// the kernels with the one-lane chain are in evaluate_fast_lane1.cu.
#include "evaluate_impl.cuh"

PPI_EVALUATOR_ENTRY_POINTS(ppi::kMathFast, 0, fast)

namespace ppi {
cudaError_t launch_predict_fast(int opset, const PredictArgs& a, int block, int grid, size_t smem, cudaStream_t s) {
   return ev::Launch<kMathFast, 0>::predict(opset, a, block, grid, smem, s);
}
}  // namespace ppi

extern "C" int32_t ppi_gpu_kernel_arch(void) {
   cudaFuncAttributes fa{};
   if (cudaFuncGetAttributes(&fa, ppi::ev::eval_kernel<ppi::kMathFast, ppi::kR, ppi::kOpsetArith, 0, 0, 0>) !=
       cudaSuccess)
      return -1;
   return fa.binaryVersion;
}
