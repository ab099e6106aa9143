// evaluate_fast.cu -- evaluator kernels instantiated for one math mode
// (separate translation units so that the build compiles them in parallel).
#include "evaluate_impl.cuh"

namespace ppi {
template struct ev::Launch<kMathFast>;
cudaError_t launch_evaluate_fast(int opset, int direct, const EvalArgs& a, int block, int grid, size_t smem,
                              cudaStream_t s) {
   return ev::Launch<kMathFast>::evaluate(opset, direct, a, block, grid, smem, s);
}
cudaError_t launch_predict_fast(int opset, const PredictArgs& a, int block, int grid, size_t smem, cudaStream_t s) {
   return ev::Launch<kMathFast>::predict(opset, a, block, grid, smem, s);
}
cudaError_t launch_evaluate_batch_fast(int opset, int direct, const BatchArgs& a, int block, int grid,
                                    size_t smem, cudaStream_t s) {
   return ev::Launch<kMathFast>::evaluate_batch(opset, direct, a, block, grid, smem, s);
}
cudaError_t evaluate_occupancy_fast(int opset, int direct, int block, size_t smem, int* per_sm) {
   return ev::Launch<kMathFast>::occupancy(opset, direct, block, smem, per_sm);
}
cudaError_t evaluate_batch_occupancy_fast(int opset, int direct, int block, size_t smem, int* per_sm) {
   return ev::Launch<kMathFast>::occupancy_batch(opset, direct, block, smem, per_sm);
}

}  // namespace ppi

extern "C" int32_t ppi_gpu_kernel_arch(void) {
   cudaFuncAttributes fa{};
   if (cudaFuncGetAttributes(&fa, ppi::ev::eval_kernel<ppi::kMathFast, ppi::kR, ppi::kOpsetArith, 0, 0>) !=
       cudaSuccess)
      return -1;
   return fa.binaryVersion;
}
