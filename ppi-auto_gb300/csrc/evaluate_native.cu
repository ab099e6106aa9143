// evaluate_native.cu -- evaluator kernels instantiated for one math mode
// (separate translation units so that the build compiles them in parallel).
#include "evaluate_impl.cuh"

namespace ppi {
template struct ev::Launch<kMathNative>;
cudaError_t launch_evaluate_native(int opset, int direct, const EvalArgs& a, int block, int grid, size_t smem,
                              cudaStream_t s) {
   return ev::Launch<kMathNative>::evaluate(opset, direct, a, block, grid, smem, s);
}
cudaError_t launch_predict_native(int opset, const PredictArgs& a, int block, int grid, size_t smem, cudaStream_t s) {
   return ev::Launch<kMathNative>::predict(opset, a, block, grid, smem, s);
}
cudaError_t launch_evaluate_batch_native(int opset, int direct, const BatchArgs& a, int block, int grid,
                                    size_t smem, cudaStream_t s) {
   return ev::Launch<kMathNative>::evaluate_batch(opset, direct, a, block, grid, smem, s);
}
cudaError_t evaluate_occupancy_native(int opset, int direct, int block, size_t smem, int* per_sm) {
   return ev::Launch<kMathNative>::occupancy(opset, direct, block, smem, per_sm);
}
cudaError_t evaluate_batch_occupancy_native(int opset, int direct, int block, size_t smem, int* per_sm) {
   return ev::Launch<kMathNative>::occupancy_batch(opset, direct, block, smem, per_sm);
}

}  // namespace ppi
