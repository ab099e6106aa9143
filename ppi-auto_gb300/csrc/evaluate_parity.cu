// evaluate_parity.cu -- evaluator kernels instantiated for one math mode
// (separate translation units so that the build compiles them in parallel).
#include "evaluate_impl.cuh"

namespace ppi {
template struct ev::Launch<kMathParity>;
cudaError_t launch_evaluate_parity(int opset, int direct, const EvalArgs& a, int block, int grid, size_t smem,
                              cudaStream_t s) {
   return ev::Launch<kMathParity>::evaluate(opset, direct, a, block, grid, smem, s);
}
cudaError_t launch_predict_parity(int opset, const PredictArgs& a, int block, int grid, size_t smem, cudaStream_t s) {
   return ev::Launch<kMathParity>::predict(opset, a, block, grid, smem, s);
}
cudaError_t launch_evaluate_batch_parity(int opset, int direct, const BatchArgs& a, int block, int grid,
                                    size_t smem, cudaStream_t s) {
   return ev::Launch<kMathParity>::evaluate_batch(opset, direct, a, block, grid, smem, s);
}
cudaError_t evaluate_occupancy_parity(int opset, int direct, int block, size_t smem, int* per_sm) {
   return ev::Launch<kMathParity>::occupancy(opset, direct, block, smem, per_sm);
}
cudaError_t evaluate_batch_occupancy_parity(int opset, int direct, int block, size_t smem, int* per_sm) {
   return ev::Launch<kMathParity>::occupancy_batch(opset, direct, block, smem, per_sm);
}

}  // namespace ppi
