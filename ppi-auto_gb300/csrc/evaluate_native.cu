// evaluate_native.cu -- evaluator kernels instantiated for one math mode
// (separate translation units so that the build compiles them in parallel);
// the kernels with the one-lane chain are in evaluate_native_lane1.cu.
#include "evaluate_impl.cuh"

PPI_EVALUATOR_ENTRY_POINTS(ppi::kMathNative, 0, native)

namespace ppi {
cudaError_t launch_predict_native(int opset, const PredictArgs& a, int block, int grid, size_t smem, cudaStream_t s) {
   return ev::Launch<kMathNative, 0>::predict(opset, a, block, grid, smem, s);
}
}  // namespace ppi

