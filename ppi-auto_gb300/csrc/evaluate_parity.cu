// evaluate_parity.cu -- evaluator kernels instantiated for one math mode
// (separate translation units so that the build compiles them in parallel);
// the kernels with the one-lane chain are in evaluate_parity_lane1.cu.
#include "evaluate_impl.cuh"

PPI_EVALUATOR_ENTRY_POINTS(ppi::kMathParity, 0, parity)

namespace ppi {
cudaError_t launch_predict_parity(int opset, const PredictArgs& a, int block, int grid, size_t smem, cudaStream_t s) {
   return ev::Launch<kMathParity, 0>::predict(opset, a, block, grid, smem, s);
}
}  // namespace ppi

