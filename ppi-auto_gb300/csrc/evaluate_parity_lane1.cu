// evaluate_parity_lane1.cu -- the evaluator kernels with the one-lane chain
// (PP populations) for one math mode, in a translation unit of their own so
// that the build compiles them in parallel with the others.
#include "evaluate_impl.cuh"

PPI_EVALUATOR_ENTRY_POINTS(ppi::kMathParity, 1, parity1)
