// evaluate_native_chunk.cu -- the chunked evaluator kernels (work items of one
// program and one record chunk, in chunk-major order) for one math mode, in
// a translation unit of their own so that the build compiles them in
// parallel with the others.
#include "evaluate_impl.cuh"

PPI_EVALUATOR_ENTRY_POINTS(ppi::kMathNative, ppi::kFamilyChunked, native2)
