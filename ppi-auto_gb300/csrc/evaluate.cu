// evaluate.cu -- launch geometry and math-mode dispatch of the evaluator
// kernels (evaluate_impl.cuh, instantiated in evaluate_{fast,parity,native}.cu).
#include <algorithm>
#include <cmath>
#include <cstdlib>

#include "ppi_internal.cuh"

namespace ppi {

cudaError_t launch_evaluate_fast(int opset, const EvalArgs& a, int block, int grid, size_t smem, cudaStream_t s);
cudaError_t launch_evaluate_parity(int opset, const EvalArgs& a, int block, int grid, size_t smem, cudaStream_t s);
cudaError_t launch_evaluate_native(int opset, const EvalArgs& a, int block, int grid, size_t smem, cudaStream_t s);
cudaError_t launch_predict_fast(int opset, const PredictArgs& a, int block, int grid, size_t smem, cudaStream_t s);
cudaError_t launch_predict_parity(int opset, const PredictArgs& a, int block, int grid, size_t smem, cudaStream_t s);
cudaError_t launch_predict_native(int opset, const PredictArgs& a, int block, int grid, size_t smem, cudaStream_t s);
cudaError_t evaluate_occupancy_fast(int opset, int block, size_t smem, int* per_sm);
cudaError_t evaluate_occupancy_parity(int opset, int block, size_t smem, int* per_sm);
cudaError_t evaluate_occupancy_native(int opset, int block, size_t smem, int* per_sm);

size_t evaluate_smem_bytes(int code_stride, int ncol, int block, int R, int lanes, bool aligned) {
   const size_t T = (size_t)block * R;
   const size_t code = ((size_t)(code_stride + 1) * sizeof(uint2) + 15) & ~(size_t)15;
   const size_t rows = (size_t)(ncol + kSlots) * T * 4;
   if (aligned) return code + std::max(rows, (size_t)lanes * 4);
   return code + rows + T * 4 + (size_t)lanes * 8;
}

cudaError_t launch_evaluate(int math, int opset, const EvalArgs& a, int block, int grid, size_t smem,
                            cudaStream_t s) {
   switch (math) {
   case kMathParity: return launch_evaluate_parity(opset, a, block, grid, smem, s);
   case kMathNative: return launch_evaluate_native(opset, a, block, grid, smem, s);
   default: return launch_evaluate_fast(opset, a, block, grid, smem, s);
   }
}

cudaError_t launch_predict(int math, int opset, const PredictArgs& a, int block, int grid, size_t smem,
                           cudaStream_t s) {
   switch (math) {
   case kMathParity: return launch_predict_parity(opset, a, block, grid, smem, s);
   case kMathNative: return launch_predict_native(opset, a, block, grid, smem, s);
   default: return launch_predict_fast(opset, a, block, grid, smem, s);
   }
}

cudaError_t evaluate_occupancy(int math, int opset, int block, size_t smem, int* per_sm) {
   switch (math) {
   case kMathParity: return evaluate_occupancy_parity(opset, block, smem, per_sm);
   case kMathNative: return evaluate_occupancy_native(opset, block, smem, per_sm);
   default: return evaluate_occupancy_fast(opset, block, smem, per_sm);
   }
}

int opset_for(const ppi_symbol_entry* symbols, int n) {
   for (int i = 0; i < n; ++i) {
      switch (symbols[i].op) {
      case PPI_OP_INVALID: case PPI_OP_ATTRIBUTE: case PPI_OP_CONST: case PPI_OP_LITERAL:
      case PPI_OP_ADD: case PPI_OP_SUB: case PPI_OP_MULT: case PPI_OP_DIV:
      case PPI_OP_ABS: case PPI_OP_POW2: case PPI_OP_NEG: case PPI_OP_EXP: case PPI_OP_SIN:
      case PPI_OP_COS: case PPI_OP_SQRT: case PPI_OP_LOG:
         break;
      default:
         return kOpsetFull;
      }
   }
   return kOpsetArith;
}

int resolve_lanes(int strategy, int lanes, int nlin, int sm_count) {
   // -cl-mls when given; else the reference's rule (accelerator.cc:296-330) on
   // a device with 1024-wide work-groups and sm_count compute units.
   if (strategy == PPI_STRATEGY_PP) return 1;
   if (lanes <= 0 && strategy == PPI_STRATEGY_PDP) return std::min(nlin, 1024);
   if (lanes <= 0) return std::min(1024, (int)std::ceil(nlin / (float)std::max(1, sm_count)));
   if (strategy == PPI_STRATEGY_PDP) return std::min(lanes, nlin);
   return lanes;
}

const char* plan_geometry(int strategy, int lanes, int math, int opset, int nlin, int ncol,
                          int code_stride, int n_max, int sm_count, Geometry* g) {
   const int L = lanes;
   if (L < 1 || L > kMaxLanes) return "lane count out of range";
   // records per thread: kR (8 measured faster than 16 on GB300: more
   // resident warps hide the dispatch latency)
   const int R = kR;
   int P;
   if (strategy == PPI_STRATEGY_PDP && L % (32 * R) == 0 && L / R <= 128) {
      P = L / R;   // lane == tile position: register accumulation
   } else {
      const int need = (strategy == PPI_STRATEGY_DP) ? L : std::min(nlin, 128 * R);
      P = std::min(128, std::max(32, ((need + R - 1) / R + 31) / 32 * 32));
   }
   if (strategy == PPI_STRATEGY_DP && L > P * R)
      return "DP lanes above 1024 records per group are not supported";
   bool aligned = strategy == PPI_STRATEGY_PDP && L == P * R;
   size_t smem = evaluate_smem_bytes(code_stride, ncol, P, R, L, aligned);
   while (smem > 200 * 1024 && P > 32 && !(strategy == PPI_STRATEGY_DP && L > (P / 2) * R)) {
      P /= 2;
      aligned = strategy == PPI_STRATEGY_PDP && L == P * R;
      smem = evaluate_smem_bytes(code_stride, ncol, P, R, L, aligned);
   }
   if (smem > 200 * 1024) return "dataset has too many columns for one shared-memory tile";
   int per_sm = 0;
   if (evaluate_occupancy(math, opset, P, smem, &per_sm) != cudaSuccess || per_sm < 1)
      return "evaluator does not fit on an SM";
   g->lanes = L;
   g->block = P;
   g->R = R;
   g->opset = opset;
   g->smem = smem;
   g->grid = std::max(1, std::min(n_max, per_sm * sm_count));
   return nullptr;
}

}  // namespace ppi
