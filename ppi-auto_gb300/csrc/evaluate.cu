// evaluate.cu -- launch geometry and math-mode dispatch of the evaluator
// kernels (evaluate_impl.cuh, instantiated in evaluate_{fast,parity,native}.cu).
#include <algorithm>
#include <cmath>
#include <cstdlib>

#include "ppi_internal.cuh"

namespace ppi {

cudaError_t launch_evaluate_fast(int R, const EvalArgs& a, int block, int grid, size_t smem, cudaStream_t s);
cudaError_t launch_evaluate_parity(int R, const EvalArgs& a, int block, int grid, size_t smem, cudaStream_t s);
cudaError_t launch_evaluate_native(int R, const EvalArgs& a, int block, int grid, size_t smem, cudaStream_t s);
cudaError_t launch_predict_fast(int R, const PredictArgs& a, int block, int grid, size_t smem, cudaStream_t s);
cudaError_t launch_predict_parity(int R, const PredictArgs& a, int block, int grid, size_t smem, cudaStream_t s);
cudaError_t launch_predict_native(int R, const PredictArgs& a, int block, int grid, size_t smem, cudaStream_t s);
cudaError_t evaluate_occupancy_fast(int R, int block, size_t smem, int* per_sm);
cudaError_t evaluate_occupancy_parity(int R, int block, size_t smem, int* per_sm);
cudaError_t evaluate_occupancy_native(int R, int block, size_t smem, int* per_sm);

size_t evaluate_smem_bytes(int code_stride, int ncol, int block, int R, int lanes, bool aligned) {
   const size_t T = (size_t)block * R;
   const size_t code = ((size_t)(code_stride + 1) * sizeof(uint2) + 15) & ~(size_t)15;
   const size_t rows = (size_t)(ncol + kSlots) * T * 4;
   if (aligned) return code + std::max(rows, (size_t)lanes * 4);
   return code + rows + T * 4 + (size_t)lanes * 8;
}

cudaError_t launch_evaluate(int math, int R, const EvalArgs& a, int block, int grid, size_t smem,
                            cudaStream_t s) {
   switch (math) {
   case kMathParity: return launch_evaluate_parity(R, a, block, grid, smem, s);
   case kMathNative: return launch_evaluate_native(R, a, block, grid, smem, s);
   default: return launch_evaluate_fast(R, a, block, grid, smem, s);
   }
}

cudaError_t launch_predict(int math, int R, const PredictArgs& a, int block, int grid, size_t smem,
                           cudaStream_t s) {
   switch (math) {
   case kMathParity: return launch_predict_parity(R, a, block, grid, smem, s);
   case kMathNative: return launch_predict_native(R, a, block, grid, smem, s);
   default: return launch_predict_fast(R, a, block, grid, smem, s);
   }
}

cudaError_t evaluate_occupancy(int math, int R, int block, size_t smem, int* per_sm) {
   switch (math) {
   case kMathParity: return evaluate_occupancy_parity(R, block, smem, per_sm);
   case kMathNative: return evaluate_occupancy_native(R, block, smem, per_sm);
   default: return evaluate_occupancy_fast(R, block, smem, per_sm);
   }
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

const char* plan_geometry(int strategy, int lanes, int math, int nlin, int ncol, int code_stride,
                          int n_max, int sm_count, Geometry* g) {
   const int L = lanes;
   if (L < 1 || L > kMaxLanes) return "lane count out of range";
   // records per thread: 8 (measured faster than 16 on GB300: more resident
   // warps hide the dispatch latency); PPI_GPU_RECORDS_PER_THREAD=16 selects
   // 16 where the lane == tile-position path allows it
   const char* env = std::getenv("PPI_GPU_RECORDS_PER_THREAD");
   const bool allow16 = env && std::atoi(env) == 16;
   int R = 8, P;
   if (strategy == PPI_STRATEGY_PDP && allow16 && L % (32 * 16) == 0 && L / 16 <= 128) {
      R = 16;
      P = L / 16;
   } else if (strategy == PPI_STRATEGY_PDP && L % (32 * 8) == 0 && L / 8 <= 128) {
      P = L / 8;
   } else {
      const int need = (strategy == PPI_STRATEGY_DP) ? L : std::min(nlin, 128 * 8);
      P = std::min(128, std::max(32, ((need + 7) / 8 + 31) / 32 * 32));
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
   if (evaluate_occupancy(math, R, P, smem, &per_sm) != cudaSuccess || per_sm < 1)
      return "evaluator does not fit on an SM";
   g->lanes = L;
   g->block = P;
   g->R = R;
   g->smem = smem;
   g->grid = std::max(1, std::min(n_max, per_sm * sm_count));
   return nullptr;
}

}  // namespace ppi
