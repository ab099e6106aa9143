// evaluate.cu -- launch geometry and math-mode dispatch of the evaluator
// kernels (evaluate_impl.cuh, instantiated in evaluate_{fast,parity,native}.cu
// and, with the one-lane chain, evaluate_{fast,parity,native}_lane1.cu).
#include <algorithm>
#include <cmath>
#include <cstdlib>

#include "ppi_internal.cuh"

namespace ppi {

// Entry points of evaluate_<math>.cu (suffix <math>), evaluate_<math>_lane1.cu
// (suffix <math>1) and evaluate_<math>_chunk.cu (suffix <math>2).
#define PPI_DECLARE_ENTRY_POINTS(S)                                                             \
   cudaError_t launch_evaluate_##S(int opset, int direct, const EvalArgs& a, int block, int grid, \
                                   size_t smem, cudaStream_t s);                              \
   cudaError_t launch_evaluate_batch_##S(int opset, int direct, const BatchArgs& a, int block,  \
                                         int grid, size_t smem, cudaStream_t s);              \
   cudaError_t evaluate_occupancy_##S(int opset, int direct, int block, size_t smem, int* per_sm); \
   cudaError_t evaluate_batch_occupancy_##S(int opset, int direct, int block, size_t smem, int* per_sm);
PPI_DECLARE_ENTRY_POINTS(fast)
PPI_DECLARE_ENTRY_POINTS(fast1)
PPI_DECLARE_ENTRY_POINTS(fast2)
PPI_DECLARE_ENTRY_POINTS(parity)
PPI_DECLARE_ENTRY_POINTS(parity1)
PPI_DECLARE_ENTRY_POINTS(parity2)
PPI_DECLARE_ENTRY_POINTS(native)
PPI_DECLARE_ENTRY_POINTS(native1)
PPI_DECLARE_ENTRY_POINTS(native2)
#undef PPI_DECLARE_ENTRY_POINTS
cudaError_t launch_predict_fast(int opset, const PredictArgs& a, int block, int grid, size_t smem, cudaStream_t s);
cudaError_t launch_predict_parity(int opset, const PredictArgs& a, int block, int grid, size_t smem, cudaStream_t s);
cudaError_t launch_predict_native(int opset, const PredictArgs& a, int block, int grid, size_t smem, cudaStream_t s);

size_t evaluate_smem_bytes(int code_stride, int rows, int block, int R, int lanes, bool aligned) {
   const size_t T = (size_t)block * R;
   const size_t code = ((size_t)(code_stride + 1) * sizeof(uint2) + 15) & ~(size_t)15;
   const size_t tile = (size_t)std::max(rows, 1) * T * 4;
   if (aligned) return code + tile;   // lane values reuse the tile
   return code + tile + (size_t)lanes * 4 + (((size_t)lanes + 15) & ~(size_t)15);
}

cudaError_t launch_evaluate(int math, int opset, int direct, const EvalArgs& a, int block, int grid,
                            size_t smem, cudaStream_t s) {
   const int k = direct & ~(kOneLane | kChunked);
   const int fam = (direct & kOneLane) ? 1 : ((direct & kChunked) ? 2 : 0);
   switch (math) {
   case kMathParity: return fam == 1 ? launch_evaluate_parity1(opset, k, a, block, grid, smem, s)
                           : fam == 2 ? launch_evaluate_parity2(opset, k, a, block, grid, smem, s)
                           : launch_evaluate_parity(opset, k, a, block, grid, smem, s);
   case kMathNative: return fam == 1 ? launch_evaluate_native1(opset, k, a, block, grid, smem, s)
                           : fam == 2 ? launch_evaluate_native2(opset, k, a, block, grid, smem, s)
                           : launch_evaluate_native(opset, k, a, block, grid, smem, s);
   default: return fam == 1 ? launch_evaluate_fast1(opset, k, a, block, grid, smem, s)
                           : fam == 2 ? launch_evaluate_fast2(opset, k, a, block, grid, smem, s)
                           : launch_evaluate_fast(opset, k, a, block, grid, smem, s);
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

cudaError_t launch_evaluate_batch(int math, int opset, int direct, const BatchArgs& a, int block, int grid,
                                  size_t smem, cudaStream_t s) {
   const int k = direct & ~(kOneLane | kChunked);
   const int fam = (direct & kOneLane) ? 1 : ((direct & kChunked) ? 2 : 0);
   switch (math) {
   case kMathParity: return fam == 1 ? launch_evaluate_batch_parity1(opset, k, a, block, grid, smem, s)
                           : fam == 2 ? launch_evaluate_batch_parity2(opset, k, a, block, grid, smem, s)
                           : launch_evaluate_batch_parity(opset, k, a, block, grid, smem, s);
   case kMathNative: return fam == 1 ? launch_evaluate_batch_native1(opset, k, a, block, grid, smem, s)
                           : fam == 2 ? launch_evaluate_batch_native2(opset, k, a, block, grid, smem, s)
                           : launch_evaluate_batch_native(opset, k, a, block, grid, smem, s);
   default: return fam == 1 ? launch_evaluate_batch_fast1(opset, k, a, block, grid, smem, s)
                           : fam == 2 ? launch_evaluate_batch_fast2(opset, k, a, block, grid, smem, s)
                           : launch_evaluate_batch_fast(opset, k, a, block, grid, smem, s);
   }
}

cudaError_t evaluate_occupancy(int math, int opset, int direct, int block, size_t smem, int* per_sm) {
   const int k = direct & ~(kOneLane | kChunked);
   const int fam = (direct & kOneLane) ? 1 : ((direct & kChunked) ? 2 : 0);
   switch (math) {
   case kMathParity: return fam == 1 ? evaluate_occupancy_parity1(opset, k, block, smem, per_sm)
                           : fam == 2 ? evaluate_occupancy_parity2(opset, k, block, smem, per_sm)
                           : evaluate_occupancy_parity(opset, k, block, smem, per_sm);
   case kMathNative: return fam == 1 ? evaluate_occupancy_native1(opset, k, block, smem, per_sm)
                           : fam == 2 ? evaluate_occupancy_native2(opset, k, block, smem, per_sm)
                           : evaluate_occupancy_native(opset, k, block, smem, per_sm);
   default: return fam == 1 ? evaluate_occupancy_fast1(opset, k, block, smem, per_sm)
                           : fam == 2 ? evaluate_occupancy_fast2(opset, k, block, smem, per_sm)
                           : evaluate_occupancy_fast(opset, k, block, smem, per_sm);
   }
}

cudaError_t evaluate_batch_occupancy(int math, int opset, int direct, int block, size_t smem, int* per_sm) {
   const int k = direct & ~(kOneLane | kChunked);
   const int fam = (direct & kOneLane) ? 1 : ((direct & kChunked) ? 2 : 0);
   switch (math) {
   case kMathParity: return fam == 1 ? evaluate_batch_occupancy_parity1(opset, k, block, smem, per_sm)
                           : fam == 2 ? evaluate_batch_occupancy_parity2(opset, k, block, smem, per_sm)
                           : evaluate_batch_occupancy_parity(opset, k, block, smem, per_sm);
   case kMathNative: return fam == 1 ? evaluate_batch_occupancy_native1(opset, k, block, smem, per_sm)
                           : fam == 2 ? evaluate_batch_occupancy_native2(opset, k, block, smem, per_sm)
                           : evaluate_batch_occupancy_native(opset, k, block, smem, per_sm);
   default: return fam == 1 ? evaluate_batch_occupancy_fast1(opset, k, block, smem, per_sm)
                           : fam == 2 ? evaluate_batch_occupancy_fast2(opset, k, block, smem, per_sm)
                           : evaluate_batch_occupancy_fast(opset, k, block, smem, per_sm);
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

int resolve_best_group(int rule, int group, int population, int sm_count) {
   if (rule == PPI_BEST_SEQUENTIAL) return 1;
   if (group > 0) return group;
   // local_size2 = min(max_local_size2, ceil(population_size / max_cu)), with
   // max_local_size2 = 1024 (the work-group limit; 48 KB of local memory / 8
   // bytes per item allows more)
   const long long cu = std::max(1, sm_count);
   return (int)std::max(1LL, std::min(1024LL, ((long long)std::max(1, population) + cu - 1) / cu));
}

const char* best_geometry(int rule, int group, int strategy, int n, BestGeo* out) {
   if (rule != PPI_BEST_ACCELERATOR && rule != PPI_BEST_SEQUENTIAL) return "unknown best-index rule";
   if (group < 1 || n < 1) return "best-index group size must be positive";
   int bits = 0;
   while (bits < 31 && (1LL << bits) < group) ++bits;
   const long long groups = ((long long)n + group - 1) / group;
   // the tie field holds (groups - 1) << bits | position in 32 bits
   if ((groups << bits) > (1LL << 32)) return "best-index group geometry does not fit the 32-bit tie field";
   out->group = group;
   out->bits = bits;
   out->groups = (int)groups;
   out->alpha_free = rule == PPI_BEST_ACCELERATOR && strategy != PPI_STRATEGY_DP;
   return nullptr;
}

const char* plan_geometry(int strategy, int lanes, int math, int opset, int nlin, int ncol,
                          int code_stride, int n_max, int sm_count, Geometry* g, bool allow_chunk) {
   const int L = lanes;
   if (L < 1 || L > kMaxLanes) return "lane count out of range";
   // records per thread: kR (8 measured faster than 16 on GB300: more
   // resident warps hide the dispatch latency)
   const int R = kR;
   constexpr size_t kSmemCap = 200 * 1024;
   int P;
   if (strategy == PPI_STRATEGY_PDP && L % (32 * R) == 0 && L / R <= 128) {
      P = L / R;   // lane == tile position: register accumulation
   } else {
      const int need = (strategy == PPI_STRATEGY_DP) ? L : std::min(nlin, 128 * R);
      P = std::min(128, std::max(32, ((need + R - 1) / R + 31) / 32 * 32));
   }
   if (strategy == PPI_STRATEGY_DP && L > P * R)
      return "DP lanes above 1024 records per group are not supported";
   const int rows_max = max_program_rows(ncol);
   auto aligned_for = [&](int p) { return strategy == PPI_STRATEGY_PDP && L == p * R; };
   // rows that fit in kSmemCap next to the code and lane buffers
   auto rows_fit = [&](int p) {
      const size_t fixed = evaluate_smem_bytes(code_stride, 0, p, R, L, aligned_for(p)) -
                           (size_t)p * R * 4;
      if (fixed >= kSmemCap) return 0;
      return (int)std::min<size_t>((kSmemCap - fixed) / ((size_t)p * R * 4), 4096);
   };
   while (P > 32 && rows_fit(P) < std::min(rows_max, kSlots + 2) &&
          !(strategy == PPI_STRATEGY_DP && L > (P / 2) * R))
      P /= 2;
   const bool aligned = aligned_for(P);
   const int fit = std::min(rows_max, rows_fit(P));
   if (fit < 1) return "lane buffers do not fit in shared memory";
   // one lane (PP, or PDP over one lane): the kernels with the one-lane chain;
   // lane == tile position over a dataset larger than L2: the chunked kernels
   // (every program walks the same records at about the same time, so a
   // record chunk comes from DRAM once and from L2 for the other programs),
   // when the population's (program, chunk) pairs fit the kernels' 32-bit
   // work counter (2^30 of them)
   const long long chunk_recs = (long long)kChunkTiles * P * R;
   const bool chunk = allow_chunk && strategy == PPI_STRATEGY_PDP && aligned_for(P) &&
                      (size_t)nlin * ncol * 4 >= kChunkMinBytes &&
                      (long long)n_max * ((nlin + chunk_recs - 1) / chunk_recs) < (1LL << 30);
   const int one = strategy != PPI_STRATEGY_DP && L == 1 ? kOneLane : (chunk ? kChunked : 0);
   auto occupancy = [&](int direct, int rows) {
      int per_sm = 0;
      const size_t smem = evaluate_smem_bytes(code_stride, rows, P, R, L, aligned);
      if (evaluate_occupancy(math, opset, direct | one, P, smem, &per_sm) != cudaSuccess) return 0;
      return per_sm;
   };
   // the most rows at the occupancy of a one-row tile
   auto best_rows = [&](int direct) {
      const int top = occupancy(direct, 1);
      int rows = 1;
      while (rows < fit && occupancy(direct, rows + 1) >= top) ++rows;
      return rows;
   };
   // main pass: programs whose columns all fit, lean kernel; when the whole
   // population is resident in one wave at a larger tile, the larger tile
   // (the most rows at which it still is: occupancy falls as rows grow).
   // Planned with each register bound of the main-pass kernel; the one with
   // more resident CTAs at its rows runs (the 64-register build only where
   // its tile lets more CTAs fit).
   auto main_rows = [&](int k) {
      int r = best_rows(k);
      if ((long long)occupancy(k, fit) * sm_count >= n_max) {
         r = fit;
      } else if ((long long)occupancy(k, r + 1) * sm_count >= n_max && r < fit) {
         int lo = r + 1, hi = fit;   // occupancy(lo) fits, occupancy(hi) does not
         while (hi - lo > 1) {
            const int mid = (lo + hi) / 2;
            if ((long long)occupancy(k, mid) * sm_count >= n_max) lo = mid;
            else hi = mid;
         }
         r = lo;
      }
      return r;
   };
   int main_kernel = 0, rows = main_rows(0);
   const int rows_hi = main_rows(kMainHi);
   if (occupancy(kMainHi, rows_hi) > occupancy(0, rows)) {
      main_kernel = kMainHi;
      rows = rows_hi;
   }
   // second pass: the rest, with the columns that do not fit read directly
   // (room at least for the deepest slot need and the target)
   // whole-quad direct reads need tiles that start on a multiple of 4
   // records: PP and PDP tiles (T records) always do, DP tiles (whole groups
   // of L records) when dp_tile_groups found a whole-quad count
   const int tile_step = strategy == PPI_STRATEGY_DP ? L * dp_tile_groups(L, P * R) : P * R;
   const int wk = tile_step % 4 == 0 ? 2 : 1;
   const int rows2 = std::max(best_rows(wk), std::min(fit, kSlots + 1));
   g->lanes = L;
   g->block = P;
   g->R = R;
   g->opset = opset;
   g->aligned = aligned;
   g->rows = rows;
   g->smem = evaluate_smem_bytes(code_stride, rows, P, R, L, aligned);
   g->per_sm[0] = occupancy(main_kernel, rows);
   g->main_kernel = main_kernel | one;
   if (g->per_sm[0] < 1) return "evaluator does not fit on an SM";
   g->grid = std::max(1, std::min(n_max, g->per_sm[0] * sm_count));
   g->wide = rows < rows_max;
   g->rows_wide = rows2;
   g->smem_wide = evaluate_smem_bytes(code_stride, rows2, P, R, L, aligned);
   g->wide_kernel = wk | one;
   g->chunked = chunk;
   g->chunk_records = kChunkTiles * P * R;
   g->n_chunks = chunk ? (nlin + g->chunk_records - 1) / g->chunk_records : 1;
   // programs per group (wide pass): their lane states and code in a quarter
   // of L2, so that the state a chunk stores is still there when the
   // program's next chunk reads it (the whole population's state, 4.6 KB a
   // program, spilled to DRAM at 30,000 programs); each group streams the
   // dataset once more. On 4M records x 32 columns and 30,000 programs the
   // wide pass moved 16.8 GB of DRAM ungrouped, 5.5 GB with half of L2 and
   // 4.9 GB with a quarter, in the same time.
   if (chunk) {
      int dev = 0, l2 = 0;
      if (cudaGetDevice(&dev) != cudaSuccess ||
          cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, dev) != cudaSuccess || l2 <= 0)
         l2 = 128 << 20;
      const size_t per = (size_t)(R + 1) * P * 4 + (size_t)code_stride * sizeof(uint2);
      g->chunk_group = (int)std::max<size_t>(2048, ((size_t)l2 / 4) / per);
   }
   g->per_sm[1] = occupancy(wk, rows2);
   if (g->per_sm[1] < 1) return "evaluator does not fit on an SM";
   g->grid_wide = std::max(1, std::min(n_max, g->per_sm[1] * sm_count));
   return nullptr;
}

}  // namespace ppi
