// batch.cu -- many populations evaluated together, one persistent launch per pass.
//
// A GE run with several islands, or several independent runs, has
// populations of very different sizes, program lengths and datasets.  One
// plain evaluation per population leaves most of the GPU idle on the small
// ones and pays a tail on every launch.  Here all programs of all populations
// form one work queue, ordered by cost (size x records, largest first, via
// 64 power-of-two buckets counted by the translator), and one persistent grid
// per pass drains it.  Each population keeps its own strategy, lane count, error
// function and accumulation order, so every fitness is bit-identical to the
// plain evaluation of that population.
//
// Each CTA stages only the columns its current program reads, so the tile's
// shared memory follows the program, not the widest dataset of the batch.
// The main pass runs every program whose tile fits its row budget (the most
// rows at full occupancy, or what the row histogram of an earlier evaluation
// asks for); the wide pass runs the rest with a larger tile.
// Per generation the device work is: memsets, the translator, the order
// scan, the order scatter and the two passes.  With PPI_BATCH_GRAPH it is
// captured once into a CUDA graph and replayed.  PPI_BATCH_AUTOTUNE sizes
// the main pass's rows from a first evaluation's row histogram, then times
// both block shapes (64 or 128 threads per CTA) and keeps the faster; it
// changes speed only, never a result.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "ppi_internal.cuh"

namespace ppi {
namespace {

// Cost buckets: [0, 64) programs of the main pass, [64, 128) of the wide pass.
constexpr int kBuckets = 128;

// Exclusive offsets of the cost buckets (one thread): the main pass's
// programs first, each pass largest bucket first; *n_main = main-pass items.
__global__ void batch_scan_kernel(const unsigned* count, unsigned* cursor, unsigned* n_main) {
   if (blockIdx.x == 0 && threadIdx.x == 0) {
      unsigned off = 0;
      for (int b = 63; b >= 0; --b) {
         cursor[b] = off;
         off += count[b];
      }
      *n_main = off;
      for (int b = 127; b >= 64; --b) {
         cursor[b] = off;
         off += count[b];
      }
   }
}

__global__ void batch_scatter_kernel(const unsigned char* bucket_of, unsigned* cursor, int* order,
                                     int total) {
   const int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i >= total) return;
   const unsigned pos = atomicAdd(&cursor[bucket_of[i]], 1u);
   order[pos] = i;
}

}  // namespace

cudaError_t launch_batch_order(const unsigned* bucket_count, unsigned* cursor,
                               const unsigned char* bucket_of, int* order, int total,
                               unsigned* n_main, cudaStream_t s) {
   batch_scan_kernel<<<1, 32, 0, s>>>(bucket_count, cursor, n_main);
   cudaError_t e = cudaGetLastError();
   if (e != cudaSuccess) return e;
   batch_scatter_kernel<<<std::max(1, (total + 255) / 256), 256, 0, s>>>(bucket_of, cursor, order, total);
   return cudaGetLastError();
}

}  // namespace ppi

using namespace ppi;

// Launch shape of the two passes.
struct BatchGeo {
   int block = 128;
   int rows = 1, grid = 1, per_sm = 1;
   int fit = 1;                        // most rows any tile can have
   size_t smem = 0;
   int rows_wide = 1, grid_wide = 1, per_sm_wide = 1;
   size_t smem_wide = 0;
   bool wide = false;
   int wide_kernel = 1;                // 2: every population PP or PDP (whole-quad direct reads)
   int main_kernel = 0;                // kMainHi: the main pass's 64-register build
                                       //   (both + kOneLane when a population has one lane)
};

struct ppi_batch {
   int device = 0, sm_count = 0, math = 0, max_size = 0, opset = kOpsetFull;
   int n_pops = 0, total = 0, code_stride = 0;
   std::string err;
   std::vector<PopDesc> host_pops;
   std::vector<float*> datasets;
   std::vector<float*> costs;
   int2* d_lut = nullptr;
   int lut_min = 0, lut_len = 0;
   PopDesc* d_pops = nullptr;
   int* d_pop_of = nullptr;
   int* d_order = nullptr;
   unsigned char* d_bucket_of = nullptr;
   unsigned* d_bucket = nullptr;       // [0, kBuckets): counts, [kBuckets, 2 kBuckets): cursors
   unsigned* d_n_main = nullptr;
   unsigned long long* d_pop_key = nullptr;
   unsigned* d_pop_done = nullptr;
   int32_t* d_best = nullptr;
   DevStats* d_stats = nullptr;
   unsigned long long* d_key = nullptr;
   int* d_status = nullptr;
   int32_t* d_ph = nullptr;
   float* d_eph = nullptr;
   int32_t* d_size = nullptr;
   float* d_fit = nullptr;
   uint2* d_code = nullptr;
   int2* d_meta = nullptr;
   uint2* d_work = nullptr;
   float* h_fit = nullptr;
   int32_t* h_best = nullptr;
   int* h_status = nullptr;
   ProgramUpload upload;   // host programs in compact form (upload.cu)
   cudaStream_t stream = nullptr;
   cudaEvent_t ev0 = nullptr, ev1 = nullptr;
   // geometry
   BatchGeo geo;
   int max_ncol = 1, max_lanes_unaligned = 0;
   bool tuned = false;
   float tune_ms[2] = {0.0f, 0.0f};
   // graph of one step, keyed by the buffers it was captured with
   cudaGraphExec_t graph = nullptr;
   const void* graph_key[6] = {};
   cudaStream_t graph_stream = nullptr;
   float last_ms = 0.0f;
   int last_launches = 0;   // kernels of the last step
};

namespace {

ppi_status bfail(ppi_batch* b, ppi_status s, const std::string& m) {
   if (b) b->err = m;
   return s;
}

#define PPI_BCUDA(b, call)                                                                  \
   do {                                                                                     \
      cudaError_t e_ = (call);                                                              \
      if (e_ != cudaSuccess)                                                                \
         return bfail((b), e_ == cudaErrorMemoryAllocation ? PPI_ERR_OUT_OF_MEMORY : PPI_ERR_CUDA, \
                      std::string(#call) + ": " + cudaGetErrorString(e_));                  \
   } while (0)

template <class T>
cudaError_t balloc(T** p, size_t count) {
   *p = nullptr;
   return cudaMalloc(reinterpret_cast<void**>(p), std::max<size_t>(count, 1) * sizeof(T));
}

void bfree_all(ppi_batch* b) {
   if (b->graph) cudaGraphExecDestroy(b->graph);
   for (float* p : b->datasets) cudaFree(p);
   for (float* p : b->costs) cudaFree(p);
   cudaFree(b->d_lut); cudaFree(b->d_pops); cudaFree(b->d_pop_of); cudaFree(b->d_order);
   cudaFree(b->d_bucket_of); cudaFree(b->d_bucket); cudaFree(b->d_pop_key); cudaFree(b->d_pop_done);
   cudaFree(b->d_best); cudaFree(b->d_stats); cudaFree(b->d_key); cudaFree(b->d_status);
   cudaFree(b->d_n_main);
   cudaFree(b->d_ph); cudaFree(b->d_eph); cudaFree(b->d_size); cudaFree(b->d_fit);
   cudaFree(b->d_code); cudaFree(b->d_meta); cudaFree(b->d_work);
   cudaFreeHost(b->h_fit); cudaFreeHost(b->h_best); cudaFreeHost(b->h_status);
   free_upload(&b->upload);
   if (b->ev0) cudaEventDestroy(b->ev0);
   if (b->ev1) cudaEventDestroy(b->ev1);
   if (b->stream) cudaStreamDestroy(b->stream);
}

// Geometry for block size P.  Main pass (programs whose columns all fit, on
// the kernel without direct reads): rows_req rows when > 0 (clamped to what
// fits), else the most rows at the occupancy of a one-row tile.  Wide pass
// (the rest, on the kernel with direct column reads): the most rows at its
// own top occupancy, and at least room for the deepest slot need and the
// target.
ppi_status batch_geometry(ppi_batch* b, int P, int rows_req, BatchGeo* g, int rows_wide_req = 0) {
   for (const PopDesc& p : b->host_pops)
      if (p.strategy == PPI_STRATEGY_DP && p.lanes > P * kR)
         return bfail(b, PPI_ERR_UNSUPPORTED, "DP lanes larger than the tile");
   constexpr size_t kSmemCap = 200 * 1024;
   const size_t T = (size_t)P * kR;
   // lane buffers of the populations that do not accumulate in registers
   int lanes_extra = 0;
   for (const PopDesc& p : b->host_pops)
      if (!(p.strategy == PPI_STRATEGY_PDP && p.lanes == (int)T)) lanes_extra = std::max(lanes_extra, p.lanes);
   auto smem_for = [&](int rows) {
      return evaluate_smem_bytes(b->code_stride, rows, P, kR, lanes_extra, lanes_extra == 0);
   };
   const size_t fixed = smem_for(1) - T * 4;
   if (fixed + T * 4 > kSmemCap) return bfail(b, PPI_ERR_UNSUPPORTED, "tile does not fit in shared memory");
   const int rows_max = max_program_rows(b->max_ncol);
   const int fit = (int)std::min<size_t>(rows_max, (kSmemCap - fixed) / (T * 4));
   // a population with one lane (PP, or PDP over one lane): the kernels
   // with the one-lane chain run the whole batch
   int one = 0;
   for (const PopDesc& p : b->host_pops)
      if (p.strategy != PPI_STRATEGY_DP && p.lanes == 1) one = kOneLane;
   auto occupancy = [&](int direct, int rows) {
      int per_sm = 0;
      if (evaluate_batch_occupancy(b->math, b->opset, direct | one, P, smem_for(rows), &per_sm) != cudaSuccess)
         return 0;
      return per_sm;
   };
   // the main pass's kernel at a row count: the 64-register build where it
   // lets more CTAs fit than the 80-register one
   auto main_kernel_for = [&](int rows) { return occupancy(kMainHi, rows) > occupancy(0, rows) ? kMainHi : 0; };
   auto occ_main = [&](int rows) { return occupancy(main_kernel_for(rows), rows); };
   auto best_rows = [&](int direct) {
      auto occ = [&](int r) { return direct == 0 ? occ_main(r) : occupancy(direct, r); };
      const int top = occ(1);
      int rows = 1;
      while (rows < fit && occ(rows + 1) >= top) ++rows;
      return rows;
   };
   // whole-quad direct reads need every tile to start on a multiple of 4
   // records: DP tiles advance by lanes * dp_tile_groups(lanes, T) records
   int wk = 2;
   for (const PopDesc& p : b->host_pops)
      if (p.strategy == PPI_STRATEGY_DP && (p.lanes * dp_tile_groups(p.lanes, (int)T)) % 4 != 0) wk = 1;
   if (occupancy(0, 1) < 1 || occupancy(wk, 1) < 1)
      return bfail(b, PPI_ERR_UNSUPPORTED, "evaluator does not fit on an SM");
   int rows = best_rows(0);
   if (rows_req > 0) rows = std::min(rows_req, fit);
   // wide pass: rows_wide_req when > 0 (the autotuner's candidates), else the
   // most rows at its top occupancy and room for the deepest slot need
   const int rows2 = rows_wide_req > 0 ? std::min(rows_wide_req, fit)
                                       : std::max(best_rows(wk), std::min(fit, kSlots + 1));
   g->block = P;
   g->fit = fit;
   g->rows = rows;
   g->smem = smem_for(rows);
   g->main_kernel = main_kernel_for(rows);
   g->per_sm = occupancy(g->main_kernel, rows);
   g->main_kernel |= one;
   if (g->per_sm < 1) return bfail(b, PPI_ERR_UNSUPPORTED, "tile does not fit on an SM");
   g->grid = std::max(1, std::min(b->total, g->per_sm * b->sm_count));
   g->rows_wide = rows2;
   g->smem_wide = smem_for(rows2);
   g->per_sm_wide = occupancy(wk, rows2);
   g->grid_wide = std::max(1, std::min(b->total, std::max(1, g->per_sm_wide) * b->sm_count));
   g->wide = rows < rows_max;
   g->wide_kernel = wk | one;
   return PPI_OK;
}

ppi_status enqueue_step(ppi_batch* b, const int32_t* ph, const float* eph, const int32_t* size,
                        float* fit, int32_t* best, cudaStream_t s, const BatchGeo& g) {
   PPI_BCUDA(b, cudaMemsetAsync(b->d_stats, 0, sizeof(DevStats), s));
   PPI_BCUDA(b, cudaMemsetAsync(b->d_bucket, 0, 2 * kBuckets * sizeof(unsigned), s));
   PPI_BCUDA(b, cudaMemsetAsync(b->d_pop_key, 0xFF, b->n_pops * sizeof(unsigned long long), s));
   PPI_BCUDA(b, cudaMemsetAsync(b->d_pop_done, 0, b->n_pops * sizeof(unsigned), s));
   TranslateArgs t{};
   t.phenotype = ph; t.ephemeral = eph; t.size = size; t.n = b->total; t.max_size = b->max_size;
   t.ncol = 1; t.nlin = 1; t.lut = b->d_lut; t.lut_min = b->lut_min; t.lut_len = b->lut_len;
   t.code = b->d_code; t.code_stride = b->code_stride; t.meta = b->d_meta; t.work = b->d_work;
   t.best_key = b->d_key; t.stats = b->d_stats; t.status = b->d_status;
   t.prot = -1; t.fold = 1;   // ncol, records and prot come from each program's population
   t.rows_main = g.rows; t.rows_wide = g.rows_wide;
   t.pop_of = b->d_pop_of; t.pops = b->d_pops; t.bucket_count = b->d_bucket; t.bucket_of = b->d_bucket_of;
   PPI_BCUDA(b, launch_translate(b->math, t, s));
   PPI_BCUDA(b, launch_batch_order(b->d_bucket, b->d_bucket + kBuckets, b->d_bucket_of, b->d_order,
                                   b->total, b->d_n_main, s));
   BatchArgs a{};
   a.pops = b->d_pops; a.pop_of = b->d_pop_of; a.order = b->d_order; a.total = b->total;
   a.code = b->d_code; a.code_stride = b->code_stride; a.meta = b->d_meta; a.size = size;
   a.fitness = fit; a.pop_key = b->d_pop_key; a.pop_done = b->d_pop_done; a.best_index = best;
   a.stats = b->d_stats; a.n_main = b->d_n_main; a.status = b->d_status;
   a.rows = g.rows; a.wide_pass = 0;
   PPI_BCUDA(b, launch_evaluate_batch(b->math, b->opset, g.main_kernel, a, g.block, g.grid, g.smem, s));
   b->last_launches = 4;   // translate, order scan, order scatter, main pass
   if (g.wide) {
      a.rows = g.rows_wide; a.wide_pass = 1;
      PPI_BCUDA(b, launch_evaluate_batch(b->math, b->opset, g.wide_kernel, a, g.block, g.grid_wide, g.smem_wide, s));
      b->last_launches = 5;
   }
   return PPI_OK;
}

// Candidate main-pass row budgets for block size P: the most rows at each of
// the three best occupancy levels (CTAs per SM).  More rows per CTA lowers
// occupancy but keeps more programs out of the wide pass.
std::vector<int> row_levels(ppi_batch* b, int P) {
   std::vector<int> out;
   BatchGeo g;
   if (batch_geometry(b, P, 0, &g) != PPI_OK) return out;
   int prev_occ = -1;
   for (int rows = 1; rows <= g.fit + 1 && (int)out.size() < 3; ++rows) {
      BatchGeo t;
      const bool ok = rows <= g.fit && batch_geometry(b, P, rows, &t) == PPI_OK;
      const int occ = ok ? t.per_sm : 0;
      if (rows > 1 && occ != prev_occ) out.push_back(rows - 1);
      if (!ok) break;
      prev_occ = occ;
   }
   return out;
}

// Wide-pass row budgets for a shape: the most rows at each of the three best
// occupancy levels of the wide pass (fewer rows stage fewer columns and read
// more directly, but let more CTAs run).
std::vector<int> wide_row_levels(ppi_batch* b, const BatchGeo& base) {
   std::vector<int> out;
   int prev_occ = -1;
   for (int rows = 1; rows <= base.fit + 1 && (int)out.size() < 3; ++rows) {
      BatchGeo t;
      const bool ok = rows <= base.fit && batch_geometry(b, base.block, base.rows, &t, rows) == PPI_OK;
      const int occ = ok ? t.per_sm_wide : 0;
      if (rows > 1 && occ != prev_occ) out.push_back(rows - 1);
      if (!ok) break;
      prev_occ = occ;
   }
   return out;
}

// Time the candidate shapes once on these inputs (twice when a step is
// short) and keep the fastest: for 128-thread CTAs every occupancy level's
// most rows, for 64-thread CTAs the level with the same shared memory per
// warp as the best 128-thread shape; then, for the shape kept, the wide
// pass's row budget at each of its best occupancy levels.
ppi_status autotune(ppi_batch* b, const int32_t* ph, const float* eph, const int32_t* size, float* fit,
                    int32_t* best, cudaStream_t s) {
   auto time_once = [&](const BatchGeo& g, float* ms) -> ppi_status {
      PPI_BCUDA(b, cudaEventRecord(b->ev0, s));
      ppi_status st = enqueue_step(b, ph, eph, size, fit, best, s, g);
      if (st != PPI_OK) return st;
      PPI_BCUDA(b, cudaEventRecord(b->ev1, s));
      PPI_BCUDA(b, cudaEventSynchronize(b->ev1));
      PPI_BCUDA(b, cudaEventElapsedTime(ms, b->ev0, b->ev1));
      return PPI_OK;
   };
   // candidates: 128-thread CTAs at the most rows of each of the best
   // occupancy levels, then 64-thread CTAs with twice the rows of the best
   // 128-thread shape (the same shared memory per warp)
   std::vector<BatchGeo> cand;
   for (int r : row_levels(b, 128)) {
      BatchGeo g;
      if (batch_geometry(b, 128, r, &g) == PPI_OK) cand.push_back(g);
   }
   if (cand.empty()) return bfail(b, PPI_ERR_UNSUPPORTED, "no block shape fits this batch");
   // Each candidate is timed in two round-robin rounds after one warm step,
   // and keeps its faster time: a single timing in a fixed order favoured the
   // later shapes while the clocks were still rising.
   std::vector<float> best_of(cand.size(), -1.0f);
   auto rounds = [&](size_t from) -> ppi_status {
      for (size_t c = from; c < cand.size(); ++c) {
         float ms;
         ppi_status st = enqueue_step(b, ph, eph, size, fit, best, s, cand[c]);   // warm
         if (st != PPI_OK) return st;
         if ((st = time_once(cand[c], &ms)) != PPI_OK) return st;
         best_of[c] = ms;
      }
      for (size_t c = from; c < cand.size(); ++c) {
         float ms;
         ppi_status st = time_once(cand[c], &ms);
         if (st != PPI_OK) return st;
         best_of[c] = std::min(best_of[c], ms);
      }
      return PPI_OK;
   };
   ppi_status st = rounds(0);
   if (st != PPI_OK) return st;
   size_t pick = 0;
   for (size_t c = 1; c < cand.size(); ++c)
      if (best_of[c] < best_of[pick]) pick = c;
   b->tune_ms[1] = best_of[pick];
   b->tune_ms[0] = -1.0f;
   BatchGeo g64;
   if (batch_geometry(b, 64, 2 * cand[pick].rows, &g64) == PPI_OK) {
      cand.push_back(g64);
      best_of.push_back(-1.0f);
      if ((st = rounds(cand.size() - 1)) != PPI_OK) return st;
      b->tune_ms[0] = best_of.back();
      if (best_of.back() < best_of[pick]) pick = cand.size() - 1;
   }
   if (cand[pick].wide) {
      const size_t from = cand.size();
      const BatchGeo kept = cand[pick];
      for (int r2 : wide_row_levels(b, kept)) {
         BatchGeo g;
         if (r2 == kept.rows_wide || batch_geometry(b, kept.block, kept.rows, &g, r2) != PPI_OK) continue;
         cand.push_back(g);
         best_of.push_back(-1.0f);
      }
      if (cand.size() > from) {
         if ((st = rounds(from)) != PPI_OK) return st;
         for (size_t c = from; c < cand.size(); ++c)
            if (best_of[c] < best_of[pick]) pick = c;
      }
   }
   b->geo = cand[pick];
   b->tuned = true;
   return PPI_OK;
}

}  // namespace

extern "C" {

ppi_status ppi_batch_create(const ppi_gpu_config* c, int32_t n_pops, const ppi_batch_population* pops,
                            ppi_batch** out) {
   if (!c || !pops || !out || n_pops < 1 || c->max_size < 1 || c->max_size > 65535 || c->math < 0 ||
       c->math > 2 || c->n_symbols < 0 || (c->n_symbols > 0 && !c->symbols) ||
       (c->best_rule != PPI_BEST_ACCELERATOR && c->best_rule != PPI_BEST_SEQUENTIAL))
      return PPI_ERR_INVALID_ARGUMENT;
   *out = nullptr;
   long long total = 0;
   for (int p = 0; p < n_pops; ++p) {
      const ppi_batch_population& q = pops[p];
      if (!q.rows || q.nlin < 1 || q.ncol < 1 || q.ncol > kMaxColumns || q.n < 1 || q.strategy < 0 || q.strategy > 2 ||
          q.error_fn < 0 || q.error_fn > 3 || q.lanes > kMaxLanes ||
          (q.error_fn == PPI_EF_COST && (!q.cost || q.cost_n < 1 || q.cost_n > 4096)))
         return PPI_ERR_INVALID_ARGUMENT;
      total += q.n;
   }
   if (total > (1 << 30)) return PPI_ERR_UNSUPPORTED;
   ppi_batch* b = new ppi_batch();
   auto bail = [&](ppi_status s) { bfree_all(b); delete b; return s; };
   int ndev = 0;
   if (cudaGetDeviceCount(&ndev) != cudaSuccess || c->device < 0 || c->device >= ndev) return bail(PPI_ERR_CUDA);
   if (cudaSetDevice(c->device) != cudaSuccess) return bail(PPI_ERR_CUDA);
   b->device = c->device;
   cudaDeviceGetAttribute(&b->sm_count, cudaDevAttrMultiProcessorCount, c->device);
   b->math = c->math;
   b->max_size = c->max_size;
   b->code_stride = 2 * c->max_size + 2;
   b->n_pops = n_pops;
   b->total = (int)total;
   b->opset = opset_for(c->symbols, c->n_symbols);
   if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess ||
       cudaEventCreate(&b->ev0) != cudaSuccess || cudaEventCreate(&b->ev1) != cudaSuccess)
      return bail(PPI_ERR_CUDA);
   // symbol table (as ppi_gpu_create)
   int mn = 0, mx = -1;
   for (int i = 0; i < c->n_symbols; ++i) {
      if (c->symbols[i].op < 0 || c->symbols[i].op >= PPI_OP_COUNT) return bail(PPI_ERR_INVALID_ARGUMENT);
      if (i == 0 || c->symbols[i].symbol < mn) mn = c->symbols[i].symbol;
      if (i == 0 || c->symbols[i].symbol > mx) mx = c->symbols[i].symbol;
   }
   if (c->n_symbols > 0 && (long long)mx - mn + 1 > (1 << 22)) return bail(PPI_ERR_UNSUPPORTED);
   std::vector<int2> lut(c->n_symbols > 0 ? (size_t)(mx - mn + 1) : 1, make_int2(PPI_OP_INVALID, 0x7fc00000));
   for (int i = 0; i < c->n_symbols; ++i) {
      int32_t bits;
      std::memcpy(&bits, &c->symbols[i].value, 4);
      lut[(size_t)(c->symbols[i].symbol - mn)] = make_int2(c->symbols[i].op, bits);
   }
   b->lut_min = mn;
   b->lut_len = c->n_symbols > 0 ? mx - mn + 1 : 0;
   if (balloc(&b->d_lut, lut.size()) != cudaSuccess ||
       cudaMemcpy(b->d_lut, lut.data(), lut.size() * sizeof(int2), cudaMemcpyHostToDevice) != cudaSuccess)
      return bail(PPI_ERR_OUT_OF_MEMORY);
   // datasets (column-major, padded) and population descriptors
   std::vector<int> pop_of((size_t)total);
   int begin = 0;
   for (int p = 0; p < n_pops; ++p) {
      const ppi_batch_population& q = pops[p];
      const int ld = (q.nlin + kColumnPad - 1) / kColumnPad * kColumnPad;
      std::vector<float> cm((size_t)ld * q.ncol, 0.0f);
      for (int i = 0; i < q.nlin; ++i)
         for (int k = 0; k < q.ncol; ++k) cm[(size_t)k * ld + i] = q.rows[(size_t)i * q.ncol + k];
      float* d = nullptr;
      if (balloc(&d, cm.size()) != cudaSuccess) return bail(PPI_ERR_OUT_OF_MEMORY);
      b->datasets.push_back(d);
      if (cudaMemcpy(d, cm.data(), cm.size() * 4, cudaMemcpyHostToDevice) != cudaSuccess) return bail(PPI_ERR_CUDA);
      float* dc = nullptr;
      if (q.error_fn == PPI_EF_COST) {
         if (balloc(&dc, (size_t)q.cost_n * q.cost_n) != cudaSuccess) return bail(PPI_ERR_OUT_OF_MEMORY);
         b->costs.push_back(dc);
         if (cudaMemcpy(dc, q.cost, (size_t)q.cost_n * q.cost_n * 4, cudaMemcpyHostToDevice) != cudaSuccess)
            return bail(PPI_ERR_CUDA);
      }
      b->max_ncol = std::max(b->max_ncol, q.ncol);
      PopDesc pd{};
      pd.data = d; pd.nlin = q.nlin; pd.ncol = q.ncol; pd.ld = ld;
      pd.strategy = q.strategy; pd.lanes = resolve_lanes(q.strategy, q.lanes, q.nlin, b->sm_count);
      pd.ef = q.error_fn; pd.reduce_max = q.reduce_max ? 1 : 0; pd.prot = q.protected_fns ? 1 : 0;
      pd.cost = dc; pd.cost_n = q.error_fn == PPI_EF_COST ? q.cost_n : 0; pd.alpha = 0.0f;
      pd.prog_begin = begin; pd.n = q.n;
      if (pd.lanes < 1 || pd.lanes > kMaxLanes) return bail(PPI_ERR_UNSUPPORTED);
      // each population is one acc_interpret call: its own best_individual geometry
      if (best_geometry(c->best_rule, resolve_best_group(c->best_rule, c->best_group, q.n, b->sm_count),
                        q.strategy, q.n, &pd.best))
         return bail(PPI_ERR_UNSUPPORTED);
      b->host_pops.push_back(pd);
      for (int i = 0; i < q.n; ++i) pop_of[(size_t)begin + i] = p;
      begin += q.n;
   }
   const size_t T = (size_t)b->total, ms = (size_t)c->max_size;
   if (balloc(&b->d_pops, n_pops) != cudaSuccess || balloc(&b->d_pop_of, T) != cudaSuccess ||
       balloc(&b->d_order, T) != cudaSuccess || balloc(&b->d_bucket_of, T) != cudaSuccess ||
       balloc(&b->d_bucket, 2 * kBuckets) != cudaSuccess || balloc(&b->d_n_main, 1) != cudaSuccess ||
       balloc(&b->d_pop_key, n_pops) != cudaSuccess ||
       balloc(&b->d_pop_done, n_pops) != cudaSuccess || balloc(&b->d_best, n_pops) != cudaSuccess ||
       balloc(&b->d_stats, 1) != cudaSuccess || balloc(&b->d_key, 1) != cudaSuccess ||
       balloc(&b->d_status, 1) != cudaSuccess || balloc(&b->d_ph, T * ms) != cudaSuccess ||
       balloc(&b->d_eph, T * ms) != cudaSuccess || balloc(&b->d_size, T) != cudaSuccess ||
       balloc(&b->d_fit, T) != cudaSuccess || balloc(&b->d_code, T * b->code_stride) != cudaSuccess ||
       balloc(&b->d_meta, T) != cudaSuccess || balloc(&b->d_work, T * 2 * ms) != cudaSuccess ||
       cudaMallocHost(reinterpret_cast<void**>(&b->h_fit), T * 4) != cudaSuccess ||
       cudaMallocHost(reinterpret_cast<void**>(&b->h_best), (size_t)n_pops * 4) != cudaSuccess ||
       cudaMallocHost(reinterpret_cast<void**>(&b->h_status), 4) != cudaSuccess)
      return bail(PPI_ERR_OUT_OF_MEMORY);
   if (cudaMemcpy(b->d_pops, b->host_pops.data(), n_pops * sizeof(PopDesc), cudaMemcpyHostToDevice) != cudaSuccess ||
       cudaMemcpy(b->d_pop_of, pop_of.data(), T * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess)
      return bail(PPI_ERR_CUDA);
   // default shape until tuned: 128 threads if it fits, else 64
   if (batch_geometry(b, 128, 0, &b->geo) != PPI_OK && batch_geometry(b, 64, 0, &b->geo) != PPI_OK)
      return bail(PPI_ERR_UNSUPPORTED);
   *out = b;
   return PPI_OK;
}

ppi_status ppi_batch_destroy(ppi_batch* b) {
   if (!b) return PPI_ERR_INVALID_ARGUMENT;
   cudaSetDevice(b->device);
   if (b->stream) cudaStreamSynchronize(b->stream);
   bfree_all(b);
   delete b;
   return PPI_OK;
}

const char* ppi_batch_last_error(const ppi_batch* b) { return b ? b->err.c_str() : "null handle"; }

ppi_status ppi_batch_set_alpha(ppi_batch* b, const float* alpha) {
   if (!b || !alpha) return PPI_ERR_INVALID_ARGUMENT;
   PPI_BCUDA(b, cudaSetDevice(b->device));
   for (int p = 0; p < b->n_pops; ++p) b->host_pops[p].alpha = alpha[p];
   PPI_BCUDA(b, cudaMemcpy(b->d_pops, b->host_pops.data(), b->n_pops * sizeof(PopDesc), cudaMemcpyHostToDevice));
   return PPI_OK;
}

ppi_status ppi_batch_evaluate_device(ppi_batch* b, const int32_t* d_ph, const float* d_eph,
                                     const int32_t* d_size, float* d_fit, int32_t* d_best,
                                     void* stream, int32_t flags) {
   if (!b || !d_ph || !d_eph || !d_size || !d_fit || !d_best) return PPI_ERR_INVALID_ARGUMENT;
   PPI_BCUDA(b, cudaSetDevice(b->device));
   cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
   if ((flags & PPI_BATCH_AUTOTUNE) && !b->tuned) {
      ppi_status st = autotune(b, d_ph, d_eph, d_size, d_fit, d_best, s);
      if (st != PPI_OK) return st;
   }
   const bool use_graph = (flags & PPI_BATCH_GRAPH) && s != nullptr;
   if (!use_graph) {
      PPI_BCUDA(b, cudaEventRecord(b->ev0, s));
      ppi_status st = enqueue_step(b, d_ph, d_eph, d_size, d_fit, d_best, s, b->geo);
      if (st != PPI_OK) return st;
      PPI_BCUDA(b, cudaEventRecord(b->ev1, s));
      return PPI_OK;
   }
   const void* key[6] = {d_ph, d_eph, d_size, d_fit, d_best,
                         reinterpret_cast<void*>((size_t)b->geo.block << 16 | (size_t)b->geo.rows)};
   if (!b->graph || std::memcmp(key, b->graph_key, sizeof key) != 0 || b->graph_stream != s) {
      if (b->graph) {
         cudaGraphExecDestroy(b->graph);
         b->graph = nullptr;
      }
      cudaGraph_t g = nullptr;
      PPI_BCUDA(b, cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
      ppi_status st = enqueue_step(b, d_ph, d_eph, d_size, d_fit, d_best, s, b->geo);
      cudaError_t ce = cudaStreamEndCapture(s, &g);
      if (st != PPI_OK) {
         if (g) cudaGraphDestroy(g);
         return st;
      }
      PPI_BCUDA(b, ce);
      ce = cudaGraphInstantiate(&b->graph, g, 0);
      cudaGraphDestroy(g);
      PPI_BCUDA(b, ce);
      std::memcpy(b->graph_key, key, sizeof key);
      b->graph_stream = s;
   }
   PPI_BCUDA(b, cudaEventRecord(b->ev0, s));
   PPI_BCUDA(b, cudaGraphLaunch(b->graph, s));
   PPI_BCUDA(b, cudaEventRecord(b->ev1, s));
   return PPI_OK;
}

ppi_status ppi_batch_evaluate(ppi_batch* b, const int32_t* ph, const float* eph, const int32_t* size,
                              float* fitness, int32_t* best_index, int32_t flags) {
   if (!b || !ph || !eph || !size || !fitness) return PPI_ERR_INVALID_ARGUMENT;
   PPI_BCUDA(b, cudaSetDevice(b->device));
   const size_t T = (size_t)b->total;
   PPI_BCUDA(b, upload_programs(&b->upload, ph, eph, size, b->total, b->max_size, b->d_ph, b->d_eph,
                                b->d_size, b->sm_count, b->stream));
   ppi_status st = ppi_batch_evaluate_device(b, b->d_ph, b->d_eph, b->d_size, b->d_fit, b->d_best,
                                             b->stream, flags);
   if (st != PPI_OK) return st;
   PPI_BCUDA(b, cudaMemcpyAsync(b->h_fit, b->d_fit, T * 4, cudaMemcpyDeviceToHost, b->stream));
   PPI_BCUDA(b, cudaMemcpyAsync(b->h_best, b->d_best, (size_t)b->n_pops * 4, cudaMemcpyDeviceToHost, b->stream));
   PPI_BCUDA(b, cudaMemcpyAsync(b->h_status, b->d_status, 4, cudaMemcpyDeviceToHost, b->stream));
   PPI_BCUDA(b, cudaStreamSynchronize(b->stream));
   std::memcpy(fitness, b->h_fit, T * 4);
   if (best_index) std::memcpy(best_index, b->h_best, (size_t)b->n_pops * 4);
   cudaEventElapsedTime(&b->last_ms, b->ev0, b->ev1);
   if (*b->h_status & kStatusStageTimeout)
      return bfail(b, PPI_ERR_DEVICE_STATUS, "a tile copy did not complete (bounded wait expired)");
   if (*b->h_status & kStatusBadInstruction)
      return bfail(b, PPI_ERR_DEVICE_STATUS, "a kernel met an instruction outside its opcode set");
   if (*b->h_status & kStatusUnsupportedProgram)
      return bfail(b, PPI_ERR_UNSUPPORTED, "a malformed program needs a deeper stack than supported");
   return PPI_OK;
}

ppi_status ppi_batch_last_kernel_ms(ppi_batch* b, float* ms) {
   if (!b || !ms) return PPI_ERR_INVALID_ARGUMENT;
   PPI_BCUDA(b, cudaEventSynchronize(b->ev1));
   PPI_BCUDA(b, cudaEventElapsedTime(ms, b->ev0, b->ev1));
   return PPI_OK;
}

ppi_status ppi_batch_last_launch_count(const ppi_batch* b, int32_t* n) {
   if (!b || !n) return PPI_ERR_INVALID_ARGUMENT;
   *n = b->last_launches;
   return PPI_OK;
}

ppi_status ppi_batch_set_shape(ppi_batch* b, int32_t block, int32_t rows) {
   if (!b || (block != 64 && block != 128) || rows < 0) return PPI_ERR_INVALID_ARGUMENT;
   PPI_BCUDA(b, cudaSetDevice(b->device));
   BatchGeo g;
   ppi_status st = batch_geometry(b, block, rows, &g);
   if (st != PPI_OK) return st;
   b->geo = g;
   b->tuned = true;   // a fixed shape is not re-tuned
   return PPI_OK;
}

ppi_status ppi_batch_shape(const ppi_batch* b, int32_t* block, int32_t* grid, int32_t* rows,
                           float* tune_ms) {
   if (!b || !block || !grid) return PPI_ERR_INVALID_ARGUMENT;
   *block = b->geo.block;
   *grid = b->geo.grid;
   if (rows) {
      rows[0] = b->geo.rows;
      rows[1] = b->geo.wide ? b->geo.rows_wide : b->geo.rows;
   }
   if (tune_ms) {
      tune_ms[0] = b->tune_ms[0];
      tune_ms[1] = b->tune_ms[1];
   }
   return PPI_OK;
}

}  // extern "C"
