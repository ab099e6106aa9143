// ppi_gpu_api.cu -- host implementation of the C ABI in include/ppi_gpu.h.
//
// State that the reference keeps in one process-global struct
// (src/interpreter/accelerator.cc:56) lives in a handle here.  One generation
// is: three H2D copies (phenotype, ephemeral, size, as accelerator.cc:668-684),
// the translator kernel, the evaluator kernel (fitness, alpha*size and arg-min
// fused), and one D2H copy of fitness + best index into pinned staging.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "ppi_internal.cuh"
#include "ppi_decode.cuh"

using namespace ppi;

namespace ppi {
// PPI's CSV reader (dataset_csv.cu): 0, or 1 / 2 with the reference's message.
int read_csv(const char* path, std::vector<float>* colmajor, int pad, int* rows, int* cols,
             std::string* msg);
}

struct ppi_gpu {
   ppi_gpu_config cfg{};
   std::vector<float> cost;
   std::string err;
   int device = 0, sm_count = 0;
   cudaStream_t stream = nullptr;
   cudaEvent_t ev0 = nullptr, ev1 = nullptr, evm = nullptr;
   // symbol lookup
   int2* d_lut = nullptr;
   int lut_min = 0, lut_len = 0;
   float* d_cost = nullptr;
   // dataset
   float* d_data = nullptr;
   int nlin = 0, ncol = 0, ld = 0;
   bool have_data = false;
   int lanes = 1;
   int opset = kOpsetFull;
   int best_group = 1;         // work-group size of the best-index rule
   Geometry geo;
   // per-generation buffers (capacity population_size)
   int32_t* d_ph = nullptr;
   float* d_eph = nullptr;
   int32_t* d_size = nullptr;
   uint2* d_code = nullptr;
   int code_stride = 0;
   int2* d_meta = nullptr;
   uint2* d_work = nullptr;
   float* d_fit = nullptr;
   unsigned long long* d_key = nullptr;
   DevStats* d_stats = nullptr;
   int* d_wide = nullptr;
   // chunked evaluation (Geometry::chunked): lane state and finished-chunk
   // counters, one per program
   float* d_chunk_state = nullptr;
   unsigned* d_chunk_done = nullptr;
   size_t chunk_cap = 0;
   int32_t* d_best = nullptr;
   int* d_status = nullptr;
   float* d_pred = nullptr;
   // pinned staging of the outputs
   float* h_fit = nullptr;
   int32_t* h_best = nullptr;
   int* h_status = nullptr;
   // pending split call
   bool pending = false;
   int pending_n = 0;
   float* out_fit = nullptr;
   int32_t* out_best = nullptr;
   // device decode
   DecodeTables dec{};
   uint8_t* d_genomes = nullptr;
   size_t genome_cap = 0;
   uint32_t* d_frames = nullptr;
   size_t frames_cap = 0;
   float last_ms = 0.0f;
   int last_launches = 0;
   int last_n = 0;                 // programs of the last translation
   // constant adjoint (allocated on first use)
   uint2* d_adj_code = nullptr;
   int2* d_adj_meta = nullptr;
   float* d_grad = nullptr;
   int* d_adj_stats = nullptr;   // max rows, max constants, work queues of the occupancy levels
   int* h_adj_stats = nullptr;
   int* d_adj_order = nullptr;
   double* d_adj_psum = nullptr;   // per program and chunk: the constants' sums
   int* d_adj_pbad = nullptr;
   ProgramUpload upload;   // host programs in compact form (upload.cu)
   size_t adj_chunk_cap = 0;       // program x chunk entries allocated
   std::vector<int2> h_adj_meta;
   std::vector<int> h_adj_order;
};

namespace {

ppi_status fail(ppi_gpu* h, ppi_status s, const std::string& msg) {
   if (h) h->err = msg;
   return s;
}

#define PPI_CUDA(h, call)                                                                   \
   do {                                                                                     \
      cudaError_t e_ = (call);                                                              \
      if (e_ != cudaSuccess)                                                                \
         return fail((h), e_ == cudaErrorMemoryAllocation ? PPI_ERR_OUT_OF_MEMORY : PPI_ERR_CUDA, \
                     std::string(#call) + ": " + cudaGetErrorString(e_));                   \
   } while (0)

template <class T>
cudaError_t dalloc(T** p, size_t count) {
   *p = nullptr;
   if (count == 0) count = 1;
   return cudaMalloc(reinterpret_cast<void**>(p), count * sizeof(T));
}

void free_all(ppi_gpu* h) {
   cudaFree(h->d_lut); cudaFree(h->d_cost); cudaFree(h->d_data);
   cudaFree(h->d_ph); cudaFree(h->d_eph); cudaFree(h->d_size); cudaFree(h->d_code);
   cudaFree(h->d_meta); cudaFree(h->d_work); cudaFree(h->d_fit); cudaFree(h->d_key);
   cudaFree(h->d_stats); cudaFree(h->d_wide); cudaFree(h->d_best); cudaFree(h->d_status); cudaFree(h->d_pred);
   cudaFree(h->d_chunk_state); cudaFree(h->d_chunk_done);
   cudaFree(h->d_genomes); cudaFree(h->d_frames);
   free_decode_tables(&h->dec);
   cudaFreeHost(h->h_fit); cudaFreeHost(h->h_best); cudaFreeHost(h->h_status);
   cudaFree(h->d_adj_code); cudaFree(h->d_adj_meta); cudaFree(h->d_grad); cudaFree(h->d_adj_stats);
   cudaFree(h->d_adj_order); cudaFree(h->d_adj_psum); cudaFree(h->d_adj_pbad);
   cudaFreeHost(h->h_adj_stats);
   free_upload(&h->upload);
   if (h->ev0) cudaEventDestroy(h->ev0);
   if (h->ev1) cudaEventDestroy(h->ev1);
   if (h->evm) cudaEventDestroy(h->evm);
   if (h->stream) cudaStreamDestroy(h->stream);
}

// Evaluator geometry for the current dataset and lane count.
ppi_status plan(ppi_gpu* h) {
   Geometry g;
   const char* why = plan_geometry(h->cfg.strategy, h->lanes, h->cfg.math, h->opset, h->nlin,
                                   h->ncol, h->code_stride, h->cfg.population_size, h->sm_count, &g,
                                   true);
   if (why) return fail(h, PPI_ERR_UNSUPPORTED, why);
   if (g.chunked) {
      // each program's lane state between chunks: R + 1 floats per thread
      const size_t per = (size_t)(g.R + 1) * g.block, pop = (size_t)h->cfg.population_size;
      if (pop * per > h->chunk_cap) {
         PPI_CUDA(h, cudaSetDevice(h->device));
         cudaFree(h->d_chunk_state);
         cudaFree(h->d_chunk_done);
         h->d_chunk_state = nullptr;
         h->d_chunk_done = nullptr;
         h->chunk_cap = 0;
         PPI_CUDA(h, dalloc(&h->d_chunk_state, pop * per));
         PPI_CUDA(h, dalloc(&h->d_chunk_done, pop));
         h->chunk_cap = pop * per;
      }
   }
   h->geo = g;
   return PPI_OK;
}

// Status word of the last kernels, as a ppi_status and message.
ppi_status device_status(ppi_gpu* h, int bits) {
   if (bits & kStatusStageTimeout)
      return fail(h, PPI_ERR_DEVICE_STATUS, "a tile copy did not complete (bounded wait expired)");
   if (bits & kStatusBadInstruction)
      return fail(h, PPI_ERR_DEVICE_STATUS, "a kernel met an instruction outside its opcode set");
   if (bits & kStatusChunkWait)
      return fail(h, PPI_ERR_DEVICE_STATUS, "a record chunk's predecessor did not finish (bounded wait expired)");
   if (bits & kStatusUnsupportedProgram)
      return fail(h, PPI_ERR_UNSUPPORTED,
                  "a malformed program needs a deeper stack than the generic interpreter's");
   return PPI_OK;
}

// Upload of a column-major, ld-padded dataset and the geometry that follows
// from it.
ppi_status install_dataset(ppi_gpu* h, const std::vector<float>& cm, int nlin, int ncol, int ld) {
   PPI_CUDA(h, cudaSetDevice(h->device));
   cudaFree(h->d_data);
   h->d_data = nullptr;
   h->have_data = false;
   PPI_CUDA(h, dalloc(&h->d_data, cm.size()));
   PPI_CUDA(h, cudaMemcpy(h->d_data, cm.data(), cm.size() * sizeof(float), cudaMemcpyHostToDevice));
   cudaFree(h->d_pred);
   h->d_pred = nullptr;
   PPI_CUDA(h, dalloc(&h->d_pred, (size_t)nlin));
   h->nlin = nlin;
   h->ncol = ncol;
   h->ld = ld;
   const int L = resolve_lanes(h->cfg.strategy, h->cfg.lanes, nlin, h->sm_count);
   if (L < 1 || L > kMaxLanes) return fail(h, PPI_ERR_UNSUPPORTED, "lane count out of range");
   h->lanes = L;
   ppi_status s = plan(h);
   if (s != PPI_OK) return s;
   h->have_data = true;
   return PPI_OK;
}

ppi_status check_ready(ppi_gpu* h, int n) {
   if (!h) return PPI_ERR_INVALID_ARGUMENT;
   if (!h->have_data) return fail(h, PPI_ERR_NOT_READY, "no dataset: call ppi_gpu_set_dataset first");
   if (h->pending) return fail(h, PPI_ERR_NOT_READY, "an evaluate_launch is still pending");
   if (n < 1 || n > h->cfg.population_size)
      return fail(h, PPI_ERR_INVALID_ARGUMENT, "n must be in [1, population_size]");
   return PPI_OK;
}

ppi_status enqueue(ppi_gpu* h, const int32_t* d_ph, const float* d_eph, const int32_t* d_size,
                   int n, float alpha, float* d_fit, int32_t* d_best, cudaStream_t s) {
   const Geometry& g = h->geo;
   TranslateArgs t{};
   t.phenotype = d_ph; t.ephemeral = d_eph; t.size = d_size; t.n = n;
   t.max_size = h->cfg.max_size; t.ncol = h->ncol; t.nlin = h->nlin;
   t.lut = h->d_lut; t.lut_min = h->lut_min; t.lut_len = h->lut_len;
   t.code = h->d_code; t.code_stride = h->code_stride; t.meta = h->d_meta; t.work = h->d_work;
   t.best_key = h->d_key; t.stats = h->d_stats; t.status = h->d_status;
   t.prot = h->cfg.protected_fns ? 1 : 0; t.fold = 1;
   t.rows_main = g.rows; t.rows_wide = g.rows_wide; t.wide_list = h->d_wide;
   EvalArgs e{};
   e.data = h->d_data; e.nlin = h->nlin; e.ncol = h->ncol; e.ld = h->ld;
   e.code = h->d_code; e.code_stride = h->code_stride; e.meta = h->d_meta; e.size = d_size;
   e.n = n; e.alpha = alpha; e.ef = h->cfg.error_fn; e.reduce_max = h->cfg.reduce_max ? 1 : 0;
   e.prot = h->cfg.protected_fns ? 1 : 0; e.cost = h->d_cost; e.cost_n = h->cfg.cost_n;
   e.strategy = h->cfg.strategy; e.lanes = h->lanes; e.fitness = d_fit; e.best_key = h->d_key;
   e.stats = h->d_stats; e.best_index = d_best; e.status = h->d_status;
   e.wide_list = h->d_wide;
   e.chunk_records = g.chunk_records; e.n_chunks = g.n_chunks; e.chunk_group = g.chunk_group;
   e.chunk_state = h->d_chunk_state; e.chunk_done = h->d_chunk_done;
   if (const char* why = best_geometry(h->cfg.best_rule, h->best_group, h->cfg.strategy, n, &e.best))
      return fail(h, PPI_ERR_UNSUPPORTED, why);
   // work items: programs, or (program, record chunk) pairs
   const int work = (int)std::min<long long>((long long)n * g.n_chunks, 1LL << 30);
   PPI_CUDA(h, cudaEventRecord(h->ev0, s));
   PPI_CUDA(h, cudaMemsetAsync(h->d_stats, 0, sizeof(DevStats), s));
   if (g.chunked) PPI_CUDA(h, cudaMemsetAsync(h->d_chunk_done, 0, (size_t)n * sizeof(unsigned), s));
   PPI_CUDA(h, launch_translate(h->cfg.math, t, s));
   h->last_n = n;
   PPI_CUDA(h, cudaEventRecord(h->evm, s));
   e.rows = g.rows; e.wide_pass = 0; e.final_pass = g.wide ? 0 : 1;
   PPI_CUDA(h, launch_evaluate(h->cfg.math, g.opset, g.main_kernel, e, g.block, std::min(g.grid, work), g.smem, s));
   h->last_launches = 2;
   if (g.wide) {
      e.rows = g.rows_wide; e.wide_pass = 1; e.final_pass = 1;
      PPI_CUDA(h, launch_evaluate(h->cfg.math, g.opset, g.wide_kernel, e, g.block, std::min(g.grid_wide, work),
                                  g.smem_wide, s));
      h->last_launches = 3;
   }
   PPI_CUDA(h, cudaEventRecord(h->ev1, s));
   return PPI_OK;
}

}  // namespace

extern "C" {

const char* ppi_gpu_version(void) { return "ppi_gpu 2 sm_103a"; }

const char* ppi_gpu_last_error(const ppi_gpu* h) { return h ? h->err.c_str() : "null handle"; }

ppi_status ppi_gpu_create(const ppi_gpu_config* c, ppi_gpu** out) {
   if (!c || !out) return PPI_ERR_INVALID_ARGUMENT;
   *out = nullptr;
   if (c->max_size < 1 || c->max_size > 65535 || c->population_size < 1 ||
       c->strategy < 0 || c->strategy > 2 || c->error_fn < 0 || c->error_fn > 3 || c->math < 0 ||
       c->math > 2 || c->lanes > kMaxLanes || c->n_symbols < 0 ||
       (c->n_symbols > 0 && !c->symbols) ||
       (c->best_rule != PPI_BEST_ACCELERATOR && c->best_rule != PPI_BEST_SEQUENTIAL))
      return PPI_ERR_INVALID_ARGUMENT;
   if (c->error_fn == PPI_EF_COST && (!c->cost || c->cost_n < 1 || c->cost_n > 4096))
      return PPI_ERR_INVALID_ARGUMENT;
   ppi_gpu* h = new ppi_gpu();
   h->cfg = *c;
   h->cfg.symbols = nullptr;
   h->cfg.cost = nullptr;
   h->device = c->device;
   auto bail = [&](ppi_status s) { free_all(h); delete h; return s; };
   int ndev = 0;
   if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) return bail(PPI_ERR_CUDA);
   if (c->device < 0 || c->device >= ndev) return bail(PPI_ERR_INVALID_ARGUMENT);
   if (cudaSetDevice(c->device) != cudaSuccess) return bail(PPI_ERR_CUDA);
   cudaDeviceGetAttribute(&h->sm_count, cudaDevAttrMultiProcessorCount, c->device);
   h->best_group = resolve_best_group(c->best_rule, c->best_group, c->population_size, h->sm_count);
   if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess ||
       cudaEventCreate(&h->ev0) != cudaSuccess || cudaEventCreate(&h->ev1) != cudaSuccess || cudaEventCreate(&h->evm) != cudaSuccess)
      return bail(PPI_ERR_CUDA);
   // Symbol -> op table, dense over [min symbol, max symbol].
   int mn = 0, mx = -1;
   for (int i = 0; i < c->n_symbols; ++i) {
      if (c->symbols[i].op < 0 || c->symbols[i].op >= PPI_OP_COUNT) return bail(PPI_ERR_INVALID_ARGUMENT);
      if (i == 0 || c->symbols[i].symbol < mn) mn = c->symbols[i].symbol;
      if (i == 0 || c->symbols[i].symbol > mx) mx = c->symbols[i].symbol;
   }
   if (c->n_symbols > 0 && (long long)mx - mn + 1 > (1 << 22)) return bail(PPI_ERR_UNSUPPORTED);
   std::vector<int2> lut(c->n_symbols > 0 ? (size_t)(mx - mn + 1) : 1,
                         make_int2(PPI_OP_INVALID, 0x7fc00000));
   for (int i = 0; i < c->n_symbols; ++i) {
      int32_t bits;
      std::memcpy(&bits, &c->symbols[i].value, 4);
      lut[(size_t)(c->symbols[i].symbol - mn)] = make_int2(c->symbols[i].op, bits);
   }
   h->opset = opset_for(c->symbols, c->n_symbols);
   h->lut_min = mn;
   h->lut_len = c->n_symbols > 0 ? mx - mn + 1 : 0;
   const size_t pop = (size_t)c->population_size, ms = (size_t)c->max_size;
   h->code_stride = 2 * c->max_size + 2;
   if (dalloc(&h->d_lut, lut.size()) != cudaSuccess ||
       dalloc(&h->d_ph, pop * ms) != cudaSuccess || dalloc(&h->d_eph, pop * ms) != cudaSuccess ||
       dalloc(&h->d_size, pop) != cudaSuccess ||
       dalloc(&h->d_code, pop * (size_t)h->code_stride) != cudaSuccess ||
       dalloc(&h->d_meta, pop) != cudaSuccess || dalloc(&h->d_work, pop * 2 * ms) != cudaSuccess ||
       dalloc(&h->d_fit, pop) != cudaSuccess || dalloc(&h->d_key, 1) != cudaSuccess ||
       dalloc(&h->d_stats, 1) != cudaSuccess || dalloc(&h->d_wide, pop) != cudaSuccess ||
       dalloc(&h->d_best, 1) != cudaSuccess || dalloc(&h->d_status, 1) != cudaSuccess ||
       cudaMallocHost(reinterpret_cast<void**>(&h->h_fit), pop * sizeof(float)) != cudaSuccess ||
       cudaMallocHost(reinterpret_cast<void**>(&h->h_best), sizeof(int32_t)) != cudaSuccess ||
       cudaMallocHost(reinterpret_cast<void**>(&h->h_status), sizeof(int)) != cudaSuccess)
      return bail(PPI_ERR_OUT_OF_MEMORY);
   if (cudaMemcpy(h->d_lut, lut.data(), lut.size() * sizeof(int2), cudaMemcpyHostToDevice) != cudaSuccess)
      return bail(PPI_ERR_CUDA);
   if (c->error_fn == PPI_EF_COST) {
      h->cost.assign(c->cost, c->cost + (size_t)c->cost_n * c->cost_n);
      if (dalloc(&h->d_cost, h->cost.size()) != cudaSuccess ||
          cudaMemcpy(h->d_cost, h->cost.data(), h->cost.size() * 4, cudaMemcpyHostToDevice) != cudaSuccess)
         return bail(PPI_ERR_OUT_OF_MEMORY);
   }
   *out = h;
   return PPI_OK;
}

ppi_status ppi_gpu_destroy(ppi_gpu* h) {
   if (!h) return PPI_ERR_INVALID_ARGUMENT;
   cudaSetDevice(h->device);
   if (h->stream) cudaStreamSynchronize(h->stream);
   free_all(h);
   delete h;
   return PPI_OK;
}

ppi_status ppi_gpu_set_dataset_rowmajor(ppi_gpu* h, const float* data, int32_t nlin, int32_t ncol) {
   if (!h || !data || nlin < 1 || ncol < 1) return fail(h, PPI_ERR_INVALID_ARGUMENT, "bad dataset");
   std::vector<const float*> rows((size_t)nlin);
   for (int i = 0; i < nlin; ++i) rows[i] = data + (size_t)i * ncol;
   return ppi_gpu_set_dataset(h, rows.data(), nlin, ncol);
}

ppi_status ppi_gpu_set_dataset(ppi_gpu* h, const float* const* rows, int32_t nlin, int32_t ncol) {
   if (!h) return PPI_ERR_INVALID_ARGUMENT;
   if (!rows || nlin < 1 || ncol < 1 || ncol > kMaxColumns)
      return fail(h, PPI_ERR_INVALID_ARGUMENT, "bad dataset");
   if (h->pending) return fail(h, PPI_ERR_NOT_READY, "an evaluate_launch is still pending");
   const int ld = (nlin + kColumnPad - 1) / kColumnPad * kColumnPad;
   // Column-major copy (the reference's -transpose layout, accelerator.cc:413-419),
   // zero-padded to a multiple of kColumnPad records.
   std::vector<float> cm((size_t)ld * ncol, 0.0f);
   for (int i = 0; i < nlin; ++i) {
      if (!rows[i]) return fail(h, PPI_ERR_INVALID_ARGUMENT, "null dataset row");
      for (int j = 0; j < ncol; ++j) cm[(size_t)j * ld + i] = rows[i][j];
   }
   return install_dataset(h, cm, nlin, ncol, ld);
}

ppi_status ppi_gpu_set_dataset_csv(ppi_gpu* h, const char* path, int32_t* nlin, int32_t* ncol) {
   if (!h) return PPI_ERR_INVALID_ARGUMENT;
   if (!path) return fail(h, PPI_ERR_INVALID_ARGUMENT, "null path");
   if (h->pending) return fail(h, PPI_ERR_NOT_READY, "an evaluate_launch is still pending");
   std::vector<float> cm;
   std::string msg;
   int rows = 0, cols = 0;
   if (read_csv(path, &cm, kColumnPad, &rows, &cols, &msg) != 0)
      return fail(h, PPI_ERR_INVALID_ARGUMENT, msg);
   if (rows < 1 || cols < 1 || cols > kMaxColumns) return fail(h, PPI_ERR_INVALID_ARGUMENT, "empty dataset");
   const ppi_status s = install_dataset(h, cm, rows, cols, (rows + kColumnPad - 1) / kColumnPad * kColumnPad);
   if (s == PPI_OK) {
      if (nlin) *nlin = rows;
      if (ncol) *ncol = cols;
   }
   return s;
}

ppi_status ppi_gpu_evaluate_launch(ppi_gpu* h, const int32_t* ph, const float* eph,
                                   const int32_t* size, int32_t n, float alpha, float* fitness,
                                   int32_t* best_index) {
   ppi_status s = check_ready(h, n);
   if (s != PPI_OK) return s;
   if (!ph || !eph || !size || !fitness) return fail(h, PPI_ERR_INVALID_ARGUMENT, "null argument");
   PPI_CUDA(h, cudaSetDevice(h->device));
   PPI_CUDA(h, upload_programs(&h->upload, ph, eph, size, n, h->cfg.max_size, h->d_ph, h->d_eph, h->d_size,
                               h->sm_count, h->stream));
   s = enqueue(h, h->d_ph, h->d_eph, h->d_size, n, alpha, h->d_fit, h->d_best, h->stream);
   if (s != PPI_OK) return s;
   PPI_CUDA(h, cudaMemcpyAsync(h->h_fit, h->d_fit, (size_t)n * 4, cudaMemcpyDeviceToHost, h->stream));
   PPI_CUDA(h, cudaMemcpyAsync(h->h_best, h->d_best, 4, cudaMemcpyDeviceToHost, h->stream));
   PPI_CUDA(h, cudaMemcpyAsync(h->h_status, h->d_status, 4, cudaMemcpyDeviceToHost, h->stream));
   h->pending = true;
   h->pending_n = n;
   h->out_fit = fitness;
   h->out_best = best_index;
   return PPI_OK;
}

ppi_status ppi_gpu_evaluate_wait(ppi_gpu* h) {
   if (!h) return PPI_ERR_INVALID_ARGUMENT;
   if (!h->pending) return fail(h, PPI_ERR_NOT_READY, "no pending evaluate_launch");
   h->pending = false;
   PPI_CUDA(h, cudaStreamSynchronize(h->stream));
   std::memcpy(h->out_fit, h->h_fit, (size_t)h->pending_n * sizeof(float));
   if (h->out_best) *h->out_best = *h->h_best;
   cudaEventElapsedTime(&h->last_ms, h->ev0, h->ev1);
   return device_status(h, *h->h_status);
}

ppi_status ppi_gpu_evaluate(ppi_gpu* h, const int32_t* ph, const float* eph, const int32_t* size,
                            int32_t n, float alpha, float* fitness, int32_t* best_index) {
   ppi_status s = ppi_gpu_evaluate_launch(h, ph, eph, size, n, alpha, fitness, best_index);
   if (s != PPI_OK) return s;
   return ppi_gpu_evaluate_wait(h);
}

ppi_status ppi_gpu_evaluate_device(ppi_gpu* h, const int32_t* d_ph, const float* d_eph,
                                   const int32_t* d_size, int32_t n, float alpha, float* d_fit,
                                   int32_t* d_best, void* stream) {
   ppi_status s = check_ready(h, n);
   if (s != PPI_OK) return s;
   if (!d_ph || !d_eph || !d_size || !d_fit || !d_best)
      return fail(h, PPI_ERR_INVALID_ARGUMENT, "null argument");
   PPI_CUDA(h, cudaSetDevice(h->device));
   return enqueue(h, d_ph, d_eph, d_size, n, alpha, d_fit, d_best,
                  reinterpret_cast<cudaStream_t>(stream));
}

ppi_status ppi_gpu_predict(ppi_gpu* h, const int32_t* ph, const float* eph, int32_t size,
                           float* out) {
   ppi_status s = check_ready(h, 1);
   if (s != PPI_OK) return s;
   if (!ph || !eph || !out || size < 0 || size > h->cfg.max_size)
      return fail(h, PPI_ERR_INVALID_ARGUMENT, "bad program");
   PPI_CUDA(h, cudaSetDevice(h->device));
   if (size > 0) {
      PPI_CUDA(h, cudaMemcpyAsync(h->d_ph, ph, (size_t)size * 4, cudaMemcpyHostToDevice, h->stream));
      PPI_CUDA(h, cudaMemcpyAsync(h->d_eph, eph, (size_t)size * 4, cudaMemcpyHostToDevice, h->stream));
   }
   PPI_CUDA(h, cudaMemcpyAsync(h->d_size, &size, 4, cudaMemcpyHostToDevice, h->stream));
   // one program: a tile with every row it can need (up to 200 KB; a
   // program needing more takes the generic form)
   const int R = kR;
   int P = 128;
   int rows = max_program_rows(h->ncol);
   while (P > 32 && evaluate_smem_bytes(h->code_stride, kSlots + 2, P, R, 0, true) > 200 * 1024) P /= 2;
   while (rows > 1 && evaluate_smem_bytes(h->code_stride, rows, P, R, 0, true) > 200 * 1024) --rows;
   const size_t smem = evaluate_smem_bytes(h->code_stride, rows, P, R, 0, true);
   if (smem > 200 * 1024) return fail(h, PPI_ERR_UNSUPPORTED, "program code too long for shared memory");
   TranslateArgs t{};
   t.phenotype = h->d_ph; t.ephemeral = h->d_eph; t.size = h->d_size; t.n = 1;
   t.max_size = h->cfg.max_size; t.ncol = h->ncol; t.nlin = h->nlin;
   t.lut = h->d_lut; t.lut_min = h->lut_min; t.lut_len = h->lut_len;
   t.code = h->d_code; t.code_stride = h->code_stride; t.meta = h->d_meta; t.work = h->d_work;
   t.best_key = h->d_key; t.stats = h->d_stats; t.status = h->d_status;
   t.prot = h->cfg.protected_fns ? 1 : 0; t.fold = 1;
   t.rows_main = rows; t.rows_wide = rows; t.wide_list = h->d_wide;
   PredictArgs p{};
   p.data = h->d_data; p.nlin = h->nlin; p.ncol = h->ncol; p.ld = h->ld;
   p.code = h->d_code; p.meta = h->d_meta; p.prot = h->cfg.protected_fns ? 1 : 0; p.out = h->d_pred;
   p.status = h->d_status;   // zeroed by the translator
   p.rows = rows;
   const int tiles = (h->nlin + P * R - 1) / (P * R);
   const int grid = std::max(1, std::min(tiles, 4 * h->sm_count));
   PPI_CUDA(h, cudaEventRecord(h->ev0, h->stream));
   PPI_CUDA(h, cudaMemsetAsync(h->d_stats, 0, sizeof(DevStats), h->stream));
   PPI_CUDA(h, launch_translate(h->cfg.math, t, h->stream));
   PPI_CUDA(h, launch_predict(h->cfg.math, h->opset, p, P, grid, smem, h->stream));
   PPI_CUDA(h, cudaEventRecord(h->ev1, h->stream));
   PPI_CUDA(h, cudaMemcpyAsync(out, h->d_pred, (size_t)h->nlin * 4, cudaMemcpyDeviceToHost, h->stream));
   PPI_CUDA(h, cudaMemcpyAsync(h->h_status, h->d_status, 4, cudaMemcpyDeviceToHost, h->stream));
   PPI_CUDA(h, cudaStreamSynchronize(h->stream));
   cudaEventElapsedTime(&h->last_ms, h->ev0, h->ev1);
   h->last_launches = 2;
   // an unsupported program predicts NaN on every record, as before
   return device_status(h, *h->h_status & (kStatusStageTimeout | kStatusBadInstruction));
}

// Adjoint launch planning: occupancy levels per R (CTAs per SM, 0 = the
// narrow fallback), the smallest level at which R = 8 is kept, and the stats
// block (max rows, constants, code words; a work queue per launch group).
constexpr int kAdjLevels = 16;
// R = 8 only at 6 or more CTAs per SM: its kernel needs 87 registers (5 CTAs
// at most), so the constant-adjoint workload (100k x 8, 10000 programs) runs
// at R = 4, measured 2.6 % faster than with R = 8 kept from 4 CTAs up.
constexpr int kAdjR8MinCtas = 6;
constexpr int kAdjMaxChunks = 32;   // record chunks (work items) per program
constexpr int kAdjStats = 3 + 2 * kAdjLevels;

ppi_status ppi_gpu_constant_gradient(ppi_gpu* h, const int32_t* ph, const float* eph,
                                     const int32_t* size, int32_t n, float* gradient) {
   ppi_status s = check_ready(h, n);
   if (s != PPI_OK) return s;
   if (!ph || !eph || !size || !gradient) return fail(h, PPI_ERR_INVALID_ARGUMENT, "null argument");
   if (h->cfg.reduce_max || (h->cfg.error_fn != PPI_EF_ABS && h->cfg.error_fn != PPI_EF_SQUARED))
      return fail(h, PPI_ERR_UNSUPPORTED,
                  "constant gradients need the sum reduction with the absolute or squared error");
   PPI_CUDA(h, cudaSetDevice(h->device));
   const size_t pop = (size_t)h->cfg.population_size, ms = (size_t)h->cfg.max_size;
   const int stride = adjoint_code_stride(h->cfg.max_size);
   if (!h->d_adj_code) {
      PPI_CUDA(h, dalloc(&h->d_adj_code, pop * stride));
      PPI_CUDA(h, dalloc(&h->d_adj_meta, pop));
      PPI_CUDA(h, dalloc(&h->d_grad, pop * ms));
      PPI_CUDA(h, dalloc(&h->d_adj_stats, kAdjStats));
      PPI_CUDA(h, cudaMallocHost(reinterpret_cast<void**>(&h->h_adj_stats), kAdjStats * sizeof(int)));
   }
   cudaStream_t st = h->stream;
   PPI_CUDA(h, cudaMemcpyAsync(h->d_ph, ph, (size_t)n * ms * 4, cudaMemcpyHostToDevice, st));
   PPI_CUDA(h, cudaMemcpyAsync(h->d_eph, eph, (size_t)n * ms * 4, cudaMemcpyHostToDevice, st));
   PPI_CUDA(h, cudaMemcpyAsync(h->d_size, size, (size_t)n * 4, cudaMemcpyHostToDevice, st));
   PPI_CUDA(h, cudaMemsetAsync(h->d_adj_stats, 0, kAdjStats * sizeof(int), st));
   PPI_CUDA(h, cudaMemsetAsync(h->d_status, 0, sizeof(int), st));
   AdjointTranslateArgs t{};
   t.phenotype = h->d_ph; t.ephemeral = h->d_eph; t.size = h->d_size; t.n = n;
   t.max_size = h->cfg.max_size; t.ncol = h->ncol;
   t.lut = h->d_lut; t.lut_min = h->lut_min; t.lut_len = h->lut_len;
   t.code = h->d_adj_code; t.code_stride = stride; t.meta = h->d_adj_meta; t.work = h->d_work;
   t.max_rows = h->d_adj_stats; t.max_consts = h->d_adj_stats + 1; t.max_code = h->d_adj_stats + 2;
   PPI_CUDA(h, launch_adjoint_translate(t, st));
   h->h_adj_meta.resize((size_t)n);
   PPI_CUDA(h, cudaMemcpyAsync(h->h_adj_stats, h->d_adj_stats, 3 * sizeof(int), cudaMemcpyDeviceToHost, st));
   PPI_CUDA(h, cudaMemcpyAsync(h->h_adj_meta.data(), h->d_adj_meta, (size_t)n * sizeof(int2),
                               cudaMemcpyDeviceToHost, st));
   PPI_CUDA(h, cudaStreamSynchronize(st));
   // Launch groups (R, L): a program runs at R = 8 records per thread when
   // that tile holds its rows (slots, kept values, columns, target) at
   // kAdjR8MinCtas or more resident CTAs per SM, else at R = 4; within an R,
   // at the occupancy level L (CTAs per SM) with the most CTAs whose tile
   // holds it.  One persistent launch per group that has programs, longest
   // programs first.  Programs too wide for a 128-thread CTA at one per SM
   // run last on narrower CTAs (level 0).
   const int rows_max = std::max(1, h->h_adj_stats[0]), nconst = std::max(1, h->h_adj_stats[1]);
   const int words = std::max(1, h->h_adj_stats[2]);
   auto occ = [&](int R, int P, int rows) {
      int per_sm = 0;
      const size_t smem = adjoint_smem_bytes(words, nconst, rows, P, R);
      if (smem > 200 * 1024 || adjoint_occupancy(h->cfg.math, h->opset, R, P, smem, &per_sm) != cudaSuccess)
         return 0;
      return per_sm;
   };
   const int P1 = 128;
   struct Levels {
      int R, top, rows[kAdjLevels];
   } lv[2] = {{8, 0, {0}}, {4, 0, {0}}};
   for (Levels& v : lv) {
      v.top = std::min(occ(v.R, P1, 1), kAdjLevels - 1);
      for (int L = v.top, r = 1; L >= 1; --L) {
         while (r < rows_max && occ(v.R, P1, r + 1) >= L) ++r;
         v.rows[L] = occ(v.R, P1, r) >= L ? r : 0;
      }
   }
   if (lv[1].top < 1) return fail(h, PPI_ERR_UNSUPPORTED, "adjoint kernel does not fit on an SM");
   int P0 = 128;
   while (P0 > 32 && occ(4, P0, rows_max) < 1) P0 /= 2;
   if (occ(4, P0, rows_max) < 1) return fail(h, PPI_ERR_UNSUPPORTED, "program too wide for shared memory");
   auto level_of = [&](const Levels& v, int rows) {
      for (int L = v.top; L >= 1; --L)
         if (rows <= v.rows[L]) return L;
      return 0;
   };
   // group index: R = 8 groups 0 .. kAdjLevels-1, R = 4 groups kAdjLevels ..
   auto group_of = [&](int rows) {
      const int L8 = level_of(lv[0], rows);
      if (L8 >= kAdjR8MinCtas) return L8;
      return kAdjLevels + level_of(lv[1], rows);
   };
   const int ngroups = 2 * kAdjLevels;
   h->h_adj_order.resize((size_t)n);
   std::vector<int> count(ngroups, 0), start(ngroups, 0), fill(ngroups, 0);
   for (int i = 0; i < n; ++i) ++count[group_of(h->h_adj_meta[i].x >> 8)];
   for (int gi = 0, o = 0; gi < ngroups; ++gi) { start[gi] = o; fill[gi] = o; o += count[gi]; }
   for (int i = 0; i < n; ++i) h->h_adj_order[fill[group_of(h->h_adj_meta[i].x >> 8)]++] = i;
   for (int gi = 0; gi < ngroups; ++gi)
      std::stable_sort(h->h_adj_order.begin() + start[gi], h->h_adj_order.begin() + start[gi] + count[gi],
                       [&](int x, int y) { return size[x] > size[y]; });
   // chunks of each program's records (work items): about 8 tiles or more
   // each, at most kAdjMaxChunks per program
   const int n_chunks = std::max(1, std::min(kAdjMaxChunks, (h->nlin + 4095) / 4096));
   const int chunk = ((h->nlin + n_chunks - 1) / n_chunks + 1023) / 1024 * 1024;
   const int chunks = (h->nlin + chunk - 1) / chunk;
   const size_t entries = (size_t)n * chunks;
   if (entries > h->adj_chunk_cap) {
      cudaFree(h->d_adj_psum);
      cudaFree(h->d_adj_pbad);
      h->d_adj_psum = nullptr;
      h->d_adj_pbad = nullptr;
      h->adj_chunk_cap = 0;
      PPI_CUDA(h, dalloc(&h->d_adj_psum, entries * kAdjMaxConsts));
      PPI_CUDA(h, dalloc(&h->d_adj_pbad, entries));
      h->adj_chunk_cap = entries;
   }
   if (!h->d_adj_order) PPI_CUDA(h, dalloc(&h->d_adj_order, pop));
   PPI_CUDA(h, cudaMemcpyAsync(h->d_adj_order, h->h_adj_order.data(), (size_t)n * sizeof(int),
                               cudaMemcpyHostToDevice, st));
   AdjointArgs a{};
   a.data = h->d_data; a.nlin = h->nlin; a.ncol = h->ncol; a.ld = h->ld;
   a.code = h->d_adj_code; a.code_stride = stride; a.code_words = words; a.meta = h->d_adj_meta;
   a.max_size = h->cfg.max_size; a.ef = h->cfg.error_fn; a.prot = h->cfg.protected_fns ? 1 : 0;
   a.max_consts = nconst; a.status = h->d_status;
   a.chunk = chunk; a.n_chunks = chunks; a.psum = h->d_adj_psum; a.pbad = h->d_adj_pbad;
   PPI_CUDA(h, cudaEventRecord(h->ev0, st));
   h->last_launches = 1;
   for (int gi = 0; gi < ngroups; ++gi) {
      if (count[gi] == 0) continue;
      const Levels& v = lv[gi < kAdjLevels ? 0 : 1];
      const int L = gi % kAdjLevels;
      const int P = L > 0 ? P1 : P0, rows = L > 0 ? v.rows[L] : rows_max;
      const int per = L > 0 ? L : occ(v.R, P0, rows_max);
      a.order = h->d_adj_order + start[gi]; a.n_items = count[gi] * chunks;
      a.queue = reinterpret_cast<unsigned*>(h->d_adj_stats + 3 + gi);
      PPI_CUDA(h, launch_adjoint(h->cfg.math, h->opset, v.R, a, P,
                                 std::max(1, std::min(a.n_items, per * h->sm_count)),
                                 adjoint_smem_bytes(words, nconst, rows, P, v.R), st));
      ++h->last_launches;
   }
   AdjointFinishArgs fa{};
   fa.code = h->d_adj_code; fa.code_stride = stride; fa.meta = h->d_adj_meta; fa.n = n;
   fa.max_size = h->cfg.max_size; fa.max_consts = nconst; fa.n_chunks = chunks;
   fa.psum = h->d_adj_psum; fa.pbad = h->d_adj_pbad; fa.grad = h->d_grad;
   PPI_CUDA(h, launch_adjoint_finish(fa, st));
   ++h->last_launches;
   PPI_CUDA(h, cudaEventRecord(h->ev1, st));
   PPI_CUDA(h, cudaMemcpyAsync(gradient, h->d_grad, (size_t)n * ms * 4, cudaMemcpyDeviceToHost, st));
   PPI_CUDA(h, cudaMemcpyAsync(h->h_status, h->d_status, sizeof(int), cudaMemcpyDeviceToHost, st));
   PPI_CUDA(h, cudaStreamSynchronize(st));
   cudaEventElapsedTime(&h->last_ms, h->ev0, h->ev1);
   return device_status(h, *h->h_status & (kStatusStageTimeout | kStatusBadInstruction));
}

ppi_status ppi_gpu_last_kernel_ms(ppi_gpu* h, float* ms) {
   if (!h || !ms) return PPI_ERR_INVALID_ARGUMENT;
   *ms = h->last_ms;
   return PPI_OK;
}

int32_t ppi_gpu_last_launch_count(const ppi_gpu* h) { return h ? h->last_launches : 0; }

ppi_status ppi_gpu_geometry(const ppi_gpu* h, int32_t* block, int32_t* rows, int32_t* n_chunks) {
   if (!h) return PPI_ERR_INVALID_ARGUMENT;
   if (!h->have_data) return PPI_ERR_NOT_READY;
   if (block) *block = h->geo.block;
   if (rows) *rows = h->geo.rows;
   if (n_chunks) *n_chunks = h->geo.n_chunks;
   return PPI_OK;
}

int32_t ppi_gpu_lanes(const ppi_gpu* h) { return (h && h->have_data) ? h->lanes : 0; }

ppi_status ppi_gpu_translation(ppi_gpu* h, int32_t n, uint32_t* code, int32_t* meta,
                               int32_t* code_stride, int32_t* opset) {
   if (!h || !code_stride || !opset) return PPI_ERR_INVALID_ARGUMENT;
   *code_stride = h->code_stride;
   *opset = h->opset;
   if (!code && !meta) return PPI_OK;
   if (n < 0 || n > h->last_n) return fail(h, PPI_ERR_INVALID_ARGUMENT, "n exceeds the last translation");
   if (n == 0) return PPI_OK;
   PPI_CUDA(h, cudaSetDevice(h->device));
   PPI_CUDA(h, cudaDeviceSynchronize());
   if (code)
      PPI_CUDA(h, cudaMemcpy(code, h->d_code, (size_t)n * h->code_stride * sizeof(uint2), cudaMemcpyDeviceToHost));
   if (meta) PPI_CUDA(h, cudaMemcpy(meta, h->d_meta, (size_t)n * sizeof(int2), cudaMemcpyDeviceToHost));
   return PPI_OK;
}

ppi_status ppi_gpu_last_stage_ms(ppi_gpu* h, float* translate_ms, float* evaluate_ms) {
   if (!h || !translate_ms || !evaluate_ms) return PPI_ERR_INVALID_ARGUMENT;
   PPI_CUDA(h, cudaEventSynchronize(h->ev1));
   PPI_CUDA(h, cudaEventElapsedTime(translate_ms, h->ev0, h->evm));
   PPI_CUDA(h, cudaEventElapsedTime(evaluate_ms, h->evm, h->ev1));
   return PPI_OK;
}

ppi_status ppi_gpu_set_grammar(ppi_gpu* h, const int32_t* rule_first, const int32_t* rule_count,
                               int32_t n_nt, const int32_t* alt_len, const int32_t* alt_syms,
                               int32_t n_alt, int32_t max_rule, int32_t t_const,
                               int32_t t_attribute) {
   if (!h) return PPI_ERR_INVALID_ARGUMENT;
   if (!rule_first || !rule_count || !alt_len || !alt_syms || n_nt < 1 || n_alt < 1 ||
       max_rule < 1)
      return fail(h, PPI_ERR_INVALID_ARGUMENT, "bad grammar tables");
   for (int i = 0; i < n_nt; ++i)
      if (rule_count[i] < 1 || rule_first[i] < 0 || rule_first[i] + rule_count[i] > n_alt)
         return fail(h, PPI_ERR_INVALID_ARGUMENT, "bad grammar tables");
   for (int a = 0; a < n_alt; ++a) {
      if (alt_len[a] < 1 || alt_len[a] > max_rule)
         return fail(h, PPI_ERR_INVALID_ARGUMENT, "bad grammar tables");
      for (int k = 0; k < alt_len[a]; ++k) {
         const int s = alt_syms[(size_t)a * max_rule + k];
         if (s < 10000 && (s < 0 || s >= n_nt))
            return fail(h, PPI_ERR_INVALID_ARGUMENT, "grammar references an undefined non-terminal");
      }
   }
   PPI_CUDA(h, cudaSetDevice(h->device));
   free_decode_tables(&h->dec);
   PPI_CUDA(h, upload_decode_tables(&h->dec, rule_first, rule_count, n_nt, alt_len, alt_syms,
                                    n_alt, max_rule, t_const, t_attribute));
   return PPI_OK;
}

static ppi_status decode_common(ppi_gpu* h, const uint8_t* genomes, int32_t n, int32_t nb,
                                int32_t bg, int32_t bc) {
   if (!h) return PPI_ERR_INVALID_ARGUMENT;
   if (!h->dec.ready) return fail(h, PPI_ERR_NOT_READY, "no grammar: call ppi_gpu_set_grammar first");
   if (h->pending) return fail(h, PPI_ERR_NOT_READY, "an evaluate_launch is still pending");
   if (!genomes || n < 1 || n > h->cfg.population_size || nb < 1 || bg < 1 || bg > 31 || bc < 1 ||
       bc > 63)
      return fail(h, PPI_ERR_INVALID_ARGUMENT, "bad decode arguments");
   PPI_CUDA(h, cudaSetDevice(h->device));
   const size_t bytes = (size_t)n * nb;
   if (bytes > h->genome_cap) {
      cudaFree(h->d_genomes);
      h->d_genomes = nullptr;
      h->genome_cap = 0;
      PPI_CUDA(h, dalloc(&h->d_genomes, bytes));
      h->genome_cap = bytes;
   }
   const size_t frames = (size_t)n * (size_t)(nb / bg + 2);
   if (frames > h->frames_cap) {
      cudaFree(h->d_frames);
      h->d_frames = nullptr;
      h->frames_cap = 0;
      PPI_CUDA(h, dalloc(&h->d_frames, frames));
      h->frames_cap = frames;
   }
   PPI_CUDA(h, cudaMemcpyAsync(h->d_genomes, genomes, bytes, cudaMemcpyHostToDevice, h->stream));
   return PPI_OK;
}

ppi_status ppi_gpu_decode(ppi_gpu* h, const uint8_t* genomes, int32_t n, int32_t nb, int32_t bg,
                          int32_t bc, float lo, float hi, int32_t* phenotype, float* ephemeral,
                          int32_t* size) {
   ppi_status s = decode_common(h, genomes, n, nb, bg, bc);
   if (s != PPI_OK) return s;
   DecodeArgs d{};
   d.t = h->dec; d.genomes = h->d_genomes; d.n = n; d.nb = nb; d.bg = bg; d.bc = bc; d.lo = lo;
   d.hi = hi; d.max_size = h->cfg.max_size; d.phenotype = h->d_ph; d.ephemeral = h->d_eph;
   d.size = h->d_size; d.frames = h->d_frames; d.frames_cap = nb / bg + 2;
   PPI_CUDA(h, cudaEventRecord(h->ev0, h->stream));
   PPI_CUDA(h, launch_decode(d, h->stream));
   PPI_CUDA(h, cudaEventRecord(h->ev1, h->stream));
   const size_t ms = (size_t)h->cfg.max_size;
   if (phenotype)
      PPI_CUDA(h, cudaMemcpyAsync(phenotype, h->d_ph, (size_t)n * ms * 4, cudaMemcpyDeviceToHost, h->stream));
   if (ephemeral)
      PPI_CUDA(h, cudaMemcpyAsync(ephemeral, h->d_eph, (size_t)n * ms * 4, cudaMemcpyDeviceToHost, h->stream));
   if (size)
      PPI_CUDA(h, cudaMemcpyAsync(size, h->d_size, (size_t)n * 4, cudaMemcpyDeviceToHost, h->stream));
   PPI_CUDA(h, cudaStreamSynchronize(h->stream));
   cudaEventElapsedTime(&h->last_ms, h->ev0, h->ev1);
   h->last_launches = 1;
   return PPI_OK;
}

ppi_status ppi_gpu_decode_evaluate(ppi_gpu* h, const uint8_t* genomes, int32_t n, int32_t nb,
                                   int32_t bg, int32_t bc, float lo, float hi, float alpha,
                                   float* fitness, int32_t* best_index, int32_t* size) {
   ppi_status s = check_ready(h, n);
   if (s != PPI_OK) return s;
   if (!fitness) return fail(h, PPI_ERR_INVALID_ARGUMENT, "null fitness");
   s = decode_common(h, genomes, n, nb, bg, bc);
   if (s != PPI_OK) return s;
   DecodeArgs d{};
   d.t = h->dec; d.genomes = h->d_genomes; d.n = n; d.nb = nb; d.bg = bg; d.bc = bc; d.lo = lo;
   d.hi = hi; d.max_size = h->cfg.max_size; d.phenotype = h->d_ph; d.ephemeral = h->d_eph;
   d.size = h->d_size; d.frames = h->d_frames; d.frames_cap = nb / bg + 2;
   PPI_CUDA(h, launch_decode(d, h->stream));
   s = enqueue(h, h->d_ph, h->d_eph, h->d_size, n, alpha, h->d_fit, h->d_best, h->stream);
   if (s != PPI_OK) return s;
   h->last_launches += 1;
   PPI_CUDA(h, cudaMemcpyAsync(h->h_fit, h->d_fit, (size_t)n * 4, cudaMemcpyDeviceToHost, h->stream));
   PPI_CUDA(h, cudaMemcpyAsync(h->h_best, h->d_best, 4, cudaMemcpyDeviceToHost, h->stream));
   PPI_CUDA(h, cudaMemcpyAsync(h->h_status, h->d_status, 4, cudaMemcpyDeviceToHost, h->stream));
   if (size)
      PPI_CUDA(h, cudaMemcpyAsync(size, h->d_size, (size_t)n * 4, cudaMemcpyDeviceToHost, h->stream));
   PPI_CUDA(h, cudaStreamSynchronize(h->stream));
   std::memcpy(fitness, h->h_fit, (size_t)n * sizeof(float));
   if (best_index) *best_index = *h->h_best;
   cudaEventElapsedTime(&h->last_ms, h->ev0, h->ev1);
   return device_status(h, *h->h_status);
}

}  // extern "C"
