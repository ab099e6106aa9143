// noalloc.cu -- ppi_gpu_evaluate_noalloc: one generation evaluated without
// allocating any memory.
//
// Some callers cannot allocate device memory at the point where they evaluate
// a population.  Examples: a host application whose device memory has already
// been reserved by another allocator (a framework's caching pool), or an
// island process that must keep a fixed footprint once it is running.  Another
// is a generation loop that cannot afford the device-wide synchronisation
// cudaMalloc/cudaFree may imply.  For them this entry point runs the same
// translator and evaluator kernels as ppi_gpu_evaluate_device, on inputs and
// outputs the caller already owns.  Their scratch memory (bytecode,
// translator work area, symbol table, counters) lives in one fixed array that
// is part of the library image.
//
// That array is a file-scope __device__ object of kNoAllocScratchBytes.  Every
// GPU that loads the library holds it until the process exits.  Host code
// cannot use the array's name as a device address.  So the first call on each
// device, with that device current, looks up its address with
// cudaGetSymbolAddress and keeps it.
//
// All calls share the one array, and each call leaves its contents behind.
// The translator rewrites everything the evaluator reads and resets the
// counters, arg-min key and status word before use.  Calls whose work overlaps
// on the GPU (different streams, or different host threads) race on the array
// and must be serialised by the caller.  The kernels' status word (a program
// the generic interpreter cannot hold, a tile copy that timed out, an
// instruction outside the kernel's opcode set) is copied to the caller's
// d_status at the end of the call's work, when the caller gives one.
#include <cstdio>
#include <cmath>
#include <cstring>
#include <mutex>

#include "ppi_internal.cuh"

namespace ppi {
namespace {

constexpr size_t kNoAllocScratchBytes = (size_t)64 << 20;   // 64 MiB
constexpr int kMaxDevices = 64;
// Widest Symbol range of the dense lookup table (as ppi_gpu_create).
constexpr int kMaxSymbolRange = 1 << 22;

__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

unsigned char* g_scratch_addr[kMaxDevices] = {};
int g_sm_count[kMaxDevices] = {};
std::mutex g_scratch_mutex;

inline size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// Dense Symbol -> {op, literal} table in the scratch; for each slot the last
// matching entry wins, as in ppi_gpu_create.
__global__ void noalloc_lut_kernel(const ppi_symbol_entry* entries, int n, int lut_min, int lut_len,
                                   int2* lut) {
   const int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i >= lut_len) return;
   int2 v = make_int2(PPI_OP_INVALID, 0x7fc00000);
   for (int k = 0; k < n; ++k)
      if (entries[k].symbol == lut_min + i) v = make_int2(entries[k].op, __float_as_int(entries[k].value));
   lut[i] = v;
}

ppi_status scratch_base(int device, unsigned char** base, int* sm_count) {
   std::lock_guard<std::mutex> lock(g_scratch_mutex);
   if (!g_scratch_addr[device]) {
      void* p = nullptr;
      if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) {
         std::fprintf(stderr, "ppi_gpu_evaluate_noalloc: cudaGetSymbolAddress failed on device %d\n", device);
         return PPI_ERR_CUDA;
      }
      int sms = 0;
      if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess || sms < 1)
         return PPI_ERR_CUDA;
      g_scratch_addr[device] = static_cast<unsigned char*>(p);
      g_sm_count[device] = sms;
   }
   *base = g_scratch_addr[device];
   *sm_count = g_sm_count[device];
   return PPI_OK;
}

// Launch geometry of recent configurations.  plan_geometry asks the runtime
// for dozens of occupancies; a generation loop calls this entry point with the
// same configuration every time, so the result is kept (a pure function of
// the key) in a small table replaced round robin.
struct GeoKey {
   int device, strategy, lanes, math, opset, nlin, ncol, code_stride, n;
};
struct GeoEntry {
   GeoKey key;
   Geometry geo;
   bool used;
};
constexpr int kGeoCacheEntries = 16;
GeoEntry g_geo_cache[kGeoCacheEntries] = {};
int g_geo_next = 0;
std::mutex g_geo_mutex;

const char* cached_geometry(const GeoKey& k, int sm_count, Geometry* out) {
   {
      std::lock_guard<std::mutex> lock(g_geo_mutex);
      for (const GeoEntry& e : g_geo_cache)
         if (e.used && std::memcmp(&e.key, &k, sizeof k) == 0) {
            *out = e.geo;
            return nullptr;
         }
   }
   Geometry g;
   if (const char* why = plan_geometry(k.strategy, k.lanes, k.math, k.opset, k.nlin, k.ncol,
                                       k.code_stride, k.n, sm_count, &g))
      return why;
   std::lock_guard<std::mutex> lock(g_geo_mutex);
   g_geo_cache[g_geo_next] = GeoEntry{k, g, true};
   g_geo_next = (g_geo_next + 1) % kGeoCacheEntries;
   *out = g;
   return nullptr;
}

}  // namespace
}  // namespace ppi

using namespace ppi;

extern "C" ppi_status ppi_gpu_evaluate_noalloc(const ppi_gpu_config* c, const float* d_data,
                                               int32_t nlin, int32_t ncol, int32_t ld,
                                               const int32_t* d_phenotype, const float* d_ephemeral,
                                               const int32_t* d_size, int32_t n, float alpha,
                                               float* d_fitness, int32_t* d_best_index,
                                               int32_t* d_status, void* stream) {
   if (!c || !d_data || !d_phenotype || !d_ephemeral || !d_size || !d_fitness || !d_best_index)
      return PPI_ERR_INVALID_ARGUMENT;
   if (c->max_size < 1 || c->max_size > 65535 || c->strategy < 0 || c->strategy > 2 ||
       c->error_fn < 0 || c->error_fn > 3 || c->math < 0 || c->math > 2 || c->lanes > kMaxLanes ||
       c->n_symbols < 0 || (c->n_symbols > 0 && !c->symbols) || n < 1 || nlin < 1 || ncol < 1 || ncol > kMaxColumns ||
       ld < nlin || (ld & 3) != 0 || (reinterpret_cast<uintptr_t>(d_data) & 15) != 0 ||
       c->device < 0 || c->device >= kMaxDevices ||
       (c->best_rule != PPI_BEST_ACCELERATOR && c->best_rule != PPI_BEST_SEQUENTIAL))
      return PPI_ERR_INVALID_ARGUMENT;
   if (c->error_fn == PPI_EF_COST && (!c->cost || c->cost_n < 1 || c->cost_n > 4096))
      return PPI_ERR_INVALID_ARGUMENT;
   for (int i = 0; i < c->n_symbols; ++i)
      if (c->symbols[i].op < 0 || c->symbols[i].op >= PPI_OP_COUNT) return PPI_ERR_INVALID_ARGUMENT;
   cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);

   // Every size check comes before the first CUDA call.  Symbol range of the table, in 64 bits: a range wider than the dense
   // table allows is rejected before any offset is derived from it.
   int mn = 0, mx = -1;
   for (int i = 0; i < c->n_symbols; ++i) {
      if (i == 0 || c->symbols[i].symbol < mn) mn = c->symbols[i].symbol;
      if (i == 0 || c->symbols[i].symbol > mx) mx = c->symbols[i].symbol;
   }
   const long long range = c->n_symbols > 0 ? (long long)mx - (long long)mn + 1 : 0;
   if (range < 0 || range > kMaxSymbolRange) {
      std::fprintf(stderr,
                   "ppi_gpu_evaluate_noalloc: the symbol table spans %lld values; at most %d are "
                   "supported\n",
                   range, kMaxSymbolRange);
      return PPI_ERR_UNSUPPORTED;
   }
   const int lut_len = (int)range;

   // Scratch layout and its size limit.
   const int code_stride = 2 * c->max_size + 2;
   const size_t off_stats = 256;
   const size_t off_entries = align256(off_stats + sizeof(DevStats));
   const size_t off_lut = align256(off_entries + (size_t)c->n_symbols * sizeof(ppi_symbol_entry));
   const size_t off_cost = align256(off_lut + (size_t)lut_len * sizeof(int2));
   const size_t cost_elems = c->error_fn == PPI_EF_COST ? (size_t)c->cost_n * c->cost_n : 0;
   const size_t off_meta = align256(off_cost + cost_elems * sizeof(float));
   const size_t off_code = align256(off_meta + (size_t)n * sizeof(int2));
   const size_t off_work = align256(off_code + (size_t)n * code_stride * sizeof(uint2));
   const size_t off_wide = align256(off_work + (size_t)n * 2 * c->max_size * sizeof(uint2));
   const size_t total = align256(off_wide + (size_t)n * sizeof(int));
   if (total > kNoAllocScratchBytes) {
      std::fprintf(stderr,
                   "ppi_gpu_evaluate_noalloc: %d programs of max_size %d need %zu bytes of scratch; "
                   "the fixed scratch holds %zu bytes (evaluate the population in smaller batches)\n",
                   n, c->max_size, total, kNoAllocScratchBytes);
      return PPI_ERR_UNSUPPORTED;
   }

   if (cudaSetDevice(c->device) != cudaSuccess) return PPI_ERR_CUDA;
   unsigned char* base = nullptr;
   int sm_count = 0;
   ppi_status st = scratch_base(c->device, &base, &sm_count);
   if (st != PPI_OK) return st;

   // Geometry: the lane rule and block choice of ppi_gpu_set_dataset.
   Geometry g;
   const int L = resolve_lanes(c->strategy, c->lanes, nlin, sm_count);
   const GeoKey gk{c->device, c->strategy, L, c->math, opset_for(c->symbols, c->n_symbols),
                   nlin, ncol, code_stride, n};
   if (cached_geometry(gk, sm_count, &g)) return PPI_ERR_UNSUPPORTED;
   auto* key = reinterpret_cast<unsigned long long*>(base);
   auto* status = reinterpret_cast<int*>(base + 8);
   auto* stats = reinterpret_cast<DevStats*>(base + off_stats);
   auto* entries = reinterpret_cast<ppi_symbol_entry*>(base + off_entries);
   auto* lut = reinterpret_cast<int2*>(base + off_lut);
   auto* cost = reinterpret_cast<float*>(base + off_cost);
   auto* meta = reinterpret_cast<int2*>(base + off_meta);
   auto* code = reinterpret_cast<uint2*>(base + off_code);
   auto* work = reinterpret_cast<uint2*>(base + off_work);
   auto* wide = reinterpret_cast<int*>(base + off_wide);

   if (c->n_symbols > 0) {
      if (cudaMemcpyAsync(entries, c->symbols, (size_t)c->n_symbols * sizeof(ppi_symbol_entry),
                          cudaMemcpyHostToDevice, s) != cudaSuccess)
         return PPI_ERR_CUDA;
      noalloc_lut_kernel<<<(lut_len + 127) / 128, 128, 0, s>>>(entries, c->n_symbols, mn, lut_len, lut);
      if (cudaGetLastError() != cudaSuccess) return PPI_ERR_CUDA;
   }
   if (cost_elems &&
       cudaMemcpyAsync(cost, c->cost, cost_elems * sizeof(float), cudaMemcpyHostToDevice, s) != cudaSuccess)
      return PPI_ERR_CUDA;

   TranslateArgs t{};
   t.phenotype = d_phenotype; t.ephemeral = d_ephemeral; t.size = d_size; t.n = n;
   t.max_size = c->max_size; t.ncol = ncol; t.nlin = nlin; t.lut = lut; t.lut_min = mn; t.lut_len = lut_len;
   t.code = code; t.code_stride = code_stride; t.meta = meta; t.work = work;
   t.best_key = key; t.stats = stats; t.status = status;
   t.prot = c->protected_fns ? 1 : 0; t.fold = 1;
   t.rows_main = g.rows; t.rows_wide = g.rows_wide; t.wide_list = wide;
   EvalArgs e{};
   e.data = d_data; e.nlin = nlin; e.ncol = ncol; e.ld = ld; e.code = code;
   e.code_stride = code_stride; e.meta = meta; e.size = d_size; e.n = n; e.alpha = alpha;
   e.ef = c->error_fn; e.reduce_max = c->reduce_max ? 1 : 0; e.prot = c->protected_fns ? 1 : 0;
   e.cost = cost; e.cost_n = c->cost_n; e.strategy = c->strategy; e.lanes = g.lanes; e.fitness = d_fitness;
   e.best_key = key; e.stats = stats; e.best_index = d_best_index; e.status = status;
   e.wide_list = wide;
   if (best_geometry(c->best_rule, resolve_best_group(c->best_rule, c->best_group, n, sm_count),
                     c->strategy, n, &e.best))
      return PPI_ERR_UNSUPPORTED;
   if (cudaMemsetAsync(stats, 0, sizeof(DevStats), s) != cudaSuccess) return PPI_ERR_CUDA;
   if (launch_translate(c->math, t, s) != cudaSuccess) return PPI_ERR_CUDA;
   e.rows = g.rows; e.wide_pass = 0; e.final_pass = g.wide ? 0 : 1;
   if (launch_evaluate(c->math, g.opset, g.main_kernel, e, g.block, g.grid, g.smem, s) != cudaSuccess)
      return PPI_ERR_CUDA;
   if (g.wide) {
      e.rows = g.rows_wide; e.wide_pass = 1; e.final_pass = 1;
      if (launch_evaluate(c->math, g.opset, g.wide_kernel, e, g.block, g.grid_wide, g.smem_wide, s) != cudaSuccess)
         return PPI_ERR_CUDA;
   }
   // the kernels' status bits, for the caller to read once the stream is done
   if (d_status && cudaMemcpyAsync(d_status, status, sizeof(int32_t), cudaMemcpyDeviceToDevice, s) != cudaSuccess)
      return PPI_ERR_CUDA;
   return PPI_OK;
}
