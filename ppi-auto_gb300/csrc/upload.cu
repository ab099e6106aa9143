// upload.cu -- programs from host memory to the device in compact form.
//
// PPI hands the evaluator its population as rows of max_size tokens
// (phenotype) and ephemerals (ppi.cc, acc_interpret's arguments), of which a
// program uses its first size[i]: on the uneven batch 16 % of the 737 MB.
// Copying the rows as they are moves the padding too, and from PPI's own
// (pageable) arrays the CUDA driver stages every byte through a bounce buffer.
// Here the used prefixes are packed on the host into a pinned staging area
// (threads over programs for large populations), copied in one transfer,
// and scattered back into the device rows by a small kernel; the translator
// reads tokens [0, size) of each row only, so the padding is never needed.
// Rows already pinned and small in total go as they are.
#include <algorithm>
#include <cstring>
#include <thread>
#include <vector>

#include "ppi_internal.cuh"

namespace ppi {
namespace {

// Staging layout (bytes): sizes (n int32) | offsets (n int64, 8-aligned) |
// tokens (int32) | ephemerals (float), the last two `total` entries each.
size_t align8(size_t x) { return (x + 7) & ~(size_t)7; }

__global__ void expand_programs(const int32_t* __restrict__ sizes, const long long* __restrict__ off,
                                const int32_t* __restrict__ tok, const float* __restrict__ eph_c, int n,
                                int max_size, int32_t* __restrict__ d_ph, float* __restrict__ d_eph,
                                int32_t* __restrict__ d_size) {
   const int lane = threadIdx.x & 31;
   const int warps = (gridDim.x * blockDim.x) >> 5;
   for (int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < n; i += warps) {
      const int sz = sizes[i];
      if (lane == 0) d_size[i] = sz;
      const int len = (sz >= 1 && sz <= max_size) ? sz : 0;
      const long long o = off[i];
      int32_t* dp = d_ph + (size_t)i * max_size;
      float* de = d_eph + (size_t)i * max_size;
      for (int k = lane; k < len; k += 32) {
         dp[k] = tok[o + k];
         de[k] = eph_c[o + k];
      }
   }
}

}  // namespace

void free_upload(ProgramUpload* u) {
   if (u->copied) {   // the last copy out of the pinned area first
      cudaEventSynchronize(u->copied);
      cudaEventDestroy(u->copied);
      u->copied = nullptr;
   }
   cudaFreeHost(u->h_stage);
   cudaFree(u->d_stage);
   u->h_stage = nullptr;
   u->d_stage = nullptr;
   u->cap = 0;
}

static bool pinned(const void* p) {
   cudaPointerAttributes at{};
   return cudaPointerGetAttributes(&at, p) == cudaSuccess && at.type == cudaMemoryTypeHost;
}

cudaError_t upload_programs(ProgramUpload* u, const int32_t* ph, const float* eph, const int32_t* size,
                            int n, int max_size, int32_t* d_ph, float* d_eph, int32_t* d_size,
                            int sm_count, cudaStream_t s) {
   if (n < 1) return cudaSuccess;
   const size_t ms = (size_t)max_size;
   // Rows already in pinned memory, and few enough bytes that packing them on
   // the host would cost more than sending the padding (measured: 30,000
   // programs of at most 128 tokens, 1.2 ms of packing against 0.1 - 1 ms of
   // padding), go as they are.
   constexpr size_t kDirectBytes = 64u << 20;
   if ((size_t)n * ms * 8 <= kDirectBytes && pinned(ph) && pinned(eph)) {
      cudaError_t e = cudaMemcpyAsync(d_ph, ph, (size_t)n * ms * 4, cudaMemcpyHostToDevice, s);
      if (e == cudaSuccess) e = cudaMemcpyAsync(d_eph, eph, (size_t)n * ms * 4, cudaMemcpyHostToDevice, s);
      if (e == cudaSuccess) e = cudaMemcpyAsync(d_size, size, (size_t)n * 4, cudaMemcpyHostToDevice, s);
      return e;
   }
   // offsets of each program's used prefix (sizes outside [1, max_size] use none)
   std::vector<long long> off((size_t)n);
   long long total = 0;
   for (int i = 0; i < n; ++i) {
      off[i] = total;
      const int sz = size[i];
      if (sz >= 1 && sz <= max_size) total += sz;
   }
   // The host rewrites the pinned area below, outside the stream's order: a
   // copy out of it that an earlier call queued (and whose caller did not
   // wait, e.g. after a failed launch) must have finished first.
   if (u->copied) {
      const cudaError_t e = cudaEventSynchronize(u->copied);
      if (e != cudaSuccess) return e;
   }
   const size_t o_off = align8((size_t)n * 4);
   const size_t o_tok = o_off + (size_t)n * 8;
   const size_t o_eph = o_tok + align8((size_t)total * 4);
   const size_t bytes = o_eph + (size_t)total * 4;
   if (bytes > u->cap) {
      // grow with some slack, so that populations of a similar size reuse it
      free_upload(u);
      const size_t cap = bytes + bytes / 4 + 4096;
      cudaError_t e = cudaMallocHost(&u->h_stage, cap);
      if (e == cudaSuccess) e = cudaMalloc(&u->d_stage, cap);
      if (e != cudaSuccess) {
         free_upload(u);
         return e;
      }
      u->cap = cap;
   }
   if (!u->copied) {
      const cudaError_t e = cudaEventCreateWithFlags(&u->copied, cudaEventDisableTiming);
      if (e != cudaSuccess) return e;
   }
   unsigned char* hs = static_cast<unsigned char*>(u->h_stage);
   std::memcpy(hs, size, (size_t)n * 4);
   std::memcpy(hs + o_off, off.data(), (size_t)n * 8);
   int32_t* tok = reinterpret_cast<int32_t*>(hs + o_tok);
   float* ephc = reinterpret_cast<float*>(hs + o_eph);
   auto pack = [&](int i0, int i1) {
      for (int i = i0; i < i1; ++i) {
         const int sz = size[i];
         if (sz < 1 || sz > max_size) continue;
         std::memcpy(tok + off[i], ph + (size_t)i * ms, (size_t)sz * 4);
         std::memcpy(ephc + off[i], eph + (size_t)i * ms, (size_t)sz * 4);
      }
   };
   // threads for large populations (about 4 MB of tokens each), the programs
   // split at equal token counts
   const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
   const int nt = (int)std::min<long long>(std::min(hw, 16u), std::max(1LL, total / (1LL << 19)));
   if (nt <= 1) {
      pack(0, n);
   } else {
      std::vector<int> cut((size_t)nt + 1, n);
      cut[0] = 0;
      for (int t = 1; t < nt; ++t)
         cut[t] = (int)(std::lower_bound(off.begin(), off.end(), total * t / nt) - off.begin());
      std::vector<std::thread> pool;
      for (int t = 0; t < nt; ++t) pool.emplace_back(pack, cut[t], cut[t + 1]);
      for (std::thread& th : pool) th.join();
   }
   cudaError_t e = cudaMemcpyAsync(u->d_stage, u->h_stage, bytes, cudaMemcpyHostToDevice, s);
   if (e == cudaSuccess) e = cudaEventRecord(u->copied, s);
   if (e != cudaSuccess) return e;
   const unsigned char* ds = static_cast<const unsigned char*>(u->d_stage);
   const int block = 256;
   const int grid = std::max(1, std::min((n + block / 32 - 1) / (block / 32), sm_count * 8));
   expand_programs<<<grid, block, 0, s>>>(reinterpret_cast<const int32_t*>(ds),
                                          reinterpret_cast<const long long*>(ds + o_off),
                                          reinterpret_cast<const int32_t*>(ds + o_tok),
                                          reinterpret_cast<const float*>(ds + o_eph), n, max_size, d_ph,
                                          d_eph, d_size);
   return cudaGetLastError();
}

}  // namespace ppi
