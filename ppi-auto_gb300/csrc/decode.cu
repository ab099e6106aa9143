// decode.cu -- genome -> program decoding on the device, one thread per
// genome.  Restates decode_rule / decode_real / decode of src/ppi.cc:106-182
// with an explicit frame stack in place of the recursion:
//  * a codon is bg bits, least significant first, and selects alternative
//    (value % number of alternatives) of the current non-terminal; a codon
//    is consumed even when the non-terminal has one alternative (:110-121);
//  * a constant is bc bits, least significant first, mapped to [lo, hi] with
//    float(v) * (hi - lo) in float, then the division by (2^bc - 1) and the
//    addition in double (:124-137); when fewer than bc bits remain it is 0
//    and no bit is consumed;
//  * the program is invalid (size 0) when a codon is needed and fewer than
//    bg bits remain, or when a non-terminal is entered at pos >= max_size
//    (:141-146).  The reference stores a terminal that follows another symbol
//    of the same alternative without checking pos, so it can write past
//    max_size (into the next program's row); such a genome is invalid here.
#include <algorithm>

#include "ppi_decode.cuh"

namespace ppi {
namespace {

__device__ __forceinline__ int decode_rule(const DecodeArgs& a, const uint8_t* g, int& allele, int nt) {
   if (allele + a.bg > a.nb) return -1;
   unsigned v = 0;
   for (int i = 0; i < a.bg; ++i)
      if (g[allele++]) v += (1u << i);
   return a.t.rule_first[nt] + (int)(v % (unsigned)a.t.rule_count[nt]);
}

__device__ __forceinline__ float decode_real(const DecodeArgs& a, const uint8_t* g, int& allele) {
   if (allele + a.bc > a.nb) return 0.0f;
   unsigned long long v = 0;
   for (int i = 0; i < a.bc; ++i)
      if (g[allele++]) v += (1ull << i);
   const float num = (float)v * (a.hi - a.lo);
   return (float)((double)a.lo + (double)num / ((double)(1ull << a.bc) - 1.0));
}

__global__ void decode_kernel(const DecodeArgs a) {
   const int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i >= a.n) return;
   const uint8_t* g = a.genomes + (size_t)i * a.nb;
   int32_t* ph = a.phenotype + (size_t)i * a.max_size;
   float* eph = a.ephemeral + (size_t)i * a.max_size;
   uint32_t* fr = a.frames + (size_t)i * a.frames_cap;
   int allele = 0, pos = 0, fp = 0;
   bool ok = true;
   // enter the start symbol (NT_INICIAL = 0)
   int r = decode_rule(a, g, allele, 0);
   if (r < 0 || pos >= a.max_size) ok = false;
   else fr[fp++] = (uint32_t)r << 8;
   while (ok && fp > 0) {
      const uint32_t f = fr[fp - 1];
      const int alt = (int)(f >> 8), k = (int)(f & 0xFFu);
      if (k >= a.t.alt_len[alt]) { --fp; continue; }
      fr[fp - 1] = f + 1u;
      const int s = a.t.alt_syms[(size_t)alt * a.t.max_rule + k];
      if (s >= 10000) {
         if (pos >= a.max_size) { ok = false; break; }
         int32_t sym = s;
         float e = 0.0f;
         if (s == a.t.t_const) e = decode_real(a, g, allele);
         else if (s >= 20000) { sym = a.t.t_attribute; e = (float)(s - 20000); }
         ph[pos] = sym;
         eph[pos] = e;
         ++pos;
      } else {
         r = decode_rule(a, g, allele, s);
         if (r < 0 || pos >= a.max_size || fp >= a.frames_cap) { ok = false; break; }
         fr[fp++] = (uint32_t)r << 8;
      }
   }
   a.size[i] = ok ? pos : 0;
}

}  // namespace

cudaError_t upload_decode_tables(DecodeTables* t, const int32_t* rule_first, const int32_t* rule_count,
                                 int n_nt, const int32_t* alt_len, const int32_t* alt_syms, int n_alt,
                                 int max_rule, int t_const, int t_attribute) {
   cudaError_t e;
   if ((e = cudaMalloc(&t->rule_first, n_nt * 4)) != cudaSuccess) return e;
   if ((e = cudaMalloc(&t->rule_count, n_nt * 4)) != cudaSuccess) return e;
   if ((e = cudaMalloc(&t->alt_len, n_alt * 4)) != cudaSuccess) return e;
   if ((e = cudaMalloc(&t->alt_syms, (size_t)n_alt * max_rule * 4)) != cudaSuccess) return e;
   if ((e = cudaMemcpy(t->rule_first, rule_first, n_nt * 4, cudaMemcpyHostToDevice)) != cudaSuccess) return e;
   if ((e = cudaMemcpy(t->rule_count, rule_count, n_nt * 4, cudaMemcpyHostToDevice)) != cudaSuccess) return e;
   if ((e = cudaMemcpy(t->alt_len, alt_len, n_alt * 4, cudaMemcpyHostToDevice)) != cudaSuccess) return e;
   if ((e = cudaMemcpy(t->alt_syms, alt_syms, (size_t)n_alt * max_rule * 4, cudaMemcpyHostToDevice)) != cudaSuccess)
      return e;
   t->n_nt = n_nt;
   t->n_alt = n_alt;
   t->max_rule = max_rule;
   t->t_const = t_const;
   t->t_attribute = t_attribute;
   t->ready = true;
   return cudaSuccess;
}

void free_decode_tables(DecodeTables* t) {
   cudaFree(t->rule_first);
   cudaFree(t->rule_count);
   cudaFree(t->alt_len);
   cudaFree(t->alt_syms);
   *t = DecodeTables{};
}

cudaError_t launch_decode(const DecodeArgs& a, cudaStream_t s) {
   const int block = 128;
   decode_kernel<<<std::max(1, (a.n + block - 1) / block), block, 0, s>>>(a);
   return cudaGetLastError();
}

}  // namespace ppi
