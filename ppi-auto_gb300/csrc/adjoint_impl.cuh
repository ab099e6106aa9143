// adjoint_impl.cuh -- the constant adjoint's kernel (forward sweep on the
// evaluator's accumulator machine, reverse sweep with the adjoint carried in
// registers), instantiated per records-per-thread R in adjoint_r4.cu and
// adjoint_r8.cu; the translator that writes its code is adjoint.cu.
#pragma once

#include <cfloat>

#include "evaluate_impl.cuh"

namespace ppi {
namespace adj {

using ev::load_row;
using ev::store_row;
using ev::tile_pos;

constexpr int kAdjFlushRecords = 128;      // per thread, between float -> double flushes
constexpr uint32_t kRevPop = 0xFEu, kRevEnd = 0xFFu;
constexpr uint32_t kAdjImm = 0x8000u;      // operand descriptor: operand-table entry (else a row)
constexpr uint32_t kAdjNone = 0xFFFFFFFFu;

// Which operand values and which own value an opcode's adjoint reads.
__host__ __device__ constexpr bool adj_reads_v(int op) {
   return op == PPI_OP_EXP || op == PPI_OP_EXP2 || op == PPI_OP_EXP10 || op == PPI_OP_LOGISTIC ||
          op == PPI_OP_GAUSS || op == PPI_OP_SQRT || op == PPI_OP_TAN || op == PPI_OP_POW || op == PPI_OP_DIV;
}
__host__ __device__ constexpr bool adj_reads_a(int op) {
   return !(op == PPI_OP_NEG || op == PPI_OP_EXP || op == PPI_OP_EXP2 || op == PPI_OP_EXP10 ||
            op == PPI_OP_LOGISTIC || op == PPI_OP_ADD || op == PPI_OP_SUB || op == PPI_OP_MEAN ||
            op == PPI_OP_DIV);
}
__host__ __device__ constexpr bool adj_reads_b(int op) {
   return op == PPI_OP_MULT || op == PPI_OP_MAX || op == PPI_OP_MIN || op == PPI_OP_MOD ||
          op == PPI_OP_POW || op == PPI_OP_DIV;
}

// ---- per-opcode adjoints ---------------------------------------------------
// Adjoints of the operands, g x d(op)/d(first, second, third operand), at
// operands a, b, c with value v and adjoint g.  Each product is formed in an
// order that does not overflow where the partial alone would (g / b before
// x v for a division by a tiny b, g / a for log).  Piecewise-constant ops
// and the protected branches have derivative 0.
template <int OP>
__device__ __forceinline__ void adj_bp(float g, float a, float b, float c, float v, int prot, float& da,
                                       float& db, float& dc) {
   const float kLn2 = 0.693147180559945309f, kLn10 = 2.30258509299404568f;
   da = 0.0f; db = 0.0f; dc = 0.0f;
   (void)b; (void)c; (void)v; (void)prot; (void)kLn2; (void)kLn10;
   if constexpr (OP == PPI_OP_ABS) da = a > 0.0f ? g : (a < 0.0f ? -g : 0.0f);
   else if constexpr (OP == PPI_OP_POW2) da = g * (2.0f * a);
   else if constexpr (OP == PPI_OP_POW3) da = g * (3.0f * (a * a));
   else if constexpr (OP == PPI_OP_POW4) da = g * (4.0f * ((a * a) * a));
   else if constexpr (OP == PPI_OP_POW5) da = g * (5.0f * (((a * a) * a) * a));
   else if constexpr (OP == PPI_OP_NEG) da = -g;
   else if constexpr (OP == PPI_OP_EXP) da = g * v;
   else if constexpr (OP == PPI_OP_EXP2) da = (g * v) * kLn2;
   else if constexpr (OP == PPI_OP_EXP10) da = (g * v) * kLn10;
   else if constexpr (OP == PPI_OP_SIN) da = g * cosf(a);
   else if constexpr (OP == PPI_OP_COS) da = -(g * sinf(a));
   else if constexpr (OP == PPI_OP_LOGISTIC) da = (g * v) * (1.0f - v);
   else if constexpr (OP == PPI_OP_GAUSS) da = ((-2.0f * g) * a) * v;
   else if constexpr (OP == PPI_OP_GAMMA) da = __uint_as_float(0x7fc00000u);   // not differentiated
   else if constexpr (OP == PPI_OP_SQRT) da = (prot && a < 0.0f) ? 0.0f : (0.5f * g) / v;
   else if constexpr (OP == PPI_OP_LOG) da = (prot && a < 1.0f) ? 0.0f : g / a;
   else if constexpr (OP == PPI_OP_LOG2) da = (prot && a < 1.0f) ? 0.0f : (g / a) / kLn2;
   else if constexpr (OP == PPI_OP_LOG10) da = (prot && a < 1.0f) ? 0.0f : (g / a) / kLn10;
   else if constexpr (OP == PPI_OP_TAN) {
      const float fa = fabsf(a);
      da = (prot && (fa == kPi2F || fa == 3.0f * kPi2F)) ? 0.0f : g + (g * v) * v;
   }
   else if constexpr (OP == PPI_OP_ADD) { da = g; db = g; }
   else if constexpr (OP == PPI_OP_SUB) { da = g; db = -g; }
   else if constexpr (OP == PPI_OP_MULT) { da = g * b; db = g * a; }
   else if constexpr (OP == PPI_OP_MEAN) { da = 0.5f * g; db = 0.5f * g; }
   else if constexpr (OP == PPI_OP_MAX) { if (a >= b) da = g; else db = g; }
   else if constexpr (OP == PPI_OP_MIN) { if (a <= b) da = g; else db = g; }
   else if constexpr (OP == PPI_OP_MOD) { da = g; db = -(g * truncf(a / b)); }
   else if constexpr (OP == PPI_OP_POW) { da = (g * b) * (v / a); db = (g * v) * logf(a); }
   else if constexpr (OP == PPI_OP_DIV) {
      if (!(prot && b == 0.0f)) {
         const float t = g / b;
         da = t;
         db = -(t * v);
      }
   }
   // comparisons, logic, rounding, step, sign, NOT: 0
}

// ---- reverse sweep ------------------------------------------------------------
// x = an operand: a tile row, or with kAdjImm an operand-table value.
template <int R>
__device__ __forceinline__ void adj_operand(uint32_t d, const float* mine, int T, int P, const uint2* tab,
                                            float (&x)[R]) {
   if (d & kAdjImm) {
      const float k = __uint_as_float(tab[d & ~kAdjImm].x);
#pragma unroll
      for (int r = 0; r < R; ++r) x[r] = k;
   } else {
      load_row(mine + (size_t)d * T, P, x);
   }
}

template <int R>
__device__ __forceinline__ float adj_sum(const float (&d)[R]) {
   float s[R];
#pragma unroll
   for (int r = 0; r < R; ++r) s[r] = d[r];
#pragma unroll
   for (int h = R / 2; h > 0; h >>= 1)
#pragma unroll
      for (int r = 0; r < h; ++r) s[r] = s[r] + s[r + h];
   return s[0];
}

// Hand a child its adjoints: carried on (g), a stack row, or a constant's
// partial sum (this thread's float partial).
template <int R>
__device__ __forceinline__ void adj_deliver(uint32_t kind, uint32_t dst, const float (&d)[R], float (&g)[R],
                                            float* mine, int T, int P, int tid, float* s_part) {
   if (kind == 1u) {
#pragma unroll
      for (int r = 0; r < R; ++r) g[r] = d[r];
   } else if (kind == 2u) {
      store_row(mine + (size_t)dst * T, P, d);
   } else if (kind == 3u) {
      s_part[dst * P + tid] += adj_sum(d);
   }
}

// Opcode lists of the reverse sweep (as the evaluator's: FULL, or the arithmetic set).
#define ADJ_ARITH_OPS(X) X(PPI_OP_ABS) X(PPI_OP_POW2) X(PPI_OP_NEG) X(PPI_OP_EXP) X(PPI_OP_SIN) \
   X(PPI_OP_COS) X(PPI_OP_SQRT) X(PPI_OP_LOG) X(PPI_OP_ADD) X(PPI_OP_SUB) X(PPI_OP_MULT) X(PPI_OP_DIV)
// the full set minus the arithmetic one
#define ADJ_FULL_REST(X) X(PPI_OP_NOT) X(PPI_OP_POW3) X(PPI_OP_POW4) X(PPI_OP_POW5) X(PPI_OP_ROUND) \
   X(PPI_OP_CEIL) X(PPI_OP_FLOOR) X(PPI_OP_EXP10) X(PPI_OP_EXP2) X(PPI_OP_STEP) X(PPI_OP_SIGN)       \
   X(PPI_OP_LOGISTIC) X(PPI_OP_GAMMA) X(PPI_OP_GAUSS) X(PPI_OP_LOG10) X(PPI_OP_LOG2) X(PPI_OP_TAN)   \
   X(PPI_OP_AND) X(PPI_OP_OR) X(PPI_OP_XOR) X(PPI_OP_GREATER) X(PPI_OP_GREATEREQUAL) X(PPI_OP_LESS)  \
   X(PPI_OP_LESSEQUAL) X(PPI_OP_EQUAL) X(PPI_OP_NOTEQUAL) X(PPI_OP_MEAN) X(PPI_OP_MAX) X(PPI_OP_MIN) \
   X(PPI_OP_MOD) X(PPI_OP_POW)

// The sine and cosine cases' long routines (cosf, sinf of the operand) run
// rolled: the R operands rotate through one inlined copy, which keeps the
// reverse interpreter's code small (it shares the instruction cache with the
// forward one).
constexpr bool kAdjRollTrig = true;
template <int OP, int R>
__device__ __forceinline__ void adj_trig_case(const float (&g)[R], float (&x)[R], float (&d0)[R]) {
#pragma unroll 1
   for (int r = 0; r < R; ++r) {
      const float t = OP == PPI_OP_SIN ? cosf(x[0]) : sinf(x[0]);
#pragma unroll
      for (int q = 0; q < R - 1; ++q) x[q] = x[q + 1];
      x[R - 1] = t;
   }
#pragma unroll
   for (int r = 0; r < R; ++r) d0[r] = OP == PPI_OP_SIN ? g[r] * x[r] : -(g[r] * x[r]);
}

// The quotient g / a of the division and logarithm cases, rolled the same
// way (numerators and denominators rotate through one inlined IEEE
// division): the same quotients as the unrolled form, a fraction of its code.
constexpr bool kAdjRollQuotient = true;
template <int R>
__device__ __forceinline__ void adj_quotients(const float (&g)[R], const float (&a)[R], float (&q)[R]) {
   float d[R];
#pragma unroll
   for (int r = 0; r < R; ++r) { q[r] = g[r]; d[r] = a[r]; }
#pragma unroll 1
   for (int r = 0; r < R; ++r) {
      const float t = q[0] / d[0];
#pragma unroll
      for (int k = 0; k < R - 1; ++k) { q[k] = q[k + 1]; d[k] = d[k + 1]; }
      q[R - 1] = t;
   }
}

// Division and logarithm partials from the rolled quotients, as adj_bp
// forms them.
template <int OP, int R>
__device__ __forceinline__ void adj_quotient_case(const float (&g)[R], const float (&x)[R], const float (&y)[R],
                                                  const float (&v)[R], int prot, float (&d0)[R], float (&d1)[R]) {
   const float kLn2 = 0.693147180559945309f, kLn10 = 2.30258509299404568f;
   float q[R];
   if constexpr (OP == PPI_OP_DIV) adj_quotients(g, y, q);
   else adj_quotients(g, x, q);
#pragma unroll
   for (int r = 0; r < R; ++r) {
      d0[r] = 0.0f;
      d1[r] = 0.0f;
      if constexpr (OP == PPI_OP_DIV) {
         if (!(prot && y[r] == 0.0f)) { d0[r] = q[r]; d1[r] = -(q[r] * v[r]); }
      } else if (!(prot && x[r] < 1.0f)) {
         d0[r] = OP == PPI_OP_LOG ? q[r] : (OP == PPI_OP_LOG2 ? q[r] / kLn2 : q[r] / kLn10);
      }
   }
}

#define ADJ_REV_CASE(OP)                                                                  \
   case OP:                                                                               \
      if constexpr (adj_reads_a(OP)) adj_operand(i0.y & 0xFFFFu, mine, T, P, tab, x);      \
      if constexpr (adj_reads_b(OP)) adj_operand(i0.y >> 16, mine, T, P, tab, y);          \
      if constexpr (adj_reads_v(OP)) load_row(mine + (size_t)(i0.x >> 16) * T, P, v);      \
      if constexpr (kAdjRollTrig && (OP == PPI_OP_SIN || OP == PPI_OP_COS)) {              \
         adj_trig_case<OP, R>(g, x, d0);                                                   \
         _Pragma("unroll") for (int r = 0; r < R; ++r) { d1[r] = 0.0f; d2[r] = 0.0f; }     \
      } else if constexpr (kAdjRollQuotient &&                                             \
                           (OP == PPI_OP_DIV || OP == PPI_OP_LOG || OP == PPI_OP_LOG2 ||    \
                            OP == PPI_OP_LOG10)) {                                         \
         adj_quotient_case<OP, R>(g, x, y, v, prot, d0, d1);                               \
         _Pragma("unroll") for (int r = 0; r < R; ++r) d2[r] = 0.0f;                       \
      } else {                                                                             \
         _Pragma("unroll") for (int r = 0; r < R; ++r)                                    \
            adj_bp<OP>(g[r], x[r], y[r], 0.0f, v[r], prot, d0[r], d1[r], d2[r]);          \
      }                                                                                    \
      break;

template <int OPSET, int R>
__device__ __forceinline__ void adj_reverse(const uint2* __restrict__ code, float* mine, int T, int P,
                                            int tid, float (&g)[R], const uint2* tab, float* s_part,
                                            int prot) {
   uint2 i0 = code[0], i1 = code[1];
   for (int pc = 2;; pc += 2) {
      const uint32_t op = i0.x & 0xFFu;
      if (op == kRevEnd) return;
      const uint2 n0 = code[pc], n1 = code[pc + 1];   // the next instruction, early
      if (op == kRevPop) {
         load_row(mine + (size_t)i0.y * T, P, g);
         i0 = n0;
         i1 = n1;
         continue;
      }
      float x[R], y[R], v[R], d0[R], d1[R], d2[R];
#pragma unroll
      for (int r = 0; r < R; ++r) { x[r] = 0.0f; y[r] = 0.0f; v[r] = 0.0f; }
      switch (op) {
      ADJ_ARITH_OPS(ADJ_REV_CASE)
      default:
         if constexpr (OPSET == kOpsetFull) {
            switch (op) {
            ADJ_FULL_REST(ADJ_REV_CASE)
            case PPI_OP_IF_THEN_ELSE:
               adj_operand(i0.y & 0xFFFFu, mine, T, P, tab, x);
#pragma unroll
               for (int r = 0; r < R; ++r) {
                  d0[r] = 0.0f;
                  d1[r] = truthy(x[r]) ? g[r] : 0.0f;
                  d2[r] = truthy(x[r]) ? 0.0f : g[r];
               }
               break;
            default:
#pragma unroll
               for (int r = 0; r < R; ++r) { d0[r] = 0.0f; d1[r] = 0.0f; d2[r] = 0.0f; }
            }
         } else {
#pragma unroll
            for (int r = 0; r < R; ++r) { d0[r] = 0.0f; d1[r] = 0.0f; d2[r] = 0.0f; }
         }
      }
      // a zero adjoint propagates zero (never 0 x inf = NaN from an infinite
      // partial); records past the end start with a zero adjoint
#pragma unroll
      for (int r = 0; r < R; ++r)
         if (g[r] == 0.0f) { d0[r] = 0.0f; d1[r] = 0.0f; d2[r] = 0.0f; }
      const uint32_t kinds = (i0.x >> 8) & 63u;
      adj_deliver(kinds & 3u, i1.x & 0xFFFFu, d0, g, mine, T, P, tid, s_part);
      adj_deliver((kinds >> 2) & 3u, i1.x >> 16, d1, g, mine, T, P, tid, s_part);
      adj_deliver(kinds >> 4, i1.y, d2, g, mine, T, P, tid, s_part);
      i0 = n0;
      i1 = n1;
   }
}

// Register bound: 4 records per thread fit 64 registers (8 CTAs per SM where
// the tile allows, no spills in fast math), measured 1.6 % faster on the
// 100k x 8 adjoint workload than the 4-CTA bound; 8 records keep 4 CTAs.
template <int R>
constexpr int adjoint_min_ctas() { return R == 4 ? 8 : 4; }

template <int MATH, int OPSET, int R>
__global__ void __launch_bounds__(128, adjoint_min_ctas<R>()) adjoint_kernel(const AdjointArgs a) {
   extern __shared__ __align__(16) unsigned char smem_raw[];
   __shared__ int s_prog, s_bad;
   __shared__ __align__(8) uint64_t s_bar;
   if (threadIdx.x == 0) ev::stager_init(&s_bar);
   __syncthreads();
   ev::Stager st{&s_bar, 0u};
   const int P = blockDim.x, tid = threadIdx.x, T = P * R;
   uint2* s_code = reinterpret_cast<uint2*>(smem_raw);
   const int W = P / 32, lane = tid & 31, warp = tid >> 5;
   double* s_sum = reinterpret_cast<double*>(smem_raw + ev::code_bytes(a.code_words));
   float* s_part = reinterpret_cast<float*>(s_sum + (size_t)a.max_consts * W);
   float* s_tile = s_part + (size_t)a.max_consts * P;
   float* mine = s_tile + tid * 4;
   const float inv_n = 1.0f / (float)a.nlin;
   const ev::Direct none{a.data, a.ld, 0, 0};
   for (;;) {
      if (tid == 0) {
         s_prog = (int)atomicAdd(a.queue, 1u);
         s_bad = 0;
      }
      __syncthreads();
      const int item = s_prog;
      if (item >= a.n_items) break;
      // work item: one chunk of one program's records
      const int prog = a.order[item / a.n_chunks];
      const int chunk = item - (item / a.n_chunks) * a.n_chunks;
      const int2 meta = a.meta[prog];
      if ((meta.x & 0xFF) != kAdjValid) {   // size 0 or malformed: the finishing kernel's
         __syncthreads();
         continue;
      }
      const uint2* code = a.code + (size_t)prog * a.code_stride;
      // The forward bytecode [ch + 2, rev) runs on the evaluator's
      // interpreter, whose dispatch admits its own cases only: the copy
      // checks the layout (header rows inside the tile, the sections inside
      // the code, the constants inside the partial-sum rows) and each forward
      // instruction as ev::load_code does, and ends the forward code with
      // M_END at rev - 1.  A program whose layout fails is skipped (status).
      const int rows0 = meta.x >> 8;
      const uint2 h0 = code[0];
      const int ch0 = code_header((int)h0.x);
      const uint2 ah0 = ch0 + 1 < meta.y ? code[ch0] : make_uint2(0u, 0u);
      const uint2 ah1 = ch0 + 1 < meta.y ? code[ch0 + 1] : make_uint2(0u, 0u);
      const bool layout_ok = meta.y <= a.code_words && h0.x <= 0xFFFFu &&
                             (int)h0.x + (int)(h0.y & 0xFFFFu) + 1 <= rows0 &&
                             (int)ah0.x > ch0 + 2 && ah0.x < ah0.y && (int)ah0.y <= meta.y &&
                             (int)ah1.x <= a.max_consts;
      if (!layout_ok) {
         if (tid == 0) {
            atomicOr(a.status, kStatusBadInstruction);
            a.pbad[(size_t)prog * a.n_chunks + chunk] = 1;
         }
         __syncthreads();
         continue;
      }
      bool bad = false;
      for (int k = tid; k < meta.y; k += P) {
         uint2 w = code[k];
         if (k >= ch0 + 2 && k < (int)ah0.x) {
            const bool ok = k == (int)ah0.x - 1 ? w.x == (uint32_t)M_END
                                                : ev::instruction_ok<OPSET>(w, rows0, a.ncol, false);
            if (!ok) {
               w = make_uint2((uint32_t)M_END, 0u);
               bad = true;
            }
         }
         s_code[k] = w;
      }
      if (bad) atomicOr(a.status, kStatusBadInstruction);
      __syncthreads();
      const uint2 hdr = s_code[0];
      const int ch = code_header((int)hdr.x);
      const uint2 ah = s_code[ch], ah2 = s_code[ch + 1];
      const uint2* fwd = s_code + ch + 2;
      const uint2* rev = s_code + ah.x;
      const uint2* tab = s_code + ah.y;
      const int nconst = (int)ah2.x;
      const uint32_t root_slot = ah2.y;
      const int trow = (int)hdr.x + (int)(hdr.y & 0xFFFFu);
      for (int q = 0; q < nconst; ++q) {
         if (lane == 0) s_sum[q * W + warp] = 0.0;
         s_part[q * P + tid] = 0.0f;
      }
      const int first = chunk * a.chunk, end = min(a.nlin, first + a.chunk);
      int tiles = 0;
      bool stop = false;
      for (int base = first; base < end; base += T) {
         __syncthreads();   // every thread is done with the previous tile's rows
         if (!ev::stage_tile(a.data, a.ncol, a.ld, s_code, s_tile, base, T, tid, P, st, a.status)) {
            stop = true;   // the tile never arrived (status recorded)
            break;
         }
         float p[R];
         ev::run_fast<MATH, R, OPSET, 0>(fwd, mine, T, P, tid, none, p, a.prot);
         // error derivative: the root's adjoint
         float ys[R], g[R];
         load_row(mine + (size_t)trow * T, P, ys);
         bool bad = false;
#pragma unroll
         for (int r = 0; r < R; ++r) {
            const float d = p[r] - ys[r];
            g[r] = 0.0f;
            if (base + tile_pos(tid, r, P) < end) {
               const float err = a.ef == PPI_EF_SQUARED ? d * d : fabsf(d);
               if (nonfinite(err)) bad = true;
               const float de = a.ef == PPI_EF_SQUARED ? 2.0f * d : (d > 0.0f ? 1.0f : (d < 0.0f ? -1.0f : 0.0f));
               g[r] = de * inv_n;
            }
         }
         if (bad) s_bad = 1;
         if (root_slot != kAdjNone) s_part[root_slot * P + tid] += adj_sum(g);
         adj_reverse<OPSET, R>(rev, mine, T, P, tid, g, tab, s_part, a.prot);
         if (++tiles == kAdjFlushRecords / R || base + T >= end) {
            // the warp's float partials into its double sum
            for (int q = 0; q < nconst; ++q) {
               double v = (double)s_part[q * P + tid];
               s_part[q * P + tid] = 0.0f;
#pragma unroll
               for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
               if (lane == 0) s_sum[q * W + warp] += v;
            }
            tiles = 0;
         }
      }
      __syncthreads();
      // this chunk's sum per constant (warps in order), and its sentinel flag
      double* out = a.psum + ((size_t)prog * a.n_chunks + chunk) * a.max_consts;
      for (int q = tid; q < nconst; q += P) {
         double sum = 0.0;
         for (int u = 0; u < W; ++u) sum += s_sum[q * W + u];
         out[q] = sum;
      }
      if (tid == 0) a.pbad[(size_t)prog * a.n_chunks + chunk] = s_bad;
      __syncthreads();
      if (stop) break;   // staging failed: this CTA takes no more work
   }
}

template <int MATH, int R>
auto kernel_for(int opset) {
   return opset == kOpsetArith ? adjoint_kernel<MATH, kOpsetArith, R> : adjoint_kernel<MATH, kOpsetFull, R>;
}

template <int R>
void (*pick(int math, int opset))(const AdjointArgs) {
   if (math == kMathParity) return kernel_for<kMathParity, R>(opset);
   if (math == kMathNative) return kernel_for<kMathNative, R>(opset);
   return kernel_for<kMathFast, R>(opset);
}

template <int R>
cudaError_t launch(int math, int opset, const AdjointArgs& a, int block, int grid, size_t smem, cudaStream_t s) {
   auto k = pick<R>(math, opset);
   cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
   if (e != cudaSuccess) return e;
   k<<<grid, block, smem, s>>>(a);
   return cudaGetLastError();
}

template <int R>
cudaError_t occupancy(int math, int opset, int block, size_t smem, int* per_sm) {
   auto k = pick<R>(math, opset);
   cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
   if (e != cudaSuccess) return e;
   return cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, k, block, smem);
}

}  // namespace adj
}  // namespace ppi
