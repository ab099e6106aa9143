// adjoint.cu -- d(fitness)/d(ephemeral constants) of every program by a
// reverse sweep over its prefix tape.  No counterpart in the reference: an
// addition for constant refinement, while the plain evaluator stays the
// fitness judge.
//
// Fitness with the sum reduction is F = (1/nlin) sum_n EF(p_n, y_n) (+ alpha
// size, constant in the ephemerals), so dF/dc = (1/nlin) sum_n EF'(p_n, y_n)
// dp_n/dc with EF' = sign(p - y) (absolute error) or 2 (p - y) (squared).
//
// Translation (one thread per program): the tokens, unfolded (constants must
// stay separate to be differentiated), become "tape code": one instruction per
// operator in the reference's evaluation order (right to left), each writing
// its value to its own tape row.  The reverse sweep visits the operators in
// prefix order (parents before children).  The adjoint of a node's first
// child is written over the node's own value row, which is dead once the node
// has been visited; the adjoints of later children wait in a small stack of
// rows (as deep as the most siblings pending at once).
//
// Evaluation (one CTA per program, persistent work queue): for each tile of
// T = P x 4 records the forward sweep is recomputed into the tape (no
// per-record tape outlives its tile), then the reverse sweep accumulates each
// constant's gradient in a per-thread float partial, added into a double sum
// every 32 tiles (few double operations, short float sums).  A thread reads and
// writes only its own 4 positions of every row, so the sweeps need no
// barriers.  Attributes and targets are read from global memory (the
// dataset stays in L2 at the sizes this serves).  Any non-finite error makes
// the fitness a sentinel value (FLT_MAX rule), whose gradient is 0.
#include <cfloat>

#include "ppi_internal.cuh"

namespace ppi {
namespace {

constexpr int kAdjR = 4;   // records per thread

// Operand descriptors: kind in bits 30-31.
enum : uint32_t { kOpdRow = 0u, kOpdAttr = 1u, kOpdConst = 2u, kOpdLiteral = 3u };
__host__ __device__ __forceinline__ uint32_t opd(uint32_t kind, uint32_t payload) { return kind << 30 | payload; }
__device__ __forceinline__ uint32_t opd_kind(uint32_t d) { return d >> 30; }
__device__ __forceinline__ uint32_t opd_val(uint32_t d) { return d & 0x3FFFFFFFu; }

// Translator scratch per token position k: w[k] = {op | sub << 16, imm};
// frames[k] = tape row of an operator; frames[max_size + k] = row that holds
// its adjoint during the reverse sweep (or, for a leaf, its table entry).
// Instruction flags: the reverse sweep visits only operators with a
// constant below them, and stores the adjoint of a first operand only when
// that operand is such an operator.
constexpr uint32_t kAdjRev = 1u << 16;     // in instruction word .x
constexpr uint32_t kAdjKeep0 = 1u << 17;   // first operand's adjoint is needed
constexpr uint32_t kAdjNoRow = 0xFFFFFFFFu;
__device__ __forceinline__ int w_op(uint2 w) { return (int)(w.x & 0xFFFFu); }
__device__ __forceinline__ int w_sub(uint2 w) { return (int)((w.x >> 16) & 0x7FFFu); }

__global__ void adjoint_translate_kernel(const AdjointTranslateArgs a) {
   const int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i >= a.n) return;
   uint4* code = a.code + (size_t)i * a.code_stride;
   const int sz = a.size[i];
   code[0] = make_uint4(0u, 0u, 0u, opd(kOpdLiteral, 0u));
   a.meta[i] = make_int2(kAdjInvalid, 0);
   if (sz <= 0 || sz > a.max_size) return;
   if (sz >= 32768) {   // subtree sizes share their word with a flag
      a.meta[i] = make_int2(kAdjUnsupported, 0);
      return;
   }
   const int32_t* ph = a.phenotype + (size_t)i * a.max_size;
   const float* eph = a.ephemeral + (size_t)i * a.max_size;
   uint2* w = a.work + (size_t)i * 2 * a.max_size;
   uint32_t* frames = reinterpret_cast<uint32_t*>(w + a.max_size);
   // ---- pass 1: ops, subtree sizes, stack discipline (right to left) ----
   int depth = 0;
   bool bad = false;
   for (int k = sz - 1; k >= 0; --k) {
      int op = PPI_OP_INVALID;
      uint32_t imm = 0x7fc00000u;
      const int li = ph[k] - a.lut_min;
      if (li >= 0 && li < a.lut_len) {
         const int2 ent = a.lut[li];
         op = ent.x;
         if (op == PPI_OP_LITERAL) imm = (uint32_t)ent.y;
         else if (op == PPI_OP_CONST) imm = __float_as_uint(eph[k]);
         else if (op == PPI_OP_ATTRIBUTE) {
            if (eph[k] >= 0.0f && eph[k] < (float)a.ncol) imm = (uint32_t)(int)eph[k];
            else { op = PPI_OP_INVALID; imm = 0x7fc00000u; }   // NaN, as the evaluator
         }
      }
      const int ar = op_arity(op);
      if (depth < ar) { bad = true; break; }
      depth = depth - ar + 1;
      int sub = 1;
      if (ar > 0) {
         const int c0 = k + 1;
         sub += w_sub(w[c0]);
         if (ar > 1) sub += w_sub(w[c0 + w_sub(w[c0])]);
         if (ar > 2) {
            const int c1 = c0 + w_sub(w[c0]);
            sub += w_sub(w[c1 + w_sub(w[c1])]);
         }
      }
      w[k] = make_uint2((uint32_t)op | ((uint32_t)sub << 16), imm);
   }
   if (bad || depth != 1 || w_sub(w[0]) != sz) {
      a.meta[i] = make_int2(kAdjUnsupported, 0);   // malformed: no gradient
      return;
   }
   // ---- tape rows (evaluation order) and the constant table ----
   int m = 0, ntab = 0, nconst = 0;
   for (int k = sz - 1; k >= 0; --k)
      if (op_arity(w_op(w[k])) > 0) frames[k] = (uint32_t)m++;
   const int ninstr = m;
   const int tab0 = 1 + 2 * ninstr;          // table entries follow the instructions
   // table entry (as uint4): {value bits, token position, gradient slot or ~0, 0}
   for (int k = 0; k < sz; ++k) {
      const int op = w_op(w[k]);
      if (op_arity(op) != 0 || op == PPI_OP_ATTRIBUTE) continue;
      const bool diff = op == PPI_OP_CONST;
      if (diff && nconst >= kAdjMaxConsts) {
         a.meta[i] = make_int2(kAdjUnsupported, 0);
         return;
      }
      code[tab0 + ntab] = make_uint4(w[k].y, (uint32_t)k, diff ? (uint32_t)nconst++ : ~0u, 0u);
      frames[a.max_size + k] = (uint32_t)ntab++;   // leaves: their table index
   }
   auto operand = [&](int c) -> uint32_t {
      const int op = w_op(w[c]);
      if (op_arity(op) > 0) return opd(kOpdRow, frames[c]);
      if (op == PPI_OP_ATTRIBUTE) return opd(kOpdAttr, w[c].y);
      return opd(op == PPI_OP_CONST ? kOpdConst : kOpdLiteral, frames[a.max_size + c]);
   };
   // ---- which operators have a constant below them (right to left) ----
   // bit 31 of w[k].x (sub < 2^15 leaves it free)
   for (int k = sz - 1; k >= 0; --k) {
      const int op = w_op(w[k]);
      const int ar = op_arity(op);
      bool has = op == PPI_OP_CONST;
      int c = k + 1;
      for (int q = 0; q < ar; ++q) {
         has = has || (w[c].x >> 31);
         c += w_sub(w[c]);
      }
      if (has) w[k].x |= 0x80000000u;
   }
   auto needs_adj = [&](int c) { return op_arity(w_op(w[c])) > 0 && (w[c].x >> 31); };
   // ---- adjoint rows: reverse sweep in prefix order ----
   // rows: [0, m) values; m: the root's adjoint; m + 1 + s: adjoint stack slot s
   int sp = 0, smax = 0;
   if (ninstr > 0) frames[a.max_size + 0] = (uint32_t)m;   // root
   for (int k = 0; k < sz; ++k) {
      const int op = w_op(w[k]);
      const int ar = op_arity(op);
      if (ar == 0) continue;
      const bool rev = (w[k].x >> 31) != 0;
      const int c0 = k + 1;
      const int c1 = c0 + w_sub(w[c0]);
      const int c2 = ar > 2 ? c1 + w_sub(w[c1]) : c1;
      uint32_t dst1 = kAdjNoRow, dst2 = kAdjNoRow;
      if (rev) {
         // the node's own adjoint: if it sits on the stack, it is the top slot
         if ((int)frames[a.max_size + k] > m) --sp;
         // later children first, so the next one visited is on top
         if (ar > 2 && needs_adj(c2)) {
            dst2 = (uint32_t)(m + 1 + sp++);
            frames[a.max_size + c2] = dst2;
         }
         if (ar > 1 && needs_adj(c1)) {
            dst1 = (uint32_t)(m + 1 + sp++);
            frames[a.max_size + c1] = dst1;
         }
         smax = max(smax, sp);
         if (needs_adj(c0)) frames[a.max_size + c0] = frames[k];   // over the node's own row
      }
      // instruction j = tape row of node k, two uint4 per instruction
      const int j = (int)frames[k];
      const uint32_t flags = (rev ? kAdjRev : 0u) | (rev && needs_adj(c0) ? kAdjKeep0 : 0u);
      code[1 + 2 * j] = make_uint4((uint32_t)op | ((uint32_t)ar << 8) | flags, frames[k], operand(c0),
                                   ar > 1 ? operand(c1) : 0u);
      code[2 + 2 * j] = make_uint4(ar > 2 ? operand(c2) : 0u, rev ? frames[a.max_size + k] : kAdjNoRow,
                                   dst1, dst2);
   }
   const int rows = m + 1 + smax;
   const int len = tab0 + ntab;
   if (len > a.code_stride) {
      a.meta[i] = make_int2(kAdjUnsupported, 0);
      return;
   }
   code[0] = make_uint4((uint32_t)ninstr, (uint32_t)ntab, (uint32_t)rows | ((uint32_t)nconst << 16),
                        operand(0));
   a.meta[i] = make_int2(kAdjValid | (rows << 8), len);
   atomicMax(a.max_rows, rows);
   atomicMax(a.max_consts, nconst);
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

// Which operand values and which own value an opcode's adjoint reads.
template <int OP> __device__ constexpr bool adj_uses_v() {
   return OP == PPI_OP_EXP || OP == PPI_OP_EXP2 || OP == PPI_OP_EXP10 || OP == PPI_OP_LOGISTIC ||
          OP == PPI_OP_GAUSS || OP == PPI_OP_SQRT || OP == PPI_OP_TAN || OP == PPI_OP_POW || OP == PPI_OP_DIV;
}
template <int OP> __device__ constexpr bool adj_uses_a() {
   return !(OP == PPI_OP_NEG || OP == PPI_OP_EXP || OP == PPI_OP_EXP2 || OP == PPI_OP_EXP10 ||
            OP == PPI_OP_LOGISTIC || OP == PPI_OP_ADD || OP == PPI_OP_SUB || OP == PPI_OP_MEAN ||
            OP == PPI_OP_DIV);
}
template <int OP> __device__ constexpr bool adj_uses_b() {
   return OP == PPI_OP_MULT || OP == PPI_OP_MAX || OP == PPI_OP_MIN || OP == PPI_OP_MOD ||
          OP == PPI_OP_POW || OP == PPI_OP_DIV;
}

__device__ __forceinline__ void adj_row(const float* s_rows, uint32_t row, int T, int tid, float (&x)[4]) {
   const float4 u = *reinterpret_cast<const float4*>(s_rows + (size_t)row * T + tid * 4);
   x[0] = u.x; x[1] = u.y; x[2] = u.z; x[3] = u.w;
}

// Values of an operand at this thread's 4 records.
__device__ __forceinline__ void adj_load(uint32_t d, const float* s_rows, int T, int tid, const uint4* s_tab,
                                         const float* data, int ld, int base, float (&x)[4]) {
   const uint32_t kind = opd_kind(d), v = opd_val(d);
   if (kind == kOpdRow) {
      const float4 u = *reinterpret_cast<const float4*>(s_rows + (size_t)v * T + tid * 4);
      x[0] = u.x; x[1] = u.y; x[2] = u.z; x[3] = u.w;
   } else if (kind == kOpdAttr) {
      const int pos = base + tid * 4;
      const float* col = data + (size_t)v * ld;
      if (pos + 3 < ld) {
         const float4 u = __ldg(reinterpret_cast<const float4*>(col + pos));
         x[0] = u.x; x[1] = u.y; x[2] = u.z; x[3] = u.w;
      } else {
#pragma unroll
         for (int r = 0; r < 4; ++r) x[r] = pos + r < ld ? __ldg(col + pos + r) : 0.0f;
      }
   } else {
      const float k = __uint_as_float(s_tab[v].x);
#pragma unroll
      for (int r = 0; r < 4; ++r) x[r] = k;
   }
}

// Deliver an operand's adjoints: its tape row `dst`, a constant's partial
// sum (this thread's float partial, flushed into a double one every
// kAdjFlush tiles), or nowhere (attributes, literals).
constexpr int kAdjFlush = 32;
__device__ __forceinline__ void adj_store(uint32_t d, uint32_t dst, const float (&x)[4], float* s_rows, int T,
                                          int tid, int P, const uint4* s_tab, float* s_part) {
   const uint32_t kind = opd_kind(d);
   if (kind == kOpdRow) {
      if (dst != kAdjNoRow)
         *reinterpret_cast<float4*>(s_rows + (size_t)dst * T + tid * 4) = make_float4(x[0], x[1], x[2], x[3]);
   } else if (kind == kOpdConst) {
      const uint32_t slot = s_tab[opd_val(d)].z;
      s_part[slot * P + tid] += (x[0] + x[1]) + (x[2] + x[3]);
   }
}

// Opcode lists of the sweeps (as the evaluator's: FULL, or the arithmetic set).
#define ADJ_ARITH_UNARY(X) X(PPI_OP_ABS) X(PPI_OP_POW2) X(PPI_OP_NEG) X(PPI_OP_EXP) X(PPI_OP_SIN) \
   X(PPI_OP_COS) X(PPI_OP_SQRT) X(PPI_OP_LOG)
#define ADJ_ARITH_BINARY(X) X(PPI_OP_ADD) X(PPI_OP_SUB) X(PPI_OP_MULT) X(PPI_OP_DIV)
// the full set minus the arithmetic one
#define ADJ_FULL_REST_U(X) X(PPI_OP_NOT) X(PPI_OP_POW3) X(PPI_OP_POW4) X(PPI_OP_POW5) X(PPI_OP_ROUND) \
   X(PPI_OP_CEIL) X(PPI_OP_FLOOR) X(PPI_OP_EXP10) X(PPI_OP_EXP2) X(PPI_OP_STEP) X(PPI_OP_SIGN)       \
   X(PPI_OP_LOGISTIC) X(PPI_OP_GAMMA) X(PPI_OP_GAUSS) X(PPI_OP_LOG10) X(PPI_OP_LOG2) X(PPI_OP_TAN)
#define ADJ_FULL_REST_B(X) X(PPI_OP_AND) X(PPI_OP_OR) X(PPI_OP_XOR) X(PPI_OP_GREATER)            \
   X(PPI_OP_GREATEREQUAL) X(PPI_OP_LESS) X(PPI_OP_LESSEQUAL) X(PPI_OP_EQUAL) X(PPI_OP_NOTEQUAL)   \
   X(PPI_OP_MEAN) X(PPI_OP_MAX) X(PPI_OP_MIN) X(PPI_OP_MOD) X(PPI_OP_POW)

// Forward sweep: every operator's value into its tape row.
#define ADJ_FWD_U(OP)                                                                   \
   case OP:                                                                             \
      _Pragma("unroll") for (int r = 0; r < 4; ++r) v[r] = unop<OP, MATH>(x[r], prot);   \
      break;
#define ADJ_FWD_B(OP)                                                                   \
   case OP:                                                                             \
      adj_load(i0.w, s_rows, T, tid, s_tab, data, ld, base, y);                         \
      _Pragma("unroll") for (int r = 0; r < 4; ++r) v[r] = binop<OP, MATH>(x[r], y[r], prot); \
      break;
// Reverse sweep: the operands' adjoints of one operator.
#define ADJ_REV_U(OP)                                                                   \
   case OP:                                                                             \
      if constexpr (adj_uses_a<OP>()) adj_load(i0.z, s_rows, T, tid, s_tab, data, ld, base, x); \
      if constexpr (adj_uses_v<OP>()) adj_row(s_rows, i0.y, T, tid, v);                 \
      _Pragma("unroll") for (int r = 0; r < 4; ++r)                                     \
         adj_bp<OP>(g[r], x[r], 0.0f, 0.0f, v[r], prot, d0[r], d1[r], d2[r]);           \
      break;
#define ADJ_REV_B(OP)                                                                   \
   case OP:                                                                             \
      if constexpr (adj_uses_a<OP>()) adj_load(i0.z, s_rows, T, tid, s_tab, data, ld, base, x); \
      if constexpr (adj_uses_b<OP>()) adj_load(i0.w, s_rows, T, tid, s_tab, data, ld, base, y); \
      if constexpr (adj_uses_v<OP>()) adj_row(s_rows, i0.y, T, tid, v);                 \
      _Pragma("unroll") for (int r = 0; r < 4; ++r)                                     \
         adj_bp<OP>(g[r], x[r], y[r], 0.0f, v[r], prot, d0[r], d1[r], d2[r]);           \
      break;

template <int MATH, int OPSET>
__device__ __forceinline__ void adj_forward(const uint4* s_code, int ninstr, float* s_rows, int T, int tid,
                                            const uint4* s_tab, const float* data, int ld, int base,
                                            int prot) {
   for (int j = 0; j < ninstr; ++j) {
      const uint4 i0 = s_code[1 + 2 * j];
      float x[4], y[4], z[4], v[4];
      adj_load(i0.z, s_rows, T, tid, s_tab, data, ld, base, x);
      switch (i0.x & 0xFFu) {
      ADJ_ARITH_UNARY(ADJ_FWD_U)
      ADJ_ARITH_BINARY(ADJ_FWD_B)
      default:
         if constexpr (OPSET == kOpsetFull) {
            switch (i0.x & 0xFFu) {
            ADJ_FULL_REST_U(ADJ_FWD_U)
            ADJ_FULL_REST_B(ADJ_FWD_B)
            case PPI_OP_IF_THEN_ELSE: {
               const uint4 i1 = s_code[2 + 2 * j];
               adj_load(i0.w, s_rows, T, tid, s_tab, data, ld, base, y);
               adj_load(i1.x, s_rows, T, tid, s_tab, data, ld, base, z);
#pragma unroll
               for (int r = 0; r < 4; ++r) v[r] = truthy(x[r]) ? y[r] : z[r];
               break;
            }
            default:
#pragma unroll
               for (int r = 0; r < 4; ++r) v[r] = __uint_as_float(0x7fc00000u);
            }
         } else {
#pragma unroll
            for (int r = 0; r < 4; ++r) v[r] = __uint_as_float(0x7fc00000u);
         }
      }
      *reinterpret_cast<float4*>(s_rows + (size_t)i0.y * T + tid * 4) = make_float4(v[0], v[1], v[2], v[3]);
   }
}

template <int MATH, int OPSET>
__device__ __forceinline__ void adj_reverse(const uint4* s_code, int ninstr, float* s_rows, int T, int tid,
                                            int P, const uint4* s_tab, float* s_part, const float* data,
                                            int ld, int base, int nlin, int prot) {
   for (int j = ninstr - 1; j >= 0; --j) {
      const uint4 i0 = s_code[1 + 2 * j];
      if (!(i0.x & kAdjRev)) continue;   // no constant below: no adjoint needed
      const uint4 i1 = s_code[2 + 2 * j];
      const int ar = (int)((i0.x >> 8) & 0xFFu);
      float x[4] = {0.0f, 0.0f, 0.0f, 0.0f}, y[4] = {0.0f, 0.0f, 0.0f, 0.0f}, z[4], v[4] = {0.0f, 0.0f, 0.0f, 0.0f};
      float g[4], d0[4], d1[4], d2[4];
      adj_row(s_rows, i1.y, T, tid, g);
      // records past the end carry no adjoint; a zero adjoint propagates
      // zero (never 0 x inf = NaN from an infinite partial)
      bool live[4];
#pragma unroll
      for (int r = 0; r < 4; ++r) {
         live[r] = base + tid * 4 + r < nlin && g[r] != 0.0f;
         if (!live[r]) g[r] = 0.0f;
      }
      switch (i0.x & 0xFFu) {
      ADJ_ARITH_UNARY(ADJ_REV_U)
      ADJ_ARITH_BINARY(ADJ_REV_B)
      default:
         if constexpr (OPSET == kOpsetFull) {
            switch (i0.x & 0xFFu) {
            ADJ_FULL_REST_U(ADJ_REV_U)
            ADJ_FULL_REST_B(ADJ_REV_B)
            case PPI_OP_IF_THEN_ELSE:
               adj_load(i0.z, s_rows, T, tid, s_tab, data, ld, base, x);
#pragma unroll
               for (int r = 0; r < 4; ++r) {
                  d0[r] = 0.0f;
                  d1[r] = truthy(x[r]) ? g[r] : 0.0f;
                  d2[r] = truthy(x[r]) ? 0.0f : g[r];
               }
               break;
            default:
#pragma unroll
               for (int r = 0; r < 4; ++r) { d0[r] = 0.0f; d1[r] = 0.0f; d2[r] = 0.0f; }
            }
         } else {
#pragma unroll
            for (int r = 0; r < 4; ++r) { d0[r] = 0.0f; d1[r] = 0.0f; d2[r] = 0.0f; }
         }
      }
#pragma unroll
      for (int r = 0; r < 4; ++r)
         if (!live[r]) { d0[r] = 0.0f; d1[r] = 0.0f; d2[r] = 0.0f; }
      adj_store(i0.z, (i0.x & kAdjKeep0) ? i0.y : kAdjNoRow, d0, s_rows, T, tid, P, s_tab, s_part);
      if (ar > 1) adj_store(i0.w, i1.z, d1, s_rows, T, tid, P, s_tab, s_part);
      if (ar > 2) adj_store(i1.x, i1.w, d2, s_rows, T, tid, P, s_tab, s_part);
   }
}

template <int MATH, int OPSET>
__global__ void __launch_bounds__(128) adjoint_kernel(const AdjointArgs a) {
   extern __shared__ __align__(16) unsigned char smem_raw[];
   __shared__ int s_prog, s_bad;
   const int P = blockDim.x, tid = threadIdx.x, T = P * kAdjR;
   uint4* s_code = reinterpret_cast<uint4*>(smem_raw);
   double* s_sum = reinterpret_cast<double*>(smem_raw + (size_t)a.code_stride * sizeof(uint4));
   float* s_part = reinterpret_cast<float*>(s_sum + (size_t)a.max_consts * P);
   float* s_rows = s_part + (size_t)a.max_consts * P;
   const float inv_n = 1.0f / (float)a.nlin;
   for (;;) {
      if (tid == 0) {
         s_prog = (int)atomicAdd(a.queue, 1u);
         s_bad = 0;
      }
      __syncthreads();
      const int item = s_prog;
      if (item >= a.n_items) break;
      const int prog = a.order ? a.order[item] : item;
      const int2 meta = a.meta[prog];
      float* grad = a.grad + (size_t)prog * a.max_size;
      if ((meta.x & 0xFF) != kAdjValid) {
         // size 0 or malformed: no gradient (zeros; malformed reports NaN)
         const float gv = (meta.x & 0xFF) == kAdjUnsupported ? __uint_as_float(0x7fc00000u) : 0.0f;
         for (int k = tid; k < a.max_size; k += P) grad[k] = gv;
         __syncthreads();
         continue;
      }
      const uint4* code = a.code + (size_t)prog * a.code_stride;
      for (int k = tid; k < meta.y; k += P) s_code[k] = code[k];
      __syncthreads();
      const uint4 hdr = s_code[0];
      const int ninstr = (int)hdr.x, ntab = (int)hdr.y, nconst = (int)(hdr.z >> 16);
      const int m = ninstr;   // row of the root's adjoint
      const uint32_t root = hdr.w;
      const uint4* s_tab = s_code + 1 + 2 * ninstr;
      for (int q = 0; q < nconst; ++q) {
         s_sum[q * P + tid] = 0.0;
         s_part[q * P + tid] = 0.0f;
      }
      int tiles = 0;
      for (int base = 0; base < a.nlin; base += T) {
         adj_forward<MATH, OPSET>(s_code, ninstr, s_rows, T, tid, s_tab, a.data, a.ld, base, a.prot);
         // prediction, error derivative, the root's adjoint
         float p[4], ys[4], e1[4];
         adj_load(root, s_rows, T, tid, s_tab, a.data, a.ld, base, p);
         adj_load(opd(kOpdAttr, (uint32_t)(a.ncol - 1)), s_rows, T, tid, s_tab, a.data, a.ld, base, ys);
         bool bad = false;
#pragma unroll
         for (int r = 0; r < 4; ++r) {
            const float d = p[r] - ys[r];
            e1[r] = 0.0f;
            if (base + tid * 4 + r < a.nlin) {
               const float err = a.ef == PPI_EF_SQUARED ? d * d : fabsf(d);
               if (nonfinite(err)) bad = true;
               const float de = a.ef == PPI_EF_SQUARED ? 2.0f * d : (d > 0.0f ? 1.0f : (d < 0.0f ? -1.0f : 0.0f));
               e1[r] = de * inv_n;
            }
         }
         if (bad) s_bad = 1;
         if (opd_kind(root) == kOpdConst) {
            const uint32_t slot = s_tab[opd_val(root)].z;
            s_part[slot * P + tid] += (e1[0] + e1[1]) + (e1[2] + e1[3]);
         }
         if (ninstr > 0)
            *reinterpret_cast<float4*>(s_rows + (size_t)m * T + tid * 4) = make_float4(e1[0], e1[1], e1[2], e1[3]);
         adj_reverse<MATH, OPSET>(s_code, ninstr, s_rows, T, tid, P, s_tab, s_part, a.data, a.ld, base,
                                  a.nlin, a.prot);
         if (++tiles == kAdjFlush || base + T >= a.nlin) {
            for (int q = 0; q < nconst; ++q) {
               s_sum[q * P + tid] += (double)s_part[q * P + tid];
               s_part[q * P + tid] = 0.0f;
            }
            tiles = 0;
         }
      }
      __syncthreads();
      // reduce the partials of each constant and write the gradient at its token
      for (int k = tid; k < a.max_size; k += P) grad[k] = 0.0f;
      __syncthreads();
      for (int t = 0; t < ntab; ++t) {
         const uint4 e = s_tab[t];
         if (e.z == ~0u) continue;
         double* pp = s_sum + e.z * P;
         for (int st = P >> 1; st > 0; st >>= 1) {
            if (tid < st) pp[tid] += pp[tid + st];
            __syncthreads();
         }
         if (tid == 0) grad[e.y] = s_bad ? 0.0f : (float)pp[0];
         __syncthreads();
      }
   }
}

}  // namespace

cudaError_t launch_adjoint_translate(const AdjointTranslateArgs& a, cudaStream_t s) {
   adjoint_translate_kernel<<<std::max(1, (a.n + 127) / 128), 128, 0, s>>>(a);
   return cudaGetLastError();
}

size_t adjoint_smem_bytes(int code_stride, int max_consts, int rows, int block) {
   return (size_t)code_stride * sizeof(uint4) + (size_t)max_consts * block * (sizeof(double) + sizeof(float)) +
          (size_t)rows * block * kAdjR * sizeof(float);
}

template <int MATH>
auto adjoint_fn(int opset) {
   return opset == kOpsetArith ? adjoint_kernel<MATH, kOpsetArith> : adjoint_kernel<MATH, kOpsetFull>;
}

void (*adjoint_pick(int math, int opset))(const AdjointArgs) {
   if (math == kMathParity) return adjoint_fn<kMathParity>(opset);
   if (math == kMathNative) return adjoint_fn<kMathNative>(opset);
   return adjoint_fn<kMathFast>(opset);
}

cudaError_t launch_adjoint(int math, int opset, const AdjointArgs& a, int block, int grid, size_t smem,
                           cudaStream_t s) {
   auto k = adjoint_pick(math, opset);
   cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
   if (e != cudaSuccess) return e;
   k<<<grid, block, smem, s>>>(a);
   return cudaGetLastError();
}

cudaError_t adjoint_occupancy(int math, int opset, int block, size_t smem, int* per_sm) {
   auto k = adjoint_pick(math, opset);
   cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
   if (e != cudaSuccess) return e;
   return cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, k, block, smem);
}

}  // namespace ppi
