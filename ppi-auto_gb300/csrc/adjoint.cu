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
// constant's gradient in a per-thread double partial.  A thread reads and
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
// its adjoint during the reverse sweep.
__device__ __forceinline__ int w_op(uint2 w) { return (int)(w.x & 0xFFFFu); }
__device__ __forceinline__ int w_sub(uint2 w) { return (int)(w.x >> 16); }

__global__ void adjoint_translate_kernel(const AdjointTranslateArgs a) {
   const int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i >= a.n) return;
   uint4* code = a.code + (size_t)i * a.code_stride;
   const int sz = a.size[i];
   code[0] = make_uint4(0u, 0u, 0u, opd(kOpdLiteral, 0u));
   a.meta[i] = make_int2(kAdjInvalid, 0);
   if (sz <= 0 || sz > a.max_size) return;
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
   // ---- adjoint rows: reverse sweep in prefix order ----
   // rows: [0, m) values; m: the root's adjoint; m + 1 + s: adjoint stack slot s
   int sp = 0, smax = 0;
   if (ninstr > 0) frames[a.max_size + 0] = (uint32_t)m;   // root
   for (int k = 0; k < sz; ++k) {
      const int op = w_op(w[k]);
      const int ar = op_arity(op);
      if (ar == 0) continue;
      // the node's own adjoint: if it sits on the stack, it is the top slot
      if ((int)frames[a.max_size + k] > m) --sp;
      const int c0 = k + 1;
      const int c1 = c0 + w_sub(w[c0]);
      const int c2 = ar > 2 ? c1 + w_sub(w[c1]) : c1;
      uint32_t dst1 = 0u, dst2 = 0u;
      // later children first, so the next one visited is on top
      if (ar > 2 && op_arity(w_op(w[c2])) > 0) {
         dst2 = (uint32_t)(m + 1 + sp++);
         frames[a.max_size + c2] = dst2;
      }
      if (ar > 1 && op_arity(w_op(w[c1])) > 0) {
         dst1 = (uint32_t)(m + 1 + sp++);
         frames[a.max_size + c1] = dst1;
      }
      smax = max(smax, sp);
      if (op_arity(w_op(w[c0])) > 0) frames[a.max_size + c0] = frames[k];   // over the node's own row
      // instruction j = tape row of node k, two uint4 per instruction
      const int j = (int)frames[k];
      code[1 + 2 * j] = make_uint4((uint32_t)op | ((uint32_t)ar << 8), frames[k], operand(c0),
                                   ar > 1 ? operand(c1) : 0u);
      code[2 + 2 * j] = make_uint4(ar > 2 ? operand(c2) : 0u, frames[a.max_size + k], dst1, dst2);
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

// ---- per-op forward values and local partials (a = left operand) ---------
template <int MATH>
__device__ __forceinline__ float adj_value(int op, float a, float b, float c, int prot) {
   switch (op) {
#define PPI_AU(OP) case OP: return unop<OP, MATH>(a, prot);
      PPI_AU(PPI_OP_NOT) PPI_AU(PPI_OP_ABS) PPI_AU(PPI_OP_POW2) PPI_AU(PPI_OP_POW3)
      PPI_AU(PPI_OP_POW4) PPI_AU(PPI_OP_POW5) PPI_AU(PPI_OP_NEG) PPI_AU(PPI_OP_ROUND)
      PPI_AU(PPI_OP_CEIL) PPI_AU(PPI_OP_FLOOR) PPI_AU(PPI_OP_EXP) PPI_AU(PPI_OP_EXP10)
      PPI_AU(PPI_OP_EXP2) PPI_AU(PPI_OP_SIN) PPI_AU(PPI_OP_COS) PPI_AU(PPI_OP_STEP)
      PPI_AU(PPI_OP_SIGN) PPI_AU(PPI_OP_LOGISTIC) PPI_AU(PPI_OP_GAMMA) PPI_AU(PPI_OP_GAUSS)
      PPI_AU(PPI_OP_SQRT) PPI_AU(PPI_OP_LOG) PPI_AU(PPI_OP_LOG10) PPI_AU(PPI_OP_LOG2)
      PPI_AU(PPI_OP_TAN)
#undef PPI_AU
#define PPI_AB(OP) case OP: return binop<OP, MATH>(a, b, prot);
      PPI_AB(PPI_OP_AND) PPI_AB(PPI_OP_OR) PPI_AB(PPI_OP_XOR) PPI_AB(PPI_OP_GREATER)
      PPI_AB(PPI_OP_GREATEREQUAL) PPI_AB(PPI_OP_LESS) PPI_AB(PPI_OP_LESSEQUAL)
      PPI_AB(PPI_OP_EQUAL) PPI_AB(PPI_OP_NOTEQUAL) PPI_AB(PPI_OP_ADD) PPI_AB(PPI_OP_SUB)
      PPI_AB(PPI_OP_MULT) PPI_AB(PPI_OP_MEAN) PPI_AB(PPI_OP_MAX) PPI_AB(PPI_OP_MIN)
      PPI_AB(PPI_OP_MOD) PPI_AB(PPI_OP_POW) PPI_AB(PPI_OP_DIV)
#undef PPI_AB
   case PPI_OP_IF_THEN_ELSE: return truthy(a) ? b : c;
   default: return __uint_as_float(0x7fc00000u);
   }
}

// Adjoints of the operands, g x d(op)/d(first, second, third operand), at
// operands a, b, c with value v and adjoint g.  Each product is formed in an
// order that does not overflow where the partial alone would (g / b before
// x v for a division by a tiny b, g / a for log).  Piecewise-constant ops
// and the protected branches have derivative 0.
__device__ __forceinline__ void adj_backprop(int op, float g, float a, float b, float c, float v,
                                             int prot, float& da, float& db, float& dc) {
   const float kLn2 = 0.693147180559945309f, kLn10 = 2.30258509299404568f;
   da = 0.0f; db = 0.0f; dc = 0.0f;
   (void)c;
   switch (op) {
   case PPI_OP_ABS: da = a > 0.0f ? g : (a < 0.0f ? -g : 0.0f); break;
   case PPI_OP_POW2: da = g * (2.0f * a); break;
   case PPI_OP_POW3: da = g * (3.0f * (a * a)); break;
   case PPI_OP_POW4: da = g * (4.0f * ((a * a) * a)); break;
   case PPI_OP_POW5: da = g * (5.0f * (((a * a) * a) * a)); break;
   case PPI_OP_NEG: da = -g; break;
   case PPI_OP_EXP: da = g * v; break;
   case PPI_OP_EXP2: da = (g * v) * kLn2; break;
   case PPI_OP_EXP10: da = (g * v) * kLn10; break;
   case PPI_OP_SIN: da = g * cosf(a); break;
   case PPI_OP_COS: da = -(g * sinf(a)); break;
   case PPI_OP_LOGISTIC: da = (g * v) * (1.0f - v); break;
   case PPI_OP_GAUSS: da = ((-2.0f * g) * a) * v; break;
   case PPI_OP_GAMMA: da = __uint_as_float(0x7fc00000u); break;   // not differentiated
   case PPI_OP_SQRT: da = (prot && a < 0.0f) ? 0.0f : (0.5f * g) / v; break;
   case PPI_OP_LOG: da = (prot && a < 1.0f) ? 0.0f : g / a; break;
   case PPI_OP_LOG2: da = (prot && a < 1.0f) ? 0.0f : (g / a) / kLn2; break;
   case PPI_OP_LOG10: da = (prot && a < 1.0f) ? 0.0f : (g / a) / kLn10; break;
   case PPI_OP_TAN: {
      const float fa = fabsf(a);
      da = (prot && (fa == kPi2F || fa == 3.0f * kPi2F)) ? 0.0f : g + (g * v) * v;
      break;
   }
   case PPI_OP_ADD: da = g; db = g; break;
   case PPI_OP_SUB: da = g; db = -g; break;
   case PPI_OP_MULT: da = g * b; db = g * a; break;
   case PPI_OP_MEAN: da = 0.5f * g; db = 0.5f * g; break;
   case PPI_OP_MAX: if (a >= b) da = g; else db = g; break;
   case PPI_OP_MIN: if (a <= b) da = g; else db = g; break;
   case PPI_OP_MOD: da = g; db = -(g * truncf(a / b)); break;
   case PPI_OP_POW: da = (g * b) * (v / a); db = (g * v) * logf(a); break;
   case PPI_OP_DIV:
      if (!(prot && b == 0.0f)) {
         const float t = g / b;
         da = t;
         db = -(t * v);
      }
      break;
   case PPI_OP_IF_THEN_ELSE: if (truthy(a)) db = g; else dc = g; break;
   default: break;   // comparisons, logic, rounding, step, sign: 0
   }
}

// Values of an operand at this thread's 4 records.
__device__ __forceinline__ float4 adj_load(uint32_t d, const float* s_rows, int T, int tid,
                                           const uint4* s_tab, const float* data, int ld, int base) {
   const uint32_t kind = opd_kind(d), v = opd_val(d);
   if (kind == kOpdRow) return *reinterpret_cast<const float4*>(s_rows + (size_t)v * T + tid * 4);
   if (kind == kOpdAttr) {
      const int pos = base + tid * 4;
      const float* col = data + (size_t)v * ld;
      if (pos + 3 < ld) return __ldg(reinterpret_cast<const float4*>(col + pos));
      float4 r;
      r.x = pos < ld ? __ldg(col + pos) : 0.0f;
      r.y = pos + 1 < ld ? __ldg(col + pos + 1) : 0.0f;
      r.z = pos + 2 < ld ? __ldg(col + pos + 2) : 0.0f;
      r.w = 0.0f;
      return r;
   }
   const float k = __uint_as_float(s_tab[v].x);
   return make_float4(k, k, k, k);
}

template <int MATH>
__global__ void __launch_bounds__(128) adjoint_kernel(const AdjointArgs a) {
   extern __shared__ __align__(16) unsigned char smem_raw[];
   __shared__ int s_prog, s_bad;
   const int P = blockDim.x, tid = threadIdx.x, T = P * kAdjR;
   uint4* s_code = reinterpret_cast<uint4*>(smem_raw);
   double* s_part = reinterpret_cast<double*>(smem_raw + (size_t)a.code_stride * sizeof(uint4));
   float* s_rows = reinterpret_cast<float*>(reinterpret_cast<unsigned char*>(s_part) +
                                            (size_t)a.max_consts * P * sizeof(double));
   const float inv_n = 1.0f / (float)a.nlin;
   for (;;) {
      if (tid == 0) {
         s_prog = (int)atomicAdd(a.queue, 1u);
         s_bad = 0;
      }
      __syncthreads();
      const int prog = s_prog;
      if (prog >= a.n) break;
      const int2 meta = a.meta[prog];
      float* grad = a.grad + (size_t)prog * a.max_size;
      if ((meta.x & 0xFF) != kAdjValid) {
         // size 0 or malformed: no gradient (zeros; malformed reports NaN)
         const float g = (meta.x & 0xFF) == kAdjUnsupported ? __uint_as_float(0x7fc00000u) : 0.0f;
         for (int k = tid; k < a.max_size; k += P) grad[k] = g;
         __syncthreads();
         continue;
      }
      const uint4* code = a.code + (size_t)prog * a.code_stride;
      for (int k = tid; k < meta.y; k += P) s_code[k] = code[k];
      __syncthreads();
      const uint4 hdr = s_code[0];
      const int ninstr = (int)hdr.x, ntab = (int)hdr.y, nconst = (int)(hdr.z >> 16);
      const int m = ninstr;   // root adjoint row
      const uint32_t root = hdr.w;
      const uint4* s_tab = s_code + 1 + 2 * ninstr;
      for (int q = 0; q < nconst; ++q) s_part[q * P + tid] = 0.0;
      for (int base = 0; base < a.nlin; base += T) {
         // forward sweep
         for (int j = 0; j < ninstr; ++j) {
            const uint4 i0 = s_code[1 + 2 * j], i1 = s_code[2 + 2 * j];
            const int op = (int)(i0.x & 0xFF), ar = (int)((i0.x >> 8) & 0xFF);
            const float4 x = adj_load(i0.z, s_rows, T, tid, s_tab, a.data, a.ld, base);
            const float4 y = ar > 1 ? adj_load(i0.w, s_rows, T, tid, s_tab, a.data, a.ld, base) : x;
            const float4 z = ar > 2 ? adj_load(i1.x, s_rows, T, tid, s_tab, a.data, a.ld, base) : x;
            float4 v;
            v.x = adj_value<MATH>(op, x.x, y.x, z.x, a.prot);
            v.y = adj_value<MATH>(op, x.y, y.y, z.y, a.prot);
            v.z = adj_value<MATH>(op, x.z, y.z, z.z, a.prot);
            v.w = adj_value<MATH>(op, x.w, y.w, z.w, a.prot);
            *reinterpret_cast<float4*>(s_rows + (size_t)i0.y * T + tid * 4) = v;
         }
         // prediction, error derivative, the root's adjoint
         const float4 p = adj_load(root, s_rows, T, tid, s_tab, a.data, a.ld, base);
         const float4 yv = adj_load(opd(kOpdAttr, (uint32_t)(a.ncol - 1)), s_rows, T, tid, s_tab, a.data,
                                    a.ld, base);
         float pr[4] = {p.x, p.y, p.z, p.w}, ys[4] = {yv.x, yv.y, yv.z, yv.w}, e1[4];
         bool bad = false;
#pragma unroll
         for (int r = 0; r < 4; ++r) {
            const int n = base + tid * 4 + r;
            const float d = pr[r] - ys[r];
            if (n < a.nlin) {
               const float err = a.ef == PPI_EF_SQUARED ? d * d : fabsf(d);
               if (nonfinite(err)) bad = true;
               const float de = a.ef == PPI_EF_SQUARED ? 2.0f * d : (d > 0.0f ? 1.0f : (d < 0.0f ? -1.0f : 0.0f));
               e1[r] = de * inv_n;
            } else {
               e1[r] = 0.0f;
            }
         }
         if (bad) s_bad = 1;
         if (opd_kind(root) == kOpdConst) {
            const uint32_t slot = s_tab[opd_val(root)].z;
            s_part[slot * P + tid] += (double)((e1[0] + e1[1]) + (e1[2] + e1[3]));
         }
         if (ninstr > 0)
            *reinterpret_cast<float4*>(s_rows + (size_t)m * T + tid * 4) = make_float4(e1[0], e1[1], e1[2], e1[3]);
         // reverse sweep: prefix order = instructions from the root down
         for (int j = ninstr - 1; j >= 0; --j) {
            const uint4 i0 = s_code[1 + 2 * j], i1 = s_code[2 + 2 * j];
            const int op = (int)(i0.x & 0xFF), ar = (int)((i0.x >> 8) & 0xFF);
            const float4 x = adj_load(i0.z, s_rows, T, tid, s_tab, a.data, a.ld, base);
            const float4 y = ar > 1 ? adj_load(i0.w, s_rows, T, tid, s_tab, a.data, a.ld, base) : x;
            const float4 z = ar > 2 ? adj_load(i1.x, s_rows, T, tid, s_tab, a.data, a.ld, base) : x;
            const float4 v = *reinterpret_cast<const float4*>(s_rows + (size_t)i0.y * T + tid * 4);
            const float4 g = *reinterpret_cast<const float4*>(s_rows + (size_t)i1.y * T + tid * 4);
            const float xs[4] = {x.x, x.y, x.z, x.w}, ysv[4] = {y.x, y.y, y.z, y.w};
            const float zs[4] = {z.x, z.y, z.z, z.w}, vs[4] = {v.x, v.y, v.z, v.w};
            const float gs[4] = {g.x, g.y, g.z, g.w};
            float d0[4], d1[4], d2[4];
#pragma unroll
            for (int r = 0; r < 4; ++r) {
               // records past the end carry no adjoint, and a zero adjoint
               // propagates zero (never 0 x inf = NaN from an infinite partial)
               const bool live = base + tid * 4 + r < a.nlin && gs[r] != 0.0f;
               adj_backprop(op, live ? gs[r] : 0.0f, xs[r], ysv[r], zs[r], vs[r], a.prot, d0[r], d1[r], d2[r]);
               if (!live) { d0[r] = 0.0f; d1[r] = 0.0f; d2[r] = 0.0f; }
            }
            const uint32_t ds[3] = {i0.z, i0.w, i1.x};
            const uint32_t dst[3] = {i0.y, i1.z, i1.w};
            const float* dd[3] = {d0, d1, d2};
#pragma unroll
            for (int c = 0; c < 3; ++c) {
               if (c >= ar) break;
               const uint32_t kind = opd_kind(ds[c]);
               if (kind == kOpdRow) {
                  *reinterpret_cast<float4*>(s_rows + (size_t)dst[c] * T + tid * 4) =
                      make_float4(dd[c][0], dd[c][1], dd[c][2], dd[c][3]);
               } else if (kind == kOpdConst) {
                  const uint32_t slot = s_tab[opd_val(ds[c])].z;
                  s_part[slot * P + tid] += (double)((dd[c][0] + dd[c][1]) + (dd[c][2] + dd[c][3]));
               }
            }
         }
      }
      __syncthreads();
      // reduce the partials of each constant and write the gradient at its token
      for (int k = tid; k < a.max_size; k += P) grad[k] = 0.0f;
      __syncthreads();
      for (int t = 0; t < ntab; ++t) {
         const uint4 e = s_tab[t];
         if (e.z == ~0u) continue;
         double* pp = s_part + e.z * P;
         for (int s = P >> 1; s > 0; s >>= 1) {
            if (tid < s) pp[tid] += pp[tid + s];
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
   return (size_t)code_stride * sizeof(uint4) + (size_t)max_consts * block * sizeof(double) +
          (size_t)rows * block * kAdjR * sizeof(float);
}

cudaError_t launch_adjoint(int math, const AdjointArgs& a, int block, int grid, size_t smem, cudaStream_t s) {
   auto k = math == kMathParity ? adjoint_kernel<kMathParity>
                                : (math == kMathNative ? adjoint_kernel<kMathNative> : adjoint_kernel<kMathFast>);
   cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
   if (e != cudaSuccess) return e;
   k<<<grid, block, smem, s>>>(a);
   return cudaGetLastError();
}

cudaError_t adjoint_occupancy(int math, int block, size_t smem, int* per_sm) {
   auto k = math == kMathParity ? adjoint_kernel<kMathParity>
                                : (math == kMathNative ? adjoint_kernel<kMathNative> : adjoint_kernel<kMathFast>);
   cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
   if (e != cudaSuccess) return e;
   return cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, k, block, smem);
}

}  // namespace ppi
