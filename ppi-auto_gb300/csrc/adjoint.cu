// adjoint.cu -- d(fitness)/d(ephemeral constants) of every program by a
// reverse sweep over its prefix tree.  No counterpart in the reference: an
// addition for constant refinement, while the plain evaluator stays the
// fitness judge.
//
// Fitness with the sum reduction is F = (1/nlin) sum_n EF(p_n, y_n) (+ alpha
// size, constant in the ephemerals), so dF/dc = (1/nlin) sum_n EF'(p_n, y_n)
// dp_n/dc with EF' = sign(p - y) (absolute error) or 2 (p - y) (squared).
//
// Translation (one thread per program) writes two programs over one tile of
// shared-memory rows:
//  * the forward sweep in the evaluator's accumulator-machine bytecode (the
//    same emission order and leaf-operand folding, but no constant folding:
//    every constant stays a separate operand), with one extra push of each
//    value the reverse sweep reads (an operand of a differentiated operator,
//    or an operator's own value) into its own tape row;
//  * the reverse sweep: one instruction per operator with a constant below
//    it, in prefix order (parents before children).  The adjoint being
//    carried sits in registers; an operator passes it on to one child and
//    leaves the adjoints of the other differentiated children in stack rows
//    (reused from the forward sweep's slot rows, free by then) that a later
//    pop resumes; a constant's adjoint goes into its partial sum.  Children
//    with the smaller stack need are followed first, so the stack is as
//    shallow as the tree allows.
// Rows: [0, S) forward slots / adjoint stack, [S, S+NT) tape values, then the
// program's record columns and the target (staged by TMA, as the evaluator).
//
// Evaluation (one CTA per program, persistent work queue): for each tile of
// T = P x R records the forward sweep is recomputed (no per-record tape
// outlives its tile), then the reverse sweep accumulates each constant's
// gradient in a per-thread float partial; every 128 records of a thread the
// warp's partials are added into its double sum (few double operations,
// short float sums).  A thread reads and writes only its own positions of
// every row, so the sweeps need no barriers.  Any non-finite error makes the
// fitness a sentinel value (FLT_MAX rule), whose gradient is 0.
//
// R (4 or 8 records per thread) is chosen per program by the host: 8 where the
// program's rows leave room for several CTAs per SM, 4 for the widest
// programs (half the shared memory per row, twice the resident warps).
#include "adjoint_impl.cuh"

namespace ppi {
namespace {

using namespace adj;

// Translator node word: op (6 bits) | forward need (5) | reverse need (5) |
// subtree size (15) | a constant at or below the node (1).
__device__ __forceinline__ uint32_t anode(int op, int fneed, int rneed, int sub, bool h) {
   return (uint32_t)op | ((uint32_t)fneed << 6) | ((uint32_t)rneed << 11) | ((uint32_t)sub << 16) |
          (h ? 0x80000000u : 0u);
}
__device__ __forceinline__ int an_op(uint32_t x) { return (int)(x & 63u); }
__device__ __forceinline__ int an_fneed(uint32_t x) { return (int)((x >> 6) & 31u); }
__device__ __forceinline__ int an_rneed(uint32_t x) { return (int)((x >> 11) & 31u); }
__device__ __forceinline__ int an_sub(uint32_t x) { return (int)((x >> 16) & 0x7FFFu); }
__device__ __forceinline__ bool an_h(uint32_t x) { return (x >> 31) != 0u; }

// Evaluator frame of the forward emission walk: node | d << 16 | state << 24.
__device__ __forceinline__ uint32_t aframe(int node, int d, int st) {
   return (uint32_t)node | ((uint32_t)d << 16) | ((uint32_t)st << 24);
}

__global__ void adjoint_translate_kernel(const AdjointTranslateArgs a) {
   const int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i >= a.n) return;
   uint2* code = a.code + (size_t)i * a.code_stride;
   const int sz = a.size[i];
   a.meta[i] = make_int2(kAdjInvalid, 0);
   if (sz <= 0 || sz > a.max_size) return;
   const int2 unsupported = make_int2(kAdjUnsupported, 0);
   if (sz >= 32768) {   // subtree sizes have 15 bits
      a.meta[i] = unsupported;
      return;
   }
   const int32_t* ph = a.phenotype + (size_t)i * a.max_size;
   const float* eph = a.ephemeral + (size_t)i * a.max_size;
   uint2* w = a.work + (size_t)i * 2 * a.max_size;
   uint32_t* frames = reinterpret_cast<uint32_t*>(w + a.max_size);
   uint32_t* info = frames + a.max_size;
   const int cap = a.code_stride;

   // ---- pass 1 (right to left): ops, subtree sizes, needs, constants below
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
      int sub = 1, fneed = 0, rneed = 0;
      bool h = op == PPI_OP_CONST;
      if (ar > 0) {
         int c[3] = {k + 1, 0, 0};
         for (int q = 1; q < ar; ++q) c[q] = c[q - 1] + an_sub(w[c[q - 1]].x);
         int n[3] = {0, 0, 0}, x[3] = {0, 0, 0}, m = 0;
         bool leaf[3] = {false, false, false};
         for (int q = 0; q < ar; ++q) {
            const uint32_t wc = w[c[q]].x;
            sub += an_sub(wc);
            h = h || an_h(wc);
            n[q] = an_fneed(wc);
            leaf[q] = op_arity(an_op(wc)) == 0;
            if (!leaf[q] && an_h(wc)) x[m++] = an_rneed(wc);
         }
         // forward need: the evaluator's rule (leaf operands folded)
         if (ar == 1) fneed = n[0];
         else if (ar == 2) {
            if (leaf[0] && leaf[1]) fneed = 0;
            else if (leaf[1]) fneed = n[0];
            else if (leaf[0]) fneed = n[1];
            else fneed = max(n[0], n[1]) + (n[0] == n[1] ? 1 : 0);
         } else {
            int p = n[0], q = n[1], r = n[2];   // sort descending
            if (p < q) { int t = p; p = q; q = t; }
            if (q < r) { int t = q; q = r; r = t; }
            if (p < q) { int t = p; p = q; q = t; }
            fneed = max(p, max(q + 1, r + 2));
         }
         // reverse need: followed children in ascending need, the others
         // waiting in stack rows meanwhile
         if (h) {
            for (int u = 1; u < m; ++u)
               for (int v = u; v > 0 && x[v - 1] > x[v]; --v) { int t = x[v]; x[v] = x[v - 1]; x[v - 1] = t; }
            for (int q = 0; q < m; ++q) rneed = max(rneed, x[q] + (m - 1 - q));
         }
      }
      if (fneed > 30 || rneed > 30) { bad = true; break; }
      w[k] = make_uint2(anode(op, fneed, rneed, sub, h), imm);
   }
   if (bad || depth != 1 || an_sub(w[0].x) != sz) {
      a.meta[i] = unsupported;   // malformed: no gradient
      return;
   }

   // ---- constants (gradient slots, prefix order) and distinct columns ----
   uint32_t* list = reinterpret_cast<uint32_t*>(code + 1);
   int nconst = 0, ncols = 0;
   for (int k = 0; k < sz; ++k) {
      const int op = an_op(w[k].x);
      info[k] = kAdjNone;
      if (op == PPI_OP_CONST) {
         if (nconst >= kAdjMaxConsts) { a.meta[i] = unsupported; return; }
         info[k] = (uint32_t)nconst++;
      } else if (op == PPI_OP_ATTRIBUTE) {
         int j = 0;
         while (j < ncols && list[j] != w[k].y) ++j;
         if (j == ncols) {
            if (code_header(ncols + 1) + 2 >= cap) { a.meta[i] = unsupported; return; }
            list[ncols++] = w[k].y;
         }
         info[k] = (uint32_t)j;
      } else if (op_arity(op) > 0) {
         info[k] = 0u;   // operator: bit 31 set once its value is kept
      }
   }
   // ---- values the reverse sweep reads: operands and own values ----------
   for (int k = 0; k < sz; ++k) {
      const int op = an_op(w[k].x);
      const int ar = op_arity(op);
      if (ar == 0 || !an_h(w[k].x)) continue;
      const int c0 = k + 1, c1 = c0 + an_sub(w[c0].x);
      if (adj_reads_v(op)) info[k] = 0x80000000u;
      if (adj_reads_a(op) && op_arity(an_op(w[c0].x)) > 0) info[c0] = 0x80000000u;
      if (ar > 1 && adj_reads_b(op) && op_arity(an_op(w[c1].x)) > 0) info[c1] = 0x80000000u;
   }
   const bool root_rev = op_arity(an_op(w[0].x)) > 0 && an_h(w[0].x);
   const int S = max(an_fneed(w[0].x), root_rev ? an_rneed(w[0].x) : 0);
   int nt = 0;
   for (int k = 0; k < sz; ++k)
      if (op_arity(an_op(w[k].x)) > 0 && (info[k] >> 31)) info[k] = 0x80000000u | (uint32_t)(S + nt++);
   const int crow0 = S + nt;             // first column row
   const int rows = crow0 + ncols + 1;   // + the target
   if (rows >= 0x7FFF) { a.meta[i] = unsupported; return; }
   code[0] = make_uint2((uint32_t)ncols, (uint32_t)crow0);   // evaluator header: all columns staged
   if (ncols & 1) list[ncols] = 0u;
   const int ch = code_header(ncols);
   int ncode = ch + 2;
   auto emit = [&](uint32_t x, uint32_t y) {
      if (ncode < cap) code[ncode] = make_uint2(x, y);
      ++ncode;
   };
   auto is_leaf = [&](int nd) { return op_arity(an_op(w[nd].x)) == 0; };
   auto is_attr = [&](int nd) { return an_op(w[nd].x) == PPI_OP_ATTRIBUTE; };
   auto leaf_imm = [&](int nd) { return is_attr(nd) ? (uint32_t)crow0 + info[nd] : w[nd].y; };
   auto kept = [&](int nd) { return !is_leaf(nd) && (info[nd] >> 31) != 0u; };
   auto trow = [&](int nd) { return info[nd] & 0xFFFFu; };

   // ---- forward sweep: the evaluator's emission, plus the kept values -----
   {
      // a push followed by a load of a tile row becomes one M_PUSH_LD
      bool after_push = false;
      uint32_t push_row = 0u;
      auto emit = [&](uint32_t x, uint32_t y) {
         if (after_push && x == M_LD_ROW && y < 0x10000u && push_row < 0x10000u) {
            if (ncode - 1 < cap) code[ncode - 1] = make_uint2(M_PUSH_LD, push_row | (y << 16));
            after_push = false;
            return;
         }
         if (ncode < cap) code[ncode] = make_uint2(x, y);
         ++ncode;
         after_push = x == M_PUSH;
         push_row = y;
      };
      int fp = 0;
      frames[fp++] = aframe(0, 0, 0);
      auto finish = [&](int nd) {
         if (kept(nd)) emit(M_PUSH, trow(nd));
      };
      while (fp > 0) {
         const uint32_t f = frames[fp - 1];
         const int node = (int)(f & 0xFFFFu), d = (int)((f >> 16) & 0xFFu), st = (int)(f >> 24);
         const int op = an_op(w[node].x);
         const int ar = op_arity(op);
         if (ar == 0) {
            emit(is_attr(node) ? M_LD_ROW : M_LD_C, leaf_imm(node));
            --fp;
            continue;
         }
         const int c0 = node + 1;
         if (ar == 1) {
            if (st == 0) { frames[fp - 1] = aframe(node, d, 1); frames[fp++] = aframe(c0, d, 0); }
            else { emit(M_UN + (uint32_t)(op - PPI_OP_NOT), 0u); finish(node); --fp; }
            continue;
         }
         const int c1 = c0 + an_sub(w[c0].x);
         if (ar == 2) {
            const uint32_t bo = (uint32_t)(op - PPI_OP_AND);
            const bool l0 = is_leaf(c0), l1 = is_leaf(c1);
            if (l0 && l1) {
               emit(is_attr(c0) ? M_LD_ROW : M_LD_C, leaf_imm(c0));
               emit((is_attr(c1) ? M_BR_L : M_BC_L) + bo, leaf_imm(c1));
               finish(node);
               --fp;
            } else if (l1) {
               if (st == 0) { frames[fp - 1] = aframe(node, d, 1); frames[fp++] = aframe(c0, d, 0); }
               else { emit((is_attr(c1) ? M_BR_L : M_BC_L) + bo, leaf_imm(c1)); finish(node); --fp; }
            } else if (l0) {
               if (st == 0) { frames[fp - 1] = aframe(node, d, 1); frames[fp++] = aframe(c1, d, 0); }
               else { emit((is_attr(c0) ? M_BR_R : M_BC_R) + bo, leaf_imm(c0)); finish(node); --fp; }
            } else {
               const bool left_first = an_fneed(w[c0].x) >= an_fneed(w[c1].x);
               const int first = left_first ? c0 : c1, second = left_first ? c1 : c0;
               if (st == 0) {
                  frames[fp - 1] = aframe(node, d, 1);
                  frames[fp++] = aframe(first, d, 0);
               } else if (st == 1) {
                  if (!kept(first)) emit(M_PUSH, (uint32_t)d);   // a kept value is in its tape row
                  frames[fp - 1] = aframe(node, d, 2);
                  frames[fp++] = aframe(second, d + 1, 0);
               } else {
                  const uint32_t row = kept(first) ? trow(first) : (uint32_t)d;
                  emit((left_first ? M_BR_R : M_BR_L) + bo, row);
                  finish(node);
                  --fp;
               }
            }
            continue;
         }
         // IF_THEN_ELSE(cond = c0, then = c1, else = c2), the evaluator's order
         const int c2 = c1 + an_sub(w[c1].x);
         int x[3] = {c0, c1, c2};
         for (int p = 0; p < 2; ++p)
            for (int q = 0; q < 2 - p; ++q)
               if (an_fneed(w[x[q]].x) < an_fneed(w[x[q + 1]].x)) { int t = x[q]; x[q] = x[q + 1]; x[q + 1] = t; }
         if (st == 0) {
            frames[fp - 1] = aframe(node, d, 1);
            frames[fp++] = aframe(x[0], d, 0);
         } else if (st == 1) {
            if (!kept(x[0])) emit(M_PUSH, (uint32_t)d);
            frames[fp - 1] = aframe(node, d, 2);
            frames[fp++] = aframe(x[1], d + 1, 0);
         } else if (st == 2) {
            if (!kept(x[1])) emit(M_PUSH, (uint32_t)(d + 1));
            frames[fp - 1] = aframe(node, d, 3);
            frames[fp++] = aframe(x[2], d + 2, 0);
         } else {
            const uint32_t ra = kept(x[0]) ? trow(x[0]) : (uint32_t)d;
            const uint32_t rb = kept(x[1]) ? trow(x[1]) : (uint32_t)(d + 1);
            auto reg = [&](int child) { return child == x[0] ? 1 : (child == x[1] ? 2 : 0); };
            const int rc = reg(c0), rt = reg(c1), re = reg(c2);
            int perm = 0;
            for (int p = 0; p < 6; ++p)
               if (ite_role(p, 0) == rc && ite_role(p, 1) == rt && ite_role(p, 2) == re) perm = p;
            emit(M_ITE + (uint32_t)perm, ra | (rb << 16));
            finish(node);
            --fp;
         }
      }
      emit(M_END, 0u);
   }

   // ---- reverse sweep ------------------------------------------------------
   // instruction (two words): {op | kinds << 8 | own-value row << 16,
   // operand a | operand b << 16}, {dst0 | dst1 << 16, dst2}; kind per child
   // (2 bits): 0 none, 1 carried on, 2 stack row dst, 3 constant slot dst
   const uint32_t rev_pc = (uint32_t)ncode;
   int ntab = nconst;   // operand table: the constants, then literal operands
   auto desc = [&](int nd) -> uint32_t {
      const int o = an_op(w[nd].x);
      if (op_arity(o) > 0) return trow(nd);
      if (o == PPI_OP_ATTRIBUTE) return (uint32_t)crow0 + info[nd];
      if (info[nd] == kAdjNone) info[nd] = (uint32_t)ntab++;   // literal or invalid leaf
      return kAdjImm | info[nd];
   };
   int max_sp = 0;
   if (root_rev) {
      int sp = 0, pend = 0, cur = 0;   // pending children in frames[]: node | row << 16
      for (;;) {
         const int op = an_op(w[cur].x), ar = op_arity(op);
         int c[3] = {cur + 1, 0, 0};
         for (int q = 1; q < ar; ++q) c[q] = c[q - 1] + an_sub(w[c[q - 1]].x);
         uint32_t kinds = 0u, dst[3] = {0u, 0u, 0u};
         int C[3], m = 0;
         for (int q = 0; q < ar; ++q) {
            const int co = an_op(w[c[q]].x);
            if (co == PPI_OP_CONST) { kinds |= 3u << (2 * q); dst[q] = info[c[q]]; }
            else if (op_arity(co) > 0 && an_h(w[c[q]].x)) C[m++] = q;
         }
         for (int u = 1; u < m; ++u)   // ascending reverse need, stable
            for (int v = u; v > 0 && an_rneed(w[c[C[v - 1]]].x) > an_rneed(w[c[C[v]]].x); --v) {
               int t = C[v]; C[v] = C[v - 1]; C[v - 1] = t;
            }
         for (int q = m - 1; q >= 1; --q) {   // the next one to resume ends on top
            kinds |= 2u << (2 * C[q]);
            dst[C[q]] = (uint32_t)sp;
            frames[pend++] = (uint32_t)c[C[q]] | ((uint32_t)sp << 16);
            ++sp;
         }
         max_sp = max(max_sp, sp);
         if (m >= 1) kinds |= 1u << (2 * C[0]);
         const uint32_t da = adj_reads_a(op) ? desc(c[0]) : 0u;
         const uint32_t db = (ar > 1 && adj_reads_b(op)) ? desc(c[1]) : 0u;
         const uint32_t vrow = adj_reads_v(op) ? trow(cur) : 0xFFFFu;
         emit((uint32_t)op | (kinds << 8) | (vrow << 16), da | (db << 16));
         emit(dst[0] | (dst[1] << 16), dst[2]);
         if (m >= 1) { cur = c[C[0]]; continue; }
         if (pend == 0) break;
         const uint32_t e = frames[--pend];
         cur = (int)(e & 0xFFFFu);
         --sp;
         emit(kRevPop, e >> 16);
         emit(0u, 0u);
      }
   }
   emit(kRevEnd, 0u);
   emit(0u, 0u);
   const uint32_t tab_pc = (uint32_t)ncode;
   if (max_sp > S || ncode + ntab > cap) { a.meta[i] = unsupported; return; }
   // operand table {value bits, token position}: constant q at entry q
   for (int k = 0; k < sz; ++k) {
      const int op = an_op(w[k].x);
      if (op_arity(op) == 0 && op != PPI_OP_ATTRIBUTE && info[k] != kAdjNone)
         code[tab_pc + info[k]] = make_uint2(w[k].y, (uint32_t)k);
   }
   ncode += ntab;
   code[ch] = make_uint2(rev_pc, tab_pc);
   code[ch + 1] = make_uint2((uint32_t)nconst, an_op(w[0].x) == PPI_OP_CONST ? info[0] : kAdjNone);
   a.meta[i] = make_int2(kAdjValid | (rows << 8), ncode);
   atomicMax(a.max_rows, rows);
   atomicMax(a.max_consts, nconst);
   atomicMax(a.max_code, ncode);
}
// Gradient of every program: its chunks' sums in chunk order, written at the
// constants' token positions (0 elsewhere and for a sentinel fitness, NaN
// for a malformed program).  One thread per program.
__global__ void adjoint_finish_kernel(const AdjointFinishArgs a) {
   const int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i >= a.n) return;
   float* grad = a.grad + (size_t)i * a.max_size;
   const int2 meta = a.meta[i];
   if ((meta.x & 0xFF) != kAdjValid) {
      const float gv = (meta.x & 0xFF) == kAdjUnsupported ? __uint_as_float(0x7fc00000u) : 0.0f;
      for (int k = 0; k < a.max_size; ++k) grad[k] = gv;
      return;
   }
   for (int k = 0; k < a.max_size; ++k) grad[k] = 0.0f;
   const uint2* code = a.code + (size_t)i * a.code_stride;
   const int ch = code_header((int)code[0].x);
   const uint2* tab = code + code[ch].y;
   const int nconst = (int)code[ch + 1].x;
   int bad = 0;
   for (int c = 0; c < a.n_chunks; ++c) bad |= a.pbad[(size_t)i * a.n_chunks + c];
   for (int q = 0; q < nconst; ++q) {
      double sum = 0.0;
      for (int c = 0; c < a.n_chunks; ++c) sum += a.psum[((size_t)i * a.n_chunks + c) * a.max_consts + q];
      grad[tab[q].y] = bad ? 0.0f : (float)sum;
   }
}

}  // namespace

cudaError_t launch_adjoint_translate(const AdjointTranslateArgs& a, cudaStream_t s) {
   adjoint_translate_kernel<<<std::max(1, (a.n + 127) / 128), 128, 0, s>>>(a);
   return cudaGetLastError();
}

cudaError_t launch_adjoint_finish(const AdjointFinishArgs& a, cudaStream_t s) {
   adjoint_finish_kernel<<<std::max(1, (a.n + 127) / 128), 128, 0, s>>>(a);
   return cudaGetLastError();
}

size_t adjoint_smem_bytes(int code_words, int max_consts, int rows, int block, int R) {
   const size_t code = ((size_t)(code_words + 1) * sizeof(uint2) + 15) & ~(size_t)15;
   return code + (size_t)max_consts * (block / 32) * sizeof(double) + (size_t)max_consts * block * sizeof(float) +
          (size_t)rows * block * R * sizeof(float);
}

cudaError_t launch_adjoint_r4(int math, int opset, const AdjointArgs& a, int block, int grid, size_t smem,
                              cudaStream_t s);
cudaError_t launch_adjoint_r8(int math, int opset, const AdjointArgs& a, int block, int grid, size_t smem,
                              cudaStream_t s);
cudaError_t adjoint_occupancy_r4(int math, int opset, int block, size_t smem, int* per_sm);
cudaError_t adjoint_occupancy_r8(int math, int opset, int block, size_t smem, int* per_sm);

cudaError_t launch_adjoint(int math, int opset, int R, const AdjointArgs& a, int block, int grid, size_t smem,
                           cudaStream_t s) {
   return R == 4 ? launch_adjoint_r4(math, opset, a, block, grid, smem, s)
                 : launch_adjoint_r8(math, opset, a, block, grid, smem, s);
}

cudaError_t adjoint_occupancy(int math, int opset, int R, int block, size_t smem, int* per_sm) {
   return R == 4 ? adjoint_occupancy_r4(math, opset, block, smem, per_sm)
                 : adjoint_occupancy_r8(math, opset, block, smem, per_sm);
}

}  // namespace ppi
