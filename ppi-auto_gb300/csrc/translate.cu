// translate.cu -- turns each decoded program (PPI's phenotype array, a prefix
// expression evaluated right to left, src/interpreter/accelerator.cl:31) into
// accumulator-machine bytecode for the evaluator.
//
// One thread per program:
//  pass 1 (right to left, the reference's evaluation order) maps every Symbol
//    to its op, checks the stack discipline, and computes for each node its
//    subtree size and register need (Sethi-Ullman number with leaf operands
//    folded into the consuming instruction);
//  pass 2 emits the instructions in an order that evaluates the child with
//    the larger need first.  Subtrees have no side effects, so the order in
//    which independent subtrees are evaluated does not change any value: every
//    node computes exactly the reference's operation on exactly the
//    reference's operands.
// Malformed programs (too few operands, or more than one value left) and
// programs needing more than kSlots registers get the generic form instead:
// the mapped tokens in evaluation order, run by a stack interpreter with the
// reference's stack semantics.
#include "ppi_internal.cuh"

namespace ppi {
namespace {

constexpr uint32_t kGenericEnd = 0xFFFFu;

// Node record in the translator scratch: x = op | need << 8 | subtree << 16.
__device__ __forceinline__ uint2 node_pack(int op, int need, int sub, uint32_t imm) {
   return make_uint2((uint32_t)op | ((uint32_t)min(need, 255) << 8) | ((uint32_t)sub << 16), imm);
}
__device__ __forceinline__ int node_op(uint2 w) { return (int)(w.x & 0xFFu); }
__device__ __forceinline__ int node_need(uint2 w) { return (int)((w.x >> 8) & 0xFFu); }
__device__ __forceinline__ int node_sub(uint2 w) { return (int)(w.x >> 16); }

// Frame of the emission walk: node | d << 16 | state << 24.
__device__ __forceinline__ uint32_t frame(int node, int d, int st) {
   return (uint32_t)node | ((uint32_t)d << 16) | ((uint32_t)st << 24);
}

__global__ void translate_kernel(const TranslateArgs a) {
   if (blockIdx.x == 0 && threadIdx.x == 0) {
      *a.best_key = ~0ull;
      a.counters[0] = 0u;
      a.counters[1] = 0u;
      *a.status = 0;
   }
   const int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i >= a.n) return;
   const int sz = a.size[i];
   if (sz <= 0 || sz > a.max_size) {
      a.meta[i] = make_int2(kKindInvalid, 0);
      return;
   }
   const int32_t* ph = a.phenotype + (size_t)i * a.max_size;
   const float* eph = a.ephemeral + (size_t)i * a.max_size;
   uint2* w = a.work + (size_t)i * 2 * a.max_size;
   uint32_t* frames = reinterpret_cast<uint32_t*>(w + a.max_size);
   uint2* code = a.code + (size_t)i * a.code_stride;
   const uint32_t qnan = 0x7fc00000u;

   // ---- pass 1 -----------------------------------------------------------
   int depth = 0, stack_need = 0;
   bool malformed = false;
   for (int k = sz - 1; k >= 0; --k) {
      const int sym = ph[k];
      int op = PPI_OP_INVALID;
      uint32_t imm = qnan;
      const int li = sym - a.lut_min;
      if (li >= 0 && li < a.lut_len) {
         const int2 e = a.lut[li];
         op = e.x;
         if (op == PPI_OP_LITERAL) imm = (uint32_t)e.y;
         else if (op == PPI_OP_CONST) imm = __float_as_uint(eph[k]);
         else if (op == PPI_OP_ATTRIBUTE) {
            const float v = eph[k];
            if (v >= 0.0f && v < (float)a.ncol) imm = (uint32_t)(int)v;
            else { op = PPI_OP_INVALID; imm = qnan; }   // defined as NaN (see ppi_gpu.h)
         }
      }
      const int ar = op_arity(op);
      int before = depth;
      if (before < ar) { malformed = true; before = ar; }   // missing operands read as NaN
      depth = before - ar + 1;
      stack_need = max(stack_need, max(before, depth));
      int need = 0, sub = 1;
      if (!malformed && ar > 0) {
         const int c0 = k + 1;
         const uint2 w0 = w[c0];
         const bool leaf0 = op_arity(node_op(w0)) == 0;
         sub += node_sub(w0);
         if (ar == 1) {
            need = node_need(w0);
         } else {
            const int c1 = c0 + node_sub(w0);
            const uint2 w1 = w[c1];
            const bool leaf1 = op_arity(node_op(w1)) == 0;
            sub += node_sub(w1);
            const int n0 = node_need(w0), n1 = node_need(w1);
            if (ar == 2) {
               if (leaf0 && leaf1) need = 0;
               else if (leaf1) need = n0;
               else if (leaf0) need = n1;
               else need = max(n0, n1) + (n0 == n1 ? 1 : 0);
            } else {
               const uint2 w2 = w[c1 + node_sub(w1)];
               sub += node_sub(w2);
               int x = n0, y = n1, z = node_need(w2);   // sort descending
               if (x < y) { int t = x; x = y; y = t; }
               if (y < z) { int t = y; y = z; z = t; }
               if (x < y) { int t = x; x = y; y = t; }
               need = max(x, max(y + 1, z + 2));
            }
         }
      }
      w[k] = node_pack(op, need, sub, imm);
   }
   if (depth != 1) malformed = true;

   // ---- pass 2: register code ---------------------------------------------
   const int cap = a.code_stride;
   int ncode = 0;
   bool fast = !malformed && node_need(w[0]) <= kSlots && node_sub(w[0]) == sz;
   if (fast) {
      int fp = 0;
      frames[fp++] = frame(0, 0, 0);
      auto emit = [&](uint32_t id, uint32_t imm) {
         if (ncode < cap) code[ncode] = make_uint2(id, imm);
         ++ncode;
      };
      auto is_leaf = [&](int node) { return op_arity(node_op(w[node])) == 0; };
      auto leaf_attr = [&](int node) { return node_op(w[node]) == PPI_OP_ATTRIBUTE; };
      const uint32_t slot0 = (uint32_t)a.ncol;   // row of slot 0
      while (fp > 0) {
         const uint32_t f = frames[fp - 1];
         const int node = (int)(f & 0xFFFFu), d = (int)((f >> 16) & 0xFFu), st = (int)(f >> 24);
         const uint2 wn = w[node];
         const int op = node_op(wn);
         const int ar = op_arity(op);
         if (ar == 0) {
            emit(op == PPI_OP_ATTRIBUTE ? M_LD_ROW : M_LD_C, wn.y);
            --fp;
            continue;
         }
         const int c0 = node + 1;
         if (ar == 1) {
            if (st == 0) { frames[fp - 1] = frame(node, d, 1); frames[fp++] = frame(c0, d, 0); }
            else { emit(M_UN + (uint32_t)(op - PPI_OP_NOT), 0u); --fp; }
            continue;
         }
         const int c1 = c0 + node_sub(w[c0]);
         if (ar == 2) {
            const uint32_t bo = (uint32_t)(op - PPI_OP_AND);
            const bool l0 = is_leaf(c0), l1 = is_leaf(c1);
            if (l0 && l1) {
               emit(leaf_attr(c0) ? M_LD_ROW : M_LD_C, w[c0].y);
               emit((leaf_attr(c1) ? M_BR_L : M_BC_L) + bo, w[c1].y);
               --fp;
            } else if (l1) {
               if (st == 0) { frames[fp - 1] = frame(node, d, 1); frames[fp++] = frame(c0, d, 0); }
               else { emit((leaf_attr(c1) ? M_BR_L : M_BC_L) + bo, w[c1].y); --fp; }
            } else if (l0) {
               if (st == 0) { frames[fp - 1] = frame(node, d, 1); frames[fp++] = frame(c1, d, 0); }
               else { emit((leaf_attr(c0) ? M_BR_R : M_BC_R) + bo, w[c0].y); --fp; }
            } else {
               const bool left_first = node_need(w[c0]) >= node_need(w[c1]);
               const int first = left_first ? c0 : c1, second = left_first ? c1 : c0;
               if (st == 0) {
                  frames[fp - 1] = frame(node, d, 1);
                  frames[fp++] = frame(first, d, 0);
               } else if (st == 1) {
                  emit(M_PUSH, slot0 + (uint32_t)d);
                  frames[fp - 1] = frame(node, d, 2);
                  frames[fp++] = frame(second, d + 1, 0);
               } else {
                  // slot d holds `first`, acc holds `second`
                  emit((left_first ? M_BR_R : M_BR_L) + bo, slot0 + (uint32_t)d);
                  --fp;
               }
            }
            continue;
         }
         // ternary IF_THEN_ELSE(cond = c0, then = c1, else = c2)
         const int c2 = c1 + node_sub(w[c1]);
         int x[3] = {c0, c1, c2};
         // order by need, descending (stable)
         for (int p = 0; p < 2; ++p)
            for (int q = 0; q < 2 - p; ++q)
               if (node_need(w[x[q]]) < node_need(w[x[q + 1]])) { int t = x[q]; x[q] = x[q + 1]; x[q + 1] = t; }
         if (st == 0) {
            frames[fp - 1] = frame(node, d, 1);
            frames[fp++] = frame(x[0], d, 0);
         } else if (st == 1) {
            emit(M_PUSH, slot0 + (uint32_t)d);
            frames[fp - 1] = frame(node, d, 2);
            frames[fp++] = frame(x[1], d + 1, 0);
         } else if (st == 2) {
            emit(M_PUSH, slot0 + (uint32_t)(d + 1));
            frames[fp - 1] = frame(node, d, 3);
            frames[fp++] = frame(x[2], d + 2, 0);
         } else {
            // x[0] -> row a (1), x[1] -> row b (2), x[2] -> acc (0)
            auto reg = [&](int child) { return child == x[0] ? 1 : (child == x[1] ? 2 : 0); };
            const int rc = reg(c0), rt = reg(c1), re = reg(c2);
            int perm = 0;
            for (int p = 0; p < 6; ++p)
               if (ite_role(p, 0) == rc && ite_role(p, 1) == rt && ite_role(p, 2) == re) perm = p;
            emit(M_ITE + (uint32_t)perm, (slot0 + (uint32_t)d) | ((slot0 + (uint32_t)d + 1) << 16));
            --fp;
         }
      }
      emit(M_END, 0u);
      if (ncode > cap) fast = false;
   }
   if (fast) {
      a.meta[i] = make_int2(kKindFast, ncode);
      return;
   }
   // ---- generic form: tokens in evaluation order ---------------------------
   if (stack_need > kGenericStack) {
      a.meta[i] = make_int2(kKindUnsupported, 0);
      return;
   }
   for (int k = sz - 1; k >= 0; --k) {
      const uint2 wn = w[k];
      code[sz - 1 - k] = make_uint2((uint32_t)node_op(wn), wn.y);
   }
   code[sz] = make_uint2(kGenericEnd, 0u);
   a.meta[i] = make_int2(kKindGeneric, sz + 1);
}

}  // namespace

cudaError_t launch_translate(const TranslateArgs& a, cudaStream_t s) {
   const int block = 128;
   const int grid = max(1, (a.n + block - 1) / block);
   translate_kernel<<<grid, block, 0, s>>>(a);
   return cudaGetLastError();
}

}  // namespace ppi
