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
// Pass 1 also folds constant subexpressions: an operator whose operands are
// all constants (CONST, literal, or already folded) becomes a literal whose
// value is computed here with the same device functions (unop/binop) and the
// same math mode the evaluator uses, so the folded value is bit-identical to
// what every record would compute.
// Malformed programs (too few operands, or more than one value left) and
// programs needing more than kSlots registers get the generic form instead:
// the mapped tokens in evaluation order, run by a stack interpreter with the
// reference's stack semantics.
// Between the passes the distinct record columns the program reads (after
// folding) are listed in the code header and given tile rows after the slot
// rows, so the evaluator stages only those columns (and the target).  A
// program's tile row count decides its pass: the main pass (rows within the
// launch's main budget), the wide pass (within the wide budget), or the
// generic form.
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

// Symbol -> (op, immediate): literal value, constant, or validated column.
__device__ __forceinline__ void map_token(const TranslateArgs& a, int sym, float e, int* op_out,
                                          uint32_t* imm_out) {
   const uint32_t qnan = 0x7fc00000u;
   int op = PPI_OP_INVALID;
   uint32_t imm = qnan;
   const int li = sym - a.lut_min;
   if (li >= 0 && li < a.lut_len) {
      const int2 ent = a.lut[li];
      op = ent.x;
      if (op == PPI_OP_LITERAL) imm = (uint32_t)ent.y;
      else if (op == PPI_OP_CONST) imm = __float_as_uint(e);
      else if (op == PPI_OP_ATTRIBUTE) {
         if (e >= 0.0f && e < (float)a.ncol) imm = (uint32_t)(int)e;
         else { op = PPI_OP_INVALID; imm = qnan; }   // defined as NaN (see ppi_gpu.h)
      }
   }
   *op_out = op;
   *imm_out = imm;
}

// Value of op applied to constant operands, in math mode MATH.
template <int MATH>
__device__ float fold(int op, float x0, float x1, float x2, int prot) {
   switch (op) {
#define PPI_FU(OP) case OP: return unop<OP, MATH>(x0, prot);
      PPI_FU(PPI_OP_NOT) PPI_FU(PPI_OP_ABS) PPI_FU(PPI_OP_POW2) PPI_FU(PPI_OP_POW3)
      PPI_FU(PPI_OP_POW4) PPI_FU(PPI_OP_POW5) PPI_FU(PPI_OP_NEG) PPI_FU(PPI_OP_ROUND)
      PPI_FU(PPI_OP_CEIL) PPI_FU(PPI_OP_FLOOR) PPI_FU(PPI_OP_EXP) PPI_FU(PPI_OP_EXP10)
      PPI_FU(PPI_OP_EXP2) PPI_FU(PPI_OP_SIN) PPI_FU(PPI_OP_COS) PPI_FU(PPI_OP_STEP)
      PPI_FU(PPI_OP_SIGN) PPI_FU(PPI_OP_LOGISTIC) PPI_FU(PPI_OP_GAMMA) PPI_FU(PPI_OP_GAUSS)
      PPI_FU(PPI_OP_SQRT) PPI_FU(PPI_OP_LOG) PPI_FU(PPI_OP_LOG10) PPI_FU(PPI_OP_LOG2)
      PPI_FU(PPI_OP_TAN)
#undef PPI_FU
#define PPI_FB(OP) case OP: return binop<OP, MATH>(x0, x1, prot);
      PPI_FB(PPI_OP_AND) PPI_FB(PPI_OP_OR) PPI_FB(PPI_OP_XOR) PPI_FB(PPI_OP_GREATER)
      PPI_FB(PPI_OP_GREATEREQUAL) PPI_FB(PPI_OP_LESS) PPI_FB(PPI_OP_LESSEQUAL)
      PPI_FB(PPI_OP_EQUAL) PPI_FB(PPI_OP_NOTEQUAL) PPI_FB(PPI_OP_ADD) PPI_FB(PPI_OP_SUB)
      PPI_FB(PPI_OP_MULT) PPI_FB(PPI_OP_MEAN) PPI_FB(PPI_OP_MAX) PPI_FB(PPI_OP_MIN)
      PPI_FB(PPI_OP_MOD) PPI_FB(PPI_OP_POW) PPI_FB(PPI_OP_DIV)
#undef PPI_FB
   case PPI_OP_IF_THEN_ELSE: return truthy(x0) ? x1 : x2;
   default: return __uint_as_float(0x7fc00000u);
   }
}

__device__ __forceinline__ bool is_const_leaf(int op) { return op == PPI_OP_CONST || op == PPI_OP_LITERAL; }

// Translation of program i (valid size): writes its code, returns its meta.
// MAPPED: ph / eph already hold each token's op and immediate bits (mapped
// by the whole warp before the walk); else the Symbols and ephemerals.
template <int MATH, bool MAPPED>
__device__ int2 translate_program(const TranslateArgs& ta, int i, int sz, const int32_t* ph, const float* eph,
                                  uint2* w, uint32_t* frames) {
   uint2* code = ta.code + (size_t)i * ta.code_stride;

   // ---- pass 1 -----------------------------------------------------------
   int depth = 0, stack_need = 0;
   bool malformed = false;
   for (int k = sz - 1; k >= 0; --k) {
      int op;
      uint32_t imm;
      if constexpr (MAPPED) {
         op = ph[k];
         imm = __float_as_uint(eph[k]);
      } else {
         map_token(ta, ph[k], eph[k], &op, &imm);
      }
      const int ar = op_arity(op);
      int before = depth;
      if (before < ar) { malformed = true; before = ar; }   // missing operands read as NaN
      depth = before - ar + 1;
      stack_need = max(stack_need, max(before, depth));
      int need = 0, sub = 1;
      if (!malformed && ar > 0 && ta.fold) {
         // children: c0 = k+1, c1 after c0's subtree, c2 after c1's
         const int c0 = k + 1;
         const int c1 = ar > 1 ? c0 + node_sub(w[c0]) : c0;
         const int c2 = ar > 2 ? c1 + node_sub(w[c1]) : c1;
         bool all_const = is_const_leaf(node_op(w[c0]));
         if (ar > 1) all_const = all_const && is_const_leaf(node_op(w[c1]));
         if (ar > 2) all_const = all_const && is_const_leaf(node_op(w[c2]));
         if (all_const) {
            const float v = fold<MATH>(op, __uint_as_float(w[c0].y), __uint_as_float(w[c1].y),
                                       __uint_as_float(w[c2].y), ta.prot);
            int s = 1 + node_sub(w[c0]);
            if (ar > 1) s += node_sub(w[c1]);
            if (ar > 2) s += node_sub(w[c2]);
            w[k] = node_pack(PPI_OP_LITERAL, 0, s, __float_as_uint(v));
            continue;
         }
      }
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

   // ---- columns: distinct record columns read, in order of first use ------
   // The tile stages them all when they fit the pass's row budget; else the
   // most-read ones, and the rest are read from global memory by the
   // instructions that use them.
   const int cap = ta.code_stride;
   const int slots = malformed ? 0 : node_need(w[0]);
   bool fast = !malformed && slots <= kSlots && node_sub(w[0]) == sz;
   int ncols = 0, nstaged = 0, rows = 0;
   if (fast) {
      // cols[j] = column | min(references, 127) << 24 | staged << 31; each
      // attribute leaf's immediate temporarily holds its column's j
      uint32_t* cols = frames + ta.max_size;   // upper half: pass 2 uses at most sz frames
      for (int p = 0; p < sz;) {
         const uint2 wn = w[p];
         const int op = node_op(wn);
         if (op == PPI_OP_LITERAL) { p += node_sub(wn); continue; }   // a folded subtree is one literal
         if (op == PPI_OP_ATTRIBUTE) {
            int j = 0;
            while (j < ncols && (cols[j] & 0xFFFFFFu) != wn.y) ++j;
            if (j == ncols) cols[ncols++] = wn.y | (1u << 24);
            else if (((cols[j] >> 24) & 0x7Fu) < 127u) cols[j] += 1u << 24;
            w[p].y = (uint32_t)j;
         }
         ++p;
      }
      // the main pass when every column fits its tile, else the wide pass
      // with as many columns staged as its tile holds
      const bool main_pass = slots + ncols + 1 <= ta.rows_main;
      const int budget = main_pass ? ta.rows_main : ta.rows_wide;
      if (slots + 1 > budget || code_header(ncols) >= cap) fast = false;
      if (fast) {
         nstaged = min(ncols, budget - slots - 1);
         for (int q = 0; q < nstaged; ++q) {
            int pick = -1;
            uint32_t most = 0;
            for (int j = 0; j < ncols; ++j) {
               const uint32_t c = (cols[j] >> 24) & 0x7Fu;
               if (!(cols[j] >> 31) && (pick < 0 || c > most)) { pick = j; most = c; }
            }
            cols[pick] |= 0x80000000u;
         }
         rows = slots + nstaged + 1;
         // header: staged columns (tile rows slots..), then the direct ones,
         // two per entry from code[1]
         uint32_t* list = reinterpret_cast<uint32_t*>(code + 1);
         int e = 0;
         for (int j = 0; j < ncols; ++j)
            if (cols[j] >> 31) list[e++] = cols[j] & 0xFFFFFFu;
         for (int j = 0; j < ncols; ++j)
            if (!(cols[j] >> 31)) list[e++] = cols[j] & 0xFFFFFFu;
         if (ncols & 1) list[ncols] = 0u;
         code[0] = make_uint2((uint32_t)nstaged, (uint32_t)slots | ((uint32_t)(ncols - nstaged) << 16));
         // operand of each column: its tile row, or the column read directly
         int row = slots;
         for (int j = 0; j < ncols; ++j)
            cols[j] = (cols[j] >> 31) ? (uint32_t)row++ : (kDirectColumn | (cols[j] & 0xFFFFFFu));
         for (int p = 0; p < sz;) {
            const uint2 wn = w[p];
            const int op = node_op(wn);
            if (op == PPI_OP_LITERAL) { p += node_sub(wn); continue; }
            if (op == PPI_OP_ATTRIBUTE) w[p].y = cols[wn.y];
            ++p;
         }
      }
   }

   // ---- pass 2: register code ---------------------------------------------
   int ncode = code_header(ncols);
   if (fast) {
      int fp = 0;
      frames[fp++] = frame(0, 0, 0);
      // a push followed by a load of a tile row becomes one M_PUSH_LD
      bool after_push = false;
      uint32_t push_row = 0u;
      auto emit = [&](uint32_t id, uint32_t imm) {
         if (after_push && id == M_LD_ROW && imm < 0x10000u && push_row < 0x10000u) {
            if (ncode - 1 < cap) code[ncode - 1] = make_uint2(M_PUSH_LD, push_row | (imm << 16));
            after_push = false;
            return;
         }
         if (ncode < cap) code[ncode] = make_uint2(id, imm);
         ++ncode;
         after_push = id == M_PUSH;
         push_row = imm;
      };
      auto is_leaf = [&](int node) { return op_arity(node_op(w[node])) == 0; };
      auto leaf_attr = [&](int node) { return node_op(w[node]) == PPI_OP_ATTRIBUTE; };
      const uint32_t slot0 = 0u;   // row of slot 0
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
            // + and x are commutative bit for bit in IEEE arithmetic: their
            // operand-first forms (_R) become accumulator-first ones (_L), so
            // fewer distinct cases run hot in the interpreter
            const bool comm = op == PPI_OP_ADD || op == PPI_OP_MULT;
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
               else { emit((leaf_attr(c0) ? (comm ? M_BR_L : M_BR_R) : (comm ? M_BC_L : M_BC_R)) + bo, w[c0].y); --fp; }
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
                  emit((left_first && !comm ? M_BR_R : M_BR_L) + bo, slot0 + (uint32_t)d);
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
      const int kind = nstaged == ncols && rows <= ta.rows_main ? kKindFast : kKindWide;
      return make_int2(kind | (rows << 8), ncode);
   }
   // ---- generic form: tokens in evaluation order ---------------------------
   if (stack_need > kGenericStack) return make_int2(kKindUnsupported, 0);
   code[0] = make_uint2(0u, 0u);          // no staged columns, no slots: the target is row 0
   for (int k = sz - 1; k >= 0; --k) {    // the original tokens: nothing folded
      int op;
      uint32_t imm;
      if constexpr (MAPPED) {
         op = ph[k];
         imm = __float_as_uint(eph[k]);
      } else {
         map_token(ta, ph[k], eph[k], &op, &imm);
      }
      code[1 + sz - 1 - k] = make_uint2((uint32_t)op, imm);
   }
   code[1 + sz] = make_uint2(kGenericEnd, 0u);
   return make_int2(kKindGeneric | (1 << 8), sz + 2);
}

// Shared memory of one program's translation (WARP = true): its tokens and
// ephemerals, the node words and both passes' frames.
__host__ __device__ inline size_t translate_smem_bytes(int max_size) { return (size_t)max_size * 24 + 16; }
constexpr size_t kTranslateSmemMax = 200 * 1024;

// One warp per program (WARP = true: populations resident in one wave): the
// warp copies the program's tokens into shared memory with coalesced loads
// and lane 0 walks it there (the translation is a serial walk per program;
// one thread per program would put 32 different walks in one warp, which
// diverge and run one after another).  One thread per program (WARP = false:
// larger populations, whose many resident warps hide the latency) with the
// scratch in the global work array.
template <int MATH, bool WARP>
__global__ void translate_kernel(const TranslateArgs a) {
   extern __shared__ __align__(16) unsigned char tsmem[];
   if (blockIdx.x == 0 && threadIdx.x == 0) {
      *a.best_key = ~0ull;
      *a.status = 0;
   }
   const int ms = a.max_size;
   const int32_t* ph;
   const float* eph;
   uint2* w;
   uint32_t* frames;
   int i;
   if constexpr (WARP) {
      // one program per 32-thread CTA: all lanes copy and map the tokens,
      // lane 0 translates
      i = blockIdx.x;
      int32_t* s_ph = reinterpret_cast<int32_t*>(tsmem);
      float* s_eph = reinterpret_cast<float*>(s_ph + ms);
      uint2* s_w = reinterpret_cast<uint2*>(s_eph + ms);   // 2 ms words in: 8-byte aligned
      uint32_t* s_fr = reinterpret_cast<uint32_t*>(s_w + ms);
      if (i >= a.n) return;
      const int sz_all = min(max(a.size[i], 0), ms);
      TranslateArgs tm = a;   // the mapping needs the program's dataset width
      if (a.pop_of) tm.ncol = a.pops[a.pop_of[i]].ncol;
      for (int k = threadIdx.x; k < sz_all; k += blockDim.x) {
         int op;
         uint32_t imm;
         map_token(tm, a.phenotype[(size_t)i * ms + k], a.ephemeral[(size_t)i * ms + k], &op, &imm);
         s_ph[k] = op;
         s_eph[k] = __uint_as_float(imm);
      }
      __syncwarp();
      if (threadIdx.x != 0) return;
      ph = s_ph;
      eph = s_eph;
      w = s_w;
      frames = s_fr;
   } else {
      i = blockIdx.x * blockDim.x + threadIdx.x;
      ph = a.phenotype + (size_t)i * ms;
      eph = a.ephemeral + (size_t)i * ms;
      w = a.work + (size_t)i * 2 * ms;
      frames = reinterpret_cast<uint32_t*>(w + ms);
   }
   if (i >= a.n) return;
   const int sz = a.size[i];
   TranslateArgs ta = a;
   long long nlin = a.nlin;
   if (a.pop_of) {
      // batch: this program's dataset width and protection
      const PopDesc& pd = a.pops[a.pop_of[i]];
      ta.ncol = pd.ncol;
      ta.prot = pd.prot;
      nlin = pd.nlin;
   }
   const bool valid = sz > 0 && sz <= a.max_size;   // sizes outside [1, max_size] are size 0
   const int2 m = valid ? translate_program<MATH, WARP>(ta, i, sz, ph, eph, w, frames) : make_int2(kKindInvalid, 0);
   a.meta[i] = m;
   const int kind = meta_kind(m);
   const unsigned long long work = valid ? (unsigned long long)sz * (unsigned long long)nlin : 0ull;
   if (a.pop_of) {
      // work order of a batch: cost buckets (cost = size x records), largest
      // first; the wide pass's programs in their own buckets
      int b = work ? 64 - __clzll(work) : 0;   // 0..63
      if (kind == kKindWide) b += 64;
      a.bucket_of[i] = (unsigned char)b;
      atomicAdd(&a.bucket_count[b], 1u);
   } else if (kind == kKindWide) {
      a.wide_list[atomicAdd(&a.stats->wide, 1u)] = i;
   }
}

template <int MATH>
cudaError_t launch_translate_math(const TranslateArgs& a, cudaStream_t s, int sm_count) {
   const size_t per_prog = translate_smem_bytes(a.max_size);
   if (a.n <= sm_count * 64 && per_prog <= kTranslateSmemMax) {
      // a population resident in one wave: a warp per program
      const cudaError_t e = cudaFuncSetAttribute(translate_kernel<MATH, true>,
                                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)per_prog);
      if (e != cudaSuccess) return e;
      translate_kernel<MATH, true><<<max(1, a.n), 32, per_prog, s>>>(a);
      return cudaGetLastError();
   }
   // larger populations: a thread per program, scratch in global memory (many
   // resident warps hide its latency; staging every thread's scratch in
   // shared memory left one warp per SM for 256-token programs, measured 3 %
   // slower on the uneven batch)
   const int grid = max(1, (a.n + 127) / 128);
   translate_kernel<MATH, false><<<grid, 128, 0, s>>>(a);
   return cudaGetLastError();
}

}  // namespace

cudaError_t launch_translate(int math, const TranslateArgs& a, cudaStream_t s) {
   int dev = 0, sm_count = 0;
   cudaGetDevice(&dev);
   cudaDeviceGetAttribute(&sm_count, cudaDevAttrMultiProcessorCount, dev);
   if (math == kMathParity) return launch_translate_math<kMathParity>(a, s, sm_count);
   if (math == kMathNative) return launch_translate_math<kMathNative>(a, s, sm_count);
   return launch_translate_math<kMathFast>(a, s, sm_count);
}

}  // namespace ppi
