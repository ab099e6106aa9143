// evaluate_impl.cuh -- fitness of every program over every record, on sm_103a.
//
// Execution model (GB300-first):
//   * one CTA of P threads evaluates one program at a time, pulling program
//     indices from a device work queue (persistent grid, one wave of CTAs);
//   * the dataset is column-major in HBM; each CTA stages a tile of
//     T = P * R records into shared memory with 16-byte vector loads: only
//     the columns the program reads (listed by the translator) and the
//     target, so shared memory per CTA follows the program, not the dataset
//     width, and attribute reads are conflict-free LDS.128;
//   * the program's bytecode sits in shared memory and every warp walks it in
//     lock step: instruction dispatch is warp-uniform (no divergence) and each
//     instruction is applied to the R records a thread holds in its
//     accumulator registers (R-way ILP); operands other than the accumulator
//     are shared-memory rows (data columns and slots);
//   * errors are reduced in exactly the order of the reference strategy:
//       PDP (lanes == T): lane = tile position, accumulated in registers;
//       PDP (other lanes) and PP (lanes == 1): per-lane accumulators in
//         shared memory, each lane adding its records in increasing order;
//       DP: per-group trees in shared memory, groups added in order;
//     then the reference's local tree (accelerator.cl:157-167, 252-262);
//   * fitness, alpha*size and the arg-min (64-bit packed atomicMin) are fused
//     into the same kernel; the last CTA to finish writes the best index;
//   * two passes with different shared-memory budgets: the main pass runs
//     every program whose tile fits its row budget (sized for occupancy),
//     the wide pass the few that need more rows.
#pragma once

#include <atomic>

#include "ppi_internal.cuh"

namespace ppi {
namespace ev {

constexpr uint32_t kGenericEnd = 0xFFFFu;

__device__ __forceinline__ size_t code_bytes(int code_stride) {
   return ((size_t)(code_stride + 1) * sizeof(uint2) + 15) & ~(size_t)15;
}

// Tile layout: a thread's R records are R/4 quads of consecutive records;
// quad i of thread tid starts at tile position (i*P + tid)*4, so the 16-byte
// accesses of a warp cover 512 contiguous bytes (no bank conflicts for any R).
__device__ __forceinline__ int tile_pos(int tid, int r, int P) { return ((r >> 2) * P + tid) * 4 + (r & 3); }

// `p` points at this thread's first quad of a row; quads are 4*P floats apart.
template <int R>
__device__ __forceinline__ void load_row(const float* p, int P, float (&x)[R]) {
   static_assert(R % 4 == 0, "rows are read as float4");
#pragma unroll
   for (int i = 0; i < R / 4; ++i) {
      const float4 u = *reinterpret_cast<const float4*>(p + (size_t)i * 4 * P);
      x[4 * i] = u.x; x[4 * i + 1] = u.y; x[4 * i + 2] = u.z; x[4 * i + 3] = u.w;
   }
}
// The current tile's view of the dataset, for operands read directly from
// global memory: base = data + tile's first record, avail = records from
// there to the end of a column's storage (ld - first record), vec = 16-byte
// loads allowed (tile base a multiple of 4 records; ld is one).
struct Direct {
   const float* base;
   int ld, avail, vec;
};

// x = the operand of an instruction: tile row `imm`, or with kDirectColumn the
// record column read from global memory (positions at or past ld read 0, as a
// staged row has them).  Kernels built with D = 0 run only programs whose
// columns are all staged, and carry no code for direct reads; D = 2 reads
// whole 16-byte quads only (tiles that start on a multiple of 4 records: PP,
// PDP, and DP when dp_tile_groups found a whole-quad group count), D = 1
// also the ragged ones.  The scalar path's code, unused in PP and PDP, cost
// the wide pass 7 % (instruction-cache misses) before D = 2.
template <int D, int R>
__device__ __forceinline__ void load_operand(uint32_t imm, const float* mine, int T, int P, int tid,
                                             const Direct& g, float (&x)[R]) {
   if (!D || !(imm & kDirectColumn)) {
      load_row(mine + (size_t)imm * T, P, x);
      return;
   }
   const float* col = g.base + (size_t)(imm & ~kDirectColumn) * g.ld;
#pragma unroll
   for (int i = 0; i < R / 4; ++i) {
      const int pos = (i * P + tid) * 4;
      if constexpr (D == 2) {
         // whole quads only: every tile starts on a multiple of 4 records and
         // the padded column length is one, so a quad is either inside the
         // column or past its end (read as 0 by the else branch).  This form
         // measured 8 % faster on the uneven batch than a zero-initialised
         // quad with a conditional load, or than the condition without g.vec.
         if (g.vec && pos + 3 < g.avail) {
            const float4 u = __ldg(reinterpret_cast<const float4*>(col + pos));
            x[4 * i] = u.x; x[4 * i + 1] = u.y; x[4 * i + 2] = u.z; x[4 * i + 3] = u.w;
         } else {
#pragma unroll
            for (int q = 0; q < 4; ++q) x[4 * i + q] = 0.0f;
         }
      } else if (g.vec && pos + 3 < g.avail) {
         const float4 u = __ldg(reinterpret_cast<const float4*>(col + pos));
         x[4 * i] = u.x; x[4 * i + 1] = u.y; x[4 * i + 2] = u.z; x[4 * i + 3] = u.w;
      } else {
#pragma unroll
         for (int q = 0; q < 4; ++q) x[4 * i + q] = (pos + q < g.avail) ? __ldg(col + pos + q) : 0.0f;
      }
   }
}

template <int R>
__device__ __forceinline__ void store_row(float* p, int P, const float (&x)[R]) {
#pragma unroll
   for (int i = 0; i < R / 4; ++i)
      *reinterpret_cast<float4*>(p + (size_t)i * 4 * P) = make_float4(x[4 * i], x[4 * i + 1], x[4 * i + 2], x[4 * i + 3]);
}

// ---- bytecode path -------------------------------------------------------------
// Opcode sets of the bytecode path.  FULL: every opcode.  ARITH: the
// arithmetic grammars' opcodes (+ - * / sin cos exp log sqrt ^2 abs neg); a
// program using anything else never reaches an ARITH kernel (the host picks
// the set from the symbol table).
#define PPI_FULL_UNARY(X) X(PPI_OP_NOT) X(PPI_OP_ABS) X(PPI_OP_POW2) X(PPI_OP_POW3) X(PPI_OP_POW4) \
   X(PPI_OP_POW5) X(PPI_OP_NEG) X(PPI_OP_ROUND) X(PPI_OP_CEIL) X(PPI_OP_FLOOR) X(PPI_OP_EXP)      \
   X(PPI_OP_EXP10) X(PPI_OP_EXP2) X(PPI_OP_SIN) X(PPI_OP_COS) X(PPI_OP_STEP) X(PPI_OP_SIGN)       \
   X(PPI_OP_LOGISTIC) X(PPI_OP_GAMMA) X(PPI_OP_GAUSS) X(PPI_OP_SQRT) X(PPI_OP_LOG)               \
   X(PPI_OP_LOG10) X(PPI_OP_LOG2) X(PPI_OP_TAN)
#define PPI_FULL_BINARY(X) X(PPI_OP_AND) X(PPI_OP_OR) X(PPI_OP_XOR) X(PPI_OP_GREATER)           \
   X(PPI_OP_GREATEREQUAL) X(PPI_OP_LESS) X(PPI_OP_LESSEQUAL) X(PPI_OP_EQUAL) X(PPI_OP_NOTEQUAL) \
   X(PPI_OP_ADD) X(PPI_OP_SUB) X(PPI_OP_MULT) X(PPI_OP_MEAN) X(PPI_OP_MAX) X(PPI_OP_MIN)        \
   X(PPI_OP_MOD) X(PPI_OP_POW) X(PPI_OP_DIV)
#define PPI_ARITH_UNARY(X) X(PPI_OP_ABS) X(PPI_OP_POW2) X(PPI_OP_NEG) X(PPI_OP_EXP) X(PPI_OP_SIN) \
   X(PPI_OP_COS) X(PPI_OP_SQRT) X(PPI_OP_LOG)
#define PPI_ARITH_BINARY(X) X(PPI_OP_ADD) X(PPI_OP_SUB) X(PPI_OP_MULT) X(PPI_OP_DIV)

// Membership in a set, from the same lists the kernels' cases come from.
#define PPI_IS_OP(OP) op == (OP) ||
__host__ __device__ constexpr bool arith_unary(int op) { return PPI_ARITH_UNARY(PPI_IS_OP) false; }
__host__ __device__ constexpr bool arith_binary(int op) { return PPI_ARITH_BINARY(PPI_IS_OP) false; }
__host__ __device__ constexpr bool full_unary(int op) { return PPI_FULL_UNARY(PPI_IS_OP) false; }
__host__ __device__ constexpr bool full_binary(int op) { return PPI_FULL_BINARY(PPI_IS_OP) false; }
#undef PPI_IS_OP

// Instruction ids that the kernel of opcode set OPSET has a case for.
template <int OPSET>
__host__ __device__ constexpr bool opset_has(uint32_t id) {
   if (id == M_END || id == M_LD_ROW || id == M_LD_C || id == M_PUSH || id == M_PUSH_LD) return true;
   if (id >= M_UN && id < M_BR_L) {
      const int op = PPI_OP_NOT + (int)(id - M_UN);
      return OPSET == kOpsetArith ? arith_unary(op) : full_unary(op);
   }
   if (id >= M_BR_L && id < M_ITE) {
      const int op = PPI_OP_AND + (int)((id - M_BR_L) % 18u);
      return OPSET == kOpsetArith ? arith_binary(op) : full_binary(op);
   }
   return OPSET == kOpsetFull && id >= M_ITE && id < M_PUSH_LD;
}

// True when instruction w can run in a kernel of opcode set OPSET over a
// tile of `rows` rows: its id is one of the kernel's cases, and every operand
// it names is a row of the tile or, where the kernel reads columns directly
// (direct), a column of the dataset.
template <int OPSET>
__device__ __forceinline__ bool instruction_ok(uint2 w, int rows, int ncol, bool direct) {
   const uint32_t id = w.x, imm = w.y, nrows = (uint32_t)rows;
   if (!opset_has<OPSET>(id)) return false;
   if (id == M_LD_ROW || (id >= M_BR_L && id < M_BC_L)) {
      if (imm & kDirectColumn) return direct && (imm & ~kDirectColumn) < (uint32_t)ncol;
      return imm < nrows;
   }
   if (id == M_PUSH) return imm < nrows;
   if (id == M_PUSH_LD || (id >= M_ITE && id < M_PUSH_LD)) return (imm & 0xFFFFu) < nrows && (imm >> 16) < nrows;
   return true;
}

// Unary opcodes whose fast-math routine is long enough that R inlined copies
// per case crowd the instruction cache (the interpreter is bound by
// instruction fetch): their case rotates the R values through one copy.
// Measured on the polynomial workload: +44% in fast math.  The native
// intrinsics and the double-precision parity routines stay unrolled (rolling
// measured slightly slower there).
// Records per iteration of a rolled case (copies of the routine inlined).
constexpr int kRollWidth = 1;
template <int OP, int MATH>
__device__ constexpr bool roll_unary() {
   return MATH == kMathFast &&
          (OP == PPI_OP_EXP || OP == PPI_OP_EXP10 || OP == PPI_OP_EXP2 || OP == PPI_OP_SIN ||
           OP == PPI_OP_COS || OP == PPI_OP_LOGISTIC || OP == PPI_OP_GAMMA || OP == PPI_OP_GAUSS ||
           OP == PPI_OP_LOG || OP == PPI_OP_LOG10 || OP == PPI_OP_LOG2 || OP == PPI_OP_TAN);
}

#define PPI_RUN_FAST_NAME run_fast_full
#define PPI_UNARY_LIST PPI_FULL_UNARY
#define PPI_BINARY_LIST PPI_FULL_BINARY
#define PPI_WITH_ITE 1
#include "run_fast.inc"
#undef PPI_RUN_FAST_NAME
#undef PPI_UNARY_LIST
#undef PPI_BINARY_LIST
#undef PPI_WITH_ITE

#define PPI_RUN_FAST_NAME run_fast_arith
#define PPI_UNARY_LIST PPI_ARITH_UNARY
#define PPI_BINARY_LIST PPI_ARITH_BINARY
#define PPI_WITH_ITE 0
#include "run_fast.inc"
#undef PPI_RUN_FAST_NAME
#undef PPI_UNARY_LIST
#undef PPI_BINARY_LIST
#undef PPI_WITH_ITE

template <int MATH, int R, int OPSET, int D>
__device__ __forceinline__ void run_fast(const uint2* __restrict__ code, float* mine, int T, int P,
                                         int tid, const Direct& g, float (&acc)[R], int prot) {
   if constexpr (OPSET == kOpsetArith) run_fast_arith<MATH, R, D>(code, mine, T, P, tid, g, acc, prot);
   else run_fast_full<MATH, R, D>(code, mine, T, P, tid, g, acc, prot);
}

// Copies a program's code (meta.y words) into shared memory, once per
// program, checking it on the way.  The header must leave the staged columns
// and the target inside the tile's `rows` rows and the column list inside the
// code; listed columns must be columns of the dataset (ncol); an instruction
// must be one of the kernel's cases and name operands inside the tile or,
// where the kernel reads columns directly (direct), the dataset; a
// generic-form token must be in the op table, an attribute inside the
// dataset.  A bad instruction or token becomes the end marker, a bad column
// column 0, a bad header an empty program, and kStatusBadInstruction is
// recorded.  An end marker also follows the code (`cap`: words the region
// holds, at least meta.y + 1).  So whatever the code buffer holds, the
// interpreters' dispatch and their shared-memory and dataset accesses stay
// inside what the kernel has.  All threads call it; the caller synchronises
// before reading s_code.
template <int OPSET>
__device__ __forceinline__ void load_code(uint2* s_code, const uint2* code, int2 meta, int cap, int rows,
                                          int ncol, bool direct, int* status, int tid, int P) {
   const bool generic = meta_kind(meta) == kKindGeneric;
   const uint2 end = make_uint2(generic ? kGenericEnd : (uint32_t)M_END, 0u);
   const uint2 hdr = code[0];
   const int k = (int)hdr.x, s = (int)(hdr.y & 0xFFFFu), d = (int)(hdr.y >> 16);
   const int first = generic ? 1 : code_header(k + d);
   const bool hdr_ok = meta.y >= 2 && meta.y < cap &&
                       (generic ? hdr.x == 0u && hdr.y == 0u
                                : (hdr.x <= 0xFFFFu && k + s + 1 <= rows && first < meta.y));
   if (!hdr_ok) {
      if (tid == 0) {
         s_code[0] = make_uint2(0u, 0u);
         s_code[1] = end;
         atomicOr(status, kStatusBadInstruction);
      }
      return;
   }
   bool bad = false;
   for (int i = tid; i < meta.y; i += P) {
      uint2 w = code[i];
      if (i >= first) {
         const bool ok = generic ? (w.x == kGenericEnd ||
                                    (w.x < (uint32_t)PPI_OP_COUNT &&
                                     (w.x != (uint32_t)PPI_OP_ATTRIBUTE || w.y < (uint32_t)ncol)))
                                 : instruction_ok<OPSET>(w, rows, ncol, direct);
         if (!ok) {
            w = end;
            bad = true;
         }
      } else if (i > 0) {
         // column-list entry i holds columns 2(i-1) and 2(i-1)+1 of the k + d listed
         if (w.x >= (uint32_t)ncol) { w.x = 0u; bad = true; }
         if (2 * i <= k + d && w.y >= (uint32_t)ncol) { w.y = 0u; bad = true; }
      }
      s_code[i] = w;
   }
   if (bad) atomicOr(status, kStatusBadInstruction);
   if (tid == 0) s_code[meta.y] = end;
}

// ---- generic stack interpreter ----------------------------------------------
template <int MATH>
__device__ __forceinline__ float generic_op(int op, float a, float b, int prot) {
   switch (op) {
#define PPI_GU(OP) case OP: return unop<OP, MATH>(a, prot);
      PPI_GU(PPI_OP_NOT) PPI_GU(PPI_OP_ABS) PPI_GU(PPI_OP_POW2) PPI_GU(PPI_OP_POW3)
      PPI_GU(PPI_OP_POW4) PPI_GU(PPI_OP_POW5) PPI_GU(PPI_OP_NEG) PPI_GU(PPI_OP_ROUND)
      PPI_GU(PPI_OP_CEIL) PPI_GU(PPI_OP_FLOOR) PPI_GU(PPI_OP_EXP) PPI_GU(PPI_OP_EXP10)
      PPI_GU(PPI_OP_EXP2) PPI_GU(PPI_OP_SIN) PPI_GU(PPI_OP_COS) PPI_GU(PPI_OP_STEP)
      PPI_GU(PPI_OP_SIGN) PPI_GU(PPI_OP_LOGISTIC) PPI_GU(PPI_OP_GAMMA) PPI_GU(PPI_OP_GAUSS)
      PPI_GU(PPI_OP_SQRT) PPI_GU(PPI_OP_LOG) PPI_GU(PPI_OP_LOG10) PPI_GU(PPI_OP_LOG2)
      PPI_GU(PPI_OP_TAN)
#undef PPI_GU
#define PPI_GB(OP) case OP: return binop<OP, MATH>(a, b, prot);
      PPI_GB(PPI_OP_AND) PPI_GB(PPI_OP_OR) PPI_GB(PPI_OP_XOR) PPI_GB(PPI_OP_GREATER)
      PPI_GB(PPI_OP_GREATEREQUAL) PPI_GB(PPI_OP_LESS) PPI_GB(PPI_OP_LESSEQUAL)
      PPI_GB(PPI_OP_EQUAL) PPI_GB(PPI_OP_NOTEQUAL) PPI_GB(PPI_OP_ADD) PPI_GB(PPI_OP_SUB)
      PPI_GB(PPI_OP_MULT) PPI_GB(PPI_OP_MEAN) PPI_GB(PPI_OP_MAX) PPI_GB(PPI_OP_MIN)
      PPI_GB(PPI_OP_MOD) PPI_GB(PPI_OP_POW) PPI_GB(PPI_OP_DIV)
#undef PPI_GB
   default: return __uint_as_float(0x7fc00000u);
   }
}

// Right-to-left stack evaluation with the reference's stack semantics
// (accelerator.cl:28-53); missing operands of a malformed program read as NaN.
// Attribute reads go straight to the dataset in global memory (positions at
// or past ld read 0, as the staged tile does).
template <int MATH, int R>
__device__ __noinline__ void run_generic(const uint2* __restrict__ code, const float* __restrict__ data,
                                         int ld, int base, int P, int tid, float* __restrict__ out,
                                         int prot) {
   float stk[kGenericStack];
   const float qnan = __uint_as_float(0x7fc00000u);
#pragma unroll 1
   for (int r = 0; r < R; ++r) {
      int top = -1;
      bool overflow = false;
      const int rec = tile_pos(tid, r, P);
#pragma unroll 1
      for (int pc = 0;; ++pc) {
         const uint2 ins = code[pc];
         const int op = (int)ins.x;
         if (ins.x == kGenericEnd) break;
         const int ar = op_arity(op);
         if (ar == 0 && top + 1 >= kGenericStack) {   // deeper than the translator admits
            overflow = true;
            break;
         }
         if (top + 1 < ar) {
            const int have = top + 1, miss = ar - have;
            for (int k = have - 1; k >= 0; --k) stk[k + miss] = stk[k];
            for (int k = 0; k < miss; ++k) stk[k] = qnan;
            top = ar - 1;
         }
         if (ar == 0) {
            float v;
            if (op == PPI_OP_ATTRIBUTE) v = (base + rec < ld) ? __ldg(data + (size_t)ins.y * ld + base + rec) : 0.0f;
            else v = __uint_as_float(ins.y);   // CONST / LITERAL value, INVALID = NaN
            stk[++top] = v;
         } else if (ar == 3) {
            stk[top - 2] = truthy(stk[top]) ? stk[top - 1] : stk[top - 2];
            top -= 2;
         } else if (ar == 2) {
            stk[top - 1] = generic_op<MATH>(op, stk[top], stk[top - 1], prot);
            --top;
         } else {
            stk[top] = generic_op<MATH>(op, stk[top], 0.0f, prot);
         }
      }
      out[r] = (top >= 0 && !overflow) ? stk[top] : qnan;
   }
}

// ---- tile staging: TMA bulk copies completed on an mbarrier ----------------
// Iterations of the barrier wait before giving up (the copies are from valid
// global memory into this CTA's shared memory, so the limit is a safety net:
// reaching it records kStatusStageTimeout and the tile is used as it is).
constexpr int kStageWaitLimit = 1 << 24;

struct Stager {
   uint64_t* bar;      // shared-memory mbarrier (arrival count 1)
   uint32_t phase;     // parity of the phase the next tile completes
};

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
   return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// One thread, once per CTA, before the first tile; then __syncthreads.
__device__ __forceinline__ void stager_init(uint64_t* bar) {
   asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(bar)));
   asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Bounded wait for the current phase of the staging mbarrier (this thread's view).
__device__ __forceinline__ bool wait_phase(const Stager& st) {
   uint32_t done = 0;
   for (int it = 0; it < kStageWaitLimit && !done; ++it) {
      asm volatile(
          "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
          : "=r"(done)
          : "r"(smem_addr(st.bar)), "r"(st.phase)
          : "memory");
   }
   return done != 0;
}

// Stage the records [base, base + T) of the program's staged columns (tile
// rows s .. s+k-1, from the code header) and of the target column (row s+k),
// and prefetch into L2 the same records of the columns it reads directly.
// When the tile starts on a 16-byte boundary (always, except DP over a lane
// count that is not a multiple of 4) one thread copies each column's segment
// with cp.async.bulk (TMA) and every thread waits on the mbarrier; otherwise
// the threads copy with 16-byte loads.  All threads call it, and it returns
// with the CTA synchronised (the tile visible to every thread).  Returns false,
// the same in every thread, when the bulk copies did not complete within the
// wait limit (kStatusStageTimeout is recorded): the CTA must stop staging and
// end its work.
__device__ __forceinline__ bool stage_tile(const float* data, int ncol, int ld, const uint2* s_code,
                                           float* s_tile, int base, int T, int tid, int P, Stager& st,
                                           int* status) {
   const uint2 hdr = s_code[0];
   const int k = (int)hdr.x, s = (int)(hdr.y & 0xFFFFu), d = (int)(hdr.y >> 16);
   const int lines = T / 32;   // 128-byte lines of one column's tile segment
   for (int q = tid; q < d * lines; q += P) {
      const int jj = k + q / lines, line = q - (q / lines) * lines;
      const uint2 pair = s_code[1 + (jj >> 1)];
      const int cidx = (int)((jj & 1) ? pair.y : pair.x);
      if (base + line * 32 < ld) {
         const float* p = data + (size_t)cidx * ld + base + line * 32;
         asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
      }
   }
   const bool bulk = (base & 3) == 0 && (reinterpret_cast<uintptr_t>(data) & 15) == 0 && (ld & 3) == 0;
   if (bulk) {
      // floats per column segment: the tile, or what is left of the column
      const int nf = min(T, ld - base);
      const uint32_t bytes = (uint32_t)nf * 4u;
      if (tid == 0) {
         // earlier generic-proxy writes to these rows before the async copies
         asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
         asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(st.bar)),
                      "r"(bytes * (uint32_t)(k + 1))
                      : "memory");
         for (int j = 0; j <= k; ++j) {
            const uint2 pair = s_code[1 + (j >> 1)];
            const int cidx = (j == k) ? ncol - 1 : (int)((j & 1) ? pair.y : pair.x);
            const float* src = data + (size_t)cidx * ld + base;
            float* dst = s_tile + (size_t)(s + j) * T;
            asm volatile(
                "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                    smem_addr(dst)),
                "l"(src), "r"(bytes), "r"(smem_addr(st.bar))
                : "memory");
         }
      }
      if (__syncthreads_and(wait_phase(st) ? 1 : 0)) {
         st.phase ^= 1u;
         return true;
      }
      // The wait ran out: the phase of the mbarrier is no longer known, so
      // this CTA stages nothing more.  Record it, give the copies in flight
      // one more bounded wait (they target this CTA's shared memory), and
      // let the caller end the CTA's work.
      if (tid == 0) atomicOr(status, kStatusStageTimeout);
      wait_phase(st);
      __syncthreads();
      return false;
   }
   for (int j = 0; j <= k; ++j) {
      const uint2 pair = s_code[1 + (j >> 1)];
      const int cidx = (j == k) ? ncol - 1 : (int)((j & 1) ? pair.y : pair.x);
      const float* src = data + (size_t)cidx * ld + base;
      float* dst = s_tile + (size_t)(s + j) * T;
      for (int t = tid * 4; t < T; t += P * 4) {
#pragma unroll
         for (int q = 0; q < 4; ++q) dst[t + q] = (base + t + q < ld) ? __ldg(src + t + q) : 0.0f;
      }
   }
   __syncthreads();
   return true;
}

__device__ __forceinline__ float reduce1(int reduce_max, float acc, float e, float fnlin) {
   if (reduce_max) {
      const float v = e * fnlin;
      return (v > acc) ? v : acc;
   }
   return acc + e;
}

// __local tree of accelerator.cl:157-167 / 252-262 over L values.
__device__ __forceinline__ void local_tree(float* pe, int L, int reduce_max, int tid, int P) {
   int p2 = 1;
   while (p2 < L) p2 <<= 1;
   for (int s = p2 >> 1; s > 0; s >>= 1) {
      for (int l = tid; l < s; l += P)
         if (l + s < L) pe[l] = reduce_max ? ((pe[l + s] > pe[l]) ? pe[l + s] : pe[l]) : pe[l] + pe[l + s];
      __syncthreads();
   }
}

template <int EF, int R>
__device__ __forceinline__ void error_row(const float (&v)[R], const float (&y)[R], float (&e)[R],
                                          const float* cost, int cn) {
#pragma unroll
   for (int r = 0; r < R; ++r) e[r] = apply_error_t<EF>(v[r], y[r], cost, cn);
}

// Lane == tile position: each of this thread's R lanes adds its record's
// error in record order, and stops at the first non-finite error
// (accelerator.cl:236).  A tile wholly inside the dataset, on lanes none of
// which has stopped, skips the per-record bounds test.
template <int RM, int R>
__device__ __forceinline__ void accumulate_lanes(float (&lacc)[R], uint32_t& ldone, const float (&e)[R],
                                                 int base, int tid, int P, int T, int nlin, float fnlin) {
   if (ldone == 0u && base + T <= nlin) {
#pragma unroll
      for (int r = 0; r < R; ++r) {
         if (nonfinite(e[r])) { lacc[r] = FLT_MAX; ldone |= 1u << r; }
         else lacc[r] = reduce1(RM, lacc[r], e[r], fnlin);
      }
      return;
   }
#pragma unroll
   for (int r = 0; r < R; ++r) {
      const int n = base + tile_pos(tid, r, P);
      if (n < nlin && !((ldone >> r) & 1u)) {
         if (nonfinite(e[r])) { lacc[r] = FLT_MAX; ldone |= 1u << r; }
         else lacc[r] = reduce1(RM, lacc[r], e[r], fnlin);
      }
   }
}

// Everything the evaluation of one program needs (one population's dataset
// and error settings, the program's translation).
struct Job {
   const float* data;
   int nlin, ncol, ld;
   int strategy, lanes, ef, reduce_max, prot, cost_n;
   const float* cost;
   float alpha;
   int2 meta;                  // {kind | rows << 8, code length}
   int size;
   const uint2* code;          // in global memory
   int rows_cap;               // tile rows of this pass (lane accumulators follow them)
   int code_cap;               // words of the shared-memory code region
   int alpha_free;             // the best index compares error/nlin without alpha*size
   int r0, r1;                 // chunked kernels: this item's records [r0, r1)
   float* state;               // chunked kernels: the program's lane state, (R + 1) x P floats
};

// Fitness of one program (valid in thread 0), in exactly the reference
// strategy's accumulation order; `sel` (thread 0) receives the value the
// best-index rule compares: the fitness, or error/nlin without alpha*size.
// `abort` becomes true (in every thread) when a tile could not be staged;
// the CTA must then take no more work.  All threads of the CTA call it; it
// starts and ends with the CTA synchronised.  s_code/s_tile: shared memory; the rows
// region holds job.rows_cap rows of T = P*R floats (slots, staged columns,
// target; row 0 is reused for the tile's errors once the program has run),
// then, unless the lane == tile-position path applies, lanes floats of lane
// accumulators and lanes bytes of lane-finished flags.
template <int MATH, int R, int OPSET, int D, int FAMILY>
__device__ float evaluate_program(const Job& j, uint2* s_code, float* s_tile, int* status, int tid,
                                  int P, Stager& st, float& sel, bool& abort) {
   const int T = P * R;
   const int L = j.lanes;
   const bool aligned = j.strategy == PPI_STRATEGY_PDP && L == T;
   const bool dp = j.strategy == PPI_STRATEGY_DP;
   const int kind = meta_kind(j.meta);
   float* s_err = s_tile;
   // the aligned path needs no error/lane buffers: its final lane values
   // reuse the start of the rows region once the last tile is done
   float* s_acc = aligned ? s_tile : s_tile + (size_t)j.rows_cap * T;
   unsigned char* s_done = reinterpret_cast<unsigned char*>(s_acc + L);
   const int Teff = dp ? L * dp_tile_groups(L, T) : T;
   const float fnlin = (float)j.nlin;
   // one lane (PP, or PDP over one lane) in a one-lane kernel: the tile's
   // first non-finite error, found by every thread
   const bool one_lane = FAMILY == kFamilyOneLane && !dp && L == 1;
   // a chunked kernel evaluates records [r0, r1) (lane == tile position),
   // the lane state coming from and going to j.state between chunks
   constexpr bool chunked = FAMILY == kFamilyChunked;
   const int r0 = chunked ? j.r0 : 0;
   const int r1 = chunked ? j.r1 : j.nlin;
   __shared__ int s_first;
   float fit = FLT_MAX;
   sel = FLT_MAX;
   if (kind == kKindInvalid || kind == kKindUnsupported) {
      // size 0 (sizes outside [1, max_size] are treated as 0)
      if (tid == 0) {
         if (kind == kKindUnsupported) atomicOr(status, kStatusUnsupportedProgram);
         if (kind == kKindInvalid && dp) {
            // every group reports MAXFLOAT (accelerator.cl:108-112); host rule
            float sum = 0.0f;
            const int G = (j.nlin + L - 1) / L;
            for (int g = 0; g < G; ++g) sum = reduce1(j.reduce_max, sum, FLT_MAX, fnlin);
            fit = nonfinite(sum) ? FLT_MAX : sum / fnlin;
            sel = fit;
         }
      }
      __syncthreads();
      return fit;
   }
   load_code<OPSET>(s_code, j.code, j.meta, j.code_cap, j.rows_cap, j.ncol, D != 0, status, tid, P);
   if (!aligned)
      for (int l = tid; l < L; l += P) { s_acc[l] = 0.0f; s_done[l] = 0; }
   __syncthreads();
   const uint2 hdr = s_code[0];   // as load_code checked it
   const uint2* prog = s_code + code_header((int)hdr.x + (int)(hdr.y >> 16));
   const int trow = (int)hdr.x + (int)(hdr.y & 0xFFFFu);
   float lacc[R];
#pragma unroll
   for (int r = 0; r < R; ++r) lacc[r] = 0.0f;
   uint32_t ldone = 0u;
   if constexpr (chunked) {
      if (r0 > 0) {   // the lanes as the previous chunk left them (bypassing L1)
#pragma unroll
         for (int r = 0; r < R; ++r) lacc[r] = __ldcg(j.state + (size_t)r * P + tid);
         ldone = __float_as_uint(__ldcg(j.state + (size_t)R * P + tid));
      }
   }
   float dsum = 0.0f;
   bool ddone = false;
   for (int base = r0; base < r1; base += Teff) {
      __syncthreads();
      if (!stage_tile(j.data, j.ncol, j.ld, s_code, s_tile, base, T, tid, P, st, status)) {
         // the tile never arrived (status recorded): no fitness for this
         // program, and the caller ends the CTA's work
         abort = true;
         fit = sel = __uint_as_float(0x7fc00000u);
         return fit;
      }
      float v[R];
      if (kind != kKindGeneric) {
         const Direct g{j.data + base, j.ld, j.ld - base, (base & 3) == 0};
         run_fast<MATH, R, OPSET, D>(prog, s_tile + tid * 4, T, P, tid, g, v, j.prot);
      } else {
         float tmp[R];
         run_generic<MATH, R>(prog, j.data, j.ld, base, P, tid, tmp, j.prot);
#pragma unroll
         for (int r = 0; r < R; ++r) v[r] = tmp[r];
      }
      float ycol[R];
      load_row(s_tile + (size_t)trow * T + tid * 4, P, ycol);
      float e[R];
      switch (j.ef) {   // one switch per tile, not per record
      case PPI_EF_ABS: error_row<PPI_EF_ABS>(v, ycol, e, j.cost, j.cost_n); break;
      case PPI_EF_SQUARED: error_row<PPI_EF_SQUARED>(v, ycol, e, j.cost, j.cost_n); break;
      case PPI_EF_MISCLASS: error_row<PPI_EF_MISCLASS>(v, ycol, e, j.cost, j.cost_n); break;
      default: error_row<PPI_EF_COST>(v, ycol, e, j.cost, j.cost_n); break;
      }
      if (aligned) {
         if (j.reduce_max) accumulate_lanes<1>(lacc, ldone, e, base, tid, P, T, j.nlin, fnlin);
         else accumulate_lanes<0>(lacc, ldone, e, base, tid, P, T, j.nlin, fnlin);
      } else {
         if (one_lane && tid == 0) s_first = T;
         __syncthreads();   // every thread is done with the rows: row 0 takes the errors
         int first = T;
#pragma unroll
         for (int r = 0; r < R; ++r) {
            const int t = tile_pos(tid, r, P);
            s_err[t] = (dp && base + t >= j.nlin) ? 0.0f : e[r];
            if (one_lane && base + t < j.nlin && nonfinite(e[r])) first = min(first, t);
         }
         if (one_lane && first < T) atomicMin(&s_first, first);
         __syncthreads();
         if (dp) {
            const int G = Teff / L;
            int p2 = 1;
            while (p2 < L) p2 <<= 1;
            for (int s = p2 >> 1; s > 0; s >>= 1) {
               for (int idx = tid; idx < G * s; idx += P) {
                  const int gi = idx / s, l = idx - gi * s;
                  if (l + s < L) {
                     float* pe = s_err + gi * L;
                     pe[l] = j.reduce_max ? ((pe[l + s] > pe[l]) ? pe[l + s] : pe[l]) : pe[l] + pe[l + s];
                  }
               }
               __syncthreads();
            }
            if (tid == 0) {
               for (int gi = 0; gi < G && !ddone; ++gi) {
                  if (base + gi * L >= j.nlin) break;
                  const float part = s_err[gi * L];
                  if (nonfinite(part)) { dsum = FLT_MAX; ddone = true; }
                  else dsum = reduce1(j.reduce_max, dsum, part, fnlin);
               }
            }
         } else if (one_lane) {
            // the one lane adds the tile's records in record order, up to the
            // first non-finite error: a chain with no test in it, operands read
            // four at a time (sequential.cc:171-179)
            if (tid == 0 && !s_done[0]) {
               const int cnt = min(T, j.nlin - base);
               const int stop = min(cnt, s_first);
               float acc = s_acc[0];
               int n = 0;
               if (j.reduce_max) {
                  for (; n < stop; ++n) {
                     const float v = s_err[n] * fnlin;
                     acc = (v > acc) ? v : acc;
                  }
               } else {
#pragma unroll 4
                  for (; n + 4 <= stop; n += 4) {
                     const float4 q = *reinterpret_cast<const float4*>(s_err + n);
                     acc = acc + q.x;
                     acc = acc + q.y;
                     acc = acc + q.z;
                     acc = acc + q.w;
                  }
                  for (; n < stop; ++n) acc = acc + s_err[n];
               }
               if (stop < cnt) { acc = FLT_MAX; s_done[0] = 1; }
               s_acc[0] = acc;
            }
         } else {
            const int end = min(base + T, j.nlin);
            const int off = base % L;
            for (int l = tid; l < L; l += P) {
               if (s_done[l]) continue;
               float acc = s_acc[l];
               int done = 0;
               for (int n = base + (l - off + L) % L; n < end; n += L) {
                  const float ev = s_err[n - base];
                  if (nonfinite(ev)) { acc = FLT_MAX; done = 1; break; }
                  acc = reduce1(j.reduce_max, acc, ev, fnlin);
               }
               s_acc[l] = acc;
               if (done) s_done[l] = 1;
            }
         }
      }
   }
   if constexpr (chunked) {
      if (r1 < j.nlin) {   // not the last chunk: keep the lanes for the next one
#pragma unroll
         for (int r = 0; r < R; ++r) __stcg(j.state + (size_t)r * P + tid, lacc[r]);
         __stcg(j.state + (size_t)R * P + tid, __uint_as_float(ldone));
         __syncthreads();
         return fit;
      }
   }
   __syncthreads();
   if (dp) {
      if (tid == 0) {
         fit = nonfinite(dsum) ? FLT_MAX : dsum / fnlin + j.alpha * (float)j.size;
         sel = fit;
      }
   } else {
      if (aligned) {
         __syncthreads();   // every thread is done with the rows region
#pragma unroll
         for (int r = 0; r < R; ++r) s_acc[tile_pos(tid, r, P)] = lacc[r];
         __syncthreads();
      }
      local_tree(s_acc, L, j.reduce_max, tid, P);
      if (tid == 0) {
         const float pe = s_acc[0];
         const float vv = nonfinite(pe) ? FLT_MAX : pe / fnlin;
         fit = vv + j.alpha * (float)j.size;
         sel = j.alpha_free ? vv : fit;
      }
   }
   __syncthreads();
   return fit;
}

// Waits of a chunked item for its program's previous chunk (each with a
// 256 ns sleep): about a second, then kStatusChunkWait and the CTA stops.
constexpr int kChunkWaitLimit = 1 << 22;

// One population: a persistent grid pulls program indices from a device
// counter; the last CTA to finish turns the packed arg-min into the index.
// Resident CTAs per SM the register allocation is bounded for: the fast and
// native interpreters fit 80 registers a thread (6 CTAs of 128 threads), the
// parity one needs the double-precision transcendentals' registers (4 CTAs).
// The main pass (D = 0) is also built at 64 registers (HI: 8 CTAs) for tiles
// small enough that 8 CTAs fit an SM's shared memory: the polynomial workload
// measured 26.5 -> 23.6 ms per evaluation there, while the 64-register build
// at a tile that still fits only 6 CTAs lost 4 % (the host picks).
constexpr int min_ctas_per_sm(int math, int hi) { return math == kMathParity ? 4 : (hi ? 8 : 6); }

template <int MATH, int R, int OPSET, int D, int HI, int FAMILY>
__global__ void __launch_bounds__(128, min_ctas_per_sm(MATH, HI)) eval_kernel(const EvalArgs a) {
   extern __shared__ __align__(16) unsigned char smem_raw[];
   __shared__ int s_prog;
   __shared__ __align__(8) uint64_t s_bar;
   if (threadIdx.x == 0) stager_init(&s_bar);
   __syncthreads();
   Stager st{&s_bar, 0u};
   const int P = blockDim.x, tid = threadIdx.x;
   uint2* s_code = reinterpret_cast<uint2*>(smem_raw);
   float* s_tile = reinterpret_cast<float*>(smem_raw + code_bytes(a.code_stride));
   Job j;
   j.data = a.data; j.nlin = a.nlin; j.ncol = a.ncol; j.ld = a.ld;
   j.strategy = a.strategy; j.lanes = a.lanes; j.ef = a.ef; j.reduce_max = a.reduce_max;
   j.prot = a.prot; j.cost = a.cost; j.cost_n = a.cost_n; j.alpha = a.alpha;
   j.rows_cap = a.rows;
   j.code_cap = a.code_stride + 1;
   j.alpha_free = a.best.alpha_free;
   unsigned* queue = a.wide_pass ? &a.stats->wide_queue : &a.stats->queue;
   const int limit = a.wide_pass ? (int)a.stats->wide : a.n;
   // chunked kernels: work items (program, record chunk), the programs in
   // groups and each group's items in chunk-major order, so that the grid
   // walks the dataset together while the group's lane states stay in L2; a
   // chunk waits (bounded) for its program's previous chunk, which an earlier
   // item holds. The main pass walks every program (skipping the wide ones)
   // in one group: its few programs' states fit, and a group of them would
   // leave fewer items between a program's chunks than the grid has CTAs.
   constexpr bool chunked = FAMILY == kFamilyChunked;
   const long long items = chunked ? (long long)limit * a.n_chunks : limit;
   const int group = a.wide_pass ? a.chunk_group : limit;
   __shared__ int s_wait_failed;
   for (;;) {
      if (tid == 0) s_prog = (int)atomicAdd(queue, 1u);
      __syncthreads();
      const int item = s_prog;
      if (item >= items) break;
      int c = 0, k = item;
      if constexpr (chunked) chunk_item(item, limit, group, a.n_chunks, &c, &k);
      const int prog = a.wide_pass ? a.wide_list[k] : k;
      j.meta = a.meta[prog];
      const int kind = meta_kind(j.meta);
      if ((!a.wide_pass && kind == kKindWide) ||
          (chunked && c > 0 && (kind == kKindInvalid || kind == kKindUnsupported))) {
         __syncthreads();   // s_prog is read by every thread before it is rewritten
         continue;
      }
      j.size = a.size[prog];
      j.code = a.code + (size_t)prog * a.code_stride;
      bool last = true;
      if constexpr (chunked) {
         j.r0 = c * a.chunk_records;
         j.r1 = min(a.nlin, j.r0 + a.chunk_records);
         j.state = a.chunk_state + (size_t)prog * (R + 1) * P;
         last = j.r1 >= a.nlin || kind == kKindInvalid || kind == kKindUnsupported;
         if (c > 0) {
            if (tid == 0) {
               volatile unsigned* done = a.chunk_done + prog;
               int it = 0;
               while (*done < (unsigned)c && it < kChunkWaitLimit) {
                  __nanosleep(256);
                  ++it;
               }
               s_wait_failed = *done < (unsigned)c;
               if (s_wait_failed) atomicOr(a.status, kStatusChunkWait);
               __threadfence();
            }
            __syncthreads();
            if (s_wait_failed) break;   // this CTA takes no more work
         }
      }
      float sel;
      bool abort = false;
      const float fit = evaluate_program<MATH, R, OPSET, D, FAMILY>(j, s_code, s_tile, a.status, tid, P, st, sel, abort);
      if (!last) {
         if (abort) break;   // no state stored: the next chunk times out (status recorded)
         // the lane state is stored: publish this chunk to the program's next one
         __threadfence();
         __syncthreads();
         if (tid == 0) atomicExch(a.chunk_done + prog, (unsigned)(c + 1));
         continue;
      }
      if (tid == 0) {
         a.fitness[prog] = fit;
         atomicMin(a.best_key, best_key(sel, best_tie(a.best, prog)));
      }
      if (abort) break;   // staging failed: this CTA takes no more work
   }
   if (a.final_pass && tid == 0) {
      __threadfence();
      const unsigned done = atomicAdd(&a.stats->finished, 1u);
      if (done == gridDim.x - 1) {
         __threadfence();
         const unsigned long long k = *reinterpret_cast<volatile unsigned long long*>(a.best_key);
         a.best_index[0] = (int32_t)best_from_tie(a.best, (uint32_t)(k & 0xFFFFFFFFull));
      }
   }
}

// Many populations in one persistent launch: work items are program indices
// in cost order (size x records, largest first); each population keeps its
// own arg-min key and completion counter, and the CTA that finishes a
// population's last program writes that population's best index.
template <int MATH, int R, int OPSET, int D, int HI, int FAMILY>
__global__ void __launch_bounds__(128, min_ctas_per_sm(MATH, HI)) eval_batch_kernel(const BatchArgs a) {
   extern __shared__ __align__(16) unsigned char smem_raw[];
   __shared__ int s_item;
   __shared__ __align__(8) uint64_t s_bar;
   if (threadIdx.x == 0) stager_init(&s_bar);
   __syncthreads();
   Stager st{&s_bar, 0u};
   const int P = blockDim.x, tid = threadIdx.x;
   uint2* s_code = reinterpret_cast<uint2*>(smem_raw);
   float* s_tile = reinterpret_cast<float*>(smem_raw + code_bytes(a.code_stride));
   const int lo = a.wide_pass ? (int)*a.n_main : 0;
   const int hi = a.wide_pass ? a.total : (int)*a.n_main;
   unsigned* queue = a.wide_pass ? &a.stats->wide_queue : &a.stats->queue;
   for (;;) {
      if (tid == 0) s_item = lo + (int)atomicAdd(queue, 1u);
      __syncthreads();
      const int item = s_item;
      if (item >= hi) break;
      const int g = a.order[item];
      const int p = a.pop_of[g];
      const PopDesc& pd = a.pops[p];
      Job j;
      j.data = pd.data; j.nlin = pd.nlin; j.ncol = pd.ncol; j.ld = pd.ld;
      j.strategy = pd.strategy; j.lanes = pd.lanes; j.ef = pd.ef; j.reduce_max = pd.reduce_max;
      j.prot = pd.prot; j.cost = pd.cost; j.cost_n = pd.cost_n; j.alpha = pd.alpha;
      j.meta = a.meta[g];
      j.size = a.size[g];
      j.code = a.code + (size_t)g * a.code_stride;
      j.rows_cap = a.rows;
      j.code_cap = a.code_stride + 1;
      j.alpha_free = pd.best.alpha_free;
      float sel;
      bool abort = false;
      const float fit = evaluate_program<MATH, R, OPSET, D, FAMILY>(j, s_code, s_tile, a.status, tid, P, st, sel, abort);
      if (abort) {   // staging failed: this CTA takes no more work
         if (tid == 0) a.fitness[g] = fit;
         break;
      }
      if (tid == 0) {
         const int local = g - pd.prog_begin;
         a.fitness[g] = fit;
         atomicMin(&a.pop_key[p], best_key(sel, best_tie(pd.best, local)));
         __threadfence();
         if (atomicAdd(&a.pop_done[p], 1u) == (unsigned)pd.n - 1) {
            __threadfence();
            const unsigned long long k = *reinterpret_cast<volatile unsigned long long*>(&a.pop_key[p]);
            a.best_index[p] = (int32_t)best_from_tie(pd.best, (uint32_t)(k & 0xFFFFFFFFull));
         }
      }
   }
}

// Per-record predictions of program 0 (ppp prediction mode).
template <int MATH, int R, int OPSET>
__global__ void __launch_bounds__(128, 4) predict_kernel(const PredictArgs a) {
   extern __shared__ __align__(16) unsigned char smem_raw[];
   __shared__ __align__(8) uint64_t s_bar;
   if (threadIdx.x == 0) stager_init(&s_bar);
   __syncthreads();
   Stager st{&s_bar, 0u};
   const int P = blockDim.x, tid = threadIdx.x, T = P * R;
   const int2 m = a.meta[0];
   uint2* s_code = reinterpret_cast<uint2*>(smem_raw);
   float* s_tile = reinterpret_cast<float*>(smem_raw + code_bytes(m.y));
   const int kind = meta_kind(m);
   const bool runs = kind == kKindFast || kind == kKindWide || kind == kKindGeneric;
   if (runs) load_code<OPSET>(s_code, a.code, m, m.y + 1, a.rows, a.ncol, true, a.status, tid, P);
   __syncthreads();
   const uint2 hdr = runs ? s_code[0] : make_uint2(0u, 0u);
   const uint2* prog = s_code + (runs ? code_header((int)hdr.x + (int)(hdr.y >> 16)) : 0);
   for (int base = blockIdx.x * T; base < a.nlin; base += gridDim.x * T) {
      __syncthreads();
      if (runs && !stage_tile(a.data, a.ncol, a.ld, s_code, s_tile, base, T, tid, P, st, a.status))
         break;   // the tile never arrived (status recorded): this CTA stops
      float v[R];
      if (kind == kKindFast || kind == kKindWide) {
         const Direct g{a.data + base, a.ld, a.ld - base, (base & 3) == 0};
         run_fast<MATH, R, OPSET, 1>(prog, s_tile + tid * 4, T, P, tid, g, v, a.prot);
      } else if (kind == kKindGeneric) {
         float tmp[R];
         run_generic<MATH, R>(prog, a.data, a.ld, base, P, tid, tmp, a.prot);
#pragma unroll
         for (int r = 0; r < R; ++r) v[r] = tmp[r];
      } else {
#pragma unroll
         for (int r = 0; r < R; ++r) v[r] = __uint_as_float(0x7fc00000u);
      }
#pragma unroll
      for (int r = 0; r < R; ++r) {
         const int n = base + tile_pos(tid, r, P);
         if (n < a.nlin) a.out[n] = v[r];
      }
   }
}


// Per-math entry points, instantiated in evaluate_<math>.cu (FAMILY = 0),
// evaluate_<math>_chunk.cu (FAMILY = 2: the chunked kernels) and
// evaluate_<math>_lane1.cu (FAMILY = 1: the kernels with the one-lane chain,
// for launches that hold a PP population; kept apart because the chain's
// code changed the register allocation of every kernel that carried it, 3 %
// on the uneven batch).  R = kR records per thread; opset 0 = FULL,
// 1 = ARITH; the kernel id (`direct`) as kMainHi describes.
template <int MATH, int FAMILY>
struct Launch {
   using EvalFn = void (*)(const EvalArgs);
   using BatchFn = void (*)(const BatchArgs);
   using PredictFn = void (*)(const PredictArgs);
   // kernel: 0 the main pass, 1 the wide pass (any tile), 2 the wide pass
   // (tiles of whole quads), kMainHi the main pass at 8 CTAs per SM (parity
   // math keeps its one register bound)
   static constexpr int kHi = MATH == kMathParity ? 0 : 1;
   template <int OPSET>
   static EvalFn eval_fn_set(int direct) {
      switch (direct) {
      case 1: return eval_kernel<MATH, kR, OPSET, 1, 0, FAMILY>;
      case 2: return eval_kernel<MATH, kR, OPSET, 2, 0, FAMILY>;
      case kMainHi: return eval_kernel<MATH, kR, OPSET, 0, kHi, FAMILY>;
      default: return eval_kernel<MATH, kR, OPSET, 0, 0, FAMILY>;
      }
   }
   // (batches have no chunked kernels: that family's entries are the plain ones)
   static constexpr int kBatchFamily = FAMILY == kFamilyChunked ? kFamilyPlain : FAMILY;
   template <int OPSET>
   static BatchFn batch_fn_set(int direct) {
      switch (direct) {
      case 1: return eval_batch_kernel<MATH, kR, OPSET, 1, 0, kBatchFamily>;
      case 2: return eval_batch_kernel<MATH, kR, OPSET, 2, 0, kBatchFamily>;
      case kMainHi: return eval_batch_kernel<MATH, kR, OPSET, 0, kHi, kBatchFamily>;
      default: return eval_batch_kernel<MATH, kR, OPSET, 0, 0, kBatchFamily>;
      }
   }
   static EvalFn eval_fn(int opset, int direct) {
      return opset ? eval_fn_set<kOpsetArith>(direct) : eval_fn_set<kOpsetFull>(direct);
   }
   static BatchFn batch_fn(int opset, int direct) {
      return opset ? batch_fn_set<kOpsetArith>(direct) : batch_fn_set<kOpsetFull>(direct);
   }
   static PredictFn predict_fn(int opset) {
      return opset ? predict_kernel<MATH, kR, kOpsetArith> : predict_kernel<MATH, kR, kOpsetFull>;
   }
   // Allow up to 200 KB of dynamic shared memory, once per kernel and device
   // (a function's attributes belong to each device's context; devices past
   // the first 64 set them on every call).
   static cudaError_t configure(int opset) {
      static std::atomic<unsigned long long> done[2];
      int dev = 0;
      cudaError_t e = cudaGetDevice(&dev);
      if (e != cudaSuccess) return e;
      const unsigned long long bit = dev >= 0 && dev < 64 ? 1ull << dev : 0ull;
      if (bit & done[opset].load(std::memory_order_acquire)) return cudaSuccess;
      const int attr = cudaFuncAttributeMaxDynamicSharedMemorySize, bytes = 200 * 1024;
      for (int direct = 0; direct <= kMainHi; ++direct) {
         e = cudaFuncSetAttribute(eval_fn(opset, direct), (cudaFuncAttribute)attr, bytes);
         if (e == cudaSuccess) e = cudaFuncSetAttribute(batch_fn(opset, direct), (cudaFuncAttribute)attr, bytes);
         if (e != cudaSuccess) return e;
      }
      e = cudaFuncSetAttribute(predict_fn(opset), (cudaFuncAttribute)attr, bytes);
      if (e == cudaSuccess) done[opset].fetch_or(bit, std::memory_order_release);
      return e;
   }
   static cudaError_t evaluate(int opset, int direct, const EvalArgs& a, int block, int grid, size_t smem,
                               cudaStream_t s) {
      cudaError_t e = configure(opset);
      if (e != cudaSuccess) return e;
      eval_fn(opset, direct)<<<grid, block, smem, s>>>(a);
      return cudaGetLastError();
   }
   static cudaError_t evaluate_batch(int opset, int direct, const BatchArgs& a, int block, int grid,
                                     size_t smem, cudaStream_t s) {
      cudaError_t e = configure(opset);
      if (e != cudaSuccess) return e;
      batch_fn(opset, direct)<<<grid, block, smem, s>>>(a);
      return cudaGetLastError();
   }
   static cudaError_t predict(int opset, const PredictArgs& a, int block, int grid, size_t smem, cudaStream_t s) {
      cudaError_t e = configure(opset);
      if (e != cudaSuccess) return e;
      predict_fn(opset)<<<grid, block, smem, s>>>(a);
      return cudaGetLastError();
   }
   static cudaError_t occupancy(int opset, int direct, int block, size_t smem, int* per_sm) {
      cudaError_t e = configure(opset);
      if (e != cudaSuccess) return e;
      return cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, eval_fn(opset, direct), block, smem);
   }
   static cudaError_t occupancy_batch(int opset, int direct, int block, size_t smem, int* per_sm) {
      cudaError_t e = configure(opset);
      if (e != cudaSuccess) return e;
      return cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, batch_fn(opset, direct), block, smem);
   }
};

}  // namespace ev
}  // namespace ppi

// Entry points of one math mode's kernel family (kFamily*), with the
// name suffix S: launch_evaluate_S, launch_evaluate_batch_S,
// evaluate_occupancy_S, evaluate_batch_occupancy_S (evaluate.cu dispatches).
#define PPI_EVALUATOR_ENTRY_POINTS(MATH, FAMILY, S)                                             \
   namespace ppi {                                                                            \
   template struct ev::Launch<MATH, FAMILY>;                                                   \
   cudaError_t launch_evaluate_##S(int opset, int direct, const EvalArgs& a, int block, int grid, \
                                   size_t smem, cudaStream_t s) {                             \
      return ev::Launch<MATH, FAMILY>::evaluate(opset, direct, a, block, grid, smem, s);       \
   }                                                                                          \
   cudaError_t launch_evaluate_batch_##S(int opset, int direct, const BatchArgs& a, int block,  \
                                         int grid, size_t smem, cudaStream_t s) {             \
      return ev::Launch<MATH, FAMILY>::evaluate_batch(opset, direct, a, block, grid, smem, s); \
   }                                                                                          \
   cudaError_t evaluate_occupancy_##S(int opset, int direct, int block, size_t smem, int* per_sm) { \
      return ev::Launch<MATH, FAMILY>::occupancy(opset, direct, block, smem, per_sm);          \
   }                                                                                          \
   cudaError_t evaluate_batch_occupancy_##S(int opset, int direct, int block, size_t smem,      \
                                            int* per_sm) {                                    \
      return ev::Launch<MATH, FAMILY>::occupancy_batch(opset, direct, block, smem, per_sm);    \
   }                                                                                          \
   }
