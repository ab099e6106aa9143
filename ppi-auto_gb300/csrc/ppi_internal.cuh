// ppi_internal.cuh -- shared definitions of the GB300 evaluator: the
// accumulator-machine bytecode that the translator emits and the evaluator
// runs, per-opcode arithmetic in the three math modes, and kernel arguments.
#pragma once

#include <cstdint>
#include <cfloat>
#include <cuda_runtime.h>

#include "ppi_gpu.h"

namespace ppi {

// Records each thread evaluates per bytecode instruction (register ILP).
constexpr int kR = 8;
// Slot rows of the accumulator machine: a well-formed program whose
// Sethi-Ullman number (with leaf operands folded into the instruction) is at
// most kSlots runs on the bytecode path.  Every binary tree of at most 255
// nodes fits in 6 slots.
constexpr int kSlots = 6;
// Largest lane count (PDP work-items per program, DP records per group).
constexpr int kMaxLanes = 4096;
// Stack depth of the generic (stack) interpreter used for malformed programs
// and programs needing more than kSlots slots.
constexpr int kGenericStack = 128;
// Column stride of the device dataset is a multiple of this.
constexpr int kColumnPad = 1024;

// Work item of the chunked kernels -> (record chunk c, program k): the
// programs in groups of `group`, each group's items chunk-major (the last
// group may be smaller). Every (c, k) with c < n_chunks, k < limit is one
// item of [0, limit * n_chunks), and (c - 1, k) always has a smaller index,
// so a chunk's wait is on an item an earlier CTA took from the queue.
__host__ __device__ inline void chunk_item(long long item, int limit, int group, int n_chunks,
                                           int* c, int* k) {
   const long long span = (long long)group * n_chunks;   // items of a full group
   const int grp = (int)(item / span);
   const int first = grp * group;
   const int gn = limit - first < group ? limit - first : group;
   const int rem = (int)(item - grp * span);
   *c = rem / gn;
   *k = first + rem - *c * gn;
}

// DP groups (L consecutive records each, reduced by their own tree and then
// added in record order) per tile of T record slots: the most that fit,
// rounded down so that the tile is a whole number of 4-record quads, so that
// every tile starts on a multiple of 4 records (bulk-copy staging and the
// whole-quad direct reads); the most that fit when no such count does (L
// above T / 4 and not a multiple of 4). Tiles hold whole groups either way,
// so the sums do not depend on the count.
__host__ __device__ inline int dp_tile_groups(int L, int T) {
   const int fit = T / L;
   const int step = (L % 4 == 0) ? 1 : ((L % 2 == 0) ? 2 : 4);   // groups per whole-quad tile step
   const int quads = fit / step * step;
   return quads > 0 ? quads : fit;
}

// Opcode sets of the evaluator's bytecode path (evaluate_impl.cuh).
enum : int { kOpsetFull = 0, kOpsetArith = 1 };
// Evaluator kernel ids (the `direct` argument of the launchers): 0 the main
// pass, 1 / 2 the wide pass (direct column reads: any tile / whole quads),
// kMainHi the main pass built for 8 resident CTAs per SM (64 registers); with
// kOneLane added, the same kernel with the one-lane chain (launches holding a
// PP population, or PDP over one lane); with kChunked added, the same kernel
// walking record chunks in chunk-major order (one PDP population over a
// dataset larger than L2).
constexpr int kMainHi = 3;
constexpr int kOneLane = 4;
constexpr int kChunked = 8;
// Kernel families (the template parameter FAMILY of the evaluator kernels).
enum : int { kFamilyPlain = 0, kFamilyOneLane = 1, kFamilyChunked = 2 };
// Chunked family: records per work item (tiles of 1024 records) and the
// smallest dataset (bytes of its columns) it is used for.
constexpr int kChunkTiles = 64;
constexpr size_t kChunkMinBytes = (size_t)64 << 20;

// Program kinds written by the translator.  meta.x = kind | rows << 8, where
// rows is the number of shared-memory rows the program's tile needs; meta.y is
// the length of its code (header included).  kKindWide: bytecode path, but
// its columns do not all fit the main pass's tile, so it runs in the wide
// pass (which reads the columns its tile cannot hold from global memory).
enum : int { kKindInvalid = 0, kKindFast = 1, kKindGeneric = 2, kKindUnsupported = 3, kKindWide = 4 };
__host__ __device__ __forceinline__ int meta_kind(int2 m) { return m.x & 0xFF; }
__host__ __device__ __forceinline__ int meta_rows(int2 m) { return m.x >> 8; }

// Code of one program: entry 0 is the header {k, s | d << 16}: the program
// stages k record columns in its tile, needs s slot rows, and reads d more
// columns directly from global memory.  Entries 1 .. (k+d+1)/2 list the k
// staged columns, then the d direct ones, two per entry (.x, .y).  The
// instructions follow.  Tile rows: 0 .. s-1 slots, s .. s+k-1 the staged
// columns, s+k the target column (the last column of the dataset).  The
// generic form has k = s = d = 0 (its attribute reads go to global memory) and
// its tokens follow the header.
__host__ __device__ __forceinline__ int code_header(int ncols) { return 1 + (ncols + 1) / 2; }
// Operand immediates of M_LD_ROW / M_BR_L / M_BR_R with this bit set name a
// record column read from global memory (low bits: the column index) instead
// of a tile row.
constexpr uint32_t kDirectColumn = 0x80000000u;
// Largest dataset width of the bytecode path (column indices share 24 bits
// with a reference count in the translator).
constexpr int kMaxColumns = (1 << 24) - 1;

// Translator statistics, zeroed before every translation.
struct DevStats {
   unsigned queue;           // work queue of the main pass
   unsigned finished;        // CTAs finished in the final pass
   unsigned wide;            // programs of the wide pass (plain evaluation)
   unsigned wide_queue;      // work queue of the wide pass
};

// Status bits reported by the kernels: a program the generic interpreter
// cannot hold; a tile copy that did not complete within the bounded wait (the
// CTA stopped); an instruction outside the running kernel's opcode set; a
// record chunk whose predecessor did not finish within the bounded wait (the
// CTA stopped).
enum : int { kStatusUnsupportedProgram = 1, kStatusStageTimeout = 2, kStatusBadInstruction = 4,
             kStatusChunkWait = 8 };

// Accumulator-machine instructions.  Each is a uint2: .x = instruction id
// below, .y = immediate: float bits of a constant, or a row index.
// The only register state is `acc` (kR record values per thread).  Every
// other operand is a "row" of the CTA's shared-memory tile (see
// code_header): slots where a pending subexpression is parked, and the
// staged record columns the program reads.  Each thread reads and writes only
// its own kR positions of a row.
enum : uint32_t {
   M_END = 0,
   M_LD_ROW = 1,                    // acc = row[imm]
   M_LD_C = 2,                      // acc = imm
   M_PUSH = 3,                      // row[imm] = acc
   M_UN = 4,                        // + (op - PPI_OP_NOT)  : acc = op(acc)
   M_BR_L = M_UN + 25,              // + (op - PPI_OP_AND)  : acc = op(acc, row[imm])
   M_BR_R = M_BR_L + 18,            //                        acc = op(row[imm], acc)
   M_BC_L = M_BR_R + 18,            //                        acc = op(acc, imm)
   M_BC_R = M_BC_L + 18,            //                        acc = op(imm, acc)
   M_ITE = M_BC_R + 18,             // + perm: rows a = imm & 0xFFFF, b = imm >> 16;
                                    //   roles of (acc, a, b) as (cond, then, else)
   M_PUSH_LD = M_ITE + 6,           // row[imm & 0xFFFF] = acc; acc = row[imm >> 16]
                                    //   (a push and the load after it, tile rows only)
   M_COUNT = M_PUSH_LD + 1
};
static_assert(PPI_OP_TAN - PPI_OP_NOT + 1 == 25, "unary op count");
static_assert(PPI_OP_DIV - PPI_OP_AND + 1 == 18, "binary op count");

// ITE permutations: perm p -> operand (0 = acc, 1 = row a, 2 = row b)
// holding cond, then, else.
__host__ __device__ constexpr int ite_role(int p, int role) {
   constexpr int t[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
   return t[p][role];
}

__host__ __device__ inline int op_arity(int op) {
   if (op == PPI_OP_IF_THEN_ELSE) return 3;
   if (op >= PPI_OP_AND && op <= PPI_OP_DIV) return 2;
   if (op >= PPI_OP_NOT && op < PPI_OP_COUNT) return 1;
   return 0;
}

// ---------------------------------------------------------------------------
// Arithmetic.  The whole library is compiled with -fmad=false, so no
// multiply-add is contracted (the reference's host compiler does not contract
// either on x86-64).  Float constants of src/interpreter/functions.h:19-57.
constexpr float kPiF = 3.14159274101257f;
constexpr float kPi2F = 1.57079637050629f;
constexpr float kEF = 2.71828174591064f;

enum : int { kMathFast = PPI_MATH_FAST, kMathParity = PPI_MATH_PARITY, kMathNative = PPI_MATH_NATIVE };

template <int MATH> __device__ __forceinline__ float f_sin(float x) {
   if constexpr (MATH == kMathParity) return (float)sin((double)x);
   else if constexpr (MATH == kMathNative) return __sinf(x);
   else return sinf(x);
}
template <int MATH> __device__ __forceinline__ float f_cos(float x) {
   if constexpr (MATH == kMathParity) return (float)cos((double)x);
   else if constexpr (MATH == kMathNative) return __cosf(x);
   else return cosf(x);
}
template <int MATH> __device__ __forceinline__ float f_tan(float x) {
   if constexpr (MATH == kMathParity) return (float)tan((double)x);
   else if constexpr (MATH == kMathNative) return __tanf(x);
   else return tanf(x);
}
template <int MATH> __device__ __forceinline__ float f_exp(float x) {
   if constexpr (MATH == kMathParity) return (float)exp((double)x);
   else if constexpr (MATH == kMathNative) return __expf(x);
   else return expf(x);
}
template <int MATH> __device__ __forceinline__ float f_exp2(float x) {
   if constexpr (MATH == kMathParity) return (float)exp2((double)x);
   else return exp2f(x);
}
template <int MATH> __device__ __forceinline__ float f_exp10(float x) {
   if constexpr (MATH == kMathParity) return (float)exp10((double)x);
   else if constexpr (MATH == kMathNative) return __exp10f(x);
   else return exp10f(x);
}
template <int MATH> __device__ __forceinline__ float f_log(float x) {
   if constexpr (MATH == kMathParity) return (float)log((double)x);
   else if constexpr (MATH == kMathNative) return __logf(x);
   else return logf(x);
}
template <int MATH> __device__ __forceinline__ float f_log2(float x) {
   if constexpr (MATH == kMathParity) return (float)log2((double)x);
   else if constexpr (MATH == kMathNative) return __log2f(x);
   else return log2f(x);
}
template <int MATH> __device__ __forceinline__ float f_log10(float x) {
   if constexpr (MATH == kMathParity) return (float)log10((double)x);
   else if constexpr (MATH == kMathNative) return __log10f(x);
   else return log10f(x);
}
template <int MATH> __device__ __forceinline__ float f_pow(float a, float b) {
   if constexpr (MATH == kMathParity) return (float)pow((double)a, (double)b);
   else if constexpr (MATH == kMathNative) return __powf(a, b);
   else return powf(a, b);
}

// Protected forms (src/interpreter/functions.h:99-193).
__device__ __forceinline__ float p_sqrt(float x, int prot) {
   float r = sqrtf(x);   // correctly rounded: equals (float)sqrt((double)x)
   return (prot && x < 0.0f) ? 1.0f : r;
}
template <int MATH> __device__ __forceinline__ float p_div(float x, float y, int prot) {
   float r;
   if constexpr (MATH == kMathNative) r = __fdividef(x, y);
   else r = x / y;
   return (prot && y == 0.0f) ? 1.0f : r;
}

// T_GAMMA (interpreter_core:127-129).  PARITY follows sequential.cc, where
// sinh and pow are double functions so x*sinh(...) and pow(...)*SQRT(...) are
// double expressions; the other modes follow the all-float OpenCL kernel.
template <int MATH> __device__ __forceinline__ float f_gamma(float x, int prot) {
   if constexpr (MATH == kMathParity) {
      double s = sinh((double)(1.0f / x));
      float a = (x / kEF) * p_sqrt((float)((double)x * s), prot);
      double p = pow((double)a, (double)x);
      return (float)(p * (double)p_sqrt(2.0f * kPiF / x, prot));
   } else {
      float a = (x / kEF) * p_sqrt(x * sinhf(1.0f / x), prot);
      return powf(a, x) * p_sqrt(2.0f * kPiF / x, prot);
   }
}

__device__ __forceinline__ bool truthy(float v) { return v != 0.0f; }   // (bool)float

template <int OP, int MATH> __device__ __forceinline__ float unop(float a, int prot) {
   if constexpr (OP == PPI_OP_NOT) return truthy(a) ? 0.0f : 1.0f;
   else if constexpr (OP == PPI_OP_ABS) return fabsf(a);
   else if constexpr (OP == PPI_OP_POW2) return a * a;
   else if constexpr (OP == PPI_OP_POW3) return (a * a) * a;
   else if constexpr (OP == PPI_OP_POW4) return ((a * a) * a) * a;
   else if constexpr (OP == PPI_OP_POW5) return (((a * a) * a) * a) * a;
   else if constexpr (OP == PPI_OP_NEG) return -a;
   else if constexpr (OP == PPI_OP_ROUND) return roundf(a);
   else if constexpr (OP == PPI_OP_CEIL) return ceilf(a);
   else if constexpr (OP == PPI_OP_FLOOR) return floorf(a);
   else if constexpr (OP == PPI_OP_EXP) return f_exp<MATH>(a);
   else if constexpr (OP == PPI_OP_EXP10) return f_exp10<MATH>(a);
   else if constexpr (OP == PPI_OP_EXP2) return f_exp2<MATH>(a);
   else if constexpr (OP == PPI_OP_SIN) return f_sin<MATH>(a);
   else if constexpr (OP == PPI_OP_COS) return f_cos<MATH>(a);
   else if constexpr (OP == PPI_OP_STEP) return (a >= 0.0f) ? 1.0f : 0.0f;
   else if constexpr (OP == PPI_OP_SIGN) return a > 0.0f ? 1.0f : (a < 0.0f ? -1.0f : 0.0f);
   else if constexpr (OP == PPI_OP_LOGISTIC) return 1.0f / (1.0f + f_exp<MATH>(-a));
   else if constexpr (OP == PPI_OP_GAMMA) return f_gamma<MATH>(a, prot);
   else if constexpr (OP == PPI_OP_GAUSS) return f_exp<MATH>(-a * a);
   else if constexpr (OP == PPI_OP_SQRT) return p_sqrt(a, prot);
   else if constexpr (OP == PPI_OP_LOG) { float r = f_log<MATH>(a); return (prot && a < 1.0f) ? 1.0f : r; }
   else if constexpr (OP == PPI_OP_LOG10) { float r = f_log10<MATH>(a); return (prot && a < 1.0f) ? 1.0f : r; }
   else if constexpr (OP == PPI_OP_LOG2) { float r = f_log2<MATH>(a); return (prot && a < 1.0f) ? 1.0f : r; }
   else {
      static_assert(OP == PPI_OP_TAN, "unary op");
      float r = f_tan<MATH>(a);
      const float fa = fabsf(a);
      return (prot && (fa == kPi2F || fa == 3.0f * kPi2F)) ? 1.0f : r;
   }
}

// a = stack[top] (left operand), b = stack[top-1] (right operand).
template <int OP, int MATH> __device__ __forceinline__ float binop(float a, float b, int prot) {
   if constexpr (OP == PPI_OP_AND) return (truthy(a) && truthy(b)) ? 1.0f : 0.0f;
   else if constexpr (OP == PPI_OP_OR) return (truthy(a) || truthy(b)) ? 1.0f : 0.0f;
   else if constexpr (OP == PPI_OP_XOR) return (truthy(a) != truthy(b)) ? 1.0f : 0.0f;
   else if constexpr (OP == PPI_OP_GREATER) return (a > b) ? 1.0f : 0.0f;
   else if constexpr (OP == PPI_OP_GREATEREQUAL) return (a >= b) ? 1.0f : 0.0f;
   else if constexpr (OP == PPI_OP_LESS) return (a < b) ? 1.0f : 0.0f;
   else if constexpr (OP == PPI_OP_LESSEQUAL) return (a <= b) ? 1.0f : 0.0f;
   else if constexpr (OP == PPI_OP_EQUAL) return (a == b) ? 1.0f : 0.0f;
   else if constexpr (OP == PPI_OP_NOTEQUAL) return (a != b) ? 1.0f : 0.0f;
   else if constexpr (OP == PPI_OP_ADD) return a + b;
   else if constexpr (OP == PPI_OP_SUB) return a - b;
   else if constexpr (OP == PPI_OP_MULT) return a * b;
   else if constexpr (OP == PPI_OP_MEAN) return (a + b) / 2.0f;
   else if constexpr (OP == PPI_OP_MAX) return fmaxf(a, b);
   else if constexpr (OP == PPI_OP_MIN) return fminf(a, b);
   else if constexpr (OP == PPI_OP_MOD) return fmodf(a, b);
   else if constexpr (OP == PPI_OP_POW) return f_pow<MATH>(a, b);
   else {
      static_assert(OP == PPI_OP_DIV, "binary op");
      return p_div<MATH>(a, b, prot);
   }
}

// ERROR(X,Y) (src/definitions.h:18); the COST form guarded as documented in
// ppi_gpu.h.
__device__ __forceinline__ float apply_error(int ef, float x, float y, const float* cost, int cn) {
   switch (ef) {
   case PPI_EF_ABS: return fabsf(x - y);
   case PPI_EF_SQUARED: { float d = x - y; return d * d; }
   case PPI_EF_MISCLASS: return (x != y) ? 1.0f : 0.0f;
   default: {
      if (x != x) return x;
      const float fn = (float)cn;
      int ix = x >= fn ? cn - 1 : (x > 0.0f ? (int)x : 0);
      int iy = y != y ? 0 : (y >= fn ? cn - 1 : (y > 0.0f ? (int)y : 0));
      return __ldg(cost + ix * cn + iy);
   }
   }
}

__device__ __forceinline__ bool nonfinite(float v) { return isinf(v) || isnan(v); }

// apply_error with the error function fixed at compile time.
template <int EF>
__device__ __forceinline__ float apply_error_t(float x, float y, const float* cost, int cn) {
   if constexpr (EF == PPI_EF_ABS) return fabsf(x - y);
   else if constexpr (EF == PPI_EF_SQUARED) { const float d = x - y; return d * d; }
   else if constexpr (EF == PPI_EF_MISCLASS) return (x != y) ? 1.0f : 0.0f;
   else return apply_error(PPI_EF_COST, x, y, cost, cn);
}

// ---------------------------------------------------------------------------
// Best index.  The reference's accelerator picks it in two steps: the
// best_individual kernel (accelerator.cl:271-313) reduces each work-group of
// `group` programs by a strided tree that replaces the left value only when
// it is strictly greater, and util::PickNBest on the host takes the smallest
// group winner, ties to the largest group (accelerator.cc:871-880).  Two
// tied programs of one group meet at the lowest bit where their positions in
// the group differ, and the one with a 0 there is on the left and wins; so
// the tree's winner is the smallest value, then the smallest bit-reversed
// position.  The whole rule is therefore one lexicographic order -- value,
// then largest group, then smallest bit-reversed position -- and one 64-bit
// atomicMin per program implements it: the orderable value bits on top, the
// tie field below.  The sequential rule (ties to the largest index,
// sequential.cc:203) is the same order with groups of one program.
struct BestGeo {
   int group;                  // programs per work-group (1: sequential rule)
   int bits;                   // ceil(log2(group)): width of a position
   int groups;                 // ceil(n / group)
   int alpha_free;             // compare error/nlin without alpha*size (PP, PDP)
};

__host__ __device__ __forceinline__ uint32_t reverse_bits(uint32_t v, int bits) {
#ifdef __CUDA_ARCH__
   return bits > 0 ? (__brev(v) >> (32 - bits)) : 0u;
#else
   uint32_t r = 0;
   for (int b = 0; b < bits; ++b) r |= ((v >> b) & 1u) << (bits - 1 - b);
   return r;
#endif
}

// Tie field of program `prog`: smaller is better.
__host__ __device__ __forceinline__ uint32_t best_tie(const BestGeo& b, int prog) {
   const uint32_t g = (uint32_t)(prog / b.group), lo = (uint32_t)(prog - (int)g * b.group);
   return (((uint32_t)b.groups - 1u - g) << b.bits) | reverse_bits(lo, b.bits);
}

__host__ __device__ __forceinline__ int best_from_tie(const BestGeo& b, uint32_t tie) {
   const uint32_t g = (uint32_t)b.groups - 1u - (b.bits < 32 ? (tie >> b.bits) : 0u);
   const uint32_t lo = reverse_bits(tie & ((1u << b.bits) - 1u), b.bits);
   return (int)(g * (uint32_t)b.group + lo);
}

// 64-bit arg-min key: float order on top (FLT_MAX sentinels included), tie below.
__host__ __device__ __forceinline__ unsigned long long best_key(float f, uint32_t tie) {
   uint32_t u;
#ifdef __CUDA_ARCH__
   u = __float_as_uint(f);
#else
   __builtin_memcpy(&u, &f, 4);
#endif
   u = (u & 0x80000000u) ? ~u : (u | 0x80000000u);
   return ((unsigned long long)u << 32) | (unsigned long long)tie;
}

// Work-group size of the reference's best_individual launch: config value,
// else min(1024, ceil(population / compute units)) (accelerator.cc:289-294,
// 348) on a device whose work-groups reach 1024 items.
int resolve_best_group(int rule, int group, int population, int sm_count);
// Geometry of the rule for n programs; nullptr, or why it cannot be encoded.
const char* best_geometry(int rule, int group, int strategy, int n, BestGeo* out);

// ---------------------------------------------------------------------------
// One population of a batch (device memory).
struct PopDesc {
   const float* data;          // column-major, column c at data + c * ld
   int nlin, ncol, ld;
   int strategy, lanes, ef, reduce_max, prot, cost_n;
   const float* cost;
   float alpha;
   int prog_begin;             // first program of the population in the flat arrays
   int n;                      // programs
   BestGeo best;               // the population's best-index rule
};

struct TranslateArgs {
   const int32_t* phenotype;   // program i at phenotype + i * max_size
   const float* ephemeral;
   const int32_t* size;
   int n, max_size, ncol, nlin;
   const int2* lut;            // lut[sym - lut_min] = {op, literal bits}
   int lut_min, lut_len;
   uint2* code;                // program i at code + i * code_stride
   int code_stride;
   int2* meta;                 // {kind | rows << 8, code length}
   uint2* work;                // translator scratch: n x max_size
   unsigned long long* best_key;
   DevStats* stats;
   int* status;
   int prot;                   // PROTECTED, for constant folding
   int fold;                   // fold constant subexpressions
   int rows_main;              // row budget of the main pass
   int rows_wide;              // row budget of the wide pass (more rows: generic form)
   int* wide_list;             // plain evaluation: programs of the wide pass
   // batches: per-program population (nullptr for one population)
   const int* pop_of;
   const PopDesc* pops;
   unsigned* bucket_count;     // cost buckets of the work order: [0, 64) main pass, [64, 128) wide
   unsigned char* bucket_of;   // bucket of each program
};

struct EvalArgs {
   const float* data;          // column-major, column c at data + c * ld
   int nlin, ncol, ld;
   const uint2* code;
   int code_stride;
   const int2* meta;
   const int32_t* size;
   int n;
   float alpha;
   int ef, reduce_max, prot;
   const float* cost;
   int cost_n;
   int strategy, lanes;
   float* fitness;
   unsigned long long* best_key;
   DevStats* stats;
   int32_t* best_index;
   int* status;
   int rows;                   // row budget of this pass's tile
   int wide_pass;              // 0: main pass (skips kKindWide), 1: programs of wide_list
   const int* wide_list;
   int final_pass;             // this pass writes the best index
   BestGeo best;               // best-index rule
   // chunked family: records per chunk, chunks per program, programs per
   // group (items walk the groups in turn, chunk-major within a group), each
   // program's lane state between chunks ((R + 1) x block floats) and its
   // finished chunk count (zeroed before the launch)
   int chunk_records, n_chunks, chunk_group;
   float* chunk_state;
   unsigned* chunk_done;
};

struct BatchArgs {
   const PopDesc* pops;
   const int* pop_of;          // population of each program
   const int* order;           // work items: program indices, largest cost first
   int total;
   const uint2* code;
   int code_stride;
   const int2* meta;
   const int32_t* size;
   float* fitness;             // flat, all populations
   unsigned long long* pop_key;
   unsigned* pop_done;
   int32_t* best_index;        // one per population
   DevStats* stats;
   const unsigned* n_main;     // order[0, *n_main): main pass; the rest: wide pass
   int* status;
   int rows;                   // row budget of this pass's tile
   int wide_pass;
};

struct PredictArgs {
   const float* data;
   int nlin, ncol, ld;
   const uint2* code;
   const int2* meta;
   int prot;
   float* out;
   int* status;                // kStatus* bits
   int rows;                   // tile rows of the launch
};

// ---------------------------------------------------------------------------
// Constant adjoint (adjoint.cu).
enum : int { kAdjInvalid = 0, kAdjValid = 1, kAdjUnsupported = 2 };
// Most ephemeral constants of one program the adjoint differentiates.
constexpr int kAdjMaxConsts = 32;
// uint2 words of one program's adjoint code: the column header and list,
// the forward bytecode (an instruction per token plus the value pushes),
// the reverse instructions (two words each, at most two per operator) and
// the operand table.
inline int adjoint_code_stride(int max_size) { return 8 * max_size + 8; }

struct AdjointTranslateArgs {
   const int32_t* phenotype;
   const float* ephemeral;
   const int32_t* size;
   int n, max_size, ncol;
   const int2* lut;
   int lut_min, lut_len;
   uint2* code;                // program i at code + i * code_stride
   int code_stride;
   int2* meta;                 // {kAdj* | rows << 8, code length}
   uint2* work;                // n x 2 max_size scratch
   int* max_rows;              // over the population (atomicMax)
   int* max_consts;
   int* max_code;              // longest code (uint2 words)
};

struct AdjointArgs {
   const float* data;          // column-major, column c at data + c * ld
   int nlin, ncol, ld;
   const uint2* code;
   int code_stride;
   int code_words;             // shared-memory code region: the longest program's code
   const int2* meta;
   int max_size, ef, prot, max_consts;
   const int* order;           // programs of this launch
   int n_items;                // work items: programs x n_chunks
   int chunk, n_chunks;        // records per work item (a multiple of 1024), chunks per program
   double* psum;               // [program][chunk][max_consts] sums of the chunks
   int* pbad;                  // [program][chunk] a non-finite error was met
   unsigned* queue;
   int* status;                // kStatus* bits (tile copy timeouts)
};

struct AdjointFinishArgs {
   const uint2* code;
   int code_stride;
   const int2* meta;
   int n, max_size, max_consts, n_chunks;
   const double* psum;
   const int* pbad;
   float* grad;                // n x max_size
};

cudaError_t launch_adjoint_translate(const AdjointTranslateArgs& a, cudaStream_t s);
cudaError_t launch_adjoint_finish(const AdjointFinishArgs& a, cudaStream_t s);
// R: records per thread, 4 or 8 (kernels of adjoint_r4.cu / adjoint_r8.cu).
cudaError_t launch_adjoint(int math, int opset, int R, const AdjointArgs& a, int block, int grid, size_t smem,
                           cudaStream_t s);
cudaError_t adjoint_occupancy(int math, int opset, int R, int block, size_t smem, int* per_sm);
size_t adjoint_smem_bytes(int code_words, int max_consts, int rows, int block, int R);

// Evaluator launch geometry: lanes, block size P, records per thread R, and
// for the main and the wide pass the row budget, dynamic shared memory and a
// one-wave persistent grid.  The main pass runs the programs whose columns
// all fit its tile, on kernels without direct column reads; the wide pass
// the rest, on kernels that read the columns their tile cannot hold from
// global memory.  wide == false when every program fits the main tile (the
// wide pass is not launched).
struct Geometry {
   int lanes = 1, block = 128, R = 8, opset = kOpsetFull;
   int rows = 1, grid = 1;
   size_t smem = 0;
   int rows_wide = 1, grid_wide = 1;
   size_t smem_wide = 0;
   bool wide = false;
   bool aligned = false;
   int per_sm[2] = {0, 0};     // resident CTAs per SM of the two passes
   int wide_kernel = 1;        // direct-read kernel of the wide pass: 2 whole quads (PP, PDP), 1 any tile
   int main_kernel = 0;        // kernel of the main pass: 0, or kMainHi when its tile fits more CTAs
                               //   (both with kOneLane added for one lane, kChunked when chunked)
   bool chunked = false;       // record chunks in chunk-major order (kChunked kernels)
   int chunk_records = 0, n_chunks = 1;
   int chunk_group = 1;        // programs whose lane state and code stay in L2 together
};
// kOpsetArith when every op of the symbol table is in the ARITH set.
int opset_for(const ppi_symbol_entry* symbols, int n);
int resolve_lanes(int strategy, int lanes, int nlin, int sm_count);
// Returns nullptr on success, else why the configuration is unsupported.
// allow_chunk: the caller can hold the chunked family's lane state.
const char* plan_geometry(int strategy, int lanes, int math, int opset, int nlin, int ncol,
                          int code_stride, int n_max, int sm_count, Geometry* g, bool allow_chunk = false);
// Largest program row count on a dataset of ncol columns.
inline int max_program_rows(int ncol) { return kSlots + ncol + 1; }

// Kernel launchers (evaluate.cu / translate.cu).
cudaError_t launch_translate(int math, const TranslateArgs& a, cudaStream_t s);

// Host programs to the device (upload.cu): the used prefix of each row packed
// into a pinned staging area, one copy, then scattered into the device rows
// (d_ph / d_eph rows of max_size; d_size gets the sizes); pinned rows of at
// most 64 MB are copied as they are.  The staging area
// grows on demand and is reused: the caller must not start another upload on
// it before the stream has passed this one.
struct ProgramUpload {
   void* h_stage = nullptr;   // pinned
   void* d_stage = nullptr;
   size_t cap = 0;
   cudaEvent_t copied = nullptr;   // after the last copy out of h_stage
};
cudaError_t upload_programs(ProgramUpload* u, const int32_t* ph, const float* eph, const int32_t* size,
                            int n, int max_size, int32_t* d_ph, float* d_eph, int32_t* d_size,
                            int sm_count, cudaStream_t s);
void free_upload(ProgramUpload* u);
cudaError_t launch_evaluate(int math, int opset, int direct, const EvalArgs& a, int block, int grid,
                            size_t smem, cudaStream_t s);
cudaError_t launch_predict(int math, int opset, const PredictArgs& a, int block, int grid, size_t smem,
                           cudaStream_t s);
cudaError_t launch_evaluate_batch(int math, int opset, int direct, const BatchArgs& a, int block,
                                  int grid, size_t smem, cudaStream_t s);
cudaError_t launch_batch_order(const unsigned* bucket_count, unsigned* cursor,
                               const unsigned char* bucket_of, int* order, int total,
                               unsigned* n_main, cudaStream_t s);
cudaError_t evaluate_occupancy(int math, int opset, int direct, int block, size_t smem, int* blocks_per_sm);
cudaError_t evaluate_batch_occupancy(int math, int opset, int direct, int block, size_t smem,
                                     int* blocks_per_sm);
size_t evaluate_smem_bytes(int code_stride, int rows, int block, int R, int lanes, bool aligned);

}  // namespace ppi
