/*
 * ppi_oracle.c -- CPU restatement of PPI's population-evaluation hot path.
 *
 * TEST INFRASTRUCTURE (see ppi_oracle.h): the checker for the CUDA evaluator
 * and the timed CPU baseline.  Parity pinned against the reference's own code
 * by tests/test_oracle_golden.py.  Build with -ffp-contract=off so that no
 * multiply-add is fused (x86-64 and aarch64 then round identically).
 *
 * What is restated, and from where:
 *   op semantics .......... src/interpreter/interpreter_core:1-151 (opcodes),
 *                           src/interpreter/functions.h:59-193 (protected math),
 *                           src/interpreter/accelerator.cl:37-51 (ATTRIBUTE,
 *                           CONST, unknown symbol -> NaN)
 *   math precision ........ float_math=0: sequential.cc calls the double libm
 *                           (<cmath> without `using std`, sequential.cc:16-76),
 *                           so sin(x) is (float)sin((double)x); float_math=1:
 *                           OpenCL float builtins (accelerator.cl)
 *   sequential / PP ....... sequential.cc:133-190, accelerator.cl:19-85
 *   PDP ................... accelerator.cl:174-268 (+ host alpha add,
 *                           accelerator.cc:848-849)
 *   DP .................... accelerator.cl:89-171 + host reduction
 *                           accelerator.cc:777-802
 *   best index ............ util::PickNBest, src/util/Util.h:158-173
 *   decode ................ src/ppi.cc:106-182
 *
 * Defined where the reference is undefined (the CUDA evaluator does the same):
 *   - an operator with too few operands on the stack (malformed program)
 *     reads NaN for the missing operand instead of stack[-1];
 *   - an attribute index outside [0, ncol) pushes NaN instead of reading
 *     outside the row;
 *   - size > max_size (the reference can decode such a size, see
 *     ppio_decode) is an invalid program, like size == 0;
 *   - COST: X is NaN -> the error is NaN; otherwise each index is (int)v
 *     clamped to [0, cost_n).
 */
#include "ppi_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* Op codes: enum ppi_op of include/ppi_gpu.h. */
enum {
   OP_INVALID = 0, OP_ATTRIBUTE, OP_CONST, OP_LITERAL,
   OP_IF_THEN_ELSE,
   OP_AND, OP_OR, OP_XOR, OP_GREATER, OP_GREATEREQUAL, OP_LESS, OP_LESSEQUAL, OP_EQUAL,
   OP_NOTEQUAL, OP_ADD, OP_SUB, OP_MULT, OP_MEAN, OP_MAX, OP_MIN, OP_MOD, OP_POW, OP_DIV,
   OP_NOT, OP_ABS, OP_POW2, OP_POW3, OP_POW4, OP_POW5, OP_NEG, OP_ROUND, OP_CEIL, OP_FLOOR,
   OP_EXP, OP_EXP10, OP_EXP2, OP_SIN, OP_COS, OP_STEP, OP_SIGN, OP_LOGISTIC, OP_GAMMA,
   OP_GAUSS, OP_SQRT, OP_LOG, OP_LOG10, OP_LOG2, OP_TAN,
   OP_COUNT
};

static int arity(int op) {
   if (op == OP_IF_THEN_ELSE) return 3;
   if (op >= OP_AND && op <= OP_DIV) return 2;
   if (op >= OP_NOT && op < OP_COUNT) return 1;
   return 0;
}

/* float constants of src/interpreter/functions.h:19-57 */
#define PPI_PI_F 3.14159274101257f
#define PPI_PI_2_F 1.57079637050629f
#define PPI_E_F 2.71828174591064f

/* ---- math, selected by float_math (functions.h:59-193) ------------------ */
static float m_sin(float x, int fm) { return fm ? sinf(x) : (float)sin((double)x); }
static float m_cos(float x, int fm) { return fm ? cosf(x) : (float)cos((double)x); }
static float m_tan(float x, int fm) { return fm ? tanf(x) : (float)tan((double)x); }
static float m_exp(float x, int fm) { return fm ? expf(x) : (float)exp((double)x); }
static float m_exp2(float x, int fm) { return fm ? exp2f(x) : (float)exp2((double)x); }
static float m_exp10(float x, int fm) { return fm ? exp10f(x) : (float)exp10((double)x); }
static float m_log(float x, int fm) { return fm ? logf(x) : (float)log((double)x); }
static float m_log2(float x, int fm) { return fm ? log2f(x) : (float)log2((double)x); }
static float m_log10(float x, int fm) { return fm ? log10f(x) : (float)log10((double)x); }
static float m_sqrt(float x, int fm) { return fm ? sqrtf(x) : (float)sqrt((double)x); }

static float f_div(float x, float y, int prot) { return (prot && y == 0.0f) ? 1.0f : x / y; }
static float f_sqrt(float x, int prot, int fm) { return (prot && x < 0.0f) ? 1.0f : m_sqrt(x, fm); }
static float f_log(float x, int prot, int fm) { return (prot && x < 1.0f) ? 1.0f : m_log(x, fm); }
static float f_log10(float x, int prot, int fm) { return (prot && x < 1.0f) ? 1.0f : m_log10(x, fm); }
static float f_log2(float x, int prot, int fm) { return (prot && x < 1.0f) ? 1.0f : m_log2(x, fm); }
static float f_tan(float x, int prot, int fm) {
   if (prot && (fabsf(x) == PPI_PI_2_F || fabsf(x) == 3.0f * PPI_PI_2_F)) return 1.0f;
   return m_tan(x, fm);
}

/* T_GAMMA (interpreter_core:127-129).  Under sequential.cc the sinh and pow
 * calls are double, so x*sinh(..) and the final product are double
 * expressions that are rounded to float where SQRT takes its float argument
 * and where the result is stored. */
static float f_gamma(float x, int prot, int fm) {
   if (fm) {
      float a = (x / PPI_E_F) * f_sqrt(x * sinhf(1.0f / x), prot, fm);
      return powf(a, x) * f_sqrt(2.0f * PPI_PI_F / x, prot, fm);
   }
   double s = sinh((double)(1.0f / x));
   float a = (x / PPI_E_F) * f_sqrt((float)((double)x * s), prot, fm);
   double p = pow((double)a, (double)x);
   return (float)(p * (double)f_sqrt(2.0f * PPI_PI_F / x, prot, fm));
}

static float f_pow(float a, float b, int fm) { return fm ? powf(a, b) : (float)pow((double)a, (double)b); }

static int truthy(float v) { return v != 0.0f; }   /* (bool)float: NaN is true */

/* One record of one program: right-to-left over the prefix array
 * (accelerator.cl:28-53, sequential.cc:142-164).  `ops` already mapped. */
static float eval_record(const int* ops, const float* lit, int size, const float* row, int ncol,
                         int prot, int fm, float* stack) {
   int top = -1;
   const float qnan = NAN;
#define POP_OK(k) (top + 1 >= (k))
   for (int i = size - 1; i >= 0; --i) {
      int op = ops[i];
      int ar = arity(op);
      if (ar > 0 && !POP_OK(ar)) {
         /* malformed: the missing (deepest) operands read as NaN */
         int have = top + 1, miss = ar - have;
         for (int k = have - 1; k >= 0; --k) stack[k + miss] = stack[k];
         for (int k = 0; k < miss; ++k) stack[k] = qnan;
         top = ar - 1;
      }
      float a = top >= 0 ? stack[top] : 0.0f;
      float b = top >= 1 ? stack[top - 1] : 0.0f;
      float r;
      switch (op) {
      case OP_ATTRIBUTE: {
         float v = lit[i];
         stack[++top] = (v >= 0.0f && v < (float)ncol) ? row[(int)v] : qnan;
         continue;
      }
      case OP_CONST: case OP_LITERAL: stack[++top] = lit[i]; continue;
      case OP_INVALID: stack[++top] = qnan; continue;
      case OP_IF_THEN_ELSE:
         stack[top - 2] = truthy(a) ? b : stack[top - 2];
         top -= 2;
         continue;
      case OP_AND: r = (truthy(a) && truthy(b)) ? 1.0f : 0.0f; break;
      case OP_OR: r = (truthy(a) || truthy(b)) ? 1.0f : 0.0f; break;
      case OP_XOR: r = (!truthy(a) != !truthy(b)) ? 1.0f : 0.0f; break;
      case OP_GREATER: r = (a > b) ? 1.0f : 0.0f; break;
      case OP_GREATEREQUAL: r = (a >= b) ? 1.0f : 0.0f; break;
      case OP_LESS: r = (a < b) ? 1.0f : 0.0f; break;
      case OP_LESSEQUAL: r = (a <= b) ? 1.0f : 0.0f; break;
      case OP_EQUAL: r = (a == b) ? 1.0f : 0.0f; break;
      case OP_NOTEQUAL: r = (a != b) ? 1.0f : 0.0f; break;
      case OP_ADD: r = a + b; break;
      case OP_SUB: r = a - b; break;
      case OP_MULT: r = a * b; break;
      case OP_MEAN: r = (a + b) / 2.0f; break;
      case OP_MAX: r = fmaxf(a, b); break;
      case OP_MIN: r = fminf(a, b); break;
      case OP_MOD: r = fmodf(a, b); break;
      case OP_POW: r = f_pow(a, b, fm); break;
      case OP_DIV: r = f_div(a, b, prot); break;
      default: r = 0.0f; break;
      }
      if (op >= OP_AND && op <= OP_DIV) {
         stack[top - 1] = r;
         --top;
         continue;
      }
      switch (op) {
      case OP_NOT: r = truthy(a) ? 0.0f : 1.0f; break;
      case OP_ABS: r = fabsf(a); break;
      case OP_POW2: r = a * a; break;
      case OP_POW3: r = a * a * a; break;
      case OP_POW4: r = a * a * a * a; break;
      case OP_POW5: r = a * a * a * a * a; break;
      case OP_NEG: r = -a; break;
      case OP_ROUND: r = roundf(a); break;
      case OP_CEIL: r = ceilf(a); break;
      case OP_FLOOR: r = floorf(a); break;
      case OP_EXP: r = m_exp(a, fm); break;
      case OP_EXP10: r = m_exp10(a, fm); break;
      case OP_EXP2: r = m_exp2(a, fm); break;
      case OP_SIN: r = m_sin(a, fm); break;
      case OP_COS: r = m_cos(a, fm); break;
      case OP_STEP: r = (a >= 0.0f) ? 1.0f : 0.0f; break;
      case OP_SIGN: r = a > 0.0f ? 1.0f : (a < 0.0f ? -1.0f : 0.0f); break;
      case OP_LOGISTIC: r = 1.0f / (1.0f + m_exp(-a, fm)); break;
      case OP_GAMMA: r = f_gamma(a, prot, fm); break;
      case OP_GAUSS: r = m_exp(-a * a, fm); break;
      case OP_SQRT: r = f_sqrt(a, prot, fm); break;
      case OP_LOG: r = f_log(a, prot, fm); break;
      case OP_LOG10: r = f_log10(a, prot, fm); break;
      case OP_LOG2: r = f_log2(a, prot, fm); break;
      case OP_TAN: r = f_tan(a, prot, fm); break;
      default: r = qnan; break;
      }
      stack[top] = r;
   }
#undef POP_OK
   return top >= 0 ? stack[top] : qnan;
}

/* ERROR(X,Y) variants (src/definitions.h:18, CMakeLists.txt:26-33). */
static float error_fn(const ppio_config* c, float x, float y) {
   switch (c->error_fn) {
   case 0: return fabsf(x - y);
   case 1: return (x - y) * (x - y);
   case 2: return (x != y) ? 1.0f : 0.0f;
   case 3: {
      if (x != x) return NAN;
      int n = c->cost_n;
      int ix = x >= (float)n ? n - 1 : (x > 0.0f ? (int)x : 0);
      int iy = y != y ? 0 : (y >= (float)n ? n - 1 : (y > 0.0f ? (int)y : 0));
      return c->cost[ix * n + iy];
   }
   }
   return NAN;
}

static int nonfinite(float v) { return isinf(v) || isnan(v); }

/* Symbol -> op lookup for one program. */
static void map_program(const ppio_config* c, const int32_t* ph, const float* eph, int size,
                        int* ops, float* lit) {
   for (int i = 0; i < size; ++i) {
      int op = OP_INVALID;
      float v = eph[i];
      for (int k = 0; k < c->n_syms; ++k)
         if (c->sym_values[k] == ph[i]) {
            op = c->sym_ops[k];
            if (op == OP_LITERAL) v = c->sym_literals[k];
            break;
         }
      ops[i] = op;
      lit[i] = v;
   }
}

/* Accumulate one error into a lane (accelerator.cl:62-70; sequential.cc:171-179).
 * Returns 1 when the lane must stop (non-finite error). */
static int accumulate(const ppio_config* c, float* pe, float err) {
   if (nonfinite(err)) { *pe = FLT_MAX; return 1; }
   if (c->reduce_max) {
      float e = err * (float)c->nlin;
      *pe = (e > *pe) ? e : *pe;
   } else {
      *pe += err;
   }
   return 0;
}

/* __local tree of accelerator.cl:157-167 / :252-262 over L values. */
static void local_tree(const ppio_config* c, float* pe, int L) {
   int p = 1;
   while (p < L) p <<= 1;
   for (int s = p / 2; s > 0; s >>= 1)
      for (int l = 0; l < s; ++l)
         if (l + s < L) {
            if (c->reduce_max) pe[l] = (pe[l + s] > pe[l]) ? pe[l + s] : pe[l];
            else pe[l] += pe[l + s];
         }
}

static float eval_program(const ppio_config* c, int strategy, int lanes, const int* ops,
                          const float* lit, int size, float alpha, float* stack, float* pe) {
   const int nlin = c->nlin, ncol = c->ncol;
   const int prot = c->protected_fns, fm = c->float_math;
   const float fnlin = (float)nlin;
   if (strategy == 1) {
      /* DP: per-group partials, then the host reduction. */
      int L = lanes, G = (nlin + L - 1) / L;
      float sum = 0.0f;
      for (int g = 0; g < G; ++g) {
         float part;
         if (size == 0) {
            part = FLT_MAX;
         } else {
            for (int l = 0; l < L; ++l) {
               int n = g * L + l;
               pe[l] = 0.0f;
               if (n < nlin) {
                  const float* row = c->rows + (size_t)n * ncol;
                  float x = eval_record(ops, lit, size, row, ncol, prot, fm, stack);
                  pe[l] = error_fn(c, x, row[ncol - 1]);
               }
            }
            local_tree(c, pe, L);
            part = pe[0];
         }
         if (nonfinite(part)) { sum = FLT_MAX; break; }
         if (c->reduce_max) {
            float e = part * fnlin;
            sum = (e > sum) ? e : sum;
         } else {
            sum += part;
         }
      }
      if (nonfinite(sum)) return FLT_MAX;
      return sum / fnlin + alpha * (float)size;
   }
   if (size == 0) return FLT_MAX;
   if (strategy == 2) {
      /* PDP: lane l takes records l, l+L, ... (accelerator.cl:195-249). */
      int L = lanes;
      for (int l = 0; l < L; ++l) {
         pe[l] = 0.0f;
         for (int n = l; n < nlin; n += L) {
            const float* row = c->rows + (size_t)n * ncol;
            float x = eval_record(ops, lit, size, row, ncol, prot, fm, stack);
            if (accumulate(c, &pe[l], error_fn(c, x, row[ncol - 1]))) break;
         }
      }
      local_tree(c, pe, L);
      float v = nonfinite(pe[0]) ? FLT_MAX : pe[0] / fnlin;
      return v + alpha * (float)size;
   }
   /* sequential / PP */
   float sum = 0.0f;
   for (int n = 0; n < nlin; ++n) {
      const float* row = c->rows + (size_t)n * ncol;
      float x = eval_record(ops, lit, size, row, ncol, prot, fm, stack);
      if (accumulate(c, &sum, error_fn(c, x, row[ncol - 1]))) break;
   }
   if (nonfinite(sum)) return FLT_MAX;
   return sum / fnlin + alpha * (float)size;
}

int ppio_evaluate(const ppio_config* c, int strategy, int lanes, const int32_t* phenotype,
                  const float* ephemeral, const int32_t* size, int max_size, int n, float alpha,
                  float* fitness) {
   if (strategy != 0 && lanes < 1) return 1;
   int failed = 0;
#ifdef _OPENMP
   int nt = c->threads > 0 ? c->threads : omp_get_max_threads();
#pragma omp parallel num_threads(nt)
#endif
   {
      int* ops = (int*)malloc(sizeof(int) * (size_t)(max_size + 1));
      float* lit = (float*)malloc(sizeof(float) * (size_t)(max_size + 1));
      float* stack = (float*)malloc(sizeof(float) * (size_t)(max_size + 4));
      float* pe = (float*)malloc(sizeof(float) * (size_t)(lanes > 0 ? lanes : 1));
      if (!ops || !lit || !stack || !pe) {
         failed = 1;
      } else {
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 1)
#endif
         for (int i = 0; i < n; ++i) {
            int sz = size[i];
            if (sz < 0 || sz > max_size) sz = 0;
            map_program(c, phenotype + (size_t)i * max_size, ephemeral + (size_t)i * max_size, sz,
                        ops, lit);
            fitness[i] = eval_program(c, strategy, lanes, ops, lit, sz, alpha, stack, pe);
         }
      }
      free(ops); free(lit); free(stack); free(pe);
   }
   return failed;
}

int ppio_predict(const ppio_config* c, const int32_t* phenotype, const float* ephemeral, int size,
                 float* out) {
   if (size < 0) return 1;
   int* ops = (int*)malloc(sizeof(int) * (size_t)(size + 1));
   float* lit = (float*)malloc(sizeof(float) * (size_t)(size + 1));
   float* stack = (float*)malloc(sizeof(float) * (size_t)(size + 4));
   if (!ops || !lit || !stack) { free(ops); free(lit); free(stack); return 1; }
   map_program(c, phenotype, ephemeral, size, ops, lit);
   for (int n = 0; n < c->nlin; ++n)
      out[n] = eval_record(ops, lit, size, c->rows + (size_t)n * c->ncol, c->ncol,
                           c->protected_fns, c->float_math, stack);
   free(ops); free(lit); free(stack);
   return 0;
}

int ppio_best_index(const float* f, int n) {
   /* priority_queue<pair<float,int>> over (-f, i): the top is the largest
    * (-f, i), i.e. the smallest f and, among equal f, the largest i.  NaN
    * never occurs in fitness (non-finite values become FLT_MAX). */
   int best = 0;
   for (int i = 1; i < n; ++i) {
      float a = -f[i], b = -f[best];
      if (a > b || (a == b)) best = i;
   }
   return best;
}

/* The accelerator's best index: the best_individual kernel
 * (src/interpreter/accelerator.cl:271-313) run with work-groups of `group`
 * items over ceil(n / group) groups, each group reducing its values by the
 * strided local tree that keeps the left operand unless it is strictly
 * greater (:290-307), then util::PickNBest(1) over the groups' winners on the
 * host (src/interpreter/accelerator.cc:871-880; src/util/Util.h:158-173):
 * the smallest winner value, ties to the largest group.  Items past n read
 * MAXFLOAT (:286); their index is never used here because a group winner is
 * a padding item only when every real item of its group exceeds MAXFLOAT,
 * which the callers' values (FLT_MAX sentinels for non-finite errors) never
 * do.  Returns -1 when n or group is not positive. */
int ppio_best_index_accelerator(const float* vec, int n, int group) {
   if (n < 1 || group < 1) return -1;
   const int groups = (n + group - 1) / group;
   float* lo_best = (float*)malloc(sizeof(float) * (size_t)group);
   int* lo_idx = (int*)malloc(sizeof(int) * (size_t)group);
   float* pb = (float*)malloc(sizeof(float) * (size_t)groups);
   int* pi = (int*)malloc(sizeof(int) * (size_t)groups);
   if (!lo_best || !lo_idx || !pb || !pi) {
      free(lo_best); free(lo_idx); free(pb); free(pi);
      return -1;
   }
   /* next_power_of_2 of the kernel: pown(2, ceil(log2(lo_size))) / 2 */
   int half = 1;
   while (half < group) half <<= 1;
   half >>= 1;
   for (int g = 0; g < groups; ++g) {
      for (int l = 0; l < group; ++l) {
         const int gl = g * group + l;
         lo_best[l] = gl < n ? vec[gl] : FLT_MAX;
         lo_idx[l] = gl < n ? gl : -1;
      }
      for (int s = half; s > 0; s /= 2)
         for (int l = 0; l < s; ++l)
            if (l + s < group && lo_best[l] > lo_best[l + s]) {
               lo_best[l] = lo_best[l + s];
               lo_idx[l] = lo_idx[l + s];
            }
      pb[g] = lo_best[0];
      pi[g] = lo_idx[0];
   }
   const int w = ppio_best_index(pb, groups);
   const int best = pi[w];
   free(lo_best); free(lo_idx); free(pb); free(pi);
   return best;
}

/* ---- decode (src/ppi.cc:106-182) ---------------------------------------- */
typedef struct {
   const int32_t *rule_first, *rule_count, *alt_len, *alt_syms;
   int max_rule, t_const, t_attribute, nb, bg, bc, max_size;
   float lo, hi;
   const uint8_t* genome;
   int32_t* ph;
   float* eph;
} dec_ctx;

/* decode_rule, src/ppi.cc:106-122: bg bits, least significant first,
 * modulo the number of alternatives; NULL (-1) when the genome is used up. */
static int decode_rule(dec_ctx* d, int* allele, int nt) {
   if (*allele + d->bg > d->nb) return -1;
   unsigned v = 0;
   for (int i = 0; i < d->bg; ++i)
      if (d->genome[(*allele)++]) v += (1u << i);
   return d->rule_first[nt] + (int)(v % (unsigned)d->rule_count[nt]);
}

/* decode_real, src/ppi.cc:124-137: float(v) * (b - a) in float, then the
 * division by (2^bc - 1.0) and the addition in double. */
static float decode_real(dec_ctx* d, int* allele) {
   if (*allele + d->bc > d->nb) return 0.0f;
   unsigned long long v = 0;
   for (int i = 0; i < d->bc; ++i)
      if (d->genome[(*allele)++]) v += (1ull << i);
   float num = (float)v * (d->hi - d->lo);
   return (float)((double)d->lo + (double)num / ((double)(1ull << d->bc) - 1.0));
}

/* decode, src/ppi.cc:139-182.  The reference writes terminals without
 * checking pos against max_size (only the entry of decode() checks it), so a
 * rule whose later symbols are terminals can write past the row and return a
 * size above max_size; that genome is invalid here (0). */
static int decode_rec(dec_ctx* d, int* allele, int pos, int nt) {
   int r = decode_rule(d, allele, nt);
   if (r < 0 || pos >= d->max_size) return 0;
   const int32_t* syms = d->alt_syms + (size_t)r * d->max_rule;
   for (int i = 0; i < d->alt_len[r]; ++i) {
      int s = syms[i];
      if (s >= 10000) {
         if (pos >= d->max_size) return -1;
         d->ph[pos] = s;
         if (s == d->t_const) {
            d->eph[pos] = decode_real(d, allele);
         } else if (s >= 20000) {
            d->ph[pos] = d->t_attribute;
            d->eph[pos] = (float)(s - 20000);
         }
         ++pos;
      } else {
         pos = decode_rec(d, allele, pos, s);
         if (pos <= 0) return pos;
      }
   }
   return pos;
}

int ppio_decode(const int32_t* rule_first, const int32_t* rule_count, const int32_t* alt_len,
                const int32_t* alt_syms, int max_rule, int t_const, int t_attribute,
                const uint8_t* genomes, int n, int nb, int bg, int bc, float lo, float hi,
                int max_size, int32_t* phenotype, float* ephemeral, int32_t* size) {
   for (int i = 0; i < n; ++i) {
      dec_ctx d = {rule_first, rule_count, alt_len, alt_syms, max_rule, t_const, t_attribute,
                   nb, bg, bc, max_size, lo, hi, genomes + (size_t)i * nb,
                   phenotype + (size_t)i * max_size, ephemeral + (size_t)i * max_size};
      int allele = 0;
      int s = decode_rec(&d, &allele, 0, 0);
      size[i] = s > 0 ? s : 0;
   }
   return 0;
}

/* One operator in the reference's float semantics (the switch of
 * eval_record, with the operands as separate values: a = stack[top],
 * b = stack[top-1], c = stack[top-2]). */
static float f_node(int op, float a, float b, float c, int prot, int fm) {
   switch (op) {
   case OP_IF_THEN_ELSE: return truthy(a) ? b : c;
   case OP_AND: return (truthy(a) && truthy(b)) ? 1.0f : 0.0f;
   case OP_OR: return (truthy(a) || truthy(b)) ? 1.0f : 0.0f;
   case OP_XOR: return (!truthy(a) != !truthy(b)) ? 1.0f : 0.0f;
   case OP_GREATER: return (a > b) ? 1.0f : 0.0f;
   case OP_GREATEREQUAL: return (a >= b) ? 1.0f : 0.0f;
   case OP_LESS: return (a < b) ? 1.0f : 0.0f;
   case OP_LESSEQUAL: return (a <= b) ? 1.0f : 0.0f;
   case OP_EQUAL: return (a == b) ? 1.0f : 0.0f;
   case OP_NOTEQUAL: return (a != b) ? 1.0f : 0.0f;
   case OP_ADD: return a + b;
   case OP_SUB: return a - b;
   case OP_MULT: return a * b;
   case OP_MEAN: return (a + b) / 2.0f;
   case OP_MAX: return fmaxf(a, b);
   case OP_MIN: return fminf(a, b);
   case OP_MOD: return fmodf(a, b);
   case OP_POW: return f_pow(a, b, fm);
   case OP_DIV: return f_div(a, b, prot);
   case OP_NOT: return truthy(a) ? 0.0f : 1.0f;
   case OP_ABS: return fabsf(a);
   case OP_POW2: return a * a;
   case OP_POW3: return a * a * a;
   case OP_POW4: return a * a * a * a;
   case OP_POW5: return a * a * a * a * a;
   case OP_NEG: return -a;
   case OP_ROUND: return roundf(a);
   case OP_CEIL: return ceilf(a);
   case OP_FLOOR: return floorf(a);
   case OP_EXP: return m_exp(a, fm);
   case OP_EXP10: return m_exp10(a, fm);
   case OP_EXP2: return m_exp2(a, fm);
   case OP_SIN: return m_sin(a, fm);
   case OP_COS: return m_cos(a, fm);
   case OP_STEP: return (a >= 0.0f) ? 1.0f : 0.0f;
   case OP_SIGN: return a > 0.0f ? 1.0f : (a < 0.0f ? -1.0f : 0.0f);
   case OP_LOGISTIC: return 1.0f / (1.0f + m_exp(-a, fm));
   case OP_GAMMA: return f_gamma(a, prot, fm);
   case OP_GAUSS: return m_exp(-a * a, fm);
   case OP_SQRT: return f_sqrt(a, prot, fm);
   case OP_LOG: return f_log(a, prot, fm);
   case OP_LOG10: return f_log10(a, prot, fm);
   case OP_LOG2: return f_log2(a, prot, fm);
   case OP_TAN: return f_tan(a, prot, fm);
   default: return NAN;
   }
}

/* ---- FP64 constant adjoint (test infrastructure) -------------------------
 * No counterpart in the reference.  The checker for the GPU constant
 * gradient: each program evaluated in double precision with the same
 * protected-function rules, F = (1/nlin) sum_n EF(p_n, y_n) with EF absolute
 * (error_fn 0) or squared (1), and dF/d constant by a reverse sweep over a
 * per-record tape of node values.  Ephemerals are given in double so that a
 * finite-difference caller can perturb them by less than a float ulp. */
static double d_value(int op, double a, double b, double c, int prot) {
   switch (op) {
   case OP_ADD: return a + b;
   case OP_SUB: return a - b;
   case OP_MULT: return a * b;
   case OP_DIV: return (prot && b == 0.0) ? 1.0 : a / b;
   case OP_MEAN: return (a + b) / 2.0;
   case OP_MAX: return fmax(a, b);
   case OP_MIN: return fmin(a, b);
   case OP_POW: return pow(a, b);
   case OP_ABS: return fabs(a);
   case OP_POW2: return a * a;
   case OP_POW3: return a * a * a;
   case OP_POW4: return a * a * a * a;
   case OP_POW5: return a * a * a * a * a;
   case OP_NEG: return -a;
   case OP_EXP: return exp(a);
   case OP_EXP2: return exp2(a);
   case OP_EXP10: return exp10(a);
   case OP_SIN: return sin(a);
   case OP_COS: return cos(a);
   case OP_LOGISTIC: return 1.0 / (1.0 + exp(-a));
   case OP_GAUSS: return exp(-a * a);
   case OP_SQRT: return (prot && a < 0.0) ? 1.0 : sqrt(a);
   case OP_LOG: return (prot && a < 1.0) ? 1.0 : log(a);
   case OP_LOG2: return (prot && a < 1.0) ? 1.0 : log2(a);
   case OP_LOG10: return (prot && a < 1.0) ? 1.0 : log10(a);
   case OP_TAN: return tan(a);
   case OP_IF_THEN_ELSE: return a != 0.0 ? b : c;
   case OP_NOT: return a != 0.0 ? 0.0 : 1.0;
   case OP_ROUND: return round(a);
   case OP_CEIL: return ceil(a);
   case OP_FLOOR: return floor(a);
   case OP_STEP: return a >= 0.0 ? 1.0 : 0.0;
   case OP_SIGN: return a > 0.0 ? 1.0 : (a < 0.0 ? -1.0 : 0.0);
   case OP_AND: return (a != 0.0 && b != 0.0) ? 1.0 : 0.0;
   case OP_OR: return (a != 0.0 || b != 0.0) ? 1.0 : 0.0;
   case OP_XOR: return ((a != 0.0) != (b != 0.0)) ? 1.0 : 0.0;
   case OP_GREATER: return a > b ? 1.0 : 0.0;
   case OP_GREATEREQUAL: return a >= b ? 1.0 : 0.0;
   case OP_LESS: return a < b ? 1.0 : 0.0;
   case OP_LESSEQUAL: return a <= b ? 1.0 : 0.0;
   case OP_EQUAL: return a == b ? 1.0 : 0.0;
   case OP_NOTEQUAL: return a != b ? 1.0 : 0.0;
   case OP_MOD: return fmod(a, b);
   default: return NAN;   /* GAMMA and unknown ops are not differentiated */
   }
}

static void d_partials(int op, double a, double b, double c, double v, int prot, double* da,
                       double* db, double* dc) {
   *da = 0.0; *db = 0.0; *dc = 0.0;
   (void)c;
   switch (op) {
   case OP_ADD: *da = 1.0; *db = 1.0; break;
   case OP_SUB: *da = 1.0; *db = -1.0; break;
   case OP_MULT: *da = b; *db = a; break;
   case OP_DIV: if (!(prot && b == 0.0)) { *da = 1.0 / b; *db = -v / b; } break;
   case OP_MEAN: *da = 0.5; *db = 0.5; break;
   case OP_MAX: if (a >= b) *da = 1.0; else *db = 1.0; break;
   case OP_MIN: if (a <= b) *da = 1.0; else *db = 1.0; break;
   case OP_POW: *da = b * v / a; *db = v * log(a); break;
   case OP_MOD: *da = 1.0; *db = -trunc(a / b); break;
   case OP_ABS: *da = a > 0.0 ? 1.0 : (a < 0.0 ? -1.0 : 0.0); break;
   case OP_POW2: *da = 2.0 * a; break;
   case OP_POW3: *da = 3.0 * a * a; break;
   case OP_POW4: *da = 4.0 * a * a * a; break;
   case OP_POW5: *da = 5.0 * a * a * a * a; break;
   case OP_NEG: *da = -1.0; break;
   case OP_EXP: *da = v; break;
   case OP_EXP2: *da = v * log(2.0); break;
   case OP_EXP10: *da = v * log(10.0); break;
   case OP_SIN: *da = cos(a); break;
   case OP_COS: *da = -sin(a); break;
   case OP_LOGISTIC: *da = v * (1.0 - v); break;
   case OP_GAUSS: *da = -2.0 * a * v; break;
   case OP_SQRT: *da = (prot && a < 0.0) ? 0.0 : 0.5 / v; break;
   case OP_LOG: *da = (prot && a < 1.0) ? 0.0 : 1.0 / a; break;
   case OP_LOG2: *da = (prot && a < 1.0) ? 0.0 : 1.0 / (a * log(2.0)); break;
   case OP_LOG10: *da = (prot && a < 1.0) ? 0.0 : 1.0 / (a * log(10.0)); break;
   case OP_TAN: *da = 1.0 + v * v; break;
   case OP_IF_THEN_ELSE: if (a != 0.0) *db = 1.0; else *dc = 1.0; break;
   case OP_GAMMA: *da = NAN; break;
   default: break;
   }
}

/* ---- FP64 re-evaluation (test infrastructure) ----------------------------
 * No counterpart in the reference.  The same programs over the same float
 * data, every node computed in double precision (double libm, the protected
 * rules of functions.h:99-193 applied to double operands), the error function
 * and the sum over records in double: the value the float evaluators
 * approximate, so their error can be stated against it. */
static double d_gamma(double x, int prot) {
   const double e = (double)PPI_E_F, pi = (double)PPI_PI_F;
   double s = x * sinh(1.0 / x);
   double a = (x / e) * ((prot && s < 0.0) ? 1.0 : sqrt(s));
   double q = 2.0 * pi / x;
   return pow(a, x) * ((prot && q < 0.0) ? 1.0 : sqrt(q));
}

static double d_node(int op, double a, double b, double c, int prot) {
   if (op == OP_GAMMA) return d_gamma(a, prot);
   if (op == OP_TAN && prot &&
       (fabs(a) == (double)PPI_PI_2_F || fabs(a) == (double)(3.0f * PPI_PI_2_F)))
      return 1.0;
   return d_value(op, a, b, c, prot);
}

static double eval_record64(const int* ops, const float* lit, int size, const float* row, int ncol,
                            int prot, double* stack) {
   int top = -1;
   for (int i = size - 1; i >= 0; --i) {
      int op = ops[i], ar = arity(op);
      if (ar > 0 && top + 1 < ar) {
         int have = top + 1, miss = ar - have;
         for (int k = have - 1; k >= 0; --k) stack[k + miss] = stack[k];
         for (int k = 0; k < miss; ++k) stack[k] = NAN;
         top = ar - 1;
      }
      if (ar == 0) {
         double v;
         if (op == OP_ATTRIBUTE) {
            float x = lit[i];
            v = (x >= 0.0f && x < (float)ncol) ? (double)row[(int)x] : NAN;
         } else if (op == OP_INVALID) {
            v = NAN;
         } else {
            v = (double)lit[i];
         }
         stack[++top] = v;
         continue;
      }
      double a = stack[top], b = ar > 1 ? stack[top - 1] : 0.0, cc = ar > 2 ? stack[top - 2] : 0.0;
      top -= ar - 1;
      stack[top] = d_node(op, a, b, cc, prot);
   }
   return top >= 0 ? stack[top] : NAN;
}

static double error_fn64(const ppio_config* c, double x, double y) {
   switch (c->error_fn) {
   case 0: return fabs(x - y);
   case 1: return (x - y) * (x - y);
   case 2: return (x != y) ? 1.0 : 0.0;
   case 3: {
      if (x != x) return NAN;
      int n = c->cost_n;
      int ix = x >= (double)n ? n - 1 : (x > 0.0 ? (int)x : 0);
      int iy = y != y ? 0 : (y >= (double)n ? n - 1 : (y > 0.0 ? (int)y : 0));
      return (double)c->cost[ix * n + iy];
   }
   }
   return NAN;
}

int ppio_evaluate64(const ppio_config* c, const int32_t* phenotype, const float* ephemeral,
                    const int32_t* size, int max_size, int n, double alpha, double* fitness) {
   int failed = 0;
#ifdef _OPENMP
   int nt = c->threads > 0 ? c->threads : omp_get_max_threads();
#pragma omp parallel num_threads(nt)
#endif
   {
      int* ops = (int*)malloc(sizeof(int) * (size_t)(max_size + 1));
      float* lit = (float*)malloc(sizeof(float) * (size_t)(max_size + 1));
      double* stack = (double*)malloc(sizeof(double) * (size_t)(max_size + 4));
      if (!ops || !lit || !stack) {
         failed = 1;
      } else {
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 1)
#endif
         for (int i = 0; i < n; ++i) {
            int sz = size[i];
            if (sz <= 0 || sz > max_size) { fitness[i] = HUGE_VAL; continue; }
            map_program(c, phenotype + (size_t)i * max_size, ephemeral + (size_t)i * max_size, sz,
                        ops, lit);
            double sum = 0.0;
            int nonfin = 0;
            for (int r = 0; r < c->nlin; ++r) {
               const float* row = c->rows + (size_t)r * c->ncol;
               double x = eval_record64(ops, lit, sz, row, c->ncol, c->protected_fns, stack);
               double e = error_fn64(c, x, (double)row[c->ncol - 1]);
               if (isinf(e) || isnan(e)) { nonfin = 1; break; }
               if (c->reduce_max) {
                  double m = e * (double)c->nlin;
                  sum = m > sum ? m : sum;
               } else {
                  sum += e;
               }
            }
            fitness[i] = nonfin ? HUGE_VAL : sum / (double)c->nlin + alpha * (double)sz;
         }
      }
      free(ops); free(lit); free(stack);
   }
   return failed;
}

int ppio_adjoint64(const ppio_config* c, const int32_t* phenotype, const double* ephemeral,
                   const int32_t* size, int max_size, int n, int float_forward, double* fitness,
                   double* grad) {
   const int nlin = c->nlin, ncol = c->ncol, prot = c->protected_fns, fm = c->float_math;
#ifdef _OPENMP
   int nt = c->threads > 0 ? c->threads : omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(nt)
#endif
   for (int i = 0; i < n; ++i) {
      int sz = size[i];
      double* g = grad + (size_t)i * max_size;
      for (int k = 0; k < max_size; ++k) g[k] = 0.0;
      if (sz <= 0 || sz > max_size) { fitness[i] = HUGE_VAL; continue; }
      int* ops = (int*)malloc(sizeof(int) * (size_t)sz * 5);
      double* val = (double*)malloc(sizeof(double) * (size_t)sz * 3);
      int* sub = ops + sz;
      int* ch = ops + 2 * sz;          /* ch[3k .. 3k+2]: children of position k */
      double* lit = val;
      double* v = val + sz;
      double* adj = val + 2 * sz;
      /* map tokens */
      for (int k = 0; k < sz; ++k) {
         int op = OP_INVALID;
         double x = ephemeral[(size_t)i * max_size + k];
         for (int q = 0; q < c->n_syms; ++q)
            if (c->sym_values[q] == phenotype[(size_t)i * max_size + k]) {
               op = c->sym_ops[q];
               if (op == OP_LITERAL) x = (double)c->sym_literals[q];
               break;
            }
         if (op == OP_ATTRIBUTE && !(x >= 0.0 && x < (double)ncol)) { op = OP_INVALID; }
         ops[k] = op;
         lit[k] = x;
      }
      /* structure (right to left): subtree sizes and children */
      int depth = 0, bad = 0;
      for (int k = sz - 1; k >= 0; --k) {
         int ar = arity(ops[k]);
         if (depth < ar) { bad = 1; break; }
         depth = depth - ar + 1;
         sub[k] = 1;
         int cpos = k + 1;
         for (int j = 0; j < 3; ++j) {
            ch[3 * k + j] = -1;
            if (j < ar) { ch[3 * k + j] = cpos; sub[k] += sub[cpos]; cpos += sub[cpos]; }
         }
      }
      if (bad || depth != 1 || sub[0] != sz) {
         fitness[i] = NAN;
         for (int k = 0; k < sz; ++k) g[k] = NAN;
         free(ops); free(val);
         continue;
      }
      double F = 0.0;
      int nonfin = 0;
      for (int r = 0; r < nlin && !nonfin; ++r) {
         const float* row = c->rows + (size_t)r * ncol;
         for (int k = sz - 1; k >= 0; --k) {
            int op = ops[k], ar = arity(op);
            if (ar == 0) {
               if (op == OP_ATTRIBUTE) v[k] = (double)row[(int)lit[k]];
               else if (op == OP_INVALID) v[k] = NAN;
               else v[k] = lit[k];
            } else {
               double a = v[ch[3 * k]], b = ar > 1 ? v[ch[3 * k + 1]] : 0.0,
                      cc = ar > 2 ? v[ch[3 * k + 2]] : 0.0;
               v[k] = float_forward ? (double)f_node(op, (float)a, (float)b, (float)cc, prot, fm)
                                    : d_value(op, a, b, cc, prot);
            }
            if (float_forward && (ops[k] == OP_CONST || ops[k] == OP_LITERAL)) v[k] = (double)(float)v[k];
         }
         double y = (double)row[ncol - 1], d = v[0] - y;
         double err = c->error_fn == 1 ? d * d : fabs(d);
         if (float_forward) {
            /* the float error and its non-finite rule, as the evaluator */
            float fd = (float)v[0] - row[ncol - 1];
            float fe = c->error_fn == 1 ? fd * fd : fabsf(fd);
            if (isinf(fe) || isnan(fe)) { nonfin = 1; break; }
         }
         if (isinf(err) || isnan(err)) { nonfin = 1; break; }
         F += err;
         adj[0] = (c->error_fn == 1 ? 2.0 * d : (d > 0.0 ? 1.0 : (d < 0.0 ? -1.0 : 0.0))) / (double)nlin;
         for (int k = 0; k < sz; ++k) {
            int op = ops[k], ar = arity(op);
            if (ar == 0) {
               if (op == OP_CONST) g[k] += adj[k];
               continue;
            }
            double a = v[ch[3 * k]], b = ar > 1 ? v[ch[3 * k + 1]] : 0.0,
                   cc = ar > 2 ? v[ch[3 * k + 2]] : 0.0, pa, pb, pc;
            d_partials(op, a, b, cc, v[k], prot, &pa, &pb, &pc);
            /* a zero adjoint propagates zero (never 0 x inf = NaN) */
            const int live = adj[k] != 0.0;
            adj[ch[3 * k]] = live ? adj[k] * pa : 0.0;
            if (ar > 1) adj[ch[3 * k + 1]] = live ? adj[k] * pb : 0.0;
            if (ar > 2) adj[ch[3 * k + 2]] = live ? adj[k] * pc : 0.0;
         }
      }
      if (nonfin) {
         fitness[i] = HUGE_VAL;
         for (int k = 0; k < sz; ++k) g[k] = 0.0;
      } else {
         fitness[i] = F / (double)nlin;
      }
      free(ops); free(val);
   }
   return 0;
}
