/*
 * ppi_oracle.h -- CPU oracle for PPI's population-evaluation hot path.
 *
 * TEST INFRASTRUCTURE.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference legs of bench.py may load this library, and only as
 * the checker or the timed CPU baseline: the product never calls it.
 *
 * Parity is pinned: tests/test_oracle_golden.py checks every entry point here
 * bit-for-bit against golden vectors produced by the reference's own code
 * (src/interpreter/sequential.cc, src/interpreter/accelerator.cl and the
 * decode functions of src/ppi.cc) compiled from its sources by
 * oracle/build_ref.py; tests/golden/make_golden.py made the vectors.
 */
#ifndef PPI_ORACLE_H
#define PPI_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
   int nlin, ncol;              /* dataset: nlin records x ncol columns, target = last column */
   const float* rows;           /* row-major nlin x ncol (the reference's float** flattened)   */
   int error_fn;                /* 0 fabs((X)-(Y)), 1 squared, 2 ((X)!=(Y)), 3 COST[X][Y]       */
   const float* cost;           /* cost_n x cost_n, row = (int)X                                */
   int cost_n;
   int reduce_max;              /* REDUCEMAX                                                    */
   int protected_fns;           /* PROTECTED                                                    */
   int float_math;              /* 0: sequential.cc (double libm); 1: OpenCL float builtins     */
   const int32_t* sym_values;   /* Symbol value -> op (ppi_op) and literal value                */
   const int32_t* sym_ops;
   const float* sym_literals;
   int n_syms;
   int threads;                 /* OpenMP threads for ppio_evaluate (<=0: all)                  */
} ppio_config;

/* strategy: 0 = sequential / PP order, 1 = DP with work-groups of `lanes`
 * records, 2 = PDP with `lanes` work-items per program.
 * Writes n fitness values (alpha * size included, as the host adds it). */
int ppio_evaluate(const ppio_config* cfg, int strategy, int lanes, const int32_t* phenotype,
                  const float* ephemeral, const int32_t* size, int max_size, int n, float alpha,
                  float* fitness);

/* Per-record prediction of one program (ppp prediction mode). */
int ppio_predict(const ppio_config* cfg, const int32_t* phenotype, const float* ephemeral,
                 int size, float* out);

/* util::PickNBest over n values (src/util/Util.h:158-173): the best index,
 * ties resolved toward the largest index. */
int ppio_best_index(const float* fitness, int n);

/* The best index acc_interpret returns: best_individual
 * (src/interpreter/accelerator.cl:271-313) over work-groups of `group`
 * values, then PickNBest(1) over the group winners
 * (src/interpreter/accelerator.cc:871-880).  PP/PDP pass the alpha-free
 * per-program values, DP the alpha-included fitness. */
int ppio_best_index_accelerator(const float* values, int n, int group);

/* FP64 re-evaluation (no counterpart in the reference): every node, the error
 * function and the record sum in double precision, records in order;
 * fitness[i] = sum/nlin + alpha*size[i] (REDUCEMAX: the max of error*nlin),
 * HUGE_VAL for size 0 or a non-finite error.  The value the float evaluators
 * approximate. */
int ppio_evaluate64(const ppio_config* cfg, const int32_t* phenotype, const float* ephemeral,
                    const int32_t* size, int max_size, int n, double alpha, double* fitness);

/* Genome decode (src/ppi.cc:106-182).  Tables as returned by
 * ppi_gpu.grammar.Grammar.decode_tables().  genomes: n x nb bytes of 0/1.
 * Rows of phenotype/ephemeral hold max_size entries.  Returns 0. */
int ppio_decode(const int32_t* rule_first, const int32_t* rule_count, const int32_t* alt_len,
                const int32_t* alt_syms, int max_rule, int t_const, int t_attribute,
                const uint8_t* genomes, int n, int nb, int bg, int bc, float lo, float hi,
                int max_size, int32_t* phenotype, float* ephemeral, int32_t* size);

/* FP64 constant adjoint (no counterpart in the reference; the checker of the
 * GPU constant gradient): fitness[i] = (1/nlin) sum_n EF(p_n, y_n) in double
 * precision with EF absolute (error_fn 0) or squared (1), HUGE_VAL when an
 * error is non-finite (gradient 0), NaN for a malformed program (gradient
 * NaN); grad[i][k] = dF/d ephemeral[i][k] at CONST tokens, 0 elsewhere.
 * ephemeral: n x max_size doubles.  float_forward = 1: the node values are
 * the reference's float values (cfg->float_math selects the libm rounding, as
 * in ppio_evaluate) and only the reverse sweep and the sums are double: the
 * gradient of exactly the function the float evaluator computes. */
int ppio_adjoint64(const ppio_config* cfg, const int32_t* phenotype, const double* ephemeral,
                   const int32_t* size, int max_size, int n, int float_forward, double* fitness,
                   double* grad);

#ifdef __cplusplus
}
#endif
#endif
