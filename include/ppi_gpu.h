/*
 * ppi_gpu.h -- C ABI of the GB300 (sm_103a) population evaluator for PPI.
 *
 * Replaces the OpenCL interpreter backend of PPI (src/interpreter/accelerator.{h,cc})
 * behind a plain C interface: plain pointers and sizes, status codes, no C++ or
 * CUDA types.  ppi-auto_gb300/adapter/accelerator_cuda.cc implements PPI's own
 * acc_interpret_init / acc_interpret / acc_print_time on top of it, so
 * src/ppi.cc and src/ppp.cc link against it unchanged.
 *
 * Which reference interface each entry point replaces:
 *   ppi_gpu_create ........... acc_interpret_init (accelerator.h:29, accelerator.cc:557-648):
 *                              device pick, kernel selection, buffer creation
 *   ppi_gpu_set_dataset ...... create_buffers (accelerator.cc:363-430): the one dataset
 *                              upload, float** rows as PPI's CSV reader builds them
 *   ppi_gpu_evaluate ......... acc_interpret (accelerator.h:36-40, accelerator.cc:651-891)
 *                              with ppp_mode = 0: fitness of every program + best index
 *   ppi_gpu_evaluate_launch /
 *   ppi_gpu_evaluate_wait .... the same call split at the point where acc_interpret runs
 *                              the island send/receive callbacks (accelerator.cc:733-743)
 *   ppi_gpu_predict .......... acc_interpret with ppp_mode = 1, prediction_mode = 1
 *                              (accelerator.cl:74,152,246; ppp.cc:98-118)
 *   ppi_gpu_set_grammar /
 *   ppi_gpu_decode ........... decode (src/ppi.cc:106-182), run on the device
 *   ppi_gpu_last_kernel_ms ... PROFILING event timing (accelerator.cc:894-940)
 *
 * Threading: one handle is used by one host thread at a time (PPI calls its
 * interpreter from the main thread only).  Several handles may coexist.
 */
#ifndef PPI_GPU_H
#define PPI_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PPI_GPU_ABI_VERSION 2

typedef enum {
   PPI_OK = 0,
   PPI_ERR_INVALID_ARGUMENT = 1,  /* bad pointer, size or configuration value        */
   PPI_ERR_CUDA = 2,              /* a CUDA call failed (message in last_error)       */
   PPI_ERR_OUT_OF_MEMORY = 3,     /* device or pinned host allocation failed          */
   PPI_ERR_UNSUPPORTED = 4,       /* configuration outside what this build supports   */
   PPI_ERR_NOT_READY = 5,         /* evaluate/predict before set_dataset, etc.        */
   PPI_ERR_DEVICE_STATUS = 6      /* a kernel reported an error through its status word */
} ppi_status;

/* Execution strategy (the reference's -strategy PP|DP|PDP, accelerator.cc:571).
 * Each reproduces the reference strategy's order of floating-point
 * accumulation, so fitness values are bit-identical to that strategy's kernel
 * given identical per-record errors:
 *   PP:  records summed in order per program (accelerator.cl:8-86; also the
 *        order of src/interpreter/sequential.cc);
 *   DP:  `lanes` records per work-group, a local tree per group, then the
 *        groups in order (accelerator.cl:89-171 + accelerator.cc:777-802);
 *   PDP: `lanes` work-items per program, work-item l summing records l, l+lanes,
 *        ..., then a local tree (accelerator.cl:174-268). */
typedef enum { PPI_STRATEGY_PP = 0, PPI_STRATEGY_DP = 1, PPI_STRATEGY_PDP = 2 } ppi_strategy;

/* ERROR(X,Y) (src/definitions.h:18): fabs((X)-(Y)), (((X)-(Y))*((X)-(Y))),
 * ((X)!=(Y)) and COST[(int)X][(int)Y].  The COST form is guarded: NaN X gives
 * a NaN error, and each index is (int)v clamped to [0, cost_n). */
typedef enum { PPI_EF_ABS = 0, PPI_EF_SQUARED = 1, PPI_EF_MISCLASS = 2, PPI_EF_COST = 3 } ppi_error_fn;

/* Transcendental arithmetic:
 *   FAST:   CUDA single-precision functions (sinf, expf, ...), within their
 *           documented ulp bounds of the correctly rounded result;
 *   PARITY: transcendental opcodes computed in double and rounded to float,
 *           as src/interpreter/sequential.cc does (it calls the double libm),
 *           which makes every prediction bit-identical to it;
 *   NATIVE: fast hardware approximations (__sinf, __expf, __fdividef, ...),
 *           the -DNATIVE build (src/interpreter/functions.h:59-193). */
typedef enum { PPI_MATH_FAST = 0, PPI_MATH_PARITY = 1, PPI_MATH_NATIVE = 2 } ppi_math;

/* Evaluator operations.  A grammar's Symbol values are mapped onto these by
 * the symbol table given to ppi_gpu_create (the `case T_X:` blocks of
 * src/interpreter/interpreter_core, and T_ATTRIBUTE / T_CONST / default of
 * accelerator.cl:37-51). */
typedef enum {
   PPI_OP_INVALID = 0,    /* unknown symbol: pushes NaN                              */
   PPI_OP_ATTRIBUTE,      /* pushes inputs[record][(int)ephemeral]                    */
   PPI_OP_CONST,          /* pushes ephemeral                                         */
   PPI_OP_LITERAL,        /* pushes the table entry's value (T_PI, T_0, T_N7, ...)    */
   PPI_OP_IF_THEN_ELSE,
   PPI_OP_AND, PPI_OP_OR, PPI_OP_XOR, PPI_OP_GREATER, PPI_OP_GREATEREQUAL, PPI_OP_LESS,
   PPI_OP_LESSEQUAL, PPI_OP_EQUAL, PPI_OP_NOTEQUAL, PPI_OP_ADD, PPI_OP_SUB, PPI_OP_MULT,
   PPI_OP_MEAN, PPI_OP_MAX, PPI_OP_MIN, PPI_OP_MOD, PPI_OP_POW, PPI_OP_DIV,
   PPI_OP_NOT, PPI_OP_ABS, PPI_OP_POW2, PPI_OP_POW3, PPI_OP_POW4, PPI_OP_POW5, PPI_OP_NEG,
   PPI_OP_ROUND, PPI_OP_CEIL, PPI_OP_FLOOR, PPI_OP_EXP, PPI_OP_EXP10, PPI_OP_EXP2,
   PPI_OP_SIN, PPI_OP_COS, PPI_OP_STEP, PPI_OP_SIGN, PPI_OP_LOGISTIC, PPI_OP_GAMMA,
   PPI_OP_GAUSS, PPI_OP_SQRT, PPI_OP_LOG, PPI_OP_LOG10, PPI_OP_LOG2, PPI_OP_TAN,
   PPI_OP_COUNT
} ppi_op;

/* One grammar terminal: its Symbol enum value, the op it performs and, for
 * PPI_OP_LITERAL, the float it pushes. */
typedef struct {
   int32_t symbol;
   int32_t op;
   float value;
} ppi_symbol_entry;

/* Which program the best index names (the `index` output of acc_interpret).
 *   ACCELERATOR (default): what src/interpreter/accelerator.cc returns.  The
 *     best_individual kernel (accelerator.cl:271-313) reduces work-groups of
 *     `best_group` programs by a strided tree that keeps the left value on
 *     ties, and util::PickNBest (src/util/Util.h:158-173) then takes the
 *     smallest group winner, ties to the largest group
 *     (accelerator.cc:871-880).  PP and PDP compare the alpha-free values
 *     error/nlin (kernel2 reads buffer_vector before the host adds
 *     alpha*size, accelerator.cc:500,720,848-849); DP compares the fitness
 *     with alpha*size (buffer_error, accelerator.cc:491,801,812).
 *   SEQUENTIAL: what src/interpreter/sequential.cc returns: PickNBest over
 *     the fitness with alpha*size, ties to the largest index (:203).
 * Both leave the fitness values unchanged. */
typedef enum { PPI_BEST_ACCELERATOR = 0, PPI_BEST_SEQUENTIAL = 1 } ppi_best_rule;

typedef struct {
   int32_t max_size;          /* MAX_PHENOTYPE_SIZE: row stride of phenotype/ephemeral  */
   int32_t population_size;   /* largest n given to evaluate                            */
   int32_t strategy;          /* ppi_strategy                                           */
   int32_t lanes;             /* PDP work-items per program / DP records per group;
                                 <= 0 picks the reference's rule for a 152-CU device   */
   int32_t error_fn;          /* ppi_error_fn                                           */
   int32_t reduce_max;        /* REDUCEMAX: maximum of error*nlin instead of the sum    */
   int32_t protected_fns;     /* PROTECTED: DIV, SQRT, LOG and TAN return 1 off-domain */
   int32_t math;              /* ppi_math                                               */
   const float* cost;         /* cost_n x cost_n, row index (int)X; PPI_EF_COST only    */
   int32_t cost_n;
   const ppi_symbol_entry* symbols;
   int32_t n_symbols;
   int32_t device;            /* CUDA device ordinal                                    */
   int32_t best_rule;         /* ppi_best_rule                                          */
   int32_t best_group;        /* ACCELERATOR: programs per best_individual work-group;
                                 <= 0 picks the reference's rule for a 152-CU device,
                                 min(1024, ceil(population_size / CUs)) (accelerator.cc:348) */
} ppi_gpu_config;

typedef struct ppi_gpu ppi_gpu;

/* Library version and build target, e.g. "ppi_gpu 1 sm_103a". */
const char* ppi_gpu_version(void);

ppi_status ppi_gpu_create(const ppi_gpu_config* config, ppi_gpu** out);
ppi_status ppi_gpu_destroy(ppi_gpu* h);

/* Message of the last failure on this handle ("" if none). */
const char* ppi_gpu_last_error(const ppi_gpu* h);

/* Dataset upload, copied once to the device in column-major order.  rows[i]
 * points at ncol floats of record i; the last column is the target (it may be
 * absent for prediction-only use). */
ppi_status ppi_gpu_set_dataset(ppi_gpu* h, const float* const* rows, int32_t nlin, int32_t ncol);
/* Same, from one row-major nlin x ncol array. */
ppi_status ppi_gpu_set_dataset_rowmajor(ppi_gpu* h, const float* data, int32_t nlin, int32_t ncol);

/* Same, straight from PPI's training CSV file into the column-major device
 * layout, read by the rules of PPI's own reader (read(), src/main.cc:32-122):
 * empty and '#' lines skipped, ',' separated, an optional header line, values
 * read as `istringstream >> float`, NaN / infinite / unreadable values and
 * ragged lines rejected.  A file the reference reader rejects is rejected
 * with PPI_ERR_INVALID_ARGUMENT and the reference's message in last_error.
 * nlin / ncol (may be NULL) receive the shape read. */
ppi_status ppi_gpu_set_dataset_csv(ppi_gpu* h, const char* path, int32_t* nlin, int32_t* ncol);

/* The same reader without a device: shape into nlin / ncol and, when
 * colmajor is not NULL, the values at colmajor[c * ld + r] (ld >= nlin,
 * capacity >= ld * ncol floats); message (may be NULL) receives the reader's
 * message.  No reference counterpart beyond read(): for callers that stage
 * the dataset themselves (e.g. ppi_gpu_evaluate_noalloc). */
ppi_status ppi_csv_read(const char* path, float* colmajor, int64_t capacity, int32_t ld,
                        int32_t* nlin, int32_t* ncol, char* message, int32_t message_len);

/* One generation: phenotype / ephemeral are n rows of max_size entries, size
 * holds n program lengths (0 = invalid program).  fitness[i] receives
 * error/nlin + alpha*size[i] (FLT_MAX for invalid or non-finite programs, as
 * the reference strategy defines); *best_index (may be NULL) receives the
 * best program under config->best_rule (ppi_best_rule above). */
ppi_status ppi_gpu_evaluate(ppi_gpu* h, const int32_t* phenotype, const float* ephemeral,
                            const int32_t* size, int32_t n, float alpha, float* fitness,
                            int32_t* best_index);

/* The same call split in two: launch copies the inputs and starts the kernels;
 * wait blocks until they finish and fills fitness / best_index (the pointers
 * given to launch must stay valid until wait returns).  Programs in pageable
 * memory (PPI's own arrays) are packed on the host before launch returns and
 * may be changed at once; programs in pinned memory of at most 64 MB of rows
 * are read by the asynchronous copy itself and must stay unchanged until wait
 * returns. */
ppi_status ppi_gpu_evaluate_launch(ppi_gpu* h, const int32_t* phenotype, const float* ephemeral,
                                   const int32_t* size, int32_t n, float alpha, float* fitness,
                                   int32_t* best_index);
ppi_status ppi_gpu_evaluate_wait(ppi_gpu* h);

/* Device-resident form: every pointer is device memory; work is queued on
 * `stream` (a cudaStream_t, NULL = the legacy default stream) and the call
 * returns without synchronising. */
ppi_status ppi_gpu_evaluate_device(ppi_gpu* h, const int32_t* d_phenotype,
                                   const float* d_ephemeral, const int32_t* d_size, int32_t n,
                                   float alpha, float* d_fitness, int32_t* d_best_index,
                                   void* stream);

/* Per-record predictions of one program (out: nlin floats). */
ppi_status ppi_gpu_predict(ppi_gpu* h, const int32_t* phenotype, const float* ephemeral,
                           int32_t size, float* out);

/* Grammar tables for device decode: alternative a = rule_first[nt] + k is
 * gramatica[nt][k] with alt_len[a] symbols alt_syms[a * max_rule ...]. */
ppi_status ppi_gpu_set_grammar(ppi_gpu* h, const int32_t* rule_first, const int32_t* rule_count,
                               int32_t n_nonterminals, const int32_t* alt_len,
                               const int32_t* alt_syms, int32_t n_alternatives, int32_t max_rule,
                               int32_t t_const, int32_t t_attribute);

/* Decode n genomes of nb bytes (one 0/1 byte per bit, GENOME_TYPE) on the
 * device, as src/ppi.cc:106-182 does with bg bits per codon and bc bits per
 * constant in [lo, hi].  Outputs (host, any may be NULL): phenotype/ephemeral
 * rows of max_size, size. */
ppi_status ppi_gpu_decode(ppi_gpu* h, const uint8_t* genomes, int32_t n, int32_t nb, int32_t bg,
                          int32_t bc, float lo, float hi, int32_t* phenotype, float* ephemeral,
                          int32_t* size);

/* Decode + evaluate in one call: genomes in, fitness / best index out. */
ppi_status ppi_gpu_decode_evaluate(ppi_gpu* h, const uint8_t* genomes, int32_t n, int32_t nb,
                                   int32_t bg, int32_t bc, float lo, float hi, float alpha,
                                   float* fitness, int32_t* best_index, int32_t* size);

/* Device time of the last evaluation's kernels, in milliseconds. */
ppi_status ppi_gpu_last_kernel_ms(ppi_gpu* h, float* ms);

/* Device time of the translator and of the evaluator kernel of the last
 * evaluate call (it waits for that call's work to finish). */
ppi_status ppi_gpu_last_stage_ms(ppi_gpu* h, float* translate_ms, float* evaluate_ms);

/* Lane count in use (PDP work-items per program, DP records per group, 1 for
 * PP), resolved by ppi_gpu_set_dataset; 0 before a dataset is set. */
int32_t ppi_gpu_lanes(const ppi_gpu* h);

/* Number of kernel launches the last evaluate / predict / decode call made. */
int32_t ppi_gpu_last_launch_count(const ppi_gpu* h);

/* Launch plan for the current dataset (no reference counterpart: the
 * evaluator's own geometry).  Each output may be NULL: block the threads per
 * CTA, rows the main pass's tile rows, n_chunks the record chunks a program is
 * evaluated in (1, or more when the programs walk a dataset larger than L2
 * together, chunk by chunk).  PPI_ERR_NOT_READY before a dataset is set. */
ppi_status ppi_gpu_geometry(const ppi_gpu* h, int32_t* block, int32_t* rows, int32_t* n_chunks);

/* Inspection of the last evaluate call's translation (waits for it).  No
 * reference counterpart: the bytecode is this library's own.  code_stride
 * receives the uint2 words of one program's code; opset the opcode set of the
 * kernels that run it (0 every opcode, 1 the arithmetic set); code (may be
 * NULL) n * code_stride * 2 uint32 words; meta (may be NULL) n * 2 int32
 * {kind | rows << 8, code length}.  n at most the last call's n. */
ppi_status ppi_gpu_translation(ppi_gpu* h, int32_t n, uint32_t* code, int32_t* meta,
                               int32_t* code_stride, int32_t* opset);

/* Compute capability the evaluator kernels were compiled for, as loaded on
 * the current device (cudaFuncAttributes::binaryVersion, 103 for sm_103a);
 * -1 when no device is usable.  No reference counterpart: a build check. */
int32_t ppi_gpu_kernel_arch(void);

/* ---- constant adjoint --------------------------------------------------------
 * No counterpart in the reference: an addition for refining the ephemeral
 * constants of programs by gradient steps, while ppi_gpu_evaluate stays the
 * fitness judge.  gradient (n x max_size) receives d(fitness)/d(ephemeral[i][k])
 * at every CONST token k of program i and 0 at the other tokens, for the
 * fitness (1/nlin) sum_n EF(X_n, Y_n) of the handle's dataset: the sum
 * reduction (REDUCEMAX is rejected) with the absolute or squared error (other
 * error functions are piecewise constant in X and are rejected).  The forward
 * sweep runs in the handle's math mode.  A program whose error is non-finite
 * on some record (its fitness is the FLT_MAX sentinel) gets a zero gradient;
 * a malformed program, or one with more than 32 constants, gets NaN.
 * Synchronous. */
ppi_status ppi_gpu_constant_gradient(ppi_gpu* h, const int32_t* phenotype, const float* ephemeral,
                                     const int32_t* size, int32_t n, float* gradient);

/* ---- batches: many populations in one step ---------------------------------
 * No single reference function: this evaluates what several acc_interpret
 * calls would (one per population, e.g. one per island or per independent
 * run) in one step: a main and a wide pass, each one persistent launch over
 * all populations' programs.  Each population keeps its own dataset,
 * strategy, lanes, error function, REDUCEMAX and PROTECTED settings, and its
 * fitness values are bit-identical to ppi_gpu_evaluate on that population
 * alone. */
typedef struct {
   const float* rows;         /* row-major nlin x ncol, target in the last column (copied) */
   int32_t nlin, ncol;
   int32_t n;                 /* programs in this population                         */
   int32_t strategy, lanes, error_fn, reduce_max, protected_fns;
   const float* cost;         /* PPI_EF_COST only (copied)                           */
   int32_t cost_n;
} ppi_batch_population;

#define PPI_BATCH_GRAPH 1     /* capture the step into a CUDA graph and replay it   */
#define PPI_BATCH_AUTOTUNE 2  /* on the first call, time the block shapes and tile row
                                 budgets (one per occupancy level), keep the fastest */

typedef struct ppi_batch ppi_batch;

/* config: max_size (row stride), math, symbols and device are used; the other
 * fields are per population. */
ppi_status ppi_batch_create(const ppi_gpu_config* config, int32_t n_pops,
                            const ppi_batch_population* pops, ppi_batch** out);
ppi_status ppi_batch_destroy(ppi_batch* b);
const char* ppi_batch_last_error(const ppi_batch* b);
/* alpha (the complexity penalty) of each population; 0 until set. */
ppi_status ppi_batch_set_alpha(ppi_batch* b, const float* alpha);
/* All populations' programs concatenated in population order (rows of
 * max_size); fitness likewise; best_index: one per population. */
ppi_status ppi_batch_evaluate(ppi_batch* b, const int32_t* phenotype, const float* ephemeral,
                              const int32_t* size, float* fitness, int32_t* best_index,
                              int32_t flags);
/* Device-resident form on `stream`; PPI_BATCH_GRAPH needs a non-NULL stream. */
ppi_status ppi_batch_evaluate_device(ppi_batch* b, const int32_t* d_phenotype,
                                     const float* d_ephemeral, const int32_t* d_size,
                                     float* d_fitness, int32_t* d_best_index, void* stream,
                                     int32_t flags);
/* Device time of the last step (waits for it). */
ppi_status ppi_batch_last_kernel_ms(ppi_batch* b, float* ms);
/* Kernels the last step launched (translator, work order, evaluator passes). */
ppi_status ppi_batch_last_launch_count(const ppi_batch* b, int32_t* n);
/* Block size and main-pass grid in use; rows (may be NULL) receives the tile
 * rows of the main and the wide pass; tune_ms (may be NULL) the autotuner's
 * timings of the 64- and 128-thread shapes at their best rows (-1: shape does
 * not fit). */
ppi_status ppi_batch_shape(const ppi_batch* b, int32_t* block, int32_t* grid, int32_t* rows,
                           float* tune_ms);
/* Fix the shape instead of tuning it: block 64 or 128 threads, and the main
 * pass's tile rows (0: the most rows at full occupancy; clamped to what fits).
 * Programs whose tile needs more rows run in the wide pass.  Changes speed
 * only, never a result. */
ppi_status ppi_batch_set_shape(ppi_batch* b, int32_t block, int32_t rows);

/* No counterpart in the reference.  One generation evaluated without
 * allocating any memory, for callers that cannot allocate where they evaluate:
 * an application whose device memory another allocator has already reserved,
 * an island process that must keep a fixed footprint once running, or a loop
 * that cannot afford the device-wide synchronisation of cudaMalloc/cudaFree.
 * The caller passes everything in device memory it owns: the dataset
 * column-major (column c at d_data + c*ld, ld >= nlin, ld a multiple of 4,
 * d_data 16-byte aligned, target in the last column), the programs (rows of
 * config->max_size) and the outputs.  Work is queued on `stream` (a
 * cudaStream_t); the call does not synchronise.  config->population_size is
 * ignored (the automatic best_group uses n); config->symbols and config->cost
 * are read from host memory by each call, with cudaMemcpyAsync.
 * Scratch comes from one fixed 64 MiB array inside the library, which every
 * GPU that loads the library holds until exit.  A batch needing more
 * (about 16,000 programs of max_size 128), or a symbol table spanning more
 * than 2^22 values, is rejected with PPI_ERR_UNSUPPORTED and a message on
 * stderr.  The first call on each device looks up the array's device address
 * (cudaGetSymbolAddress) and caches the launch geometry.  All calls share the
 * array: calls that overlap on the GPU race, so serialise them.  d_status (device memory, may be NULL) receives the
 * kernels' status bits once the call's work is done: 0 when every program
 * ran; 1 a malformed program needs a deeper stack than the generic
 * interpreter's (its fitness is FLT_MAX); 2 a tile copy did not complete
 * within its bounded wait; 4 an instruction outside the kernel's opcode set
 * (the fitness values are not to be used after 2 or 4). */
ppi_status ppi_gpu_evaluate_noalloc(const ppi_gpu_config* config, const float* d_data,
                                    int32_t nlin, int32_t ncol, int32_t ld,
                                    const int32_t* d_phenotype, const float* d_ephemeral,
                                    const int32_t* d_size, int32_t n, float alpha,
                                    float* d_fitness, int32_t* d_best_index, int32_t* d_status,
                                    void* stream);

#ifdef __cplusplus
}
#endif
#endif
