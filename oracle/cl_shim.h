/*
 * cl_shim.h -- lets the reference's OpenCL C kernel file
 * (src/interpreter/accelerator.cl) compile as host C++ so that its
 * evaluate_pp / evaluate_dp / evaluate_pdp / best_individual kernels can be
 * executed on the CPU as a parity oracle.
 *
 * TEST INFRASTRUCTURE ONLY: nothing in the product links this file.
 *
 * Each OpenCL work-item is a std::thread; the work-item's ids live in
 * thread_local storage and barrier() is a std::barrier shared by the
 * work-items of one work-group.  Math builtins resolve to the float
 * overloads of <cmath> (OpenCL C semantics: sin(float) is a float function),
 * which is what an OpenCL CPU device such as POCL provides.
 */
#ifndef PPI_CL_SHIM_H
#define PPI_CL_SHIM_H

#include <cfloat>
#include <cmath>
#include <barrier>

using std::sin; using std::cos; using std::tan; using std::exp; using std::exp2;
using std::log; using std::log2; using std::log10; using std::sqrt; using std::pow;
using std::fabs; using std::fmod; using std::fmax; using std::fmin; using std::round;
using std::ceil; using std::floor; using std::sinh; using std::isinf; using std::isnan;

#define __kernel
#define __global
#define __local
#define CLK_LOCAL_MEM_FENCE 1
#ifndef MAXFLOAT
#define MAXFLOAT FLT_MAX
#endif

struct ppi_cl_item {
   int global_id, local_id, group_id, local_size, num_groups;
   std::barrier<>* bar;
};
extern thread_local ppi_cl_item ppi_cl_cur;

static inline int get_global_id(int) { return ppi_cl_cur.global_id; }
static inline int get_local_id(int) { return ppi_cl_cur.local_id; }
static inline int get_group_id(int) { return ppi_cl_cur.group_id; }
static inline int get_local_size(int) { return ppi_cl_cur.local_size; }
static inline int get_num_groups(int) { return ppi_cl_cur.num_groups; }
static inline void barrier(int) { if (ppi_cl_cur.bar) ppi_cl_cur.bar->arrive_and_wait(); }
static inline float pown(float x, int n) { return std::pow(x, (float)n); }

/* OpenCL float builtins that <cmath> spells differently. */
static inline float exp10(float x) { return ::exp10f(x); }
static inline float native_divide(float x, float y) { return x / y; }
static inline float native_sin(float x) { return std::sin(x); }
static inline float native_cos(float x) { return std::cos(x); }
static inline float native_tan(float x) { return std::tan(x); }
static inline float native_sqrt(float x) { return std::sqrt(x); }
static inline float native_exp(float x) { return std::exp(x); }
static inline float native_exp2(float x) { return std::exp2(x); }
static inline float native_exp10(float x) { return ::exp10f(x); }
static inline float native_log(float x) { return std::log(x); }
static inline float native_log2(float x) { return std::log2(x); }
static inline float native_log10(float x) { return std::log10(x); }

#endif
