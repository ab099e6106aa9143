// opcost.cu -- how fast this GPU computes each evaluator opcode's arithmetic
// alone: the evaluator's own per-opcode routines (unop / binop of
// ppi_internal.cuh) applied to 8 independent values per thread in a register
// loop over the whole GPU, with no interpreter, no data movement and no
// reduction.  The benchmark turns these rates and a workload's opcode
// histogram into the op-mix ceiling of its roofline: the throughput the
// evaluator would reach if every token cost only its arithmetic.
//
// Measurement code for bench.py only (libppi_opcost.so); the evaluator
// library does not contain it.
#include <cuda_runtime.h>

#include "ppi_internal.cuh"

namespace {

constexpr int kVals = 8;

// OP < 0: the loop alone (the input step and the sum), subtracted by the host.
template <int OP>
__global__ void __launch_bounds__(256) op_loop_kernel(float* out, int iters, float lo, float hi, float k,
                                                      int prot) {
   const int g = blockIdx.x * blockDim.x + threadIdx.x;
   const float span = hi - lo;
   const float d = span / (1021.0f * (float)iters);
   float t[kVals], s[kVals];
#pragma unroll
   for (int r = 0; r < kVals; ++r) {
      t[r] = lo + span * (float)((g * kVals + r) % 1021) / 1021.0f;
      s[r] = 0.0f;
   }
#pragma unroll 1
   for (int i = 0; i < iters; ++i) {
#pragma unroll
      for (int r = 0; r < kVals; ++r) {
         float y;
         if constexpr (OP < 0) y = t[r];
         else if constexpr (OP >= PPI_OP_NOT) y = ppi::unop<OP, ppi::kMathFast>(t[r], prot);
         else y = ppi::binop<OP, ppi::kMathFast>(t[r], k, prot);
         s[r] += y;
         t[r] += d;
      }
   }
   float acc = 0.0f;
#pragma unroll
   for (int r = 0; r < kVals; ++r) acc += s[r];
   out[g] = acc;
}

using Kernel = void (*)(float*, int, float, float, float, int);

template <int OP>
Kernel kernel_of(int op) {
   if constexpr (OP >= PPI_OP_COUNT) {
      return nullptr;
   } else {
      if (op == OP) return op_loop_kernel<OP>;
      return kernel_of<OP + 1>(op);
   }
}

}  // namespace

extern "C" {

// Times `iters` loop iterations of opcode `op` (fast math; -1: the loop
// alone) over blocks_per_sm x SMs blocks of 256 threads, inputs spread over
// [lo, hi), binary opcodes with the constant k as right operand.  *ms: device
// time of one launch (best of `reps`, after one warm launch); *ops: opcode
// evaluations per launch.  Returns 0, or a CUDA error code.
int ppi_opcost_measure(int op, int prot, int iters, int reps, float lo, float hi, float k,
                       float* ms, double* ops) {
   Kernel kern = op < 0 ? op_loop_kernel<-1>
                        : (op >= PPI_OP_AND && op < PPI_OP_COUNT ? kernel_of<PPI_OP_AND>(op) : nullptr);
   if (!kern || iters < 1 || reps < 1 || !ms || !ops) return (int)cudaErrorInvalidValue;
   int dev = 0, sms = 0, per_sm = 0;
   cudaError_t e = cudaGetDevice(&dev);
   if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
   if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 256, 0);
   if (e != cudaSuccess) return (int)e;
   const int blocks = sms * (per_sm > 0 ? per_sm : 1);
   float* out = nullptr;
   cudaEvent_t a = nullptr, b = nullptr;
   e = cudaMalloc(&out, (size_t)blocks * 256 * sizeof(float));
   if (e == cudaSuccess) e = cudaEventCreate(&a);
   if (e == cudaSuccess) e = cudaEventCreate(&b);
   float best = -1.0f;
   for (int rep = 0; e == cudaSuccess && rep <= reps; ++rep) {
      cudaEventRecord(a);
      kern<<<blocks, 256>>>(out, iters, lo, hi, k, prot);
      cudaEventRecord(b);
      e = cudaEventSynchronize(b);
      float t = 0.0f;
      if (e == cudaSuccess) e = cudaEventElapsedTime(&t, a, b);
      if (rep > 0 && (best < 0.0f || t < best)) best = t;   // rep 0 warms up
   }
   if (a) cudaEventDestroy(a);
   if (b) cudaEventDestroy(b);
   cudaFree(out);
   if (e != cudaSuccess) return (int)e;
   *ms = best;
   *ops = (double)blocks * 256.0 * kVals * (double)iters;
   return 0;
}

}  // extern "C"
