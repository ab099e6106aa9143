// ref_cl_driver.cc -- runs the reference's OpenCL kernels
// (src/interpreter/accelerator.cl: evaluate_pp :8-86, evaluate_dp :89-171,
// evaluate_pdp :174-268, best_individual :271-313) on the CPU through
// cl_shim.h.  Launch geometry and the host-side steps around each kernel
// follow src/interpreter/accelerator.cc (build_kernel :296-330, the DP host
// reduction :777-802, the alpha add :848-849, PickNBest :874-880).
//
// TEST INFRASTRUCTURE ONLY.  Built by oracle/build_ref.py into oracle/_ref/;
// never linked into the product.
#include "cl_shim.h"

#include <vector>
#include <thread>
#include <limits>
#include <queue>
#include <utility>

thread_local ppi_cl_item ppi_cl_cur;

#include ACCEL_CL_PATH

namespace {

// Runs `fn` once per work-item of `groups` work-groups of `local` items.
// Work-groups run one after the other; the items of a group run as threads
// so that barrier() works.
template <class F>
void run_ndrange(int groups, int local, bool needs_barrier, F fn) {
   for (int g = 0; g < groups; ++g) {
      if (!needs_barrier) {
         for (int l = 0; l < local; ++l) {
            ppi_cl_cur = ppi_cl_item{g * local + l, l, g, local, groups, nullptr};
            fn();
         }
         continue;
      }
      std::barrier<> bar(local);
      std::vector<std::thread> th;
      th.reserve(local);
      for (int l = 0; l < local; ++l) {
         th.emplace_back([&, l]() {
            ppi_cl_cur = ppi_cl_item{g * local + l, l, g, local, groups, &bar};
            fn();
         });
      }
      for (auto& t : th) t.join();
   }
}

// util::PickNBest (src/util/Util.h:158-173), restated for the shim driver.
void pick_n_best(int n, int* best, int num, const float* err, const int* idx) {
   std::priority_queue<std::pair<float, int>> q;
   for (int i = 0; i < num; ++i) q.push(std::pair<float, int>(err[i] * (-1.0f), i));
   for (int i = 0; i < n; ++i) {
      best[i] = idx ? idx[q.top().second] : q.top().second;
      q.pop();
   }
}

void run_best(const float* vec, int pop, int local2, int* best_index) {
   int groups = (pop + local2 - 1) / local2;
   std::vector<float> pb(groups);
   std::vector<int> pi(groups);
   std::vector<float> lb(local2);
   std::vector<int> li(local2, 0);
   run_ndrange(groups, local2, true, [&]() {
      best_individual(vec, pb.data(), pi.data(), lb.data(), li.data(), pop);
   });
   pick_n_best(1, best_index, groups, pb.data(), pi.data());
}

}  // namespace

extern "C" {

int ref_cl_max_phenotype_size() { return MAX_PHENOTYPE_SIZE; }

// strategy: 0 = PP, 1 = DP, 2 = PDP.  inputs: row-major nlin x ncol.
// local1 / local2: work-group sizes of the evaluate and best kernels.
// Writes nInd fitness values (alpha added as the host does) or nlin
// predictions, and the best index when best_index != NULL.
int ref_cl_evaluate(int strategy, const int* phenotype, const float* ephemeral,
                    const int* size, const float* inputs, int nlin, int ncol,
                    int nInd, int prediction_mode, int local1, int local2,
                    float alpha, float* out, int* best_index) {
   const Symbol* ph = reinterpret_cast<const Symbol*>(phenotype);
   if (strategy == 0) {
      std::vector<float> vec(prediction_mode ? nlin : nInd);
      int groups = (nInd + local1 - 1) / local1;
      run_ndrange(groups, local1, false, [&]() {
         evaluate_pp(ph, ephemeral, size, inputs, vec.data(), nlin, ncol, prediction_mode, nInd);
      });
      if (prediction_mode) {
         for (int i = 0; i < nlin; ++i) out[i] = vec[i];
         return 0;
      }
      if (best_index) run_best(vec.data(), nInd, local2, best_index);
      for (int i = 0; i < nInd; ++i) out[i] = vec[i] + alpha * size[i];
      return 0;
   }
   if (strategy == 2) {
      std::vector<float> vec(prediction_mode ? nlin : nInd);
      std::vector<float> pe(local1);
      run_ndrange(nInd, local1, true, [&]() {
         evaluate_pdp(ph, ephemeral, size, inputs, vec.data(), nlin, ncol, prediction_mode, pe.data());
      });
      if (prediction_mode) {
         for (int i = 0; i < nlin; ++i) out[i] = vec[i];
         return 0;
      }
      if (best_index) run_best(vec.data(), nInd, local2, best_index);
      for (int i = 0; i < nInd; ++i) out[i] = vec[i] + alpha * size[i];
      return 0;
   }
   if (strategy == 1) {
      int groups = (nlin + local1 - 1) / local1;
      std::vector<float> vec(prediction_mode ? (size_t)groups * local1 : (size_t)groups * nInd);
      std::vector<float> pe(local1);
      run_ndrange(groups, local1, true, [&]() {
         evaluate_dp(ph, ephemeral, size, inputs, vec.data(), nlin, ncol, prediction_mode, pe.data(), nInd);
      });
      if (prediction_mode) {
         for (int i = 0; i < nlin; ++i) out[i] = vec[i];
         return 0;
      }
      // Host reduction of the per-group partials (accelerator.cc:780-802).
      for (int i = 0; i < nInd; ++i) {
         float sum = 0.0f;
         for (int g = 0; g < groups; ++g) {
            float error = vec[(size_t)i * groups + g];
            if (std::isinf(error) || std::isnan(error)) { sum = std::numeric_limits<float>::max(); break; }
#ifdef REDUCEMAX
            sum = (error * nlin > sum) ? error * nlin : sum;
#else
            sum += error;
#endif
         }
         if (std::isnan(sum) || std::isinf(sum))
            out[i] = std::numeric_limits<float>::max();
         else
            out[i] = sum / nlin + alpha * size[i];
      }
      if (best_index) run_best(out, nInd, local2, best_index);
      return 0;
   }
   return 1;
}

}  // extern "C"
