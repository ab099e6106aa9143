// accelerator_cuda.cc -- PPI's interpreter interface implemented on the GB300
// evaluator.  Drop-in replacement for src/interpreter/accelerator.cc: the
// same three functions with the same signatures (accelerator.h:29, 36-40, 48),
// called unchanged by src/ppi.cc:361, 606-610, 838 and src/ppp.cc:87,
// 105-129.  Built against PPI's generated headers (<symbol>, <definitions.h>,
// <costmatrix>) and the grammar's Symbol -> op table <ppi_symbol_map>
// (python3 -m ppi_gpu.codegen --map-only).
//
// What maps where:
//   ERROR(X,Y), REDUCEMAX, PROTECTED, NATIVE, COST (definitions.h,
//     costmatrix)          -> ppi_gpu_config error_fn / reduce_max /
//                             protected_fns / math / cost
//   -strategy PP|DP|PDP    -> ppi_gpu_config.strategy (default PDP,
//                             accelerator.cc:571)
//   -cl-mls N              -> lanes (work-items per program / records per group)
//   -cl-d N                -> CUDA device N; -cl-p, -type and -transpose are
//                             accepted and have no effect (one platform, the
//                             device layout is always column-major)
//   -v                     -> device and geometry lines on stdout
// Math mode: NATIVE builds use the hardware approximations; otherwise the
// CUDA single-precision functions, or the double-precision path that matches
// src/interpreter/sequential.cc bit for bit when PPI_GPU_MATH=parity.
#include "accelerator.h"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <queue>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "ppi_gpu.h"
#include <ppi_symbol_map>

namespace {

// COST is defined by <costmatrix> inside a function when the build has one;
// this namespace-scope object stands in when it has not.
struct ppi_no_cost {};
[[maybe_unused]] ppi_no_cost COST;

template <size_t N, size_t M>
void cost_table(const float (&c)[N][M], std::vector<float>& out, int& n) {
   n = (int)N;
   out.assign(&c[0][0], &c[0][0] + N * M);
}
inline void cost_table(const ppi_no_cost&, std::vector<float>& out, int& n) {
   out.clear();
   n = 0;
}

#define PPI_ADAPTER_STR2(...) #__VA_ARGS__
#define PPI_ADAPTER_STR(...) PPI_ADAPTER_STR2(__VA_ARGS__)

// The build's ERROR(X,Y) as one of the evaluator's error functions.
int error_function(bool have_cost) {
   std::string ef = PPI_ADAPTER_STR(ERROR(X, Y));
   std::string s;
   for (char ch : ef)
      if (ch != ' ' && ch != '\t') s += ch;
   if (s == "fabs((X)-(Y))") return PPI_EF_ABS;
   if (s == "(((X)-(Y))*((X)-(Y)))") return PPI_EF_SQUARED;
   if (s == "((X)!=(Y))") return PPI_EF_MISCLASS;
   if (have_cost && (s == "COST[(int)X][(int)Y]" || s.find("COST,X,Y") != std::string::npos))
      return PPI_EF_COST;
   return -1;
}

struct State {
   ppi_gpu* h = nullptr;
   bool verbose = false;
   int nlin = 0;
   double time_gen_kernel = 0.0, time_total_kernel = 0.0, gpops_gen = 0.0;
} data;

struct Options {
   std::string strategy = "PDP";
   std::string dataset;      // -d / --dataset: the CSV main.cc read (src/main.cc:141,152)
   int lanes = -1, device = 0;
   bool verbose = false, ok = true;
};

// Flags of acc_interpret_init (accelerator.cc:565-571): "-flag value" or
// "--long-name value"; unknown flags are ignored and "--" ends the scan, as
// PPI's CmdLine::Parser does.
Options parse(int argc, char** argv) {
   Options o;
   for (int i = 1; i < argc; ++i) {
      const std::string a = argv[i];
      if (a == "--") break;
      const bool has_value = i + 1 < argc;
      if (a == "-v" || a == "--verbose") {
         o.verbose = true;
      } else if ((a == "-strategy") && has_value) {
         std::string v = argv[++i];
         if (v == "pp" || v == "PP") o.strategy = "PP";
         else if (v == "dp" || v == "DP") o.strategy = "DP";
         else if (v == "pdp" || v == "PDP") o.strategy = "PDP";
         else { std::fprintf(stderr, "Valid strategy: PP, DP and PDP.\n"); o.ok = false; }
      } else if ((a == "-cl-mls" || a == "--cl-max-local-size") && has_value) {
         o.lanes = std::atoi(argv[++i]);
      } else if ((a == "-d" || a == "--dataset") && has_value) {
         o.dataset = argv[++i];
      } else if ((a == "-cl-d" || a == "--cl-device-id") && has_value) {
         o.device = std::max(0, std::atoi(argv[++i]));
      } else if ((a == "-type") && has_value) {
         std::string v = argv[++i];
         if (v == "CPU" || v == "cpu") {
            std::fprintf(stderr, "Not a single compatible type found.\n");
            o.ok = false;
         }
      } else if ((a == "-cl-p" || a == "--cl-platform-id") && has_value) {
         ++i;
      }
   }
   return o;
}

void check(ppi_status s, const char* what) {
   if (s != PPI_OK) {
      std::string msg = std::string(what) + ": " + (data.h ? ppi_gpu_last_error(data.h) : "") +
                        " (status " + std::to_string((int)s) + ")";
      std::fprintf(stderr, "\nERROR(kernel1): %s\n", msg.c_str());
      throw std::runtime_error(msg);
   }
}

// util::PickNBest (src/util/Util.h:158-173) for best_size > 1.
void pick_n_best(int n, int* best, int num, const float* err) {
   std::priority_queue<std::pair<float, int>> q;
   for (int i = 0; i < num; ++i) q.push(std::pair<float, int>(err[i] * (-1.0f), i));
   for (int i = 0; i < n && !q.empty(); ++i) {
      best[i] = q.top().second;
      q.pop();
   }
}

}  // namespace

int acc_interpret_init(int argc, char** argv, const unsigned size, const unsigned max_arity,
                       const unsigned population_size, float** input, int nlin, int ncol,
                       int ppp_mode, int prediction_mode) {
   (void)max_arity;   // only sized the OpenCL private stack
   Options o = parse(argc, argv);
   if (!o.ok) return 1;
   if (ncol < 0) {
      std::fprintf(stderr, "Missing number of columns of dataset.\n");
      return 1;
   }
   std::vector<float> cost;
   int cost_n = 0;
   {
#include <costmatrix>
      cost_table(COST, cost, cost_n);
   }
   ppi_gpu_config c;
   std::memset(&c, 0, sizeof c);
   c.max_size = (int32_t)size;
   c.population_size = ppp_mode ? 1 : (int32_t)population_size;
   c.strategy = o.strategy == "PP" ? PPI_STRATEGY_PP : o.strategy == "DP" ? PPI_STRATEGY_DP : PPI_STRATEGY_PDP;
   c.lanes = o.lanes;
   c.error_fn = error_function(cost_n > 0);
   if (c.error_fn < 0) {
      std::fprintf(stderr, "Unsupported error function %s.\n", PPI_ADAPTER_STR(ERROR(X, Y)));
      return 1;
   }
#ifdef REDUCEMAX
   c.reduce_max = 1;
#endif
#ifdef PROTECTED
   c.protected_fns = 1;
#endif
#ifdef NATIVE
   c.math = PPI_MATH_NATIVE;
#else
   {
      const char* m = std::getenv("PPI_GPU_MATH");
      c.math = (m && std::strcmp(m, "parity") == 0) ? PPI_MATH_PARITY : PPI_MATH_FAST;
   }
#endif
   c.cost = cost_n ? cost.data() : nullptr;
   c.cost_n = cost_n;
   c.symbols = ppi_symbol_map;
   c.n_symbols = (int32_t)(sizeof(ppi_symbol_map) / sizeof(ppi_symbol_map[0]));
   c.device = o.device;
   if (data.h) {
      ppi_gpu_destroy(data.h);
      data.h = nullptr;
   }
   ppi_status s = ppi_gpu_create(&c, &data.h);
   if (s != PPI_OK) {
      std::fprintf(stderr, "Error in CUDA initialization phase (status %d).\n", (int)s);
      return 1;
   }
   // The dataset: straight from the CSV file main.cc read (the same reader
   // rules, columns written in the device layout) when the command line names
   // it and it gives main.cc's shape; else from main.cc's float** rows.
   bool from_file = false;
   if (!o.dataset.empty()) {
      int32_t rows = 0, cols = 0;
      from_file = ppi_gpu_set_dataset_csv(data.h, o.dataset.c_str(), &rows, &cols) == PPI_OK &&
                  rows == nlin && cols == ncol;
   }
   if (!from_file) {
      s = ppi_gpu_set_dataset(data.h, input, nlin, ncol);
      if (s != PPI_OK) {
         std::fprintf(stderr, "Error in build the kernel: %s\n", ppi_gpu_last_error(data.h));
         return 1;
      }
   }
   data.nlin = nlin;
   data.verbose = o.verbose;
   if (o.verbose)
      std::printf("\nDevice: CUDA %d (%s), strategy %s, work-items per program/group: %d, dataset %s\n",
                  o.device, ppi_gpu_version(), o.strategy.c_str(), (int)ppi_gpu_lanes(data.h),
                  from_file ? "read from the CSV file" : "from the host rows");
   (void)prediction_mode;
   return 0;
}

void acc_interpret(Symbol* phenotype, float* ephemeral, int* size,
#ifdef PROFILING
                   unsigned long sum_size_gen,
#endif
                   float* vector, int nInd, void (*send)(Population*),
                   int (*receive)(GENOME_TYPE**), Population* migrants, int* nImmigrants,
                   int* index, int* best_size, int ppp_mode, int prediction_mode, float alpha) {
   if (!data.h) throw std::runtime_error("acc_interpret called before acc_interpret_init");
   const int32_t* ph = reinterpret_cast<const int32_t*>(phenotype);
   if (ppp_mode && prediction_mode) {
      check(ppi_gpu_predict(data.h, ph, ephemeral, size[0], vector), "ppi_gpu_predict");
   } else if (ppp_mode) {
      check(ppi_gpu_evaluate(data.h, ph, ephemeral, size, 1, alpha, vector, nullptr), "ppi_gpu_evaluate");
   } else {
      int32_t best = 0;
      check(ppi_gpu_evaluate_launch(data.h, ph, ephemeral, size, nInd, alpha, vector, &best),
            "ppi_gpu_evaluate_launch");
      // island exchange overlaps the kernels (accelerator.cc:736-743)
      send(migrants);
      *nImmigrants = receive(migrants->genome);
      check(ppi_gpu_evaluate_wait(data.h), "ppi_gpu_evaluate_wait");
      if (*best_size <= 1) {
         index[0] = best;
      } else {
         if (*best_size > nInd) *best_size = nInd;
         pick_n_best(*best_size, index, nInd, vector);
      }
   }
   float ms = 0.0f;
   ppi_gpu_last_kernel_ms(data.h, &ms);
   data.time_gen_kernel = ms / 1e3;
   data.time_total_kernel += ms / 1e3;
#ifdef PROFILING
   data.gpops_gen = data.time_gen_kernel > 0 ? (sum_size_gen * (double)data.nlin) / data.time_gen_kernel : 0.0;
#endif
}

#ifdef PROFILING
void acc_print_time(bool total, unsigned long long sum_size) {
   const double t = total ? data.time_total_kernel : data.time_gen_kernel;
   const double gpops = total ? (t > 0 ? (sum_size * (double)data.nlin) / t : 0.0) : data.gpops_gen;
   std::printf(", time_kernel[1]: %lf, time_kernel[2]: %lf", t, 0.0);
   std::printf("; gpops_kernel: %lf", gpops);
}
#endif
