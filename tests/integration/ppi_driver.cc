// ppi_driver.cc -- calls the interpreter interface the way PPI does, for the
// adapter's integration tests: acc_interpret_init once, then
//   mode 0 (evolution, src/ppi.cc:361, 606-610): one acc_interpret per
//          generation with send/receive island callbacks and best index;
//   mode 1 (ppp test, src/ppp.cc:87, 125-129): one program, its error;
//   mode 2 (ppp prediction, src/ppp.cc:87, 105-109): one program, one value
//          per record.
// Input file: int32 header {mode, nlin, ncol, n, max_size, generations},
// float alpha, nlin*ncol floats (row-major), then per generation phenotype
// (n*max_size int32), ephemeral (n*max_size float), size (n int32).
// Output file: per generation the n (or nlin) result floats, the best index
// and the order in which the callbacks ran.  Remaining argv: PPI's flags.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "accelerator.h"

static int g_events = 0, g_send_at = -1, g_recv_at = -1;
static void on_send(Population*) { g_send_at = g_events++; }
static int on_receive(GENOME_TYPE**) { g_recv_at = g_events++; return 0; }

int main(int argc, char** argv) {
   if (argc < 3) { std::fprintf(stderr, "usage: %s in out [flags]\n", argv[0]); return 2; }
   FILE* in = std::fopen(argv[1], "rb");
   FILE* out = std::fopen(argv[2], "wb");
   if (!in || !out) return 2;
   int hdr[6];
   float alpha;
   if (std::fread(hdr, 4, 6, in) != 6 || std::fread(&alpha, 4, 1, in) != 1) return 2;
   const int mode = hdr[0], nlin = hdr[1], ncol = hdr[2], n = hdr[3], mps = hdr[4], gens = hdr[5];
   std::vector<float> rows((size_t)nlin * ncol);
   if (std::fread(rows.data(), 4, rows.size(), in) != rows.size()) return 2;
   std::vector<float*> input(nlin);
   for (int i = 0; i < nlin; ++i) input[i] = rows.data() + (size_t)i * ncol;
   // argv for acc_interpret_init: program name + flags after the two files
   std::vector<char*> av;
   av.push_back(argv[0]);
   for (int i = 3; i < argc; ++i) av.push_back(argv[i]);
   const int ppp = mode != 0, pred = mode == 2;
   if (acc_interpret_init((int)av.size(), av.data(), (unsigned)mps, ppp ? (unsigned)-1 : 2u,
                          (unsigned)n, input.data(), nlin, ncol, ppp, pred)) {
      std::fprintf(stderr, "Error in initialization phase.\n");
      return 3;
   }
   std::vector<Symbol> ph((size_t)n * mps);
   std::vector<float> eph((size_t)n * mps), result(pred ? nlin : n);
   std::vector<int> size(n);
   GENOME_TYPE allele[16] = {};
   GENOME_TYPE* genomes[1] = {allele};
   float fit[1];
   Population migrants{genomes, fit};
   for (int g = 0; g < gens; ++g) {
      if (std::fread(ph.data(), 4, ph.size(), in) != ph.size() ||
          std::fread(eph.data(), 4, eph.size(), in) != eph.size() ||
          std::fread(size.data(), 4, size.size(), in) != size.size())
         return 2;
      int index[1] = {-1}, best_size = 1, nimm = -1;
      g_events = 0; g_send_at = g_recv_at = -1;
      unsigned long sum = 0;
      for (int i = 0; i < n; ++i) sum += (unsigned long)size[i];
      if (mode == 0)
         acc_interpret(ph.data(), eph.data(), size.data(),
#ifdef PROFILING
                       sum,
#endif
                       result.data(), n, &on_send, &on_receive, &migrants, &nimm, index, &best_size,
                       0, 0, alpha);
      else
         acc_interpret(ph.data(), eph.data(), size.data(),
#ifdef PROFILING
                       0,
#endif
                       result.data(), 1, NULL, NULL, NULL, NULL, NULL, NULL, 1, pred, 0.0f);
      (void)sum;
      std::fwrite(result.data(), 4, result.size(), out);
      int tail[4] = {index[0], g_send_at, g_recv_at, nimm};
      std::fwrite(tail, 4, 4, out);
   }
#ifdef PROFILING
   acc_print_time(true, 1);
   std::printf("\n");
#endif
   std::fclose(out);
   return 0;
}
