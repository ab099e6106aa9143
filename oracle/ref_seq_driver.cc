// ref_seq_driver.cc -- C entry points around the reference's sequential
// interpreter (src/interpreter/sequential.cc: seq_interpret_init :82-115,
// seq_interpret :117-209, seq_interpret_destroy :211-216) so that Python
// tests can call it through ctypes.
//
// TEST INFRASTRUCTURE ONLY.  Built by oracle/build_ref.py into oracle/_ref/
// together with the reference's sequential.cc; never linked into the product.
#include <vector>
#include "sequential.h"

extern "C" {

// rows: row-major nlin x ncol (the last column is the target, as in the
// reference's dataset reader).
void ref_seq_init(unsigned max_size, const float* rows, int nlin, int ncol) {
   std::vector<float*> ptr(nlin);
   for (int i = 0; i < nlin; ++i) ptr[i] = const_cast<float*>(rows + (size_t)i * ncol);
   seq_interpret_init(max_size, ptr.data(), nlin, ncol);
}

void ref_seq_interpret(const int* phenotype, const float* ephemeral, const int* size,
                       float* vector, int nInd, int* index, int best_size,
                       int ppp_mode, int prediction_mode, float alpha) {
   int bs = best_size;
   seq_interpret(reinterpret_cast<Symbol*>(const_cast<int*>(phenotype)),
                 const_cast<float*>(ephemeral), const_cast<int*>(size), vector, nInd,
                 index, &bs, ppp_mode, prediction_mode, alpha);
}

void ref_seq_destroy() { seq_interpret_destroy(); }

}  // extern "C"
