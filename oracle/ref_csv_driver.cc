// ref_csv_driver.cc -- harness around the reference's CSV dataset reader.
// build_ref.py extracts read() (src/main.cc:32-119) verbatim from the
// reference source into oracle/_ref/csv_extract.inc; it calls
// util::StringTo from src/util/Util.h.  This file exports a C entry point
// that returns the reader's status, shape and values.
//
// TEST INFRASTRUCTURE ONLY.  Never linked into the product.
#include <cmath>
#include <cstdio>
#include <fstream>
#include <sstream>
#include <string>

#include "Util.h"

#include "csv_extract.inc"

extern "C" int ref_csv_read(const char* path, float* rowmajor, long capacity, int* nlin, int* ncol) {
   float** input = nullptr;
   int nc = 0, nl = 0;
   const int rc = read(path, input, nc, nl);
   *nlin = nl;
   *ncol = nc;
   if (rc == 0 && rowmajor && (long)nl * nc <= capacity)
      for (int i = 0; i < nl; ++i)
         for (int j = 0; j < nc; ++j) rowmajor[(long)i * nc + j] = input[i][j];
   if (input) {
      for (int i = 0; i < nl; ++i) delete[] input[i];
      delete[] input;
   }
   std::fflush(stderr);
   return rc;
}
