// ppi_decode.cuh -- device genome decoder (src/ppi.cc:106-182).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace ppi {

// Grammar tables on the device: alternative a = rule_first[nt] + k is
// gramatica[nt][k] (the generated `grammar` header), alt_len[a] symbols at
// alt_syms[a * max_rule ...].
struct DecodeTables {
   int32_t* rule_first = nullptr;
   int32_t* rule_count = nullptr;
   int32_t* alt_len = nullptr;
   int32_t* alt_syms = nullptr;
   int n_nt = 0, n_alt = 0, max_rule = 0, t_const = -1, t_attribute = -1;
   bool ready = false;
};

struct DecodeArgs {
   DecodeTables t;
   const uint8_t* genomes;   // n x nb bytes, one 0/1 byte per bit
   int n, nb, bg, bc;
   float lo, hi;
   int max_size;
   int32_t* phenotype;       // n x max_size
   float* ephemeral;
   int32_t* size;
   uint32_t* frames;         // n x frames_cap scratch
   int frames_cap;
};

cudaError_t upload_decode_tables(DecodeTables* t, const int32_t* rule_first, const int32_t* rule_count,
                                 int n_nt, const int32_t* alt_len, const int32_t* alt_syms, int n_alt,
                                 int max_rule, int t_const, int t_attribute);
void free_decode_tables(DecodeTables* t);
cudaError_t launch_decode(const DecodeArgs& a, cudaStream_t s);

}  // namespace ppi
