// ref_decode_driver.cc -- harness around the reference's genome decoder.
// build_ref.py extracts decode_rule / decode_real / decode
// (src/ppi.cc:106-182) verbatim from the reference source into
// oracle/_ref/<config>/decode_extract.inc; this file supplies the few
// globals those functions read (the `data` fields that ppi_init fills at
// src/ppi.cc:260-307 and the generated grammar tables) and exports a C entry
// point.
//
// TEST INFRASTRUCTURE ONLY.  Never linked into the product.
#include <cstddef>
#include <symbol>

typedef bool GENOME_TYPE;          // src/individual:11

#include <grammar>

namespace {
struct {
   int number_of_bits;
   int bits_per_gene;
   int bits_per_constant;
   float interval[2];
   unsigned max_size_phenotype;
} data;
}  // namespace

#include "decode_extract.inc"

extern "C" {

int ref_max_quant_simbolos_por_regra() { return MAX_QUANT_SIMBOLOS_POR_REGRA; }
int ref_num_rules() { return (int)(sizeof(gramatica) / sizeof(t_rule**)); }
int ref_rule_count(int nt) { return (int)tamanhos[nt]; }

// genomes: n x nb bytes (0/1); rows of `stride` entries in phenotype and
// ephemeral (stride >= mps; the reference can write past mps, see
// src/ppi.cc:148-174, so callers pass slack); allele_out receives the number
// of bits consumed.
void ref_decode(const unsigned char* genomes, int n, int nb, int bg, int bc,
                float lo, float hi, unsigned mps, int stride,
                int* phenotype, float* ephemeral, int* size, int* allele_out) {
   data.number_of_bits = nb;
   data.bits_per_gene = bg;
   data.bits_per_constant = bc;
   data.interval[0] = lo;
   data.interval[1] = hi;
   data.max_size_phenotype = mps;
   for (int i = 0; i < n; ++i) {
      int allele = 0;
      size[i] = decode(reinterpret_cast<const GENOME_TYPE*>(genomes + (size_t)i * nb), &allele,
                       reinterpret_cast<Symbol*>(phenotype + (size_t)i * stride),
                       ephemeral + (size_t)i * stride, 0, NT_INICIAL);
      if (allele_out) allele_out[i] = allele;
   }
}

}  // extern "C"
