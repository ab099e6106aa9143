/* The interpreter interface PPI's ppi.cc and ppp.cc call (the declarations of
 * PPI's src/interpreter/accelerator.h), for building the adapter outside PPI's
 * tree.  Inside PPI's tree the adapter includes PPI's own accelerator.h. */
#ifndef accelerator_h
#define accelerator_h

#include <definitions.h>
#include <symbol>
#include "individual"

int acc_interpret_init(int argc, char** argv, const unsigned size, const unsigned max_arity,
                       const unsigned population_size, float** input, int nlin, int ncol,
                       int ppp_mode, int prediction_mode);

void acc_interpret(Symbol* phenotype, float* ephemeral, int* size,
#ifdef PROFILING
                   unsigned long sum_size_gen,
#endif
                   float* vector, int nInd, void (*send)(Population*),
                   int (*receive)(GENOME_TYPE**), Population* migrants, int* nImmigrants,
                   int* index, int* best_size, int ppp_mode, int prediction_mode, float alpha);

#ifdef PROFILING
void acc_print_time(bool total, unsigned long long sum_size);
#endif

#endif
