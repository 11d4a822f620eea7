/*
 * ref_stubs.c -- TEST INFRASTRUCTURE.  Linked only into oracle/_ref, the
 * reference's own C sources compiled from the read-only reference tree.
 *
 * Those C files also reference 2-D Fortran kernels and the unused "Medium"
 * 3-D reinitialisation kernel, none of which has a C restatement (the 3-D
 * quasi-static path never calls them).  These definitions only satisfy the
 * linker; reaching one of them means a test drove a path outside the oracle.
 */
#include <stdio.h>
#include <stdlib.h>

#define REF_STUB(name)                                                        \
  void name(void)                                                             \
  {                                                                           \
    fprintf(stderr, "oracle/_ref: %s is outside the restated 3-D path\n", #name); \
    abort();                                                                  \
  }

REF_STUB(computereinitializationeqnrhs2d_)
REF_STUB(computereinitializationeqnrhs3d_)
REF_STUB(qss2dcomputedistanceforsubcellfix_)
REF_STUB(qss2dcomputereinitializationeqnrhssubcellfixorder1_)
REF_STUB(qss2dgetrhs2nd_)
REF_STUB(qss2dgetrhs2ndconst_)
REF_STUB(qss2dgetrhs3rd_)
REF_STUB(qss2dgetrhs3rdconst_)
REF_STUB(qss2drk1step_)
REF_STUB(qss2dsignedlinearextrapolation_)
REF_STUB(qss2dtvdrk2stage2_)

/* thread count of the reference's OpenMP z-slab decomposition, for tests */
#include <omp.h>
void oracle_set_threads(int t) { omp_set_num_threads(t); }
