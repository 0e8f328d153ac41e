// FP64 kernels compiled without FMA contraction (-fmad=false): each a*b+c
// rounds twice, as the reference CPU code does.
#define SGB_NS sgb_fp64_exact
#define SGB_REAL double
#define SGB_TABLE ops_fp64_exact
#define SGB_VARIANT_NAME "fp64"
#define SGB_USES_PATCHES 0
#include "variant_def.cuh"
