// FP64 kernels with FMA contraction.
#define SGB_NS sgb_fp64_fast
#define SGB_REAL double
#define SGB_TABLE ops_fp64_fast
#define SGB_VARIANT_NAME "fp64_fma"
#define SGB_USES_PATCHES 1
#include "variant_def.cuh"
