// Mixed precision: FP32 element math and solver vectors, FP64 state and dots.
#define SGB_NS sgb_mixed
#define SGB_REAL float
#define SGB_TABLE ops_mixed
#define SGB_VARIANT_NAME "mixed"
#define SGB_USES_PATCHES 1
#include "variant_def.cuh"
