/*
 * transport_exact_mcml_dynamic.cu - Layered-medium transport kernels, dynamic scheduling and
 * the launcher, in EXACT math: IEEE arithmetic without FMA contraction (built with
 * -fmad=false) and the portable log/exp/sincos/powr routines; bit-identical to a CPU
 * evaluation of the same algorithm.
 */
#define MCGB_FAST_MATH 0
#define MCGB_NS mcgb_exact
#define MCGB_MEDIUM 0
#define MCGB_PART 1
#include "transport_tu.cuh"
