/*
 * transport_fast_mcvox_static.cu - Voxelized-medium transport kernels, static scheduling, in
 * FAST math: special-function- unit log2/sin/cos/ex2 and approximate division and square root
 * (built with -use_fast_math); the reference's MC_USE_NATIVE_MATH.
 */
#define MCGB_FAST_MATH 1
#define MCGB_NS mcgb_fast
#define MCGB_MEDIUM 1
#define MCGB_PART 0
#include "transport_tu.cuh"
