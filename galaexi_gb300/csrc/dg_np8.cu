// Kernels for N = 7 (N+1 = 8 nodes per direction).
#define GX_NP 8
#include "dg_np.cuh"
