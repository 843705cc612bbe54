// Kernels for N = 1 (N+1 = 2 nodes per direction).
#define GX_NP 2
#include "dg_np.cuh"
