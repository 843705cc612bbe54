// Kernels for N = 2 (N+1 = 3 nodes per direction).
#define GX_NP 3
#include "dg_np.cuh"
