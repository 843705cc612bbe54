// Kernels for N = 9 (N+1 = 10 nodes per direction).
#define GX_NP 10
#include "dg_np.cuh"
