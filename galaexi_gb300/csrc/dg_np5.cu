// Kernels for N = 4 (N+1 = 5 nodes per direction).
#define GX_NP 5
#include "dg_np.cuh"
