// Kernels for N = 3 (N+1 = 4 nodes per direction).
#define GX_NP 4
#include "dg_np.cuh"
