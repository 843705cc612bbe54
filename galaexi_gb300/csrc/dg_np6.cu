// Kernels for N = 5 (N+1 = 6 nodes per direction).
#define GX_NP 6
#include "dg_np.cuh"
