// Kernels for N = 6 (N+1 = 7 nodes per direction).
#define GX_NP 7
#include "dg_np.cuh"
