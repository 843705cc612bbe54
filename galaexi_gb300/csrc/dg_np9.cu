// Kernels for N = 8 (N+1 = 9 nodes per direction).
#define GX_NP 9
#include "dg_np.cuh"
