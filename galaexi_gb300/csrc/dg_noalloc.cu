// Allocation-free variant of the CFL/DFL time-step reduction (dg_calc_timestep_noalloc).
//
// Its scratch -- one (convective, viscous) eigenvalue pair per element, the two reduced time
// steps and a bad-node counter -- lives in a file-scope static device array instead of memory the
// library allocates.  The array is part of the loaded module, so every GPU that loads the library
// keeps it (DG_NOALLOC_MAX_ELEMS * 16 bytes + 256 bytes) until the process exits.
#include <cuda_runtime.h>
#include <cmath>
#include <cstring>
#include <string>

#include "../../include/galaexi_gb300.h"
#include "dg_host.h"

using gxh::set_error;

namespace {

constexpr int kTail = 32;  // doubles after the per-element pairs: [0] dt_conv, [1] dt_visc, [2] bad counter
static __device__ __align__(256) double g_noalloc_scratch[2 * (size_t)DG_NOALLOC_MAX_ELEMS + kTail];

// Device address of g_noalloc_scratch in the current device's context.  The host-side name of the
// array is not a device address; the address is looked up on every call (a host-side table lookup),
// so that a context torn down and created again (cudaDeviceReset) never leaves a stale address.
int scratch_ptr(double** out) {
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess || !p) {
    set_error(std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    return DG_ERR_CUDA;
  }
  *out = static_cast<double*>(p);
  return DG_OK;
}

// pass 1: per-element maximum eigenvalues (CalcMaxEigenvalue, calctimestep.f90:192-296), reading the
// reference layouts U(5,n,n,n,e), Metrics_*Tilde(3,n,n,n,e), sJ(n,n,n,e)
__global__ void __launch_bounds__(1024)
k_cfl_elem(const double* __restrict__ U, const double* __restrict__ Mf, const double* __restrict__ Mg,
           const double* __restrict__ Mh, const double* __restrict__ sJ, int n3, double kappa, double mu0,
           int parabolic, double KappasPr_max, double* __restrict__ scratch) {
  __shared__ double red[6][32];
  const int e = blockIdx.x, node = threadIdx.x;
  double lam[6] = {0, 0, 0, 0, 0, 0};
  unsigned long long* bad = reinterpret_cast<unsigned long long*>(scratch + 2 * (size_t)DG_NOALLOC_MAX_ELEMS + 2);
  if (node < n3) {
    const size_t g = (size_t)e * n3 + node;
    const double* u = U + 5 * g;
    const double srho = 1. / u[0];
    const double vel[3] = {u[1] * srho, u[2] * srho, u[3] * srho};
    const double p = (kappa - 1.) * (u[4] - 0.5 * (vel[0] * u[1] + vel[1] * u[2] + vel[2] * u[3]));
    if (!(u[0] > 0.) || !(p > 0.) || !isfinite(u[4]) || !isfinite(u[1] + u[2] + u[3])) atomicAdd(bad, 1ULL);
    const double c = sqrt(kappa * p * srho);
    const double sj = sJ[g];
    const double vs[3] = {vel[0] * sj, vel[1] * sj, vel[2] * sj};
    const double* Ms[3] = {Mf + 3 * g, Mg + 3 * g, Mh + 3 * g};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const double m0 = Ms[d][0], m1 = Ms[d][1], m2 = Ms[d][2];
      const double adv = sj * sqrt(m0 * m0 + m1 * m1 + m2 * m2);
      lam[d] = fabs(m0 * vs[0] + m1 * vs[1] + m2 * vs[2]) + c * adv;
      if (parabolic) {
        const double vis = KappasPr_max * ((m0 * sj) * (m0 * sj) + (m1 * sj) * (m1 * sj) + (m2 * sj) * (m2 * sj));
        lam[3 + d] = mu0 * srho * vis;
      }
    }
  }
#pragma unroll
  for (int d = 0; d < 6; ++d) {
    double v = lam[d];
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    if ((threadIdx.x & 31) == 0) red[d][threadIdx.x >> 5] = v;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const int nw = (blockDim.x + 31) / 32;
    double mx[6];
    for (int d = 0; d < 6; ++d) {
      mx[d] = red[d][0];
      for (int w = 1; w < nw; ++w) mx[d] = fmax(mx[d], red[d][w]);
    }
    scratch[2 * (size_t)e] = mx[0] + mx[1] + mx[2];
    scratch[2 * (size_t)e + 1] = mx[3] + mx[4] + mx[5];
  }
}

// pass 2: one block, min over elements of CFLScale*2/lambda_conv and DFLScale*4/lambda_visc
__global__ void __launch_bounds__(1024)
k_cfl_min(int nElems, int parabolic, double CFLScale, double DFLScale, double* __restrict__ scratch) {
  __shared__ double red[2][32];
  double dc = HUGE_VAL, dv = HUGE_VAL;
  for (int e = threadIdx.x; e < nElems; e += blockDim.x) {
    dc = fmin(dc, CFLScale * 2. / scratch[2 * (size_t)e]);
    if (parabolic) dv = fmin(dv, DFLScale * 4. / scratch[2 * (size_t)e + 1]);
  }
  for (int o = 16; o > 0; o >>= 1) {
    dc = fmin(dc, __shfl_xor_sync(0xffffffffu, dc, o));
    dv = fmin(dv, __shfl_xor_sync(0xffffffffu, dv, o));
  }
  if ((threadIdx.x & 31) == 0) { red[0][threadIdx.x >> 5] = dc; red[1][threadIdx.x >> 5] = dv; }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x / 32); ++w) { dc = fmin(dc, red[0][w]); dv = fmin(dv, red[1][w]); }
    dc = fmin(dc, red[0][0]);
    dv = fmin(dv, red[1][0]);
    scratch[2 * (size_t)DG_NOALLOC_MAX_ELEMS + 0] = dc;
    scratch[2 * (size_t)DG_NOALLOC_MAX_ELEMS + 1] = dv;
  }
}

// CFL / DFL scaling of FillCFL_DFL for Carpenter RK4-5 (same tables as dg_calc_timestep)
double cfl_alpha(int node_type, int N) {
  static const double G[15] = {2.0351, 1.7595, 1.5401, 1.3702, 1.2375, 1.1318, 1.0440, 0.9709,
                               0.9079, 0.8539, 0.8066, 0.7650, 0.7290, 0.6952, 0.6660};
  static const double GL[15] = {4.7497, 3.4144, 2.8451, 2.4739, 2.2027, 1.9912, 1.8225, 1.6830,
                                1.5682, 1.4692, 1.3849, 1.3106, 1.2454, 1.1880, 1.1362};
  const int i = (N < 15 ? N : 15) - 1;
  return node_type == DG_NODETYPE_GAUSS ? G[i] : GL[i];
}
double dfl_alpha(int node_type, int N) {
  static const double G[10] = {1.12, 0.76, 0.55, 0.41, 0.32, 0.25, 0.20, 0.17, 0.14, 0.12};
  static const double GL[10] = {4.50, 1.95, 1.18, 0.79, 0.56, 0.42, 0.32, 0.25, 0.20, 0.17};
  const int i = (N < 10 ? N : 10) - 1;
  return node_type == DG_NODETYPE_GAUSS ? G[i] : GL[i];
}

}  // namespace

extern "C" int dg_calc_timestep_noalloc(int N, int node_type, int nElems, int parabolic, double kappa, double mu0,
                                        double Pr, const double* d_U, const double* d_metrics_f,
                                        const double* d_metrics_g, const double* d_metrics_h, const double* d_sJ,
                                        double cfl_scale, double dfl_scale, double* dt_out, void* stream) {
  if (N < 1 || N > DG_MAX_N || (node_type != DG_NODETYPE_GAUSS && node_type != DG_NODETYPE_GAUSS_LOBATTO)) {
    set_error("dg_calc_timestep_noalloc: bad N or node type");
    return DG_ERR_ARG;
  }
  if (nElems < 1 || nElems > DG_NOALLOC_MAX_ELEMS) {
    set_error("dg_calc_timestep_noalloc: nElems must be in 1.." + std::to_string(DG_NOALLOC_MAX_ELEMS) +
              " (size of the static scratch array)");
    return DG_ERR_ARG;
  }
  if (!d_U || !d_metrics_f || !d_metrics_g || !d_metrics_h || !d_sJ || !dt_out || !(kappa > 1.) ||
      (parabolic && !(Pr > 0.))) {
    set_error("dg_calc_timestep_noalloc: bad argument");
    return DG_ERR_ARG;
  }
  double* scratch = nullptr;
  if (int rc = scratch_ptr(&scratch)) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  const int n3 = (N + 1) * (N + 1) * (N + 1);
  const double cflS = cfl_scale * cfl_alpha(node_type, N) / (2. * N + 1.);
  const double dflS = dfl_scale * dfl_alpha(node_type, N) * 1.853 / ((2. * N + 1.) * (2. * N + 1.));
  const double kpr = (4. / 3. > kappa / Pr) ? 4. / 3. : kappa / Pr;
  double* tail = scratch + 2 * (size_t)DG_NOALLOC_MAX_ELEMS;
  // the scratch keeps the previous call's contents: clear the bad-node counter
  cudaError_t e = cudaMemsetAsync(tail + 2, 0, sizeof(unsigned long long), st);
  if (e != cudaSuccess) { set_error(std::string("clear scratch: ") + cudaGetErrorString(e)); return DG_ERR_CUDA; }
  k_cfl_elem<<<nElems, ((n3 + 31) / 32) * 32, 0, st>>>(d_U, d_metrics_f, d_metrics_g, d_metrics_h, d_sJ, n3, kappa,
                                                       mu0, parabolic, kpr, scratch);
  k_cfl_min<<<1, 1024, 0, st>>>(nElems, parabolic, cflS, dflS, scratch);
  e = cudaGetLastError();
  if (e != cudaSuccess) { set_error(std::string("k_cfl launch: ") + cudaGetErrorString(e)); return DG_ERR_CUDA; }
  double h[3];
  e = cudaMemcpyAsync(h, tail, sizeof(h), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) { set_error(std::string("read dt: ") + cudaGetErrorString(e)); return DG_ERR_CUDA; }
  unsigned long long bad;
  static_assert(sizeof(bad) == sizeof(double), "counter slot");
  std::memcpy(&bad, &h[2], sizeof(bad));
  *dt_out = h[0] < h[1] ? h[0] : h[1];
  if (bad) { set_error("state holds NaN/Inf or non-positive density/pressure"); return DG_ERR_NAN; }
  return DG_OK;
}
