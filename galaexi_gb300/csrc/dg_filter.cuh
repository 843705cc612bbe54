// Filtering of the solution at the start of the operator (DGTimeDerivative_weakForm step 1,
// src/dg/dg.f90:330): U <- FilterMat x FilterMat x FilterMat U per element, in place, FP64.
//   k_filter      cut-off and modal filters (Filter -> ChangeBasis3D_GPU, filter.f90:272-311,
//                 interpolation/changeBasis.t90:287-359): xi, eta, zeta sweeps in that order
//   k_filter_laf  the adaptive filter LAF (Filter_LAF, filter.f90:318-474): per element the kinetic
//                 energy of the filtered field and of the removed fluctuations decide whether the
//                 filtered field replaces the element's solution; per-element state lim, eRatio, r,
//                 and the previous energies persist between calls.
#pragma once
#include "dg_kernels.cuh"

namespace gx {

// the three sweeps on an element held in shared memory as X[v][node] (node = i + n*(j + n*k)), one
// thread per node; the partial results stay in registers across the barriers, so one buffer suffices.
// Every thread of the block calls it (it holds barriers); inactive threads only wait.
template <int NP>
__device__ __forceinline__ void filter_sweeps(double (*X)[NP * NP * NP], const double* F, int node, bool active) {
  constexpr int n = NP;
  const int i = node % n, j = (node / n) % n, k = node / (n * n);
#pragma unroll 1
  for (int dir = 0; dir < 3; ++dir) {
    double acc[5] = {0., 0., 0., 0., 0.};
    if (active) {
      const int stride = dir == 0 ? 1 : (dir == 1 ? n : n * n);
      const int ii = dir == 0 ? i : (dir == 1 ? j : k);
      const int base = node - ii * stride;
#pragma unroll
      for (int l = 0; l < n; ++l) {
        const double f = F[ii + n * l];
#pragma unroll
        for (int v = 0; v < 5; ++v) acc[v] = acc[v] + f * X[v][base + l * stride];
      }
    }
    __syncthreads();
    if (active) {
#pragma unroll
      for (int v = 0; v < 5; ++v) X[v][node] = acc[v];
    }
    __syncthreads();
  }
}

template <int NP>
__global__ void __launch_bounds__(EPBof<NP>::v * NP * NP * NP)
k_filter(double* __restrict__ U, const double* __restrict__ Fm, int nElems) {
  constexpr int n3 = NP * NP * NP, EPB = EPBof<NP>::v;
  __shared__ double F[NP * NP];
  __shared__ double X[EPB][5][n3];
  for (int t = threadIdx.x; t < NP * NP; t += blockDim.x) F[t] = Fm[t];
  const int e0 = blockIdx.x * EPB;
  const int nloc = min(EPB, nElems - e0);
  double* Ub = U + (size_t)e0 * 5 * n3;
  for (int t = threadIdx.x; t < nloc * 5 * n3; t += blockDim.x) {
    const int el = t / (5 * n3), r = t - el * 5 * n3;
    X[el][r % 5][r / 5] = Ub[t];
  }
  __syncthreads();
  const int el = threadIdx.x / n3, node = threadIdx.x - el * n3;
  filter_sweeps<NP>(X[el < EPB ? el : 0], F, node, el < nloc);
  for (int t = threadIdx.x; t < nloc * 5 * n3; t += blockDim.x) {
    const int e = t / (5 * n3), r = t - e * 5 * n3;
    Ub[t] = X[e][r % 5][r / 5];
  }
}

// LAF state per element: lim, eRatio, r, ekin_avg_old, ekin_fluc_avg_old
struct LafState {
  double* s;   // [5][nElems]
  const double* iw;  // IntegrationWeight [e][n3], normalised by the element volume
  double alpha, normMod;
};

// deterministic block sum of K values per thread (fixed shuffle tree, then the warps in order);
// every thread receives the sums
template <int K>
__device__ __forceinline__ void block_sum(double (&v)[K], double (*part)[32]) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int c = 0; c < K; ++c)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v[c] += __shfl_down_sync(0xffffffffu, v[c], o);
  if (lane == 0)
#pragma unroll
    for (int c = 0; c < K; ++c) part[c][wid] = v[c];
  __syncthreads();
#pragma unroll
  for (int c = 0; c < K; ++c) {
    double s = 0.;
    for (int w = 0; w < nw; ++w) s = s + part[c][w];
    v[c] = s;
  }
  __syncthreads();
}

// one element per block, one thread per node (the block is padded to whole warps)
template <int NP>
__global__ void __launch_bounds__(((NP * NP * NP + 31) / 32) * 32)
k_filter_laf(double* __restrict__ U, const double* __restrict__ Fm, int nElems, LafState S) {
  constexpr int n3 = NP * NP * NP;
  __shared__ double F[NP * NP];
  __shared__ double X[5][n3];
  __shared__ double part[3][32];
  __shared__ int apply;
  const int e = blockIdx.x, node = threadIdx.x;
  const bool active = node < n3;
  for (int t = threadIdx.x; t < NP * NP; t += blockDim.x) F[t] = Fm[t];
  double* Ue = U + (size_t)e * 5 * n3;
  double u0[5] = {1., 0., 0., 0., 0.};
  if (active) {
#pragma unroll
    for (int v = 0; v < 5; ++v) u0[v] = Ue[node * 5 + v];
#pragma unroll
    for (int v = 0; v < 5; ++v) X[v][node] = u0[v];
  }
  __syncthreads();
  filter_sweeps<NP>(X, F, active ? node : 0, active);
  const double w = active ? S.iw[(size_t)e * n3 + node] : 0.;
  const double rho = u0[0];
  double uf[3] = {0., 0., 0.};
  if (active) { uf[0] = X[1][node]; uf[1] = X[2][node]; uf[2] = X[3][node]; }
  // element mean velocity of the filtered field, U_Avg(2:4)
  double avg[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) avg[c] = uf[c] / rho * w;
  block_sum<3>(avg, part);
  // kinetic energies of the fluctuations removed by the filter and of the filtered field
  double en[2] = {0., 0.};
  if (active) {
    const double f1 = u0[1] - uf[0], f2 = u0[2] - uf[1], f3 = u0[3] - uf[2];
    const double r2 = rho * rho;
    en[0] = (f1 * f1 / r2 + f3 * f3 / r2 + f2 * f2 / r2) * w;
    const double d1 = uf[0] - avg[0], d2 = uf[1] - avg[1], d3 = uf[2] - avg[2];
    en[1] = (d1 * d1 / r2 + d2 * d2 / r2 + d3 * d3 / r2) * w;
  }
  block_sum<2>(en, part);
  if (threadIdx.x == 0) {
    const double fluc = en[0], kin = en[1];
    double* lim = S.s;
    double* eRatio = S.s + nElems;
    double* r = S.s + 2 * (size_t)nElems;
    double* kin_old = S.s + 3 * (size_t)nElems;
    double* fluc_old = S.s + 4 * (size_t)nElems;
    eRatio[e] = (fluc / kin) * S.normMod;
    lim[e] = fmax(lim[e], 1.0e-8);
    const double dfl = fluc - fluc_old[e];
    const double dedt_lim = fabs(kin - kin_old[e]) / dfl;
    int ap = 0;
    if (dedt_lim > 1.0 && dfl > 0.) lim[e] = eRatio[e];
    else if (dfl < 0.) lim[e] = eRatio[e];
    else if (eRatio[e] > lim[e] * S.alpha) { ap = 1; r[e] = r[e] + 1.; }
    kin_old[e] = kin;
    fluc_old[e] = fluc;
    apply = ap;
  }
  __syncthreads();
  if (apply && active) {
#pragma unroll
    for (int v = 0; v < 5; ++v) Ue[node * 5 + v] = X[v][node];
  }
}

}  // namespace gx
