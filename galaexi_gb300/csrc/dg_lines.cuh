// Split-form volume integral of the mixed (FP32) form with one thread per 1D line of an element.
//
// VolInt_splitForm (src/dg/volint.f90:211-353, SplitVolumeFlux* of splitflux.f90:145-730) sums, for
// every node i of a line, DVolSurf(l,i) * F#(U_i, U_l; (M_i + M_l)/2) over the line's nodes l.  In the
// element-per-block kernel the line's nodes sit in shared memory and every pair costs ~20 shared-memory
// accesses (the partner's node data, and the read-modify-write of its accumulators), which bounds the
// FP32 kernel.  Here a thread holds its whole line in registers: the node data (rho, u, v, w, the
// momentum pressure, the form's auxiliary variable and the line direction's metric terms) and the five
// accumulators of every node.  All n(n-1)/2 pairs run fully unrolled for the compile-time n with each
// pair flux evaluated once and added to both nodes, and the DVolSurf coefficients are compile-time
// indexed kernel parameters (constant-bank operands of the FMAs).  A block is one element's 3 n^2
// lines; the three directions' sums of a node meet in shared memory (padded so that neither the
// line-ordered writes nor the node-ordered reads conflict at N = 7) and the node's split volume term
// is written to Vs[e][5][n^3], which k_volume adds to its viscous volume and surface terms.
// Registers: ~9 n + 5 n values per thread, so the kernel is instantiated for n <= 8 and the forms
// whose pair flux needs no momenta (SD, KG, PI).
#pragma once
#include "dg_physics.cuh"

namespace gx {

// DVolSurf(l,i) at d[l + NP*i], pre-scaled for the form (PI: 1/8, see the pair flux below)
template <int NP> struct LineDVS { float d[NP * NP]; };

template <int NP> __host__ __device__ constexpr int line_pad(int dir) {
  // row strides of the three directions' result regions: with n = 8 these make the bank of
  // (row l, line) distinct for the 32 lines a warp writes and for the 32 nodes a warp reads
  return NP * NP + (dir == 0 ? 4 : (dir == 1 ? 8 : 0));
}
template <int NP> __host__ __device__ constexpr int line_red_words() {
  return 5 * NP * (line_pad<NP>(0) + line_pad<NP>(1) + line_pad<NP>(2));
}
template <int SPLIT> struct LinesForm {
  static constexpr bool v = SPLIT == DG_SPLIT_PI || SPLIT == DG_SPLIT_KG || SPLIT == DG_SPLIT_SD;
};
template <int NP, typename R, int SPLIT> struct UseLines {
  static constexpr bool v = sizeof(R) == 4 && NP >= 4 && NP <= 8 && LinesForm<SPLIT>::v;
};

template <int NP, int SPLIT>
__global__ void __launch_bounds__(3 * NP * NP, 2)
k_split_lines(const float* __restrict__ Pvol, const float* __restrict__ Met, LineDVS<NP> dvs, Gas<float> gas,
              int nElems, float* __restrict__ Vs) {
  constexpr int n = NP, n2 = NP * NP, n3 = NP * NP * NP;
  constexpr int P0 = line_pad<NP>(0), P1 = line_pad<NP>(1), P2 = line_pad<NP>(2);
  constexpr int OFF1 = 5 * n * P0, OFF2 = OFF1 + 5 * n * P1;
  __shared__ float red[line_red_words<NP>()];
  const int e = blockIdx.x;
  if (e >= nElems) return;
  const int tid = threadIdx.x;
  const int dir = tid / n2, li = tid - dir * n2;
  int base, stride;
  if (dir == 0) { base = n * li; stride = 1; }
  else if (dir == 1) { base = (li % n) + n2 * (li / n); stride = n; }
  else { base = li; stride = n2; }
  const float* P = Pvol + (size_t)e * 7 * n3;
  const float* M = Met + ((size_t)e * 10 + 3 * dir) * n3;
  // the line's node data
  float rho[n], u[n], v[n], w[n], pm[n], aux[n], m0[n], m1[n], m2[n];
#pragma unroll
  for (int l = 0; l < n; ++l) {
    const int node = base + l * stride;
    rho[l] = P[node];
    u[l] = P[n3 + node];
    v[l] = P[2 * n3 + node];
    w[l] = P[3 * n3 + node];
    const float pmom = P[4 * n3 + node];  // momentum pressure (p' = p - p_ref in the mixed form)
    const float srho = P[6 * n3 + node];
    m0[l] = M[node];
    m1[l] = M[n3 + node];
    m2[l] = M[2 * n3 + node];
    const float pabs = p_abs(pmom, gas);
    const float E = pabs * gas.sKappaM1 + 0.5f * rho[l] * (u[l] * u[l] + v[l] * v[l] + w[l] * w[l]);
    aux[l] = pair_aux<SPLIT, float>(rho[l], u[l], v[l], w[l], E, pabs, srho);
    pm[l] = (SPLIT == DG_SPLIT_PI) ? 4.f * pmom : pmom;  // PI: 4p (exact scaling, see below)
  }
  float acc[n][5];
#pragma unroll
  for (int l = 0; l < n; ++l)
#pragma unroll
    for (int c = 0; c < 5; ++c) acc[l][c] = 0.f;
#pragma unroll
  for (int a = 0; a < n - 1; ++a) {
#pragma unroll
    for (int b = a + 1; b < n; ++b) {
      const float Ms0 = m0[a] + m0[b], Ms1 = m1[a] + m1[b], Ms2 = m2[a] + m2[b];
      float F[5];
      if constexpr (SPLIT == DG_SPLIT_PI) {
        // 8 x the PI flux, the density row at 4 x (doubled at the end); DVolSurf carries the 1/8
        const float rs = rho[a] + rho[b], us = u[a] + u[b], vs = v[a] + v[b], ws = w[a] + w[b];
        const float ps4 = pm[a] + pm[b];
        const float Vsum = Ms0 * us + Ms1 * vs + Ms2 * ws;
        const float q8 = rs * Vsum;
        F[0] = q8;
        F[1] = q8 * us + ps4 * Ms0;
        F[2] = q8 * vs + ps4 * Ms1;
        F[3] = q8 * ws + ps4 * Ms2;
        F[4] = q8 * (aux[a] + aux[b]);
      } else {
        PairNode<float> A, B;
        A.rho = rho[a]; A.u = u[a]; A.v = v[a]; A.w = w[a]; A.pm = pm[a]; A.aux = aux[a];
        B.rho = rho[b]; B.u = u[b]; B.v = v[b]; B.w = w[b]; B.pm = pm[b]; B.aux = aux[b];
        A.m1 = A.m2 = A.m3 = B.m1 = B.m2 = B.m3 = 0.f;
        split_pair_flux<SPLIT, float>(A, B, Ms0, Ms1, Ms2, 2.f * gas.pref, F);
      }
      const float dba = dvs.d[b + n * a], dab = dvs.d[a + n * b];  // DVolSurf(l=b,i=a), DVolSurf(l=a,i=b)
#pragma unroll
      for (int c = 0; c < 5; ++c) {
        acc[a][c] = acc[a][c] + dba * F[c];
        acc[b][c] = acc[b][c] + dab * F[c];
      }
    }
  }
  // the three directions' sums of every node meet in shared memory
  float* R0 = red + (dir == 0 ? 0 : (dir == 1 ? OFF1 : OFF2));
  const int Pd = dir == 0 ? P0 : (dir == 1 ? P1 : P2);
#pragma unroll
  for (int l = 0; l < n; ++l)
#pragma unroll
    for (int c = 0; c < 5; ++c)
      R0[(c * n + l) * Pd + li] = (SPLIT == DG_SPLIT_PI && c == 0) ? 2.f * acc[l][c] : acc[l][c];
  __syncthreads();
  float* out = Vs + (size_t)e * 5 * n3;
  for (int t = tid; t < 5 * n3; t += blockDim.x) {
    const int c = t / n3, node = t - c * n3;
    const int i = node % n, j = (node / n) % n, k = node / n2;
    out[t] = red[(c * n + i) * P0 + j + n * k] + red[OFF1 + (c * n + j) * P1 + i + n * k] +
             red[OFF2 + (c * n + k) * P2 + i + n * j];
  }
}

}  // namespace gx
