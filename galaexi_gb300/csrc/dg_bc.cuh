// Boundary conditions of the Navier-Stokes operator (equations/navierstokes/idealgas/getboundaryflux.f90):
// the boundary state (GetBoundaryState :262-487), the boundary flux (GetBoundaryFlux_GPU :542-838)
// and the lifting flux (Lifting_GetBoundaryFlux_Kernel :945-1019), for BC types
//   2 (Dirichlet from a reference state), 3 (adiabatic no-slip wall), 4 (isothermal no-slip wall),
//   9 / 91 (slip walls), 23 (outflow Mach number), 24 (pressure outflow), 25 (subsonic outflow),
//   27 (subsonic inflow from total temperature / pressure).
// BC sides are the first nBCSides sides; each has only its master element.  Primitive states are
// (rho, u, v, w, p, T) with absolute pressure p.
#pragma once
#include "dg_physics.cuh"

namespace gx {

// Reference states are (rho, u, v, w, p, T) -- for type 27: (T_t, a1, a2, a3, p_t, -) with a the
// inflow direction (converted from the angles on the host); each BC side carries its type and a
// 0-based reference-state index.

template <typename R> __device__ __forceinline__ R bc_pow(R x, double e) { return (R)::pow((double)x, e); }
template <int K> __device__ __forceinline__ Dual<K> bc_pow(Dual<K> x, double e) {
  Dual<K> r;
  r.v = ::pow(x.v, e);
  const double d = e * ::pow(x.v, e - 1.);
#pragma unroll
  for (int k = 0; k < K; ++k) r.d[k] = d * x.d[k];
  return r;
}

// PRESSURE_RIEMANN_PURE (idealgas/eos.f90:605-628): wall pressure from the local Riemann problem,
// P in the normal frame (VEL1 = normal velocity)
template <typename R>
__device__ __forceinline__ R pressure_riemann(const R P[6], R kappa) {
  if (P[1] <= R(0)) {  // rarefaction
    const double kf = 2. * (double)kappa / ((double)kappa - 1.);
    const R base = fmax(R(0.0001), R(1) + R(0.5) * (kappa - R(1)) * P[1] / sqrt(kappa * P[4] / P[0]));
    return P[4] * bc_pow(base, kf);
  }
  const R ar = R(2) / ((kappa + R(1)) * P[0]);
  const R br = (kappa - R(1)) / (kappa + R(1)) * P[4];
  return P[4] + P[1] / ar * R(0.5) * (P[1] + sqrt(P[1] * P[1] + R(4) * ar * (P[4] + br)));
}

// GetBoundaryState: Pm the inner face state, Pb the boundary state (both Cartesian velocities)
template <typename R>
__device__ __forceinline__ void bc_state(int type, const R Pm[6], const R* ref, const R nv[3], const R t1[3],
                                         const R t2[3], R kappa, R Rgas, R Pb[6]) {
  if (type == 2) {
#pragma unroll
    for (int c = 0; c < 6; ++c) Pb[c] = ref[c];
    return;
  }
  R B[6];
  B[0] = Pm[0];
  B[1] = Pm[1] * nv[0] + Pm[2] * nv[1] + Pm[3] * nv[2];
  B[2] = Pm[1] * t1[0] + Pm[2] * t1[1] + Pm[3] * t1[2];
  B[3] = Pm[1] * t2[0] + Pm[2] * t2[1] + Pm[3] * t2[2];
  B[4] = Pm[4];
  B[5] = Pm[5];
  if (type == 3 || type == 4) {  // adiabatic / isothermal no-slip wall
    B[4] = pressure_riemann(B, kappa);
    B[1] = R(0); B[2] = R(0); B[3] = R(0);
    B[5] = (type == 3) ? Pm[5] : ref[5];
    B[0] = B[4] / (B[5] * Rgas);
  } else if (type == 9 || type == 91) {  // slip wall
    B[4] = pressure_riemann(B, kappa);
    B[1] = R(0);
    B[0] = Pm[0];
    B[5] = B[4] / (B[0] * Rgas);
  } else if (type == 23) {  // outflow Mach number
    const R MaOut = ref[1];
    const R c = sqrt(kappa * B[4] / B[0]);
    const R Ma = B[1] / c;
    R pb;
    if (Ma < R(1)) {
      const double ex = (double)kappa / ((double)kappa - 1.);
      const R pt = B[4] * bc_pow(R(1) + R(0.5) * (kappa - R(1)) * Ma * Ma, ex);
      pb = pt * bc_pow(R(1) + R(0.5) * (kappa - R(1)) * MaOut * MaOut, -ex);
    } else {
      pb = B[4] + R(0.5) * B[0] * (B[1] * B[1] + B[2] * B[2] + B[3] * B[3]);
    }
    B[0] = kappa * pb / (c * c);
    B[4] = pb;
    B[5] = B[4] / (Rgas * B[0]);
  } else if (type == 24) {  // pressure outflow
    const R c = sqrt(kappa * B[4] / B[0]);
    const R Ma = B[1] / c;
    if (Ma < R(1)) {
      const R pb = ref[4];
      B[0] = kappa * pb / (c * c);
      B[4] = pb;
      B[5] = B[4] / (Rgas * B[0]);
    }
  } else if (type == 25) {  // subsonic outflow
    const R c = sqrt(kappa * B[4] / B[0]);
    const R Ma = B[1] / c;
    R pb;
    if (Ma < R(1)) pb = ref[4];
    else pb = B[4] + R(0.5) * B[0] * (B[1] * B[1] + B[2] * B[2] + B[3] * B[3]);
    if (B[1] < R(0)) {
      B[1] = fabs(B[1]);
      B[2] = R(0);
      B[3] = R(0);
    }
    B[0] = kappa * pb / (c * c);
    B[4] = ref[4];
    B[5] = B[4] / (Rgas * B[0]);
  } else if (type == 27) {  // subsonic inflow
    const R Tt = ref[0], pt = ref[4];
    const R a[3] = {ref[1], ref[2], ref[3]};
    const R A = R(-1) * (a[0] * nv[0] + a[1] * nv[1] + a[2] * nv[2]);
    const R c = sqrt(kappa * B[4] / B[0]);
    const R Rplus = -B[1] - R(2) * c / (kappa - R(1));
    const R t1_ = A * A + R(2) / (kappa - R(1));
    const R t2_ = R(2) * Rplus;
    const R t3_ = (kappa - R(1)) / R(2) * (Rplus * Rplus) - kappa * Rgas * Tt * (A * A);
    const R disc = sqrt(t2_ * t2_ - R(4) * t1_ * t3_);
    const R cb = fmax((-t2_ + disc) / (R(2) * t1_), (-t2_ - disc) / (R(2) * t1_));
    const R Tb = cb * cb / (kappa * Rgas);
    const R Ma = sqrt(R(2) / (kappa - R(1)) * (Tt / Tb - R(1)));
    const R pb = pt * bc_pow(R(1) + R(0.5) * (kappa - R(1)) * (Ma * Ma), -(double)kappa / ((double)kappa - 1.));
    const R U = Ma * sqrt(kappa * Rgas * Tb);
    B[0] = pb / (Rgas * Tb);
    B[1] = U * (a[0] * nv[0] + a[1] * nv[1] + a[2] * nv[2]);
    B[2] = U * (a[0] * t1[0] + a[1] * t1[1] + a[2] * t1[2]);
    B[3] = U * (a[0] * t2[0] + a[1] * t2[1] + a[2] * t2[2]);
    B[4] = pb;
    B[5] = Tb;
  }
  Pb[0] = B[0];
  Pb[1] = B[1] * nv[0] + B[2] * t1[0] + B[3] * t2[0];
  Pb[2] = B[1] * nv[1] + B[2] * t1[1] + B[3] * t2[1];
  Pb[3] = B[1] * nv[2] + B[2] * t1[2] + B[3] * t2[2];
  Pb[4] = B[4];
  Pb[5] = B[5];
}

// PrimToCons (idealgas/eos.f90:467-489) from primitives with absolute pressure
template <typename R>
__device__ __forceinline__ void prim_to_cons_face(const R P[6], const Gas<R>& g, R U[5]) {
  U[0] = P[0];
  U[1] = P[1] * P[0];
  U[2] = P[2] * P[0];
  U[3] = P[3] * P[0];
  U[4] = P[4] * g.sKappaM1 + R(0.5) * (U[1] * P[1] + U[2] * P[2] + U[3] * P[3]);
}

__device__ __forceinline__ bool bc_riemann_type(int type) {
  return type == 2 || type == 23 || type == 24 || type == 25 || type == 27;
}

// Lifting_GetBoundaryFlux_Kernel as a ghost state: the BR1 lifting of the face uses
// 0.5 (P_master + P_ghost) (weak) / 0.5 (P_ghost - P_master) (strong); with the ghost state
// 2 F - P_master for the reference's boundary lifting value F both forms reproduce it.
// Lifted variables (rho, u, v, w, T).
template <typename R>
__device__ __forceinline__ void bc_lift_ghost(int type, const R Pm[6], const R Pb[6], R ghost[5]) {
  const R pm[5] = {Pm[0], Pm[1], Pm[2], Pm[3], Pm[5]};
  R F[5];
  if (bc_riemann_type(type)) {
    const R pb[5] = {Pb[0], Pb[1], Pb[2], Pb[3], Pb[5]};
#pragma unroll
    for (int c = 0; c < 5; ++c) F[c] = R(0.5) * (pm[c] + pb[c]);
  } else if (type == 3 || type == 4) {
    F[0] = Pb[0]; F[1] = R(0); F[2] = R(0); F[3] = R(0); F[4] = Pb[5];
  } else {  // 9, 91
    F[0] = Pm[0]; F[1] = Pb[1]; F[2] = Pb[2]; F[3] = Pb[3]; F[4] = Pm[5];
  }
#pragma unroll
  for (int c = 0; c < 5; ++c) ghost[c] = R(2) * F[c] - pm[c];
}

// Wall gradients (GetBoundaryFlux_GPU :655-830): type 9 projects all gradients onto the wall
// plane; type 91 the temperature gradient, and keeps only the normal-normal and tangential-
// tangential parts of the velocity gradient
template <typename R>
__device__ __forceinline__ void bc_wall_gradients(int type, const R nv[3], const R t1[3], const R t2[3], R gx[5],
                                                  R gy[5], R gz[5]) {
  const R M00 = R(1) - nv[0] * nv[0], M11 = R(1) - nv[1] * nv[1], M22 = R(1) - nv[2] * nv[2];
  const R M01 = -nv[0] * nv[1], M02 = -nv[0] * nv[2], M21 = -nv[2] * nv[1];
  if (type == 9) {
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      const R x = gx[v], y = gy[v], z = gz[v];
      gx[v] = M00 * x + M01 * y + M02 * z;
      gy[v] = M01 * x + M11 * y + M21 * z;
      gz[v] = M02 * x + M21 * y + M22 * z;
    }
    return;
  }
  // 91
  {
    const R x = gx[4], y = gy[4], z = gz[4];
    gx[4] = M00 * x + M01 * y + M02 * z;
    gy[4] = M01 * x + M11 * y + M21 * z;
    gz[4] = M02 * x + M21 * y + M22 * z;
  }
  const R* G[3] = {gx, gy, gz};
  R vN[3], vT1[3], vT2[3];  // d/dx_d of (v.n, v.t1, v.t2)
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    vN[d] = nv[0] * G[d][1] + nv[1] * G[d][2] + nv[2] * G[d][3];
    vT1[d] = t1[0] * G[d][1] + t1[1] * G[d][2] + t1[2] * G[d][3];
    vT2[d] = t2[0] * G[d][1] + t2[1] * G[d][2] + t2[2] * G[d][3];
  }
  const R nN = nv[0] * vN[0] + nv[1] * vN[1] + nv[2] * vN[2];
  const R t1T1 = t1[0] * vT1[0] + t1[1] * vT1[1] + t1[2] * vT1[2];
  const R t1T2 = t1[0] * vT2[0] + t1[1] * vT2[1] + t1[2] * vT2[2];
  const R t2T1 = t2[0] * vT1[0] + t2[1] * vT1[1] + t2[2] * vT1[2];
  const R t2T2 = t2[0] * vT2[0] + t2[1] * vT2[1] + t2[2] * vT2[2];
  R xN[3], xT1[3], xT2[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    xN[d] = nv[d] * nN;
    xT1[d] = t1[d] * t1T1 + t2[d] * t2T1;
    xT2[d] = t1[d] * t1T2 + t2[d] * t2T2;
  }
  R* Gw[3] = {gx, gy, gz};
#pragma unroll
  for (int d = 0; d < 3; ++d)
#pragma unroll
    for (int c = 0; c < 3; ++c) Gw[d][1 + c] = nv[c] * xN[d] + t1[c] * xT1[d] + t2[c] * xT2[d];
}

}  // namespace gx
