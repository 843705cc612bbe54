// Pointwise physics of the compressible Navier-Stokes DGSEM operator, device side.
//
// Templated on the compute type R (double for the plain path, float for the bulk of the mixed
// path).  The formulas are those of the reference (citations per function); the two-point
// volume fluxes are rewritten in contravariant form (see split_pair_flux) so that one pair
// evaluation costs ~25 FP64 instructions instead of the reference's three Cartesian fluxes
// followed by a metric contraction.  All are branch-uniform within a launch (the solver and
// split choice are launch constants).
#pragma once
#include <cuda_runtime.h>
#include <math.h>
#include <type_traits>
#include "../../include/galaexi_gb300.h"
#include "dg_dual.cuh"
#include "dg_convert.cuh"

namespace gx {

// Gas constants.  pref is the reference pressure of the mixed form: there, the pressure held in the
// primitive arrays is p' = p - pref (computed in FP64 from the FP64 state) and the momentum pressure
// terms of the volume and surface fluxes use p'.  A constant pressure offset drops out of the full
// operator for free-stream-preserving metrics, so this is exact in exact arithmetic; it keeps the
// O(1) pressure differences of low-Mach flows from drowning in FP32 round-off of p ~ 1/(kappa Ma^2).
// In the FP64 form pref is zero and never applied (kOffset<double> is false).
template <typename R> struct Gas {
  R kappa, kappaM1, sKappaM1, R_gas, mu, lambda, sR;
  R pref;
  double prefD, kappaM1D, sRD;
};
template <typename R> struct OffsetOf { static constexpr bool v = false; };
template <> struct OffsetOf<float> { static constexpr bool v = true; };

// compute type R from a state value of type S (FP64, or dual numbers in the tangent-linear operator)
template <typename R, typename S> __device__ __forceinline__ R narrow(const S& x) {
  if constexpr (OffsetOf<R>::v && std::is_same<S, double>::value) return f64_to_f32_rn(x);
  else return (R)x;
}
// state type S from a compute-type value x
template <typename S, typename R> __device__ __forceinline__ S widen(const R& x) {
  if constexpr (std::is_same<R, float>::value && std::is_same<S, double>::value) return f32_to_f64(x);
  else return (S)x;
}

// ConsToPrim of the mixed form from FP32 density and momenta c and the FP64 energy E: velocities and
// kinetic energy in FP32 (relative error ~1e-7 of quantities that are themselves rounded to FP32), the
// energy difference E - ke and p' = p - p_ref in FP64, where the cancellation at low Mach would lose
// the pressure fluctuations
template <typename R>
__device__ __forceinline__ void cons_to_prim_mixed(const R c[4], double E, const Gas<R>& g, R prim[6], R& srho) {
  const R sr = R(1) / c[0];
  const R v1 = c[1] * sr, v2 = c[2] * sr, v3 = c[3] * sr;
  const R ke = R(0.5) * (c[1] * v1 + c[2] * v2 + c[3] * v3);
  const double p = g.kappaM1D * (E - f32_to_f64(ke));
  srho = sr;
  prim[0] = c[0];
  prim[1] = v1;
  prim[2] = v2;
  prim[3] = v3;
  prim[4] = f64_to_f32_rn(p - g.prefD);
  prim[5] = f64_to_f32_rn(p) * sr * g.sR;
}

// ConsToPrim (idealgas/eos.f90:212-239) from the FP64 state: rho, u, v, w, p (p' in the mixed form), T, 1/rho
template <typename R, typename S>
__device__ __forceinline__ void cons_to_prim_d(const S u[5], const Gas<R>& g, R prim[6], R& srho) {
  if constexpr (!OffsetOf<R>::v) {
    srho = R(1) / (R)u[0];
    prim[0] = (R)u[0];
    prim[1] = (R)u[1] * srho;
    prim[2] = (R)u[2] * srho;
    prim[3] = (R)u[3] * srho;
    prim[4] = g.kappaM1 * ((R)u[4] - R(0.5) * ((R)u[1] * prim[1] + (R)u[2] * prim[2] + (R)u[3] * prim[3]));
    prim[5] = prim[4] * srho * g.sR;
  } else {
    const R c[4] = {narrow<R>(u[0]), narrow<R>(u[1]), narrow<R>(u[2]), narrow<R>(u[3])};
    cons_to_prim_mixed(c, (double)u[4], g, prim, srho);
  }
}
// absolute pressure from the stored one
template <typename R>
__device__ __forceinline__ R p_abs(R pstored, const Gas<R>& g) {
  if constexpr (OffsetOf<R>::v) return pstored + g.pref;
  else return pstored;
}

// ---------------------------------------------------------------------------------------------
// Two-point volume fluxes (splitflux.f90:145-730) in contravariant form.
// With Ms = M_a + M_b (the metric sum; the reference averages 0.5*(MRef+M)) and the pair sums
// rs = rho_a+rho_b, us = u_a+u_b, ..., the reference's  sum_d 0.5*Ms_d * f_d  becomes a
// function of the contravariant velocity Vs = Ms . us; algebraically identical to the reference.
// Node data: c = (rho, m1, m2, m3), v = (u, v, w), pm = momentum pressure (p, or p' in the mixed
// form), aux = the per-node energy quantity of the flux: H=(E+p)/rho (PI), E/rho (KG), E+p (DU, SD),
// rho*e+p = E - rho|v|^2/2 + p (MO).  pref2 = 2*pref (KG's energy term needs the absolute p sum).
// ---------------------------------------------------------------------------------------------
template <typename R>
struct PairNode {
  R rho, m1, m2, m3, u, v, w, pm, aux;
};

template <int SPLIT, typename R>
__device__ __forceinline__ R pair_aux(R rho, R u, R v, R w, R E, R pabs, R srho) {
  if (SPLIT == DG_SPLIT_PI) return (E + pabs) * srho;
  if (SPLIT == DG_SPLIT_KG) return E * srho;
  if (SPLIT == DG_SPLIT_MO) return E - R(0.5) * rho * (u * u + v * v + w * w) + pabs;
  return E + pabs;  // DU, SD
}

template <int SPLIT, typename R>
__device__ __forceinline__ void split_pair_flux(const PairNode<R>& a, const PairNode<R>& b, R Ms0, R Ms1, R Ms2,
                                                R pref2, R F[5]) {
  if (SPLIT == DG_SPLIT_PI || SPLIT == DG_SPLIT_KG) {
    const R rs = a.rho + b.rho, us = a.u + b.u, vs = a.v + b.v, ws = a.w + b.w, ps = a.pm + b.pm;
    const R Vs = Ms0 * us + Ms1 * vs + Ms2 * ws;
    const R q = R(0.125) * rs * Vs;
    const R hp = R(0.5) * ps;
    F[0] = R(2) * q;
    F[1] = q * us + hp * Ms0;
    F[2] = q * vs + hp * Ms1;
    F[3] = q * ws + hp * Ms2;
    if (SPLIT == DG_SPLIT_PI) F[4] = q * (a.aux + b.aux);
    else F[4] = q * (a.aux + b.aux) + R(0.25) * (OffsetOf<R>::v ? ps + pref2 : ps) * Vs;
  } else if (SPLIT == DG_SPLIT_DU) {
    const R rs = a.rho + b.rho, us = a.u + b.u, vs = a.v + b.v, ws = a.w + b.w, ps = a.pm + b.pm;
    const R Vs = Ms0 * us + Ms1 * vs + Ms2 * ws;
    const R qv = R(0.25) * Vs;
    const R hp = R(0.5) * ps;
    F[0] = qv * rs;
    F[1] = qv * (a.m1 + b.m1) + hp * Ms0;
    F[2] = qv * (a.m2 + b.m2) + hp * Ms1;
    F[3] = qv * (a.m3 + b.m3) + hp * Ms2;
    F[4] = qv * (a.aux + b.aux);
  } else if (SPLIT == DG_SPLIT_SD) {
    const R Va = Ms0 * a.u + Ms1 * a.v + Ms2 * a.w;
    const R Vb = Ms0 * b.u + Ms1 * b.v + Ms2 * b.w;
    const R ra = a.rho * Va, rb = b.rho * Vb;
    const R hp = R(0.5) * (a.pm + b.pm);
    F[0] = R(0.5) * (ra + rb);
    F[1] = R(0.5) * (ra * a.u + rb * b.u) + hp * Ms0;
    F[2] = R(0.5) * (ra * a.v + rb * b.v) + hp * Ms1;
    F[3] = R(0.5) * (ra * a.w + rb * b.w) + hp * Ms2;
    F[4] = R(0.5) * (a.aux * Va + b.aux * Vb);
  } else {  // DG_SPLIT_MO
    const R us = a.u + b.u, vs = a.v + b.v, ws = a.w + b.w, ps = a.pm + b.pm;
    const R Va = Ms0 * a.u + Ms1 * a.v + Ms2 * a.w;
    const R Vb = Ms0 * b.u + Ms1 * b.v + Ms2 * b.w;
    const R MsM = Ms0 * (a.m1 + b.m1) + Ms1 * (a.m2 + b.m2) + Ms2 * (a.m3 + b.m3);
    const R hp = R(0.5) * ps;
    F[0] = R(0.5) * MsM;
    F[1] = R(0.25) * MsM * us + hp * Ms0;
    F[2] = R(0.25) * MsM * vs + hp * Ms1;
    F[3] = R(0.25) * MsM * ws + hp * Ms2;
    const R ka = a.u * a.u + a.v * a.v + a.w * a.w, kb = b.u * b.u + b.v * b.v + b.w * b.w;
    const R ra = a.rho * Va, rb = b.rho * Vb;
    const R dota = a.u * us + a.v * vs + a.w * ws, dotb = b.u * us + b.v * vs + b.w * ws;
    F[4] = R(0.5) * (a.aux * Va + b.aux * Vb + R(0.5) * (ra * dota + rb * dotb) - R(0.5) * (ra * ka + rb * kb));
  }
}

// ---------------------------------------------------------------------------------------------
// Face states in the normal frame (riemann.f90:237-275): the extended state of the reference
// ---------------------------------------------------------------------------------------------
template <typename R>
struct Ext {
  R rho, srho, m1, m2, m3, E, v1, v2, v3, p, pm;  // p absolute, pm the momentum pressure (p or p')
};

// Split surface fluxes (splitflux.f90:270-761), the central part of the split-form Riemann solvers
template <typename R>
__device__ __forceinline__ void split_surface_flux(int split, const Ext<R>& L, const Ext<R>& Rr, R F[5]) {
  switch (split) {
    case DG_SPLIT_SD:
      F[0] = R(0.5) * (L.m1 + Rr.m1);
      F[1] = R(0.5) * (L.m1 * L.v1 + L.pm + Rr.m1 * Rr.v1 + Rr.pm);
      F[2] = R(0.5) * (L.m1 * L.v2 + Rr.m1 * Rr.v2);
      F[3] = R(0.5) * (L.m1 * L.v3 + Rr.m1 * Rr.v3);
      F[4] = R(0.5) * ((L.E + L.p) * L.v1 + (Rr.E + Rr.p) * Rr.v1);
      break;
    case DG_SPLIT_DU:
      F[0] = R(0.25) * (L.rho + Rr.rho) * (L.v1 + Rr.v1);
      F[1] = R(0.25) * (L.m1 + Rr.m1) * (L.v1 + Rr.v1) + R(0.5) * (L.pm + Rr.pm);
      F[2] = R(0.25) * (L.m2 + Rr.m2) * (L.v1 + Rr.v1);
      F[3] = R(0.25) * (L.m3 + Rr.m3) * (L.v1 + Rr.v1);
      F[4] = R(0.25) * (L.E + Rr.E + L.p + Rr.p) * (L.v1 + Rr.v1);
      break;
    case DG_SPLIT_KG: {
      const R eL = L.E * L.srho, eR = Rr.E * Rr.srho;
      const R rs = L.rho + Rr.rho, us = L.v1 + Rr.v1;
      F[0] = R(0.25) * rs * us;
      F[1] = R(0.125) * rs * us * us + R(0.5) * (L.pm + Rr.pm);
      F[2] = R(0.125) * rs * us * (L.v2 + Rr.v2);
      F[3] = R(0.125) * rs * us * (L.v3 + Rr.v3);
      F[4] = R(0.125) * rs * (eL + eR) * us + R(0.25) * (L.p + Rr.p) * us;
    } break;
    case DG_SPLIT_MO: {
      const R rL = L.E - R(0.5) * L.rho * (L.v1 * L.v1 + L.v2 * L.v2 + L.v3 * L.v3) + L.p;
      const R rR = Rr.E - R(0.5) * Rr.rho * (Rr.v1 * Rr.v1 + Rr.v2 * Rr.v2 + Rr.v3 * Rr.v3) + Rr.p;
      const R ms = L.m1 + Rr.m1;
      F[0] = R(0.5) * ms;
      F[1] = R(0.25) * ms * (L.v1 + Rr.v1) + R(0.5) * (L.pm + Rr.pm);
      F[2] = R(0.25) * ms * (L.v2 + Rr.v2);
      F[3] = R(0.25) * ms * (L.v3 + Rr.v3);
      F[4] = R(0.5) * (rL * L.v1 + rR * Rr.v1) +
             R(0.25) * (L.m1 * L.v1 + Rr.m1 * Rr.v1) * (L.v1 + Rr.v1) +
             R(0.25) * (L.m1 * L.v2 + Rr.m1 * Rr.v2) * (L.v2 + Rr.v2) +
             R(0.25) * (L.m1 * L.v3 + Rr.m1 * Rr.v3) * (L.v3 + Rr.v3) -
             R(0.25) * (L.m1 * L.v1 * L.v1 + Rr.m1 * Rr.v1 * Rr.v1) -
             R(0.25) * (L.m1 * L.v2 * L.v2 + Rr.m1 * Rr.v2 * Rr.v2) -
             R(0.25) * (L.m1 * L.v3 * L.v3 + Rr.m1 * Rr.v3 * Rr.v3);
    } break;
    default: {  // PI
      const R HL = (L.E + L.p) * L.srho, HR = (Rr.E + Rr.p) * Rr.srho;
      const R rs = L.rho + Rr.rho, us = L.v1 + Rr.v1;
      F[0] = R(0.25) * rs * us;
      F[1] = R(0.125) * rs * us * us + R(0.5) * (L.pm + Rr.pm);
      F[2] = R(0.125) * rs * us * (L.v2 + Rr.v2);
      F[3] = R(0.125) * rs * us * (L.v3 + Rr.v3);
      F[4] = R(0.125) * rs * (HL + HR) * us;
    } break;
  }
}

// EvalEulerFlux1D_fast (flux.f90:1123-1143)
template <typename R>
__device__ __forceinline__ void euler_flux_1d(const Ext<R>& U, R F[5]) {
  F[0] = U.m1;
  F[1] = U.m1 * U.v1 + U.pm;
  F[2] = U.m1 * U.v2;
  F[3] = U.m1 * U.v3;
  F[4] = (U.E + U.p) * U.v1;
}

// The approximate Riemann solvers of riemann.f90:707-1257 in the rotated frame.
template <typename R>
__device__ __forceinline__ void riemann_solver(int riemann, int split, const Ext<R>& L, const Ext<R>& Rr,
                                               R kappa, R F[5]) {
  const R km1 = kappa - R(1);
  R FL[5], FR[5];
  if (split < 0 || riemann == DG_RIEMANN_HLL || riemann == DG_RIEMANN_HLLC || riemann == DG_RIEMANN_HLLE ||
      riemann == DG_RIEMANN_HLLEM) {
    euler_flux_1d(L, FL);
    euler_flux_1d(Rr, FR);
  }
  const R dU[5] = {Rr.rho - L.rho, Rr.m1 - L.m1, Rr.m2 - L.m2, Rr.m3 - L.m3, Rr.E - L.E};
  if (riemann == DG_RIEMANN_LF) {
    const R cL = sqrt(kappa * L.p * L.srho), cR = sqrt(kappa * Rr.p * Rr.srho);
    const R lam = fmax(fabs(Rr.v1), fabs(L.v1)) + fmax(cL, cR);
    if (split < 0) {
#pragma unroll
      for (int v = 0; v < 5; ++v) F[v] = R(0.5) * ((FL[v] + FR[v]) - lam * dU[v]);
    } else {
      split_surface_flux(split, L, Rr, F);
#pragma unroll
      for (int v = 0; v < 5; ++v) F[v] = F[v] - R(0.5) * lam * dU[v];
    }
    return;
  }
  if (riemann == DG_RIEMANN_AVERAGE) {
    split_surface_flux(split, L, Rr, F);
    return;
  }
  // Roe mean values (shared by all remaining solvers)
  const R HL = (L.E + L.p) * L.srho, HR = (Rr.E + Rr.p) * Rr.srho;
  const R sqL = sqrt(L.rho), sqR = sqrt(Rr.rho);
  const R ssq = R(1) / (sqL + sqR);
  const R rv0 = (sqR * Rr.v1 + sqL * L.v1) * ssq;
  const R rv1 = (sqR * Rr.v2 + sqL * L.v2) * ssq;
  const R rv2 = (sqR * Rr.v3 + sqL * L.v3) * ssq;
  const R RoeH = (sqR * HR + sqL * HL) * ssq;
  const R absVel = rv0 * rv0 + rv1 * rv1 + rv2 * rv2;
  const R Roec = sqrt(km1 * (RoeH - R(0.5) * absVel));
  const R r1[5] = {R(1), rv0 - Roec, rv1, rv2, RoeH - rv0 * Roec};
  const R r2[5] = {R(1), rv0, rv1, rv2, R(0.5) * absVel};
  const R r5[5] = {R(1), rv0 + Roec, rv1, rv2, RoeH + rv0 * Roec};
  if (riemann == DG_RIEMANN_ROE || riemann == DG_RIEMANN_ROEL2) {
    R d[6] = {dU[0], dU[1], dU[2], dU[3], dU[4], R(0)};
    d[5] = d[4] - (d[2] - rv1 * d[0]) * rv1 - (d[3] - rv2 * d[0]) * rv2;
    if (riemann == DG_RIEMANN_ROEL2) {
      const R Ma = sqrt(absVel) / (Roec * sqrt(kappa));
      d[1] *= Ma; d[2] *= Ma; d[3] *= Ma;
    }
    const R A3 = d[2] - rv1 * d[0];
    const R A4 = d[3] - rv2 * d[0];
    const R A2 = km1 / (Roec * Roec) * (d[0] * (RoeH - rv0 * rv0) - d[5] + rv0 * d[1]);
    const R A1 = R(0.5) / Roec * (d[0] * (rv0 + Roec) - d[1] - Roec * A2);
    const R A5 = d[0] - A1 - A2;
    const R w1 = A1 * fabs(rv0 - Roec), w2 = A2 * fabs(rv0), w3 = A3 * fabs(rv0), w4 = A4 * fabs(rv0),
            w5 = A5 * fabs(rv0 + Roec);
    R diss[5];
    diss[0] = w1 + w2 + w5;
    diss[1] = w1 * r1[1] + w2 * r2[1] + w5 * r5[1];
    diss[2] = w1 * r1[2] + w2 * r2[2] + w3 + w5 * r5[2];
    diss[3] = w1 * r1[3] + w2 * r2[3] + w4 + w5 * r5[3];
    diss[4] = w1 * r1[4] + w2 * r2[4] + w3 * rv1 + w4 * rv2 + w5 * r5[4];
    if (split < 0) {
#pragma unroll
      for (int v = 0; v < 5; ++v) F[v] = R(0.5) * ((FL[v] + FR[v]) - diss[v]);
    } else {
      split_surface_flux(split, L, Rr, F);
#pragma unroll
      for (int v = 0; v < 5; ++v) F[v] = F[v] - R(0.5) * diss[v];
    }
    return;
  }
  if (riemann == DG_RIEMANN_ROEENTROPYFIX) {
    const R cL = sqrt(kappa * L.p * L.srho), cR = sqrt(kappa * Rr.p * Rr.srho);
    const R RoeDens = sqrt(L.rho * Rr.rho);
    const R d0 = Rr.rho - L.rho, d1 = Rr.v1 - L.v1, d2 = Rr.v2 - L.v2, d3 = Rr.v3 - L.v3, d4 = Rr.p - L.p;
    const R tmp = R(0.5) / (Roec * Roec);
    const R A[5] = {tmp * (d4 - RoeDens * Roec * d1), d0 - d4 * R(2) * tmp, RoeDens * d2, RoeDens * d3,
                    tmp * (d4 + RoeDens * Roec * d1)};
    R a[5] = {rv0 - Roec, rv0, rv0, rv0, rv0 + Roec};
    const R al[5] = {L.v1 - cL, L.v1, L.v1, L.v1, L.v1 + cL};
    const R ar[5] = {Rr.v1 - cR, Rr.v1, Rr.v1, Rr.v1, Rr.v1 + cR};
#pragma unroll
    for (int i = 0; i < 5; ++i) {
      const R da = fmax(R(0), fmax(a[i] - al[i], ar[i] - a[i]));
      if (fabs(a[i]) < da) a[i] = R(0.5) * (a[i] * a[i] / da + da);
      else a[i] = fabs(a[i]);
    }
    const R w1 = A[0] * a[0], w2 = A[1] * a[1], w3 = A[2] * a[2], w4 = A[3] * a[3], w5 = A[4] * a[4];
    R diss[5];
    diss[0] = w1 + w2 + w5;
    diss[1] = w1 * r1[1] + w2 * r2[1] + w5 * r5[1];
    diss[2] = w1 * r1[2] + w2 * r2[2] + w3 + w5 * r5[2];
    diss[3] = w1 * r1[3] + w2 * r2[3] + w4 + w5 * r5[3];
    diss[4] = w1 * r1[4] + w2 * r2[4] + w3 * rv1 + w4 * rv2 + w5 * r5[4];
    if (split < 0) {
#pragma unroll
      for (int v = 0; v < 5; ++v) F[v] = R(0.5) * ((FL[v] + FR[v]) - diss[v]);
    } else {
      split_surface_flux(split, L, Rr, F);
#pragma unroll
      for (int v = 0; v < 5; ++v) F[v] = F[v] - R(0.5) * diss[v];
    }
    return;
  }
  if (riemann == DG_RIEMANN_HLLC) {
    const R Ssl = rv0 - Roec, Ssr = rv0 + Roec;
    if (Ssl >= R(0)) {
#pragma unroll
      for (int v = 0; v < 5; ++v) F[v] = FL[v];
    } else if (Ssr <= R(0)) {
#pragma unroll
      for (int v = 0; v < 5; ++v) F[v] = FR[v];
    } else {
      const R sMuL = Ssl - L.v1, sMuR = Ssr - Rr.v1;
      const R SStar = (Rr.p - L.p + L.m1 * sMuL - Rr.m1 * sMuR) / (L.rho * sMuL - Rr.rho * sMuR);
      const bool left = (Ssl <= R(0)) && (SStar >= R(0));
      const Ext<R>& S = left ? L : Rr;
      const R sMu = left ? sMuL : sMuR;
      const R Ss = left ? Ssl : Ssr;
      const R* Fs = left ? FL : FR;
      const R EStar = S.E * S.srho + (SStar - S.v1) * (SStar + S.p * S.srho / sMu);
      const R fac = S.rho * sMu / (Ss - SStar);
      const R Ust[5] = {fac, fac * SStar, fac * S.v2, fac * S.v3, fac * EStar};
      const R Sc[5] = {S.rho, S.m1, S.m2, S.m3, S.E};
#pragma unroll
      for (int v = 0; v < 5; ++v) F[v] = Fs[v] + Ss * (Ust[v] - Sc[v]);
    }
    return;
  }
  // HLL, HLLE, HLLEM
  R Ssl, Ssr;
  if (riemann == DG_RIEMANN_HLL) {
    Ssl = rv0 - Roec; Ssr = rv0 + Roec;
  } else {
    const R beta = sqrt(R(0.5) * km1 / kappa);
    const R cL = sqrt(kappa * L.p * L.srho), cR = sqrt(kappa * Rr.p * Rr.srho);
    Ssl = fmin(fmin(rv0 - Roec, L.v1 - beta * cL), R(0));
    Ssr = fmax(fmax(rv0 + Roec, Rr.v1 + beta * cR), R(0));
  }
  if (Ssl >= R(0)) {
#pragma unroll
    for (int v = 0; v < 5; ++v) F[v] = FL[v];
  } else if (Ssr <= R(0)) {
#pragma unroll
    for (int v = 0; v < 5; ++v) F[v] = FR[v];
  } else {
    R jump[5] = {dU[0], dU[1], dU[2], dU[3], dU[4]};
    if (riemann == DG_RIEMANN_HLLEM) {
      const R RoeDens = sqrt(L.rho * Rr.rho);
      const R delta = Roec / (Roec + fabs(R(0.5) * (Ssl + Ssr)));
      const R A2 = (Rr.rho - L.rho) - (Rr.p - L.p) / (Roec * Roec);
      const R A3 = RoeDens * (Rr.v2 - L.v2);
      const R A4 = RoeDens * (Rr.v3 - L.v3);
      jump[0] -= delta * (A2);
      jump[1] -= delta * (rv0 * A2);
      jump[2] -= delta * (rv1 * A2 + A3);
      jump[3] -= delta * (rv2 * A2 + A4);
      jump[4] -= delta * (R(0.5) * absVel * A2 + rv1 * A3 + rv2 * A4);
    }
    const R s = R(1) / (Ssr - Ssl);
#pragma unroll
    for (int v = 0; v < 5; ++v) F[v] = (Ssr * FL[v] - Ssl * FR[v] + Ssl * Ssr * jump[v]) * s;
  }
}

// Riemann (riemann.f90:216-289): rotate (u,v,w) into (n,t1,t2), solve, back-rotate momentum
template <typename R>
__device__ __forceinline__ void riemann_face(int riemann, int split, const R UL[5], const R UR[5], const R PL[6],
                                             const R PR[6], const R nv[3], const R t1[3], const R t2[3],
                                             const Gas<R>& gas, R Fout[5]) {
  const R kappa = gas.kappa;
  Ext<R> L, Rr;
  L.rho = UL[0]; L.srho = R(1) / L.rho; L.E = UL[4]; L.pm = PL[4]; L.p = p_abs(PL[4], gas);
  L.v1 = PL[1] * nv[0] + PL[2] * nv[1] + PL[3] * nv[2];
  L.v2 = PL[1] * t1[0] + PL[2] * t1[1] + PL[3] * t1[2];
  L.v3 = PL[1] * t2[0] + PL[2] * t2[1] + PL[3] * t2[2];
  L.m1 = L.rho * L.v1; L.m2 = L.rho * L.v2; L.m3 = L.rho * L.v3;
  Rr.rho = UR[0]; Rr.srho = R(1) / Rr.rho; Rr.E = UR[4]; Rr.pm = PR[4]; Rr.p = p_abs(PR[4], gas);
  Rr.v1 = PR[1] * nv[0] + PR[2] * nv[1] + PR[3] * nv[2];
  Rr.v2 = PR[1] * t1[0] + PR[2] * t1[1] + PR[3] * t1[2];
  Rr.v3 = PR[1] * t2[0] + PR[2] * t2[1] + PR[3] * t2[2];
  Rr.m1 = Rr.rho * Rr.v1; Rr.m2 = Rr.rho * Rr.v2; Rr.m3 = Rr.rho * Rr.v3;
  R F[5];
  riemann_solver(riemann, split, L, Rr, kappa, F);
  Fout[0] = F[0];
  Fout[1] = nv[0] * F[1] + t1[0] * F[2] + t2[0] * F[3];
  Fout[2] = nv[1] * F[1] + t1[1] * F[2] + t2[1] * F[3];
  Fout[3] = nv[2] * F[1] + t1[2] * F[2] + t2[2] * F[3];
  Fout[4] = F[4];
}

// Viscous stress tensor and (tau.v + q) rows (flux.f90:509-697): g = lifted gradients (rho,u,v,w,T)
template <typename R>
__device__ __forceinline__ void visc_stress(const R gx[5], const R gy[5], const R gz[5], const R vel[3], R mu,
                                            R lambda, R tau[6], R tq[3]) {
  const R s23 = R(2) / R(3), s43 = R(4) / R(3);
  const R txx = mu * (s43 * gx[1] - s23 * gy[2] - s23 * gz[3]);
  const R tyy = mu * (-s23 * gx[1] + s43 * gy[2] - s23 * gz[3]);
  const R tzz = mu * (-s23 * gx[1] - s23 * gy[2] + s43 * gz[3]);
  const R txy = mu * (gy[1] + gx[2]);
  const R txz = mu * (gz[1] + gx[3]);
  const R tyz = mu * (gz[2] + gy[3]);
  tq[0] = txx * vel[0] + txy * vel[1] + txz * vel[2] + lambda * gx[4];
  tq[1] = txy * vel[0] + tyy * vel[1] + tyz * vel[2] + lambda * gy[4];
  tq[2] = txz * vel[0] + tyz * vel[1] + tzz * vel[2] + lambda * gz[4];
  tau[0] = txx; tau[1] = tyy; tau[2] = tzz; tau[3] = txy; tau[4] = txz; tau[5] = tyz;
}

// EvalNormalDiffFlux3D (flux.f90:779-847): the diffusive flux projected on n (momentum + energy)
template <typename R>
__device__ __forceinline__ void normal_diff_flux(const R P[6], const R gx[5], const R gy[5], const R gz[5],
                                                 const R nv[3], R mu, R lambda, R f[5]) {
  R tau[6], tq[3];
  const R vel[3] = {P[1], P[2], P[3]};
  visc_stress(gx, gy, gz, vel, mu, lambda, tau, tq);
  f[0] = R(0);
  f[1] = -nv[0] * tau[0] - nv[1] * tau[3] - nv[2] * tau[4];
  f[2] = -nv[0] * tau[3] - nv[1] * tau[1] - nv[2] * tau[5];
  f[3] = -nv[0] * tau[4] - nv[1] * tau[5] - nv[2] * tau[2];
  f[4] = -nv[0] * tq[0] - nv[1] * tq[1] - nv[2] * tq[2];
}

}  // namespace gx
