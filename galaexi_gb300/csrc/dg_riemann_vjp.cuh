// Hand-written transposes (reverse mode) of the Riemann fluxes of dg_physics.cuh for the FP64
// adjoint: Lax-Friedrichs, Roe and Roe with entropy fix (riemann.f90:707-989), with the central part
// either the plain flux average (weak form) or the PI / KG split surface flux (splitflux.f90:270-761).
// Every line mirrors one forward line of riemann_solver / split_surface_flux / riemann_face, in
// reverse order; fmax/fabs branches are taken as the forward (and the Dual<K> path) takes them.
// The other solver / split combinations use the forward-mode Jacobian (Dual<10>) in ka_face.
#pragma once
#include "dg_physics.cuh"

namespace gx {

// Transpose of ConsToPrim (idealgas/eos.f90:212-239) at the conservative state U, given cotangents of
// rho, (u,v,w), p, T, 1/rho, and of the conservative E and momenta used directly; accumulates into Ub.
__device__ __forceinline__ void prim_vjp(const double U[5], double kappaM1, double sR, double rb, double ub,
                                         double vb, double wb, double pb, double Tb, double srhob, double Eb,
                                         double m1b, double m2b, double m3b, double Ub[5]) {
  const double srho = 1. / U[0];
  const double vel[3] = {U[1] * srho, U[2] * srho, U[3] * srho};
  const double p = kappaM1 * (U[4] - 0.5 * (U[1] * vel[0] + U[2] * vel[1] + U[3] * vel[2]));
  // T = p * srho / R
  pb += Tb * srho * sR;
  srhob += Tb * p * sR;
  // p = (kappa-1) (E - 0.5 m.v)
  Eb += kappaM1 * pb;
  const double hp = -0.5 * kappaM1 * pb;
  m1b += hp * vel[0]; m2b += hp * vel[1]; m3b += hp * vel[2];
  ub += hp * U[1]; vb += hp * U[2]; wb += hp * U[3];
  // v = m * srho
  m1b += ub * srho; m2b += vb * srho; m3b += wb * srho;
  srhob += ub * U[1] + vb * U[2] + wb * U[3];
  rb += -srhob * srho * srho;
  Ub[0] += rb; Ub[1] += m1b; Ub[2] += m2b; Ub[3] += m3b; Ub[4] += Eb;
}

struct ExtB {
  double rho, srho, m1, m2, m3, E, v1, v2, v3, p;
};

__device__ __forceinline__ bool riemann_vjp_supported(int riemann, int split) {
  return (riemann == DG_RIEMANN_LF || riemann == DG_RIEMANN_ROE || riemann == DG_RIEMANN_ROEENTROPYFIX) &&
         (split == DG_SPLIT_NONE || split == DG_SPLIT_PI || split == DG_SPLIT_KG);
}
inline bool riemann_vjp_supported_host(int riemann, int split) {
  return (riemann == DG_RIEMANN_LF || riemann == DG_RIEMANN_ROE || riemann == DG_RIEMANN_ROEENTROPYFIX) &&
         (split == DG_SPLIT_NONE || split == DG_SPLIT_PI || split == DG_SPLIT_KG);
}

__device__ __forceinline__ double sgn1(double x) { return x < 0. ? -1. : 1.; }

// central part: 0.5 (F(L) + F(R)) (EvalEulerFlux1D_fast, flux.f90:1123-1143) or a split surface flux
__device__ __forceinline__ void central_vjp(int split, const Ext<double>& L, const Ext<double>& R, const double Fb[5],
                                            ExtB& Lb, ExtB& Rb) {
  if (split < 0) {
    const Ext<double>* X[2] = {&L, &R};
    ExtB* Xb[2] = {&Lb, &Rb};
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      const Ext<double>& U = *X[s];
      ExtB& B = *Xb[s];
      const double c0 = 0.5 * Fb[0], c1 = 0.5 * Fb[1], c2 = 0.5 * Fb[2], c3 = 0.5 * Fb[3], c4 = 0.5 * Fb[4];
      B.m1 += c0 + c1 * U.v1 + c2 * U.v2 + c3 * U.v3;
      B.v1 += c1 * U.m1 + c4 * (U.E + U.p);
      B.p += c1 + c4 * U.v1;
      B.v2 += c2 * U.m1;
      B.v3 += c3 * U.m1;
      B.E += c4 * U.v1;
    }
    return;
  }
  const double rs = L.rho + R.rho, us = L.v1 + R.v1, v2s = L.v2 + R.v2, v3s = L.v3 + R.v3;
  if (split == DG_SPLIT_PI) {
    const double HL = (L.E + L.p) * L.srho, HR = (R.E + R.p) * R.srho, Hs = HL + HR;
    const double rsb = 0.25 * us * Fb[0] + 0.125 * us * us * Fb[1] + 0.125 * us * v2s * Fb[2] +
                       0.125 * us * v3s * Fb[3] + 0.125 * Hs * us * Fb[4];
    const double usb = 0.25 * rs * Fb[0] + 0.25 * rs * us * Fb[1] + 0.125 * rs * v2s * Fb[2] +
                       0.125 * rs * v3s * Fb[3] + 0.125 * rs * Hs * Fb[4];
    const double pb = 0.5 * Fb[1];
    const double v2b = 0.125 * rs * us * Fb[2], v3b = 0.125 * rs * us * Fb[3];
    const double Hb = 0.125 * rs * us * Fb[4];
    Lb.rho += rsb; Rb.rho += rsb;
    Lb.v1 += usb; Rb.v1 += usb;
    Lb.p += pb + Hb * L.srho; Rb.p += pb + Hb * R.srho;
    Lb.v2 += v2b; Rb.v2 += v2b;
    Lb.v3 += v3b; Rb.v3 += v3b;
    Lb.E += Hb * L.srho; Rb.E += Hb * R.srho;
    Lb.srho += Hb * (L.E + L.p); Rb.srho += Hb * (R.E + R.p);
  } else {  // KG
    const double eL = L.E * L.srho, eR = R.E * R.srho, es = eL + eR, ps = L.p + R.p;
    const double rsb = 0.25 * us * Fb[0] + 0.125 * us * us * Fb[1] + 0.125 * us * v2s * Fb[2] +
                       0.125 * us * v3s * Fb[3] + 0.125 * es * us * Fb[4];
    const double usb = 0.25 * rs * Fb[0] + 0.25 * rs * us * Fb[1] + 0.125 * rs * v2s * Fb[2] +
                       0.125 * rs * v3s * Fb[3] + 0.125 * rs * es * Fb[4] + 0.25 * ps * Fb[4];
    const double pb = 0.5 * Fb[1] + 0.25 * us * Fb[4];
    const double v2b = 0.125 * rs * us * Fb[2], v3b = 0.125 * rs * us * Fb[3];
    const double eb = 0.125 * rs * us * Fb[4];
    Lb.rho += rsb; Rb.rho += rsb;
    Lb.v1 += usb; Rb.v1 += usb;
    Lb.p += pb; Rb.p += pb;
    Lb.v2 += v2b; Rb.v2 += v2b;
    Lb.v3 += v3b; Rb.v3 += v3b;
    Lb.E += eb * L.srho; Rb.E += eb * R.srho;
    Lb.srho += eb * L.E; Rb.srho += eb * R.E;
  }
}

// sound speed c = sqrt(kappa p / rho) transposed
__device__ __forceinline__ void sound_vjp(const Ext<double>& X, double kappa, double c, double cb, ExtB& Xb) {
  const double h = cb * kappa / (2. * c);
  Xb.p += h * X.srho;
  Xb.srho += h * X.p;
}

// the rotated-frame solver transposed: Fb (rotated) -> Ext cotangents
__device__ __forceinline__ void riemann_solver_vjp(int riemann, int split, const Ext<double>& L, const Ext<double>& R,
                                                   double kappa, const double Fb[5], ExtB& Lb, ExtB& Rb) {
  const double km1 = kappa - 1.;
  central_vjp(split, L, R, Fb, Lb, Rb);
  const double dU[5] = {R.rho - L.rho, R.m1 - L.m1, R.m2 - L.m2, R.m3 - L.m3, R.E - L.E};
  double dUb[5] = {0, 0, 0, 0, 0};
  if (riemann == DG_RIEMANN_LF) {
    const double cL = sqrt(kappa * L.p * L.srho), cR = sqrt(kappa * R.p * R.srho);
    const double aR = fabs(R.v1), aL = fabs(L.v1);
    const double lam = (aL > aR ? aL : aR) + (cR > cL ? cR : cL);
    double lamb = 0.;
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      dUb[v] = -0.5 * lam * Fb[v];
      lamb += -0.5 * Fb[v] * dU[v];
    }
    if (aL > aR) Lb.v1 += lamb * sgn1(L.v1);
    else Rb.v1 += lamb * sgn1(R.v1);
    if (cR > cL) sound_vjp(R, kappa, cR, lamb, Rb);
    else sound_vjp(L, kappa, cL, lamb, Lb);
  } else {
    // Roe mean values
    const double HL = (L.E + L.p) * L.srho, HR = (R.E + R.p) * R.srho;
    const double qL = sqrt(L.rho), qR = sqrt(R.rho);
    const double ssq = 1. / (qL + qR);
    const double rv0 = (qR * R.v1 + qL * L.v1) * ssq;
    const double rv1 = (qR * R.v2 + qL * L.v2) * ssq;
    const double rv2 = (qR * R.v3 + qL * L.v3) * ssq;
    const double H = (qR * HR + qL * HL) * ssq;
    const double a2 = rv0 * rv0 + rv1 * rv1 + rv2 * rv2;
    const double c = sqrt(km1 * (H - 0.5 * a2));
    const double r1_1 = rv0 - c, r1_4 = H - rv0 * c, r2_1 = rv0, r2_4 = 0.5 * a2, r5_1 = rv0 + c, r5_4 = H + rv0 * c;
    double rv0b = 0., rv1b = 0., rv2b = 0., Hb = 0., cb = 0., a2b = 0.;
    // wave strengths and eigenvalue moduli
    double A[5], ev[5];
    // ROE
    double d5 = 0., X1 = 0., X2 = 0.;
    // ROEENTROPYFIX
    double cL = 0., cR = 0., RD = 0., tmp = 0., dd[5] = {0, 0, 0, 0, 0}, araw[5], al[5], ar[5], da[5];
    int pick[5];  // 0: da = 0, 1: a - al, 2: ar - a ; bit 4: entropy-fix branch
    if (riemann == DG_RIEMANN_ROE) {
      d5 = dU[4] - (dU[2] - rv1 * dU[0]) * rv1 - (dU[3] - rv2 * dU[0]) * rv2;
      A[2] = dU[2] - rv1 * dU[0];
      A[3] = dU[3] - rv2 * dU[0];
      X2 = dU[0] * (H - rv0 * rv0) - d5 + rv0 * dU[1];
      A[1] = km1 / (c * c) * X2;
      X1 = dU[0] * (rv0 + c) - dU[1] - c * A[1];
      A[0] = 0.5 / c * X1;
      A[4] = dU[0] - A[0] - A[1];
      ev[0] = fabs(rv0 - c); ev[1] = fabs(rv0); ev[2] = ev[1]; ev[3] = ev[1]; ev[4] = fabs(rv0 + c);
    } else {
      cL = sqrt(kappa * L.p * L.srho); cR = sqrt(kappa * R.p * R.srho);
      RD = sqrt(L.rho * R.rho);
      dd[0] = R.rho - L.rho; dd[1] = R.v1 - L.v1; dd[2] = R.v2 - L.v2; dd[3] = R.v3 - L.v3; dd[4] = R.p - L.p;
      tmp = 0.5 / (c * c);
      A[0] = tmp * (dd[4] - RD * c * dd[1]);
      A[1] = dd[0] - dd[4] * 2. * tmp;
      A[2] = RD * dd[2];
      A[3] = RD * dd[3];
      A[4] = tmp * (dd[4] + RD * c * dd[1]);
      araw[0] = rv0 - c; araw[1] = rv0; araw[2] = rv0; araw[3] = rv0; araw[4] = rv0 + c;
      al[0] = L.v1 - cL; al[1] = L.v1; al[2] = L.v1; al[3] = L.v1; al[4] = L.v1 + cL;
      ar[0] = R.v1 - cR; ar[1] = R.v1; ar[2] = R.v1; ar[3] = R.v1; ar[4] = R.v1 + cR;
#pragma unroll
      for (int i = 0; i < 5; ++i) {
        const double x1 = araw[i] - al[i], x2 = ar[i] - araw[i];
        const double inner = x2 > x1 ? x2 : x1;
        const int ip = x2 > x1 ? 2 : 1;
        da[i] = inner > 0. ? inner : 0.;
        pick[i] = inner > 0. ? ip : 0;
        if (fabs(araw[i]) < da[i]) {
          ev[i] = 0.5 * (araw[i] * araw[i] / da[i] + da[i]);
          pick[i] |= 16;
        } else {
          ev[i] = fabs(araw[i]);
        }
      }
    }
    const double w[5] = {A[0] * ev[0], A[1] * ev[1], A[2] * ev[2], A[3] * ev[3], A[4] * ev[4]};
    // diss = w1 r1 + w2 r2 + w5 r5 + (0, 0, w3, w4, w3 rv1 + w4 rv2);  F = central - 0.5 diss
    double db[5];
#pragma unroll
    for (int v = 0; v < 5; ++v) db[v] = -0.5 * Fb[v];
    double wb[5];
    wb[0] = db[0] + db[1] * r1_1 + db[2] * rv1 + db[3] * rv2 + db[4] * r1_4;
    wb[1] = db[0] + db[1] * r2_1 + db[2] * rv1 + db[3] * rv2 + db[4] * r2_4;
    wb[4] = db[0] + db[1] * r5_1 + db[2] * rv1 + db[3] * rv2 + db[4] * r5_4;
    wb[2] = db[2] + db[4] * rv1;
    wb[3] = db[3] + db[4] * rv2;
    rv1b += db[2] * (w[0] + w[1] + w[4]) + db[4] * w[2];
    rv2b += db[3] * (w[0] + w[1] + w[4]) + db[4] * w[3];
    {
      const double r11b = db[1] * w[0], r14b = db[4] * w[0];
      const double r21b = db[1] * w[1], r24b = db[4] * w[1];
      const double r51b = db[1] * w[4], r54b = db[4] * w[4];
      rv0b += r11b; cb -= r11b;
      Hb += r14b; rv0b -= r14b * c; cb -= r14b * rv0;
      rv0b += r21b;
      a2b += 0.5 * r24b;
      rv0b += r51b; cb += r51b;
      Hb += r54b; rv0b += r54b * c; cb += r54b * rv0;
    }
    double Ab[5], evb[5];
#pragma unroll
    for (int i = 0; i < 5; ++i) { Ab[i] = wb[i] * ev[i]; evb[i] = wb[i] * A[i]; }
    if (riemann == DG_RIEMANN_ROE) {
      // ev = |rv0 - c|, |rv0| (x3), |rv0 + c|
      const double s1 = sgn1(rv0 - c), s2 = sgn1(rv0), s5 = sgn1(rv0 + c);
      rv0b += evb[0] * s1; cb -= evb[0] * s1;
      rv0b += (evb[1] + evb[2] + evb[3]) * s2;
      rv0b += evb[4] * s5; cb += evb[4] * s5;
      // A5 = dU0 - A1 - A2
      dUb[0] += Ab[4]; Ab[0] -= Ab[4]; Ab[1] -= Ab[4];
      // A1 = 0.5/c X1,  X1 = dU0 (rv0 + c) - dU1 - c A2
      const double X1b = Ab[0] * 0.5 / c;
      cb -= Ab[0] * A[0] / c;
      dUb[0] += X1b * (rv0 + c); rv0b += X1b * dU[0]; cb += X1b * dU[0]; dUb[1] -= X1b; cb -= X1b * A[1];
      Ab[1] -= X1b * c;
      // A2 = km1/c^2 X2,  X2 = dU0 (H - rv0^2) - d5 + rv0 dU1
      const double X2b = Ab[1] * km1 / (c * c);
      cb -= 2. * Ab[1] * A[1] / c;
      dUb[0] += X2b * (H - rv0 * rv0); Hb += X2b * dU[0]; rv0b += X2b * (-2. * rv0 * dU[0] + dU[1]);
      const double d5b = -X2b;
      dUb[1] += X2b * rv0;
      // A3, A4
      dUb[2] += Ab[2]; rv1b -= Ab[2] * dU[0]; dUb[0] -= Ab[2] * rv1;
      dUb[3] += Ab[3]; rv2b -= Ab[3] * dU[0]; dUb[0] -= Ab[3] * rv2;
      // d5 = dU4 - y1 rv1 - y2 rv2
      dUb[4] += d5b;
      const double y1 = dU[2] - rv1 * dU[0], y2 = dU[3] - rv2 * dU[0];
      const double y1b = -d5b * rv1, y2b = -d5b * rv2;
      rv1b -= d5b * y1; rv2b -= d5b * y2;
      dUb[2] += y1b; rv1b -= y1b * dU[0]; dUb[0] -= y1b * rv1;
      dUb[3] += y2b; rv2b -= y2b * dU[0]; dUb[0] -= y2b * rv2;
    } else {
      // entropy-fixed eigenvalues
      double arb[5] = {0, 0, 0, 0, 0}, alb[5] = {0, 0, 0, 0, 0}, arrb[5] = {0, 0, 0, 0, 0};
#pragma unroll
      for (int i = 0; i < 5; ++i) {
        double dab = 0.;
        if (pick[i] & 16) {
          arb[i] += evb[i] * araw[i] / da[i];
          dab += evb[i] * 0.5 * (1. - araw[i] * araw[i] / (da[i] * da[i]));
        } else {
          arb[i] += evb[i] * sgn1(araw[i]);
        }
        const int ip = pick[i] & 3;
        if (ip == 1) { arb[i] += dab; alb[i] -= dab; }
        else if (ip == 2) { arrb[i] += dab; arb[i] -= dab; }
      }
      // araw = rv0 -+ c, rv0 ; al = v1L -+ cL ; ar = v1R -+ cR
      rv0b += arb[0] + arb[1] + arb[2] + arb[3] + arb[4];
      cb += -arb[0] + arb[4];
      Lb.v1 += alb[0] + alb[1] + alb[2] + alb[3] + alb[4];
      const double cLb = -alb[0] + alb[4];
      Rb.v1 += arrb[0] + arrb[1] + arrb[2] + arrb[3] + arrb[4];
      const double cRb = -arrb[0] + arrb[4];
      // A from the primitive jumps
      const double x = RD * c * dd[1];
      double tmpb = Ab[0] * (dd[4] - x) + Ab[4] * (dd[4] + x) - 2. * Ab[1] * dd[4];
      double ddb[5];
      ddb[4] = (Ab[0] + Ab[4]) * tmp - 2. * Ab[1] * tmp;
      const double xb = tmp * (Ab[4] - Ab[0]);
      double RDb = xb * c * dd[1] + Ab[2] * dd[2] + Ab[3] * dd[3];
      cb += xb * RD * dd[1];
      ddb[1] = xb * RD * c;
      ddb[0] = Ab[1];
      ddb[2] = Ab[2] * RD;
      ddb[3] = Ab[3] * RD;
      cb += tmpb * (-2. * tmp / c);
      // RD = sqrt(rhoL rhoR)
      Lb.rho += RDb * R.rho / (2. * RD);
      Rb.rho += RDb * L.rho / (2. * RD);
      Rb.rho += ddb[0]; Lb.rho -= ddb[0];
      Rb.v1 += ddb[1]; Lb.v1 -= ddb[1];
      Rb.v2 += ddb[2]; Lb.v2 -= ddb[2];
      Rb.v3 += ddb[3]; Lb.v3 -= ddb[3];
      Rb.p += ddb[4]; Lb.p -= ddb[4];
      sound_vjp(L, kappa, cL, cLb, Lb);
      sound_vjp(R, kappa, cR, cRb, Rb);
    }
    // c = sqrt(km1 (H - a2/2))
    const double zb = cb / (2. * c);
    Hb += zb * km1;
    a2b -= 0.5 * zb * km1;
    rv0b += 2. * a2b * rv0; rv1b += 2. * a2b * rv1; rv2b += 2. * a2b * rv2;
    // Roe averages
    double qLb = 0., qRb = 0., ssqb = 0.;
    const double HRb = Hb * qR * ssq, HLb = Hb * qL * ssq;
    qRb += Hb * HR * ssq; qLb += Hb * HL * ssq; ssqb += Hb * (qR * HR + qL * HL);
    Rb.v1 += rv0b * qR * ssq; Lb.v1 += rv0b * qL * ssq;
    qRb += rv0b * R.v1 * ssq; qLb += rv0b * L.v1 * ssq; ssqb += rv0b * (qR * R.v1 + qL * L.v1);
    Rb.v2 += rv1b * qR * ssq; Lb.v2 += rv1b * qL * ssq;
    qRb += rv1b * R.v2 * ssq; qLb += rv1b * L.v2 * ssq; ssqb += rv1b * (qR * R.v2 + qL * L.v2);
    Rb.v3 += rv2b * qR * ssq; Lb.v3 += rv2b * qL * ssq;
    qRb += rv2b * R.v3 * ssq; qLb += rv2b * L.v3 * ssq; ssqb += rv2b * (qR * R.v3 + qL * L.v3);
    qLb -= ssqb * ssq * ssq; qRb -= ssqb * ssq * ssq;
    Lb.rho += qLb / (2. * qL); Rb.rho += qRb / (2. * qR);
    Lb.E += HLb * L.srho; Lb.p += HLb * L.srho; Lb.srho += HLb * (L.E + L.p);
    Rb.E += HRb * R.srho; Rb.p += HRb * R.srho; Rb.srho += HRb * (R.E + R.p);
  }
  // dU = R - L over (rho, m1, m2, m3, E)
  Rb.rho += dUb[0]; Lb.rho -= dUb[0];
  Rb.m1 += dUb[1]; Lb.m1 -= dUb[1];
  Rb.m2 += dUb[2]; Lb.m2 -= dUb[2];
  Rb.m3 += dUb[3]; Lb.m3 -= dUb[3];
  Rb.E += dUb[4]; Lb.E -= dUb[4];
}

// Ext state of one side (riemann_face) and its transpose back to the conservative face state
__device__ __forceinline__ void make_ext(const double U[5], const double nv[3], const double t1[3], const double t2[3],
                                         double kappaM1, Ext<double>& X) {
  const double sr = 1. / U[0];
  const double u = U[1] * sr, v = U[2] * sr, w = U[3] * sr;
  X.rho = U[0];
  X.srho = 1. / X.rho;
  X.E = U[4];
  X.p = kappaM1 * (U[4] - 0.5 * (U[1] * u + U[2] * v + U[3] * w));
  X.pm = X.p;
  X.v1 = u * nv[0] + v * nv[1] + w * nv[2];
  X.v2 = u * t1[0] + v * t1[1] + w * t1[2];
  X.v3 = u * t2[0] + v * t2[1] + w * t2[2];
  X.m1 = X.rho * X.v1; X.m2 = X.rho * X.v2; X.m3 = X.rho * X.v3;
}

__device__ __forceinline__ void ext_vjp(const double U[5], const Ext<double>& X, ExtB& B, const double nv[3],
                                        const double t1[3], const double t2[3], double kappaM1, double sR, double Ub[5]) {
  B.v1 += B.m1 * X.rho; B.v2 += B.m2 * X.rho; B.v3 += B.m3 * X.rho;
  B.rho += B.m1 * X.v1 + B.m2 * X.v2 + B.m3 * X.v3;
  const double ub = nv[0] * B.v1 + t1[0] * B.v2 + t2[0] * B.v3;
  const double vb = nv[1] * B.v1 + t1[1] * B.v2 + t2[1] * B.v3;
  const double wb = nv[2] * B.v1 + t1[2] * B.v2 + t2[2] * B.v3;
  B.rho += -B.srho * X.srho * X.srho;
  prim_vjp(U, kappaM1, sR, B.rho, ub, vb, wb, B.p, 0., 0., B.E, 0., 0., 0., Ub);
}

}  // namespace gx
