// ============================================================================================
// TEST INFRASTRUCTURE -- the oracle.
//
// A plain C++ restatement, on the CPU, of GALAEXI's DGSEM right-hand side
// (DGTimeDerivative_weakForm) and its low-storage RK stepper.  It exists only to check
// the CUDA path: the tests, the smoke check and bench.py's CPU-baseline leg call it; the
// product never does.  Every routine follows the reference routine named beside it, in
// the reference's loop and summation order (the GPU kernels of GALAEXI, thread-per-DOF /
// thread-per-face-node, executed here as plain loops).  Paths are relative to the
// reference project root.
//
// Parity pins: the basis routines are checked against unitTests/NodesAndWeights.bin and
// unitTests/DerivativeMatrix.bin, the host ProlongToFace / SurfInt restatements against
// unitTests/ProlongToFace_*3D.bin and unitTests/SurfInt_*3D.bin (tests/test_oracle_golden.py).
// The Riemann solvers, split fluxes, lifting and the RK stepper have no golden vectors in
// the reference; for them this restatement follows the formulas line by line.
//
// Array layouts are the reference's Fortran (column-major) layouts with 0-based C indices.
// ============================================================================================
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>
#include <algorithm>
#include <omp.h>

#include "../include/galaexi_gb300.h"

namespace orc {

// ---------------------------------------------------------------------------------------
// flexi.h side flags (src/flexi.h:98-115)
// ---------------------------------------------------------------------------------------
enum { ZETA_MINUS = 1, ETA_MINUS = 2, XI_PLUS = 3, ETA_PLUS = 4, XI_MINUS = 5, ZETA_PLUS = 6 };
static const double PP_Pi = 3.141592653589793238462643383279502884197;
static const double PP_RealTolerance = 2.220446049250313e-16;  // EPSILON(1.0_8)
static inline double sq(double x) { return x * x; }  // Fortran x**2

// ---------------------------------------------------------------------------------------
// Basis: src/interpolation/basis.f90
// ---------------------------------------------------------------------------------------
// LegendrePolynomialAndDerivative  basis.f90:195-234 (normalised Legendre polynomials)
static void LegendrePolynomialAndDerivative(int N_in, double x, double& L, double& Lder) {
  if (N_in == 0) { L = 1.; Lder = 0.; }
  else if (N_in == 1) { L = x; Lder = 1.; }
  else {
    double L_Nm2 = 1., L_Nm1 = x, Lder_Nm2 = 0., Lder_Nm1 = 1.;
    for (int iL = 2; iL <= N_in; ++iL) {
      L = ((double)(2 * iL - 1) * x * L_Nm1 - (double)(iL - 1) * L_Nm2) / (double)iL;
      Lder = iL * L_Nm1 + x * Lder_Nm1;
      L_Nm2 = L_Nm1; L_Nm1 = L; Lder_Nm2 = Lder_Nm1; Lder_Nm1 = Lder;
    }
  }
  L = L * std::sqrt((double)N_in + 0.5);
  Lder = Lder * std::sqrt((double)N_in + 0.5);
}

// LegendreGaussNodesAndWeights  basis.f90:417-486
static void LegendreGaussNodesAndWeights(int N_in, double* xGP, double* wGP) {
  const int nIter = 10;
  const double Tol = 1.e-15;
  if (N_in == 0) { xGP[0] = 0.; if (wGP) wGP[0] = 2.; return; }
  if (N_in == 1) {
    xGP[0] = -std::sqrt(1. / 3.); xGP[N_in] = -xGP[0];
    if (wGP) { wGP[0] = 1.; wGP[1] = 1.; }
    return;
  }
  double cheb_tmp = 2. * std::atan(1.) / (double)(N_in + 1);
  for (int iGP = 0; iGP <= (N_in + 1) / 2 - 1; ++iGP) {
    xGP[iGP] = -std::cos(cheb_tmp * (double)(2 * iGP + 1));
    double L, Lder;
    for (int iter = 0; iter <= nIter; ++iter) {
      LegendrePolynomialAndDerivative(N_in + 1, xGP[iGP], L, Lder);
      double dx = -L / Lder;
      xGP[iGP] = xGP[iGP] + dx;
      if (std::fabs(dx) < Tol * std::fabs(xGP[iGP])) break;
    }
    LegendrePolynomialAndDerivative(N_in + 1, xGP[iGP], L, Lder);
    xGP[N_in - iGP] = -xGP[iGP];
    if (wGP) {
      wGP[iGP] = (2. * N_in + 3) / ((1. - xGP[iGP] * xGP[iGP]) * Lder * Lder);
      wGP[N_in - iGP] = wGP[iGP];
    }
  }
  if (N_in % 2 == 0) {
    double L, Lder;
    xGP[N_in / 2] = 0.;
    LegendrePolynomialAndDerivative(N_in + 1, xGP[N_in / 2], L, Lder);
    if (wGP) wGP[N_in / 2] = (2. * N_in + 3) / (Lder * Lder);
  }
}

// qAndLEvaluation  basis.f90:527-556
static void qAndLEvaluation(int N_in, double x, double& q, double& qder, double& L) {
  double L_Nm2 = 1., L_Nm1 = x;
  L = x;
  for (int iL = 2; iL <= N_in; ++iL) {
    L = ((double)(2 * iL - 1) * x * L_Nm1 - (double)(iL - 1) * L_Nm2) / (double)iL;
    L_Nm2 = L_Nm1; L_Nm1 = L;
  }
  q = (double)(2 * N_in + 1) / (double)(N_in + 1) * (x * L - L_Nm2);
  qder = (double)(2 * N_in + 1) * L;
}

// LegGaussLobNodesAndWeights  basis.f90:567-630
static void LegGaussLobNodesAndWeights(int N_in, double* xGP, double* wGP) {
  const int nIter = 10;
  const double Tol = 1.e-15;
  xGP[0] = -1.; xGP[N_in] = 1.;
  double w0 = 2. / (double)(N_in * (N_in + 1));
  if (wGP) { wGP[0] = w0; wGP[N_in] = w0; }
  if (N_in > 1) {
    double cont1 = PP_Pi / (double)N_in;
    double cont2 = 3. / ((double)(8 * N_in) * PP_Pi);
    for (int iGP = 1; iGP <= (N_in + 1) / 2 - 1; ++iGP) {
      xGP[iGP] = -std::cos(cont1 * ((double)iGP + 0.25) - cont2 / ((double)iGP + 0.25));
      double q, qder, L;
      for (int iter = 0; iter <= nIter; ++iter) {
        qAndLEvaluation(N_in, xGP[iGP], q, qder, L);
        double dx = -q / qder;
        xGP[iGP] = xGP[iGP] + dx;
        if (std::fabs(dx) < Tol * std::fabs(xGP[iGP])) break;
      }
      qAndLEvaluation(N_in, xGP[iGP], q, qder, L);
      xGP[N_in - iGP] = -xGP[iGP];
      if (wGP) { wGP[iGP] = w0 / (L * L); wGP[N_in - iGP] = wGP[iGP]; }
    }
  }
  if (N_in % 2 == 0) {
    double q, qder, L;
    xGP[N_in / 2] = 0.;
    qAndLEvaluation(N_in, xGP[N_in / 2], q, qder, L);
    if (wGP) wGP[N_in / 2] = w0 / (L * L);
  }
}

// ChebyGaussLobNodesAndWeights  basis.f90:269-291
static void ChebyGaussLobNodesAndWeights(int N_in, double* xGP, double* wGP) {
  for (int i = 0; i <= N_in; ++i) xGP[i] = -std::cos(i / (double)N_in * PP_Pi);
  if (wGP) {
    for (int i = 0; i <= N_in; ++i) wGP[i] = PP_Pi / (double)N_in;
    wGP[0] *= 0.5; wGP[N_in] *= 0.5;
  }
}

// BarycentricWeights  basis.f90:638-655
static void BarycentricWeights(int N_in, const double* xGP, double* wBary) {
  for (int i = 0; i <= N_in; ++i) wBary[i] = 1.;
  for (int i = 1; i <= N_in; ++i)
    for (int j = 0; j <= i - 1; ++j) {
      wBary[j] = wBary[j] * (xGP[j] - xGP[i]);
      wBary[i] = wBary[i] * (xGP[i] - xGP[j]);
    }
  for (int i = 0; i <= N_in; ++i) wBary[i] = 1. / wBary[i];
}

// PolynomialDerivativeMatrix  basis.f90:664-690  (D(iGP,iLagrange), column-major)
static void PolynomialDerivativeMatrix(int N_in, const double* xGP, double* D) {
  const int n = N_in + 1;
  std::vector<double> wBary(n);
  BarycentricWeights(N_in, xGP, wBary.data());
  for (int i = 0; i < n * n; ++i) D[i] = 0.;
  for (int iL = 0; iL <= N_in; ++iL)
    for (int iGP = 0; iGP <= N_in; ++iGP)
      if (iL != iGP) {
        D[iGP + n * iL] = wBary[iL] / (wBary[iGP] * (xGP[iGP] - xGP[iL]));
        D[iGP + n * iGP] = D[iGP + n * iGP] - D[iGP + n * iL];
      }
}

// ALMOSTEQUAL  basis.f90:700-715
static bool AlmostEqual(double x, double y) {
  if (x == 0. || y == 0.) return std::fabs(x - y) <= 2. * PP_RealTolerance;
  return (std::fabs(x - y) <= PP_RealTolerance * std::fabs(x)) &&
         (std::fabs(x - y) <= PP_RealTolerance * std::fabs(y));
}

// LagrangeInterpolationPolys  basis.f90:720-752
static void LagrangeInterpolationPolys(double x, int N_in, const double* xGP, const double* wBary,
                                       double* L) {
  bool xEqualGP = false;
  for (int i = 0; i <= N_in; ++i) {
    L[i] = 0.;
    if (AlmostEqual(x, xGP[i])) { L[i] = 1.; xEqualGP = true; }
  }
  if (xEqualGP) return;
  double DummySum = 0.;
  for (int i = 0; i <= N_in; ++i) { L[i] = wBary[i] / (x - xGP[i]); DummySum += L[i]; }
  for (int i = 0; i <= N_in; ++i) L[i] = L[i] / DummySum;
}

// GetNodesAndWeights  src/interpolation/interpolation.f90:199-318
// node types: 1 Gauss, 2 Gauss-Lobatto, 3 Chebyshev-Gauss-Lobatto, 4 visu (equidistant)
static void GetNodesAndWeights(int N_in, int node_type, double* x, double* w, double* wBary) {
  std::vector<double> wl(N_in + 1);
  double* ww = w ? w : wl.data();
  switch (node_type) {
    case 1: LegendreGaussNodesAndWeights(N_in, x, ww); break;
    case 2: LegGaussLobNodesAndWeights(N_in, x, ww); break;
    case 3: ChebyGaussLobNodesAndWeights(N_in, x, ww); break;
    case 4:
      for (int i = 0; i <= N_in; ++i) x[i] = 2. * (double)i / (double)N_in - 1.;
      for (int i = 0; i <= N_in; ++i) ww[i] = 2. / (double)N_in;
      ww[0] *= 0.5; ww[N_in] *= 0.5;
      break;
  }
  if (wBary) BarycentricWeights(N_in, x, wBary);
}

struct Basis {
  int N, n, node_type;
  std::vector<double> xGP, wGP, wBary, L_Minus, L_Plus;
  std::vector<double> D, D_T, D_Hat, D_Hat_T, L_HatMinus, L_HatPlus, DVolSurf;
  double d(int i, int j) const { return D[i + n * j]; }
};

// InitInterpolationBasis (interpolation.f90:161-193) + InitDGbasis (src/dg/dg.f90:181-242)
static void build_basis(int N, int node_type, Basis& B) {
  B.N = N; B.n = N + 1; B.node_type = node_type;
  const int n = N + 1;
  B.xGP.assign(n, 0.); B.wGP.assign(n, 0.); B.wBary.assign(n, 0.);
  B.L_Minus.assign(n, 0.); B.L_Plus.assign(n, 0.);
  GetNodesAndWeights(N, node_type, B.xGP.data(), B.wGP.data(), B.wBary.data());
  LagrangeInterpolationPolys(1., N, B.xGP.data(), B.wBary.data(), B.L_Plus.data());
  LagrangeInterpolationPolys(-1., N, B.xGP.data(), B.wBary.data(), B.L_Minus.data());
  B.D.assign(n * n, 0.); B.D_T.assign(n * n, 0.);
  PolynomialDerivativeMatrix(N, B.xGP.data(), B.D.data());
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) B.D_T[i + n * j] = B.D[j + n * i];
  // PolynomialMassMatrix (basis.f90:761-807) without EXACT_MM: M=diag(w), Minv=diag(1/w)
  std::vector<double> Minv(n);
  for (int i = 0; i < n; ++i) Minv[i] = 1. / B.wGP[i];
  // D_Hat = -MATMUL(Minv, MATMUL(TRANSPOSE(D), M))  (dg.f90:222)
  B.D_Hat.assign(n * n, 0.); B.D_Hat_T.assign(n * n, 0.);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      // (D^T M)(i,j) = D(j,i) * w(j) ; (Minv * .)(i,j) = Minv(i) * D(j,i) * w(j)
      double dtm = B.D[j + n * i] * B.wGP[j];
      B.D_Hat[i + n * j] = -(Minv[i] * dtm);
    }
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) B.D_Hat_T[i + n * j] = B.D_Hat[j + n * i];
  // DVolSurf (dg.f90:228-234)
  B.DVolSurf = B.D_T;
  B.DVolSurf[0] = B.DVolSurf[0] + 1.0 / (2.0 * B.wGP[0]);
  B.DVolSurf[N + n * N] = B.DVolSurf[N + n * N] - 1.0 / (2.0 * B.wGP[N]);
  // L_HatPlus = MATMUL(Minv, L_Plus) (dg.f90:240-241)
  B.L_HatPlus.assign(n, 0.); B.L_HatMinus.assign(n, 0.);
  for (int i = 0; i < n; ++i) {
    B.L_HatPlus[i] = Minv[i] * B.L_Plus[i];
    B.L_HatMinus[i] = Minv[i] * B.L_Minus[i];
  }
}

// ---------------------------------------------------------------------------------------
// Mappings: src/mesh/mappings.f90
// ---------------------------------------------------------------------------------------
// Flip_S2M  mappings.f90:248-272
static void Flip_S2M(int N, int p, int q, int flip, int& a, int& b) {
  switch (flip) {
    case 0: a = p; b = q; break;
    case 1: a = q; b = p; break;
    case 2: a = N - p; b = q; break;
    case 3: a = N - q; b = N - p; break;
    default: a = p; b = N - q; break;
  }
}
// CGNS_SideToVol2  mappings.f90:376-409
static void CGNS_SideToVol2(int N, int p, int q, int locSide, int& a, int& b) {
  switch (locSide) {
    case XI_MINUS: a = q; b = p; break;
    case XI_PLUS: a = p; b = q; break;
    case ETA_MINUS: a = p; b = q; break;
    case ETA_PLUS: a = N - p; b = q; break;
    case ZETA_MINUS: a = q; b = p; break;
    default: a = p; b = q; break;  // ZETA_PLUS
  }
}
// SideToVol2 = CGNS_SideToVol2(Flip_M2S(p,q))  mappings.f90:460-478
static void SideToVol2(int N, int p, int q, int flip, int locSide, int& a, int& b) {
  int pp, qq;
  Flip_S2M(N, p, q, flip, pp, qq);  // Flip_M2S == Flip_S2M
  CGNS_SideToVol2(N, pp, qq, locSide, a, b);
}

// ---------------------------------------------------------------------------------------
// Mesh / operator context
// ---------------------------------------------------------------------------------------
struct Mesh {
  int nElems, nSides;
  const double *Mf, *Mg, *Mh, *sJ, *nv, *t1, *t2, *SurfElem;
  const int *E2S, *S2E;
};

struct Ctx {
  dg_config cfg;
  Basis B;
  Mesh M;
  int n, n2, n3;
  // S2V2(2,0:N,0:N,0:4,1:6)
  std::vector<int> S2V2, S2V2_inv;
  int s2v2(int c, int p, int q, int flip, int locSide) const {
    return S2V2[c + 2 * (p + n * (q + n * (flip + 5 * (locSide - 1))))];
  }
  int s2v2_inv(int c, int a, int b, int flip, int locSide) const {
    return S2V2_inv[c + 2 * (a + n * (b + n * (flip + 5 * (locSide - 1))))];
  }
  // solution filter (InitFilter, filter.f90:100-222): FilterMat(i,l) column-major, LAF weights/normMod
  std::vector<double> FilterMat, IntegrationWeight;
  double normMod = 0.;
  // boundary sides 0..nBCSides-1 (InitBC, getboundaryflux.f90:87-256): type, 0-based RefState index,
  // RefStatePrim (rho, u, v, w, p, T) per state
  int nBCSides = 0;
  std::vector<int> bctype, bcstate;
  std::vector<double> refprim;
  // index helpers (0-based element / side)
  size_t vol(int i, int j, int k, int e) const { return (size_t)i + n * (j + n * (k + (size_t)n * e)); }
  size_t fac(int p, int q, int s) const { return (size_t)p + n * (q + (size_t)n * s); }
  int e2s(int c, int loc, int e) const { return M.E2S[c + 3 * ((loc - 1) + 6 * e)]; }  // 1-based loc
  int s2e(int c, int s) const { return M.S2E[c + 5 * s]; }
};

static void build_s2v2(Ctx& C) {
  const int N = C.B.N, n = N + 1;
  C.S2V2.assign(2 * n * n * 5 * 6, 0);
  for (int l = 1; l <= 6; ++l)
    for (int f = 0; f <= 4; ++f)
      for (int q = 0; q <= N; ++q)
        for (int p = 0; p <= N; ++p) {
          int a, b;
          SideToVol2(N, p, q, f, l, a, b);
          C.S2V2[0 + 2 * (p + n * (q + n * (f + 5 * (l - 1))))] = a;
          C.S2V2[1 + 2 * (p + n * (q + n * (f + 5 * (l - 1))))] = b;
        }
  // S2V2_inv  mappings.f90:165-177
  C.S2V2_inv.assign(C.S2V2.size(), -1);
  for (int l = 1; l <= 6; ++l)
    for (int f = 0; f <= 4; ++f)
      for (int q = 0; q <= N; ++q)
        for (int p = 0; p <= N; ++p) {
          int a = C.s2v2(0, p, q, f, l), b = C.s2v2(1, p, q, f, l);
          C.S2V2_inv[0 + 2 * (a + n * (b + n * (f + 5 * (l - 1))))] = p;
          C.S2V2_inv[1 + 2 * (a + n * (b + n * (f + 5 * (l - 1))))] = q;
        }
}

// ---------------------------------------------------------------------------------------
// Equation of state and fluxes: src/equations/navierstokes
// ---------------------------------------------------------------------------------------
enum { DENS = 0, MOM1 = 1, MOM2 = 2, MOM3 = 3, ENER = 4 };              // cons
enum { VEL1 = 1, VEL2 = 2, VEL3 = 3, PRES = 4, TEMP = 5 };              // prim
// extended state U_LL(1:11) of eos.h:115-131, 0-based
enum { EXT_DENS = 0, EXT_MOM1 = 1, EXT_MOM2 = 2, EXT_MOM3 = 3, EXT_ENER = 4, EXT_SRHO = 5,
       EXT_VEL1 = 6, EXT_VEL2 = 7, EXT_VEL3 = 8, EXT_PRES = 9, EXT_TEMP = 10 };
static const int PRIM_LIFT[5] = {0, 1, 2, 3, 5};  // eos.h:143 (/1,2,3,4,6/)

// ConsToPrim  idealgas/eos.f90:212-239
static inline void ConsToPrim(double* prim, const double* cons, double Kappa, double R) {
  double sRho = 1. / cons[DENS];
  prim[DENS] = cons[DENS];
  prim[VEL1] = cons[MOM1] * sRho;
  prim[VEL2] = cons[MOM2] * sRho;
  prim[VEL3] = cons[MOM3] * sRho;
  prim[PRES] = (Kappa - 1.) * (cons[ENER] - 0.5 * (cons[MOM1] * prim[VEL1] + cons[MOM2] * prim[VEL2] +
                                                   cons[MOM3] * prim[VEL3]));
  prim[TEMP] = prim[PRES] * sRho / R;
}

// EvalEulerFlux1D_fast  flux.f90:1123-1143
static inline void EvalEulerFlux1D_fast(const double* U, double* F) {
  F[DENS] = U[EXT_MOM1];
  F[MOM1] = U[EXT_MOM1] * U[EXT_VEL1] + U[EXT_PRES];
  F[MOM2] = U[EXT_MOM1] * U[EXT_VEL2];
  F[MOM3] = U[EXT_MOM1] * U[EXT_VEL3];
  F[ENER] = (U[EXT_ENER] + U[EXT_PRES]) * U[EXT_VEL1];
}

// ---- split fluxes: splitflux.f90 ----
// Flux = 0.5*(MRef1+M1)*f + 0.5*(MRef3+M3)*h + 0.5*(MRef2+M2)*g   (order of the reference)
static inline void combine(const double* MRef, const double* M, const double* f, const double* g,
                           const double* h, double* Flux) {
  for (int v = 0; v < 5; ++v)
    Flux[v] = 0.5 * (MRef[0] + M[0]) * f[v] + 0.5 * (MRef[2] + M[2]) * h[v] + 0.5 * (MRef[1] + M[1]) * g[v];
}
// SplitVolumeFluxSD  splitflux.f90:145-206
static void SplitVolumeFluxSD(const double* UR, const double* PR, const double* U, const double* P,
                              const double* MRef, const double* M, double* Flux) {
  double f[5], g[5], h[5];
  double rhoEpRef = UR[ENER] + PR[PRES], rhoEp = U[ENER] + P[PRES];
  f[DENS] = (UR[MOM1] + U[MOM1]);
  f[MOM1] = (UR[MOM1] * PR[VEL1] + PR[PRES] + U[MOM1] * P[VEL1] + P[PRES]);
  f[MOM2] = (UR[MOM1] * PR[VEL2] + U[MOM1] * P[VEL2]);
  f[MOM3] = (UR[MOM1] * PR[VEL3] + U[MOM1] * P[VEL3]);
  f[ENER] = (rhoEpRef * PR[VEL1] + rhoEp * P[VEL1]);
  g[DENS] = (UR[MOM2] + U[MOM2]);
  g[MOM1] = (UR[MOM1] * PR[VEL2] + U[MOM1] * P[VEL2]);
  g[MOM2] = (UR[MOM2] * PR[VEL2] + PR[PRES] + U[MOM2] * P[VEL2] + P[PRES]);
  g[MOM3] = (UR[MOM2] * PR[VEL3] + U[MOM2] * P[VEL3]);
  g[ENER] = (rhoEpRef * PR[VEL2] + rhoEp * P[VEL2]);
  h[DENS] = (UR[MOM3] + U[MOM3]);
  h[MOM1] = (UR[MOM1] * PR[VEL3] + U[MOM1] * P[VEL3]);
  h[MOM2] = (UR[MOM2] * PR[VEL3] + U[MOM2] * P[VEL3]);
  h[MOM3] = (UR[MOM3] * PR[VEL3] + PR[PRES] + U[MOM3] * P[VEL3] + P[PRES]);
  h[ENER] = (rhoEpRef * PR[VEL3] + rhoEp * P[VEL3]);
  combine(MRef, M, f, g, h, Flux);
}
// SplitVolumeFluxDU  splitflux.f90:313-380
static void SplitVolumeFluxDU(const double* UR, const double* PR, const double* U, const double* P,
                              const double* MRef, const double* M, double* Flux) {
  double f[5], g[5], h[5];
  f[DENS] = 0.5 * (UR[DENS] + U[DENS]) * (PR[VEL1] + P[VEL1]);
  f[MOM1] = 0.5 * (UR[MOM1] + U[MOM1]) * (PR[VEL1] + P[VEL1]) + (PR[PRES] + P[PRES]);
  f[MOM2] = 0.5 * (UR[MOM2] + U[MOM2]) * (PR[VEL1] + P[VEL1]);
  f[MOM3] = 0.5 * (UR[MOM3] + U[MOM3]) * (PR[VEL1] + P[VEL1]);
  f[ENER] = 0.5 * (UR[ENER] + U[ENER] + PR[PRES] + P[PRES]) * (PR[VEL1] + P[VEL1]);
  g[DENS] = 0.5 * (UR[DENS] + U[DENS]) * (PR[VEL2] + P[VEL2]);
  g[MOM1] = 0.5 * (UR[MOM1] + U[MOM1]) * (PR[VEL2] + P[VEL2]);
  g[MOM2] = 0.5 * (UR[MOM2] + U[MOM2]) * (PR[VEL2] + P[VEL2]) + (PR[PRES] + P[PRES]);
  g[MOM3] = 0.5 * (UR[MOM3] + U[MOM3]) * (PR[VEL2] + P[VEL2]);
  g[ENER] = 0.5 * (UR[ENER] + U[ENER] + PR[PRES] + P[PRES]) * (PR[VEL2] + P[VEL2]);
  h[DENS] = 0.5 * (UR[DENS] + U[DENS]) * (PR[VEL3] + P[VEL3]);
  h[MOM1] = 0.5 * (UR[MOM1] + U[MOM1]) * (PR[VEL3] + P[VEL3]);
  h[MOM2] = 0.5 * (UR[MOM2] + U[MOM2]) * (PR[VEL3] + P[VEL3]);
  h[MOM3] = 0.5 * (UR[MOM3] + U[MOM3]) * (PR[VEL3] + P[VEL3]) + (PR[PRES] + P[PRES]);
  h[ENER] = 0.5 * (UR[ENER] + U[ENER] + PR[PRES] + P[PRES]) * (PR[VEL3] + P[VEL3]);
  combine(MRef, M, f, g, h, Flux);
}
// SplitVolumeFluxKG  splitflux.f90:416-488
static void SplitVolumeFluxKG(const double* UR, const double* PR, const double* U, const double* P,
                              const double* MRef, const double* M, double* Flux) {
  double f[5], g[5], h[5];
  double ERef = UR[ENER] / UR[DENS], E = U[ENER] / U[DENS];
  f[DENS] = 0.5 * (UR[DENS] + U[DENS]) * (PR[VEL1] + P[VEL1]);
  f[MOM1] = 0.25 * (UR[DENS] + U[DENS]) * sq(PR[VEL1] + P[VEL1]) + (PR[PRES] + P[PRES]);
  f[MOM2] = 0.25 * (UR[DENS] + U[DENS]) * (PR[VEL1] + P[VEL1]) * (PR[VEL2] + P[VEL2]);
  f[MOM3] = 0.25 * (UR[DENS] + U[DENS]) * (PR[VEL1] + P[VEL1]) * (PR[VEL3] + P[VEL3]);
  f[ENER] = 0.25 * (UR[DENS] + U[DENS]) * (PR[VEL1] + P[VEL1]) * (ERef + E) +
            0.5 * (PR[PRES] + P[PRES]) * (PR[VEL1] + P[VEL1]);
  g[DENS] = 0.5 * (UR[DENS] + U[DENS]) * (PR[VEL2] + P[VEL2]);
  g[MOM1] = f[MOM2];
  g[MOM2] = 0.25 * (UR[DENS] + U[DENS]) * sq(PR[VEL2] + P[VEL2]) + (PR[PRES] + P[PRES]);
  g[MOM3] = 0.25 * (UR[DENS] + U[DENS]) * (PR[VEL2] + P[VEL2]) * (PR[VEL3] + P[VEL3]);
  g[ENER] = 0.25 * (UR[DENS] + U[DENS]) * (PR[VEL2] + P[VEL2]) * (ERef + E) +
            0.5 * (PR[PRES] + P[PRES]) * (PR[VEL2] + P[VEL2]);
  h[DENS] = 0.5 * (UR[DENS] + U[DENS]) * (PR[VEL3] + P[VEL3]);
  h[MOM1] = f[MOM3];
  h[MOM2] = g[MOM3];
  h[MOM3] = 0.25 * (UR[DENS] + U[DENS]) * sq(PR[VEL3] + P[VEL3]) + (PR[PRES] + P[PRES]);
  h[ENER] = 0.25 * (UR[DENS] + U[DENS]) * (PR[VEL3] + P[VEL3]) * (ERef + E) +
            0.5 * (PR[PRES] + P[PRES]) * (PR[VEL3] + P[VEL3]);
  combine(MRef, M, f, g, h, Flux);
}
// SplitVolumeFluxMO  splitflux.f90:523-611
static void SplitVolumeFluxMO(const double* UR, const double* PR, const double* U, const double* P,
                              const double* MRef, const double* M, double* Flux) {
  double f[5], g[5], h[5];
  double rhoepRef = UR[ENER] - 0.5 * UR[DENS] * (PR[VEL1] * PR[VEL1] + PR[VEL2] * PR[VEL2] + PR[VEL3] * PR[VEL3]) + PR[PRES];
  double rhoep = U[ENER] - 0.5 * U[DENS] * (P[VEL1] * P[VEL1] + P[VEL2] * P[VEL2] + P[VEL3] * P[VEL3]) + P[PRES];
  const int mom[3] = {MOM1, MOM2, MOM3};
  double* F[3] = {f, g, h};
  for (int d = 0; d < 3; ++d) {
    double* o = F[d];
    const int md = mom[d];
    const int vd = VEL1 + d;
    o[DENS] = (UR[md] + U[md]);
    o[MOM1] = 0.5 * (UR[md] + U[md]) * (PR[VEL1] + P[VEL1]) + (d == 0 ? (PR[PRES] + P[PRES]) : 0.);
    o[MOM2] = 0.5 * (UR[md] + U[md]) * (PR[VEL2] + P[VEL2]) + (d == 1 ? (PR[PRES] + P[PRES]) : 0.);
    o[MOM3] = 0.5 * (UR[md] + U[md]) * (PR[VEL3] + P[VEL3]) + (d == 2 ? (PR[PRES] + P[PRES]) : 0.);
    o[ENER] = (rhoepRef * PR[vd] + rhoep * P[vd]) +
              0.5 * (UR[md] * PR[VEL1] + U[md] * P[VEL1]) * (PR[VEL1] + P[VEL1]) +
              0.5 * (UR[md] * PR[VEL2] + U[md] * P[VEL2]) * (PR[VEL2] + P[VEL2]) +
              0.5 * (UR[md] * PR[VEL3] + U[md] * P[VEL3]) * (PR[VEL3] + P[VEL3]) -
              0.5 * (UR[md] * PR[VEL1] * PR[VEL1] + U[md] * P[VEL1] * P[VEL1]) -
              0.5 * (UR[md] * PR[VEL2] * PR[VEL2] + U[md] * P[VEL2] * P[VEL2]) -
              0.5 * (UR[md] * PR[VEL3] * PR[VEL3] + U[md] * P[VEL3] * P[VEL3]);
  }
  combine(MRef, M, f, g, h, Flux);
}
// SplitVolumeFluxPI  splitflux.f90:669-730
static void SplitVolumeFluxPI(const double* UR, const double* PR, const double* U, const double* P,
                              const double* MRef, const double* M, double* Flux) {
  double f[5], g[5], h[5];
  double HRef = (UR[ENER] + PR[PRES]) / UR[DENS];
  double H = (U[ENER] + P[PRES]) / U[DENS];
  f[DENS] = 0.5 * (UR[DENS] + U[DENS]) * (PR[VEL1] + P[VEL1]);
  f[MOM1] = 0.25 * (UR[DENS] + U[DENS]) * sq(PR[VEL1] + P[VEL1]) + (PR[PRES] + P[PRES]);
  f[MOM2] = 0.25 * (UR[DENS] + U[DENS]) * (PR[VEL1] + P[VEL1]) * (PR[VEL2] + P[VEL2]);
  f[MOM3] = 0.25 * (UR[DENS] + U[DENS]) * (PR[VEL1] + P[VEL1]) * (PR[VEL3] + P[VEL3]);
  f[ENER] = 0.25 * (UR[DENS] + U[DENS]) * (PR[VEL1] + P[VEL1]) * (HRef + H);
  g[DENS] = 0.5 * (UR[DENS] + U[DENS]) * (PR[VEL2] + P[VEL2]);
  g[MOM1] = f[MOM2];
  g[MOM2] = 0.25 * (UR[DENS] + U[DENS]) * sq(PR[VEL2] + P[VEL2]) + (PR[PRES] + P[PRES]);
  g[MOM3] = 0.25 * (UR[DENS] + U[DENS]) * (PR[VEL2] + P[VEL2]) * (PR[VEL3] + P[VEL3]);
  g[ENER] = 0.25 * (UR[DENS] + U[DENS]) * (PR[VEL2] + P[VEL2]) * (HRef + H);
  h[DENS] = 0.5 * (UR[DENS] + U[DENS]) * (PR[VEL3] + P[VEL3]);
  h[MOM1] = f[MOM3];
  h[MOM2] = g[MOM3];
  h[MOM3] = 0.25 * (UR[DENS] + U[DENS]) * sq(PR[VEL3] + P[VEL3]) + (PR[PRES] + P[PRES]);
  h[ENER] = 0.25 * (UR[DENS] + U[DENS]) * (PR[VEL3] + P[VEL3]) * (HRef + H);
  combine(MRef, M, f, g, h, Flux);
}
static void SplitVolumeFlux(int split, const double* UR, const double* PR, const double* U,
                            const double* P, const double* MRef, const double* M, double* Flux) {
  switch (split) {
    case DG_SPLIT_SD: SplitVolumeFluxSD(UR, PR, U, P, MRef, M, Flux); break;
    case DG_SPLIT_MO: SplitVolumeFluxMO(UR, PR, U, P, MRef, M, Flux); break;
    case DG_SPLIT_DU: SplitVolumeFluxDU(UR, PR, U, P, MRef, M, Flux); break;
    case DG_SPLIT_KG: SplitVolumeFluxKG(UR, PR, U, P, MRef, M, Flux); break;
    default: SplitVolumeFluxPI(UR, PR, U, P, MRef, M, Flux); break;
  }
}

// ---- split surface fluxes (extended states U_LL, U_RR) ----
// SplitSurfaceFluxSD  splitflux.f90:270-301
static void SplitSurfaceFluxSD(const double* L, const double* R, double* F) {
  F[DENS] = 0.5 * (L[EXT_MOM1] + R[EXT_MOM1]);
  F[MOM1] = 0.5 * (L[EXT_MOM1] * L[EXT_VEL1] + L[EXT_PRES] + R[EXT_MOM1] * R[EXT_VEL1] + R[EXT_PRES]);
  F[MOM2] = 0.5 * (L[EXT_MOM1] * L[EXT_VEL2] + R[EXT_MOM1] * R[EXT_VEL2]);
  F[MOM3] = 0.5 * (L[EXT_MOM1] * L[EXT_VEL3] + R[EXT_MOM1] * R[EXT_VEL3]);
  F[ENER] = 0.5 * ((L[EXT_ENER] + L[EXT_PRES]) * L[EXT_VEL1] + (R[EXT_ENER] + R[EXT_PRES]) * R[EXT_VEL1]);
}
// SplitSurfaceFluxDU  splitflux.f90:385-411
static void SplitSurfaceFluxDU(const double* L, const double* R, double* F) {
  F[DENS] = 0.25 * (L[EXT_DENS] + R[EXT_DENS]) * (L[EXT_VEL1] + R[EXT_VEL1]);
  F[MOM1] = 0.25 * (L[EXT_MOM1] + R[EXT_MOM1]) * (L[EXT_VEL1] + R[EXT_VEL1]) + 0.5 * (L[EXT_PRES] + R[EXT_PRES]);
  F[MOM2] = 0.25 * (L[EXT_MOM2] + R[EXT_MOM2]) * (L[EXT_VEL1] + R[EXT_VEL1]);
  F[MOM3] = 0.25 * (L[EXT_MOM3] + R[EXT_MOM3]) * (L[EXT_VEL1] + R[EXT_VEL1]);
  F[ENER] = 0.25 * (L[EXT_ENER] + R[EXT_ENER] + L[EXT_PRES] + R[EXT_PRES]) * (L[EXT_VEL1] + R[EXT_VEL1]);
}
// SplitSurfaceFluxKG  splitflux.f90:493-518
static void SplitSurfaceFluxKG(const double* L, const double* R, double* F) {
  double E_LL = L[EXT_ENER] / L[EXT_DENS], E_RR = R[EXT_ENER] / R[EXT_DENS];
  F[DENS] = 0.25 * (L[EXT_DENS] + R[EXT_DENS]) * (L[EXT_VEL1] + R[EXT_VEL1]);
  F[MOM1] = 0.125 * (L[EXT_DENS] + R[EXT_DENS]) * sq(L[EXT_VEL1] + R[EXT_VEL1]) + 0.5 * (L[EXT_PRES] + R[EXT_PRES]);
  F[MOM2] = 0.125 * (L[EXT_DENS] + R[EXT_DENS]) * (L[EXT_VEL1] + R[EXT_VEL1]) * (L[EXT_VEL2] + R[EXT_VEL2]);
  F[MOM3] = 0.125 * (L[EXT_DENS] + R[EXT_DENS]) * (L[EXT_VEL1] + R[EXT_VEL1]) * (L[EXT_VEL3] + R[EXT_VEL3]);
  F[ENER] = 0.125 * (L[EXT_DENS] + R[EXT_DENS]) * (E_LL + E_RR) * (L[EXT_VEL1] + R[EXT_VEL1]) +
            0.25 * (L[EXT_PRES] + R[EXT_PRES]) * (L[EXT_VEL1] + R[EXT_VEL1]);
}
// SplitSurfaceFluxMO  splitflux.f90:616-664
static void SplitSurfaceFluxMO(const double* L, const double* R, double* F) {
  double rL = L[EXT_ENER] - 0.5 * L[EXT_DENS] * (L[EXT_VEL1] * L[EXT_VEL1] + L[EXT_VEL2] * L[EXT_VEL2] + L[EXT_VEL3] * L[EXT_VEL3]) + L[EXT_PRES];
  double rR = R[EXT_ENER] - 0.5 * R[EXT_DENS] * (R[EXT_VEL1] * R[EXT_VEL1] + R[EXT_VEL2] * R[EXT_VEL2] + R[EXT_VEL3] * R[EXT_VEL3]) + R[EXT_PRES];
  F[DENS] = 0.5 * (L[EXT_MOM1] + R[EXT_MOM1]);
  F[MOM1] = 0.25 * (L[EXT_MOM1] + R[EXT_MOM1]) * (L[EXT_VEL1] + R[EXT_VEL1]) + 0.5 * (L[EXT_PRES] + R[EXT_PRES]);
  F[MOM2] = 0.25 * (L[EXT_MOM1] + R[EXT_MOM1]) * (L[EXT_VEL2] + R[EXT_VEL2]);
  F[MOM3] = 0.25 * (L[EXT_MOM1] + R[EXT_MOM1]) * (L[EXT_VEL3] + R[EXT_VEL3]);
  F[ENER] = 0.5 * (rL * L[EXT_VEL1] + rR * R[EXT_VEL1]) +
            0.25 * (L[EXT_MOM1] * L[EXT_VEL1] + R[EXT_MOM1] * R[EXT_VEL1]) * (L[EXT_VEL1] + R[EXT_VEL1]) +
            0.25 * (L[EXT_MOM1] * L[EXT_VEL2] + R[EXT_MOM1] * R[EXT_VEL2]) * (L[EXT_VEL2] + R[EXT_VEL2]) +
            0.25 * (L[EXT_MOM1] * L[EXT_VEL3] + R[EXT_MOM1] * R[EXT_VEL3]) * (L[EXT_VEL3] + R[EXT_VEL3]) -
            0.25 * (L[EXT_MOM1] * L[EXT_VEL1] * L[EXT_VEL1] + R[EXT_MOM1] * R[EXT_VEL1] * R[EXT_VEL1]) -
            0.25 * (L[EXT_MOM1] * L[EXT_VEL2] * L[EXT_VEL2] + R[EXT_MOM1] * R[EXT_VEL2] * R[EXT_VEL2]) -
            0.25 * (L[EXT_MOM1] * L[EXT_VEL3] * L[EXT_VEL3] + R[EXT_MOM1] * R[EXT_VEL3] * R[EXT_VEL3]);
}
// SplitSurfaceFluxPI  splitflux.f90:735-761
static void SplitSurfaceFluxPI(const double* L, const double* R, double* F) {
  double H_LL = (L[EXT_ENER] + L[EXT_PRES]) / L[EXT_DENS];
  double H_RR = (R[EXT_ENER] + R[EXT_PRES]) / R[EXT_DENS];
  F[DENS] = 0.25 * (L[EXT_DENS] + R[EXT_DENS]) * (L[EXT_VEL1] + R[EXT_VEL1]);
  F[MOM1] = 0.125 * (L[EXT_DENS] + R[EXT_DENS]) * sq(L[EXT_VEL1] + R[EXT_VEL1]) + 0.5 * (L[EXT_PRES] + R[EXT_PRES]);
  F[MOM2] = 0.125 * (L[EXT_DENS] + R[EXT_DENS]) * (L[EXT_VEL1] + R[EXT_VEL1]) * (L[EXT_VEL2] + R[EXT_VEL2]);
  F[MOM3] = 0.125 * (L[EXT_DENS] + R[EXT_DENS]) * (L[EXT_VEL1] + R[EXT_VEL1]) * (L[EXT_VEL3] + R[EXT_VEL3]);
  F[ENER] = 0.125 * (L[EXT_DENS] + R[EXT_DENS]) * (H_LL + H_RR) * (L[EXT_VEL1] + R[EXT_VEL1]);
}
static void SplitSurfaceFlux(int split, const double* L, const double* R, double* F) {
  switch (split) {
    case DG_SPLIT_SD: SplitSurfaceFluxSD(L, R, F); break;
    case DG_SPLIT_MO: SplitSurfaceFluxMO(L, R, F); break;
    case DG_SPLIT_DU: SplitSurfaceFluxDU(L, R, F); break;
    case DG_SPLIT_KG: SplitSurfaceFluxKG(L, R, F); break;
    default: SplitSurfaceFluxPI(L, R, F); break;
  }
}

// ---- Riemann solvers: riemann.f90:707-1257 ----
#define SPEEDOFSOUND_HE(UE) (std::sqrt(Kappa * UE[EXT_PRES] * UE[EXT_SRHO]))
#define TOTALENTHALPY_HE(UE) ((UE[EXT_ENER] + UE[EXT_PRES]) * UE[EXT_SRHO])
#define TOTALENERGY_HE(UE) (UE[EXT_ENER] * UE[EXT_SRHO])

struct RoeMeans { double RoeVel[3], RoeH, Roec, absVel; };
static inline void roe_means(const double* L, const double* R, double Kappa, RoeMeans& m, bool use_macro_c) {
  double H_L = TOTALENTHALPY_HE(L), H_R = TOTALENTHALPY_HE(R);
  double SqrtRho_L = std::sqrt(L[EXT_DENS]), SqrtRho_R = std::sqrt(R[EXT_DENS]);
  double sSqrtRho = 1. / (SqrtRho_L + SqrtRho_R);
  for (int d = 0; d < 3; ++d) m.RoeVel[d] = (SqrtRho_R * R[EXT_VEL1 + d] + SqrtRho_L * L[EXT_VEL1 + d]) * sSqrtRho;
  m.RoeH = (SqrtRho_R * H_R + SqrtRho_L * H_L) * sSqrtRho;
  m.absVel = m.RoeVel[0] * m.RoeVel[0] + m.RoeVel[1] * m.RoeVel[1] + m.RoeVel[2] * m.RoeVel[2];
  // ROEC_RIEMANN_H (eos.h:70); HLLC writes the same expression with absVel (riemann.f90:776)
  (void)use_macro_c;
  m.Roec = std::sqrt((Kappa - 1.) * (m.RoeH - 0.5 * m.absVel));
}

static void Riemann_Solver(const dg_config& cfg, double* F, const double* F_L, const double* F_R,
                           const double* L, const double* R) {
  const double Kappa = cfg.kappa;
  const bool split = cfg.split_dg >= 0;
  switch (cfg.riemann) {
    case DG_RIEMANN_LF: {  // riemann.f90:707-733
      double LambdaMax = std::max(std::fabs(R[EXT_VEL1]), std::fabs(L[EXT_VEL1])) +
                         std::max(SPEEDOFSOUND_HE(L), SPEEDOFSOUND_HE(R));
      if (!split) {
        for (int v = 0; v < 5; ++v) F[v] = 0.5 * ((F_L[v] + F_R[v]) - LambdaMax * (R[v] - L[v]));
      } else {
        SplitSurfaceFlux(cfg.split_dg, L, R, F);
        for (int v = 0; v < 5; ++v) F[v] = F[v] - 0.5 * LambdaMax * (R[v] - L[v]);
      }
    } break;
    case DG_RIEMANN_HLLC: {  // riemann.f90:738-804
      RoeMeans m; roe_means(L, R, Kappa, m, false);
      double Ssl = m.RoeVel[0] - m.Roec, Ssr = m.RoeVel[0] + m.Roec;
      if (Ssl >= 0.) { for (int v = 0; v < 5; ++v) F[v] = F_L[v]; }
      else if (Ssr <= 0.) { for (int v = 0; v < 5; ++v) F[v] = F_R[v]; }
      else {
        double sMu_L = Ssl - L[EXT_VEL1], sMu_R = Ssr - R[EXT_VEL1];
        double SStar = (R[EXT_PRES] - L[EXT_PRES] + L[EXT_MOM1] * sMu_L - R[EXT_MOM1] * sMu_R) /
                       (L[EXT_DENS] * sMu_L - R[EXT_DENS] * sMu_R);
        double U_Star[5];
        if ((Ssl <= 0.) && (SStar >= 0.)) {
          double EStar = TOTALENERGY_HE(L) + (SStar - L[EXT_VEL1]) * (SStar + L[EXT_PRES] * L[EXT_SRHO] / sMu_L);
          double fac = L[EXT_DENS] * sMu_L / (Ssl - SStar);
          U_Star[0] = fac * 1.; U_Star[1] = fac * SStar; U_Star[2] = fac * L[EXT_VEL2];
          U_Star[3] = fac * L[EXT_VEL3]; U_Star[4] = fac * EStar;
          for (int v = 0; v < 5; ++v) F[v] = F_L[v] + Ssl * (U_Star[v] - L[v]);
        } else {
          double EStar = TOTALENERGY_HE(R) + (SStar - R[EXT_VEL1]) * (SStar + R[EXT_PRES] * R[EXT_SRHO] / sMu_R);
          double fac = R[EXT_DENS] * sMu_R / (Ssr - SStar);
          U_Star[0] = fac * 1.; U_Star[1] = fac * SStar; U_Star[2] = fac * R[EXT_VEL2];
          U_Star[3] = fac * R[EXT_VEL3]; U_Star[4] = fac * EStar;
          for (int v = 0; v < 5; ++v) F[v] = F_R[v] + Ssr * (U_Star[v] - R[v]);
        }
      }
    } break;
    case DG_RIEMANN_ROE:
    case DG_RIEMANN_ROEL2: {  // riemann.f90:809-878 and 994-1070
      RoeMeans m; roe_means(L, R, Kappa, m, true);
      const double* RoeVel = m.RoeVel;
      double RoeH = m.RoeH, Roec = m.Roec, absVel = m.absVel;
      double a[5] = {RoeVel[0] - Roec, RoeVel[0], RoeVel[0], RoeVel[0], RoeVel[0] + Roec};
      double r1[5] = {1., a[0], RoeVel[1], RoeVel[2], RoeH - RoeVel[0] * Roec};
      double r2[5] = {1., RoeVel[0], RoeVel[1], RoeVel[2], 0.5 * absVel};
      double r3[5] = {0., 0., 1., 0., RoeVel[1]};
      double r4[5] = {0., 0., 0., 1., RoeVel[2]};
      double r5[5] = {1., a[4], RoeVel[1], RoeVel[2], RoeH + RoeVel[0] * Roec};
      double dU[6];
      for (int v = 0; v < 5; ++v) dU[v] = R[v] - L[v];
      dU[5] = dU[4] - (dU[2] - RoeVel[1] * dU[0]) * RoeVel[1] - (dU[3] - RoeVel[2] * dU[0]) * RoeVel[2];
      if (cfg.riemann == DG_RIEMANN_ROEL2) {
        double Ma_loc = std::sqrt(absVel) / (Roec * std::sqrt(Kappa));
        for (int v = 1; v <= 3; ++v) dU[v] = dU[v] * Ma_loc;
      }
      double Alpha3 = dU[2] - RoeVel[1] * dU[0];
      double Alpha4 = dU[3] - RoeVel[2] * dU[0];
      // ALPHA2_RIEMANN_H  eos.h:71
      double Alpha2 = (Kappa - 1.) / (Roec * Roec) * (dU[0] * (RoeH - RoeVel[0] * RoeVel[0]) - dU[5] + RoeVel[0] * dU[1]);
      double Alpha1 = 0.5 / Roec * (dU[0] * (RoeVel[0] + Roec) - dU[1] - Roec * Alpha2);
      double Alpha5 = dU[0] - Alpha1 - Alpha2;
      if (!split) {
        for (int v = 0; v < 5; ++v)
          F[v] = 0.5 * ((F_L[v] + F_R[v]) - Alpha1 * std::fabs(a[0]) * r1[v] - Alpha2 * std::fabs(a[1]) * r2[v] -
                        Alpha3 * std::fabs(a[2]) * r3[v] - Alpha4 * std::fabs(a[3]) * r4[v] -
                        Alpha5 * std::fabs(a[4]) * r5[v]);
      } else {
        SplitSurfaceFlux(cfg.split_dg, L, R, F);
        for (int v = 0; v < 5; ++v)
          F[v] = F[v] - 0.5 * (Alpha1 * std::fabs(a[0]) * r1[v] + Alpha2 * std::fabs(a[1]) * r2[v] +
                               Alpha3 * std::fabs(a[2]) * r3[v] + Alpha4 * std::fabs(a[3]) * r4[v] +
                               Alpha5 * std::fabs(a[4]) * r5[v]);
      }
    } break;
    case DG_RIEMANN_ROEENTROPYFIX: {  // riemann.f90:885-989
      double c_L = SPEEDOFSOUND_HE(L), c_R = SPEEDOFSOUND_HE(R);
      RoeMeans m; roe_means(L, R, Kappa, m, true);
      const double* RoeVel = m.RoeVel;
      double RoeH = m.RoeH, Roec = m.Roec, absVel = m.absVel;
      double RoeDens = std::sqrt(L[EXT_DENS] * R[EXT_DENS]);
      double dU[5];
      dU[0] = R[EXT_DENS] - L[EXT_DENS];
      dU[1] = R[EXT_VEL1] - L[EXT_VEL1];
      dU[2] = R[EXT_VEL2] - L[EXT_VEL2];
      dU[3] = R[EXT_VEL3] - L[EXT_VEL3];
      dU[4] = R[EXT_PRES] - L[EXT_PRES];
      double a[5] = {RoeVel[0] - Roec, RoeVel[0], RoeVel[0], RoeVel[0], RoeVel[0] + Roec};
      double r1[5] = {1., a[0], RoeVel[1], RoeVel[2], RoeH - RoeVel[0] * Roec};
      double r2[5] = {1., RoeVel[0], RoeVel[1], RoeVel[2], 0.5 * absVel};
      double r3[5] = {0., 0., 1., 0., RoeVel[1]};
      double r4[5] = {0., 0., 0., 1., RoeVel[2]};
      double r5[5] = {1., a[4], RoeVel[1], RoeVel[2], RoeH + RoeVel[0] * Roec};
      double tmp = 0.5 / (Roec * Roec);
      double Alpha[5];
      Alpha[0] = tmp * (dU[4] - RoeDens * Roec * dU[1]);
      Alpha[1] = dU[0] - dU[4] * 2. * tmp;
      Alpha[2] = RoeDens * dU[2];
      Alpha[3] = RoeDens * dU[3];
      Alpha[4] = tmp * (dU[4] + RoeDens * Roec * dU[1]);
      double al[5] = {L[EXT_VEL1] - c_L, L[EXT_VEL1], L[EXT_VEL1], L[EXT_VEL1], L[EXT_VEL1] + c_L};
      double ar[5] = {R[EXT_VEL1] - c_R, R[EXT_VEL1], R[EXT_VEL1], R[EXT_VEL1], R[EXT_VEL1] + c_R};
      for (int i = 0; i < 5; ++i) {
        double da = std::max(0., std::max(a[i] - al[i], ar[i] - a[i]));
        if (std::fabs(a[i]) < da) a[i] = 0.5 * (a[i] * a[i] / da + da);
        else a[i] = std::fabs(a[i]);
      }
      if (!split) {
        for (int v = 0; v < 5; ++v)
          F[v] = 0.5 * ((F_L[v] + F_R[v]) - Alpha[0] * a[0] * r1[v] - Alpha[1] * a[1] * r2[v] -
                        Alpha[2] * a[2] * r3[v] - Alpha[3] * a[3] * r4[v] - Alpha[4] * a[4] * r5[v]);
      } else {
        SplitSurfaceFlux(cfg.split_dg, L, R, F);
        for (int v = 0; v < 5; ++v)
          F[v] = F[v] - 0.5 * (Alpha[0] * a[0] * r1[v] + Alpha[1] * a[1] * r2[v] + Alpha[2] * a[2] * r3[v] +
                               Alpha[3] * a[3] * r4[v] + Alpha[4] * a[4] * r5[v]);
      }
    } break;
    case DG_RIEMANN_HLL:
    case DG_RIEMANN_HLLE: {  // riemann.f90:1075-1121, 1126-1170
      RoeMeans m; roe_means(L, R, Kappa, m, true);
      double Ssl, Ssr;
      if (cfg.riemann == DG_RIEMANN_HLL) {
        Ssl = m.RoeVel[0] - m.Roec; Ssr = m.RoeVel[0] + m.Roec;
      } else {
        double beta = std::sqrt(0.5 * (Kappa - 1.) / Kappa);  // BETA_RIEMANN_H eos.h:69
        Ssl = std::min(std::min(m.RoeVel[0] - m.Roec, L[EXT_VEL1] - beta * SPEEDOFSOUND_HE(L)), 0.);
        Ssr = std::max(std::max(m.RoeVel[0] + m.Roec, R[EXT_VEL1] + beta * SPEEDOFSOUND_HE(R)), 0.);
      }
      if (Ssl >= 0.) { for (int v = 0; v < 5; ++v) F[v] = F_L[v]; }
      else if (Ssr <= 0.) { for (int v = 0; v < 5; ++v) F[v] = F_R[v]; }
      else {
        for (int v = 0; v < 5; ++v) F[v] = (Ssr * F_L[v] - Ssl * F_R[v] + Ssl * Ssr * (R[v] - L[v])) / (Ssr - Ssl);
      }
    } break;
    case DG_RIEMANN_HLLEM: {  // riemann.f90:1175-1233
      RoeMeans m; roe_means(L, R, Kappa, m, true);
      double RoeDens = std::sqrt(L[EXT_DENS] * R[EXT_DENS]);
      double beta = std::sqrt(0.5 * (Kappa - 1.) / Kappa);
      double Ssl = std::min(std::min(m.RoeVel[0] - m.Roec, L[EXT_VEL1] - beta * SPEEDOFSOUND_HE(L)), 0.);
      double Ssr = std::max(std::max(m.RoeVel[0] + m.Roec, R[EXT_VEL1] + beta * SPEEDOFSOUND_HE(R)), 0.);
      if (Ssl >= 0.) { for (int v = 0; v < 5; ++v) F[v] = F_L[v]; }
      else if (Ssr <= 0.) { for (int v = 0; v < 5; ++v) F[v] = F_R[v]; }
      else {
        double delta = m.Roec / (m.Roec + std::fabs(0.5 * (Ssl + Ssr)));
        double A2 = (R[EXT_DENS] - L[EXT_DENS]) - (R[EXT_PRES] - L[EXT_PRES]) / (m.Roec * m.Roec);
        double A3 = RoeDens * (R[EXT_VEL2] - L[EXT_VEL2]);
        double A4 = RoeDens * (R[EXT_VEL3] - L[EXT_VEL3]);
        double r2[5] = {1., m.RoeVel[0], m.RoeVel[1], m.RoeVel[2], 0.5 * m.absVel};
        double r3[5] = {0., 0., 1., 0., m.RoeVel[1]};
        double r4[5] = {0., 0., 0., 1., m.RoeVel[2]};
        for (int v = 0; v < 5; ++v)
          F[v] = (Ssr * F_L[v] - Ssl * F_R[v] +
                  Ssl * Ssr * (R[v] - L[v] - delta * (r2[v] * A2 + r3[v] * A3 + r4[v] * A4))) / (Ssr - Ssl);
      }
    } break;
    default:  // DG_RIEMANN_AVERAGE  riemann.f90:1239-1257
      SplitSurfaceFlux(cfg.split_dg, L, R, F);
      break;
  }
}

// Riemann  riemann.f90:216-289 (rotation into the normal frame, back-rotation)
static void Riemann(const dg_config& cfg, double* FOut, const double* U_L, const double* U_R,
                    const double* P_L, const double* P_R, const double* nv, const double* t1, const double* t2) {
  double LL[11], RR[11], F_L[5] = {0, 0, 0, 0, 0}, F_R[5] = {0, 0, 0, 0, 0}, F[5];
  auto fill = [&](double* E, const double* Uc, const double* P) {
    E[EXT_DENS] = Uc[DENS];
    E[EXT_SRHO] = 1. / E[EXT_DENS];
    E[EXT_ENER] = Uc[ENER];
    E[EXT_PRES] = P[PRES];
    E[EXT_VEL1] = P[VEL1] * nv[0] + P[VEL2] * nv[1] + P[VEL3] * nv[2];
    E[EXT_VEL2] = P[VEL1] * t1[0] + P[VEL2] * t1[1] + P[VEL3] * t1[2];
    E[EXT_MOM1] = E[EXT_DENS] * E[EXT_VEL1];
    E[EXT_MOM2] = E[EXT_DENS] * E[EXT_VEL2];
    E[EXT_VEL3] = P[VEL1] * t2[0] + P[VEL2] * t2[1] + P[VEL3] * t2[2];
    E[EXT_MOM3] = E[EXT_DENS] * E[EXT_VEL3];
    E[EXT_TEMP] = 0.;
  };
  fill(LL, U_L, P_L);
  fill(RR, U_R, P_R);
  if (cfg.split_dg < 0) {
    EvalEulerFlux1D_fast(LL, F_L);
    EvalEulerFlux1D_fast(RR, F_R);
  }
  Riemann_Solver(cfg, F, F_L, F_R, LL, RR);
  FOut[DENS] = F[DENS];
  for (int d = 0; d < 3; ++d) FOut[MOM1 + d] = nv[d] * F[MOM1] + t1[d] * F[MOM2] + t2[d] * F[MOM3];
  FOut[ENER] = F[ENER];
}

// EvalNormalDiffFlux3D  flux.f90:779-847
static void EvalNormalDiffFlux3D(const double* P, const double* gx, const double* gy, const double* gz, double* f,
                                 const double* nv, double mu, double lambda) {
  const double s23 = 2. / 3., s43 = 4. / 3.;
  double tau_xx = mu * (s43 * gx[1] - s23 * gy[2] - s23 * gz[3]);
  double tau_yy = mu * (-s23 * gx[1] + s43 * gy[2] - s23 * gz[3]);
  double tau_zz = mu * (-s23 * gx[1] - s23 * gy[2] + s43 * gz[3]);
  double tau_xy = mu * (gy[1] + gx[2]);
  double tau_xz = mu * (gz[1] + gx[3]);
  double tau_yz = mu * (gz[2] + gy[3]);
  f[DENS] = 0.;
  f[MOM1] = -nv[0] * tau_xx - nv[1] * tau_xy - nv[2] * tau_xz;
  f[MOM2] = -nv[0] * tau_xy - nv[1] * tau_yy - nv[2] * tau_yz;
  f[MOM3] = -nv[0] * tau_xz - nv[1] * tau_yz - nv[2] * tau_zz;
  f[ENER] = -nv[0] * (tau_xx * P[VEL1] + tau_xy * P[VEL2] + tau_xz * P[VEL3] + lambda * gx[4]) -
            nv[1] * (tau_xy * P[VEL1] + tau_yy * P[VEL2] + tau_yz * P[VEL3] + lambda * gy[4]) -
            nv[2] * (tau_xz * P[VEL1] + tau_yz * P[VEL2] + tau_zz * P[VEL3] + lambda * gz[4]);
}

// EvalTransformedEulerFlux3D_fast  flux.f90:137-186
static void EvalTransformedEulerFlux3D_fast(const double* U, const double* P, double* f, double* g, double* h,
                                            const double* Mf, const double* Mg, const double* Mh) {
  double Ep = (U[ENER] + P[PRES]) / U[DENS];
  const double* Ms[3] = {Mf, Mg, Mh};
  double* out[3] = {f, g, h};
  for (int d = 0; d < 3; ++d) {
    const double* M = Ms[d];
    double Mmom = M[0] * U[MOM1] + M[1] * U[MOM2] + M[2] * U[MOM3];
    out[d][DENS] = Mmom;
    out[d][MOM1] = Mmom * P[VEL1] + M[0] * P[PRES];
    out[d][MOM2] = Mmom * P[VEL2] + M[1] * P[PRES];
    out[d][MOM3] = Mmom * P[VEL3] + M[2] * P[PRES];
    out[d][ENER] = Mmom * Ep;
  }
}

// shared viscous stress part of flux.f90:509-697
static void visc_terms(const double* P, const double* gx, const double* gy, const double* gz, double mu, double lambda,
                       double tau[6], double tq[3]) {
  const double s23 = 2. / 3., s43 = 4. / 3.;
  double tau_xx = mu * (s43 * gx[1] - s23 * gy[2] - s23 * gz[3]);
  double tau_yy = mu * (-s23 * gx[1] + s43 * gy[2] - s23 * gz[3]);
  double tau_zz = mu * (-s23 * gx[1] - s23 * gy[2] + s43 * gz[3]);
  double tau_xy = mu * (gy[1] + gx[2]);
  double tau_xz = mu * (gz[1] + gx[3]);
  double tau_yz = mu * (gz[2] + gy[3]);
  tq[0] = tau_xx * P[VEL1] + tau_xy * P[VEL2] + tau_xz * P[VEL3] + lambda * gx[4];
  tq[1] = tau_xy * P[VEL1] + tau_yy * P[VEL2] + tau_yz * P[VEL3] + lambda * gy[4];
  tq[2] = tau_xz * P[VEL1] + tau_yz * P[VEL2] + tau_zz * P[VEL3] + lambda * gz[4];
  tau[0] = tau_xx; tau[1] = tau_yy; tau[2] = tau_zz; tau[3] = tau_xy; tau[4] = tau_xz; tau[5] = tau_yz;
}

// EvalTransformedEulerDiffFlux3D  flux.f90:509-614
static void EvalTransformedEulerDiffFlux3D(const double* U, const double* P, const double* gx, const double* gy,
                                           const double* gz, double* f, double* g, double* h, const double* Mf,
                                           const double* Mg, const double* Mh, double mu, double lambda) {
  double tau[6], tq[3];
  visc_terms(P, gx, gy, gz, mu, lambda, tau, tq);
  double Ep = (U[ENER] + P[PRES]) / U[DENS];
  const double txx = tau[0], tyy = tau[1], tzz = tau[2], txy = tau[3], txz = tau[4], tyz = tau[5];
  const double* Ms[3] = {Mf, Mg, Mh};
  double* out[3] = {f, g, h};
  for (int d = 0; d < 3; ++d) {
    const double* M = Ms[d];
    double Mmom = M[0] * U[MOM1] + M[1] * U[MOM2] + M[2] * U[MOM3];
    out[d][DENS] = Mmom;
    out[d][MOM1] = Mmom * P[VEL1] + M[0] * P[PRES] - M[0] * txx - M[1] * txy - M[2] * txz;
    out[d][MOM2] = Mmom * P[VEL2] + M[1] * P[PRES] - M[0] * txy - M[1] * tyy - M[2] * tyz;
    out[d][MOM3] = Mmom * P[VEL3] + M[2] * P[PRES] - M[0] * txz - M[1] * tyz - M[2] * tzz;
    out[d][ENER] = Mmom * Ep - M[0] * tq[0] - M[1] * tq[1] - M[2] * tq[2];
  }
}

// EvalTransformedDiffFlux3D  flux.f90:619-697
static void EvalTransformedDiffFlux3D(const double* P, const double* gx, const double* gy, const double* gz,
                                      double* f, double* g, double* h, const double* Mf, const double* Mg,
                                      const double* Mh, double mu, double lambda) {
  double tau[6], tq[3];
  visc_terms(P, gx, gy, gz, mu, lambda, tau, tq);
  const double txx = tau[0], tyy = tau[1], tzz = tau[2], txy = tau[3], txz = tau[4], tyz = tau[5];
  const double* Ms[3] = {Mf, Mg, Mh};
  double* out[3] = {f, g, h};
  for (int d = 0; d < 3; ++d) {
    const double* M = Ms[d];
    out[d][DENS] = 0.;
    out[d][MOM1] = -M[0] * txx - M[1] * txy - M[2] * txz;
    out[d][MOM2] = -M[0] * txy - M[1] * tyy - M[2] * tyz;
    out[d][MOM3] = -M[0] * txz - M[1] * tyz - M[2] * tzz;
    out[d][ENER] = -M[0] * tq[0] - M[1] * tq[1] - M[2] * tq[2];
  }
}

// ---------------------------------------------------------------------------------------
// Boundary conditions: equations/navierstokes/idealgas/getboundaryflux.f90
// ---------------------------------------------------------------------------------------
// PRESSURE_RIEMANN_PURE  idealgas/eos.f90:605-628 (U_Prim in the side-normal frame)
static double PRESSURE_RIEMANN_PURE(const double* U_Prim, double Kappa) {
  double P_RP;
  if (U_Prim[VEL1] <= 0.) {  // rarefaction
    const double kappaFac = 2. * Kappa / (Kappa - 1.);
    P_RP = U_Prim[PRES] *
           std::pow(std::max(0.0001, (1. + 0.5 * (Kappa - 1.) * U_Prim[VEL1] / std::sqrt(Kappa * U_Prim[PRES] / U_Prim[DENS]))),
                    kappaFac);
  } else {  // shock
    const double ar = 2. / ((Kappa + 1.) * U_Prim[DENS]);
    const double br = (Kappa - 1.) / (Kappa + 1.) * U_Prim[PRES];
    P_RP = U_Prim[PRES] + U_Prim[VEL1] / ar * 0.5 *
                              (U_Prim[VEL1] + std::sqrt(U_Prim[VEL1] * U_Prim[VEL1] + 4. * ar * (U_Prim[PRES] + br)));
  }
  return P_RP;
}

// GetBoundaryState  getboundaryflux.f90:262-487
static void GetBoundaryState(int BCType, double* UPrim_Out, const double* UPrim_master, const double* RefStatePrim,
                             const double* NormVec, const double* TangVec1, const double* TangVec2, double kappa,
                             double R) {
  if (BCType == 2) {
    for (int c = 0; c < 6; ++c) UPrim_Out[c] = RefStatePrim[c];
    return;
  }
  auto dot3 = [](const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; };
  double B[6];
  B[DENS] = UPrim_master[DENS];
  B[VEL1] = dot3(&UPrim_master[VEL1], NormVec);
  B[VEL2] = dot3(&UPrim_master[VEL1], TangVec1);
  B[VEL3] = dot3(&UPrim_master[VEL1], TangVec2);
  B[PRES] = UPrim_master[PRES];
  B[TEMP] = UPrim_master[TEMP];
  switch (BCType) {
    case 3:
    case 4:  // adiabatic / isothermal wall
      B[PRES] = PRESSURE_RIEMANN_PURE(B, kappa);
      B[VEL1] = 0.; B[VEL2] = 0.; B[VEL3] = 0.;
      B[TEMP] = BCType == 3 ? UPrim_master[TEMP] : RefStatePrim[TEMP];
      B[DENS] = B[PRES] / (B[TEMP] * R);
      break;
    case 9:
    case 91:  // slip wall
      B[PRES] = PRESSURE_RIEMANN_PURE(B, kappa);
      B[VEL1] = 0.;
      B[DENS] = UPrim_master[DENS];
      B[TEMP] = B[PRES] / (B[DENS] * R);
      break;
    case 23: {  // outflow Mach number
      const double MaOut = RefStatePrim[1];
      const double c = std::sqrt(kappa * B[PRES] / B[DENS]);
      const double Ma = B[VEL1] / c;
      double pb;
      if (Ma < 1) {
        const double pt = B[PRES] * (std::pow(1 + 0.5 * (kappa - 1) * Ma * Ma, kappa / (kappa - 1.)));
        pb = pt * (std::pow(1 + 0.5 * (kappa - 1) * MaOut * MaOut, -kappa / (kappa - 1.)));
      } else {
        pb = B[PRES] + 0.5 * B[DENS] * dot3(&B[VEL1], &B[VEL1]);
      }
      B[DENS] = kappa * pb / (c * c);
      B[PRES] = pb;
      B[TEMP] = B[PRES] / (R * B[DENS]);
      break;
    }
    case 24: {  // pressure outflow
      const double c = std::sqrt(kappa * B[PRES] / B[DENS]);
      const double Ma = B[VEL1] / c;
      if (Ma < 1) {
        const double pb = RefStatePrim[4];
        B[DENS] = kappa * pb / (c * c);
        B[PRES] = pb;
        B[TEMP] = B[PRES] / (R * B[DENS]);
      }
      break;
    }
    case 25: {  // subsonic outflow
      const double c = std::sqrt(kappa * B[PRES] / B[DENS]);
      const double Ma = B[VEL1] / c;
      const double pb = Ma < 1 ? RefStatePrim[4] : B[PRES] + 0.5 * B[DENS] * dot3(&B[VEL1], &B[VEL1]);
      if (B[VEL1] < 0.) {
        B[VEL1] = std::fabs(B[VEL1]);
        B[VEL2] = 0.;
        B[VEL3] = 0.;
      }
      B[DENS] = kappa * pb / (c * c);
      B[PRES] = RefStatePrim[4];
      B[TEMP] = B[PRES] / (R * B[DENS]);
      break;
    }
    case 27: {  // subsonic inflow
      const double Tt = RefStatePrim[0], pt = RefStatePrim[4];
      const double* a = &RefStatePrim[1];
      const double A = -1. * dot3(a, NormVec);
      const double c = std::sqrt(kappa * B[PRES] / B[DENS]);
      const double Rplus = -B[VEL1] - 2. * c / (kappa - 1.);
      const double tmp1 = A * A + 2. / (kappa - 1.);
      const double tmp2 = 2 * Rplus;
      const double tmp3 = (kappa - 1.) / 2. * (Rplus * Rplus) - kappa * R * Tt * (A * A);
      const double cb = std::max((-tmp2 + std::sqrt(tmp2 * tmp2 - 4 * tmp1 * tmp3)) / (2 * tmp1),
                                 (-tmp2 - std::sqrt(tmp2 * tmp2 - 4 * tmp1 * tmp3)) / (2 * tmp1));
      const double Tb = cb * cb / (kappa * R);
      const double Ma = std::sqrt(2. / (kappa - 1.) * (Tt / Tb - 1.));
      const double pb = pt * std::pow(1. + 0.5 * (kappa - 1.) * (Ma * Ma), -kappa / (kappa - 1.));
      const double U = Ma * std::sqrt(kappa * R * Tb);
      B[DENS] = pb / (R * Tb);
      B[VEL1] = U * dot3(a, NormVec);
      B[VEL2] = U * dot3(a, TangVec1);
      B[VEL3] = U * dot3(a, TangVec2);
      B[PRES] = pb;
      B[TEMP] = Tb;
      break;
    }
  }
  UPrim_Out[DENS] = B[DENS];
  for (int d = 0; d < 3; ++d) UPrim_Out[VEL1 + d] = B[VEL1] * NormVec[d] + B[VEL2] * TangVec1[d] + B[VEL3] * TangVec2[d];
  UPrim_Out[PRES] = B[PRES];
  UPrim_Out[TEMP] = B[TEMP];
}

// PrimToCons  idealgas/eos.f90:467-489
static void PrimToCons(const double* prim, double* cons, double Kappa) {
  cons[DENS] = prim[DENS];
  cons[MOM1] = prim[VEL1] * prim[DENS];
  cons[MOM2] = prim[VEL2] * prim[DENS];
  cons[MOM3] = prim[VEL3] * prim[DENS];
  cons[ENER] = prim[PRES] / (Kappa - 1.) + 0.5 * (cons[MOM1] * prim[VEL1] + cons[MOM2] * prim[VEL2] + cons[MOM3] * prim[VEL3]);
}

// EvalDiffFlux3D  flux.f90:702-760
static void EvalDiffFlux3D(const double* P, const double* gx, const double* gy, const double* gz, double* f, double* g,
                           double* h, double mu, double lambda) {
  const double s23 = 2. / 3., s43 = 4. / 3.;
  const double tau_xx = mu * (s43 * gx[1] - s23 * gy[2] - s23 * gz[3]);
  const double tau_yy = mu * (-s23 * gx[1] + s43 * gy[2] - s23 * gz[3]);
  const double tau_zz = mu * (-s23 * gx[1] - s23 * gy[2] + s43 * gz[3]);
  const double tau_xy = mu * (gy[1] + gx[2]);
  const double tau_xz = mu * (gz[1] + gx[3]);
  const double tau_yz = mu * (gz[2] + gy[3]);
  f[DENS] = 0.; f[MOM1] = -tau_xx; f[MOM2] = -tau_xy; f[MOM3] = -tau_xz;
  f[ENER] = -tau_xx * P[VEL1] - tau_xy * P[VEL2] - tau_xz * P[VEL3] - lambda * gx[4];
  g[DENS] = 0.; g[MOM1] = -tau_xy; g[MOM2] = -tau_yy; g[MOM3] = -tau_yz;
  g[ENER] = -tau_xy * P[VEL1] - tau_yy * P[VEL2] - tau_yz * P[VEL3] - lambda * gy[4];
  h[DENS] = 0.; h[MOM1] = -tau_xz; h[MOM2] = -tau_yz; h[MOM3] = -tau_zz;
  h[ENER] = -tau_xz * P[VEL1] - tau_yz * P[VEL2] - tau_zz * P[VEL3] - lambda * gz[4];
}

// GetBoundaryFlux_GPU  getboundaryflux.f90:542-838, one face point; Flux before the SurfElem factor
static void GetBoundaryFlux(const Ctx& C, const double* UPrim_master, const double* gx, const double* gy,
                            const double* gz, const double* nv, const double* t1, const double* t2, int BCType,
                            const double* RefStatePrim, double* Flux) {
  const dg_config& cfg = C.cfg;
  const double Kappa = cfg.kappa, mu = cfg.mu0, lambda = cfg.mu0 * cfg.R * cfg.kappa / ((cfg.kappa - 1.) * cfg.Pr);
  double UPrim_boundary[6];
  GetBoundaryState(BCType, UPrim_boundary, UPrim_master, RefStatePrim, nv, t1, t2, Kappa, cfg.R);
  if (BCType == 2 || BCType == 23 || BCType == 24 || BCType == 25 || BCType == 27) {
    double UCons_master[5], UCons_boundary[5];
    PrimToCons(UPrim_master, UCons_master, Kappa);
    PrimToCons(UPrim_boundary, UCons_boundary, Kappa);
    Riemann(cfg, Flux, UCons_master, UCons_boundary, UPrim_master, UPrim_boundary, nv, t1, t2);
    if (cfg.parabolic) {
      // ViscousFlux  riemann.f90:489-546 with the master gradients on both sides
      double fL[5], gL[5], hL[5], fR[5], gR[5], hR[5];
      EvalDiffFlux3D(UPrim_master, gx, gy, gz, fL, gL, hL, mu, lambda);
      EvalDiffFlux3D(UPrim_boundary, gx, gy, gz, fR, gR, hR, mu, lambda);
      for (int v = 0; v < 5; ++v)
        Flux[v] = Flux[v] + 0.5 * (nv[0] * (fL[v] + fR[v]) + nv[1] * (gL[v] + gR[v]) + nv[2] * (hL[v] + hR[v]));
    }
    return;
  }
  // walls: F = (0, p n, 0)
  Flux[DENS] = 0.;
  for (int d = 0; d < 3; ++d) Flux[MOM1 + d] = UPrim_boundary[PRES] * nv[d];
  Flux[ENER] = 0.;
  if (!cfg.parabolic) return;
  double Fd[5], Gd[5], Hd[5];
  if (BCType == 3 || BCType == 4) {
    EvalDiffFlux3D(UPrim_boundary, gx, gy, gz, Fd, Gd, Hd, mu, lambda);
    if (BCType == 3) { Fd[ENER] = 0.; Gd[ENER] = 0.; Hd[ENER] = 0.; }
  } else if (BCType == 9) {
    // BCGradMat = I - n n^T applied to all gradients
    double M[3][3];
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) M[a][b] = (a == b ? 1. : 0.) - nv[a] * nv[b];
    M[1][0] = M[0][1]; M[2][0] = M[0][2]; M[1][2] = M[2][1];
    double fx[5], fy[5], fz[5];
    for (int v = 0; v < 5; ++v) {
      fx[v] = M[0][0] * gx[v] + M[0][1] * gy[v] + M[0][2] * gz[v];
      fy[v] = M[1][0] * gx[v] + M[1][1] * gy[v] + M[1][2] * gz[v];
      fz[v] = M[2][0] * gx[v] + M[2][1] * gy[v] + M[2][2] * gz[v];
    }
    EvalDiffFlux3D(UPrim_boundary, fx, fy, fz, Fd, Gd, Hd, mu, lambda);
  } else {  // 91
    double M[3][3];
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) M[a][b] = (a == b ? 1. : 0.) - nv[a] * nv[b];
    M[1][0] = M[0][1]; M[2][0] = M[0][2]; M[1][2] = M[2][1];
    const double* G[3] = {gx, gy, gz};
    double fl[3][5] = {{0}};  // the density gradient is not used by EvalDiffFlux3D
    for (int d = 0; d < 3; ++d) fl[d][4] = M[d][0] * gx[4] + M[d][1] * gy[4] + M[d][2] * gz[4];
    // gradients of the wall-aligned velocities
    double vN[3], vT1[3], vT2[3];
    for (int d = 0; d < 3; ++d) {
      vN[d] = nv[0] * G[d][1] + nv[1] * G[d][2] + nv[2] * G[d][3];
      vT1[d] = t1[0] * G[d][1] + t1[1] * G[d][2] + t1[2] * G[d][3];
      vT2[d] = t2[0] * G[d][1] + t2[1] * G[d][2] + t2[2] * G[d][3];
    }
    // derivatives along n, t1, t2; normal-tangential couplings set to zero
    const double n_vN = nv[0] * vN[0] + nv[1] * vN[1] + nv[2] * vN[2];
    const double n_vT1 = 0., n_vT2 = 0., t1_vN = 0., t2_vN = 0.;
    const double t1_vT1 = t1[0] * vT1[0] + t1[1] * vT1[1] + t1[2] * vT1[2];
    const double t1_vT2 = t1[0] * vT2[0] + t1[1] * vT2[1] + t1[2] * vT2[2];
    const double t2_vT1 = t2[0] * vT1[0] + t2[1] * vT1[1] + t2[2] * vT1[2];
    const double t2_vT2 = t2[0] * vT2[0] + t2[1] * vT2[1] + t2[2] * vT2[2];
    double xN[3], xT1[3], xT2[3];
    for (int d = 0; d < 3; ++d) {
      xN[d] = nv[d] * n_vN + t1[d] * t1_vN + t2[d] * t2_vN;
      xT1[d] = nv[d] * n_vT1 + t1[d] * t1_vT1 + t2[d] * t2_vT1;
      xT2[d] = nv[d] * n_vT2 + t1[d] * t1_vT2 + t2[d] * t2_vT2;
    }
    for (int d = 0; d < 3; ++d)
      for (int c = 0; c < 3; ++c) fl[d][1 + c] = nv[c] * xN[d] + t1[c] * xT1[d] + t2[c] * xT2[d];
    EvalDiffFlux3D(UPrim_boundary, fl[0], fl[1], fl[2], Fd, Gd, Hd, mu, lambda);
  }
  for (int v = 0; v < 5; ++v) Flux[v] = Flux[v] + nv[0] * Fd[v] + nv[1] * Gd[v] + nv[2] * Hd[v];
}

// Lifting_GetBoundaryFlux_Kernel  getboundaryflux.f90:945-1019, one face point, SurfElem included
static void Lifting_GetBoundaryFlux(const Ctx& C, const double* UPrim_master, const double* nv, const double* t1,
                                    const double* t2, double SurfElem, int BCType, const double* RefStatePrim,
                                    bool doWeakLifting, double* Flux) {
  double UPrim_boundary[6], Flux_loc[5];
  GetBoundaryState(BCType, UPrim_boundary, UPrim_master, RefStatePrim, nv, t1, t2, C.cfg.kappa, C.cfg.R);
  if (BCType == 2 || BCType == 23 || BCType == 24 || BCType == 25 || BCType == 27) {
    for (int iv = 0; iv < 5; ++iv) Flux_loc[iv] = 0.5 * (UPrim_master[PRIM_LIFT[iv]] + UPrim_boundary[PRIM_LIFT[iv]]);
  } else if (BCType == 3 || BCType == 4) {
    Flux_loc[0] = UPrim_boundary[DENS];
    Flux_loc[1] = 0.; Flux_loc[2] = 0.; Flux_loc[3] = 0.;
    Flux_loc[4] = UPrim_boundary[TEMP];
  } else {  // 9, 91
    Flux_loc[0] = UPrim_master[DENS];
    for (int d = 0; d < 3; ++d) Flux_loc[1 + d] = UPrim_boundary[VEL1 + d];
    Flux_loc[4] = UPrim_master[TEMP];
  }
  if (!doWeakLifting)
    for (int iv = 0; iv < 5; ++iv) Flux_loc[iv] = Flux_loc[iv] - UPrim_master[PRIM_LIFT[iv]];
  for (int iv = 0; iv < 5; ++iv) Flux[iv] = Flux_loc[iv] * SurfElem;
}

// ---------------------------------------------------------------------------------------
// Operator pieces
// ---------------------------------------------------------------------------------------
// EvalElemFaceG/GL_Device (prolongtoface.t90:168-344): thread per (elem, locSide, p, q)
static void ProlongToFace_GPUorder(const Ctx& C, int nVar, const double* Uvol, double* Uface_master,
                                   double* Uface_slave) {
  const int N = C.B.N, n = C.n;
  const bool gauss = C.B.node_type == DG_NODETYPE_GAUSS;
#pragma omp parallel for schedule(static)
  for (int e = 0; e < C.M.nElems; ++e)
    for (int loc = 1; loc <= 6; ++loc)
      for (int p = 0; p <= N; ++p)
        for (int q = 0; q <= N; ++q) {
          int SideID = C.e2s(0, loc, e) - 1;
          int flip = C.e2s(1, loc, e);
          int i = C.s2v2(0, p, q, flip, loc), j = C.s2v2(1, p, q, flip, loc);
          double Uf[16];
          auto at = [&](int a, int b, int c, int v) { return Uvol[v + nVar * C.vol(a, b, c, e)]; };
          const double* Lv = (loc == XI_MINUS || loc == ETA_MINUS || loc == ZETA_MINUS) ? C.B.L_Minus.data()
                                                                                         : C.B.L_Plus.data();
          for (int v = 0; v < nVar; ++v) {
            double s;
            if (gauss) {
              switch (loc) {
                case XI_MINUS: case XI_PLUS:
                  s = at(0, i, j, v) * Lv[0]; for (int l = 1; l <= N; ++l) s = s + at(l, i, j, v) * Lv[l]; break;
                case ETA_MINUS: case ETA_PLUS:
                  s = at(i, 0, j, v) * Lv[0]; for (int l = 1; l <= N; ++l) s = s + at(i, l, j, v) * Lv[l]; break;
                default:
                  s = at(i, j, 0, v) * Lv[0]; for (int l = 1; l <= N; ++l) s = s + at(i, j, l, v) * Lv[l]; break;
              }
            } else {
              switch (loc) {
                case XI_MINUS: s = at(0, i, j, v); break;
                case ETA_MINUS: s = at(i, 0, j, v); break;
                case ZETA_MINUS: s = at(i, j, 0, v); break;
                case XI_PLUS: s = at(N, i, j, v); break;
                case ETA_PLUS: s = at(i, N, j, v); break;
                default: s = at(i, j, N, v); break;
              }
            }
            Uf[v] = s;
          }
          double* dst = (flip == 0) ? Uface_master : Uface_slave;
          for (int v = 0; v < nVar; ++v) dst[v + nVar * C.fac(p, q, SideID)] = Uf[v];
        }
}

// SurfInt_Device / SurfInt_Device_Single_Flux (surfint.t90:352-725): per DOF gather over locSide 1..6.
// mode 0: Flux_master / Flux_slave with master +, slave - (DG operator);
// mode 1: single flux, sig = +1 both sides (strong lifting); mode 2: single flux, sig = +-1 (weak lifting).
static void SurfInt_GPUorder(const Ctx& C, int nVar, const double* Flux_master, const double* Flux_slave, double* Ut,
                             int mode, bool doApplyJacobian) {
  const int N = C.B.N;
  const bool gauss = C.B.node_type == DG_NODETYPE_GAUSS;
  const double* Lm = C.B.L_HatMinus.data();
  const double* Lp = C.B.L_HatPlus.data();
#pragma omp parallel for schedule(static)
  for (int e = 0; e < C.M.nElems; ++e)
    for (int k = 0; k <= N; ++k)
      for (int j = 0; j <= N; ++j)
        for (int i = 0; i <= N; ++i) {
          double Ut_loc[16];
          for (int v = 0; v < nVar; ++v) Ut_loc[v] = 0.;
          for (int loc = 1; loc <= 6; ++loc) {
            int SideID = C.e2s(0, loc, e) - 1;
            int flip = C.e2s(1, loc, e);
            bool isMaster = flip == 0;
            int a, b, l;
            bool minus;
            switch (loc) {
              case XI_MINUS: a = j; b = k; l = i; minus = true; break;
              case ETA_MINUS: a = i; b = k; l = j; minus = true; break;
              case ZETA_MINUS: a = i; b = j; l = k; minus = true; break;
              case XI_PLUS: a = j; b = k; l = i; minus = false; break;
              case ETA_PLUS: a = i; b = k; l = j; minus = false; break;
              default: a = i; b = j; l = k; minus = false; break;
            }
            double Lhat;
            if (gauss) Lhat = minus ? Lm[l] : Lp[l];
            else {
              if (minus && l != 0) continue;
              if (!minus && l != N) continue;
              Lhat = minus ? Lm[0] : Lp[N];
            }
            // The GPU reference reads S2V2(:,a,b,flip,loc) here; the host reference (surfint.t90:59-104)
            // scatters with S2V2 and so gathers with its inverse.  The inverse is used (identical when
            // S2V2 is an involution, which holds for every flip/side combination of the meshes built here).
            int p = C.s2v2_inv(0, a, b, flip, loc), q = C.s2v2_inv(1, a, b, flip, loc);
            size_t f = C.fac(p, q, SideID);
            if (mode == 0) {
              if (isMaster) for (int v = 0; v < nVar; ++v) Ut_loc[v] = Ut_loc[v] + Flux_master[v + nVar * f] * Lhat;
              else for (int v = 0; v < nVar; ++v) Ut_loc[v] = Ut_loc[v] - Flux_slave[v + nVar * f] * Lhat;
            } else {
              double sig = 1.;
              if (mode == 2) sig = 2. * (double)C.e2s(2, loc, e) - 1.;
              for (int v = 0; v < nVar; ++v) Ut_loc[v] = Ut_loc[v] + sig * Flux_master[v + nVar * f] * Lhat;
            }
          }
          size_t id = C.vol(i, j, k, e);
          for (int v = 0; v < nVar; ++v) {
            if (doApplyJacobian) Ut[v + nVar * id] = C.M.sJ[id] * (Ut[v + nVar * id] + Ut_loc[v]);
            else Ut[v + nVar * id] = Ut[v + nVar * id] + Ut_loc[v];
          }
        }
}

struct Work {
  // LAF filter state per element (filter_vars.f90): lim, eRatio, r, ekin_avg_old, ekin_fluc_avg_old
  std::vector<double> lim, eRatio, r, ekin_avg_old, ekin_fluc_avg_old;
  std::vector<double> UPrim, U_master, U_slave, UPrim_master, UPrim_slave, Flux_master, Flux_slave;
  std::vector<double> gradUx, gradUy, gradUz, gx_m, gy_m, gz_m, gx_s, gy_s, gz_s, liftflux;
  std::vector<double> f, g, h;
};

static void alloc_work(const Ctx& C, Work& W) {
  size_t nDOF = (size_t)C.n3 * C.M.nElems, nF = (size_t)C.n2 * C.M.nSides;
  W.UPrim.assign(6 * nDOF, 0.);
  W.U_master.assign(5 * nF, 0.); W.U_slave.assign(5 * nF, 0.);
  W.UPrim_master.assign(6 * nF, 0.); W.UPrim_slave.assign(6 * nF, 0.);
  W.Flux_master.assign(5 * nF, 0.); W.Flux_slave.assign(5 * nF, 0.);
  W.f.assign(5 * nDOF, 0.); W.g.assign(5 * nDOF, 0.); W.h.assign(5 * nDOF, 0.);
  if (C.cfg.parabolic) {
    W.gradUx.assign(5 * nDOF, 0.); W.gradUy.assign(5 * nDOF, 0.); W.gradUz.assign(5 * nDOF, 0.);
    W.gx_m.assign(5 * nF, 0.); W.gy_m.assign(5 * nF, 0.); W.gz_m.assign(5 * nF, 0.);
    W.gx_s.assign(5 * nF, 0.); W.gy_s.assign(5 * nF, 0.); W.gz_s.assign(5 * nF, 0.);
    W.liftflux.assign(5 * nF, 0.);
  }
}

static inline double thermal_conductivity(const dg_config& c, double mu) {
  // THERMAL_CONDUCTIVITY_EOS  eos.h:110
  return mu * c.R * c.kappa / ((c.kappa - 1.) * c.Pr);
}

// Volume part of the lifting (gradients in physical space without the Jacobian factor)
static void Lifting_VolInt(const Ctx& C, Work& W, bool weak) {
  const int N = C.B.N, n = C.n;
  if (weak || C.cfg.do_conservative_lifting) {
    // Lifting_VolInt_Conservative  lifting_volint.t90:345-455
    const std::vector<double>& DM = weak ? C.B.D_Hat_T : C.B.D_T;
    double* grads[3] = {W.gradUx.data(), W.gradUy.data(), W.gradUz.data()};
    for (int dir = 0; dir < 3; ++dir) {
#pragma omp parallel for schedule(static)
      for (int e = 0; e < C.M.nElems; ++e) {
        std::vector<double> UEf(5 * C.n3), UEg(5 * C.n3), UEh(5 * C.n3);
        for (int k = 0; k <= N; ++k) for (int j = 0; j <= N; ++j) for (int i = 0; i <= N; ++i) {
          size_t id = C.vol(i, j, k, e);
          size_t lid = (size_t)i + n * (j + n * k);
          for (int iv = 0; iv < 5; ++iv) {
            double u = W.UPrim[PRIM_LIFT[iv] + 6 * id];
            UEf[iv + 5 * lid] = C.M.Mf[dir + 3 * id] * u;
            UEg[iv + 5 * lid] = C.M.Mg[dir + 3 * id] * u;
            UEh[iv + 5 * lid] = C.M.Mh[dir + 3 * id] * u;
          }
        }
        for (int k = 0; k <= N; ++k) for (int j = 0; j <= N; ++j) for (int i = 0; i <= N; ++i) {
          size_t id = C.vol(i, j, k, e);
          for (int iv = 0; iv < 5; ++iv) {
            auto L = [&](int a, int b, int c) { return (size_t)a + n * (b + n * c); };
            double s = DM[0 + n * i] * UEf[iv + 5 * L(0, j, k)] + DM[0 + n * k] * UEh[iv + 5 * L(i, j, 0)] +
                       DM[0 + n * j] * UEg[iv + 5 * L(i, 0, k)];
            for (int l = 1; l <= N; ++l)
              s = s + DM[l + n * i] * UEf[iv + 5 * L(l, j, k)] + DM[l + n * k] * UEh[iv + 5 * L(i, j, l)] +
                  DM[l + n * j] * UEg[iv + 5 * L(i, l, k)];
            grads[dir][iv + 5 * id] = s;
          }
        }
      }
    }
  } else {
    // Lifting_VolInt_Nonconservative_GPU_Kernel  lifting_volint.t90:262-328
    const double* DT = C.B.D_T.data();
#pragma omp parallel for schedule(static)
    for (int e = 0; e < C.M.nElems; ++e)
      for (int k = 0; k <= N; ++k) for (int j = 0; j <= N; ++j) for (int i = 0; i <= N; ++i) {
        double gxi[5] = {0, 0, 0, 0, 0}, geta[5] = {0, 0, 0, 0, 0}, gzeta[5] = {0, 0, 0, 0, 0};
        for (int l = 0; l <= N; ++l)
          for (int iv = 0; iv < 5; ++iv) {
            gxi[iv] = gxi[iv] + DT[l + n * i] * W.UPrim[PRIM_LIFT[iv] + 6 * C.vol(l, j, k, e)];
            geta[iv] = geta[iv] + DT[l + n * j] * W.UPrim[PRIM_LIFT[iv] + 6 * C.vol(i, l, k, e)];
            gzeta[iv] = gzeta[iv] + DT[l + n * k] * W.UPrim[PRIM_LIFT[iv] + 6 * C.vol(i, j, l, e)];
          }
        size_t id = C.vol(i, j, k, e);
        for (int iv = 0; iv < 5; ++iv) {
          W.gradUx[iv + 5 * id] = C.M.Mf[0 + 3 * id] * gxi[iv] + C.M.Mg[0 + 3 * id] * geta[iv] + C.M.Mh[0 + 3 * id] * gzeta[iv];
          W.gradUy[iv + 5 * id] = C.M.Mf[1 + 3 * id] * gxi[iv] + C.M.Mg[1 + 3 * id] * geta[iv] + C.M.Mh[1 + 3 * id] * gzeta[iv];
          W.gradUz[iv + 5 * id] = C.M.Mf[2 + 3 * id] * gxi[iv] + C.M.Mg[2 + 3 * id] * geta[iv] + C.M.Mh[2 + 3 * id] * gzeta[iv];
        }
      }
  }
}

// Lifting_BR1  src/dg/lifting/lifting_br1.t90:47-167 (no MPI)
static void Lifting_BR1(const Ctx& C, Work& W) {
  const int N = C.B.N, n = C.n;
  const size_t nF = (size_t)C.n2 * C.M.nSides;
  const bool weak = C.cfg.do_weak_lifting != 0;
  // Lifting_FillFlux_BC (lifting_fillflux.t90:109-140) on the BC sides, Lifting_FillFlux
  // (lifting_fillflux.t90:39-103) on the inner sides
  double sig = weak ? 1. : -1.;
  const long long nFbc = (long long)C.n2 * C.nBCSides;
#pragma omp parallel for schedule(static)
  for (long long fidx = 0; fidx < (long long)nF; ++fidx) {
    if (fidx < nFbc) {
      const int s = (int)(fidx / C.n2);
      Lifting_GetBoundaryFlux(C, &W.UPrim_master[6 * fidx], &C.M.nv[3 * fidx], &C.M.t1[3 * fidx], &C.M.t2[3 * fidx],
                              C.M.SurfElem[fidx], C.bctype[s], &C.refprim[6 * C.bcstate[s]], weak,
                              &W.liftflux[5 * fidx]);
      continue;
    }
    for (int iv = 0; iv < 5; ++iv)
      W.liftflux[iv + 5 * fidx] = 0.5 * C.M.SurfElem[fidx] *
                                  (sig * W.UPrim_master[PRIM_LIFT[iv] + 6 * fidx] + W.UPrim_slave[PRIM_LIFT[iv] + 6 * fidx]);
  }
  // Lifting_FillFlux_NormVec  lifting_fillflux.t90:212-256 (stored in gradU*_master)
#pragma omp parallel for schedule(static)
  for (long long fidx = 0; fidx < (long long)nF; ++fidx)
    for (int iv = 0; iv < 5; ++iv) {
      W.gx_m[iv + 5 * fidx] = W.liftflux[iv + 5 * fidx] * C.M.nv[0 + 3 * fidx];
      W.gy_m[iv + 5 * fidx] = W.liftflux[iv + 5 * fidx] * C.M.nv[1 + 3 * fidx];
      W.gz_m[iv + 5 * fidx] = W.liftflux[iv + 5 * fidx] * C.M.nv[2 + 3 * fidx];
    }
  Lifting_VolInt(C, W, weak);
  // SurfIntLifting with doApplyJacobian  (surfint.t90:295-347, 591-725)
  int mode = weak ? 2 : 1;
  SurfInt_GPUorder(C, 5, W.gx_m.data(), nullptr, W.gradUx.data(), mode, true);
  SurfInt_GPUorder(C, 5, W.gy_m.data(), nullptr, W.gradUy.data(), mode, true);
  SurfInt_GPUorder(C, 5, W.gz_m.data(), nullptr, W.gradUz.data(), mode, true);
  // ProlongToFaceLifting
  ProlongToFace_GPUorder(C, 5, W.gradUx.data(), W.gx_m.data(), W.gx_s.data());
  ProlongToFace_GPUorder(C, 5, W.gradUy.data(), W.gy_m.data(), W.gy_s.data());
  ProlongToFace_GPUorder(C, 5, W.gradUz.data(), W.gz_m.data(), W.gz_s.data());
  (void)n;
}

// Lifting_BR2 + Lifting_SurfInt_BR2  src/dg/lifting/lifting_br2.t90:43-310 (always strong form; no MPI,
// no mortars).  The volume gradient gets the same surface lifting as BR1; the face
// traces are the prolonged volume-only gradient plus etaBR2 times the lifting of that face's own jump.
static void Lifting_BR2(const Ctx& C, Work& W) {
  const int N = C.B.N;
  const size_t nF = (size_t)C.n2 * C.M.nSides, nDOF = (size_t)C.n3 * C.M.nElems;
  const bool gauss = C.B.node_type == DG_NODETYPE_GAUSS;
  // Lifting_FillFlux (strong: 0.5*SurfElem*(U_slave - U_master); BC sides: the strong boundary
  // lifting flux of Lifting_GetBoundaryFlux) and the normal components
  std::vector<double> FX(5 * nF), FY(5 * nF), FZ(5 * nF);
  const long long nFbc = (long long)C.n2 * C.nBCSides;
#pragma omp parallel for schedule(static)
  for (long long f = 0; f < (long long)nF; ++f) {
    double bfl[5];
    if (f < nFbc) {
      const int s = (int)(f / C.n2);
      Lifting_GetBoundaryFlux(C, &W.UPrim_master[6 * f], &C.M.nv[3 * f], &C.M.t1[3 * f], &C.M.t2[3 * f],
                              C.M.SurfElem[f], C.bctype[s], &C.refprim[6 * C.bcstate[s]], false, bfl);
    }
    for (int iv = 0; iv < 5; ++iv) {
      const double fl = f < nFbc ? bfl[iv]
                                 : 0.5 * C.M.SurfElem[f] * (-1. * W.UPrim_master[PRIM_LIFT[iv] + 6 * f] +
                                                            W.UPrim_slave[PRIM_LIFT[iv] + 6 * f]);
      FX[iv + 5 * f] = fl * C.M.nv[0 + 3 * f];
      FY[iv + 5 * f] = fl * C.M.nv[1 + 3 * f];
      FZ[iv + 5 * f] = fl * C.M.nv[2 + 3 * f];
    }
  }
  Lifting_VolInt(C, W, false);
  // ApplyJacobianLifting
#pragma omp parallel for schedule(static)
  for (long long id = 0; id < (long long)nDOF; ++id)
    for (int iv = 0; iv < 5; ++iv) {
      W.gradUx[iv + 5 * id] = W.gradUx[iv + 5 * id] * C.M.sJ[id];
      W.gradUy[iv + 5 * id] = W.gradUy[iv + 5 * id] * C.M.sJ[id];
      W.gradUz[iv + 5 * id] = W.gradUz[iv + 5 * id] * C.M.sJ[id];
    }
  // ProlongToFaceLifting of the volume-only gradients
  ProlongToFace_GPUorder(C, 5, W.gradUx.data(), W.gx_m.data(), W.gx_s.data());
  ProlongToFace_GPUorder(C, 5, W.gradUy.data(), W.gy_m.data(), W.gy_s.data());
  ProlongToFace_GPUorder(C, 5, W.gradUz.data(), W.gz_m.data(), W.gz_s.data());
  // Lifting_SurfInt_BR2: slave sides first, then master sides, sequentially in side order
  const double eta = C.cfg.eta_br2;
  const double* Flux[3] = {FX.data(), FY.data(), FZ.data()};
  double* grad[3] = {W.gradUx.data(), W.gradUy.data(), W.gradUz.data()};
  double* gm[3] = {W.gx_m.data(), W.gy_m.data(), W.gz_m.data()};
  double* gs[3] = {W.gx_s.data(), W.gy_s.data(), W.gz_s.data()};
  const int lmax = gauss ? N : 0;
  for (int d = 0; d < 3; ++d) {
    for (int pass = 0; pass < 2; ++pass) {
      for (int s = 0; s < C.M.nSides; ++s) {
        // SideToElem(S2E_ELEM_ID, S2E_NB_ELEM_ID, S2E_LOC_SIDE_ID, S2E_NB_LOC_SIDE_ID, S2E_FLIP), 1-based
        const int e = (pass == 0 ? C.s2e(1, s) : C.s2e(0, s)) - 1;
        if (e < 0) continue;
        const int loc = pass == 0 ? C.s2e(3, s) : C.s2e(2, s);
        const int flip = pass == 0 ? C.s2e(4, s) : 0;
        double* gface = pass == 0 ? gs[d] : gm[d];
        const bool minus = loc == XI_MINUS || loc == ETA_MINUS || loc == ZETA_MINUS;
        for (int q = 0; q <= N; ++q)
          for (int p = 0; p <= N; ++p) {
            const int a = C.s2v2(0, p, q, flip, loc), b = C.s2v2(1, p, q, flip, loc);
            const size_t f = C.fac(p, q, s);
            for (int l = 0; l <= lmax; ++l) {
              // CGNS_SideToVol: distance l from the face -> volume index along the normal
              const int lv = minus ? l : N - l;
              size_t id;
              if (loc == XI_MINUS || loc == XI_PLUS) id = C.vol(lv, a, b, e);
              else if (loc == ETA_MINUS || loc == ETA_PLUS) id = C.vol(a, lv, b, e);
              else id = C.vol(a, b, lv, e);
              for (int iv = 0; iv < 5; ++iv) {
                const double Floc = C.M.sJ[id] * Flux[d][iv + 5 * f] * C.B.L_HatMinus[l];
                grad[d][iv + 5 * id] = grad[d][iv + 5 * id] + Floc;
                gface[iv + 5 * f] = gface[iv + 5 * f] + eta * C.B.L_Minus[l] * Floc;
              }
            }
          }
      }
    }
  }
}

// ApplyDMatrix_Kernel  applydmatrix.t90:19-75
static void ApplyDMatrix_GPUorder(const Ctx& C, double* Ut, const double* f, const double* g, const double* h,
                                  bool doOverwrite) {
  const int N = C.B.N, n = C.n;
  const double* DHT = C.B.D_Hat_T.data();
#pragma omp parallel for schedule(static)
  for (int e = 0; e < C.M.nElems; ++e)
    for (int k = 0; k <= N; ++k) for (int j = 0; j <= N; ++j) for (int i = 0; i <= N; ++i) {
      double loc[5] = {0, 0, 0, 0, 0};
      for (int l = 0; l <= N; ++l)
        for (int v = 0; v < 5; ++v)
          loc[v] = loc[v] + DHT[l + n * i] * f[v + 5 * C.vol(l, j, k, e)] + DHT[l + n * k] * h[v + 5 * C.vol(i, j, l, e)] +
                   DHT[l + n * j] * g[v + 5 * C.vol(i, l, k, e)];
      size_t id = C.vol(i, j, k, e);
      for (int v = 0; v < 5; ++v) Ut[v + 5 * id] = doOverwrite ? loc[v] : Ut[v + 5 * id] + loc[v];
    }
}

// ---------------------------------------------------------------------------------------
// Filter: src/filter/filter.f90
// ---------------------------------------------------------------------------------------
// INVERSE (mathtools; LAPACK DGETRF/DGETRI in the reference): Gauss-Jordan elimination with partial
// pivoting, column-major n x n
static void INVERSE(int n, const std::vector<double>& A, std::vector<double>& Ainv) {
  std::vector<double> M(A);
  Ainv.assign(n * n, 0.);
  for (int i = 0; i < n; ++i) Ainv[i + n * i] = 1.;
  for (int c = 0; c < n; ++c) {
    int p = c;
    for (int r = c + 1; r < n; ++r) if (std::fabs(M[r + n * c]) > std::fabs(M[p + n * c])) p = r;
    if (p != c)
      for (int k = 0; k < n; ++k) { std::swap(M[c + n * k], M[p + n * k]); std::swap(Ainv[c + n * k], Ainv[p + n * k]); }
    const double d = M[c + n * c];
    for (int k = 0; k < n; ++k) { M[c + n * k] /= d; Ainv[c + n * k] /= d; }
    for (int r = 0; r < n; ++r) {
      if (r == c) continue;
      const double f = M[r + n * c];
      if (f == 0.) continue;
      for (int k = 0; k < n; ++k) { M[r + n * k] -= f * M[c + n * k]; Ainv[r + n * k] -= f * Ainv[c + n * k]; }
    }
  }
}

// buildLegendreVdm  basis.f90:100-160 (default branch: sVdm_Leg = INVERSE(Vdm_Leg))
static void buildLegendreVdm(int N_In, const double* xi_In, std::vector<double>& Vdm_Leg, std::vector<double>& sVdm_Leg) {
  const int n = N_In + 1;
  Vdm_Leg.assign(n * n, 0.);
  for (int i = 0; i <= N_In; ++i)
    for (int j = 0; j <= N_In; ++j) {
      double dummy;
      LegendrePolynomialAndDerivative(j, xi_In[i], Vdm_Leg[i + n * j], dummy);
    }
  INVERSE(n, Vdm_Leg, sVdm_Leg);
}

// InitializeVandermonde  basis.f90:168-186: Vdm(iXi,:) = l(xi_Out(iXi)), (0:N_Out,0:N_In)
static void InitializeVandermonde(int N_In, int N_Out, const double* wBary_In, const double* xi_In,
                                  const double* xi_Out, double* Vdm) {
  std::vector<double> row(N_In + 1);
  for (int iXi = 0; iXi <= N_Out; ++iXi) {
    LagrangeInterpolationPolys(xi_Out[iXi], N_In, xi_In, wBary_In, row.data());
    for (int j = 0; j <= N_In; ++j) Vdm[iXi + (N_Out + 1) * j] = row[j];
  }
}

// GetVandermonde  interpolation.f90:324-395 (column-major Vdm_In_Out(0:N_out,0:N_in), Vdm_Out_In(0:N_in,0:N_out))
static void GetVandermonde(int N_in, int nt_in, int N_out, int nt_out, double* Vdm_In_Out, double* Vdm_Out_In,
                           bool modal) {
  const int ni = N_in + 1, no = N_out + 1;
  if (nt_in == nt_out && N_in == N_out) {
    for (int t = 0; t < ni * ni; ++t) { Vdm_In_Out[t] = 0.; if (Vdm_Out_In) Vdm_Out_In[t] = 0.; }
    for (int i = 0; i < ni; ++i) { Vdm_In_Out[i + ni * i] = 1.; if (Vdm_Out_In) Vdm_Out_In[i + ni * i] = 1.; }
    return;
  }
  std::vector<double> xin(ni), xout(no), wbin(ni), wbout(no);
  GetNodesAndWeights(N_in, nt_in, xin.data(), nullptr, wbin.data());
  GetNodesAndWeights(N_out, nt_out, xout.data(), nullptr, wbout.data());
  std::vector<double> VLi, sVLi, VLo, sVLo;
  if (modal) {
    buildLegendreVdm(N_in, xin.data(), VLi, sVLi);
    buildLegendreVdm(N_out, xout.data(), VLo, sVLo);
  }
  if (N_out < N_in && modal) {
    // MATMUL(Vdm_Leg_Out(0:N_Out,0:N_Out), sVdm_Leg_In(0:N_Out,0:N_In))
    for (int i = 0; i < no; ++i)
      for (int j = 0; j < ni; ++j) {
        double acc = 0.;
        for (int k = 0; k < no; ++k) acc = acc + VLo[i + no * k] * sVLi[k + ni * j];
        Vdm_In_Out[i + no * j] = acc;
      }
  } else {
    InitializeVandermonde(N_in, N_out, wbin.data(), xin.data(), xout.data(), Vdm_In_Out);
  }
  if (Vdm_Out_In) {
    if (N_in < N_out && modal) {
      // MATMUL(Vdm_Leg_In(0:N_In,0:N_In), sVdm_Leg_Out(0:N_In,0:N_Out))
      for (int i = 0; i < ni; ++i)
        for (int j = 0; j < no; ++j) {
          double acc = 0.;
          for (int k = 0; k < ni; ++k) acc = acc + VLi[i + ni * k] * sVLo[k + no * j];
          Vdm_Out_In[i + ni * j] = acc;
        }
    } else {
      InitializeVandermonde(N_out, N_in, wbout.data(), xout.data(), xin.data(), Vdm_Out_In);
    }
  }
}

// ChangeBasis3D_XYZ  changeBasis.t90 (ChangeBasis3D :231-279 with one Vandermonde per direction):
// xi, eta, zeta sweeps, each output accumulated over the input index in increasing order
static void ChangeBasis3D_XYZ(int nVar, int NIn, int NOut, const double* Vx, const double* Vy, const double* Vz,
                              const double* X_In, double* X_Out) {
  const int ni = NIn + 1, no = NOut + 1;
  std::vector<double> B1((size_t)nVar * no * ni * ni, 0.), B2((size_t)nVar * no * no * ni, 0.);
  for (int kI = 0; kI < ni; ++kI) for (int jI = 0; jI < ni; ++jI) for (int iI = 0; iI < ni; ++iI)
    for (int iO = 0; iO < no; ++iO)
      for (int v = 0; v < nVar; ++v)
        B1[v + nVar * (iO + no * (jI + (size_t)ni * kI))] =
            B1[v + nVar * (iO + no * (jI + (size_t)ni * kI))] + Vx[iO + no * iI] * X_In[v + nVar * (iI + ni * (jI + (size_t)ni * kI))];
  for (int kI = 0; kI < ni; ++kI) for (int jI = 0; jI < ni; ++jI) for (int jO = 0; jO < no; ++jO)
    for (int iO = 0; iO < no; ++iO)
      for (int v = 0; v < nVar; ++v)
        B2[v + nVar * (iO + no * (jO + (size_t)no * kI))] =
            B2[v + nVar * (iO + no * (jO + (size_t)no * kI))] + Vy[jO + no * jI] * B1[v + nVar * (iO + no * (jI + (size_t)ni * kI))];
  for (size_t t = 0; t < (size_t)nVar * no * no * no; ++t) X_Out[t] = 0.;
  for (int kI = 0; kI < ni; ++kI) for (int kO = 0; kO < no; ++kO) for (int jO = 0; jO < no; ++jO)
    for (int iO = 0; iO < no; ++iO)
      for (int v = 0; v < nVar; ++v)
        X_Out[v + nVar * (iO + no * (jO + (size_t)no * kO))] =
            X_Out[v + nVar * (iO + no * (jO + (size_t)no * kO))] + Vz[kO + no * kI] * B2[v + nVar * (iO + no * (jO + (size_t)no * kI))];
}

// ---------------------------------------------------------------------------------------
// Geometry: src/mesh/metrics.f90 (BuildCoords, CalcMetrics, CalcSurfMetrics, SurfMetricsFromJa)
// for the default path of the reference: no octree (interpolateFromTree = F), curl-form metrics
// (crossProductMetrics = F, mesh.f90:65-67), 3D, no mortars.  Arrays in Fortran layout:
// NodeCoords(3,0:NGeo,0:NGeo,0:NGeo,nElems), XCL(3,0:N,0:N,0:N), dXCL(3,3,...) = (dd,nn),
// JaCL(3,3,...) = (dd,nn).
// ---------------------------------------------------------------------------------------
// ChangeBasis2D  changeBasis.t90:101-143 (Dim1 variables per node)
static void ChangeBasis2D(int Dim1, int NIn, int NOut, const double* Vdm, const double* X_In, double* X_Out) {
  const int ni = NIn + 1, no = NOut + 1;
  std::vector<double> B1((size_t)Dim1 * no * ni, 0.);
  for (int jI = 0; jI < ni; ++jI) for (int iI = 0; iI < ni; ++iI)
    for (int iO = 0; iO < no; ++iO)
      for (int v = 0; v < Dim1; ++v)
        B1[v + Dim1 * (iO + no * jI)] = B1[v + Dim1 * (iO + no * jI)] + Vdm[iO + no * iI] * X_In[v + Dim1 * (iI + ni * jI)];
  for (size_t t = 0; t < (size_t)Dim1 * no * no; ++t) X_Out[t] = 0.;
  for (int jI = 0; jI < ni; ++jI) for (int jO = 0; jO < no; ++jO)
    for (int iO = 0; iO < no; ++iO)
      for (int v = 0; v < Dim1; ++v)
        X_Out[v + Dim1 * (iO + no * jO)] = X_Out[v + Dim1 * (iO + no * jO)] + Vdm[jO + no * jI] * B1[v + Dim1 * (iO + no * jI)];
}
// ChangeBasisVolume = ChangeBasis3D (changeBasis.t90:237-283): one Vandermonde in all three directions
static void ChangeBasis3D(int Dim1, int NIn, int NOut, const double* Vdm, const double* X_In, double* X_Out) {
  ChangeBasis3D_XYZ(Dim1, NIn, NOut, Vdm, Vdm, Vdm, X_In, X_Out);
}
// GetDerivativeMatrix  interpolation.f90:401-416
static void GetDerivativeMatrix(int N_in, int node_type, double* D) {
  std::vector<double> x(N_in + 1);
  GetNodesAndWeights(N_in, node_type, x.data(), nullptr, nullptr);
  PolynomialDerivativeMatrix(N_in, x.data(), D);
}

static const int kNormalDirs[7] = {0, 3, 2, 1, 2, 1, 3};           // mesh_vars.f90:111 (1-based local side)
static const int kTangDirs[7] = {0, 1, 3, 2, 3, 2, 1};             // mesh_vars.f90:113
static const double kNormalSigns[7] = {0., -1., -1., 1., 1., -1., 1.};  // mesh_vars.f90:118

// SurfMetricsFromJa  metrics.f90:752-789 for one side: Ja_Face(3,3,0:N,0:N) -> NormVec, TangVec1,
// TangVec2 (3,0:N,0:N), SurfElem (0:N,0:N)
static void SurfMetricsFromJa(int Nloc, int NormalDir, int TangDir, double NormalSign, const double* Ja_Face,
                              double* NormVec, double* TangVec1, double* TangVec2, double* SurfElem) {
  const int n = Nloc + 1;
  auto J = [&](int dd, int nn, int p, int q) { return Ja_Face[(dd - 1) + 3 * ((nn - 1) + 3 * (p + n * q))]; };
  for (int q = 0; q <= Nloc; ++q)
    for (int p = 0; p <= Nloc; ++p) {
      const size_t f = (size_t)p + n * q;
      double s = 0.;
      for (int c = 1; c <= 3; ++c) s = s + sq(J(NormalDir, c, p, q));
      SurfElem[f] = std::sqrt(s);
      double* nv = NormVec + 3 * f;
      for (int c = 1; c <= 3; ++c) nv[c - 1] = NormalSign * J(NormalDir, c, p, q) / SurfElem[f];
      double dot = 0.;
      for (int c = 1; c <= 3; ++c) dot = dot + J(TangDir, c, p, q) * nv[c - 1];
      double* t1 = TangVec1 + 3 * f;
      for (int c = 1; c <= 3; ++c) t1[c - 1] = J(TangDir, c, p, q) - dot * nv[c - 1];
      double tn = 0.;
      for (int c = 0; c < 3; ++c) tn = tn + sq(t1[c]);
      tn = std::sqrt(tn);
      for (int c = 0; c < 3; ++c) t1[c] = t1[c] / tn;
      double* t2 = TangVec2 + 3 * f;  // CROSS (mathtools.f90:153-165)
      t2[0] = nv[1] * t1[2] - nv[2] * t1[1];
      t2[1] = nv[2] * t1[0] - nv[0] * t1[2];
      t2[2] = nv[0] * t1[1] - nv[1] * t1[0];
    }
}

// Volume node of the face-plane position (a,b) of local side iLocSide (the planes of metrics.f90:663-676)
static size_t face_plane_node(int Nloc, int iLocSide, int a, int b) {
  const int n = Nloc + 1;
  int i, j, k;
  switch (iLocSide) {
    case XI_MINUS: i = 0; j = a; k = b; break;
    case XI_PLUS: i = Nloc; j = a; k = b; break;
    case ETA_MINUS: i = a; j = 0; k = b; break;
    case ETA_PLUS: i = a; j = Nloc; k = b; break;
    case ZETA_MINUS: i = a; j = b; k = 0; break;
    default: i = a; j = b; k = Nloc; break;
  }
  return (size_t)i + n * (j + (size_t)n * k);
}

struct MetricsOut {
  double *Elem_xGP, *Mf, *Mg, *Mh, *sJ, *NormVec, *TangVec1, *TangVec2, *SurfElem, *Face_xGP;
};

// BuildCoords (metrics.f90:85-160) + CalcMetrics (:171-560) + CalcSurfMetrics (:596-750); returns the
// number of solution nodes with a scaled Jacobian below 0.01 (the reference aborts on those,
// metrics.f90:345-352) or -1 for a negative one
static int CalcMetrics(int N, int NodeType, int NGeo, int nElems, const double* NodeCoords, const int* ElemToSide,
                       const MetricsOut& o) {
  const int NGeoRef = 3 * NGeo;  // mesh.f90:370
  const int n = N + 1, g = NGeo + 1, r = NGeoRef + 1, n3 = n * n * n, g3 = g * g * g, r3 = r * r * r;
  const int CL = 3, VISU = 4;
  // 1.a-1.f, 2., 2.d: Vandermonde and derivative matrices (column-major (0:N_out,0:N_in))
  std::vector<double> Vdm_EQNGeo_CLNGeo(g * g), Vdm_CLNGeo_CLN(n * g), DCL_NGeo(g * g), Vdm_CLNGeo_NGeoRef(r * g),
      Vdm_NGeoRef_N(n * r), DCL_N(n * n), Vdm_CLN_N(n * n);
  GetVandermonde(NGeo, VISU, NGeo, CL, Vdm_EQNGeo_CLNGeo.data(), nullptr, false);
  GetVandermonde(NGeo, CL, N, CL, Vdm_CLNGeo_CLN.data(), nullptr, false);
  GetDerivativeMatrix(NGeo, CL, DCL_NGeo.data());
  GetVandermonde(NGeo, CL, NGeoRef, NodeType, Vdm_CLNGeo_NGeoRef.data(), nullptr, false);
  GetVandermonde(NGeoRef, NodeType, N, NodeType, Vdm_NGeoRef_N.data(), nullptr, true);
  GetDerivativeMatrix(N, CL, DCL_N.data());
  GetVandermonde(N, CL, N, NodeType, Vdm_CLN_N.data(), nullptr, false);
  // BuildCoords: Vdm_EQNGeo_CLNloc = MATMUL(Vdm_CLNloc_Nloc, Vdm_EQNGeo_CLNloc)
  std::vector<double> Vdm_EQNGeo_CLNloc(n * g), Vdm_BC(n * g), Vdm_CLNloc_Nloc(n * n);
  GetVandermonde(NGeo, VISU, N, CL, Vdm_EQNGeo_CLNloc.data(), nullptr, false);
  GetVandermonde(N, CL, N, NodeType, Vdm_CLNloc_Nloc.data(), nullptr, false);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < g; ++j) {
      double acc = 0.;
      for (int k = 0; k < n; ++k) acc = acc + Vdm_CLNloc_Nloc[i + n * k] * Vdm_EQNGeo_CLNloc[k + n * j];
      Vdm_BC[i + n * j] = acc;
    }
  int bad = 0;
  std::vector<double> XCL_NGeo(3 * g3), XCL_N(3 * n3), dXCL_NGeo(9 * g3), dX_NGeoRef(9 * r3), detJac_Ref(r3),
      DetJac_N(n3), dXCL_N(9 * n3), R_CL_N(9 * n3), JaCL_N(9 * n3), slice_g(3 * g3), slice_r(3 * r3), slice_n(3 * n3);
  std::vector<double> tmp(3 * n * n), tmp2(3 * n * n), Ja_Face_l(9 * n * n);
  auto G = [&](int i, int j, int k) { return (size_t)i + g * (j + (size_t)g * k); };
  auto NI = [&](int i, int j, int k) { return (size_t)i + n * (j + (size_t)n * k); };
  for (int iElem = 0; iElem < nElems; ++iElem) {
    const double* NC = NodeCoords + (size_t)3 * g3 * iElem;
    if (o.Elem_xGP) ChangeBasis3D(3, NGeo, N, Vdm_BC.data(), NC, o.Elem_xGP + (size_t)3 * n3 * iElem);
    // 1.a, 1.b
    ChangeBasis3D(3, NGeo, NGeo, Vdm_EQNGeo_CLNGeo.data(), NC, XCL_NGeo.data());
    ChangeBasis3D(3, NGeo, N, Vdm_CLNGeo_CLN.data(), XCL_NGeo.data(), XCL_N.data());
    // 1.c dXCL_NGeo(dd,nn,i,j,k)
    std::fill(dXCL_NGeo.begin(), dXCL_NGeo.end(), 0.);
    for (int k = 0; k < g; ++k) for (int j = 0; j < g; ++j) for (int i = 0; i < g; ++i) {
      double* d = &dXCL_NGeo[9 * G(i, j, k)];
      for (int ll = 0; ll < g; ++ll)
        for (int nn = 0; nn < 3; ++nn) {
          d[0 + 3 * nn] = d[0 + 3 * nn] + DCL_NGeo[i + g * ll] * XCL_NGeo[nn + 3 * G(ll, j, k)];
          d[1 + 3 * nn] = d[1 + 3 * nn] + DCL_NGeo[j + g * ll] * XCL_NGeo[nn + 3 * G(i, ll, k)];
          d[2 + 3 * nn] = d[2 + 3 * nn] + DCL_NGeo[k + g * ll] * XCL_NGeo[nn + 3 * G(i, j, ll)];
        }
    }
    // 1.d dX_NGeoRef(:,nn,...) = ChangeBasisVolume of dXCL_NGeo(:,nn,...)
    for (int nn = 0; nn < 3; ++nn) {
      for (int t = 0; t < g3; ++t)
        for (int dd = 0; dd < 3; ++dd) slice_g[dd + 3 * t] = dXCL_NGeo[dd + 3 * nn + 9 * t];
      ChangeBasis3D(3, NGeo, NGeoRef, Vdm_CLNGeo_NGeoRef.data(), slice_g.data(), slice_r.data());
      for (int t = 0; t < r3; ++t)
        for (int dd = 0; dd < 3; ++dd) dX_NGeoRef[dd + 3 * nn + 9 * t] = slice_r[dd + 3 * t];
    }
    // 1.e detJac_Ref (left to right, from the initial 0)
    for (int t = 0; t < r3; ++t) {
      auto X = [&](int a, int b) { return dX_NGeoRef[(a - 1) + 3 * (b - 1) + 9 * t]; };
      detJac_Ref[t] = 0. + X(1, 1) * (X(2, 2) * X(3, 3) - X(3, 2) * X(2, 3)) +
                      X(2, 1) * (X(3, 2) * X(1, 3) - X(1, 2) * X(3, 3)) + X(3, 1) * (X(1, 2) * X(2, 3) - X(2, 2) * X(1, 3));
    }
    // 1.f modal projection NGeoRef -> N, sJ, scaled-Jacobian check
    ChangeBasis3D(1, NGeoRef, N, Vdm_NGeoRef_N.data(), detJac_Ref.data(), DetJac_N.data());
    double mx = DetJac_N[0];
    for (int t = 1; t < n3; ++t) mx = std::max(mx, DetJac_N[t]);
    for (int t = 0; t < n3; ++t) {
      o.sJ[(size_t)n3 * iElem + t] = 1. / DetJac_N[t];
      if (DetJac_N[t] <= 0.) bad = -1;
      else if (bad >= 0 && DetJac_N[t] / mx < 0.01) bad++;
    }
    // 2.a dXCL_N
    std::fill(dXCL_N.begin(), dXCL_N.end(), 0.);
    if (N >= NGeo) {
      for (int nn = 0; nn < 3; ++nn) {
        for (int t = 0; t < g3; ++t)
          for (int dd = 0; dd < 3; ++dd) slice_g[dd + 3 * t] = dXCL_NGeo[dd + 3 * nn + 9 * t];
        ChangeBasis3D(3, NGeo, N, Vdm_CLNGeo_CLN.data(), slice_g.data(), slice_n.data());
        for (int t = 0; t < n3; ++t)
          for (int dd = 0; dd < 3; ++dd) dXCL_N[dd + 3 * nn + 9 * t] = slice_n[dd + 3 * t];
      }
    } else {
      for (int k = 0; k < n; ++k) for (int j = 0; j < n; ++j) for (int i = 0; i < n; ++i) {
        double* d = &dXCL_N[9 * NI(i, j, k)];
        for (int ll = 0; ll < n; ++ll)
          for (int nn = 0; nn < 3; ++nn) {
            d[0 + 3 * nn] = d[0 + 3 * nn] + DCL_N[i + n * ll] * XCL_N[nn + 3 * NI(ll, j, k)];
            d[1 + 3 * nn] = d[1 + 3 * nn] + DCL_N[j + n * ll] * XCL_N[nn + 3 * NI(i, ll, k)];
            d[2 + 3 * nn] = d[2 + 3 * nn] + DCL_N[k + n * ll] * XCL_N[nn + 3 * NI(i, j, ll)];
          }
      }
    }
    // 2.b curl form: R_CL_N(dd,nn) = 1/2 (XCL_N x d/dxi_dd XCL_N)_nn, JaCL_N = -(curl R)
    for (int t = 0; t < n3; ++t) {
      const double* x = &XCL_N[3 * t];
      const double* d = &dXCL_N[9 * t];
      double* R = &R_CL_N[9 * t];
      for (int dd = 0; dd < 3; ++dd) {
        R[dd + 3 * 0] = 0.5 * (x[2] * d[dd + 3 * 1] - x[1] * d[dd + 3 * 2]);
        R[dd + 3 * 1] = 0.5 * (x[0] * d[dd + 3 * 2] - x[2] * d[dd + 3 * 0]);
        R[dd + 3 * 2] = 0.5 * (x[1] * d[dd + 3 * 0] - x[0] * d[dd + 3 * 1]);
      }
    }
    std::fill(JaCL_N.begin(), JaCL_N.end(), 0.);
    for (int k = 0; k < n; ++k) for (int j = 0; j < n; ++j) for (int i = 0; i < n; ++i) {
      double* Ja = &JaCL_N[9 * NI(i, j, k)];
      for (int q = 0; q < n; ++q)
        for (int nn = 0; nn < 3; ++nn) {
          Ja[0 + 3 * nn] = Ja[0 + 3 * nn] - DCL_N[j + n * q] * R_CL_N[2 + 3 * nn + 9 * NI(i, q, k)];
          Ja[1 + 3 * nn] = Ja[1 + 3 * nn] - DCL_N[k + n * q] * R_CL_N[0 + 3 * nn + 9 * NI(i, j, q)];
          Ja[2 + 3 * nn] = Ja[2 + 3 * nn] - DCL_N[i + n * q] * R_CL_N[1 + 3 * nn + 9 * NI(q, j, k)];
        }
      for (int q = 0; q < n; ++q)
        for (int nn = 0; nn < 3; ++nn) {
          Ja[0 + 3 * nn] = Ja[0 + 3 * nn] + DCL_N[k + n * q] * R_CL_N[1 + 3 * nn + 9 * NI(i, j, q)];
          Ja[1 + 3 * nn] = Ja[1 + 3 * nn] + DCL_N[i + n * q] * R_CL_N[2 + 3 * nn + 9 * NI(q, j, k)];
          Ja[2 + 3 * nn] = Ja[2 + 3 * nn] + DCL_N[j + n * q] * R_CL_N[0 + 3 * nn + 9 * NI(i, q, k)];
        }
    }
    // 2.c Metrics_fTilde/gTilde/hTilde = ChangeBasisVolume(Vdm_CLN_N) of JaCL_N(dd,1:3,...)
    double* outs[3] = {o.Mf, o.Mg, o.Mh};
    for (int dd = 0; dd < 3; ++dd) {
      for (int t = 0; t < n3; ++t)
        for (int nn = 0; nn < 3; ++nn) slice_n[nn + 3 * t] = JaCL_N[dd + 3 * nn + 9 * t];
      ChangeBasis3D(3, N, N, Vdm_CLN_N.data(), slice_n.data(), outs[dd] + (size_t)3 * n3 * iElem);
    }
    // CalcSurfMetrics: master sides (flip 0) of this element
    for (int iLocSide = 1; iLocSide <= 6; ++iLocSide) {
      const int* es = ElemToSide + 3 * ((iLocSide - 1) + 6 * (size_t)iElem);
      if (es[1] != 0) continue;
      const size_t SideID = (size_t)es[0] - 1;
      auto sidemap = [&](int p, int q, int& a, int& b) { SideToVol2(N, p, q, 0, iLocSide, a, b); };
      if (o.Face_xGP) {
        for (int b = 0; b < n; ++b) for (int a = 0; a < n; ++a)
          for (int c = 0; c < 3; ++c) tmp[c + 3 * (a + n * b)] = XCL_N[c + 3 * face_plane_node(N, iLocSide, a, b)];
        ChangeBasis2D(3, N, N, Vdm_CLN_N.data(), tmp.data(), tmp2.data());
        for (int q = 0; q < n; ++q) for (int p = 0; p < n; ++p) {
          int a, b;
          sidemap(p, q, a, b);
          for (int c = 0; c < 3; ++c) o.Face_xGP[c + 3 * (p + n * (q + (size_t)n * SideID))] = tmp2[c + 3 * (a + n * b)];
        }
      }
      std::fill(Ja_Face_l.begin(), Ja_Face_l.end(), 0.);
      for (int dd = 0; dd < 3; ++dd) {
        for (int b = 0; b < n; ++b) for (int a = 0; a < n; ++a)
          for (int nn = 0; nn < 3; ++nn) tmp[nn + 3 * (a + n * b)] = JaCL_N[dd + 3 * nn + 9 * face_plane_node(N, iLocSide, a, b)];
        ChangeBasis2D(3, N, N, Vdm_CLN_N.data(), tmp.data(), tmp2.data());
        for (int q = 0; q < n; ++q) for (int p = 0; p < n; ++p) {
          int a, b;
          sidemap(p, q, a, b);
          for (int nn = 0; nn < 3; ++nn) Ja_Face_l[dd + 3 * (nn + 3 * (p + n * q))] = tmp2[nn + 3 * (a + n * b)];
        }
      }
      const size_t f0 = (size_t)n * n * SideID;
      SurfMetricsFromJa(N, kNormalDirs[iLocSide], kTangDirs[iLocSide], kNormalSigns[iLocSide], Ja_Face_l.data(),
                        o.NormVec + 3 * f0, o.TangVec1 + 3 * f0, o.TangVec2 + 3 * f0, o.SurfElem + f0);
    }
  }
  return bad;
}

// InitFilter (filter.f90:100-222) with HestFilter (:231-263) and buildLegendreVdm (basis.f90:100-160)
static int InitFilter(Ctx& C) {
  const dg_config& c = C.cfg;
  if (c.filter_type == DG_FILTER_NONE) return 0;
  const int N = C.B.N, n = N + 1;
  std::vector<double> Fd(n * n, 0.);
  if (c.filter_type == DG_FILTER_CUTOFF || c.filter_type == DG_FILTER_LAF) {
    if (c.n_filter < 0 || c.n_filter > N) return -1;
    for (int iDeg = 0; iDeg <= c.n_filter; ++iDeg) Fd[iDeg + n * iDeg] = 1.;
  } else if (c.filter_type == DG_FILTER_MODAL) {
    const double alpha = c.hest_filter_param[0], sExp = c.hest_filter_param[1];
    const double etac = c.hest_filter_param[2] / (double)(N + 1);
    for (int iDeg = 0; iDeg <= std::min((int)c.hest_filter_param[2] - 1, N); ++iDeg) Fd[iDeg + n * iDeg] = 1.;
    if (alpha >= 0.)
      for (int iDeg = (int)c.hest_filter_param[2]; iDeg <= N; ++iDeg) {
        const double eta = (double)(iDeg + 1) / (double)(N + 1);
        Fd[iDeg + n * iDeg] = std::exp(-alpha * std::pow((eta - etac) / (1. - etac), sExp));
      }
  } else {
    return -1;
  }
  std::vector<double> Vdm_Leg, sVdm_Leg;
  buildLegendreVdm(N, C.B.xGP.data(), Vdm_Leg, sVdm_Leg);
  // FilterMat = MATMUL(MATMUL(Vdm_Leg, FilterMat), sVdm_Leg)
  std::vector<double> T(n * n, 0.);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      double acc = 0.;
      for (int k = 0; k < n; ++k) acc = acc + Vdm_Leg[i + n * k] * Fd[k + n * j];
      T[i + n * j] = acc;
    }
  C.FilterMat.assign(n * n, 0.);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      double acc = 0.;
      for (int k = 0; k < n; ++k) acc = acc + T[i + n * k] * sVdm_Leg[k + n * j];
      C.FilterMat[i + n * j] = acc;
    }
  if (c.filter_type == DG_FILTER_LAF) {
    const int n3 = C.n3;
    C.IntegrationWeight.assign((size_t)n3 * C.M.nElems, 0.);
    for (int e = 0; e < C.M.nElems; ++e) {
      double Vol = 0.;
      for (int k = 0; k <= N; ++k) for (int j = 0; j <= N; ++j) for (int i = 0; i <= N; ++i) {
        const size_t id = C.vol(i, j, k, e);
        C.IntegrationWeight[id] = C.B.wGP[i] * C.B.wGP[j] * C.B.wGP[k] / C.M.sJ[id];
        Vol = Vol + C.IntegrationWeight[id];
      }
      for (int t = 0; t < n3; ++t) C.IntegrationWeight[(size_t)e * n3 + t] = C.IntegrationWeight[(size_t)e * n3 + t] / Vol;
    }
    C.normMod = (std::pow((double)c.n_filter + 1, -2. / 3.) - std::pow(2., -2. / 3.)) /
                (std::pow((double)(N + 1), -2. / 3.) - std::pow((double)(c.n_filter + 1), -2. / 3.));
  }
  return 0;
}

// one element through the three 1D sweeps xi, eta, zeta (Filter -> ChangeBasis3D_GPU,
// changeBasis.t90:287-359; same accumulation order as the host ChangeBasis3D)
static void filter_element(const Ctx& C, const double* Uin, double* Uout) {
  const double* F = C.FilterMat.data();
  ChangeBasis3D_XYZ(5, C.B.N, C.B.N, F, F, F, Uin, Uout);
}

// Filter (filter.f90:272-311) or Filter_LAF (filter.f90:318-474), in place
static void ApplyFilter(const Ctx& C, Work& W, double* U) {
  const int n3 = C.n3;
  if (C.cfg.filter_type != DG_FILTER_LAF) {
#pragma omp parallel for schedule(static)
    for (int e = 0; e < C.M.nElems; ++e) {
      std::vector<double> Uf(5 * n3);
      filter_element(C, &U[(size_t)5 * n3 * e], Uf.data());
      std::memcpy(&U[(size_t)5 * n3 * e], Uf.data(), sizeof(double) * 5 * n3);
    }
    return;
  }
  const double LAF_alpha = C.cfg.laf_alpha;
#pragma omp parallel for schedule(static)
  for (int e = 0; e < C.M.nElems; ++e) {
    double* Ue = &U[(size_t)5 * n3 * e];
    const double* IW = &C.IntegrationWeight[(size_t)n3 * e];
    std::vector<double> Uf(5 * n3);
    filter_element(C, Ue, Uf.data());
    double U_Avg[5] = {0., 0., 0., 0., 0.};
    for (int t = 0; t < n3; ++t)
      for (int c = 1; c <= 3; ++c) U_Avg[c] = U_Avg[c] + Uf[c + 5 * t] / Ue[0 + 5 * t] * IW[t];
    double ekin_avg = 0., ekin_fluc_avg = 0.;
    for (int t = 0; t < n3; ++t) {
      const double r2 = Ue[5 * t] * Ue[5 * t];
      const double f1 = Ue[1 + 5 * t] - Uf[1 + 5 * t], f2 = Ue[2 + 5 * t] - Uf[2 + 5 * t], f3 = Ue[3 + 5 * t] - Uf[3 + 5 * t];
      ekin_fluc_avg = ekin_fluc_avg + (f1 * f1 / r2 + f3 * f3 / r2 + f2 * f2 / r2) * IW[t];
      ekin_avg = ekin_avg + ((Uf[1 + 5 * t] - U_Avg[1]) * (Uf[1 + 5 * t] - U_Avg[1]) / r2 +
                             (Uf[2 + 5 * t] - U_Avg[2]) * (Uf[2 + 5 * t] - U_Avg[2]) / r2 +
                             (Uf[3 + 5 * t] - U_Avg[3]) * (Uf[3 + 5 * t] - U_Avg[3]) / r2) * IW[t];
    }
    W.eRatio[e] = (ekin_fluc_avg / ekin_avg) * C.normMod;
    W.lim[e] = std::max(W.lim[e], 1.0E-8);
    const double dedt_lim = std::fabs(ekin_avg - W.ekin_avg_old[e]) / ((ekin_fluc_avg - W.ekin_fluc_avg_old[e]));
    if ((dedt_lim > 1.0) && ((ekin_fluc_avg - W.ekin_fluc_avg_old[e]) > 0.)) {
      W.lim[e] = W.eRatio[e];
    } else if ((ekin_fluc_avg - W.ekin_fluc_avg_old[e]) < 0.) {
      W.lim[e] = W.eRatio[e];
    } else if (W.eRatio[e] > W.lim[e] * LAF_alpha) {
      std::memcpy(Ue, Uf.data(), sizeof(double) * 5 * n3);
      W.r[e] = W.r[e] + 1.;
    }
    W.ekin_avg_old[e] = ekin_avg;
    W.ekin_fluc_avg_old[e] = ekin_fluc_avg;
  }
}

// DGTimeDerivative_weakForm  src/dg/dg.f90:255-425 (periodic/inner sides, no MPI, no filter/source)
static void DGTimeDerivative(const Ctx& C, Work& W, double* U, double* Ut) {
  const dg_config& cfg = C.cfg;
  const int N = C.B.N, n = C.n;
  const size_t nDOF = (size_t)C.n3 * C.M.nElems, nF = (size_t)C.n2 * C.M.nSides;
  const double Kappa = cfg.kappa, R = cfg.R;
  // 1. Filter the solution vector, in place
  if (cfg.filter_type != DG_FILTER_NONE) ApplyFilter(C, W, U);
  // 2. ProlongToFaceCons
  ProlongToFace_GPUorder(C, 5, U, W.U_master.data(), W.U_slave.data());
  // 3. ConsToPrim volume
#pragma omp parallel for schedule(static)
  for (long long id = 0; id < (long long)nDOF; ++id) ConsToPrim(&W.UPrim[6 * id], &U[5 * id], Kappa, R);
  // 5. GetPrimitiveStateSurface (version 1: prims of prolonged conservative traces)
  // (BC sides, the first nBCSides, have no slave element)
  const long long nFbc = (long long)C.n2 * C.nBCSides;
#pragma omp parallel for schedule(static)
  for (long long f = 0; f < (long long)nF; ++f) {
    ConsToPrim(&W.UPrim_master[6 * f], &W.U_master[5 * f], Kappa, R);
    if (f >= nFbc) ConsToPrim(&W.UPrim_slave[6 * f], &W.U_slave[5 * f], Kappa, R);
  }
  // 6. Lifting
  if (cfg.parabolic) {
    if (cfg.lifting == DG_LIFTING_BR2) Lifting_BR2(C, W);
    else Lifting_BR1(C, W);
  }
  // 8. VolInt
  const double mu = cfg.mu0, lambda = thermal_conductivity(cfg, cfg.mu0);
  if (cfg.split_dg < 0) {
    // VolInt_weakForm  volint.f90:129-188 -> EvalTransformedFlux3D_Kernel flux.f90:304-345 -> ApplyDMatrix
#pragma omp parallel for schedule(static)
    for (long long id = 0; id < (long long)nDOF; ++id) {
      if (cfg.parabolic)
        EvalTransformedEulerDiffFlux3D(&U[5 * id], &W.UPrim[6 * id], &W.gradUx[5 * id], &W.gradUy[5 * id],
                                       &W.gradUz[5 * id], &W.f[5 * id], &W.g[5 * id], &W.h[5 * id], &C.M.Mf[3 * id],
                                       &C.M.Mg[3 * id], &C.M.Mh[3 * id], mu, lambda);
      else
        EvalTransformedEulerFlux3D_fast(&U[5 * id], &W.UPrim[6 * id], &W.f[5 * id], &W.g[5 * id], &W.h[5 * id],
                                        &C.M.Mf[3 * id], &C.M.Mg[3 * id], &C.M.Mh[3 * id]);
    }
    ApplyDMatrix_GPUorder(C, Ut, W.f.data(), W.g.data(), W.h.data(), true);
  } else {
    // VolInt_splitForm  volint.f90:211-244: viscous weak part first (overwrite), then the split kernel adds
    if (cfg.parabolic) {
#pragma omp parallel for schedule(static)
      for (long long id = 0; id < (long long)nDOF; ++id)
        EvalTransformedDiffFlux3D(&W.UPrim[6 * id], &W.gradUx[5 * id], &W.gradUy[5 * id], &W.gradUz[5 * id],
                                  &W.f[5 * id], &W.g[5 * id], &W.h[5 * id], &C.M.Mf[3 * id], &C.M.Mg[3 * id],
                                  &C.M.Mh[3 * id], mu, lambda);
      ApplyDMatrix_GPUorder(C, Ut, W.f.data(), W.g.data(), W.h.data(), true);
    }
    // VolInt_splitForm_Kernel  volint.f90:265-353
    const double* DVS = C.B.DVolSurf.data();
#pragma omp parallel for schedule(static)
    for (int e = 0; e < C.M.nElems; ++e)
      for (int k = 0; k <= N; ++k) for (int j = 0; j <= N; ++j) for (int i = 0; i <= N; ++i) {
        double tmp[5] = {0, 0, 0, 0, 0}, F[5];
        size_t id = C.vol(i, j, k, e);
        for (int l = 0; l <= N; ++l) {
          size_t ld = C.vol(l, j, k, e);
          SplitVolumeFlux(cfg.split_dg, &U[5 * id], &W.UPrim[6 * id], &U[5 * ld], &W.UPrim[6 * ld], &C.M.Mf[3 * id],
                          &C.M.Mf[3 * ld], F);
          for (int v = 0; v < 5; ++v) tmp[v] = tmp[v] + DVS[l + n * i] * F[v];
        }
        for (int l = 0; l <= N; ++l) {
          size_t ld = C.vol(i, l, k, e);
          SplitVolumeFlux(cfg.split_dg, &U[5 * id], &W.UPrim[6 * id], &U[5 * ld], &W.UPrim[6 * ld], &C.M.Mg[3 * id],
                          &C.M.Mg[3 * ld], F);
          for (int v = 0; v < 5; ++v) tmp[v] = tmp[v] + DVS[l + n * j] * F[v];
        }
        for (int l = 0; l <= N; ++l) {
          size_t ld = C.vol(i, j, l, e);
          SplitVolumeFlux(cfg.split_dg, &U[5 * id], &W.UPrim[6 * id], &U[5 * ld], &W.UPrim[6 * ld], &C.M.Mh[3 * id],
                          &C.M.Mh[3 * ld], F);
          for (int v = 0; v < 5; ++v) tmp[v] = tmp[v] + DVS[l + n * k] * F[v];
        }
        for (int v = 0; v < 5; ++v) Ut[v + 5 * id] = cfg.parabolic ? Ut[v + 5 * id] + tmp[v] : tmp[v];
      }
  }
  // 11. FillFlux  fillflux.f90:45-172: BC sides (GetBoundaryFlux), inner sides (Riemann, viscous
  // flux), then SurfElem and the copy to the slave side
#pragma omp parallel for schedule(static)
  for (long long f = 0; f < (long long)nF; ++f) {
    double* Fm = &W.Flux_master[5 * f];
    if (f < nFbc) {
      const int s = (int)(f / C.n2);
      const double* gx = cfg.parabolic ? &W.gx_m[5 * f] : nullptr;
      const double* gy = cfg.parabolic ? &W.gy_m[5 * f] : nullptr;
      const double* gz = cfg.parabolic ? &W.gz_m[5 * f] : nullptr;
      GetBoundaryFlux(C, &W.UPrim_master[6 * f], gx, gy, gz, &C.M.nv[3 * f], &C.M.t1[3 * f], &C.M.t2[3 * f],
                      C.bctype[s], &C.refprim[6 * C.bcstate[s]], Fm);
      for (int v = 0; v < 5; ++v) {
        Fm[v] = Fm[v] * C.M.SurfElem[f];
        W.Flux_slave[v + 5 * f] = Fm[v];
      }
      continue;
    }
    Riemann(cfg, Fm, &W.U_master[5 * f], &W.U_slave[5 * f], &W.UPrim_master[6 * f], &W.UPrim_slave[6 * f],
            &C.M.nv[3 * f], &C.M.t1[3 * f], &C.M.t2[3 * f]);
    if (cfg.parabolic) {
      // ViscousFlux_Kernel_CUDA  riemann.f90:638-700
      double nd[5];
      EvalNormalDiffFlux3D(&W.UPrim_master[6 * f], &W.gx_m[5 * f], &W.gy_m[5 * f], &W.gz_m[5 * f], nd, &C.M.nv[3 * f],
                           mu, lambda);
      for (int v = 0; v < 5; ++v) Fm[v] = Fm[v] + 0.5 * nd[v];
      EvalNormalDiffFlux3D(&W.UPrim_slave[6 * f], &W.gx_s[5 * f], &W.gy_s[5 * f], &W.gz_s[5 * f], nd, &C.M.nv[3 * f],
                           mu, lambda);
      for (int v = 0; v < 5; ++v) Fm[v] = Fm[v] + 0.5 * nd[v];
    }
    for (int v = 0; v < 5; ++v) {
      Fm[v] = Fm[v] * C.M.SurfElem[f];
      W.Flux_slave[v + 5 * f] = Fm[v];
    }
  }
  // 11.5 SurfIntCons (doApplyJacobian=.FALSE.)
  SurfInt_GPUorder(C, 5, W.Flux_master.data(), W.Flux_slave.data(), Ut, 0, false);
  // 12. Ut = -Ut ; 14. ApplyJacobian (applyjacobian.t90:196-224)
#pragma omp parallel for schedule(static)
  for (long long id = 0; id < (long long)nDOF; ++id)
    for (int v = 0; v < 5; ++v) {
      Ut[v + 5 * id] = Ut[v + 5 * id] * -1.;
      Ut[v + 5 * id] = Ut[v + 5 * id] * C.M.sJ[id];
    }
  (void)n;
}

// Carpenter-Kennedy RK4-5 coefficients  timedisc_vars.f90:213-227
static const double RKA[6] = {0., 0., 567301805773.0 / 1357537059087.0, 2404267990393.0 / 2016746695238.0,
                              3550918686646.0 / 2091501179385.0, 1275806237668.0 / 842570457699.0};
static const double RKb[6] = {0., 1432997174477.0 / 9575080441755.0, 5161836677717.0 / 13612068292357.0,
                              1720146321549.0 / 2090206949498.0, 3134564353537.0 / 4481467310338.0,
                              2277821191437.0 / 14882151754819.0};
static const double RKc[6] = {0., 0., 1432997174477.0 / 9575080441755.0, 2526269341429.0 / 6820363962896.0,
                              2006345519317.0 / 3224310063776.0, 2802321613138.0 / 2924317926251.0};

// TimeStepByLSERKW2  timestep.f90:49-120 with VAXPB_OUT_VAXPB_IN  vector.f90:163-183
static void LSERKW2(const Ctx& C, Work& W, double t, double dt, double* U, double* Ut_tmp, double* Ut) {
  const size_t nTotalU = (size_t)5 * C.n3 * C.M.nElems;
  for (int s = 1; s <= 5; ++s) {
    double tStage = (s == 1) ? t : t + RKc[s] * dt;
    DGTimeDerivative(C, W, U, Ut);
    (void)tStage;
    double mRKA = (s == 1) ? 0. : -1. * RKA[s];
    double b_dt = RKb[s] * dt;
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < (long long)nTotalU; ++i) {
      Ut_tmp[i] = Ut_tmp[i] * mRKA + Ut[i];
      U[i] = U[i] + Ut_tmp[i] * b_dt;
    }
  }
}

// CFL scaling tables for Carpenter RK4-5 (timedisc_vars.f90:193-206) and DFL (timedisc_vars.f90:104-108)
static double cfl_alpha(int node_type, int N) {
  static const double G[15] = {2.0351, 1.7595, 1.5401, 1.3702, 1.2375, 1.1318, 1.0440, 0.9709,
                               0.9079, 0.8539, 0.8066, 0.7650, 0.7290, 0.6952, 0.6660};
  static const double GL[15] = {4.7497, 3.4144, 2.8451, 2.4739, 2.2027, 1.9912, 1.8225, 1.6830,
                                1.5682, 1.4692, 1.3849, 1.3106, 1.2454, 1.1880, 1.1362};
  int i = std::min(15, N) - 1;
  return node_type == DG_NODETYPE_GAUSS ? G[i] : GL[i];
}
static double dfl_alpha(int node_type, int N) {
  static const double G[10] = {1.12, 0.76, 0.55, 0.41, 0.32, 0.25, 0.20, 0.17, 0.14, 0.12};
  static const double GL[10] = {4.50, 1.95, 1.18, 0.79, 0.56, 0.42, 0.32, 0.25, 0.20, 0.17};
  int i = std::min(10, N) - 1;
  return node_type == DG_NODETYPE_GAUSS ? G[i] : GL[i];
}

// CALCTIMESTEP + CalcMaxEigenvalue  calctimestep.f90:51-296, FillCFL_DFL  timedisc_func.f90:480-550.
// The reference's convective reduction is written MIN(TimeStep_Conv,CFL)*2/lambda (calctimestep.f90:157);
// this restatement takes the intended min over elements of CFL*2/lambda_e (as the viscous reduction does).
static double CalcTimeStep(const Ctx& C, const double* U, double CFLin, double DFLin, int* errType) {
  const dg_config& cfg = C.cfg;
  const int N = C.B.N, n = C.n;
  double CFLScale = CFLin * cfl_alpha(cfg.node_type, N) / (2. * N + 1.);
  double DFLScale = DFLin * dfl_alpha(cfg.node_type, N) * 1.853 / ((2. * N + 1.) * (2. * N + 1.));
  double KappasPr_max = std::max(4. / 3., cfg.kappa / cfg.Pr);
  double tsc = HUGE_VAL, tsv = HUGE_VAL;
  int bad = 0;
#pragma omp parallel for schedule(static) reduction(min : tsc, tsv) reduction(+ : bad)
  for (int e = 0; e < C.M.nElems; ++e) {
    // Max_Lambda over (j,k) slices then MAXVAL per direction
    double mx[6] = {0, 0, 0, 0, 0, 0};
    for (int k = 0; k <= N; ++k) for (int j = 0; j <= N; ++j) {
      double tmp[6] = {0, 0, 0, 0, 0, 0};
      for (int i = 0; i <= N; ++i) {
        size_t id = C.vol(i, j, k, e);
        const double* u = &U[5 * id];
        double srho = 1. / u[0];
        double vel[3] = {u[1] * srho, u[2] * srho, u[3] * srho};
        double p = (cfg.kappa - 1.) * (u[4] - 0.5 * (vel[0] * u[1] + vel[1] * u[2] + vel[2] * u[3]));
        if (!(u[0] > 0.) || !(p > 0.) || !std::isfinite(u[4])) bad++;
        double c = std::sqrt(cfg.kappa * p * srho);
        double sj = C.M.sJ[id];
        double vsJ[3] = {vel[0] * sj, vel[1] * sj, vel[2] * sj};
        const double* Ms[3] = {&C.M.Mf[3 * id], &C.M.Mg[3 * id], &C.M.Mh[3 * id]};
        for (int d = 0; d < 3; ++d) {
          const double* M = Ms[d];
          double adv = sj * std::sqrt(M[0] * M[0] + M[1] * M[1] + M[2] * M[2]);  // MetricsAdv
          tmp[d] = std::max(tmp[d], std::fabs(M[0] * vsJ[0] + M[1] * vsJ[1] + M[2] * vsJ[2]) + c * adv);
          if (cfg.parabolic) {
            double vis = KappasPr_max * ((M[0] * sj) * (M[0] * sj) + (M[1] * sj) * (M[1] * sj) + (M[2] * sj) * (M[2] * sj));
            tmp[3 + d] = std::max(tmp[3 + d], cfg.mu0 * srho * vis);
          }
        }
      }
      for (int d = 0; d < 6; ++d) mx[d] = std::max(mx[d], tmp[d]);
    }
    double lam_c = mx[0] + mx[1] + mx[2];
    double lam_v = mx[3] + mx[4] + mx[5];
    tsc = std::min(tsc, CFLScale * 2. / lam_c);
    if (cfg.parabolic) tsv = std::min(tsv, DFLScale * 4. / lam_v);
  }
  if (errType) *errType = bad ? 1 : 0;
  (void)n;
  return std::min(tsc, tsv);
}

}  // namespace orc

// =========================================================================================
// C interface of the oracle (called by tests through ctypes)
// =========================================================================================
using namespace orc;

struct orc_handle {
  Ctx C;
  Work W;
  std::vector<double> Ut;
};

extern "C" {

int orc_set_threads(int n) {
  if (n > 0) omp_set_num_threads(n);
  return omp_get_max_threads();
}

// nodes/weights/barycentric weights for the four node types of unitTests/NodesAndWeights.f90
int orc_nodes_weights(int N, int node_type, double* x, double* w, double* wbary) {
  GetNodesAndWeights(N, node_type, x, w, wbary);
  return 0;
}

int orc_derivative_matrix(int N, int node_type, double* D) {
  std::vector<double> x(N + 1);
  GetNodesAndWeights(N, node_type, x.data(), nullptr, nullptr);
  PolynomialDerivativeMatrix(N, x.data(), D);
  return 0;
}

int orc_dg_basis(int N, int node_type, double* xGP, double* wGP, double* wBary, double* L_minus, double* L_plus,
                 double* D, double* D_hat_T, double* L_hat_minus, double* L_hat_plus, double* DVolSurf) {
  Basis B;
  build_basis(N, node_type, B);
  int n = N + 1;
  auto cp = [](double* dst, const std::vector<double>& s) { if (dst) std::memcpy(dst, s.data(), s.size() * sizeof(double)); };
  cp(xGP, B.xGP); cp(wGP, B.wGP); cp(wBary, B.wBary); cp(L_minus, B.L_Minus); cp(L_plus, B.L_Plus);
  cp(D, B.D); cp(D_hat_T, B.D_Hat_T); cp(L_hat_minus, B.L_HatMinus); cp(L_hat_plus, B.L_HatPlus);
  cp(DVolSurf, B.DVolSurf);
  (void)n;
  return 0;
}

int orc_s2v2(int N, int* s2v2) {
  Ctx C;
  C.B.N = N; C.n = N + 1;
  build_s2v2(C);
  std::memcpy(s2v2, C.S2V2.data(), C.S2V2.size() * sizeof(int));
  return 0;
}

// Host ProlongToFace (prolongtoface.t90:20-110) for the golden single-element check: every side is a
// master side of element 1 (SideToElem from UnittestElementData3D.bin).
int orc_prolong_to_face_host(int N, int nVar, int node_type, const double* L_minus, const double* L_plus,
                             const int* side_to_elem, int nSides, const int* s2v2, const double* Uvol,
                             double* Uface_master) {
  const int n = N + 1;
  std::vector<double> Uface((size_t)nVar * n * n);
  for (int s = 0; s < nSides; ++s) {
    int elem = side_to_elem[0 + 5 * s];
    if (elem <= 0) continue;
    int locSide = side_to_elem[2 + 5 * s];
    const double* Ue = Uvol + (size_t)nVar * n * n * n * (elem - 1);
    auto at = [&](int a, int b, int c, int v) { return Ue[v + nVar * (a + n * (b + n * c))]; };
    for (int b = 0; b <= N; ++b) for (int a = 0; a <= N; ++a) for (int v = 0; v < nVar; ++v) {
      double sum;
      const double* Lv = (locSide == XI_MINUS || locSide == ETA_MINUS || locSide == ZETA_MINUS) ? L_minus : L_plus;
      if (node_type == DG_NODETYPE_GAUSS) {
        switch (locSide) {
          case XI_MINUS: case XI_PLUS:
            sum = at(0, a, b, v) * Lv[0]; for (int l = 1; l <= N; ++l) sum = sum + at(l, a, b, v) * Lv[l]; break;
          case ETA_MINUS: case ETA_PLUS:
            sum = at(a, 0, b, v) * Lv[0]; for (int l = 1; l <= N; ++l) sum = sum + at(a, l, b, v) * Lv[l]; break;
          default:
            sum = at(a, b, 0, v) * Lv[0]; for (int l = 1; l <= N; ++l) sum = sum + at(a, b, l, v) * Lv[l]; break;
        }
      } else {
        switch (locSide) {
          case XI_MINUS: sum = at(0, a, b, v); break;
          case ETA_MINUS: sum = at(a, 0, b, v); break;
          case ZETA_MINUS: sum = at(a, b, 0, v); break;
          case XI_PLUS: sum = at(N, a, b, v); break;
          case ETA_PLUS: sum = at(a, N, b, v); break;
          default: sum = at(a, b, N, v); break;
        }
      }
      Uface[v + nVar * (a + n * b)] = sum;
    }
    for (int q = 0; q <= N; ++q) for (int p = 0; p <= N; ++p) {
      int a = s2v2[0 + 2 * (p + n * (q + n * (0 + 5 * (locSide - 1))))];
      int b = s2v2[1 + 2 * (p + n * (q + n * (0 + 5 * (locSide - 1))))];
      for (int v = 0; v < nVar; ++v) Uface_master[v + nVar * (p + n * (q + (size_t)n * s))] = Uface[v + nVar * (a + n * b)];
    }
  }
  return 0;
}

// Host SurfInt (surfint.t90:19-232) for the golden single-element check (master sides only).
int orc_surf_int_host(int N, int nVar, int node_type, const double* L_hat_minus, const double* L_hat_plus,
                      const int* side_to_elem, int nSides, const int* s2v2, const double* Flux_master, double* Ut) {
  const int n = N + 1;
  std::vector<double> FluxTmp((size_t)nVar * n * n);
  for (int s = 0; s < nSides; ++s) {
    int elem = side_to_elem[0 + 5 * s];
    if (elem <= 0) continue;
    int loc = side_to_elem[2 + 5 * s];
    for (int q = 0; q <= N; ++q) for (int p = 0; p <= N; ++p) {
      int a = s2v2[0 + 2 * (p + n * (q + n * (0 + 5 * (loc - 1))))];
      int b = s2v2[1 + 2 * (p + n * (q + n * (0 + 5 * (loc - 1))))];
      for (int v = 0; v < nVar; ++v) FluxTmp[v + nVar * (a + n * b)] = Flux_master[v + nVar * (p + n * (q + (size_t)n * s))];
    }
    double* Ue = Ut + (size_t)nVar * n * n * n * (elem - 1);
    auto at = [&](int a, int b, int c, int v) -> double& { return Ue[v + nVar * (a + n * (b + n * c))]; };
    bool minus = (loc == XI_MINUS || loc == ETA_MINUS || loc == ZETA_MINUS);
    const double* Lh = minus ? L_hat_minus : L_hat_plus;
    for (int b = 0; b <= N; ++b) for (int a = 0; a <= N; ++a) for (int v = 0; v < nVar; ++v) {
      double fl = FluxTmp[v + nVar * (a + n * b)];
      if (node_type == DG_NODETYPE_GAUSS) {
        for (int l = 0; l <= N; ++l) {
          switch (loc) {
            case XI_MINUS: case XI_PLUS: at(l, a, b, v) = at(l, a, b, v) + fl * Lh[l]; break;
            case ETA_MINUS: case ETA_PLUS: at(a, l, b, v) = at(a, l, b, v) + fl * Lh[l]; break;
            default: at(a, b, l, v) = at(a, b, l, v) + fl * Lh[l]; break;
          }
        }
      } else {
        double lh = minus ? L_hat_minus[0] : L_hat_plus[N];
        switch (loc) {
          case XI_MINUS: at(0, a, b, v) += fl * lh; break;
          case ETA_MINUS: at(a, 0, b, v) += fl * lh; break;
          case ZETA_MINUS: at(a, b, 0, v) += fl * lh; break;
          case XI_PLUS: at(N, a, b, v) += fl * lh; break;
          case ETA_PLUS: at(a, N, b, v) += fl * lh; break;
          default: at(a, b, N, v) += fl * lh; break;
        }
      }
    }
  }
  return 0;
}

// ---- full operator ----
orc_handle* orc_create(const dg_config* cfg, int nElems, int nSides, const double* Mf, const double* Mg,
                       const double* Mh, const double* sJ, const double* nv, const double* t1, const double* t2,
                       const double* SurfElem, const int* E2S, const int* S2E) {
  orc_handle* h = new orc_handle();
  h->C.cfg = *cfg;
  build_basis(cfg->N, cfg->node_type, h->C.B);
  h->C.n = cfg->N + 1; h->C.n2 = h->C.n * h->C.n; h->C.n3 = h->C.n2 * h->C.n;
  h->C.M = Mesh{nElems, nSides, Mf, Mg, Mh, sJ, nv, t1, t2, SurfElem, E2S, S2E};
  build_s2v2(h->C);
  alloc_work(h->C, h->W);
  h->Ut.assign((size_t)5 * h->C.n3 * nElems, 0.);
  if (InitFilter(h->C) != 0) { delete h; return nullptr; }
  // LAF state initial values (filter.f90:195-199)
  h->W.lim.assign(nElems, 1E-8); h->W.eRatio.assign(nElems, 0.); h->W.r.assign(nElems, 0.);
  h->W.ekin_avg_old.assign(nElems, 1.E-16); h->W.ekin_fluc_avg_old.assign(nElems, 1.E-16);
  return h;
}

// GetVandermonde / ChangeBasis3D(_XYZ) for the golden checks against unitTests/{Vandermonde,ChangeBasis}.bin
int orc_get_vandermonde(int N_in, int nt_in, int N_out, int nt_out, int modal, double* Vdm_In_Out, double* Vdm_Out_In) {
  GetVandermonde(N_in, nt_in, N_out, nt_out, Vdm_In_Out, Vdm_Out_In, modal != 0);
  return 0;
}
int orc_change_basis_3d(int nVar, int NIn, int NOut, const double* Vx, const double* Vy, const double* Vz,
                        const double* X_In, double* X_Out) {
  ChangeBasis3D_XYZ(nVar, NIn, NOut, Vx, Vy, Vz, X_In, X_Out);
  return 0;
}

// The oracle's own geometry: BuildCoords + CalcMetrics + CalcSurfMetrics from the equidistant NodeCoords
// (3,0:NGeo,0:NGeo,0:NGeo,nElems) and ElemToSide(3,6,nElems) (1-based side IDs; the master sides, flip
// 0, receive the side vectors).  Elem_xGP and Face_xGP may be null.  Returns the count of solution
// nodes with a scaled Jacobian below 0.01, or -1 for a non-positive Jacobian.
int orc_calc_metrics(int N, int node_type, int NGeo, int nElems, const double* NodeCoords, const int* ElemToSide,
                     double* Elem_xGP, double* Mf, double* Mg, double* Mh, double* sJ, double* NormVec, double* TangVec1,
                     double* TangVec2, double* SurfElem, double* Face_xGP) {
  MetricsOut o{Elem_xGP, Mf, Mg, Mh, sJ, NormVec, TangVec1, TangVec2, SurfElem, Face_xGP};
  return CalcMetrics(N, node_type, NGeo, nElems, NodeCoords, ElemToSide, o);
}

int orc_laf_state(orc_handle* h, double* lim, double* eRatio, double* r) {
  const size_t nE = h->C.M.nElems;
  if (lim) std::memcpy(lim, h->W.lim.data(), nE * sizeof(double));
  if (eRatio) std::memcpy(eRatio, h->W.eRatio.data(), nE * sizeof(double));
  if (r) std::memcpy(r, h->W.r.data(), nE * sizeof(double));
  return 0;
}

void orc_destroy(orc_handle* h) { delete h; }

// Boundary conditions of the first nBCSides sides: BC type and 1-based RefState index per side, RefState
// rows (rho, u, v, w, p) as in the parameter file.  RefStatePrim(TEMP) as InitEquation
// (equation.f90:136-147); type 27 states (Tt, alpha, beta, -, pt) turned into the inflow direction as
// InitBC (getboundaryflux.f90:199-208).
int orc_set_boundaries(orc_handle* h, int nBCSides, const int* bc_type, const int* bc_state, int nRefState,
                       const double* refstate) {
  Ctx& C = h->C;
  C.nBCSides = nBCSides;
  C.bctype.assign(bc_type, bc_type + nBCSides);
  C.bcstate.resize(nBCSides);
  C.refprim.assign((size_t)6 * std::max(1, nRefState), 0.);
  for (int r = 0; r < nRefState; ++r) {
    for (int c = 0; c < 5; ++c) C.refprim[6 * r + c] = refstate[5 * r + c];
    C.refprim[6 * r + TEMP] = C.refprim[6 * r + PRES] * (1. / C.refprim[6 * r + DENS]) / C.cfg.R;
  }
  std::vector<char> done(std::max(1, nRefState), 0);
  for (int s = 0; s < nBCSides; ++s) {
    const int t = bc_type[s];
    if (t != 2 && t != 3 && t != 4 && t != 9 && t != 91 && t != 23 && t != 24 && t != 25 && t != 27) return -1;
    int st = bc_state[s] - 1;
    if (st < 0 || st >= nRefState) {
      if (t != 3 && t != 9 && t != 91) return -2;
      st = 0;
    }
    C.bcstate[s] = st;
    if (t == 27 && !done[st]) {
      done[st] = 1;
      double* q = &C.refprim[6 * st];
      const double talpha = std::tan(PP_Pi / 180. * q[1]), tbeta = std::tan(PP_Pi / 180. * q[2]);
      q[VEL1] = 1. / std::sqrt((1. + talpha * talpha + tbeta * tbeta));
      q[VEL2] = talpha / std::sqrt((1. + talpha * talpha + tbeta * tbeta));
      q[VEL3] = tbeta / std::sqrt((1. + talpha * talpha + tbeta * tbeta));
    }
  }
  return 0;
}

int orc_rhs(orc_handle* h, double* U, double* Ut) {
  DGTimeDerivative(h->C, h->W, U, Ut);
  return 0;
}

// intermediate arrays after the last orc_rhs call (for localising mismatches in tests)
int orc_get_work(orc_handle* h, int which, double* out) {
  const std::vector<double>* src = nullptr;
  switch (which) {
    case 0: src = &h->W.UPrim; break;
    case 1: src = &h->W.gradUx; break;
    case 2: src = &h->W.gradUy; break;
    case 3: src = &h->W.gradUz; break;
    case 4: src = &h->W.Flux_master; break;
    case 5: src = &h->W.U_master; break;
    case 6: src = &h->W.U_slave; break;
    default: return -1;
  }
  std::memcpy(out, src->data(), src->size() * sizeof(double));
  return 0;
}

int orc_lserk_steps(orc_handle* h, double t, double dt, int nSteps, double* U, double* Ut_tmp) {
  for (int s = 0; s < nSteps; ++s) LSERKW2(h->C, h->W, t + s * dt, dt, U, Ut_tmp, h->Ut.data());
  return 0;
}

double orc_calc_timestep(orc_handle* h, const double* U, double cfl, double dfl, int* errType) {
  return CalcTimeStep(h->C, U, cfl, dfl, errType);
}

}  // extern "C"
