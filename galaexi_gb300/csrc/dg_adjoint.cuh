// Discrete adjoint of the FP64 DGSEM operator: the transpose of the linearisation of
// DGTimeDerivative_weakForm (src/dg/dg.f90:255-425) about a state U, applied to a cotangent Ut_bar,
// and fused with the reverse LSERK-W2 stage.
//
// The forward operator is  Ut = -sJ (VolInt(U, P, G) + SurfInt(F)),  F = SE (Riemann(U_f, P_f) +
// 0.5 f_v(P_m, G_m) + 0.5 f_v(P_s, G_s)),  G = Lifting(P, P_f),  P = prim(U),  U_f = Prolong(U).
// One adjoint evaluation re-runs the forward k_prolong and k_lift (P, U_f, P_f, G, G_f of the state),
// then:
//   ka_face   thread per face node   a = -sJ Ut_bar gathered to the face (transposed SurfInt), the
//                                    Riemann flux transposed through its local 5x10 Jacobian (forward
//                                    mode, Dual<10>), the BR1 viscous flux transposed by hand
//                                    -> cotangents of U_f (5) and G_f (15) on both sides
//   ka_volume element per block      transposed split-form flux differencing (pair symmetric; the PI
//                                    and KG two-point fluxes depend on node pairs only through sums),
//                                    transposed weak-form volume integral (D_hat^T), viscous volume
//                                    flux, gradient cotangents (volume + face traces), transposed
//                                    lifting volume integral, ConsToPrim -> U cotangent (volume part),
//                                    and the per-element share of the lifting jump cotangent
//   ka_jump   thread per face node   the lifting jump cotangents of both elements through ConsToPrim of
//                                    the face states, added to the face cotangents (Navier-Stokes)
//   ka_final  thread per node        transposed ProlongToFace of the face cotangents, and the reverse RK
//                                    stage  Ubar += dR^T(K_bar + b dt Ubar),  K_bar = -RKA (K_bar + b dt Ubar)
// The viscosity derivative <Ut_bar, dR/dmu> is accumulated on the way (R is linear in mu at fixed
// Prandtl number): per-block partial sums, reduced in a fixed order by k_adj_sum.
//
//   ka_bc_face / ka_bc_jump   the boundary sides' flux and lifting ghost state, transposed through
//                             local Jacobians on dual numbers (meshes with boundary sides)
// Supported forms: Gauss or Gauss-Lobatto nodes; weak form or split form PI / KG; any Riemann solver;
// Euler or Navier-Stokes with BR1 lifting in strong form (non-conservative or conservative volume
// part); periodic meshes and meshes with boundary sides of the types of dg_bc.cuh.
#pragma once
#include "dg_kernels.cuh"
#include "dg_riemann_vjp.cuh"

namespace gx {

// cotangent source: Ut_bar = A + beta * B (B may be null)
struct CotSrc {
  const double* A;
  const double* B;
  double beta;
};
__device__ __forceinline__ void cot_at(const CotSrc& c, size_t g, double out[5]) {
#pragma unroll
  for (int v = 0; v < 5; ++v) out[v] = c.A[g + v];
  if (c.B) {
#pragma unroll
    for (int v = 0; v < 5; ++v) out[v] = out[v] + c.beta * c.B[g + v];
  }
}

struct AdjLaunch {
  int nElems, nSides;
  int gauss, riemann, split, parabolic, lift_mode;
  double mu, lambda, lamc;  // mu, lambda, lambda/mu (the thermal conductivity per unit viscosity)
  double inv_mu;            // 1/mu, or 0 for mu = 0
  double kappa, sR;
  // boundary sides (the first nBCSides sides): type, 0-based reference state, states [state][6]
  int nBCSides;
  const int* bctype;
  const int* bcstate;
  const double* bcref;
};

// Transpose of one directional BR1 viscous flux  f = normal_diff_flux(P, g, nv, mu, lambda)
// (flux.f90:779-847) down to the cotangents of tau (6) and tq = tau.v + lambda grad T (3);
// visc_close_vjp then maps them to the gradient (15) and velocity (3) cotangents.
__device__ __forceinline__ void visc_dir_vjp(const double nv[3], const double fb[5], double taub[6], double tqb[3]) {
  // f1..3 = -n . tau rows, f4 = -n . tq
  taub[0] -= nv[0] * fb[1]; taub[3] -= nv[1] * fb[1]; taub[4] -= nv[2] * fb[1];
  taub[3] -= nv[0] * fb[2]; taub[1] -= nv[1] * fb[2]; taub[5] -= nv[2] * fb[2];
  taub[4] -= nv[0] * fb[3]; taub[5] -= nv[1] * fb[3]; taub[2] -= nv[2] * fb[3];
  tqb[0] -= nv[0] * fb[4]; tqb[1] -= nv[1] * fb[4]; tqb[2] -= nv[2] * fb[4];
}
// closes a viscous transpose: tq = tau.v + lambda grad T, tau = mu (grad v + grad v^T - 2/3 div v I)
__device__ __forceinline__ void visc_close_vjp(const double tau[6], const double vel[3], double mu, double lambda,
                                               double taub[6], const double tqb[3], double gb[15], double velb[3]) {
  // tq0 = txx u + txy v + txz w + l Tx ; tq1 = txy u + tyy v + tyz w + l Ty ; tq2 = txz u + tyz v + tzz w + l Tz
  taub[0] += tqb[0] * vel[0];
  taub[3] += tqb[0] * vel[1] + tqb[1] * vel[0];
  taub[4] += tqb[0] * vel[2] + tqb[2] * vel[0];
  taub[1] += tqb[1] * vel[1];
  taub[5] += tqb[1] * vel[2] + tqb[2] * vel[1];
  taub[2] += tqb[2] * vel[2];
  velb[0] += tqb[0] * tau[0] + tqb[1] * tau[3] + tqb[2] * tau[4];
  velb[1] += tqb[0] * tau[3] + tqb[1] * tau[1] + tqb[2] * tau[5];
  velb[2] += tqb[0] * tau[4] + tqb[1] * tau[5] + tqb[2] * tau[2];
  gb[4] += lambda * tqb[0];
  gb[9] += lambda * tqb[1];
  gb[14] += lambda * tqb[2];
  // tau from the gradients: gx = gb[0..4], gy = gb[5..9], gz = gb[10..14]
  const double s23 = 2. / 3., s43 = 4. / 3.;
  gb[1] += mu * (s43 * taub[0] - s23 * taub[1] - s23 * taub[2]);
  gb[7] += mu * (-s23 * taub[0] + s43 * taub[1] - s23 * taub[2]);
  gb[13] += mu * (-s23 * taub[0] - s23 * taub[1] + s43 * taub[2]);
  gb[6] += mu * taub[3];  // d/dy u
  gb[2] += mu * taub[3];  // d/dx v
  gb[11] += mu * taub[4]; // d/dz u
  gb[3] += mu * taub[4];  // d/dx w
  gb[12] += mu * taub[5]; // d/dz v
  gb[8] += mu * taub[5];  // d/dy w
}

// Transpose of the PI / KG two-point flux (split_pair_flux) with respect to the pair sums
// (rs, us, vs, ws, ps, auxs); both nodes of the pair receive the same cotangents.
template <int SPLIT>
__device__ __forceinline__ void pair_sum_vjp(double rs, double us, double vs, double ws, double ps, double auxs,
                                             double Ms0, double Ms1, double Ms2, const double Fb[5], double sb[6]) {
  if constexpr (SPLIT == DG_SPLIT_PI) {
    // Fb arrives scaled by 1/8 (DVolSurf / 8) with its density row doubled (2a staged): every
    // constant below is folded that way, by powers of two, so the result has the same bits
    const double Vs = Ms0 * us + Ms1 * vs + Ms2 * ws;
    const double q8 = rs * Vs;
    const double qb8 = Fb[0] + Fb[1] * us + Fb[2] * vs + Fb[3] * ws + Fb[4] * auxs;
    sb[1] = Fb[1] * q8; sb[2] = Fb[2] * q8; sb[3] = Fb[3] * q8;
    sb[4] = 4. * (Fb[1] * Ms0 + Fb[2] * Ms1 + Fb[3] * Ms2);
    sb[5] = Fb[4] * q8;
    const double Vsb = rs * qb8;
    sb[0] = Vs * qb8;
    sb[1] += Ms0 * Vsb; sb[2] += Ms1 * Vsb; sb[3] += Ms2 * Vsb;
    return;
  }
  const double Vs = Ms0 * us + Ms1 * vs + Ms2 * ws;
  const double q = 0.125 * rs * Vs;
  double qb = 2. * Fb[0] + Fb[1] * us + Fb[2] * vs + Fb[3] * ws + Fb[4] * auxs;
  double Vsb = 0.;
  sb[1] = Fb[1] * q; sb[2] = Fb[2] * q; sb[3] = Fb[3] * q;
  sb[4] = 0.5 * (Fb[1] * Ms0 + Fb[2] * Ms1 + Fb[3] * Ms2);
  sb[5] = Fb[4] * q;
  if (SPLIT == DG_SPLIT_KG) {  // F4 += 0.25 ps Vs
    sb[4] += 0.25 * Vs * Fb[4];
    Vsb += 0.25 * ps * Fb[4];
  }
  Vsb += 0.125 * rs * qb;
  sb[0] = 0.125 * Vs * qb;
  sb[1] += Ms0 * Vsb; sb[2] += Ms1 * Vsb; sb[3] += Ms2 * Vsb;
}

// ---------------------------------------------------------------------------------------------
// ka_face: thread per face node
// ---------------------------------------------------------------------------------------------
template <int NP, bool HAND>
__global__ void __launch_bounds__(128)
ka_face(CotSrc cs, const double* __restrict__ Met, const double* __restrict__ Uf, const double* __restrict__ Pf,
        const double* __restrict__ Gf, const double* __restrict__ Fgeo, const int* __restrict__ S2E,
        DevBasis<double> basis, Gas<double> gas, AdjLaunch L, double* __restrict__ UfB, double* __restrict__ GfB,
        double* __restrict__ mupart) {
  constexpr int n = NP, n2 = NP * NP, n3 = NP * NP * NP, N = NP - 1;
  __shared__ double red[4];
  // connected sides only (nBCSides .. nSides-1); the BC sides are ka_bc_face's
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x + (long long)L.nBCSides * n2;
  double mub = 0.;
  if (t < (long long)L.nSides * n2) {
    const int side = (int)(t / n2), pq = (int)(t - (long long)side * n2);
    const int p = pq % n, q = pq / n;
    const size_t S = L.nSides;
    const int* se2 = S2E + (size_t)side * 5;
    // transposed SurfInt: Fbar = sum over the master line (+) and the slave line (-) of L_hat * a
    double Fb[5] = {0, 0, 0, 0, 0};
#pragma unroll
    for (int slot = 0; slot < 2; ++slot) {
      const int e = slot == 0 ? se2[0] : se2[2];
      const int ls = slot == 0 ? se2[1] : se2[3];
      const int flip = slot == 0 ? 0 : se2[4];
      int a, b;
      s2v2(N, p, q, flip, ls, a, b);
      const bool minus = is_minus(ls);
      const double sgn = slot == 0 ? 1. : -1.;
      const int l0 = L.gauss ? 0 : (minus ? 0 : N), l1 = L.gauss ? N : l0;
      for (int l = l0; l <= l1; ++l) {
        const double Lh = L.gauss ? (minus ? basis.Lhm[l] : basis.Lhp[l]) : (minus ? basis.Lhm[0] : basis.Lhp[N]);
        const int node = face_node(n, ls, a, b, l);
        const double sj = Met[((size_t)e * 10 + 9) * n3 + node];
        double ub[5];
        cot_at(cs, ((size_t)e * n3 + node) * 5, ub);
        const double w = -sgn * Lh * sj;
#pragma unroll
        for (int v = 0; v < 5; ++v) Fb[v] = Fb[v] + w * ub[v];
      }
    }
    const double* fg = Fgeo + (size_t)side * 10 * n2 + pq;
    const double se = fg[9 * n2];
#pragma unroll
    for (int v = 0; v < 5; ++v) Fb[v] *= se;
    // Riemann flux transposed through its local Jacobian: d F / d (U_L, U_R), forward mode
    double ULb[5] = {0, 0, 0, 0, 0}, URb[5] = {0, 0, 0, 0, 0};
    double ULv[5], URv[5];
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      ULv[v] = Uf[(size_t)side * 5 * n2 + v * n2 + pq];
      URv[v] = Uf[(S + side) * 5 * n2 + v * n2 + pq];
    }
    if constexpr (HAND) {
      const double nv[3] = {fg[0], fg[n2], fg[2 * n2]};
      const double t1[3] = {fg[3 * n2], fg[4 * n2], fg[5 * n2]};
      const double t2[3] = {fg[6 * n2], fg[7 * n2], fg[8 * n2]};
      Ext<double> Le, Re;
      make_ext(ULv, nv, t1, t2, gas.kappaM1, Le);
      make_ext(URv, nv, t1, t2, gas.kappaM1, Re);
      const double Fr[5] = {Fb[0], nv[0] * Fb[1] + nv[1] * Fb[2] + nv[2] * Fb[3],
                            t1[0] * Fb[1] + t1[1] * Fb[2] + t1[2] * Fb[3], t2[0] * Fb[1] + t2[1] * Fb[2] + t2[2] * Fb[3],
                            Fb[4]};
      ExtB Lb = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0}, Rb = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
      riemann_solver_vjp(L.riemann, L.split, Le, Re, gas.kappa, Fr, Lb, Rb);
      ext_vjp(ULv, Le, Lb, nv, t1, t2, gas.kappaM1, L.sR, ULb);
      ext_vjp(URv, Re, Rb, nv, t1, t2, gas.kappaM1, L.sR, URb);
    } else {
      using D10 = Dual<10>;
      D10 UL[5], UR[5], PL[6], PR[6], sL, sR_, F[5];
#pragma unroll
      for (int v = 0; v < 5; ++v) {
        UL[v] = D10(ULv[v]); UL[v].d[v] = 1.;
        UR[v] = D10(URv[v]); UR[v].d[5 + v] = 1.;
      }
      Gas<D10> g;
      g.kappa = D10(gas.kappa); g.kappaM1 = D10(gas.kappaM1); g.sKappaM1 = D10(gas.sKappaM1);
      g.R_gas = D10(gas.R_gas); g.mu = D10(gas.mu); g.lambda = D10(gas.lambda); g.sR = D10(gas.sR);
      g.pref = D10(0.); g.prefD = 0.; g.kappaM1D = gas.kappaM1D; g.sRD = gas.sRD;
      cons_to_prim_d(UL, g, PL, sL);
      cons_to_prim_d(UR, g, PR, sR_);
      const D10 nv[3] = {D10(fg[0]), D10(fg[n2]), D10(fg[2 * n2])};
      const D10 t1[3] = {D10(fg[3 * n2]), D10(fg[4 * n2]), D10(fg[5 * n2])};
      const D10 t2[3] = {D10(fg[6 * n2]), D10(fg[7 * n2]), D10(fg[8 * n2])};
      riemann_face(L.riemann, L.split, UL, UR, PL, PR, nv, t1, t2, g, F);
#pragma unroll
      for (int w = 0; w < 5; ++w) {
#pragma unroll
        for (int v = 0; v < 5; ++v) {
          ULb[v] += Fb[w] * F[w].d[v];
          URb[v] += Fb[w] * F[w].d[5 + v];
        }
      }
    }
    if (L.parabolic) {
      const double nv[3] = {fg[0], fg[n2], fg[2 * n2]};
      const double fb[5] = {0.5 * Fb[0], 0.5 * Fb[1], 0.5 * Fb[2], 0.5 * Fb[3], 0.5 * Fb[4]};
#pragma unroll
      for (int slot = 0; slot < 2; ++slot) {
        const double* gsrc = Gf + ((size_t)slot * S + side) * 15 * n2 + pq;
        const double* psrc = Pf + ((size_t)slot * S + side) * 6 * n2 + pq;
        double gg[15];
#pragma unroll
        for (int c = 0; c < 15; ++c) gg[c] = gsrc[c * n2];
        const double vel[3] = {psrc[n2], psrc[2 * n2], psrc[3 * n2]};
        double tau[6], tq[3];
        visc_stress(gg, gg + 5, gg + 10, vel, L.mu, L.lambda, tau, tq);
        double taub[6] = {0, 0, 0, 0, 0, 0}, tqb[3] = {0, 0, 0}, gb[15], velb[3] = {0, 0, 0};
#pragma unroll
        for (int c = 0; c < 15; ++c) gb[c] = 0.;
        visc_dir_vjp(nv, fb, taub, tqb);
        // d F / d mu = F_visc / mu (the viscous flux is linear in mu at fixed Prandtl number), so
        // <fb, dF/dmu> = (taub . tau + tqb . tq) / mu before taub is closed
        const double fvis = taub[0] * tau[0] + taub[1] * tau[1] + taub[2] * tau[2] + taub[3] * tau[3] +
                            taub[4] * tau[4] + taub[5] * tau[5] + tqb[0] * tq[0] + tqb[1] * tq[1] + tqb[2] * tq[2];
        if (L.inv_mu > 0.) {
          mub += fvis * L.inv_mu;
        } else {
          double fd1[5];
          const double P6[6] = {psrc[0], vel[0], vel[1], vel[2], psrc[4 * n2], psrc[5 * n2]};
          normal_diff_flux(P6, gg, gg + 5, gg + 10, nv, 1., L.lamc, fd1);
#pragma unroll
          for (int v = 1; v < 5; ++v) mub += fb[v] * fd1[v];
        }
        visc_close_vjp(tau, vel, L.mu, L.lambda, taub, tqb, gb, velb);
        double* gout = GfB + ((size_t)slot * S + side) * 15 * n2 + pq;
#pragma unroll
        for (int c = 0; c < 15; ++c) gout[c * n2] = gb[c];
        prim_vjp(slot == 0 ? ULv : URv, gas.kappaM1, L.sR, 0., velb[0], velb[1], velb[2], 0., 0., 0., 0., 0., 0., 0.,
                 slot == 0 ? ULb : URb);
      }
    }
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      UfB[(size_t)side * 5 * n2 + v * n2 + pq] = ULb[v];
      UfB[(S + side) * 5 * n2 + v * n2 + pq] = URb[v];
    }
  }
  // block partial of dR/dmu
  for (int o = 16; o > 0; o >>= 1) mub += __shfl_xor_sync(0xffffffffu, mub, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mub;
  __syncthreads();
  if (threadIdx.x == 0) mupart[blockIdx.x] = red[0] + red[1] + red[2] + red[3];
}


// ---------------------------------------------------------------------------------------------
// ka_volume: element per block (EPBof<NP> elements, one thread per node)
// ---------------------------------------------------------------------------------------------
// shared memory per element: a (5 n^3), node data / gradient cotangents (15 n^3), pair-sum
// cotangent accumulators / lifting weights (18 n^3)
template <int NP> constexpr int adj_vol_words() { return 38 * NP * NP * NP; }

template <int NP, int SPLIT, int PARAB>
__global__ void __launch_bounds__(EPBof<NP>::v * NP * NP * NP)
ka_volume(CotSrc cs, const double* __restrict__ U, const double* __restrict__ Pvol, const double* __restrict__ Gvol,
          const double* __restrict__ Met, const double* __restrict__ Fgeo, const int* __restrict__ E2S,
          DevBasis<double> basis, AdjLaunch L, const double* __restrict__ GfB, double* __restrict__ UBv,
          double* __restrict__ JB, double* __restrict__ mupart) {
  constexpr int n = NP, n2 = NP * NP, n3 = NP * NP * NP, EPB = EPBof<NP>::v, N = NP - 1;
  __shared__ SBasis<NP, double> sb;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double* const sm = reinterpret_cast<double*>(smem_raw);
  load_basis(sb, basis);
  if constexpr (SPLIT == DG_SPLIT_PI) {
    // the 1/8 of the PI pair cotangents folded into DVolSurf (exact scaling, see pair_sum_vjp)
    __syncthreads();
    for (int t = threadIdx.x; t < NP * NP; t += blockDim.x) sb.DVS[t] = sb.DVS[t] * 0.125;
  }
  const int e0 = blockIdx.x * EPB;
  const int nloc = min(EPB, L.nElems - e0);
  const int tid = threadIdx.x;
  const bool active = tid < nloc * n3;
  const int el = tid / n3, node = tid - (tid / n3) * n3;
  const int e = e0 + el;
  const int i = node % n, j = (node / n) % n, k = node / n2;
  const int snode = vsw<NP>(node);  // shared-memory position of this node (conflict-free at N=7)
  double* Aa = sm + (size_t)el * 38 * n3;  // [5][n3]   a = -sJ Ut_bar
  double* Bs = Aa + 5 * n3;                // [15][n3]  node data (split), later gradient cotangents
  double* Cs = Aa + 20 * n3;               // [18][n3]  pair-sum cotangents (3 dirs x 6), later lifting weights
  const double* M = Met + (size_t)e * 10 * n3 + node;
  const double* P = Pvol + (size_t)e * 7 * n3 + node;
  const size_t gU = ((size_t)e * n3 + node) * 5;
  double mub = 0.;

  // ---- phase A: a, node data of the two-point fluxes, zero accumulators
  if (active) {
    double ub[5];
    cot_at(cs, gU, ub);
    const double sj = M[9 * n3];
#pragma unroll
    for (int v = 0; v < 5; ++v) Aa[v * n3 + snode] = -sj * ub[v];
    // PI: the density row is staged doubled (exact), as pair_sum_vjp expects; the split forms' viscous
    // part (phase C) reads the momentum and energy rows only
    if constexpr (SPLIT == DG_SPLIT_PI) Aa[snode] = 2. * Aa[snode];
    if constexpr (SPLIT >= 0) {
      const double E = U[gU + 4];
      const double rho = P[0], uu = P[n3], vv = P[2 * n3], ww = P[3 * n3], pm = P[4 * n3];
      Bs[0 * n3 + snode] = rho;
      Bs[1 * n3 + snode] = uu;
      Bs[2 * n3 + snode] = vv;
      Bs[3 * n3 + snode] = ww;
      Bs[4 * n3 + snode] = pm;
      Bs[5 * n3 + snode] = pair_aux<SPLIT, double>(rho, uu, vv, ww, E, pm, P[6 * n3]);
#pragma unroll
      for (int c = 0; c < 9; ++c) Bs[(6 + c) * n3 + snode] = M[c * n3];
#pragma unroll
      for (int c = 0; c < 18; ++c) Cs[c * n3 + snode] = 0.;
    }
  }
  __syncthreads();

  // ---- phase B: transposed split-form flux differencing, one thread per line (pair symmetric)
  if constexpr (SPLIT >= 0) {
    const int lel = tid / (3 * n2);
    const bool lactive = (lel < nloc) && (tid < EPB * 3 * n2);
    if (lactive) {
      const int lr = tid - lel * 3 * n2;
      const int dir = lr / n2, li = lr - dir * n2;
      const double* Al = sm + (size_t)lel * 38 * n3;
      const double* Bl = Al + 5 * n3;
      double* Cl = const_cast<double*>(Al) + 20 * n3 + dir * 6 * n3;
      int base, stride;
      if (dir == 0) { base = n * li; stride = 1; }
      else if (dir == 1) { base = (li % n) + n2 * (li / n); stride = n; }
      else { base = li; stride = n2; }
      const int mc = 6 + 3 * dir;
#pragma unroll 1
      for (int a = 0; a < NP - 1; ++a) {
        const int na = vsw<NP>(base + a * stride);
        const double ra = Bl[na], ua = Bl[n3 + na], va = Bl[2 * n3 + na], wa = Bl[3 * n3 + na],
                     pa = Bl[4 * n3 + na], xa = Bl[5 * n3 + na];
        const double ma0 = Bl[mc * n3 + na], ma1 = Bl[(mc + 1) * n3 + na], ma2 = Bl[(mc + 2) * n3 + na];
        double aa[5];
#pragma unroll
        for (int v = 0; v < 5; ++v) aa[v] = Al[v * n3 + na];
        double acc[6];
#pragma unroll
        for (int c = 0; c < 6; ++c) acc[c] = Cl[c * n3 + na];
#pragma unroll 4
        for (int b = a + 1; b < NP; ++b) {
          const int nb = vsw<NP>(base + b * stride);
          const double dba = sb.DVS[b + n * a], dab = sb.DVS[a + n * b];
          double Fb[5];
#pragma unroll
          for (int v = 0; v < 5; ++v) Fb[v] = dba * aa[v] + dab * Al[v * n3 + nb];
          double sbar[6];
          pair_sum_vjp<SPLIT>(ra + Bl[nb], ua + Bl[n3 + nb], va + Bl[2 * n3 + nb], wa + Bl[3 * n3 + nb],
                              pa + Bl[4 * n3 + nb], xa + Bl[5 * n3 + nb], ma0 + Bl[mc * n3 + nb],
                              ma1 + Bl[(mc + 1) * n3 + nb], ma2 + Bl[(mc + 2) * n3 + nb], Fb, sbar);
#pragma unroll
          for (int c = 0; c < 6; ++c) {
            acc[c] += sbar[c];
            Cl[c * n3 + nb] += sbar[c];
          }
        }
#pragma unroll
        for (int c = 0; c < 6; ++c) Cl[c * n3 + na] = acc[c];
      }
    }
    __syncthreads();
  }

  // ---- phase C: per node: pair cotangents, transposed weak volume integral, viscous volume flux
  double rb = 0., ub_ = 0., vb = 0., wb = 0., pb = 0., xb = 0., srb = 0., Eb = 0., m1b = 0., m2b = 0., m3b = 0.;
  double gb[15];
#pragma unroll
  for (int c = 0; c < 15; ++c) gb[c] = 0.;
  if (active) {
    if constexpr (SPLIT >= 0) {
      double s6[6];
#pragma unroll
      for (int c = 0; c < 6; ++c) s6[c] = Cs[c * n3 + snode] + Cs[(6 + c) * n3 + snode] + Cs[(12 + c) * n3 + snode];
      rb = s6[0]; ub_ = s6[1]; vb = s6[2]; wb = s6[3]; pb = s6[4]; xb = s6[5];
    }
    if (SPLIT < 0 || PARAB) {
      // transposed ApplyDMatrix: flb[d][v](y) = sum over the d-line of D_hat^T(l_y, i_x) a(x)
      double flb[3][5];
#pragma unroll
      for (int d = 0; d < 3; ++d)
#pragma unroll
        for (int v = 0; v < 5; ++v) flb[d][v] = 0.;
      constexpr int v0 = (SPLIT < 0) ? 0 : 1;  // the viscous fluxes have no density row
#pragma unroll
      for (int l = 0; l < n; ++l) {
        const double ci = sb.DhatT[i + n * l], cj = sb.DhatT[j + n * l], ck = sb.DhatT[k + n * l];
        const int ni = vsw<NP>(l + n * (j + n * k)), nj = vsw<NP>(i + n * (l + n * k)), nk = vsw<NP>(i + n * (j + n * l));
#pragma unroll
        for (int v = v0; v < 5; ++v) {
          flb[0][v] += ci * Aa[v * n3 + ni];
          flb[1][v] += cj * Aa[v * n3 + nj];
          flb[2][v] += ck * Aa[v * n3 + nk];
        }
      }
      const double Ms[3][3] = {{M[0], M[n3], M[2 * n3]}, {M[3 * n3], M[4 * n3], M[5 * n3]},
                               {M[6 * n3], M[7 * n3], M[8 * n3]}};
      const double vel[3] = {P[n3], P[2 * n3], P[3 * n3]};
      if (SPLIT < 0) {
        // EvalTransformedEulerFlux3D: fl[d] = Mmom (1, v, Ep) + Ms[d] p (momentum rows)
        const double m[3] = {U[gU + 1], U[gU + 2], U[gU + 3]};
        const double E = U[gU + 4], p = P[4 * n3], srho = P[6 * n3];
        const double Ep = (E + p) * srho;
        double Epb = 0.;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          const double Mmom = Ms[d][0] * m[0] + Ms[d][1] * m[1] + Ms[d][2] * m[2];
          const double Mmb = flb[d][0] + flb[d][1] * vel[0] + flb[d][2] * vel[1] + flb[d][3] * vel[2] + flb[d][4] * Ep;
          ub_ += flb[d][1] * Mmom; vb += flb[d][2] * Mmom; wb += flb[d][3] * Mmom;
          pb += flb[d][1] * Ms[d][0] + flb[d][2] * Ms[d][1] + flb[d][3] * Ms[d][2];
          Epb += flb[d][4] * Mmom;
          m1b += Mmb * Ms[d][0]; m2b += Mmb * Ms[d][1]; m3b += Mmb * Ms[d][2];
        }
        Eb += Epb * srho;
        pb += Epb * srho;
        srb += Epb * (E + p);
      }
      if (PARAB) {
        const double* G = Gvol + (size_t)e * 15 * n3 + node;
        double gg[15];
#pragma unroll
        for (int c = 0; c < 15; ++c) gg[c] = G[c * n3];
        double tau[6], tq[3];
        visc_stress(gg, gg + 5, gg + 10, vel, L.mu, L.lambda, tau, tq);
        double taub[6] = {0, 0, 0, 0, 0, 0}, tqb[3] = {0, 0, 0}, velb[3] = {0, 0, 0};
#pragma unroll
        for (int d = 0; d < 3; ++d) visc_dir_vjp(Ms[d], flb[d], taub, tqb);
        // d/dmu of the viscous contravariant fluxes = the fluxes / mu: (taub . tau + tqb . tq) / mu
        if (L.inv_mu > 0.) {
          mub += (taub[0] * tau[0] + taub[1] * tau[1] + taub[2] * tau[2] + taub[3] * tau[3] + taub[4] * tau[4] +
                  taub[5] * tau[5] + tqb[0] * tq[0] + tqb[1] * tq[1] + tqb[2] * tq[2]) * L.inv_mu;
        } else {
          double tau1[6], tq1[3];
          visc_stress(gg, gg + 5, gg + 10, vel, 1., L.lamc, tau1, tq1);
          mub += taub[0] * tau1[0] + taub[1] * tau1[1] + taub[2] * tau1[2] + taub[3] * tau1[3] + taub[4] * tau1[4] +
                 taub[5] * tau1[5] + tqb[0] * tq1[0] + tqb[1] * tq1[1] + tqb[2] * tq1[2];
        }
        visc_close_vjp(tau, vel, L.mu, L.lambda, taub, tqb, gb, velb);
        ub_ += velb[0]; vb += velb[1]; wb += velb[2];
      }
    }
  }
  __syncthreads();  // all reads of a, node data and pair accumulators are complete

  // ---- phase D: gradient cotangents (volume + face traces) and the lifting weights
  if (PARAB && active) {
    // transposed ProlongToFaceLifting: the face-trace cotangents come back to the line nodes
#pragma unroll
    for (int ls = 1; ls <= 6; ++ls) {
      int a, b, l;
      switch (ls) {
        case L_XI_MINUS: case L_XI_PLUS: a = j; b = k; l = i; break;
        case L_ETA_MINUS: case L_ETA_PLUS: a = i; b = k; l = j; break;
        default: a = i; b = j; l = k; break;
      }
      const bool minus = is_minus(ls);
      double Lv;
      if (L.gauss) Lv = minus ? sb.Lm[l] : sb.Lp[l];
      else {
        if (l != (minus ? 0 : N)) continue;
        Lv = 1.;
      }
      const int side = E2S[(e * 6 + ls - 1) * 2 + 0];
      const int flip = E2S[(e * 6 + ls - 1) * 2 + 1];
      int p, q;
      s2v2_inv(N, a, b, flip, ls, p, q);
      const double* gf = GfB + ((size_t)(flip == 0 ? 0 : 1) * L.nSides + side) * 15 * n2 + p + n * q;
#pragma unroll
      for (int c = 0; c < 15; ++c) gb[c] += Lv * gf[c * n2];
    }
    const double sj = M[9 * n3];
#pragma unroll
    for (int c = 0; c < 15; ++c) Bs[c * n3 + snode] = gb[c];
    if (L.lift_mode == 0) {
      // h_dir[v] = sJ sum_d Mdir_d Gbar_d[v]
#pragma unroll
      for (int dir = 0; dir < 3; ++dir) {
        const double m0 = sj * M[(3 * dir) * n3], m1 = sj * M[(3 * dir + 1) * n3], m2 = sj * M[(3 * dir + 2) * n3];
#pragma unroll
        for (int v = 0; v < 5; ++v) Cs[(dir * 5 + v) * n3 + snode] = m0 * gb[v] + m1 * gb[5 + v] + m2 * gb[10 + v];
      }
    } else {
      // conservative: h'_d[v] = sJ Gbar_d[v]
#pragma unroll
      for (int c = 0; c < 15; ++c) Cs[c * n3 + snode] = sj * gb[c];
    }
  }
  __syncthreads();

  if (active) {
    if (PARAB) {
      // transposed lifting volume integral -> cotangents of (rho, u, v, w, T) at this node
      double lb[5] = {0, 0, 0, 0, 0};
      if (L.lift_mode == 0) {
#pragma unroll
        for (int l = 0; l < n; ++l) {
          const double ci = sb.D[l + n * i], cj = sb.D[l + n * j], ck = sb.D[l + n * k];
          const int ni = vsw<NP>(l + n * (j + n * k)), nj = vsw<NP>(i + n * (l + n * k)),
                    nk = vsw<NP>(i + n * (j + n * l));
#pragma unroll
          for (int v = 0; v < 5; ++v)
            lb[v] += ci * Cs[v * n3 + ni] + cj * Cs[(5 + v) * n3 + nj] + ck * Cs[(10 + v) * n3 + nk];
        }
      } else {
        // g_d(x) = sJ(x) sum_dir sum_l D(i_x,l) Mdir_d(x_l) P(x_l): the metric sits at the summed node
#pragma unroll
        for (int dir = 0; dir < 3; ++dir) {
          const double m0 = M[(3 * dir) * n3], m1 = M[(3 * dir + 1) * n3], m2 = M[(3 * dir + 2) * n3];
          const int ii = dir == 0 ? i : (dir == 1 ? j : k);
#pragma unroll
          for (int l = 0; l < n; ++l) {
            const double c = sb.D[l + n * ii];
            const int nx = vsw<NP>(dir == 0 ? l + n * (j + n * k) : (dir == 1 ? i + n * (l + n * k) : i + n * (j + n * l)));
#pragma unroll
            for (int v = 0; v < 5; ++v)
              lb[v] += c * (m0 * Cs[v * n3 + nx] + m1 * Cs[(5 + v) * n3 + nx] + m2 * Cs[(10 + v) * n3 + nx]);
          }
        }
      }
      rb += lb[0]; ub_ += lb[1]; vb += lb[2]; wb += lb[3];
      const double Tb = lb[4];
      // split aux: PI H = (E + p)/rho, KG E/rho
      const double srho = P[6 * n3];
      if constexpr (SPLIT == DG_SPLIT_PI) {
        Eb += xb * srho; pb += xb * srho; srb += xb * (U[gU + 4] + P[4 * n3]);
      } else if constexpr (SPLIT == DG_SPLIT_KG) {
        Eb += xb * srho; srb += xb * U[gU + 4];
      }
      const double Un[5] = {U[gU], U[gU + 1], U[gU + 2], U[gU + 3], U[gU + 4]};
      double Ub[5] = {0, 0, 0, 0, 0};
      prim_vjp(Un, L.kappa - 1., L.sR, rb, ub_, vb, wb, pb, Tb, srb, Eb, m1b, m2b, m3b, Ub);
#pragma unroll
      for (int v = 0; v < 5; ++v) UBv[gU + v] = Ub[v];
    } else {
      const double srho = P[6 * n3];
      if constexpr (SPLIT == DG_SPLIT_PI) {
        Eb += xb * srho; pb += xb * srho; srb += xb * (U[gU + 4] + P[4 * n3]);
      } else if constexpr (SPLIT == DG_SPLIT_KG) {
        Eb += xb * srho; srb += xb * U[gU + 4];
      }
      const double Un[5] = {U[gU], U[gU + 1], U[gU + 2], U[gU + 3], U[gU + 4]};
      double Ub[5] = {0, 0, 0, 0, 0};
      prim_vjp(Un, L.kappa - 1., L.sR, rb, ub_, vb, wb, pb, 0., srb, Eb, m1b, m2b, m3b, Ub);
#pragma unroll
      for (int v = 0; v < 5; ++v) UBv[gU + v] = Ub[v];
    }
  }
  // lifting jump cotangent, this element's share: JB[slot][side][v][pq] =
  //   sum over the line (GL: the face node) of L_hat 0.5 SE sJ n . Gbar
  if (PARAB) {
    for (int t = threadIdx.x; t < nloc * 6 * n2; t += blockDim.x) {
      const int el2 = t / (6 * n2), r = t - el2 * 6 * n2;
      const int ls = r / n2 + 1, pq = r - (ls - 1) * n2;
      const int p = pq % n, q = pq / n;
      const int e2 = e0 + el2;
      const int side = E2S[(e2 * 6 + ls - 1) * 2 + 0];
      const int flip = E2S[(e2 * 6 + ls - 1) * 2 + 1];
      int a, b;
      s2v2(N, p, q, flip, ls, a, b);
      const bool minus = is_minus(ls);
      const double* fg = Fgeo + (size_t)side * 10 * n2 + pq;
      const double nv[3] = {fg[0], fg[n2], fg[2 * n2]};
      const double hse = 0.5 * fg[9 * n2];
      const double* Bl = sm + (size_t)el2 * 38 * n3 + 5 * n3;
      const double* sJe = Met + ((size_t)e2 * 10 + 9) * n3;
      double jb[5] = {0, 0, 0, 0, 0};
      const int l0 = L.gauss ? 0 : (minus ? 0 : N), l1 = L.gauss ? N : l0;
      for (int l = l0; l <= l1; ++l) {
        const double Lh = L.gauss ? (minus ? sb.Lhm[l] : sb.Lhp[l]) : (minus ? sb.Lhm[0] : sb.Lhp[N]);
        const int x = face_node(n, ls, a, b, l), sx = vsw<NP>(x);
        const double w = Lh * hse * sJe[x];
#pragma unroll
        for (int v = 0; v < 5; ++v)
          jb[v] += w * (nv[0] * Bl[v * n3 + sx] + nv[1] * Bl[(5 + v) * n3 + sx] + nv[2] * Bl[(10 + v) * n3 + sx]);
      }
      double* out = JB + ((size_t)(flip == 0 ? 0 : 1) * L.nSides + side) * 5 * n2 + pq;
#pragma unroll
      for (int v = 0; v < 5; ++v) out[v * n2] = jb[v];
    }
  }
  // block partial of dR/dmu in a fixed order (the block's last warp may be partial: no shuffles
  // across it); the a-area of the shared memory is free again here
  __syncthreads();
  sm[threadIdx.x] = mub;
  __syncthreads();
  if (threadIdx.x < 32) {
    double s = 0.;
    for (int t = threadIdx.x; t < (int)blockDim.x; t += 32) s += sm[t];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (threadIdx.x == 0) mupart[blockIdx.x] = s;
  }
}

// ---------------------------------------------------------------------------------------------
// ka_jump: thread per face node; the lifting surface term 0.5 SE (P_slave - P_master) n transposed
// through ConsToPrim of both face states, added to the face-state cotangents in place
// ---------------------------------------------------------------------------------------------
static __global__ void __launch_bounds__(256)
ka_jump(const double* __restrict__ Uf, const double* __restrict__ JB, AdjLaunch L, int n2, double* __restrict__ UfB) {
  // connected sides only; the BC sides' lifting jump goes through the ghost state (ka_bc_jump)
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x + (long long)L.nBCSides * n2;
  if (t >= (long long)L.nSides * n2) return;
  const int side = (int)(t / n2), pq = (int)(t - (long long)side * n2);
  const size_t S = L.nSides;
  double jb[5];
#pragma unroll
  for (int v = 0; v < 5; ++v)
    jb[v] = JB[(size_t)side * 5 * n2 + v * n2 + pq] + JB[(S + side) * 5 * n2 + v * n2 + pq];
#pragma unroll
  for (int slot = 0; slot < 2; ++slot) {
    const double sg = slot == 0 ? -1. : 1.;
    double uf[5], fb[5];
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      uf[v] = Uf[((size_t)slot * S + side) * 5 * n2 + v * n2 + pq];
      fb[v] = UfB[((size_t)slot * S + side) * 5 * n2 + v * n2 + pq];
    }
    prim_vjp(uf, L.kappa - 1., L.sR, sg * jb[0], sg * jb[1], sg * jb[2], sg * jb[3], 0., sg * jb[4], 0., 0., 0., 0.,
             0., fb);
#pragma unroll
    for (int v = 0; v < 5; ++v) UfB[((size_t)slot * S + side) * 5 * n2 + v * n2 + pq] = fb[v];
  }
}

// ---------------------------------------------------------------------------------------------
// Boundary sides.  The forward boundary flux k_bc_face (GetBoundaryFlux_GPU, getboundaryflux.f90:
// 542-838) and the lifting ghost state of k_bc_lift_ghost (Lifting_GetBoundaryFlux_Kernel, :945-1019)
// depend on the master face state U_f (through ConsToPrim) and, for the flux, on the master face
// gradients G_f and the viscosity.  Their transposes take the local Jacobians by forward-mode dual
// numbers (the forward device code instantiated on Dual<K>): few face nodes are boundary nodes.
// ---------------------------------------------------------------------------------------------
template <int K>
__device__ __forceinline__ Gas<Dual<K>> dual_gas(const Gas<double>& g, int mu_slot, double lamc) {
  using D = Dual<K>;
  Gas<D> r;
  r.kappa = D(g.kappa); r.kappaM1 = D(g.kappaM1); r.sKappaM1 = D(g.sKappaM1); r.R_gas = D(g.R_gas);
  r.mu = D(g.mu); r.lambda = D(g.lambda); r.sR = D(g.sR);
  r.pref = D(0.); r.prefD = 0.; r.kappaM1D = g.kappaM1D; r.sRD = g.sRD;
  if (mu_slot >= 0) { r.mu.d[mu_slot] = 1.; r.lambda.d[mu_slot] = lamc; }
  return r;
}

// ka_bc_face: thread per BC face node.  Flux cotangent (transposed SurfInt of the master element,
// times SurfElem) through the boundary flux's Jacobian with respect to U_f (5), the lifted gradients
// of u, v, w, T in x, y, z (12) and mu (slot 17): cotangents of U_f and G_f of the master side and
// the block's share of <Ut_bar, dR/dmu>.
template <int NP>
__global__ void __launch_bounds__(128)
ka_bc_face(CotSrc cs, const double* __restrict__ Met, const double* __restrict__ Uf, const double* __restrict__ Gf,
           const double* __restrict__ Fgeo, const int* __restrict__ S2E, DevBasis<double> basis, Gas<double> gas,
           AdjLaunch L, double* __restrict__ UfB, double* __restrict__ GfB, double* __restrict__ mupart) {
  constexpr int n = NP, n2 = NP * NP, n3 = NP * NP * NP, N = NP - 1;
  using D = Dual<18>;
  __shared__ double red[4];
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double mub = 0.;
  if (t < (long long)L.nBCSides * n2) {
    const int side = (int)(t / n2), pq = (int)(t - (long long)side * n2);
    const int p = pq % n, q = pq / n;
    const int e = S2E[(size_t)side * 5], ls = S2E[(size_t)side * 5 + 1];
    int a, b;
    s2v2(N, p, q, 0, ls, a, b);
    const bool minus = is_minus(ls);
    double Fb[5] = {0, 0, 0, 0, 0};
    const int l0 = L.gauss ? 0 : (minus ? 0 : N), l1 = L.gauss ? N : l0;
    for (int l = l0; l <= l1; ++l) {
      const double Lh = L.gauss ? (minus ? basis.Lhm[l] : basis.Lhp[l]) : (minus ? basis.Lhm[0] : basis.Lhp[N]);
      const int node = face_node(n, ls, a, b, l);
      const double sj = Met[((size_t)e * 10 + 9) * n3 + node];
      double ub[5];
      cot_at(cs, ((size_t)e * n3 + node) * 5, ub);
      const double w = -Lh * sj;
#pragma unroll
      for (int v = 0; v < 5; ++v) Fb[v] = Fb[v] + w * ub[v];
    }
    const double* fg = Fgeo + (size_t)side * 10 * n2 + pq;
    const double se = fg[9 * n2];
#pragma unroll
    for (int v = 0; v < 5; ++v) Fb[v] *= se;
    // the boundary flux on dual numbers: seeds U_f (0..4), gradients of u, v, w, T (5..16), mu (17)
    const Gas<D> g = dual_gas<18>(gas, 17, L.lamc);
    D U[5], PL[6], srho, gx[5], gy[5], gz[5];
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      U[v] = D(Uf[(size_t)side * 5 * n2 + v * n2 + pq]);
      U[v].d[v] = 1.;
    }
    cons_to_prim_d(U, g, PL, srho);
    const double* gm = Gf + (size_t)side * 15 * n2 + pq;
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      gx[v] = D(L.parabolic ? gm[v * n2] : 0.);
      gy[v] = D(L.parabolic ? gm[(5 + v) * n2] : 0.);
      gz[v] = D(L.parabolic ? gm[(10 + v) * n2] : 0.);
    }
#pragma unroll
    for (int v = 1; v < 5; ++v) { gx[v].d[4 + v] = 1.; gy[v].d[8 + v] = 1.; gz[v].d[12 + v] = 1.; }
    const D nv[3] = {D(fg[0]), D(fg[n2]), D(fg[2 * n2])};
    const D t1[3] = {D(fg[3 * n2]), D(fg[4 * n2]), D(fg[5 * n2])};
    const D t2[3] = {D(fg[6 * n2]), D(fg[7 * n2]), D(fg[8 * n2])};
    const double* rs = L.bcref + 6 * L.bcstate[side];
    const D ref[6] = {D(rs[0]), D(rs[1]), D(rs[2]), D(rs[3]), D(rs[4]), D(rs[5])};
    D F[5];
    bc_face_flux(L.bctype[side], PL, gx, gy, gz, nv, t1, t2, ref, g, L.riemann, L.split, L.parabolic, F);
    double ub[5] = {0, 0, 0, 0, 0}, gb[15];
#pragma unroll
    for (int c = 0; c < 15; ++c) gb[c] = 0.;
#pragma unroll
    for (int w = 0; w < 5; ++w) {
#pragma unroll
      for (int v = 0; v < 5; ++v) ub[v] += Fb[w] * F[w].d[v];
#pragma unroll
      for (int v = 1; v < 5; ++v) {
        gb[v] += Fb[w] * F[w].d[4 + v];
        gb[5 + v] += Fb[w] * F[w].d[8 + v];
        gb[10 + v] += Fb[w] * F[w].d[12 + v];
      }
      mub += Fb[w] * F[w].d[17];
    }
#pragma unroll
    for (int v = 0; v < 5; ++v) UfB[(size_t)side * 5 * n2 + v * n2 + pq] = ub[v];
    if (L.parabolic) {
#pragma unroll
      for (int c = 0; c < 15; ++c) GfB[(size_t)side * 15 * n2 + c * n2 + pq] = gb[c];
    }
  }
  for (int o = 16; o > 0; o >>= 1) mub += __shfl_xor_sync(0xffffffffu, mub, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mub;
  __syncthreads();
  if (threadIdx.x == 0) mupart[blockIdx.x] = red[0] + red[1] + red[2] + red[3];
}

// ka_bc_jump: thread per BC face node.  The master element's lifting used the jump ghost(P_m) - P_m of
// the lifted variables (rho, u, v, w, T); its cotangent (the master share of JB) goes through that jump's
// Jacobian with respect to U_f (ConsToPrim, GetBoundaryState, the ghost state) into the U_f cotangent.
static __global__ void __launch_bounds__(256)
ka_bc_jump(const double* __restrict__ Uf, const double* __restrict__ JB, const double* __restrict__ Fgeo,
           Gas<double> gas, AdjLaunch L, int n2, double* __restrict__ UfB) {
  using D = Dual<5>;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)L.nBCSides * n2) return;
  const int side = (int)(t / n2), pq = (int)(t - (long long)side * n2);
  const Gas<D> g = dual_gas<5>(gas, -1, 0.);
  D U[5], Pm[6], srho, Pb[6], gh[5];
#pragma unroll
  for (int v = 0; v < 5; ++v) {
    U[v] = D(Uf[(size_t)side * 5 * n2 + v * n2 + pq]);
    U[v].d[v] = 1.;
  }
  cons_to_prim_d(U, g, Pm, srho);
  const double* fg = Fgeo + (size_t)side * 10 * n2 + pq;
  const D nv[3] = {D(fg[0]), D(fg[n2]), D(fg[2 * n2])};
  const D t1[3] = {D(fg[3 * n2]), D(fg[4 * n2]), D(fg[5 * n2])};
  const D t2[3] = {D(fg[6 * n2]), D(fg[7 * n2]), D(fg[8 * n2])};
  const double* rs = L.bcref + 6 * L.bcstate[side];
  const D ref[6] = {D(rs[0]), D(rs[1]), D(rs[2]), D(rs[3]), D(rs[4]), D(rs[5])};
  const int bt = L.bctype[side];
  bc_state(bt, Pm, ref, nv, t1, t2, g.kappa, g.R_gas, Pb);
  bc_lift_ghost(bt, Pm, Pb, gh);
  const int liftc[5] = {0, 1, 2, 3, 5};
  double ub[5];
#pragma unroll
  for (int v = 0; v < 5; ++v) ub[v] = UfB[(size_t)side * 5 * n2 + v * n2 + pq];
#pragma unroll
  for (int c = 0; c < 5; ++c) {
    const double jb = JB[(size_t)side * 5 * n2 + c * n2 + pq];
    const D jump = gh[c] - Pm[liftc[c]];
#pragma unroll
    for (int v = 0; v < 5; ++v) ub[v] += jb * jump.d[v];
  }
#pragma unroll
  for (int v = 0; v < 5; ++v) UfB[(size_t)side * 5 * n2 + v * n2 + pq] = ub[v];
}

// ---------------------------------------------------------------------------------------------
// ka_final: thread per node; transposed ProlongToFace of the face cotangents, then output
// mode 0: Ubar_out = dR^T Ut_bar;  mode 1 (reverse RK stage): K = Kbar + b dt Ubar,
//   Ubar += dR^T K,  Kbar = mRKA K   (Ut_bar = K was the cotangent source of the stage)
// ---------------------------------------------------------------------------------------------
template <int NP>
__global__ void __launch_bounds__(256)
ka_final(const double* __restrict__ UBv, const double* __restrict__ UfB, const int* __restrict__ E2S,
         DevBasis<double> basis, AdjLaunch L, int mode, double* __restrict__ Uout, double* __restrict__ Ubar,
         double* __restrict__ Kbar, double b_dt, double mRKA) {
  constexpr int n = NP, n2 = NP * NP, n3 = NP * NP * NP, N = NP - 1;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)L.nElems * n3) return;
  const int e = (int)(t / n3), node = (int)(t - (long long)e * n3);
  const int i = node % n, j = (node / n) % n, k = node / n2;
  const size_t S = L.nSides;
  double Ub[5];
#pragma unroll
  for (int v = 0; v < 5; ++v) Ub[v] = UBv[t * 5 + v];
#pragma unroll
  for (int ls = 1; ls <= 6; ++ls) {
    int a, b, l;
    switch (ls) {
      case L_XI_MINUS: case L_XI_PLUS: a = j; b = k; l = i; break;
      case L_ETA_MINUS: case L_ETA_PLUS: a = i; b = k; l = j; break;
      default: a = i; b = j; l = k; break;
    }
    const bool minus = is_minus(ls);
    double Lv;
    if (L.gauss) Lv = minus ? basis.Lm[l] : basis.Lp[l];
    else {
      if (l != (minus ? 0 : N)) continue;
      Lv = 1.;
    }
    const int side = E2S[(e * 6 + ls - 1) * 2 + 0];
    const int flip = E2S[(e * 6 + ls - 1) * 2 + 1];
    const int slot = flip == 0 ? 0 : 1;
    int p, q;
    s2v2_inv(N, a, b, flip, ls, p, q);
    const int pq = p + n * q;
#pragma unroll
    for (int v = 0; v < 5; ++v) Ub[v] += Lv * UfB[((size_t)slot * S + side) * 5 * n2 + v * n2 + pq];
  }
  if (mode == 0) {
#pragma unroll
    for (int v = 0; v < 5; ++v) Uout[t * 5 + v] = Ub[v];
  } else {
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      const double ubar = Ubar[t * 5 + v];
      const double K = Kbar[t * 5 + v] + b_dt * ubar;
      Ubar[t * 5 + v] = ubar + Ub[v];
      Kbar[t * 5 + v] = mRKA * K;
    }
  }
}

// fixed-order sum of the per-block partials into *acc (one block)
static __global__ void __launch_bounds__(256) k_adj_sum(const double* __restrict__ part, int cnt, double* __restrict__ acc) {
  __shared__ double s[256];
  double v = 0.;
  for (int t = threadIdx.x; t < cnt; t += 256) v += part[t];
  s[threadIdx.x] = v;
  __syncthreads();
  for (int h = 128; h > 0; h >>= 1) {
    if (threadIdx.x < h) s[threadIdx.x] += s[threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x == 0) *acc += s[0];
}

}  // namespace gx
