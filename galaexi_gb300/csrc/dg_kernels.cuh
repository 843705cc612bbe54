// Fused DGSEM kernels for sm_103a.
//
// One RHS evaluation (DGTimeDerivative_weakForm, src/dg/dg.f90:255-425) runs as four launches:
//   k_prolong  element-per-block   ConsToPrim (volume) + ProlongToFace + ConsToPrim (faces)
//   k_lift     element-per-block   BR1 lifting: volume part, surface part, Jacobian, gradient traces
//   k_face     thread-per-face-node Riemann solver + BR1 viscous flux + SurfElem
//   k_volume   element-per-block   volume integral (weak or split form, viscous part), surface
//                                  integral, sign, Jacobian, and optionally the LSERK-W2 stage update
// (k_lift is skipped for the Euler equations; a solution filter adds k_filter / k_filter_laf in front,
// meshes with boundary sides add k_bc_lift_ghost before k_lift and k_bc_face beside k_face.)  The
// reference runs ~25-35 launches per stage with full-size intermediates; here the element's state
// lives in shared memory inside each phase.
//
// Layouts (internal, all per element contiguous so that element blocks load coalesced):
//   Pvol [e][7][n^3]     rho,u,v,w,p,T,1/rho                 (compute type R)
//   Gvol [e][15][n^3]    d/dx (rho,u,v,w,T), d/dy (..), d/dz (..)
//   Met  [e][10][n^3]    Mf(3), Mg(3), Mh(3), sJ
//   Uf   [slot][side][5][n^2], Pf [slot][side][6][n^2], Gf [slot][side][15][n^2]  (slot 0 master, 1 slave)
//   Fgeo [side][10][n^2] nv(3), t1(3), t2(3), SurfElem
//   Flux [side][5][n^2]
// The caller's U / Ut / Ut_tmp keep the reference layout (5,0:N,0:N,0:N,nElems), FP64.
#pragma once
#include "dg_physics.cuh"
#include "dg_bc.cuh"
#include "dg_tma.cuh"

namespace gx {

enum { L_ZETA_MINUS = 1, L_ETA_MINUS = 2, L_XI_PLUS = 3, L_ETA_PLUS = 4, L_XI_MINUS = 5, L_ZETA_PLUS = 6 };

// Side <-> volume index maps of src/mesh/mappings.f90 (CGNS_SideToVol2 after Flip_M2S), computed
// arithmetically instead of read from the S2V2 table.  Both factors are involutions.
__device__ __forceinline__ void flip_map(int N, int p, int q, int flip, int& a, int& b) {
  switch (flip) {
    case 0: a = p; b = q; break;
    case 1: a = q; b = p; break;
    case 2: a = N - p; b = q; break;
    case 3: a = N - q; b = N - p; break;
    default: a = p; b = N - q; break;
  }
}
__device__ __forceinline__ void cgns_map(int N, int p, int q, int ls, int& a, int& b) {
  switch (ls) {
    case L_XI_MINUS: case L_ZETA_MINUS: a = q; b = p; break;
    case L_ETA_PLUS: a = N - p; b = q; break;
    default: a = p; b = q; break;
  }
}
// S2V2(p,q,flip,ls): side node (master frame) -> volume face coordinates (a,b)
__device__ __forceinline__ void s2v2(int N, int p, int q, int flip, int ls, int& a, int& b) {
  int pp, qq;
  flip_map(N, p, q, flip, pp, qq);
  cgns_map(N, pp, qq, ls, a, b);
}
// inverse: volume face coordinates (a,b) -> side node (p,q)
__device__ __forceinline__ void s2v2_inv(int N, int a, int b, int flip, int ls, int& p, int& q) {
  int pp, qq;
  cgns_map(N, a, b, ls, pp, qq);
  flip_map(N, pp, qq, flip, p, q);
}
// volume node of face coordinates (a,b) at line position l for local side ls
__device__ __forceinline__ int face_node(int n, int ls, int a, int b, int l) {
  switch (ls) {
    case L_XI_MINUS: case L_XI_PLUS: return l + n * (a + n * b);
    case L_ETA_MINUS: case L_ETA_PLUS: return a + n * (l + n * b);
    default: return a + n * (b + n * l);
  }
}
__device__ __forceinline__ bool is_minus(int ls) { return ls == L_XI_MINUS || ls == L_ETA_MINUS || ls == L_ZETA_MINUS; }

template <typename R>
struct DevBasis {
  const R* D;          // D(i,l), column-major (0:N,0:N)
  const R* DhatT;      // D_hat^T(l,i)
  const R* DVS;        // DVolSurf(l,i)
  const R* Lm;         // L_minus(0:N)
  const R* Lp;         // L_plus(0:N)
  const R* Lhm;        // L_hat_minus(0:N)
  const R* Lhp;        // L_hat_plus(0:N)
};

// shared copy of the 1D operators (n^2 entries each)
template <int NP, typename R>
struct SBasis {
  R D[NP * NP], DhatT[NP * NP], DVS[NP * NP], Lm[NP], Lp[NP], Lhm[NP], Lhp[NP];
};
template <int NP, typename R>
__device__ __forceinline__ void load_basis(SBasis<NP, R>& s, const DevBasis<R>& b) {
  for (int t = threadIdx.x; t < NP * NP; t += blockDim.x) {
    s.D[t] = b.D[t]; s.DhatT[t] = b.DhatT[t]; s.DVS[t] = b.DVS[t];
  }
  for (int t = threadIdx.x; t < NP; t += blockDim.x) {
    s.Lm[t] = b.Lm[t]; s.Lp[t] = b.Lp[t]; s.Lhm[t] = b.Lhm[t]; s.Lhp[t] = b.Lhp[t];
  }
}

struct Launch {
  int nElems, nSides;
  int gauss;        // 1: Gauss nodes (prolongation by interpolation), 0: Gauss-Lobatto
  int riemann, split, parabolic;
  int lift_mode;    // 0: strong non-conservative, 1: strong conservative, 2: weak
  int br2;          // 1: BR2 face traces (lifting_br2.t90:191-310), strong form only
  double eta_br2;   // BR2 penalty etaBR2
  // boundary sides: the first nBCSides sides; per side BC type and reference-state index, and the
  // reference states (compute type, [state][6]); see dg_bc.cuh
  int nBCSides;
  const int* bctype;
  const int* bcstate;
  const void* bcref;
};

// Shared-memory position of node i + n(j + nk) in the element stagings of k_lift and k_volume.  N=7: the i and j bits
// are XOR-swizzled with bits of j and k so that the x-, y- and z-line threads of phase B and the
// node threads hit 32 distinct FP32 banks (two wavefronts per FP64 access); the plain layout gave
// 8-way (FP32) and 16-way (FP64) conflicts on the x-lines.  An involution that permutes each block
// of 32 consecutive nodes.
template <int NP>
__device__ __forceinline__ int vsw(int node) {
  if constexpr (NP == 8) {
    const int kk = (node >> 6) & 3;
    return node ^ ((((node >> 5) & 1) << 2) | kk | (kk << 3));
  } else {
    return node;
  }
}

template <int NP> struct EPBof { static constexpr int v = (NP * NP * NP >= 128) ? 1 : (256 / (NP * NP * NP)); };
// k_lift: shared-memory slots per element of the region that holds the lifted primitives (5 n^3) and
// later the surface flux vectors of one normal direction (2 faces x 15 x n^2)
__host__ __device__ constexpr int lift_ps_slots(int NP) { return 5 * NP * NP * NP > 30 * NP * NP ? 5 * NP * NP * NP : 30 * NP * NP; }

// =====================================================================================
// k_prolong: ConsToPrim_Volume + ProlongToFace_CUDA + GetPrimitiveStateSurface.  At least two
// blocks per SM for the FP64 form (FP64-issue bound); three for the mixed form up to N = 7, whose FP64
// work is only E - ke and p - p_ref once its conversions run on the integer pipes (latency bound).
// =====================================================================================
template <int NP, typename R> struct ProlongMinBlocks {
  // three blocks per SM where they fit the SM's 2048 threads (the mixed form up to N = 7), else two;
  // the mixed form's element of 216 threads (N = 5) five
  static constexpr int v =
      (OffsetOf<R>::v && NP == 6) ? 5 : ((OffsetOf<R>::v && 3 * EPBof<NP>::v * NP * NP * NP <= 2048) ? 3 : 2);
};
template <int NP, typename R, typename S = double>
__global__ void __launch_bounds__(EPBof<NP>::v * NP * NP * NP, ProlongMinBlocks<NP, R>::v)
k_prolong(const S* __restrict__ U, const int* __restrict__ E2S, const double* __restrict__ Lm,
          const double* __restrict__ Lp, Gas<R> gas, Launch L, R* __restrict__ Pvol, R* __restrict__ Uf,
          R* __restrict__ Pf) {
  constexpr int n = NP, n2 = NP * NP, n3 = NP * NP * NP, EPB = EPBof<NP>::v, N = NP - 1;
  // mixed form: FP32 copies of density and momenta (converted once per node; Gauss nodes interpolate
  // them to the faces in FP32), the energy in FP64.  Static shared memory is limited to 48 KB, so N = 9
  // keeps the plain FP64 interpolation.
  constexpr bool C32 = OffsetOf<R>::v && (size_t)EPB * n3 * (5 * sizeof(S) + 4 * sizeof(R)) <= 40 * 1024;
  __shared__ SBasis<NP, double> sb;
  __shared__ S Us[EPB][5][n3];
  __shared__ R Cs[C32 ? EPB : 1][4][C32 ? n3 : 1];
  __shared__ R Lf[2][NP];
  for (int t = threadIdx.x; t < NP; t += blockDim.x) {
    sb.Lm[t] = Lm[t]; sb.Lp[t] = Lp[t];
    Lf[0][t] = (R)Lm[t]; Lf[1][t] = (R)Lp[t];
  }
  const int e0 = blockIdx.x * EPB;
  const int nloc = min(EPB, L.nElems - e0);
  // coalesced load of the element block (AoS (5,n^3) per element in global memory)
  const S* Ub = U + (size_t)e0 * 5 * n3;
  for (int t = threadIdx.x; t < nloc * 5 * n3; t += blockDim.x) {
    int el = t / (5 * n3), r = t - el * 5 * n3;
    Us[el][r % 5][r / 5] = Ub[t];
  }
  __syncthreads();
  // Volume prims.  On Gauss-Lobatto nodes a face trace is the face node's own state, so the node's
  // thread writes the traces of the faces it lies on (the same bits as a second ConsToPrim of the
  // copied trace, without its FP64 work).
  for (int t = threadIdx.x; t < nloc * n3; t += blockDim.x) {
    int el = t / n3, node = t - el * n3;
    R prim[6], srho;
    R uo[5];
    if constexpr (C32) {
      const R c[4] = {narrow<R>(Us[el][0][node]), narrow<R>(Us[el][1][node]), narrow<R>(Us[el][2][node]),
                      narrow<R>(Us[el][3][node])};
      if (L.gauss) {
#pragma unroll
        for (int v = 0; v < 4; ++v) Cs[el][v][node] = c[v];
      }
      const double E = Us[el][4][node];
      cons_to_prim_mixed(c, E, gas, prim, srho);
#pragma unroll
      for (int v = 0; v < 4; ++v) uo[v] = c[v];
      uo[4] = R(0);
      if (!L.gauss) uo[4] = narrow<R>(E);
    } else {
      const S u[5] = {Us[el][0][node], Us[el][1][node], Us[el][2][node], Us[el][3][node], Us[el][4][node]};
      cons_to_prim_d(u, gas, prim, srho);
#pragma unroll
      for (int v = 0; v < 5; ++v) uo[v] = (R)u[v];
    }
    R* P = Pvol + (size_t)(e0 + el) * 7 * n3 + node;
#pragma unroll
    for (int c = 0; c < 6; ++c) P[c * n3] = prim[c];
    P[6 * n3] = srho;
    if (!L.gauss) {
      const int i = node % n, j = (node / n) % n, k = node / n2;
      const int e = e0 + el;
      // local side ls, face coordinates (a,b) of this node on it (face_node(n, ls, a, b, 0 or N) == node)
      auto put = [&](int ls, int a, int b) {
        const int side = E2S[(e * 6 + ls - 1) * 2 + 0];
        const int flip = E2S[(e * 6 + ls - 1) * 2 + 1];
        int p, q;
        s2v2_inv(N, a, b, flip, ls, p, q);
        const int slot = (flip == 0) ? 0 : 1;
        R* uf = Uf + ((size_t)slot * L.nSides + side) * 5 * n2 + p + n * q;
        R* pf = Pf + ((size_t)slot * L.nSides + side) * 6 * n2 + p + n * q;
#pragma unroll
        for (int v = 0; v < 5; ++v) uf[v * n2] = uo[v];
#pragma unroll
        for (int c = 0; c < 6; ++c) pf[c * n2] = prim[c];
      };
      if (i == 0) put(L_XI_MINUS, j, k);
      if (i == N) put(L_XI_PLUS, j, k);
      if (j == 0) put(L_ETA_MINUS, i, k);
      if (j == N) put(L_ETA_PLUS, i, k);
      if (k == 0) put(L_ZETA_MINUS, i, j);
      if (k == N) put(L_ZETA_PLUS, i, j);
    }
  }
  if (!L.gauss) return;
  if constexpr (C32) __syncthreads();
  // Gauss nodes: face traces interpolated with L_minus / L_plus (ProlongToFace), then ConsToPrim
  for (int t = threadIdx.x; t < nloc * 6 * n2; t += blockDim.x) {
    int el = t / (6 * n2), r = t - el * 6 * n2;
    int ls = r / n2 + 1, pq = r - (ls - 1) * n2;
    int p = pq % n, q = pq / n;
    int e = e0 + el;
    int side = E2S[(e * 6 + ls - 1) * 2 + 0];
    int flip = E2S[(e * 6 + ls - 1) * 2 + 1];
    int a, b;
    s2v2(N, p, q, flip, ls, a, b);
    R prim[6], srho;
    R uo[5];
    if constexpr (C32) {
      const R* Lv = Lf[is_minus(ls) ? 0 : 1];
      const double* Ld = is_minus(ls) ? sb.Lm : sb.Lp;
      const int n0 = face_node(n, ls, a, b, 0);
      R c[4];
#pragma unroll
      for (int v = 0; v < 4; ++v) c[v] = Cs[el][v][n0] * Lv[0];
      double E = Us[el][4][n0] * Ld[0];
#pragma unroll
      for (int l = 1; l < n; ++l) {
        const int nl = face_node(n, ls, a, b, l);
#pragma unroll
        for (int v = 0; v < 4; ++v) c[v] = c[v] + Cs[el][v][nl] * Lv[l];
        E = E + Us[el][4][nl] * Ld[l];
      }
      cons_to_prim_mixed(c, E, gas, prim, srho);
#pragma unroll
      for (int v = 0; v < 4; ++v) uo[v] = c[v];
      uo[4] = narrow<R>(E);
    } else {
      S u[5];
      const double* Lv = is_minus(ls) ? sb.Lm : sb.Lp;
#pragma unroll
      for (int v = 0; v < 5; ++v) {
        S s = Us[el][v][face_node(n, ls, a, b, 0)] * Lv[0];
#pragma unroll
        for (int l = 1; l < n; ++l) s = s + Us[el][v][face_node(n, ls, a, b, l)] * Lv[l];
        u[v] = s;
      }
      cons_to_prim_d(u, gas, prim, srho);
#pragma unroll
      for (int v = 0; v < 5; ++v) uo[v] = (R)u[v];
    }
    const int slot = (flip == 0) ? 0 : 1;
    R* uf = Uf + ((size_t)slot * L.nSides + side) * 5 * n2 + pq;
    R* pf = Pf + ((size_t)slot * L.nSides + side) * 6 * n2 + pq;
#pragma unroll
    for (int v = 0; v < 5; ++v) uf[v * n2] = uo[v];
#pragma unroll
    for (int c = 0; c < 6; ++c) pf[c * n2] = prim[c];
  }
}

// =====================================================================================
// k_lift: Lifting_BR1 (lifting_br1.t90:47-167): volume part + surface part + sJ, then
// ProlongToFaceLifting.  Lifted variables (rho,u,v,w,T) = PRIM_LIFT (eos.h:143).
// =====================================================================================
// Boundary sides in the lifting: the slave slot of a BC side (no slave element) receives the ghost
// state 2F - P_master of the lifted variables (rho,u,v,w,T) for the reference's boundary lifting value
// F (Lifting_GetBoundaryFlux_Kernel, getboundaryflux.f90:945-1019); the BR1 flux 0.5 (P_master +
// ghost) (weak) and 0.5 (ghost - P_master) (strong), and the BR2 jump, then reproduce it, so the
// lifting kernel itself carries no boundary code.  Thread per BC face node.
template <typename R>
__global__ void __launch_bounds__(256)
k_bc_lift_ghost(R* __restrict__ Pf, const R* __restrict__ Fgeo, Gas<R> gas, Launch L, int n2) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)L.nBCSides * n2) return;
  const int side = (int)(t / n2), pq = (int)(t - (long long)side * n2);
  const R* pm = Pf + (size_t)side * 6 * n2 + pq;
  const R* fg = Fgeo + (size_t)side * 10 * n2 + pq;
  R Pm[6];
#pragma unroll
  for (int c = 0; c < 6; ++c) Pm[c] = pm[c * n2];
  Pm[4] = p_abs(Pm[4], gas);
  const R nv[3] = {fg[0], fg[n2], fg[2 * n2]};
  const R t1[3] = {fg[3 * n2], fg[4 * n2], fg[5 * n2]};
  const R t2[3] = {fg[6 * n2], fg[7 * n2], fg[8 * n2]};
  const int bt = L.bctype[side];
  const R* ref = static_cast<const R*>(L.bcref) + 6 * L.bcstate[side];
  R Pb[6], gh[5];
  bc_state(bt, Pm, ref, nv, t1, t2, gas.kappa, gas.R_gas, Pb);
  bc_lift_ghost(bt, Pm, Pb, gh);
  R* ps = Pf + ((size_t)L.nSides + side) * 6 * n2 + pq;
  const int liftc[5] = {0, 1, 2, 3, 5};
#pragma unroll
  for (int v = 0; v < 5; ++v) ps[liftc[v] * n2] = gh[v];
}

// V0 = 1 skips the density gradient, which no flux of the operator reads (EvalDiffFlux3D uses the
// velocity and temperature gradients only); Gvol/Gf then hold no density entries.
// FP32 (mixed form) blocks of at most 256 threads: four blocks per SM (at most 72 registers); the
// FP32 kernel is latency bound, and at two blocks per SM (107 registers at N=5) only 14 warps hid it
template <int NP, typename R> struct LiftMinBlocks {
  // FP32: four blocks per SM for blocks of at most 256 threads, five for one element of 216 (N = 5)
  static constexpr int v =
      (sizeof(R) == 4 && EPBof<NP>::v * NP * NP * NP <= 256) ? (EPBof<NP>::v == 1 ? 5 : 4) : 2;
};

template <int NP, typename R, int V0 = 0>
__global__ void __launch_bounds__(EPBof<NP>::v * NP * NP * NP, LiftMinBlocks<NP, R>::v)
k_lift(const R* __restrict__ Pvol, const R* __restrict__ Met, const R* __restrict__ Pf, const R* __restrict__ Fgeo,
       const int* __restrict__ E2S, DevBasis<R> basis, Launch L, R* __restrict__ Gvol, R* __restrict__ Gf) {
  constexpr int n = NP, n2 = NP * NP, n3 = NP * NP * NP, EPB = EPBof<NP>::v, N = NP - 1;
  __shared__ SBasis<NP, R> sb;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  R (*Ps)[5][n3] = reinterpret_cast<R (*)[5][n3]>(smem_raw);                                   // [EPB][5][n3]
  R (*Gs)[15][n3] = reinterpret_cast<R (*)[15][n3]>(smem_raw + sizeof(R) * (size_t)EPB * lift_ps_slots(NP)); // [EPB][15][n3]
  load_basis(sb, basis);
  const int e0 = blockIdx.x * EPB;
  const int nloc = min(EPB, L.nElems - e0);
  const int liftc[5] = {0, 1, 2, 3, 5};
  const bool facepass = !L.gauss && !L.br2;
  if constexpr (sizeof(R) == 4 && EPB == 1) {
    // FP32 form: the metric terms and the six faces' traces and geometry, read after the volume part,
    // are pulled into L2 while the block loads and differentiates its primitives
    if (threadIdx.x == 32 && nloc > 0) {
      const R* m = Met + (size_t)e0 * 10 * n3;
      if (bulk_ok(m, m, 10 * n3 * sizeof(R))) bulk_prefetch_l2(m, 10 * n3 * sizeof(R));
    }
    if (threadIdx.x >= 64 && threadIdx.x < 70 && nloc > 0) {
      const size_t side = (size_t)E2S[((size_t)e0 * 6 + threadIdx.x - 64) * 2];
      const R* pm = Pf + side * 6 * n2;
      const R* ps = Pf + ((size_t)L.nSides + side) * 6 * n2;
      const R* fg = Fgeo + side * 10 * n2;
      if (bulk_ok(pm, ps, 6 * n2 * sizeof(R)) && bulk_ok(fg, fg, 10 * n2 * sizeof(R))) {
        bulk_prefetch_l2(pm, 6 * n2 * sizeof(R));
        bulk_prefetch_l2(ps, 6 * n2 * sizeof(R));
        bulk_prefetch_l2(fg, 10 * n2 * sizeof(R));
      }
    }
  }
  const R sigflux = (L.lift_mode == 2) ? R(1) : R(-1);
  for (int t = threadIdx.x; t < nloc * 5 * n3; t += blockDim.x) {
    int el = t / (5 * n3), r = t - el * 5 * n3;
    int c = r / n3, node = r - c * n3;
    Ps[el][c][vsw<NP>(node)] = Pvol[(size_t)(e0 + el) * 7 * n3 + liftc[c] * n3 + node];
  }
  __syncthreads();
  // thread per (element, node): the block has EPB * n^3 threads
  const int el = threadIdx.x / n3, node = threadIdx.x - el * n3;
  const bool act = el < nloc;
  const int e = e0 + el;
  const int i = node % n, j = (node / n) % n, k = node / n2;
  R g[3][5];
  R sj = R(0);
  if (act) {
    const R* M = Met + (size_t)e * 10 * n3 + node;
    sj = M[9 * n3];
    if (L.lift_mode == 0) {
      // Lifting_VolInt_Nonconservative_GPU_Kernel (lifting_volint.t90:262-328), with the Jacobian of
      // the surface integral (surfint.t90:718-723) folded into the metric terms
      R gxi[5], geta[5], gzeta[5];
#pragma unroll
      for (int v = V0; v < 5; ++v) { gxi[v] = R(0); geta[v] = R(0); gzeta[v] = R(0); }
#pragma unroll
      for (int l = 0; l < n; ++l) {
        const R dxi = sb.D[i + n * l], deta = sb.D[j + n * l], dzeta = sb.D[k + n * l];
#pragma unroll
        for (int v = V0; v < 5; ++v) {
          gxi[v] = gxi[v] + dxi * Ps[el][v][vsw<NP>(l + n * (j + n * k))];
          geta[v] = geta[v] + deta * Ps[el][v][vsw<NP>(i + n * (l + n * k))];
          gzeta[v] = gzeta[v] + dzeta * Ps[el][v][vsw<NP>(i + n * (j + n * l))];
        }
      }
      const R mf[3] = {sj * M[0], sj * M[n3], sj * M[2 * n3]}, mg[3] = {sj * M[3 * n3], sj * M[4 * n3], sj * M[5 * n3]},
              mh[3] = {sj * M[6 * n3], sj * M[7 * n3], sj * M[8 * n3]};
#pragma unroll
      for (int d = 0; d < 3; ++d)
#pragma unroll
        for (int v = V0; v < 5; ++v) g[d][v] = mf[d] * gxi[v] + mg[d] * geta[v] + mh[d] * gzeta[v];
    } else {
      // Lifting_VolInt_Conservative (lifting_volint.t90:345-455): D_T (strong) or D_hat_T (weak)
      const R* Dm = (L.lift_mode == 2) ? sb.DhatT : sb.D;  // DhatT(l,i) vs D_T(l,i) = D(i,l)
      const R* Me = Met + (size_t)e * 10 * n3;
#pragma unroll
      for (int d = 0; d < 3; ++d) {
#pragma unroll
        for (int v = V0; v < 5; ++v) g[d][v] = R(0);
        for (int l = 0; l < n; ++l) {
          R ci, cj, ck;
          if (L.lift_mode == 2) { ci = Dm[l + n * i]; cj = Dm[l + n * j]; ck = Dm[l + n * k]; }
          else { ci = Dm[i + n * l]; cj = Dm[j + n * l]; ck = Dm[k + n * l]; }
          const int ni = l + n * (j + n * k), nj = i + n * (l + n * k), nk = i + n * (j + n * l);
          const R wf = ci * Me[(0 + d) * n3 + ni], wh = ck * Me[(6 + d) * n3 + nk], wg = cj * Me[(3 + d) * n3 + nj];
#pragma unroll
          for (int v = V0; v < 5; ++v)
            g[d][v] = g[d][v] + wf * Ps[el][v][vsw<NP>(ni)] + wh * Ps[el][v][vsw<NP>(nk)] + wg * Ps[el][v][vsw<NP>(nj)];
        }
#pragma unroll
        for (int v = V0; v < 5; ++v) g[d][v] = sj * g[d][v];
      }
    }
    if (L.br2 || facepass) {
      // BR2: the face traces prolong the volume part only (ApplyJacobianLifting before
      // ProlongToFaceLifting, lifting_br2.t90:120-147); Gauss-Lobatto BR1: the surface part is added
      // to the shared copy by face-node threads below
#pragma unroll
      for (int d = 0; d < 3; ++d)
#pragma unroll
        for (int v = V0; v < 5; ++v) Gs[el][d * 5 + v][vsw<NP>(node)] = g[d][v];
    }
  }
  if (facepass) {
    __syncthreads();
    // surface part on Gauss-Lobatto nodes, one thread per face node, one normal direction per pass
    // (the two faces of a direction share no node); only face nodes do surface work, so no warp
    // executes the side bodies of nodes that are not on that face
#pragma unroll 1
    for (int dir = 0; dir < 3; ++dir) {
      for (int t = threadIdx.x; t < nloc * 2 * n2; t += blockDim.x) {
        const int el = t / (2 * n2), r = t - el * 2 * n2;
        const bool minus = r < n2;
        const int ab = minus ? r : r - n2;
        const int a = ab % n, b = ab / n;
        const int ls = dir == 0 ? (minus ? L_XI_MINUS : L_XI_PLUS)
                                : (dir == 1 ? (minus ? L_ETA_MINUS : L_ETA_PLUS) : (minus ? L_ZETA_MINUS : L_ZETA_PLUS));
        const int node = face_node(n, ls, a, b, minus ? 0 : N), snode = vsw<NP>(node);
        const int e = e0 + el;
        const R Lhat = minus ? sb.Lhm[0] : sb.Lhp[N];
        const int side = E2S[(e * 6 + ls - 1) * 2 + 0];
        const int flip = E2S[(e * 6 + ls - 1) * 2 + 1];
        int p, q;
        s2v2_inv(N, a, b, flip, ls, p, q);
        const int pq = p + n * q;
        const R* pm = Pf + (size_t)side * 6 * n2 + pq;
        const R* ps = Pf + ((size_t)L.nSides + side) * 6 * n2 + pq;
        const R* fg = Fgeo + (size_t)side * 10 * n2 + pq;
        const R sj = Met[((size_t)e * 10 + 9) * n3 + node];
        const R sig = (L.lift_mode == 2) ? ((flip == 0) ? R(1) : R(-1)) : R(1);
        const R wgt = sig * Lhat * R(0.5) * fg[9 * n2] * sj;
        const R nvv[3] = {wgt * fg[0], wgt * fg[n2], wgt * fg[2 * n2]};
#pragma unroll
        for (int v = V0; v < 5; ++v) {
          const int c = liftc[v];
          const R fl = sigflux * pm[c * n2] + ps[c * n2];
#pragma unroll
          for (int d = 0; d < 3; ++d) Gs[el][d * 5 + v][snode] = Gs[el][d * 5 + v][snode] + fl * nvv[d];
        }
      }
      __syncthreads();
    }
    if (act) {
      R* G = Gvol + (size_t)e * 15 * n3 + node;
#pragma unroll
      for (int c = 0; c < 15; ++c)
        if (c % 5 >= V0) G[c * n3] = Gs[el][c][vsw<NP>(node)];
    }
  } else {
    // surface part (SurfInt_Device_Single_Flux, surfint.t90:591-725) of the BR1 flux
    // 0.5*SurfElem*(sig*U_master + U_slave) (Lifting_FillFlux, lifting_fillflux.t90:39-103) times the
    // normal (Lifting_FillFlux_NormVec, :212-256), times L_hat and the Jacobian.  One normal direction
    // per pass: the threads of the two faces' nodes put the flux vectors F = 0.5*SurfElem*flux*n of
    // their node into shared memory (over the lifted primitives, which are no longer read), then every
    // node adds sJ*(Lhat_minus(l)*F_minus + Lhat_plus(l)*F_plus) of its line (Gauss nodes) or of its
    // face (Gauss-Lobatto nodes, BR2).  Each face node's data is read from global memory once.
    R (*Fs)[2][15][n2] = reinterpret_cast<R (*)[2][15][n2]>(smem_raw);  // [EPB][minus/plus][15][n2]
#pragma unroll 1
    for (int dir = 0; dir < 3; ++dir) {
      __syncthreads();
      for (int t = threadIdx.x; t < nloc * 2 * n2; t += blockDim.x) {
        const int fe = t / (2 * n2), r = t - fe * 2 * n2;
        const int mp = r < n2 ? 0 : 1;
        const int ab = r - mp * n2;
        const int a = ab % n, b = ab / n;
        const int ls = dir == 0 ? (mp == 0 ? L_XI_MINUS : L_XI_PLUS)
                                : (dir == 1 ? (mp == 0 ? L_ETA_MINUS : L_ETA_PLUS) : (mp == 0 ? L_ZETA_MINUS : L_ZETA_PLUS));
        const int ef = e0 + fe;
        const int side = E2S[(ef * 6 + ls - 1) * 2 + 0];
        const int flip = E2S[(ef * 6 + ls - 1) * 2 + 1];
        int p, q;
        s2v2_inv(N, a, b, flip, ls, p, q);
        const int pq = p + n * q;
        const R* pm = Pf + (size_t)side * 6 * n2 + pq;
        const R* ps = Pf + ((size_t)L.nSides + side) * 6 * n2 + pq;
        const R* fg = Fgeo + (size_t)side * 10 * n2 + pq;
        const R sig = (L.lift_mode == 2) ? ((flip == 0) ? R(1) : R(-1)) : R(1);
        const R wgt = sig * R(0.5) * fg[9 * n2];
        const R nvv[3] = {wgt * fg[0], wgt * fg[n2], wgt * fg[2 * n2]};
#pragma unroll
        for (int v = V0; v < 5; ++v) {
          const int c = liftc[v];
          const R fl = sigflux * pm[c * n2] + ps[c * n2];
#pragma unroll
          for (int d = 0; d < 3; ++d) Fs[fe][mp][d * 5 + v][ab] = fl * nvv[d];
        }
      }
      __syncthreads();
      if (act) {
        const int a = dir == 0 ? j : i, b = dir == 2 ? j : k, l = dir == 0 ? i : (dir == 1 ? j : k);
        const int ab = a + n * b;
        if (L.gauss) {
          const R cm = sj * sb.Lhm[l], cp = sj * sb.Lhp[l];
#pragma unroll
          for (int d = 0; d < 3; ++d)
#pragma unroll
            for (int v = V0; v < 5; ++v)
              g[d][v] = g[d][v] + cm * Fs[el][0][d * 5 + v][ab] + cp * Fs[el][1][d * 5 + v][ab];
        } else if (l == 0 || l == N) {
          const int mp = l == 0 ? 0 : 1;
          const R cf = sj * (l == 0 ? sb.Lhm[0] : sb.Lhp[N]);
#pragma unroll
          for (int d = 0; d < 3; ++d)
#pragma unroll
            for (int v = V0; v < 5; ++v) g[d][v] = g[d][v] + cf * Fs[el][mp][d * 5 + v][ab];
        }
      }
    }
    if (act) {
      R* G = Gvol + (size_t)e * 15 * n3 + node;
#pragma unroll
      for (int d = 0; d < 3; ++d)
#pragma unroll
        for (int v = V0; v < 5; ++v) {
          const R val = g[d][v];
          if (!L.br2) Gs[el][d * 5 + v][vsw<NP>(node)] = val;
          G[(d * 5 + v) * n3] = val;
        }
    }
  }
  __syncthreads();
  // ProlongToFaceLifting
  for (int t = threadIdx.x; t < nloc * 6 * n2; t += blockDim.x) {
    int el = t / (6 * n2), r = t - el * 6 * n2;
    int ls = r / n2 + 1, pq = r - (ls - 1) * n2;
    int p = pq % n, q = pq / n;
    int e = e0 + el;
    int side = E2S[(e * 6 + ls - 1) * 2 + 0];
    int flip = E2S[(e * 6 + ls - 1) * 2 + 1];
    int a, b;
    s2v2(N, p, q, flip, ls, a, b);
    const int slot = (flip == 0) ? 0 : 1;
    R* gf = Gf + ((size_t)slot * L.nSides + side) * 15 * n2 + pq;
    // BR2 (Lifting_SurfInt_BR2, lifting_br2.t90:191-310): the trace also gets etaBR2 times the
    // lifting of this face's own strong flux 0.5*SurfElem*(U_slave - U_master)*n, prolonged back:
    // eta * Flux * sum_l L(l) * Lhat(l) * sJ(l) over the line normal to the face (GL: face node only)
    R bw = R(0);
    const R* pm = nullptr;
    const R* ps = nullptr;
    const R* fg = nullptr;
    if (L.br2) {
      const R* Lv = is_minus(ls) ? sb.Lm : sb.Lp;
      const R* Lh = is_minus(ls) ? sb.Lhm : sb.Lhp;
      const R* sJe = Met + ((size_t)e * 10 + 9) * n3;
      const int l0 = L.gauss ? 0 : (is_minus(ls) ? 0 : N), l1 = L.gauss ? N : l0;
      for (int l = l0; l <= l1; ++l) bw = bw + Lv[l] * Lh[l] * sJe[face_node(n, ls, a, b, l)];
      fg = Fgeo + (size_t)side * 10 * n2 + pq;
      bw = R(L.eta_br2) * R(0.5) * fg[9 * n2] * bw;
      pm = Pf + (size_t)side * 6 * n2 + pq;
      ps = Pf + ((size_t)L.nSides + side) * 6 * n2 + pq;
    }
    for (int c = 0; c < 15; ++c) {
      if (c % 5 < V0) continue;
      R s;
      if (!L.gauss) {
        s = Gs[el][c][vsw<NP>(face_node(n, ls, a, b, is_minus(ls) ? 0 : N))];
      } else {
        const R* Lv = is_minus(ls) ? sb.Lm : sb.Lp;
        s = Gs[el][c][vsw<NP>(face_node(n, ls, a, b, 0))] * Lv[0];
#pragma unroll
        for (int l = 1; l < n; ++l) s = s + Gs[el][c][vsw<NP>(face_node(n, ls, a, b, l))] * Lv[l];
      }
      if (L.br2) {
        const int d = c / 5, v = c - 5 * d;
        s = s + bw * (ps[liftc[v] * n2] - pm[liftc[v] * n2]) * fg[d * n2];
      }
      gf[c * n2] = s;
    }
  }
}

// GetBoundaryFlux_GPU (getboundaryflux.f90:542-838) at one face node, without the SurfElem factor:
// PL the inner face state (momentum pressure in slot 4), g* the inner face gradients (clobbered by the
// wall projections), ref the side's reference state.  Templated on the arithmetic type, so that the
// adjoint obtains its local Jacobian by forward-mode dual numbers.
template <typename R>
__device__ __forceinline__ void bc_face_flux(int bt, const R PL[6], R gx[5], R gy[5], R gz[5], const R nv[3],
                                             const R t1[3], const R t2[3], const R* ref, const Gas<R>& gas,
                                             int riemann, int split, int parabolic, R F[5]) {
  R Pm[6], Pb[6];
#pragma unroll
  for (int c = 0; c < 6; ++c) Pm[c] = PL[c];
  Pm[4] = p_abs(PL[4], gas);
  bc_state(bt, Pm, ref, nv, t1, t2, gas.kappa, gas.R_gas, Pb);
  R fd[5];
  if (bc_riemann_type(bt)) {
    // Riemann solver between the inner state and the boundary state (both via PrimToCons)
    R Uc[5], Ub[5], Ps[6];
    prim_to_cons_face(Pm, gas, Uc);
    prim_to_cons_face(Pb, gas, Ub);
#pragma unroll
    for (int c = 0; c < 6; ++c) Ps[c] = Pb[c];
    Ps[4] = OffsetOf<R>::v ? Pb[4] - gas.pref : Pb[4];
    riemann_face(riemann, split, Uc, Ub, PL, Ps, nv, t1, t2, gas, F);
    if (parabolic) {
      normal_diff_flux(PL, gx, gy, gz, nv, gas.mu, gas.lambda, fd);
#pragma unroll
      for (int v = 0; v < 5; ++v) F[v] = F[v] + R(0.5) * fd[v];
      normal_diff_flux(Pb, gx, gy, gz, nv, gas.mu, gas.lambda, fd);
#pragma unroll
      for (int v = 0; v < 5; ++v) F[v] = F[v] + R(0.5) * fd[v];
    }
  } else {
    // walls: pressure flux, plus the viscous flux of the wall state
    const R pw = OffsetOf<R>::v ? Pb[4] - gas.pref : Pb[4];
    F[0] = R(0);
    F[1] = pw * nv[0];
    F[2] = pw * nv[1];
    F[3] = pw * nv[2];
    F[4] = R(0);
    if (parabolic) {
      if (bt == 9 || bt == 91) bc_wall_gradients(bt, nv, t1, t2, gx, gy, gz);
      normal_diff_flux(Pb, gx, gy, gz, nv, gas.mu, gas.lambda, fd);
      if (bt == 3) fd[4] = R(0);
#pragma unroll
      for (int v = 0; v < 5; ++v) F[v] = F[v] + fd[v];
    }
  }
}

// k_bc_face: GetBoundaryFlux_GPU with the SurfElem factor of FillFlux (fillflux.f90:162-170), thread
// per face node of the BC sides (a launch of its own, so that the boundary code does not weigh on the
// registers of k_face)
template <typename R>
__global__ void __launch_bounds__(256)
k_bc_face(const R* __restrict__ Pf, const R* __restrict__ Gf, const R* __restrict__ Fgeo, Gas<R> gas, Launch L,
          int n2, R* __restrict__ Flux) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)L.nBCSides * n2) return;
  const int side = (int)(t / n2), pq = (int)(t - (long long)side * n2);
  const int bt = L.bctype[side];
  const R* ref = static_cast<const R*>(L.bcref) + 6 * L.bcstate[side];
  const R* pf = Pf + (size_t)side * 6 * n2 + pq;
  const R* gm = Gf + (size_t)side * 15 * n2 + pq;
  const R* fg = Fgeo + (size_t)side * 10 * n2 + pq;
  R* out = Flux + (size_t)side * 5 * n2 + pq;
  R PL[6];
#pragma unroll
  for (int c = 0; c < 6; ++c) PL[c] = pf[c * n2];
  const R nv[3] = {fg[0], fg[n2], fg[2 * n2]};
  const R t1[3] = {fg[3 * n2], fg[4 * n2], fg[5 * n2]};
  const R t2[3] = {fg[6 * n2], fg[7 * n2], fg[8 * n2]};
  const R se = fg[9 * n2];
  R gx[5], gy[5], gz[5];
  if (L.parabolic) {
#pragma unroll
    for (int v = 0; v < 5; ++v) { gx[v] = gm[v * n2]; gy[v] = gm[(5 + v) * n2]; gz[v] = gm[(10 + v) * n2]; }
  }
  R F[5];
  bc_face_flux(bt, PL, gx, gy, gz, nv, t1, t2, ref, gas, L.riemann, L.split, L.parabolic, F);
#pragma unroll
  for (int v = 0; v < 5; ++v) out[v * n2] = F[v] * se;
}

// =====================================================================================
// k_face: FillFlux (fillflux.f90:45-172): Riemann + ViscousFlux + SurfElem, thread per face node
// (128-thread blocks, at most 128 registers: four blocks per SM instead of one 256-thread block; the
// FP32 form, which streams its face data, eight at 64 registers)
// =====================================================================================
template <typename R> struct FaceMinBlocks { static constexpr int v = sizeof(R) == 4 ? 8 : 4; };
template <typename R>
__global__ void __launch_bounds__(128, FaceMinBlocks<R>::v)
k_face(const R* __restrict__ Uf, const R* __restrict__ Pf, const R* __restrict__ Gf, const R* __restrict__ Fgeo,
       Gas<R> gas, Launch L, int n2, R* __restrict__ Flux) {
  // connected sides only (nBCSides .. nSides-1); the BC sides are k_bc_face's
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x + (long long)L.nBCSides * n2;
  if (t >= (long long)L.nSides * n2) return;
  const int side = (int)(t / n2), pq = (int)(t - (long long)side * n2);
  const size_t S = L.nSides;
  R UL[5], UR[5], PL[6], PR[6];
#pragma unroll
  for (int v = 0; v < 5; ++v) {
    UL[v] = Uf[(size_t)side * 5 * n2 + v * n2 + pq];
    UR[v] = Uf[(S + side) * 5 * n2 + v * n2 + pq];
  }
#pragma unroll
  for (int c = 0; c < 6; ++c) {
    PL[c] = Pf[(size_t)side * 6 * n2 + c * n2 + pq];
    PR[c] = Pf[(S + side) * 6 * n2 + c * n2 + pq];
  }
  const R* fg = Fgeo + (size_t)side * 10 * n2 + pq;
  const R nv[3] = {fg[0], fg[n2], fg[2 * n2]};
  const R t1[3] = {fg[3 * n2], fg[4 * n2], fg[5 * n2]};
  const R t2[3] = {fg[6 * n2], fg[7 * n2], fg[8 * n2]};
  const R se = fg[9 * n2];
  R F[5];
  riemann_face(L.riemann, L.split, UL, UR, PL, PR, nv, t1, t2, gas, F);
  if (L.parabolic) {
    // ViscousFlux_Kernel_CUDA (riemann.f90:638-700): F = F + 0.5*f(L); F = F + 0.5*f(R)
    R gx[5], gy[5], gz[5], fd[5];
    const R* gm = Gf + (size_t)side * 15 * n2 + pq;
#pragma unroll
    for (int v = 0; v < 5; ++v) { gx[v] = gm[v * n2]; gy[v] = gm[(5 + v) * n2]; gz[v] = gm[(10 + v) * n2]; }
    normal_diff_flux(PL, gx, gy, gz, nv, gas.mu, gas.lambda, fd);
#pragma unroll
    for (int v = 0; v < 5; ++v) F[v] = F[v] + R(0.5) * fd[v];
    const R* gs = Gf + (S + side) * 15 * n2 + pq;
#pragma unroll
    for (int v = 0; v < 5; ++v) { gx[v] = gs[v * n2]; gy[v] = gs[(5 + v) * n2]; gz[v] = gs[(10 + v) * n2]; }
    normal_diff_flux(PR, gx, gy, gz, nv, gas.mu, gas.lambda, fd);
#pragma unroll
    for (int v = 0; v < 5; ++v) F[v] = F[v] + R(0.5) * fd[v];
  }
  R* out = Flux + (size_t)side * 5 * n2 + pq;
#pragma unroll
  for (int v = 0; v < 5; ++v) out[v * n2] = F[v] * se;
}

// =====================================================================================
// k_volume: VolInt (weak: volint.f90:129-188 / split: volint.f90:211-353) + SurfIntCons
// (surfint.t90:352-586) + VAX_GPU(-1) + ApplyJacobian, and in RK mode the fused
// VAXPB_OUT_VAXPB_IN stage update (vector.f90:163-183).
// =====================================================================================
// staging slots per node of k_volume (see there); shared by the kernel and its launch code.  FP32 (mixed
// form) at N <= 7 also stages the metric terms of the split-form phase (9 slots after its node data),
// which FP64 reads through L1 so that two blocks fit an SM
template <int NP, typename R>
__host__ __device__ constexpr bool vol_metrics_staged(int split) { return sizeof(R) == 4 && split >= 0 && NP <= 8; }
template <int NP, typename R>
__host__ __device__ constexpr int vol_stage_slots(int split, int parab) {
  const int base = split < 0 ? 15 : (parab ? 12 : (split == DG_SPLIT_PI ? 6 : 9));
  const int met = vol_metrics_staged<NP, R>(split) ? (split == DG_SPLIT_PI ? 6 : 9) + 9 : 0;
  return base > met ? base : met;
}
// threads per 1D line in the split-form phase of k_volume: FP32 (mixed form) at N = 5..7 splits the
// rows of each line's pair triangle between two threads (with their own accumulators), since the
// FP32 phase is latency bound with one thread per line; FP64 keeps one thread (FP64-issue bound)
template <int NP, typename R>
__host__ __device__ constexpr int vol_line_threads() {
  return (sizeof(R) == 4 && 6 * NP * NP <= NP * NP * NP && NP <= 8) ? 2 : 1;
}
// rows a of the pair triangle (a, b > a; n-1-a pairs) taken by the second thread of a line: r0 <= a < r1,
// chosen to balance the pair counts of the two threads
template <int NP>
struct LineSplit {
  static constexpr int pairs(int r0, int r1) { return r0 >= r1 ? 0 : (NP - 1 - r0) + pairs(r0 + 1, r1); }
  static constexpr int cost(int r0, int r1) {
    return pairs(r0, r1) > NP * (NP - 1) / 2 - pairs(r0, r1) ? pairs(r0, r1) : NP * (NP - 1) / 2 - pairs(r0, r1);
  }
  static constexpr int best(int which) {
    int b0 = 0, b1 = 0, bc = 1 << 30;
    for (int r0 = 0; r0 < NP; ++r0)
      for (int r1 = r0; r1 < NP; ++r1)
        if (cost(r0, r1) < bc) { bc = cost(r0, r1); b0 = r0; b1 = r1; }
    return which == 0 ? b0 : b1;
  }
  static constexpr int r0 = best(0), r1 = best(1);
};

template <typename S>
struct RKArgsT {
  S* U;              // in/out (RK mode)
  S* Ut_tmp;         // in/out (RK mode)
  S* Ut;             // out (RHS mode)
  double mRKA, b_dt;
};
using RKArgs = RKArgsT<double>;

// S: type of the state arrays U, Ut, Ut_tmp (double; Dual<1> for the tangent-linear operator)
template <int NP, typename R, int SPLIT, int PARAB, typename S = double>
__global__ void __launch_bounds__(EPBof<NP>::v * NP * NP * NP)
k_volume(const S* __restrict__ U, const R* __restrict__ Pvol, const R* __restrict__ Gvol,
         const R* __restrict__ Met, const R* __restrict__ Flux, const int* __restrict__ E2S, DevBasis<R> basis,
         Gas<R> gas, Launch L, RKArgsT<S> rk, int rkmode) {
  constexpr int n = NP, n2 = NP * NP, n3 = NP * NP * NP, EPB = EPBof<NP>::v, N = NP - 1;
  // staging slots per node: the flux-form fluxes of phase A (15; split form: the 12 non-zero viscous
  // ones), then the node data of phase B (PI: rho, aux, u, v, w, p; other split forms also m1..m3);
  // the metrics of phase B are read from global memory (L1), so that at N=7 two blocks fit an SM
  constexpr int NA = vol_stage_slots<NP, R>(SPLIT, PARAB);
  constexpr int S_RHO = 0, S_AUX = 1, S_U = 2, S_V = 3, S_W = 4, S_PM = 5, S_M1 = 6, S_M2 = 7, S_M3 = 8;
  constexpr bool MST = vol_metrics_staged<NP, R>(SPLIT);        // metric terms of phase B staged
  constexpr int S_MET = (SPLIT == DG_SPLIT_PI) ? 6 : 9;          // their slots: S_MET + 3*dir + c
  __shared__ SBasis<NP, R> sb;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int NH = vol_line_threads<NP, R>();
  R* A = reinterpret_cast<R*>(smem_raw);             // [EPB][NA][n3]
  R* AccD = A + (size_t)EPB * NA * n3;               // [EPB][NH][3][5][n3]  (split form only)
  load_basis(sb, basis);
  if constexpr (SPLIT == DG_SPLIT_PI) {
    // PI pair fluxes are evaluated as 8F (see phase B): fold the 1/8 into DVolSurf (exact scaling)
    __syncthreads();
    for (int t = threadIdx.x; t < NP * NP; t += blockDim.x) sb.DVS[t] = sb.DVS[t] * R(0.125);
  }
  const int e0 = blockIdx.x * EPB;
  const int nloc = min(EPB, L.nElems - e0);
  const int tid = threadIdx.x;
  const bool active = tid < nloc * n3;
  if constexpr (sizeof(R) == 4 && EPB == 1 && std::is_same<S, double>::value) {
    // FP32 form: the six faces' fluxes and the FP64 state and RK register, read by the surface
    // integral and the stage update at the end, are pulled into L2 while the volume part runs
    if (tid == 32 && nloc > 0 && rkmode) {
      const double* u = rk.U + (size_t)e0 * 5 * n3;
      const double* r = rk.Ut_tmp + (size_t)e0 * 5 * n3;
      if (bulk_ok(u, r, 5 * n3 * 8)) {
        bulk_prefetch_l2(u, 5 * n3 * 8);
        bulk_prefetch_l2(r, 5 * n3 * 8);
      }
    }
    if (tid >= 64 && tid < 70 && nloc > 0) {
      const R* fx = Flux + (size_t)E2S[((size_t)e0 * 6 + tid - 64) * 2] * 5 * n2;
      if (bulk_ok(fx, fx, 5 * n2 * sizeof(R))) bulk_prefetch_l2(fx, 5 * n2 * sizeof(R));
    }
  }
  const int el = tid / n3, node = tid - (tid / n3) * n3;
  const int e = e0 + el;
  const int i = node % n, j = (node / n) % n, k = node / n2;
  const int snode = vsw<NP>(node);  // shared-memory position of this node
  R* Ae = A + (size_t)el * NA * n3;
  R vacc[5] = {0, 0, 0, 0, 0};  // this node's volume integral, kept in registers through phase B

  // ---- phase A: flux-form volume part (weak Euler/NS, or the viscous part of the split form)
  if (SPLIT < 0 || PARAB) {
    if (active) {
      const R* M = Met + (size_t)e * 10 * n3 + node;
      const R* P = Pvol + (size_t)e * 7 * n3 + node;
      const R Ms[3][3] = {{M[0], M[n3], M[2 * n3]}, {M[3 * n3], M[4 * n3], M[5 * n3]}, {M[6 * n3], M[7 * n3], M[8 * n3]}};
      const R vel[3] = {P[n3], P[2 * n3], P[3 * n3]};
      R fl[3][5];
      R tau[6] = {0, 0, 0, 0, 0, 0}, tq[3] = {0, 0, 0};
      if (PARAB) {
        const R* G = Gvol + (size_t)e * 15 * n3 + node;
        R gx[5], gy[5], gz[5];
#pragma unroll
        for (int v = 0; v < 5; ++v) { gx[v] = G[v * n3]; gy[v] = G[(5 + v) * n3]; gz[v] = G[(10 + v) * n3]; }
        visc_stress(gx, gy, gz, vel, gas.mu, gas.lambda, tau, tq);
      }
      if (SPLIT < 0) {
        // EvalTransformedEulerFlux3D_fast (flux.f90:137-186) / EvalTransformedEulerDiffFlux3D (:509-614)
        const S* Un = U + ((size_t)e * n3 + node) * 5;
        const R m1 = narrow<R>(Un[1]), m2 = narrow<R>(Un[2]), m3 = narrow<R>(Un[3]), E = narrow<R>(Un[4]);
        const R p = P[4 * n3], srho = P[6 * n3];  // p: momentum pressure (p' in the mixed form)
        const R Ep = (E + p_abs(p, gas)) * srho;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          const R Mmom = Ms[d][0] * m1 + Ms[d][1] * m2 + Ms[d][2] * m3;
          fl[d][0] = Mmom;
          fl[d][1] = Mmom * vel[0] + Ms[d][0] * p;
          fl[d][2] = Mmom * vel[1] + Ms[d][1] * p;
          fl[d][3] = Mmom * vel[2] + Ms[d][2] * p;
          fl[d][4] = Mmom * Ep;
          if (PARAB) {
            fl[d][1] = fl[d][1] - Ms[d][0] * tau[0] - Ms[d][1] * tau[3] - Ms[d][2] * tau[4];
            fl[d][2] = fl[d][2] - Ms[d][0] * tau[3] - Ms[d][1] * tau[1] - Ms[d][2] * tau[5];
            fl[d][3] = fl[d][3] - Ms[d][0] * tau[4] - Ms[d][1] * tau[5] - Ms[d][2] * tau[2];
            fl[d][4] = fl[d][4] - Ms[d][0] * tq[0] - Ms[d][1] * tq[1] - Ms[d][2] * tq[2];
          }
        }
      } else {
        // EvalTransformedDiffFlux3D (flux.f90:619-697)
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          fl[d][0] = R(0);
          fl[d][1] = -Ms[d][0] * tau[0] - Ms[d][1] * tau[3] - Ms[d][2] * tau[4];
          fl[d][2] = -Ms[d][0] * tau[3] - Ms[d][1] * tau[1] - Ms[d][2] * tau[5];
          fl[d][3] = -Ms[d][0] * tau[4] - Ms[d][1] * tau[5] - Ms[d][2] * tau[2];
          fl[d][4] = -Ms[d][0] * tq[0] - Ms[d][1] * tq[1] - Ms[d][2] * tq[2];
        }
      }
      // slot of flux (d, v): d*5+v, or d*4+v-1 for the split form's viscous fluxes (no density row)
      constexpr int v0 = (SPLIT < 0) ? 0 : 1, nvs = 5 - v0;
#pragma unroll
      for (int d = 0; d < 3; ++d)
#pragma unroll
        for (int v = v0; v < 5; ++v) Ae[(d * nvs + v - v0) * n3 + snode] = fl[d][v];
    }
    __syncthreads();
    if (active) {
      // ApplyDMatrix_Kernel (applydmatrix.t90:19-75), order f, h, g
      constexpr int v0 = (SPLIT < 0) ? 0 : 1, nvs = 5 - v0;
#pragma unroll
      for (int l = 0; l < n; ++l) {
        const R ci = sb.DhatT[l + n * i], ck = sb.DhatT[l + n * k], cj = sb.DhatT[l + n * j];
        const int ni = vsw<NP>(l + n * (j + n * k)), nk = vsw<NP>(i + n * (j + n * l)),
                  nj = vsw<NP>(i + n * (l + n * k));
#pragma unroll
        for (int v = v0; v < 5; ++v)
          vacc[v] = vacc[v] + ci * Ae[(0 * nvs + v - v0) * n3 + ni] + ck * Ae[(2 * nvs + v - v0) * n3 + nk] +
                    cj * Ae[(1 * nvs + v - v0) * n3 + nj];
      }
    }
  }

  // ---- phase B: split-form flux differencing with pair symmetry, one thread per 1D line.
  // Node a keeps its sum in registers over its pairs (a,b>a); node b's share goes to the line
  // owner's per-direction shared accumulator, so no two threads ever write the same entry.
  if constexpr (SPLIT >= 0) {
    __syncthreads();  // phase A reads of the staging area are complete
    if (active) {
      const S* Un = U + ((size_t)e * n3 + node) * 5;
      const R* P = Pvol + (size_t)e * 7 * n3 + node;
      const R E = narrow<R>(Un[4]);
      const R rho = P[0], uu = P[n3], vv = P[2 * n3], ww = P[3 * n3], pm = P[4 * n3];
      Ae[S_RHO * n3 + snode] = rho;
      Ae[S_AUX * n3 + snode] = pair_aux<SPLIT, R>(rho, uu, vv, ww, E, p_abs(pm, gas), P[6 * n3]);
      Ae[S_U * n3 + snode] = uu;
      Ae[S_V * n3 + snode] = vv;
      Ae[S_W * n3 + snode] = ww;
      Ae[S_PM * n3 + snode] = (SPLIT == DG_SPLIT_PI) ? R(4) * pm : pm;  // PI: 4p (exact scaling)
      if constexpr (SPLIT != DG_SPLIT_PI) {
        Ae[S_M1 * n3 + snode] = narrow<R>(Un[1]);
        Ae[S_M2 * n3 + snode] = narrow<R>(Un[2]);
        Ae[S_M3 * n3 + snode] = narrow<R>(Un[3]);
      }
      if constexpr (MST) {
        const R* Mn = Met + (size_t)e * 10 * n3 + node;
#pragma unroll
        for (int c = 0; c < 9; ++c) Ae[(S_MET + c) * n3 + snode] = Mn[c * n3];
      }
      R* Ad = AccD + (size_t)el * NH * 15 * n3;
#pragma unroll
      for (int c = 0; c < NH * 15; ++c) Ad[c * n3 + snode] = R(0);
    }
    __syncthreads();
    const int lel = tid / (NH * 3 * n2);
    const bool lactive = (lel < nloc) && (tid < EPB * NH * 3 * n2);  // 3*n2 <= n3 for NP >= 3; 6*n2 <= n3 if NH = 2
    if (lactive) {
      const int lh = tid - lel * NH * 3 * n2;
      const int half = lh / (3 * n2), lr = lh - half * 3 * n2;
      const int dir = lr / n2, li = lr - dir * n2;
      const R* Al = A + (size_t)lel * NA * n3;
      R* Ad = AccD + (((size_t)lel * NH + half) * 3 + dir) * 5 * n3;
      int base, stride;  // nodes of the line: base + l*stride
      if (dir == 0) { base = n * li; stride = 1; }
      else if (dir == 1) { base = (li % n) + n2 * (li / n); stride = n; }
      else { base = li; stride = n2; }
      // this direction's metric terms: staged (indexed by shared-memory position) or through L1
      const R* Ml = MST ? Al + (S_MET + 3 * dir) * n3 : Met + ((size_t)(e0 + lel) * 10 + 3 * dir) * n3;
#pragma unroll 1
      for (int a = 0; a < NP - 1; ++a) {
        if constexpr (NH == 2) {
          if ((a >= LineSplit<NP>::r0 && a < LineSplit<NP>::r1) != (half == 1)) continue;
        }
        const int na = base + a * stride, sna = vsw<NP>(na);
        PairNode<R> A_;
        A_.rho = Al[S_RHO * n3 + sna]; A_.aux = Al[S_AUX * n3 + sna];
        A_.u = Al[S_U * n3 + sna]; A_.v = Al[S_V * n3 + sna]; A_.w = Al[S_W * n3 + sna]; A_.pm = Al[S_PM * n3 + sna];
        if constexpr (SPLIT != DG_SPLIT_PI) {
          A_.m1 = Al[S_M1 * n3 + sna]; A_.m2 = Al[S_M2 * n3 + sna]; A_.m3 = Al[S_M3 * n3 + sna];
        } else {
          A_.m1 = A_.m2 = A_.m3 = R(0);
        }
        const int ma = MST ? sna : na;
        const R ma0 = Ml[ma], ma1 = Ml[n3 + ma], ma2 = Ml[2 * n3 + ma];
        R sa[5];
#pragma unroll
        for (int v = 0; v < 5; ++v) sa[v] = Ad[v * n3 + sna];
#pragma unroll 4
        for (int b = a + 1; b < NP; ++b) {
          const int nb = base + b * stride, snb = vsw<NP>(nb);
          PairNode<R> B_;
          B_.rho = Al[S_RHO * n3 + snb]; B_.aux = Al[S_AUX * n3 + snb];
          B_.u = Al[S_U * n3 + snb]; B_.v = Al[S_V * n3 + snb]; B_.w = Al[S_W * n3 + snb]; B_.pm = Al[S_PM * n3 + snb];
          if constexpr (SPLIT != DG_SPLIT_PI) {
            B_.m1 = Al[S_M1 * n3 + snb]; B_.m2 = Al[S_M2 * n3 + snb]; B_.m3 = Al[S_M3 * n3 + snb];
          } else {
            B_.m1 = B_.m2 = B_.m3 = R(0);
          }
          const int mb = MST ? snb : nb;
          const R Ms0 = ma0 + Ml[mb], Ms1 = ma1 + Ml[n3 + mb], Ms2 = ma2 + Ml[2 * n3 + mb];
          R F[5];
          if constexpr (SPLIT == DG_SPLIT_PI) {
            // 8 x the PI flux of split_pair_flux, with the density row at 4 x (its accumulators are
            // doubled at the end); every factor is a power of two, so the rounding is unchanged
            const R rs = A_.rho + B_.rho, us = A_.u + B_.u, vs = A_.v + B_.v, ws = A_.w + B_.w;
            const R ps4 = A_.pm + B_.pm;
            const R Vs = Ms0 * us + Ms1 * vs + Ms2 * ws;
            const R q8 = rs * Vs;
            F[0] = q8;
            F[1] = q8 * us + ps4 * Ms0;
            F[2] = q8 * vs + ps4 * Ms1;
            F[3] = q8 * ws + ps4 * Ms2;
            F[4] = q8 * (A_.aux + B_.aux);
          } else {
            split_pair_flux<SPLIT, R>(A_, B_, Ms0, Ms1, Ms2, R(2) * gas.pref, F);
          }
          const R dba = sb.DVS[b + n * a], dab = sb.DVS[a + n * b];  // DVolSurf(l=b,i=a), DVolSurf(l=a,i=b)
#pragma unroll
          for (int v = 0; v < 5; ++v) {
            sa[v] = sa[v] + dba * F[v];
            Ad[v * n3 + snb] += dab * F[v];
          }
        }
#pragma unroll
        for (int v = 0; v < 5; ++v) Ad[v * n3 + sna] = sa[v];
      }
    }
    __syncthreads();
    if (active) {
      const R* Ad = AccD + (size_t)el * NH * 15 * n3;
#pragma unroll
      for (int v = 0; v < 5; ++v) {
        R sv = Ad[v * n3 + snode] + Ad[(5 + v) * n3 + snode] + Ad[(10 + v) * n3 + snode];
        if constexpr (NH == 2) sv = sv + (Ad[(15 + v) * n3 + snode] + Ad[(20 + v) * n3 + snode] + Ad[(25 + v) * n3 + snode]);
        if (SPLIT == DG_SPLIT_PI && v == 0) sv = sv * R(2);
        vacc[v] = vacc[v] + sv;
      }
    }
  }

  // ---- phase C: surface integral, -1, Jacobian, output / RK stage
  R ut[5];
#pragma unroll
  for (int v = 0; v < 5; ++v) ut[v] = R(0);
  if (!L.gauss) {
    // Gauss-Lobatto: only face nodes receive surface terms; add them by face-node threads, one
    // normal direction per pass (the two faces of a direction share no node), into the staging area
    __syncthreads();  // every read of the staging area is complete
    for (int t = threadIdx.x; t < nloc * 5 * n3; t += blockDim.x) {
      const int el2 = t / (5 * n3), r = t - el2 * 5 * n3;
      A[(size_t)el2 * NA * n3 + r] = R(0);
    }
    __syncthreads();
#pragma unroll 1
    for (int dir = 0; dir < 3; ++dir) {
      for (int t = threadIdx.x; t < nloc * 2 * n2; t += blockDim.x) {
        const int el2 = t / (2 * n2), r = t - el2 * 2 * n2;
        const bool minus = r < n2;
        const int ab = minus ? r : r - n2;
        const int a = ab % n, b = ab / n;
        const int ls = dir == 0 ? (minus ? L_XI_MINUS : L_XI_PLUS)
                                : (dir == 1 ? (minus ? L_ETA_MINUS : L_ETA_PLUS) : (minus ? L_ZETA_MINUS : L_ZETA_PLUS));
        const int fnode = face_node(n, ls, a, b, minus ? 0 : N);
        const int e2 = e0 + el2;
        const R Lhat = minus ? sb.Lhm[0] : sb.Lhp[N];
        const int side = E2S[(e2 * 6 + ls - 1) * 2 + 0];
        const int flip = E2S[(e2 * 6 + ls - 1) * 2 + 1];
        int p, q;
        s2v2_inv(N, a, b, flip, ls, p, q);
        const R* fx = Flux + (size_t)side * 5 * n2 + p + n * q;
        R* Su = A + (size_t)el2 * NA * n3 + vsw<NP>(fnode);
        if (flip == 0) {
#pragma unroll
          for (int v = 0; v < 5; ++v) Su[v * n3] = Su[v * n3] + fx[v * n2] * Lhat;
        } else {
#pragma unroll
          for (int v = 0; v < 5; ++v) Su[v * n3] = Su[v * n3] - fx[v * n2] * Lhat;
        }
      }
      __syncthreads();
    }
    if (!active) return;
#pragma unroll
    for (int v = 0; v < 5; ++v) ut[v] = Ae[v * n3 + snode];
  }
  if constexpr (SPLIT < 0) {
    static_assert(30 * n2 <= NA * n3, "face fluxes of six faces fit the staging area");
    if (L.gauss) {
      // Gauss nodes: every node of a line gets L_hat(l) times the flux of the line's two faces.  The
      // fluxes of the element block's six faces (slave sides negated) are put into the staging area
      // once, 30 n^2 <= 15 n^3 slots per element, and the nodes read them from there.
      __syncthreads();  // every read of the staging area is complete
      for (int t = threadIdx.x; t < nloc * 6 * n2; t += blockDim.x) {
        const int el2 = t / (6 * n2), r = t - el2 * 6 * n2;
        const int ls = r / n2 + 1, ab = r - (ls - 1) * n2;
        const int a = ab % n, b = ab / n;
        const int e2 = e0 + el2;
        const int side = E2S[(e2 * 6 + ls - 1) * 2 + 0];
        const int flip = E2S[(e2 * 6 + ls - 1) * 2 + 1];
        int p, q;
        s2v2_inv(N, a, b, flip, ls, p, q);
        const R* fx = Flux + (size_t)side * 5 * n2 + p + n * q;
        R* Fv = A + (size_t)el2 * NA * n3 + (ls - 1) * 5 * n2 + ab;
        if (flip == 0) {
#pragma unroll
          for (int v = 0; v < 5; ++v) Fv[v * n2] = fx[v * n2];
        } else {
#pragma unroll
          for (int v = 0; v < 5; ++v) Fv[v * n2] = -fx[v * n2];
        }
      }
      __syncthreads();
      if (!active) return;
#pragma unroll
      for (int ls = 1; ls <= 6; ++ls) {
        int a, b, l;
        switch (ls) {
          case L_XI_MINUS: case L_XI_PLUS: a = j; b = k; l = i; break;
          case L_ETA_MINUS: case L_ETA_PLUS: a = i; b = k; l = j; break;
          default: a = i; b = j; l = k; break;
        }
        const R Lhat = is_minus(ls) ? sb.Lhm[l] : sb.Lhp[l];
        const R* Fv = Ae + (ls - 1) * 5 * n2 + a + n * b;
#pragma unroll
        for (int v = 0; v < 5; ++v) ut[v] = ut[v] + Fv[v * n2] * Lhat;
      }
    }
  }
  if (!active) return;
  const R sj = Met[(size_t)e * 10 * n3 + 9 * n3 + node];
  const size_t g = ((size_t)e * n3 + node) * 5;
#pragma unroll
  for (int v = 0; v < 5; ++v) {
    R val = vacc[v] + ut[v];
    val = val * R(-1);
    val = val * sj;
    if (rkmode == 0) {
      rk.Ut[g + v] = widen<S>(val);
    } else {
      const S utmp = rk.Ut_tmp[g + v] * rk.mRKA + widen<S>(val);
      rk.Ut_tmp[g + v] = utmp;
      rk.U[g + v] = rk.U[g + v] + utmp * rk.b_dt;
    }
  }
}

// =====================================================================================
// CFL: CalcMaxEigenvalue (calctimestep.f90:192-296) + min reduction (FP64 throughout)
// =====================================================================================
__device__ __forceinline__ void atomic_min_pos(double* addr, double val) {
  // positive doubles order like their bit patterns
  unsigned long long* a = reinterpret_cast<unsigned long long*>(addr);
  unsigned long long v = (unsigned long long)__double_as_longlong(val);
  atomicMin(a, v);
}

// one block per element, blockDim = n^3 rounded up to a warp multiple
template <int NP>
__global__ void __launch_bounds__(1024)
k_cfl(const double* __restrict__ U, const double* __restrict__ MetD, const double* __restrict__ Cm, int nElems,
      double kappa, double mu0, int parabolic, double CFLScale, double DFLScale, double* __restrict__ dt2,
      unsigned long long* __restrict__ bad) {
  constexpr int n3 = NP * NP * NP;
  constexpr int NW = (n3 + 31) / 32;
  __shared__ double red[6][NW];
  const int e = blockIdx.x;
  const int node = threadIdx.x;
  double lam[6] = {0, 0, 0, 0, 0, 0};
  if (node < n3) {
    const double* u = U + ((size_t)e * n3 + node) * 5;
    const double srho = 1. / u[0];
    const double vel[3] = {u[1] * srho, u[2] * srho, u[3] * srho};
    const double p = (kappa - 1.) * (u[4] - 0.5 * (vel[0] * u[1] + vel[1] * u[2] + vel[2] * u[3]));
    if (!(u[0] > 0.) || !(p > 0.) || !isfinite(u[4]) || !isfinite(u[1] + u[2] + u[3])) atomicAdd(bad, 1ULL);
    const double c = sqrt(kappa * p * srho);
    const double* M = MetD + (size_t)e * 10 * n3 + node;
    const double* C = Cm + (size_t)e * 6 * n3 + node;  // MetricsAdv(1:3), MetricsVisc(1:3)
    const double sj = M[9 * n3];
    const double vs[3] = {vel[0] * sj, vel[1] * sj, vel[2] * sj};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const double m0 = M[(3 * d) * n3], m1 = M[(3 * d + 1) * n3], m2 = M[(3 * d + 2) * n3];
      lam[d] = fabs(m0 * vs[0] + m1 * vs[1] + m2 * vs[2]) + c * C[d * n3];
      if (parabolic) lam[3 + d] = mu0 * srho * C[(3 + d) * n3];
    }
  }
  // max over the element's nodes: warp shuffle, then across the element's warps
#pragma unroll
  for (int d = 0; d < 6; ++d) {
    double v = lam[d];
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    if ((threadIdx.x & 31) == 0) red[d][threadIdx.x >> 5] = v;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double mx[6];
    for (int d = 0; d < 6; ++d) {
      mx[d] = red[d][0];
      for (int w = 1; w < NW; ++w) mx[d] = fmax(mx[d], red[d][w]);
    }
    atomic_min_pos(dt2, CFLScale * 2. / (mx[0] + mx[1] + mx[2]));
    if (parabolic) atomic_min_pos(dt2 + 1, DFLScale * 4. / (mx[3] + mx[4] + mx[5]));
  }
}

// state scan: NaN/Inf, non-positive density or pressure
static __global__ void k_check(const double* __restrict__ U, long long nNodes, double kappa, unsigned long long* __restrict__ bad) {
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < nNodes; t += (long long)gridDim.x * blockDim.x) {
    const double* u = U + t * 5;
    const double p = (kappa - 1.) * (u[4] - 0.5 * (u[1] * u[1] + u[2] * u[2] + u[3] * u[3]) / u[0]);
    if (!(u[0] > 0.) || !(p > 0.) || !isfinite(u[1] + u[2] + u[3] + u[4])) atomicAdd(bad, 1ULL);
  }
}

}  // namespace gx

#include "dg_lines.cuh"
