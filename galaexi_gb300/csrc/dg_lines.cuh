// Kernels of the mixed (FP32) form on Gauss-Lobatto nodes: two with one thread per 1D line of an
// element, and a prolongation with one thread per node.
//
// k_volume_lines: the volume kernel of the split form.  VolInt_splitForm (src/dg/volint.f90:211-353,
// SplitVolumeFlux* of splitflux.f90:145-730) sums, for every node i of a line, DVolSurf(l,i) *
// F#(U_i, U_l; (M_i + M_l)/2) over the line's nodes l; the viscous part (VolInt_weakForm_Visc,
// volint.f90:238-240, with EvalTransformedDiffFlux3D, flux.f90:619-697) adds D_hat^T(l,i) * f_visc(l)
// along the same lines.  In the element-per-block kernel (k_volume) the line's nodes sit in shared
// memory and every pair costs ~20 shared-memory accesses (the partner's node data and the
// read-modify-write of its accumulators), which bounds the FP32 kernel.  Here a thread holds its whole
// line in registers: the node data (rho, u, v, w, the momentum pressure, the form's auxiliary variable
// and the line direction's metric terms) and the five accumulators of every node.  All n(n-1)/2 pairs
// run fully unrolled for the compile-time n, each pair flux evaluated once and added to both nodes;
// then the line direction's contravariant viscous fluxes of its nodes (from the lifted gradients) are
// contracted with D_hat^T.  DVolSurf and D_hat^T are compile-time indexed kernel parameters
// (constant-bank operands of the FMAs).  The three directions' sums of a node meet in shared memory
// (padded so that neither the line-ordered writes nor the node-ordered reads conflict at N = 7), and
// the block's threads then finish node by node: the Gauss-Lobatto surface integral of the face fluxes
// (SurfIntCons, surfint.t90:352-586), -1 and the Jacobian; last, one value per thread in turn, the
// output or the LSERK-W2 stage update (vector.f90:163-183) in FP64.
// The kernel is persistent (a block walks the elements b, b + gridDim.x, ...) and double-buffered: the
// slabs of the block's next element (primitives, metric terms, lifted gradients, each contiguous in
// memory, and the element's row of E2S) are copied into shared memory by the tensor memory
// accelerator (cp.async.bulk, dg_tma.cuh) while the block computes the current one, and its FP64 state
// and RK register are pulled into L2 (cp.async.bulk.prefetch), so that the few warps of a block (two
// blocks of 168 registers per SM at n = 8) seldom wait for memory.  Where a slab is not 16-byte aligned
// (odd n) the threads copy it.
//
// k_prolong_gl: ConsToPrim and the face traces, persistent and double-buffered the same way.
//
// k_lift_lines: the BR1 lifting (Lifting_BR1, lifting_br1.t90:47-167, strong non-conservative form,
// Gauss-Lobatto nodes).  The line threads differentiate u, v, w and T along their line (D(i,l) as
// kernel parameters); the node-by-node finish applies the metric terms and the Jacobian
// (Lifting_VolInt_Nonconservative, lifting_volint.t90:262-328), adds the surface part of the faces the
// node lies on (0.5 SurfElem (P_slave - P_master) n L_hat sJ, lifting_fillflux.t90:39-103, 212-256,
// surfint.t90:591-725) and writes the gradients and their face traces (ProlongToFaceLifting: on
// Gauss-Lobatto nodes the node's own value).  The density gradient, which no flux reads, is not formed.
// A block is one element; the metric terms and face data of its finish are pulled into L2 while its
// lines differentiate.
//
// Registers: ~9 n + 5 n values per thread, so the line kernels are instantiated for n <= 8, the volume
// kernel for the forms whose pair flux needs no momenta (SD, KG, PI).
#pragma once
#include "dg_physics.cuh"
#include "dg_tma.cuh"

namespace gx {

// 1D operators of the volume line kernel: DVolSurf(l,i) at dvs[l + NP*i] (pre-scaled by 1/8 for PI,
// see below), D_hat^T(l,i) at dht[l + NP*i], and the Gauss-Lobatto surface weights L_hat_minus(0),
// L_hat_plus(N)
template <int NP> struct LineBasis {
  float dvs[NP * NP];
  float dht[NP * NP];
  float lhm0, lhpN;
};
// 1D operators of the lifting line kernel: D(i,l) at D[i + NP*l]
template <int NP> struct LiftBasis {
  float D[NP * NP];
  float lhm0, lhpN;
};

template <int NP> __host__ __device__ constexpr int line_pad(int dir) {
  // row strides of the three directions' result regions: with n = 8 these make the bank of
  // (row l, line) distinct for the 32 lines a warp writes and for the 32 nodes a warp reads
  return NP * NP + (dir == 0 ? 4 : (dir == 1 ? 8 : 0));
}
template <int NP> __host__ __device__ constexpr int line_red_words(int vars) {
  return vars * NP * (line_pad<NP>(0) + line_pad<NP>(1) + line_pad<NP>(2));
}
template <int SPLIT> struct LinesForm {
  static constexpr bool v = SPLIT == DG_SPLIT_PI || SPLIT == DG_SPLIT_KG || SPLIT == DG_SPLIT_SD;
};
template <int NP, typename R, int SPLIT> struct UseLines {
  static constexpr bool v = sizeof(R) == 4 && NP >= 4 && NP <= 8 && LinesForm<SPLIT>::v;
};
template <int NP, typename R> struct UseLiftLines {
  static constexpr bool v = sizeof(R) == 4 && NP >= 4 && NP <= 8;
};

__host__ __device__ constexpr size_t round16(size_t b) { return (b + 15) / 16 * 16; }

// shared-memory layout of k_volume_lines, one buffer (bytes): region A holds the lifted gradients
// (12 slots: u, v, w, T in x, y, z; the density gradient is not read) and the primitives rho, u, v,
// w, p, 1/rho (6 slots), later the three directions' sums; then the metric terms and sJ (10 slots)
// and the element's row of E2S.  A slot is n^3 floats in the node order of the state.  The kernel holds two buffers; at n = 8 they
// take 112 KB, so that two blocks share an SM.
template <int NP> struct VolLinesSmem {
  static constexpr int SS = NP * NP * NP;  // slot stride (words)
  static constexpr size_t A = round16(18 * SS * 4 > line_red_words<NP>(5) * 4 ? 18 * SS * 4 : line_red_words<NP>(5) * 4);
  static constexpr size_t G = 0, P = 12 * SS * 4, M = A;
  static constexpr size_t E = M + round16(10 * SS * 4);
  static constexpr size_t buffer = E + 64;
  static constexpr size_t bytes = 2 * buffer;
};

// copy `bytes` from src to dst in shared memory: one bulk copy issued by thread 0 where `bulk`
// (source, destination and size 16-byte aligned), else the block's threads copy words
__device__ __forceinline__ void stage_bytes(void* dst, const void* src, unsigned bytes, bool bulk, uint64_t* bar) {
  if (bulk) {
    if (threadIdx.x == 0) bulk_g2s(dst, src, bytes, bar);
  } else {
    const unsigned* s = static_cast<const unsigned*>(src);
    unsigned* d = static_cast<unsigned*>(dst);
    for (unsigned t = threadIdx.x; t < bytes / 4; t += blockDim.x) d[t] = s[t];
  }
}

// C consecutive nodes l0 .. l0+C-1 of a line of one slot: word base + l * step; on the xi lines
// (step 1) of n = 4, 8 four nodes are one aligned float4
template <int NP, int C>
__device__ __forceinline__ void line_chunk(const float* s, int dir, int base, int step, int l0, float (&x)[C]) {
  if constexpr (C == 4 && NP % 4 == 0) {
    if (dir == 0) {
      const float4 t = *reinterpret_cast<const float4*>(s + base + l0);
      x[0] = t.x; x[1] = t.y; x[2] = t.z; x[3] = t.w;
      return;
    }
  }
#pragma unroll
  for (int c = 0; c < C; ++c) x[c] = s[base + (l0 + c) * step];
}
template <int NP>
__device__ __forceinline__ void line_load(const float* s, int dir, int base, int step, float (&x)[NP]) {
  constexpr int C = NP % 4 == 0 ? 4 : 1;
#pragma unroll
  for (int l0 = 0; l0 < NP; l0 += C) {
    float t[C];
    line_chunk<NP, C>(s, dir, base, step, l0, t);
#pragma unroll
    for (int c = 0; c < C; ++c) x[l0 + c] = t[c];
  }
}

// the faces a node (i,j,k) lies on, in normal-direction order: local side and face coordinates
template <int NP>
__device__ __forceinline__ bool node_face(int f, int i, int j, int k, int& ls, int& a, int& b) {
  constexpr int N = NP - 1;
  switch (f) {
    case 0: ls = L_XI_MINUS; a = j; b = k; return i == 0;
    case 1: ls = L_XI_PLUS; a = j; b = k; return i == N;
    case 2: ls = L_ETA_MINUS; a = i; b = k; return j == 0;
    case 3: ls = L_ETA_PLUS; a = i; b = k; return j == N;
    case 4: ls = L_ZETA_MINUS; a = i; b = j; return k == 0;
    default: ls = L_ZETA_PLUS; a = i; b = j; return k == N;
  }
}

// Persistent: block b computes elements b, b + gridDim.x, ...  The slabs of the block's next element
// are copied into one of two shared-memory buffers while it computes the current one from the other.
template <int NP, int SPLIT, int PARAB>
__global__ void __launch_bounds__(3 * NP * NP, 2)
k_volume_lines(const float* __restrict__ Pvol, const float* __restrict__ Gvol, const float* __restrict__ Met,
               const float* __restrict__ Flux, const int* __restrict__ E2S, LineBasis<NP> lb, Gas<float> gas,
               int nElems, double* __restrict__ Ut, double* __restrict__ Uio, double* __restrict__ Ut_tmp, double mRKA,
               double b_dt, int rkmode, int* __restrict__ err) {
  constexpr int n = NP, n2 = NP * NP, n3 = NP * NP * NP, N = NP - 1;
  constexpr int P0 = line_pad<NP>(0), P1 = line_pad<NP>(1), P2 = line_pad<NP>(2);
  constexpr int OFF1 = 5 * n * P0, OFF2 = OFF1 + 5 * n * P1;
  constexpr int SS = n3;
  constexpr int C = NP % 4 == 0 ? 4 : 1;  // nodes per chunk of the viscous phase
  using L = VolLinesSmem<NP>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ uint64_t bar[2];
  const int tid = threadIdx.x;
  if ((int)blockIdx.x >= nElems) return;
  // bulk copies where the element's slabs start 16-byte aligned (n^3 a multiple of 4); else the
  // threads copy
  const bool bulk = (n3 % 4 == 0) && bulk_ok(Pvol, Met, 16) && bulk_ok(Gvol, Gvol, 16);
  const bool ebulk = bulk_ok(E2S, E2S, 16);  // a row of E2S is 48 bytes
  // the RK register and state of the next element, and the face fluxes of the current one, are
  // pulled into L2 ahead of the node-by-node finish that reads them
  const bool upre = rkmode && (n3 % 2 == 0) && bulk_ok(Uio, Ut_tmp, 16);
  const bool fpre = (n2 % 4 == 0) && bulk_ok(Flux, Flux, 16);
  const unsigned txb = (bulk ? (unsigned)((6 + 10 + (PARAB ? 12 : 0)) * n3 * 4) : 0u) + (ebulk ? 48u : 0u);
  if (tid == 0) { mbar_init(&bar[0]); mbar_init(&bar[1]); }
  __syncthreads();
  // queue the slabs of element e into buffer b; the barrier is armed with the byte count first
  auto issue = [&](int e, int b) {
    unsigned char* B = smem_raw + (size_t)b * L::buffer;
    if (tid == 0) mbar_arrive_expect(&bar[b], txb);
    const float* Pg = Pvol + (size_t)e * 7 * n3;
    stage_bytes(B + L::P, Pg, 5 * n3 * 4, bulk, &bar[b]);                  // rho, u, v, w, p
    stage_bytes(B + L::P + 5 * n3 * 4, Pg + 6 * n3, n3 * 4, bulk, &bar[b]);  // 1/rho
    stage_bytes(B + L::M, Met + (size_t)e * 10 * n3, 10 * n3 * 4, bulk, &bar[b]);
    stage_bytes(B + L::E, E2S + (size_t)e * 12, 48, ebulk, &bar[b]);
    if (upre && tid == 32) {
      bulk_prefetch_l2(Uio + (size_t)e * 5 * n3, 5 * n3 * 8);
      bulk_prefetch_l2(Ut_tmp + (size_t)e * 5 * n3, 5 * n3 * 8);
    }
    if (PARAB) {
      const float* Gg = Gvol + (size_t)e * 15 * n3;
#pragma unroll
      for (int d = 0; d < 3; ++d)  // the gradients of u, v, w, T in x, y, z
        stage_bytes(B + L::G + 4 * d * n3 * 4, Gg + (5 * d + 1) * n3, 4 * n3 * 4, bulk, &bar[b]);
    }
  };
  issue(blockIdx.x, 0);
  int k = 0;
  for (int e = blockIdx.x; e < nElems; e += gridDim.x, ++k) {
    const int cb = k & 1;
    const int en = e + gridDim.x;
    if (en < nElems) issue(en, cb ^ 1);  // the other buffer was released at the end of the last element
    __syncthreads();                     // the threads' own copies
    if (__syncthreads_or(!mbar_wait(&bar[cb], (k >> 1) & 1, err))) {
      // the copies did not complete in time: wait (bounded) for those into the other buffer, and leave
      if (en < nElems) mbar_wait(&bar[cb ^ 1], ((k + 1) >> 1) & 1, nullptr);
      return;
    }
    unsigned char* B = smem_raw + (size_t)cb * L::buffer;
    float* const red = reinterpret_cast<float*>(B);  // the directions' sums, after the line phase
    const float* const Gs = reinterpret_cast<const float*>(B + L::G);
    const float* const Ps = reinterpret_cast<const float*>(B + L::P);
    const float* const Ms = reinterpret_cast<const float*>(B + L::M);
    const int* const es = reinterpret_cast<const int*>(B + L::E);  // E2S row: side, flip of the six local sides
    if (fpre && tid >= 64 && tid < 70) bulk_prefetch_l2(Flux + (size_t)es[(tid - 64) * 2] * 5 * n2, 5 * n2 * 4);
    const int dir = tid / n2, li = tid - dir * n2;
    int base, step;
    if (dir == 0) { base = n * li; step = 1; }
    else if (dir == 1) { base = (li % n) + n2 * (li / n); step = n; }
    else { base = li; step = n2; }
    const float* M = Ms + 3 * dir * SS;
    float acc[n][5];
    float m0[n], m1[n], m2[n], u[n], v[n], w[n];
    line_load<NP>(Ps + SS, dir, base, step, u);
    line_load<NP>(Ps + 2 * SS, dir, base, step, v);
    line_load<NP>(Ps + 3 * SS, dir, base, step, w);
    line_load<NP>(M, dir, base, step, m0);
    line_load<NP>(M + SS, dir, base, step, m1);
    line_load<NP>(M + 2 * SS, dir, base, step, m2);
    {
      // the line's node data
      float rho[n], pm[n], aux[n];
      line_load<NP>(Ps, dir, base, step, rho);
      line_load<NP>(Ps + 4 * SS, dir, base, step, pm);  // momentum pressure (p' = p - p_ref in the mixed form)
      line_load<NP>(Ps + 5 * SS, dir, base, step, aux);  // 1/rho, replaced by the form's auxiliary variable
#pragma unroll
      for (int l = 0; l < n; ++l) {
        const float pmom = pm[l];
        const float pabs = p_abs(pmom, gas);
        const float E = pabs * gas.sKappaM1 + 0.5f * rho[l] * (u[l] * u[l] + v[l] * v[l] + w[l] * w[l]);
        aux[l] = pair_aux<SPLIT, float>(rho[l], u[l], v[l], w[l], E, pabs, aux[l]);
        pm[l] = (SPLIT == DG_SPLIT_PI) ? 4.f * pmom : pmom;  // PI: 4p (exact scaling, see below)
      }
#pragma unroll
      for (int l = 0; l < n; ++l)
#pragma unroll
        for (int c = 0; c < 5; ++c) acc[l][c] = 0.f;
      // split form: every pair of the line once, added to both of its nodes
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
            PairNode<float> A, Bn;
            A.rho = rho[a]; A.u = u[a]; A.v = v[a]; A.w = w[a]; A.pm = pm[a]; A.aux = aux[a];
            Bn.rho = rho[b]; Bn.u = u[b]; Bn.v = v[b]; Bn.w = w[b]; Bn.pm = pm[b]; Bn.aux = aux[b];
            A.m1 = A.m2 = A.m3 = Bn.m1 = Bn.m2 = Bn.m3 = 0.f;
            split_pair_flux<SPLIT, float>(A, Bn, Ms0, Ms1, Ms2, 2.f * gas.pref, F);
          }
          const float dba = lb.dvs[b + n * a], dab = lb.dvs[a + n * b];  // DVolSurf(l=b,i=a), DVolSurf(l=a,i=b)
#pragma unroll
          for (int c = 0; c < 5; ++c) {
            acc[a][c] = acc[a][c] + dba * F[c];
            acc[b][c] = acc[b][c] + dab * F[c];
          }
        }
      }
      if constexpr (SPLIT == DG_SPLIT_PI) {
#pragma unroll
        for (int l = 0; l < n; ++l) acc[l][0] = 2.f * acc[l][0];
      }
    }
    if constexpr (PARAB) {
      // viscous part: the line direction's contravariant viscous flux of each node (EvalTransformedDiffFlux3D
      // with the direction's metric terms), added to every node of the line with D_hat^T
#pragma unroll
      for (int l0 = 0; l0 < n; l0 += C) {
        float g[12][C];  // d(u, v, w, T)/dx, then /dy, /dz of the chunk's nodes
#pragma unroll
        for (int s = 0; s < 12; ++s) line_chunk<NP, C>(Gs + s * SS, dir, base, step, l0, g[s]);
#pragma unroll
        for (int c = 0; c < C; ++c) {
          const int l = l0 + c;
          float gx[5], gy[5], gz[5];
          gx[0] = gy[0] = gz[0] = 0.f;  // no flux reads the density gradient
#pragma unroll
          for (int q = 1; q < 5; ++q) { gx[q] = g[q - 1][c]; gy[q] = g[3 + q][c]; gz[q] = g[7 + q][c]; }
          const float vel[3] = {u[l], v[l], w[l]};
          float tau[6], tq[3];
          visc_stress(gx, gy, gz, vel, gas.mu, gas.lambda, tau, tq);
          float fv[4];
          fv[0] = -m0[l] * tau[0] - m1[l] * tau[3] - m2[l] * tau[4];
          fv[1] = -m0[l] * tau[3] - m1[l] * tau[1] - m2[l] * tau[5];
          fv[2] = -m0[l] * tau[4] - m1[l] * tau[5] - m2[l] * tau[2];
          fv[3] = -m0[l] * tq[0] - m1[l] * tq[1] - m2[l] * tq[2];
#pragma unroll
          for (int i = 0; i < n; ++i) {
            const float d = lb.dht[l + n * i];
#pragma unroll
            for (int q = 1; q < 5; ++q) acc[i][q] = acc[i][q] + d * fv[q - 1];
          }
        }
      }
    }
    __syncthreads();  // every read of the gradients and primitives, which the sums overwrite
    // the three directions' sums of every node meet in shared memory
    float* R0 = red + (dir == 0 ? 0 : (dir == 1 ? OFF1 : OFF2));
    const int Pd = dir == 0 ? P0 : (dir == 1 ? P1 : P2);
#pragma unroll
    for (int l = 0; l < n; ++l)
#pragma unroll
      for (int c = 0; c < 5; ++c) R0[(c * n + l) * Pd + li] = acc[l][c];
    // face fluxes of the node-by-node finish (pulled into L2 at the start of the element), loaded
    // before the barrier, all at once: Gauss-Lobatto surface integral of the faces a node lies on
    constexpr int NPT = (n3 + 3 * n2 - 1) / (3 * n2);  // nodes per thread
    float ut[NPT][5];
#pragma unroll
    for (int it = 0; it < NPT; ++it) {
      const int node = tid + it * 3 * n2;
#pragma unroll
      for (int c = 0; c < 5; ++c) ut[it][c] = 0.f;
      if (node < n3) {
        const int i = node % n, j = (node / n) % n, kk = node / n2;
#pragma unroll
        for (int f = 0; f < 6; ++f) {
          int ls, a, b;
          if (!node_face<NP>(f, i, j, kk, ls, a, b)) continue;
          const int side = es[(ls - 1) * 2 + 0], flip = es[(ls - 1) * 2 + 1];
          int p, q;
          s2v2_inv(N, a, b, flip, ls, p, q);
          const float* fx = Flux + (size_t)side * 5 * n2 + p + n * q;
          const float Lhat = is_minus(ls) ? lb.lhm0 : lb.lhpN;
          if (flip == 0) {
#pragma unroll
            for (int c = 0; c < 5; ++c) ut[it][c] = ut[it][c] + fx[c * n2] * Lhat;
          } else {
#pragma unroll
            for (int c = 0; c < 5; ++c) ut[it][c] = ut[it][c] - fx[c * n2] * Lhat;
          }
        }
      }
    }
    __syncthreads();
    // node by node: volume sum + surface integral, -1, Jacobian -> Ut in FP32, node-major [n3][5], in
    // the metric slots 0-4 (read only by the line phase)
    float* const Xs = reinterpret_cast<float*>(B + L::M);
#pragma unroll
    for (int it = 0; it < NPT; ++it) {
      const int node = tid + it * 3 * n2;
      if (node < n3) {
        const int i = node % n, j = (node / n) % n, kk = node / n2;
        const float sj = Ms[9 * SS + node];
#pragma unroll
        for (int c = 0; c < 5; ++c) {
          const float vs = red[(c * n + i) * P0 + j + n * kk] + red[OFF1 + (c * n + j) * P1 + i + n * kk] +
                           red[OFF2 + (c * n + kk) * P2 + i + n * j];
          float x = vs + ut[it][c];
          x = x * -1.f;
          Xs[node * 5 + c] = x * sj;
        }
      }
    }
    __syncthreads();
    // output / LSERK-W2 stage in FP64 (vector.f90:163-183; the widening of Ut on the integer pipes, which
    // leaves the FP64 pipe to the two FMAs of the stage), one value per thread in turn: the element's
    // (5, n^3) record is contiguous, so the loads and stores coalesce; the loads of a thread's values
    // are issued together (the state and RK register were pulled into L2 one element ahead)
    {
      constexpr int NV = 5 * n3, T3 = 3 * n2, NIT = (NV + T3 - 1) / T3;
      const size_t g0 = (size_t)e * NV;
      if (rkmode == 0) {
#pragma unroll
        for (int it = 0; it < NIT; ++it) {
          const int t = tid + it * T3;
          if (t < NV) Ut[g0 + t] = f32_to_f64(Xs[t]);
        }
      } else {
        constexpr int BATCH = 7;
#pragma unroll
        for (int i0 = 0; i0 < NIT; i0 += BATCH) {
          double tr[BATCH], ur[BATCH];
#pragma unroll
          for (int q = 0; q < BATCH; ++q) {
            const int t = tid + (i0 + q) * T3;
            if (i0 + q < NIT && t < NV) { tr[q] = Ut_tmp[g0 + t]; ur[q] = Uio[g0 + t]; }
          }
#pragma unroll
          for (int q = 0; q < BATCH; ++q) {
            const int t = tid + (i0 + q) * T3;
            if (i0 + q < NIT && t < NV) {
              const double utmp = tr[q] * mRKA + f32_to_f64(Xs[t]);
              Ut_tmp[g0 + t] = utmp;
              Uio[g0 + t] = ur[q] + utmp * b_dt;
            }
          }
        }
      }
    }
    // this buffer is refilled by the bulk copies of the element after next: order this element's
    // shared-memory accesses before them
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
  }
}

// k_prolong_gl: ConsToPrim of the volume and the face traces (ProlongToFace on Gauss-Lobatto nodes:
// the node's own values; prolongtoface.t90:116-344, GetPrimitiveStateSurface) of the mixed form, as
// k_prolong computes them (cons_to_prim_mixed; the same bits).  Persistent: a block walks the elements
// b, b + gridDim.x, ...; each element's FP64 state (one contiguous (5, n^3) record) and its row of E2S
// are copied into one of two shared-memory buffers by a bulk copy while the block converts the
// previous element, so that the block does not wait for its loads.  n^3 threads, one per node; even
// n (the record is then a multiple of 16 bytes).
template <int NP, typename R, typename S> struct UseProlongGL {
  static constexpr bool v = sizeof(R) == 4 && std::is_same<S, double>::value && NP % 2 == 0 && NP >= 6 && NP <= 8;
};
template <int NP> struct ProlongGLSmem {
  static constexpr size_t ubytes = (size_t)5 * NP * NP * NP * 8;
  static constexpr size_t buffer = round16(ubytes) + 64;  // the state, then the E2S row
  static constexpr size_t bytes = 2 * buffer;
};

template <int NP>
__global__ void __launch_bounds__(NP * NP * NP, 3)
k_prolong_gl(const double* __restrict__ U, const int* __restrict__ E2S, Gas<float> gas, int nElems, int nSides,
             float* __restrict__ Pvol, float* __restrict__ Uf, float* __restrict__ Pf, int* __restrict__ err) {
  constexpr int n = NP, n2 = NP * NP, n3 = NP * NP * NP, N = NP - 1;
  using L = ProlongGLSmem<NP>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ uint64_t bar[2];
  const int tid = threadIdx.x;
  if ((int)blockIdx.x >= nElems) return;
  const bool bulk = bulk_ok(U, E2S, 16);
  if (tid == 0) { mbar_init(&bar[0]); mbar_init(&bar[1]); }
  __syncthreads();
  auto issue = [&](int e, int b) {
    unsigned char* B = smem_raw + (size_t)b * L::buffer;
    if (tid == 0) mbar_arrive_expect(&bar[b], bulk ? (unsigned)(L::ubytes + 48) : 0u);
    stage_bytes(B, U + (size_t)e * 5 * n3, (unsigned)L::ubytes, bulk, &bar[b]);
    stage_bytes(B + round16(L::ubytes), E2S + (size_t)e * 12, 48, bulk, &bar[b]);
  };
  issue(blockIdx.x, 0);
  int k = 0;
  for (int e = blockIdx.x; e < nElems; e += gridDim.x, ++k) {
    const int cb = k & 1;
    const int en = e + gridDim.x;
    if (en < nElems) issue(en, cb ^ 1);  // the other buffer was released at the end of the last element
    __syncthreads();                     // the threads' own copies
    if (__syncthreads_or(!mbar_wait(&bar[cb], (k >> 1) & 1, err))) {
      if (en < nElems) mbar_wait(&bar[cb ^ 1], ((k + 1) >> 1) & 1, nullptr);
      return;
    }
    const double* Us = reinterpret_cast<const double*>(smem_raw + (size_t)cb * L::buffer);  // [n3][5]
    const int* es = reinterpret_cast<const int*>(smem_raw + (size_t)cb * L::buffer + round16(L::ubytes));
    const int node = tid;
    const float c[4] = {f64_to_f32_rn(Us[node * 5]), f64_to_f32_rn(Us[node * 5 + 1]), f64_to_f32_rn(Us[node * 5 + 2]),
                        f64_to_f32_rn(Us[node * 5 + 3])};
    const double E = Us[node * 5 + 4];
    float prim[6], srho;
    cons_to_prim_mixed(c, E, gas, prim, srho);
    const float uo[5] = {c[0], c[1], c[2], c[3], f64_to_f32_rn(E)};
    float* P = Pvol + (size_t)e * 7 * n3 + node;
#pragma unroll
    for (int q = 0; q < 6; ++q) P[q * n3] = prim[q];
    P[6 * n3] = srho;
    // the traces of the faces the node lies on
    const int i = node % n, j = (node / n) % n, kk = node / n2;
#pragma unroll
    for (int f = 0; f < 6; ++f) {
      int ls, a, b;
      if (!node_face<NP>(f, i, j, kk, ls, a, b)) continue;
      const int side = es[(ls - 1) * 2 + 0], flip = es[(ls - 1) * 2 + 1];
      int p, q;
      s2v2_inv(N, a, b, flip, ls, p, q);
      const int slot = (flip == 0) ? 0 : 1;
      float* uf = Uf + ((size_t)slot * nSides + side) * 5 * n2 + p + n * q;
      float* pf = Pf + ((size_t)slot * nSides + side) * 6 * n2 + p + n * q;
#pragma unroll
      for (int v = 0; v < 5; ++v) uf[v * n2] = uo[v];
#pragma unroll
      for (int v = 0; v < 6; ++v) pf[v * n2] = prim[v];
    }
    // this buffer is refilled by the bulk copy of the element after next
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
  }
}

template <int NP>
__global__ void __launch_bounds__(3 * NP * NP, 6)
k_lift_lines(const float* __restrict__ Pvol, const float* __restrict__ Met, const float* __restrict__ Pf,
             const float* __restrict__ Fgeo, const int* __restrict__ E2S, LiftBasis<NP> lb, int nElems, int nSides,
             float* __restrict__ Gvol, float* __restrict__ Gf) {
  constexpr int n = NP, n2 = NP * NP, n3 = NP * NP * NP, N = NP - 1;
  constexpr int P0 = line_pad<NP>(0), P1 = line_pad<NP>(1), P2 = line_pad<NP>(2);
  constexpr int OFF1 = 4 * n * P0, OFF2 = OFF1 + 4 * n * P1;
  __shared__ float red[line_red_words<NP>(4)];
  __shared__ int es[12];  // E2S row: side, flip of the six local sides
  const int e = blockIdx.x;
  if (e >= nElems) return;
  const int tid = threadIdx.x;
  // the node-by-node part reads the element's metric terms and, on its faces, both face traces and the
  // face geometry: they are pulled into L2 while the lines differentiate
  if (tid < 12) es[tid] = E2S[(size_t)e * 12 + tid];
  if (tid == 32) {
    const float* m = Met + (size_t)e * 10 * n3;
    if (bulk_ok(m, m, 10 * n3 * 4)) bulk_prefetch_l2(m, 10 * n3 * 4);
  }
  if (tid >= 64 && tid < 70) {
    // the rows the finish reads: u, v, w (rows 1-3) and T (row 5) of both traces, the normal (rows
    // 0-2) and SurfElem (row 9) of the geometry
    const size_t side = (size_t)E2S[(size_t)e * 12 + (tid - 64) * 2];
    const float* pm = Pf + side * 6 * n2;
    const float* ps = Pf + ((size_t)nSides + side) * 6 * n2;
    const float* fg = Fgeo + side * 10 * n2;
    if (bulk_ok(pm, ps, n2 * 4) && bulk_ok(fg, fg, n2 * 4)) {
      bulk_prefetch_l2(pm + n2, 3 * n2 * 4);
      bulk_prefetch_l2(pm + 5 * n2, n2 * 4);
      bulk_prefetch_l2(ps + n2, 3 * n2 * 4);
      bulk_prefetch_l2(ps + 5 * n2, n2 * 4);
      bulk_prefetch_l2(fg, 3 * n2 * 4);
      bulk_prefetch_l2(fg + 9 * n2, n2 * 4);
    }
  }
  {
    const int dir = tid / n2, li = tid - dir * n2;
    int base, stride;
    if (dir == 0) { base = n * li; stride = 1; }
    else if (dir == 1) { base = (li % n) + n2 * (li / n); stride = n; }
    else { base = li; stride = n2; }
    const float* P = Pvol + (size_t)e * 7 * n3;
    const int slot[4] = {1, 2, 3, 5};  // u, v, w, T
    float x[4][n];
#pragma unroll
    for (int l = 0; l < n; ++l)
#pragma unroll
      for (int c = 0; c < 4; ++c) x[c][l] = P[slot[c] * n3 + base + l * stride];
    float* R0 = red + (dir == 0 ? 0 : (dir == 1 ? OFF1 : OFF2));
    const int Pd = dir == 0 ? P0 : (dir == 1 ? P1 : P2);
#pragma unroll
    for (int i = 0; i < n; ++i)
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        float s = 0.f;
#pragma unroll
        for (int l = 0; l < n; ++l) s = s + lb.D[i + n * l] * x[c][l];
        R0[(c * n + i) * Pd + li] = s;
      }
  }
  __syncthreads();
  const int* e2s = es;
  const int liftc[4] = {1, 2, 3, 5};
  for (int node = tid; node < n3; node += blockDim.x) {
    const int i = node % n, j = (node / n) % n, k = node / n2;
    const float* M = Met + (size_t)e * 10 * n3 + node;
    const float sj = M[9 * n3];
    const float mf[3] = {sj * M[0], sj * M[n3], sj * M[2 * n3]}, mg[3] = {sj * M[3 * n3], sj * M[4 * n3], sj * M[5 * n3]},
                mh[3] = {sj * M[6 * n3], sj * M[7 * n3], sj * M[8 * n3]};
    float g[3][4];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const float gxi = red[(c * n + i) * P0 + j + n * k];
      const float geta = red[OFF1 + (c * n + j) * P1 + i + n * k];
      const float gzeta = red[OFF2 + (c * n + k) * P2 + i + n * j];
#pragma unroll
      for (int d = 0; d < 3; ++d) g[d][c] = mf[d] * gxi + mg[d] * geta + mh[d] * gzeta;
    }
    // surface part of the faces the node lies on, one normal direction after the other
#pragma unroll
    for (int f = 0; f < 6; ++f) {
      int ls, a, b;
      if (!node_face<NP>(f, i, j, k, ls, a, b)) continue;
      const int side = e2s[(ls - 1) * 2 + 0], flip = e2s[(ls - 1) * 2 + 1];
      int p, q;
      s2v2_inv(N, a, b, flip, ls, p, q);
      const int pq = p + n * q;
      const float* pm = Pf + (size_t)side * 6 * n2 + pq;
      const float* ps = Pf + ((size_t)nSides + side) * 6 * n2 + pq;
      const float* fg = Fgeo + (size_t)side * 10 * n2 + pq;
      const float Lhat = is_minus(ls) ? lb.lhm0 : lb.lhpN;
      const float wgt = Lhat * 0.5f * fg[9 * n2] * sj;
      const float nvv[3] = {wgt * fg[0], wgt * fg[n2], wgt * fg[2 * n2]};
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const float fl = -pm[liftc[c] * n2] + ps[liftc[c] * n2];
#pragma unroll
        for (int d = 0; d < 3; ++d) g[d][c] = g[d][c] + fl * nvv[d];
      }
    }
    float* G = Gvol + (size_t)e * 15 * n3 + node;
#pragma unroll
    for (int d = 0; d < 3; ++d)
#pragma unroll
      for (int c = 0; c < 4; ++c) G[(d * 5 + 1 + c) * n3] = g[d][c];
    // face traces: on Gauss-Lobatto nodes the node's own gradient
#pragma unroll
    for (int f = 0; f < 6; ++f) {
      int ls, a, b;
      if (!node_face<NP>(f, i, j, k, ls, a, b)) continue;
      const int side = e2s[(ls - 1) * 2 + 0], flip = e2s[(ls - 1) * 2 + 1];
      int p, q;
      s2v2_inv(N, a, b, flip, ls, p, q);
      float* gf = Gf + (((size_t)(flip == 0 ? 0 : 1) * nSides + side) * 15) * n2 + p + n * q;
#pragma unroll
      for (int d = 0; d < 3; ++d)
#pragma unroll
        for (int c = 0; c < 4; ++c) gf[(d * 5 + 1 + c) * n2] = g[d][c];
    }
  }
}

}  // namespace gx
