// C ABI of the GB300 DGSEM operator: context, mesh upload, RHS, LSERK stepping, CFL time step.
// The entry points replace the reference's module-global operator (see include/galaexi_gb300.h).
#include <cuda_runtime.h>
#include <cstdio>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/galaexi_gb300.h"
#include "dg_host.h"
#include "dg_ctx.h"
#include "dg_tma.cuh"

using gxh::set_error;

namespace {

// Carpenter-Kennedy RK4-5 (timedisc_vars.f90:213-227), stage s = 1..5
const double kRKA[6] = {0., 0., 567301805773.0 / 1357537059087.0, 2404267990393.0 / 2016746695238.0,
                        3550918686646.0 / 2091501179385.0, 1275806237668.0 / 842570457699.0};
const double kRKb[6] = {0., 1432997174477.0 / 9575080441755.0, 5161836677717.0 / 13612068292357.0,
                        1720146321549.0 / 2090206949498.0, 3134564353537.0 / 4481467310338.0,
                        2277821191437.0 / 14882151754819.0};
// CFL / DFL scaling of FillCFL_DFL (timedisc_func.f90:480-550) for Carpenter RK4-5
// (CFLScaleAlpha timedisc_vars.f90:193-206, DFLScaleAlpha timedisc_vars.f90:104-108, RelativeDFL 1.853)
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

const gxc::NPTable* table_for(int n) {
  switch (n) {
    case 2: return &gx_np_table_2;
    case 3: return &gx_np_table_3;
    case 4: return &gx_np_table_4;
    case 5: return &gx_np_table_5;
    case 6: return &gx_np_table_6;
    case 7: return &gx_np_table_7;
    case 8: return &gx_np_table_8;
    case 9: return &gx_np_table_9;
    case 10: return &gx_np_table_10;
  }
  return nullptr;
}

#define CUDA_TRY(call, what)                                                                  \
  do {                                                                                        \
    cudaError_t _e = (call);                                                                  \
    if (_e != cudaSuccess) {                                                                  \
      set_error(std::string(what) + ": " + cudaGetErrorString(_e));                          \
      return DG_ERR_CUDA;                                                                     \
    }                                                                                         \
  } while (0)

template <typename R>
int upload_basis(dg_ctx* ctx, gxc::PrecData<R>& P) {
  const int n = ctx->n;
  std::vector<R> h(3 * n * n + 4 * n);
  for (int t = 0; t < n * n; ++t) {
    h[t] = (R)ctx->B.D[t];
    h[n * n + t] = (R)ctx->B.DhatT[t];
    h[2 * n * n + t] = (R)ctx->B.DVS[t];
  }
  for (int t = 0; t < n; ++t) {
    h[3 * n * n + t] = (R)ctx->B.Lm[t];
    h[3 * n * n + n + t] = (R)ctx->B.Lp[t];
    h[3 * n * n + 2 * n + t] = (R)ctx->B.Lhm[t];
    h[3 * n * n + 3 * n + t] = (R)ctx->B.Lhp[t];
  }
  if (!P.basis.alloc(h.size())) { set_error("cudaMalloc basis"); return DG_ERR_ALLOC; }
  CUDA_TRY(cudaMemcpy(P.basis.p, h.data(), h.size() * sizeof(R), cudaMemcpyHostToDevice), "upload basis");
  return DG_OK;
}

int run_rhs(dg_ctx* ctx, const double* U, gx::RKArgs rk, int rkmode, cudaStream_t st) {
  const gxc::NPTable* T = table_for(ctx->n);
  if (!T) { set_error("unsupported N"); return DG_ERR_UNSUPPORTED; }
  const int rc = ctx->cfg.precision == DG_PRECISION_FP64 ? T->rhs_d(ctx, U, rk, rkmode, st)
                                                         : T->rhs_f(ctx, U, rk, rkmode, st);
  ctx->grad_ok = rc == DG_OK && ctx->cfg.parabolic;
  return rc;
}

// Gvol [e][d*5+v][node] (d = x,y,z; v = rho,u,v,w,T) -> GradUx/y/z(v, node, e) in FP64
template <typename R>
__global__ void __launch_bounds__(256) k_export_grad(const R* __restrict__ G, long long nNodes, int n3,
                                                     double* __restrict__ gx_, double* __restrict__ gy_,
                                                     double* __restrict__ gz_) {
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < nNodes;
       idx += (long long)gridDim.x * blockDim.x) {
    const long long e = idx / n3, node = idx - e * n3;
    const R* g = G + e * 15 * n3 + node;
    double* out[3] = {gx_, gy_, gz_};
#pragma unroll
    for (int d = 0; d < 3; ++d)
#pragma unroll
      for (int v = 0; v < 5; ++v) out[d][idx * 5 + v] = (double)g[(d * 5 + v) * n3];
  }
}

template <typename R>
int alloc_prec(dg_ctx* ctx, gxc::PrecData<R>& P, const std::vector<double>& met, const std::vector<double>& fgeo) {
  const size_t nE = ctx->nElems, nS = ctx->nSides, n2 = ctx->n2, n3 = ctx->n3;
  const bool par = ctx->cfg.parabolic != 0;
  bool ok = P.Met.alloc(nE * 10 * n3) && P.Fgeo.alloc(nS * 10 * n2) && P.Pvol.alloc(nE * 7 * n3) &&
            P.Uf.alloc(2 * nS * 5 * n2) && P.Pf.alloc(2 * nS * 6 * n2) && P.Flux.alloc(nS * 5 * n2);
  if (ok && par) ok = P.Gvol.alloc(nE * 15 * n3) && P.Gf.alloc(2 * nS * 15 * n2);
  if (!ok) { set_error("cudaMalloc scratch"); return DG_ERR_ALLOC; }
  std::vector<R> hm(met.size()), hg(fgeo.size());
  for (size_t t = 0; t < met.size(); ++t) hm[t] = (R)met[t];
  for (size_t t = 0; t < fgeo.size(); ++t) hg[t] = (R)fgeo[t];
  CUDA_TRY(cudaMemcpy(P.Met.p, hm.data(), hm.size() * sizeof(R), cudaMemcpyHostToDevice), "upload metrics");
  CUDA_TRY(cudaMemcpy(P.Fgeo.p, hg.data(), hg.size() * sizeof(R), cudaMemcpyHostToDevice), "upload face geometry");
  return DG_OK;
}

int check_ctx(dg_ctx* ctx, bool need_mesh) {
  if (!ctx) { set_error("null context"); return DG_ERR_ARG; }
  if (need_mesh && !ctx->mesh_ok) { set_error("dg_set_mesh has not been called"); return DG_ERR_ARG; }
  if (need_mesh && !ctx->bc_ok) { set_error("the mesh has BC sides: call dg_set_boundaries first"); return DG_ERR_ARG; }
  return DG_OK;
}

// FMA-chain microkernel: 8 independent dependency chains per thread
template <typename T>
__global__ void __launch_bounds__(256) k_fma_peak(T* out, int iters, T a, T b) {
  T x[8];
#pragma unroll
  for (int c = 0; c < 8; ++c) x[c] = (T)(threadIdx.x + c) * (T)1e-7;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int c = 0; c < 8; ++c) x[c] = fma(x[c], a, b);
  }
  T s = 0;
#pragma unroll
  for (int c = 0; c < 8; ++c) s += x[c];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// A bulk-copy wait that runs out: the barrier is armed for 16 bytes that no copy delivers (none is
// issued) and every thread of the block waits with `limit` polls, then the block returns.  Records
// the wait's duration (%globaltimer, ns) of thread 0.
__global__ void k_selftest_bulk_wait(long long limit, int* err, long long* ns) {
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) gx::mbar_init(&bar);
  __syncthreads();
  if (threadIdx.x == 0) gx::mbar_arrive_expect(&bar, 16);
  long long t0, t1;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0)::"memory");
  gx::mbar_wait(&bar, 0, err, limit);
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t1)::"memory");
  if (threadIdx.x == 0) *ns = t1 - t0;
}

template <typename T>
int fma_peak(double* gflops) {
  int dev = 0, nsm = 0;
  CUDA_TRY(cudaGetDevice(&dev), "cudaGetDevice");
  CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev), "SM count");
  const int threads = 256, blocks = nsm * 16;
  const int iters = sizeof(T) == 8 ? 4096 : 65536;
  T* out = nullptr;
  CUDA_TRY(cudaMalloc(&out, sizeof(T) * threads * blocks), "cudaMalloc");
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  for (int rep = 0; rep < 4; ++rep) {
    cudaEventRecord(e0);
    k_fma_peak<T><<<blocks, threads>>>(out, iters, (T)0.999999, (T)1e-7);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0 && ms < best) best = ms;
  }
  cudaError_t err = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (err != cudaSuccess) { set_error(std::string("fma peak: ") + cudaGetErrorString(err)); return DG_ERR_CUDA; }
  *gflops = 2.0 * 8.0 * (double)iters * threads * blocks / (best * 1e-3) * 1e-9;
  return DG_OK;
}

}  // namespace

// ---------------------------------------------------------------------------------------------
// tangent-linear and adjoint helpers
// ---------------------------------------------------------------------------------------------
namespace {

using D1 = gx::Dual<1>;

__global__ void k_to_dual(const double* __restrict__ in, D1* __restrict__ out, size_t cnt) {
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < cnt; t += (size_t)gridDim.x * blockDim.x)
    out[t] = D1(in[t]);
}
__global__ void k_pack(const double* __restrict__ v, const double* __restrict__ d, D1* __restrict__ out, size_t cnt) {
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < cnt; t += (size_t)gridDim.x * blockDim.x) {
    D1 x(v[t]);
    x.d[0] = d ? d[t] : 0.;
    out[t] = x;
  }
}
__global__ void k_unpack(const D1* __restrict__ in, double* __restrict__ v, double* __restrict__ d, size_t cnt) {
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < cnt; t += (size_t)gridDim.x * blockDim.x) {
    if (v) v[t] = in[t].v;
    if (d) d[t] = in[t].d[0];
  }
}
int grid_for(size_t cnt) {
  size_t g = (cnt + 255) / 256;
  return (int)(g > 152 * 32 ? 152 * 32 : (g < 1 ? 1 : g));
}

// volume integrals over the state: rho, m1, m2, m3, E, kinetic energy 0.5 |m|^2 / rho
// (quadrature on the solution nodes: w_i w_j w_k / sJ); per-block partials part[6][gridDim]
__global__ void __launch_bounds__(256) k_integrals(const double* __restrict__ U, const double* __restrict__ MetD,
                                                   const double* __restrict__ wq, int n, int nElems,
                                                   double* __restrict__ part) {
  __shared__ double red[6][8];
  const int n3 = n * n * n;
  const long long nn = (long long)nElems * n3;
  double acc[6] = {0, 0, 0, 0, 0, 0};
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < nn; t += (long long)gridDim.x * blockDim.x) {
    const long long e = t / n3;
    const int node = (int)(t - e * n3);
    const int i = node % n, j = (node / n) % n, k = node / (n * n);
    const double w = wq[i] * wq[j] * wq[k] / MetD[(e * 10 + 9) * n3 + node];
    const double* u = U + t * 5;
    acc[0] += w * u[0]; acc[1] += w * u[1]; acc[2] += w * u[2]; acc[3] += w * u[3]; acc[4] += w * u[4];
    acc[5] += w * 0.5 * (u[1] * u[1] + u[2] * u[2] + u[3] * u[3]) / u[0];
  }
#pragma unroll
  for (int c = 0; c < 6; ++c) {
    double v = acc[c];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) red[c][threadIdx.x >> 5] = v;
  }
  __syncthreads();
  if (threadIdx.x < 6) {
    double v = 0.;
    for (int w = 0; w < 8; ++w) v += red[threadIdx.x][w];
    part[(size_t)threadIdx.x * gridDim.x + blockIdx.x] = v;
  }
}
// gradient of the kinetic-energy integral with respect to U
__global__ void k_ke_grad(const double* __restrict__ U, const double* __restrict__ MetD, const double* __restrict__ wq,
                          int n, int nElems, double* __restrict__ G) {
  const int n3 = n * n * n;
  const long long nn = (long long)nElems * n3;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < nn; t += (long long)gridDim.x * blockDim.x) {
    const long long e = t / n3;
    const int node = (int)(t - e * n3);
    const int i = node % n, j = (node / n) % n, k = node / (n * n);
    const double w = wq[i] * wq[j] * wq[k] / MetD[(e * 10 + 9) * n3 + node];
    const double* u = U + t * 5;
    const double sr = 1. / u[0];
    const double ke = 0.5 * (u[1] * u[1] + u[2] * u[2] + u[3] * u[3]) * sr;
    G[t * 5 + 0] = -w * ke * sr;
    G[t * 5 + 1] = w * u[1] * sr;
    G[t * 5 + 2] = w * u[2] * sr;
    G[t * 5 + 3] = w * u[3] * sr;
    G[t * 5 + 4] = 0.;
  }
}

int need_fp64(dg_ctx* ctx, const char* what) {
  if (ctx->cfg.precision != DG_PRECISION_FP64) {
    set_error(std::string(what) + ": FP64 operator only");
    return DG_ERR_UNSUPPORTED;
  }
  return DG_OK;
}

int tlm_setup(dg_ctx* ctx) {
  if (int rc = need_fp64(ctx, "tangent-linear operator")) return rc;
  if (ctx->cfg.filter_type) { set_error("tangent-linear operator: no solution filter"); return DG_ERR_UNSUPPORTED; }
  if (ctx->cfg.split_dg != DG_SPLIT_NONE && ctx->cfg.split_dg != DG_SPLIT_PI && ctx->cfg.split_dg != DG_SPLIT_KG) {
    set_error("tangent-linear operator: split forms PI and KG only"); return DG_ERR_UNSUPPORTED;
  }
  if (ctx->nBCSides && !ctx->bcref_t.p) {  // (again after dg_set_boundaries)
    if (!ctx->bcref_t.alloc(ctx->bcref_d.n)) { set_error("cudaMalloc tangent-linear boundary states"); return DG_ERR_ALLOC; }
    k_to_dual<<<grid_for(ctx->bcref_d.n), 256>>>(ctx->bcref_d.p, ctx->bcref_t.p, ctx->bcref_d.n);
    CUDA_TRY(cudaDeviceSynchronize(), "tangent-linear boundary states");
  }
  if (ctx->t_ok) return DG_OK;
  const gxc::NPTable* T = table_for(ctx->n);
  if (int rc = T->configure_t()) return rc;
  const size_t nE = ctx->nElems, nS = ctx->nSides, n2 = ctx->n2, n3 = ctx->n3;
  gxc::PrecData<D1>& P = ctx->t;
  bool ok = P.basis.alloc(ctx->d.basis.n) && P.Met.alloc(ctx->d.Met.n) && P.Fgeo.alloc(ctx->d.Fgeo.n) &&
            P.Pvol.alloc(nE * 7 * n3) && P.Uf.alloc(2 * nS * 5 * n2) && P.Pf.alloc(2 * nS * 6 * n2) &&
            P.Flux.alloc(nS * 5 * n2) && ctx->Ud.alloc(nE * 5 * n3) && ctx->Utd.alloc(nE * 5 * n3);
  if (ok && ctx->cfg.parabolic) ok = P.Gvol.alloc(nE * 15 * n3) && P.Gf.alloc(2 * nS * 15 * n2);
  if (!ok) { set_error("cudaMalloc tangent-linear data"); return DG_ERR_ALLOC; }
  k_to_dual<<<grid_for(P.basis.n), 256>>>(ctx->d.basis.p, P.basis.p, P.basis.n);
  k_to_dual<<<grid_for(P.Met.n), 256>>>(ctx->d.Met.p, P.Met.p, P.Met.n);
  k_to_dual<<<grid_for(P.Fgeo.n), 256>>>(ctx->d.Fgeo.p, P.Fgeo.p, P.Fgeo.n);
  CUDA_TRY(cudaDeviceSynchronize(), "tangent-linear set-up");
  ctx->t_ok = true;
  return DG_OK;
}

int adj_setup(dg_ctx* ctx) {
  if (int rc = need_fp64(ctx, "adjoint")) return rc;
  if (ctx->cfg.filter_type) { set_error("adjoint: no solution filter"); return DG_ERR_UNSUPPORTED; }
  const dg_config& c = ctx->cfg;
  if (c.split_dg != DG_SPLIT_NONE && c.split_dg != DG_SPLIT_PI && c.split_dg != DG_SPLIT_KG) {
    set_error("adjoint: split forms PI and KG only"); return DG_ERR_UNSUPPORTED;
  }
  if (c.parabolic && (c.lifting != DG_LIFTING_BR1 || c.do_weak_lifting)) {
    set_error("adjoint: BR1 lifting in strong form only"); return DG_ERR_UNSUPPORTED;
  }
  if (ctx->UBv.p) return DG_OK;
  const gxc::NPTable* T = table_for(ctx->n);
  if (int rc = T->configure_a()) return rc;
  const size_t nE = ctx->nElems, nS = ctx->nSides, n2 = ctx->n2, n3 = ctx->n3;
  const size_t epb = n3 >= 128 ? 1 : 256 / n3;
  // partial sums of dR/dmu: ka_face (connected sides), ka_volume, ka_bc_face (BC sides)
  const size_t nparts = (nS * n2 + 127) / 128 + 1 + (nE + epb - 1) / epb;
  const size_t ipart = 6 * (size_t)grid_for(nE * n3);
  bool ok = ctx->UfB.alloc(2 * nS * 5 * n2) && ctx->JB.alloc(2 * nS * 5 * n2) && ctx->UBv.alloc(nE * 5 * n3) &&
            ctx->part.alloc(nparts > ipart ? nparts : ipart) && ctx->acc.alloc(8);
  if (ok) ok = ctx->GfB.alloc(2 * nS * 15 * n2);
  if (!ok) { ctx->UBv.release(); set_error("cudaMalloc adjoint scratch"); return DG_ERR_ALLOC; }
  // the face gradient cotangents stay zero for the Euler equations
  CUDA_TRY(cudaMemset(ctx->GfB.p, 0, ctx->GfB.n * sizeof(double)), "clear face gradient cotangents");
  CUDA_TRY(cudaMemset(ctx->JB.p, 0, ctx->JB.n * sizeof(double)), "clear lifting cotangents");
  return DG_OK;
}

int integrals(dg_ctx* ctx, const double* d_U, double out[6], cudaStream_t st) {
  const size_t nn = (size_t)ctx->nElems * ctx->n3;
  const int grid = grid_for(nn);
  if (!ctx->part.p || ctx->part.n < (size_t)6 * grid) {
    if (!ctx->part.alloc((size_t)6 * grid)) { set_error("cudaMalloc"); return DG_ERR_ALLOC; }
  }
  if (!ctx->acc.p && !ctx->acc.alloc(8)) { set_error("cudaMalloc"); return DG_ERR_ALLOC; }
  CUDA_TRY(cudaMemsetAsync(ctx->acc.p, 0, 8 * sizeof(double), st), "clear");
  k_integrals<<<grid, 256, 0, st>>>(d_U, ctx->metd, ctx->wq.p, ctx->n, ctx->nElems, ctx->part.p);
  for (int c = 0; c < 6; ++c) gx::k_adj_sum<<<1, 256, 0, st>>>(ctx->part.p + (size_t)c * grid, grid, ctx->acc.p + c);
  ctx->launches += 7;
  CUDA_TRY(cudaGetLastError(), "integrals launch");
  CUDA_TRY(cudaMemcpyAsync(out, ctx->acc.p, 6 * sizeof(double), cudaMemcpyDeviceToHost, st), "read integrals");
  CUDA_TRY(cudaStreamSynchronize(st), "sync integrals");
  return DG_OK;
}

// one forward LSERK stage (1..5) on (W, K)
int fwd_stage(dg_ctx* ctx, int stage, double dt, double* W, double* K, cudaStream_t st) {
  gx::RKArgs rk{W, K, nullptr, stage == 1 ? 0. : -1. * kRKA[stage], kRKb[stage] * dt};
  return run_rhs(ctx, W, rk, 1, st);
}
// one reverse LSERK stage at the stage input X
int rev_stage(dg_ctx* ctx, int stage, double dt, const double* X, double* Ubar, double* Kbar, cudaStream_t st) {
  const double b = kRKb[stage] * dt, mA = stage == 1 ? 0. : -1. * kRKA[stage];
  gx::CotSrc cs{Kbar, Ubar, b};
  return table_for(ctx->n)->adj(ctx, X, cs, 1, nullptr, Ubar, Kbar, b, mA, ctx->acc.p, st);
}

}  // namespace

extern "C" {

int dg_selftest_bulk_wait(long long polls, double* seconds) {
  if (polls < 1 || !seconds) { set_error("dg_selftest_bulk_wait: bad argument"); return DG_ERR_ARG; }
  gxc::DBuf<int> err;
  gxc::DBuf<long long> ns;
  if (!err.alloc(1) || !ns.alloc(1)) { set_error("dg_selftest_bulk_wait: device allocation failed"); return DG_ERR_CUDA; }
  CUDA_TRY(cudaMemset(err.p, 0, sizeof(int)), "cudaMemset");
  k_selftest_bulk_wait<<<1, 64>>>(polls, err.p, ns.p);
  CUDA_TRY(cudaGetLastError(), "k_selftest_bulk_wait launch");
  CUDA_TRY(cudaDeviceSynchronize(), "k_selftest_bulk_wait");
  int f = 0;
  long long t = 0;
  CUDA_TRY(cudaMemcpy(&f, err.p, sizeof(int), cudaMemcpyDeviceToHost), "read error flag");
  CUDA_TRY(cudaMemcpy(&t, ns.p, sizeof(long long), cudaMemcpyDeviceToHost), "read duration");
  *seconds = t * 1e-9;
  if (!f) return DG_OK;
  set_error("a kernel's wait for its bulk copies into shared memory ran out (self-test)");
  return DG_ERR_TIMEOUT;
}

int dg_measure_fma_peak(int precision, double* gflops) {
  if (!gflops) { set_error("null output"); return DG_ERR_ARG; }
  return precision == 0 ? fma_peak<double>(gflops) : fma_peak<float>(gflops);
}

int dg_profile_stage(dg_ctx* ctx, double* d_U, double* d_Ut_tmp, double dt, int reps, double* ms_out, void* stream) {
  if (int rc = check_ctx(ctx, true)) return rc;
  if (!d_U || !d_Ut_tmp || !ms_out || reps < 1) { set_error("dg_profile_stage: bad argument"); return DG_ERR_ARG; }
  cudaStream_t st = (cudaStream_t)stream;
  cudaEvent_t ev[5];
  for (int i = 0; i < 5; ++i) CUDA_TRY(cudaEventCreate(&ev[i]), "cudaEventCreate");
  double acc[5] = {0, 0, 0, 0, 0};
  int rc = DG_OK;
  for (int r = 0; r < reps && rc == DG_OK; ++r) {
    const int stage = 2 + (r % 4);
    gx::RKArgs rk{d_U, d_Ut_tmp, nullptr, -1. * kRKA[stage], kRKb[stage] * dt};
    rc = table_for(ctx->n)->stage_events(ctx, d_U, rk, st, ev);
    if (rc != DG_OK) break;
    if (cudaEventSynchronize(ev[4]) != cudaSuccess) { set_error("event sync"); rc = DG_ERR_CUDA; break; }
    float ms[4];
    for (int k = 0; k < 4; ++k) cudaEventElapsedTime(&ms[k], ev[k], ev[k + 1]);
    float tot = 0;
    cudaEventElapsedTime(&tot, ev[0], ev[4]);
    for (int k = 0; k < 4; ++k) acc[k] += ms[k];
    acc[4] += tot;
  }
  for (int i = 0; i < 5; ++i) cudaEventDestroy(ev[i]);
  if (rc != DG_OK) return rc;
  for (int k = 0; k < 5; ++k) ms_out[k] = acc[k] / reps;
  return DG_OK;
}


int dg_ctx_create(const dg_config* cfg, dg_ctx** out) {
  if (!cfg || !out) { set_error("dg_ctx_create: null argument"); return DG_ERR_ARG; }
  *out = nullptr;
  if (cfg->N < 1 || cfg->N > DG_MAX_N) { set_error("N out of range 1..DG_MAX_N"); return DG_ERR_ARG; }
  if (cfg->node_type != DG_NODETYPE_GAUSS && cfg->node_type != DG_NODETYPE_GAUSS_LOBATTO) {
    set_error("unknown node type"); return DG_ERR_ARG;
  }
  if (cfg->riemann < DG_RIEMANN_LF || cfg->riemann > DG_RIEMANN_AVERAGE) { set_error("unknown Riemann solver"); return DG_ERR_ARG; }
  if (cfg->split_dg < DG_SPLIT_NONE || cfg->split_dg > DG_SPLIT_PI) { set_error("unknown SplitDG"); return DG_ERR_ARG; }
  if (cfg->split_dg >= 0 && cfg->node_type != DG_NODETYPE_GAUSS_LOBATTO) {
    // InitSplitDG (splitflux.f90:115-119)
    set_error("Wrong Pointset: Gauss-Lobatto-Points are mandatory for using SplitDG"); return DG_ERR_ARG;
  }
  if (cfg->split_dg >= 0 && (cfg->riemann == DG_RIEMANN_HLL || cfg->riemann == DG_RIEMANN_HLLC ||
                             cfg->riemann == DG_RIEMANN_HLLE || cfg->riemann == DG_RIEMANN_HLLEM)) {
    // src/CMakeLists.txt:108-127 rejects the HLL family with split fluxes
    set_error("HLL-type Riemann solvers are not available with split-form DG"); return DG_ERR_ARG;
  }
  if (cfg->split_dg < 0 && cfg->riemann == DG_RIEMANN_AVERAGE) { set_error("Riemann=avg needs SplitDG"); return DG_ERR_ARG; }
  if (cfg->split_dg >= 0 && cfg->N < 2) { set_error("split form needs N >= 2"); return DG_ERR_UNSUPPORTED; }
  if (cfg->lifting != DG_LIFTING_BR1 && cfg->lifting != DG_LIFTING_BR2) { set_error("bad lifting"); return DG_ERR_ARG; }
  if (cfg->parabolic && cfg->lifting == DG_LIFTING_BR2 && cfg->do_weak_lifting) {
    // the BR2 lifting is always in strong form (lifting.f90:103)
    set_error("BR2 lifting is strong-form only: doWeakLifting must be F"); return DG_ERR_ARG;
  }
  if (!(cfg->kappa > 1.) || !(cfg->R > 0.)) { set_error("bad kappa or R"); return DG_ERR_ARG; }
  if (cfg->parabolic && !(cfg->Pr > 0.)) { set_error("bad Pr"); return DG_ERR_ARG; }
  if (cfg->precision != DG_PRECISION_FP64 && cfg->precision != DG_PRECISION_MIXED) { set_error("bad precision"); return DG_ERR_ARG; }
  std::vector<double> fmat;
  if (cfg->filter_type < DG_FILTER_NONE || cfg->filter_type > DG_FILTER_LAF) { set_error("unknown FilterType"); return DG_ERR_ARG; }
  if (cfg->filter_type != DG_FILTER_NONE && gxh::filter_matrix(*cfg, fmat) != 0) {
    set_error("filter: NFilter must be in 0..N (cut-off and LAF)"); return DG_ERR_ARG;
  }
  dg_ctx* ctx = new dg_ctx();
  ctx->cfg = *cfg;
  ctx->N = cfg->N;
  ctx->n = cfg->N + 1;
  ctx->n2 = ctx->n * ctx->n;
  ctx->n3 = ctx->n2 * ctx->n;
  gxh::basis_1d(cfg->N, cfg->node_type, ctx->B);
  const gxc::NPTable* T = table_for(ctx->n);
  int rc = upload_basis(ctx, ctx->d);
  if (rc == DG_OK && cfg->precision == DG_PRECISION_MIXED) rc = upload_basis(ctx, ctx->f);
  if (rc == DG_OK) rc = (cfg->precision == DG_PRECISION_FP64) ? T->configure_d() : T->configure_f();
  if (rc == DG_OK && !(ctx->red.alloc(2) && ctx->bad.alloc(1) && ctx->kerr.alloc(1))) { set_error("cudaMalloc"); rc = DG_ERR_ALLOC; }
  if (rc == DG_OK && cudaMemset(ctx->kerr.p, 0, sizeof(int)) != cudaSuccess) { set_error("clear error flag"); rc = DG_ERR_CUDA; }
  if (rc == DG_OK && !fmat.empty()) {
    if (!ctx->filt.alloc(fmat.size())) { set_error("cudaMalloc filter"); rc = DG_ERR_ALLOC; }
    else if (cudaMemcpy(ctx->filt.p, fmat.data(), fmat.size() * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess) {
      set_error("upload FilterMat"); rc = DG_ERR_CUDA;
    }
    // normMod of the LAF filter (filter.f90:194)
    const double Nf = (double)cfg->n_filter, Np = (double)cfg->N;
    ctx->laf_norm = (std::pow(Nf + 1., -2. / 3.) - std::pow(2., -2. / 3.)) /
                    (std::pow(Np + 1., -2. / 3.) - std::pow(Nf + 1., -2. / 3.));
  }
  if (rc != DG_OK) { dg_ctx_destroy(ctx); return rc; }
  *out = ctx;
  return DG_OK;
}

int dg_ctx_destroy(dg_ctx* ctx) {
  if (!ctx) return DG_OK;
  ctx->d.release();
  ctx->f.release();
  ctx->MetD.release();
  ctx->E2S.release();
  ctx->red.release();
  ctx->bad.release();
  ctx->kerr.release();
  ctx->S2E.release(); ctx->wq.release();
  ctx->bctype.release(); ctx->bcstate.release(); ctx->bcref_d.release(); ctx->bcref_f.release(); ctx->bcref_t.release();
  ctx->t.release(); ctx->Ud.release(); ctx->Utd.release();
  ctx->UfB.release(); ctx->GfB.release(); ctx->JB.release(); ctx->UBv.release(); ctx->part.release();
  ctx->acc.release(); ctx->W.release(); ctx->K.release(); ctx->tape.store.release();
  ctx->filt.release(); ctx->laf.release(); ctx->cflm.release();
  delete ctx;
  return DG_OK;
}

int dg_set_mesh(dg_ctx* ctx, int nElems, int nSides, int nBCSides, const double* Mf, const double* Mg,
                const double* Mh, const double* sJ, const double* nv, const double* t1, const double* t2,
                const double* se, const int* e2s, const int* s2e) {
  if (int rc = check_ctx(ctx, false)) return rc;
  if (nElems < 1 || nSides < 1 || !Mf || !Mg || !Mh || !sJ || !nv || !t1 || !t2 || !se || !e2s || !s2e) {
    set_error("dg_set_mesh: bad argument"); return DG_ERR_ARG;
  }
  if (nBCSides < 0 || nBCSides > nSides) { set_error("dg_set_mesh: bad nBCSides"); return DG_ERR_ARG; }
  const int n = ctx->n, n2 = ctx->n2, n3 = ctx->n3;
  // validate connectivity: every side has one master (flip 0) and one slave (flip 1..4)
  std::vector<int> seen((size_t)nSides * 2, 0);
  std::vector<int> he2s((size_t)nElems * 12);
  for (int e = 0; e < nElems; ++e)
    for (int ls = 0; ls < 6; ++ls) {
      const int side = e2s[3 * (ls + 6 * (size_t)e)] - 1, flip = e2s[3 * (ls + 6 * (size_t)e) + 1];
      if (side < 0 || side >= nSides || flip < 0 || flip > 4) { set_error("ElemToSide out of range"); return DG_ERR_ARG; }
      seen[2 * (size_t)side + (flip == 0 ? 0 : 1)]++;
      he2s[(e * 6 + ls) * 2] = side;
      he2s[(e * 6 + ls) * 2 + 1] = flip;
    }
  for (size_t t = 0; t < seen.size(); ++t)
    if (seen[t] != ((t & 1) && (int)(t / 2) < nBCSides ? 0 : 1)) {
      set_error("every inner side needs one master and one slave element, every BC side (the first nBCSides) one "
                "master");
      return DG_ERR_ARG;
    }
  (void)s2e;
  // pack metrics [e][10][n3] and face geometry [side][10][n2]
  std::vector<double> met((size_t)nElems * 10 * n3), fgeo((size_t)nSides * 10 * n2);
  for (size_t e = 0; e < (size_t)nElems; ++e)
    for (int node = 0; node < n3; ++node) {
      const size_t g = e * n3 + node;
      for (int c = 0; c < 3; ++c) {
        met[(e * 10 + c) * n3 + node] = Mf[3 * g + c];
        met[(e * 10 + 3 + c) * n3 + node] = Mg[3 * g + c];
        met[(e * 10 + 6 + c) * n3 + node] = Mh[3 * g + c];
      }
      met[(e * 10 + 9) * n3 + node] = sJ[g];
    }
  for (size_t s = 0; s < (size_t)nSides; ++s)
    for (int pq = 0; pq < n2; ++pq) {
      const size_t g = s * n2 + pq;
      for (int c = 0; c < 3; ++c) {
        fgeo[(s * 10 + c) * n2 + pq] = nv[3 * g + c];
        fgeo[(s * 10 + 3 + c) * n2 + pq] = t1[3 * g + c];
        fgeo[(s * 10 + 6 + c) * n2 + pq] = t2[3 * g + c];
      }
      fgeo[(s * 10 + 9) * n2 + pq] = se[g];
    }
  (void)n;
  ctx->nElems = nElems;
  ctx->nSides = nSides;
  ctx->d.release();
  ctx->f.release();
  int rc = upload_basis(ctx, ctx->d);
  if (rc == DG_OK) {
    if (ctx->cfg.precision == DG_PRECISION_FP64) {
      rc = alloc_prec(ctx, ctx->d, met, fgeo);
    } else {
      rc = upload_basis(ctx, ctx->f);
      if (rc == DG_OK) rc = alloc_prec(ctx, ctx->f, met, fgeo);
    }
  }
  if (rc != DG_OK) return rc;
  if (!ctx->E2S.alloc(he2s.size())) { set_error("cudaMalloc mesh"); return DG_ERR_ALLOC; }
  if (ctx->cfg.precision == DG_PRECISION_FP64) {
    ctx->MetD.release();
    ctx->metd = ctx->d.Met.p;  // same layout and precision: no second copy
  } else {
    if (!ctx->MetD.alloc(met.size())) { set_error("cudaMalloc mesh"); return DG_ERR_ALLOC; }
    CUDA_TRY(cudaMemcpy(ctx->MetD.p, met.data(), met.size() * sizeof(double), cudaMemcpyHostToDevice), "upload metrics");
    ctx->metd = ctx->MetD.p;
  }
  CUDA_TRY(cudaMemcpy(ctx->E2S.p, he2s.data(), he2s.size() * sizeof(int), cudaMemcpyHostToDevice), "upload E2S");
  // SideToElem on the device, from the validated ElemToSide: master elem/side, slave elem/side, flip
  std::vector<int> hs2e((size_t)nSides * 5, 0);
  for (int e = 0; e < nElems; ++e)
    for (int ls = 0; ls < 6; ++ls) {
      const int side = he2s[(e * 6 + ls) * 2], flip = he2s[(e * 6 + ls) * 2 + 1];
      int* q = &hs2e[(size_t)side * 5];
      if (flip == 0) { q[0] = e; q[1] = ls + 1; }
      else { q[2] = e; q[3] = ls + 1; q[4] = flip; }
    }
  if (!ctx->S2E.alloc(hs2e.size()) || !ctx->wq.alloc(n)) { set_error("cudaMalloc mesh"); return DG_ERR_ALLOC; }
  CUDA_TRY(cudaMemcpy(ctx->S2E.p, hs2e.data(), hs2e.size() * sizeof(int), cudaMemcpyHostToDevice), "upload S2E");
  CUDA_TRY(cudaMemcpy(ctx->wq.p, ctx->B.w.data(), n * sizeof(double), cudaMemcpyHostToDevice), "upload weights");
  ctx->nBCSides = nBCSides;
  ctx->bc_ok = nBCSides == 0;
  ctx->bctype.release(); ctx->bcstate.release(); ctx->bcref_d.release(); ctx->bcref_f.release(); ctx->bcref_t.release();
  ctx->t_ok = false;
  ctx->tape.ok = false;
  ctx->t.release(); ctx->Ud.release(); ctx->Utd.release();
  ctx->UfB.release(); ctx->GfB.release(); ctx->JB.release(); ctx->UBv.release(); ctx->part.release();
  ctx->W.release(); ctx->K.release(); ctx->tape.store.release();
  // MetricsAdv and MetricsVisc of InitCalctimestep (navierstokes/calctimestep.f90:51-92), FP64
  {
    const dg_config& c = ctx->cfg;
    const double kpr = (4. / 3. > c.kappa / c.Pr) ? 4. / 3. : c.kappa / c.Pr;  // KAPPASPR_MAX_TIMESTEP_H
    std::vector<double> h((size_t)nElems * 6 * n3);
    const double* Ms[3] = {Mf, Mg, Mh};
    for (size_t e = 0; e < (size_t)nElems; ++e)
      for (int t = 0; t < n3; ++t) {
        const size_t id = e * n3 + t;
        const double sj = sJ[id];
        for (int d = 0; d < 3; ++d) {
          const double* m = Ms[d] + 3 * id;
          h[(e * 6 + d) * n3 + t] = sj * std::sqrt(m[0] * m[0] + m[1] * m[1] + m[2] * m[2]);
          h[(e * 6 + 3 + d) * n3 + t] = kpr * ((m[0] * sj) * (m[0] * sj) + (m[1] * sj) * (m[1] * sj) + (m[2] * sj) * (m[2] * sj));
        }
      }
    if (!ctx->cflm.alloc(h.size())) { set_error("cudaMalloc CFL metrics"); return DG_ERR_ALLOC; }
    CUDA_TRY(cudaMemcpy(ctx->cflm.p, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice), "upload CFL metrics");
  }
  ctx->laf.release();
  if (ctx->cfg.filter_type == DG_FILTER_LAF) {
    // IntegrationWeight = w_i w_j w_k / sJ normalised by the element volume, and the initial state
    // lim = 1e-8, eRatio = r = 0, previous energies 1e-16 (InitFilter, filter.f90:170-199)
    const size_t nE = nElems;
    std::vector<double> h(5 * nE + nE * n3);
    for (size_t e = 0; e < nE; ++e) {
      h[e] = 1e-8; h[nE + e] = 0.; h[2 * nE + e] = 0.; h[3 * nE + e] = 1e-16; h[4 * nE + e] = 1e-16;
      double* iw = &h[5 * nE + e * n3];
      double vol = 0.;
      for (int k = 0; k < n; ++k) for (int j = 0; j < n; ++j) for (int i = 0; i < n; ++i) {
        const int node = i + n * (j + n * k);
        iw[node] = ctx->B.w[i] * ctx->B.w[j] * ctx->B.w[k] / sJ[e * n3 + node];
        vol = vol + iw[node];
      }
      for (int t = 0; t < n3; ++t) iw[t] = iw[t] / vol;
    }
    if (!ctx->laf.alloc(h.size())) { set_error("cudaMalloc LAF state"); return DG_ERR_ALLOC; }
    CUDA_TRY(cudaMemcpy(ctx->laf.p, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice), "upload LAF state");
  }
  ctx->mesh_ok = true;
  ctx->grad_ok = false;
  return DG_OK;
}

int dg_laf_state(dg_ctx* ctx, double* lim, double* eRatio, double* r) {
  if (int rc = check_ctx(ctx, true)) return rc;
  if (ctx->cfg.filter_type != DG_FILTER_LAF || !ctx->laf.p) { set_error("dg_laf_state: FilterType is not LAF"); return DG_ERR_ARG; }
  const size_t nE = ctx->nElems;
  CUDA_TRY(cudaDeviceSynchronize(), "LAF state");
  if (lim) CUDA_TRY(cudaMemcpy(lim, ctx->laf.p, nE * sizeof(double), cudaMemcpyDeviceToHost), "LAF lim");
  if (eRatio) CUDA_TRY(cudaMemcpy(eRatio, ctx->laf.p + nE, nE * sizeof(double), cudaMemcpyDeviceToHost), "LAF eRatio");
  if (r) CUDA_TRY(cudaMemcpy(r, ctx->laf.p + 2 * nE, nE * sizeof(double), cudaMemcpyDeviceToHost), "LAF r");
  return DG_OK;
}

int dg_set_boundaries(dg_ctx* ctx, const int* bc_type, const int* bc_state, int nRefState, const double* refstate) {
  if (!ctx || !ctx->mesh_ok) { set_error("dg_set_boundaries: call dg_set_mesh first"); return DG_ERR_ARG; }
  const int nb = ctx->nBCSides;
  if (nb == 0) { ctx->bc_ok = true; return DG_OK; }
  if (!bc_type || !bc_state || nRefState < 1 || !refstate) { set_error("dg_set_boundaries: bad argument"); return DG_ERR_ARG; }
  std::vector<int> st(nb);
  for (int s = 0; s < nb; ++s) {
    const int t = bc_type[s];
    if (t != 2 && t != 3 && t != 4 && t != 9 && t != 91 && t != 23 && t != 24 && t != 25 && t != 27) {
      set_error("dg_set_boundaries: BC type " + std::to_string(t) + " is not supported"); return DG_ERR_UNSUPPORTED;
    }
    st[s] = bc_state[s] - 1;  // 1-based as in BoundaryType(BC_STATE)
    const bool needs_state = t != 3 && t != 9 && t != 91;
    if (needs_state && (st[s] < 0 || st[s] >= nRefState)) { set_error("dg_set_boundaries: BC state out of range"); return DG_ERR_ARG; }
    if (st[s] < 0 || st[s] >= nRefState) st[s] = 0;
  }
  // RefStatePrim as InitEquation (equation.f90:136-147) builds it: T = p * (1/rho) / R
  std::vector<double> rd((size_t)nRefState * 6);
  std::vector<float> rf((size_t)nRefState * 6);
  for (int r = 0; r < nRefState; ++r) {
    const double* q = refstate + 5 * (size_t)r;
    for (int c = 0; c < 5; ++c) rd[6 * r + c] = q[c];
    rd[6 * r + 5] = q[4] * (1. / q[0]) / ctx->cfg.R;
  }
  // type 27 states: (Tt, alpha, beta, -, pt), angles in degrees -> the inflow direction a(1:3)
  // (InitBC, getboundaryflux.f90:199-208), once per state
  std::vector<char> done(nRefState, 0);
  for (int s = 0; s < nb; ++s) {
    if (bc_type[s] != 27 || done[st[s]]) continue;
    done[st[s]] = 1;
    double* q = &rd[6 * (size_t)st[s]];
    const double pi = 3.141592653589793238462643383279502884197;
    const double ta = std::tan(pi / 180. * q[1]), tb = std::tan(pi / 180. * q[2]);
    q[1] = 1. / std::sqrt(1. + ta * ta + tb * tb);
    q[2] = ta / std::sqrt(1. + ta * ta + tb * tb);
    q[3] = tb / std::sqrt(1. + ta * ta + tb * tb);
  }
  for (size_t i = 0; i < rd.size(); ++i) rf[i] = (float)rd[i];
  if (!ctx->bctype.alloc(nb) || !ctx->bcstate.alloc(nb) || !ctx->bcref_d.alloc(rd.size()) || !ctx->bcref_f.alloc(rf.size())) {
    set_error("cudaMalloc boundaries"); return DG_ERR_ALLOC;
  }
  CUDA_TRY(cudaMemcpy(ctx->bctype.p, bc_type, nb * sizeof(int), cudaMemcpyHostToDevice), "upload BC types");
  CUDA_TRY(cudaMemcpy(ctx->bcstate.p, st.data(), nb * sizeof(int), cudaMemcpyHostToDevice), "upload BC states");
  CUDA_TRY(cudaMemcpy(ctx->bcref_d.p, rd.data(), rd.size() * sizeof(double), cudaMemcpyHostToDevice), "upload RefStates");
  CUDA_TRY(cudaMemcpy(ctx->bcref_f.p, rf.data(), rf.size() * sizeof(float), cudaMemcpyHostToDevice), "upload RefStates");
  ctx->bc_ok = true;
  return DG_OK;
}

int dg_rhs(dg_ctx* ctx, double t, double* d_U, double* d_Ut, void* stream) {
  if (int rc = check_ctx(ctx, true)) return rc;
  if (!d_U || !d_Ut) { set_error("dg_rhs: null state"); return DG_ERR_ARG; }
  (void)t;  // periodic meshes: no time-dependent boundary states or sources
  gx::RKArgs rk{nullptr, nullptr, d_Ut, 0., 0.};
  cudaStream_t st = (cudaStream_t)stream;
  return run_rhs(ctx, d_U, rk, 0, st);
}

int dg_lserk_steps(dg_ctx* ctx, double t, double dt, int nSteps, double* d_U, double* d_Ut_tmp, void* stream) {
  if (int rc = check_ctx(ctx, true)) return rc;
  if (!d_U || !d_Ut_tmp || nSteps < 0) { set_error("dg_lserk_steps: bad argument"); return DG_ERR_ARG; }
  cudaStream_t st = (cudaStream_t)stream;
  for (int s = 0; s < nSteps; ++s) {
    for (int stage = 1; stage <= 5; ++stage) {
      // TimeStepByLSERKW2 (timestep.f90:83-104): mRKA = 0 at stage 1, -RKA(stage) otherwise
      gx::RKArgs rk{d_U, d_Ut_tmp, nullptr, stage == 1 ? 0. : -1. * kRKA[stage], kRKb[stage] * dt};
      int rc = run_rhs(ctx, d_U, rk, 1, st);
      if (rc != DG_OK) return rc;
    }
  }
  (void)t;
  return DG_OK;
}

int dg_lserk_step(dg_ctx* ctx, double t, double dt, double* d_U, double* d_Ut_tmp, void* stream) {
  return dg_lserk_steps(ctx, t, dt, 1, d_U, d_Ut_tmp, stream);
}

// the error flag of the kernels' bounded waits (read after the stream has been synchronised)
static int kernel_wait_status(dg_ctx* ctx, cudaStream_t st) {
  int f = 0;
  CUDA_TRY(cudaMemcpyAsync(&f, ctx->kerr.p, sizeof(int), cudaMemcpyDeviceToHost, st), "read error flag");
  CUDA_TRY(cudaStreamSynchronize(st), "sync error flag");
  if (!f) return DG_OK;
  CUDA_TRY(cudaMemsetAsync(ctx->kerr.p, 0, sizeof(int), st), "clear error flag");
  set_error("a kernel's wait for its bulk copies into shared memory ran out; results since the last check are invalid");
  return DG_ERR_TIMEOUT;
}

int dg_calc_timestep(dg_ctx* ctx, const double* d_U, double cfl_scale, double dfl_scale, double* dt_out, void* stream) {
  if (int rc = check_ctx(ctx, true)) return rc;
  if (!d_U || !dt_out) { set_error("dg_calc_timestep: null argument"); return DG_ERR_ARG; }
  cudaStream_t st = (cudaStream_t)stream;
  const int N = ctx->N;
  const dg_config& c = ctx->cfg;
  const double cflS = cfl_scale * cfl_alpha(c.node_type, N) / (2. * N + 1.);
  const double dflS = dfl_scale * dfl_alpha(c.node_type, N) * 1.853 / ((2. * N + 1.) * (2. * N + 1.));
  const double kpr = (4. / 3. > c.kappa / c.Pr) ? 4. / 3. : c.kappa / c.Pr;  // KAPPASPR_MAX_TIMESTEP_H
  const double init[2] = {HUGE_VAL, HUGE_VAL};
  CUDA_TRY(cudaMemcpyAsync(ctx->red.p, init, sizeof(init), cudaMemcpyHostToDevice, st), "reset dt");
  CUDA_TRY(cudaMemsetAsync(ctx->bad.p, 0, sizeof(unsigned long long), st), "reset flag");
  if (int rc = table_for(ctx->n)->cfl(ctx, d_U, cflS, dflS, kpr, st)) return rc;
  double h[2];
  unsigned long long bad = 0;
  CUDA_TRY(cudaMemcpyAsync(h, ctx->red.p, sizeof(h), cudaMemcpyDeviceToHost, st), "read dt");
  CUDA_TRY(cudaMemcpyAsync(&bad, ctx->bad.p, sizeof(bad), cudaMemcpyDeviceToHost, st), "read flag");
  CUDA_TRY(cudaStreamSynchronize(st), "sync dt");
  *dt_out = h[0] < h[1] ? h[0] : h[1];
  if (int rc = kernel_wait_status(ctx, st)) return rc;
  if (bad) { set_error("state holds NaN/Inf or non-positive density/pressure"); return DG_ERR_NAN; }
  return DG_OK;
}

int dg_check_state(dg_ctx* ctx, const double* d_U, long long* bad_count, void* stream) {
  if (int rc = check_ctx(ctx, true)) return rc;
  if (!d_U || !bad_count) { set_error("dg_check_state: null argument"); return DG_ERR_ARG; }
  cudaStream_t st = (cudaStream_t)stream;
  CUDA_TRY(cudaMemsetAsync(ctx->bad.p, 0, sizeof(unsigned long long), st), "reset flag");
  const long long nNodes = (long long)ctx->nElems * ctx->n3;
  int grid = (int)((nNodes + 255) / 256);
  if (grid > 152 * 32) grid = 152 * 32;
  gx::k_check<<<grid, 256, 0, st>>>(d_U, nNodes, ctx->cfg.kappa, ctx->bad.p);
  ctx->launches++;
  CUDA_TRY(cudaGetLastError(), "k_check launch");
  unsigned long long bad = 0;
  CUDA_TRY(cudaMemcpyAsync(&bad, ctx->bad.p, sizeof(bad), cudaMemcpyDeviceToHost, st), "read flag");
  CUDA_TRY(cudaStreamSynchronize(st), "sync check");
  *bad_count = (long long)bad;
  if (int rc = kernel_wait_status(ctx, st)) return rc;
  return bad ? DG_ERR_NAN : DG_OK;
}

int dg_get_gradients(dg_ctx* ctx, double* d_gradUx, double* d_gradUy, double* d_gradUz, void* stream) {
  if (int rc = check_ctx(ctx, true)) return rc;
  if (!d_gradUx || !d_gradUy || !d_gradUz) { set_error("dg_get_gradients: null argument"); return DG_ERR_ARG; }
  if (!ctx->cfg.parabolic) { set_error("dg_get_gradients: operator is not parabolic"); return DG_ERR_UNSUPPORTED; }
  if (!ctx->grad_ok) { set_error("dg_get_gradients: no RHS evaluated on this mesh yet"); return DG_ERR_ARG; }
  cudaStream_t st = (cudaStream_t)stream;
  if (!ctx->grad_rho) {
    // the operator lifts without the density gradient; complete it from the stored primitive state
    if (int rc = table_for(ctx->n)->relift(ctx, st)) return rc;
    ctx->grad_rho = true;
  }
  const long long nNodes = (long long)ctx->nElems * ctx->n3;
  int grid = (int)((nNodes + 255) / 256);
  if (grid > 152 * 16) grid = 152 * 16;
  if (ctx->cfg.precision == DG_PRECISION_FP64)
    k_export_grad<double><<<grid, 256, 0, st>>>(ctx->d.Gvol.p, nNodes, ctx->n3, d_gradUx, d_gradUy, d_gradUz);
  else
    k_export_grad<float><<<grid, 256, 0, st>>>(ctx->f.Gvol.p, nNodes, ctx->n3, d_gradUx, d_gradUy, d_gradUz);
  ctx->launches++;
  CUDA_TRY(cudaGetLastError(), "k_export_grad launch");
  return DG_OK;
}

long long dg_kernel_launch_count(const dg_ctx* ctx) { return ctx ? ctx->launches : 0; }

int dg_set_pressure_offset(dg_ctx* ctx, double p_ref) {
  if (int rc = check_ctx(ctx, false)) return rc;
  if (!(p_ref >= 0.) || !std::isfinite(p_ref)) { set_error("pressure offset must be finite and >= 0"); return DG_ERR_ARG; }
  ctx->pref = p_ref;
  return DG_OK;
}

int dg_integrals(dg_ctx* ctx, const double* d_U, double* out6, void* stream) {
  if (int rc = check_ctx(ctx, true)) return rc;
  if (!d_U || !out6) { set_error("dg_integrals: null argument"); return DG_ERR_ARG; }
  return integrals(ctx, d_U, out6, (cudaStream_t)stream);
}

int dg_kinetic_energy(dg_ctx* ctx, const double* d_U, double* J, double* d_dJdU, void* stream) {
  if (int rc = check_ctx(ctx, true)) return rc;
  if (!d_U || !J) { set_error("dg_kinetic_energy: null argument"); return DG_ERR_ARG; }
  cudaStream_t st = (cudaStream_t)stream;
  double out[6];
  if (int rc = integrals(ctx, d_U, out, st)) return rc;
  *J = out[5];
  if (d_dJdU) {
    k_ke_grad<<<grid_for((size_t)ctx->nElems * ctx->n3), 256, 0, st>>>(d_U, ctx->metd, ctx->wq.p, ctx->n,
                                                                     ctx->nElems, d_dJdU);
    ctx->launches++;
    CUDA_TRY(cudaGetLastError(), "k_ke_grad launch");
  }
  return DG_OK;
}

int dg_rhs_jvp(dg_ctx* ctx, double t, const double* d_U, const double* d_Udot, double mu_dot, double* d_Ut,
               double* d_Utdot, void* stream) {
  if (int rc = check_ctx(ctx, true)) return rc;
  if (!d_U || !d_Utdot) { set_error("dg_rhs_jvp: null argument"); return DG_ERR_ARG; }
  if (int rc = tlm_setup(ctx)) return rc;
  (void)t;
  cudaStream_t st = (cudaStream_t)stream;
  const size_t cnt = (size_t)ctx->nElems * 5 * ctx->n3;
  k_pack<<<grid_for(cnt), 256, 0, st>>>(d_U, d_Udot, ctx->Ud.p, cnt);
  gx::RKArgsT<D1> rk{nullptr, nullptr, ctx->Utd.p, 0., 0.};
  if (int rc = table_for(ctx->n)->rhs_t(ctx, ctx->Ud.p, rk, 0, mu_dot, st)) return rc;
  k_unpack<<<grid_for(cnt), 256, 0, st>>>(ctx->Utd.p, d_Ut, d_Utdot, cnt);
  ctx->launches += 2;
  CUDA_TRY(cudaGetLastError(), "dg_rhs_jvp");
  return DG_OK;
}

int dg_tlm_steps(dg_ctx* ctx, double t, double dt, int nSteps, double* d_U, double* d_Udot, double mu_dot,
                 double* d_Ut_tmp, void* stream) {
  if (int rc = check_ctx(ctx, true)) return rc;
  if (!d_U || !d_Udot || !d_Ut_tmp || nSteps < 0) { set_error("dg_tlm_steps: bad argument"); return DG_ERR_ARG; }
  if (int rc = tlm_setup(ctx)) return rc;
  (void)t;
  cudaStream_t st = (cudaStream_t)stream;
  const size_t cnt = (size_t)ctx->nElems * 5 * ctx->n3;
  k_pack<<<grid_for(cnt), 256, 0, st>>>(d_U, d_Udot, ctx->Ud.p, cnt);
  k_pack<<<grid_for(cnt), 256, 0, st>>>(d_Ut_tmp, nullptr, ctx->Utd.p, cnt);
  for (int s = 0; s < nSteps; ++s)
    for (int stage = 1; stage <= 5; ++stage) {
      gx::RKArgsT<D1> rk{ctx->Ud.p, ctx->Utd.p, nullptr, stage == 1 ? 0. : -1. * kRKA[stage], kRKb[stage] * dt};
      if (int rc = table_for(ctx->n)->rhs_t(ctx, ctx->Ud.p, rk, 1, mu_dot, st)) return rc;
    }
  k_unpack<<<grid_for(cnt), 256, 0, st>>>(ctx->Ud.p, d_U, d_Udot, cnt);
  k_unpack<<<grid_for(cnt), 256, 0, st>>>(ctx->Utd.p, d_Ut_tmp, nullptr, cnt);
  ctx->launches += 4;
  CUDA_TRY(cudaGetLastError(), "dg_tlm_steps");
  return DG_OK;
}

int dg_rhs_vjp(dg_ctx* ctx, double t, const double* d_U, const double* d_Utbar, double* d_Ubar, double* mu_bar,
               void* stream) {
  if (int rc = check_ctx(ctx, true)) return rc;
  if (!d_U || !d_Utbar || !d_Ubar) { set_error("dg_rhs_vjp: null argument"); return DG_ERR_ARG; }
  if (int rc = adj_setup(ctx)) return rc;
  (void)t;
  cudaStream_t st = (cudaStream_t)stream;
  CUDA_TRY(cudaMemsetAsync(ctx->acc.p, 0, sizeof(double), st), "clear");
  gx::CotSrc cs{d_Utbar, nullptr, 0.};
  if (int rc = table_for(ctx->n)->adj(ctx, d_U, cs, 0, d_Ubar, nullptr, nullptr, 0., 0., ctx->acc.p, st)) return rc;
  if (mu_bar) {
    CUDA_TRY(cudaMemcpyAsync(mu_bar, ctx->acc.p, sizeof(double), cudaMemcpyDeviceToHost, st), "read mu_bar");
    CUDA_TRY(cudaStreamSynchronize(st), "sync");
  }
  return DG_OK;
}

int dg_adjoint_scratch_bytes(dg_ctx* ctx, size_t* bytes) {
  if (int rc = check_ctx(ctx, true)) return rc;
  if (!bytes) { set_error("dg_adjoint_scratch_bytes: null argument"); return DG_ERR_ARG; }
  const size_t nE = ctx->nElems, nS = ctx->nSides, n2 = ctx->n2, n3 = ctx->n3, S = nE * 5 * n3;
  size_t b = S;  // the reverse sweep's second K (plans 2 and 3), allocated per sweep
  if (!ctx->UBv.p) b += 2 * nS * 5 * n2 + 2 * nS * 5 * n2 + S + 2 * nS * 15 * n2 + 8 + 6 * (size_t)grid_for(nE * n3) +
                        (nS * n2 + 127) / 128 + nE;
  if (!ctx->W.p) b += 2 * S;
  *bytes = b * sizeof(double);
  return DG_OK;
}

int dg_adjoint_forward(dg_ctx* ctx, double t0, double dt, int nSteps, const double* d_U0, double* d_U_final,
                       size_t budget_bytes, int* plan_out, void* stream) {
  if (int rc = check_ctx(ctx, true)) return rc;
  if (!d_U0 || nSteps < 1) { set_error("dg_adjoint_forward: bad argument"); return DG_ERR_ARG; }
  if (int rc = adj_setup(ctx)) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  AdjTape& T = ctx->tape;
  T.ok = false;
  T.store.release();
  const size_t S = (size_t)ctx->nElems * 5 * ctx->n3;
  const size_t bytes = S * sizeof(double);
  if (!ctx->W.p && !(ctx->W.alloc(S) && ctx->K.alloc(S))) { set_error("cudaMalloc adjoint work states"); return DG_ERR_ALLOC; }
  const size_t slots_max = budget_bytes / bytes;
  // plan 1: every stage input; plan 2: segment starts + the stage inputs of one segment (one extra
  // forward sweep; the first stage input of a segment is its start, stored once); plan 3: segment
  // starts + step starts of one segment + the stage inputs of one step (two extra forward sweeps)
  int plan = 0, k = 0, nSeg = 0;
  size_t slots = 0;
  if ((size_t)5 * nSteps <= slots_max) { plan = 1; k = nSteps; nSeg = 1; slots = (size_t)5 * nSteps; }
  else {
    size_t best = (size_t)-1; int bk = 0;
    for (int kk = 1; kk <= nSteps; ++kk) {
      const size_t need = (size_t)((nSteps + kk - 1) / kk) + (size_t)5 * kk - 1;
      if (need < best) { best = need; bk = kk; }
    }
    if (best <= slots_max) { plan = 2; k = bk; nSeg = (nSteps + bk - 1) / bk; slots = best; }
    else {
      best = (size_t)-1; bk = 0;
      for (int kk = 1; kk <= nSteps; ++kk) {
        const size_t need = (size_t)((nSteps + kk - 1) / kk) + (size_t)kk + 5;
        if (need < best) { best = need; bk = kk; }
      }
      if (best <= slots_max) { plan = 3; k = bk; nSeg = (nSteps + bk - 1) / bk; slots = best; }
    }
  }
  if (!plan) { set_error("dg_adjoint_forward: checkpoint budget too small for this window"); return DG_ERR_ALLOC; }
  if (!T.store.alloc(slots * S)) { set_error("cudaMalloc checkpoints"); return DG_ERR_ALLOC; }
  // the first segment is the short one, so that the last segment, whose checkpoints this sweep
  // records directly (the reverse sweep starts there and recomputes nothing for it), has k steps
  T.plan = plan; T.k = k; T.nSeg = nSeg; T.nSteps = nSteps; T.t0 = t0; T.dt = dt; T.state = S;
  T.r = nSteps - (nSeg - 1) * k;
  double* W = ctx->W.p;
  double* K = ctx->K.p;
  double* buf = T.store.p + (size_t)nSeg * S;  // plans 2 and 3: the buffer of one segment
  const int nL = T.seg_start(nSeg - 1);
  CUDA_TRY(cudaMemcpyAsync(W, d_U0, bytes, cudaMemcpyDeviceToDevice, st), "copy U0");
  CUDA_TRY(cudaMemsetAsync(K, 0, bytes, st), "clear K");
  for (int nstep = 0; nstep < nSteps; ++nstep) {
    const int sg = T.seg_of(nstep);
    if (plan != 1 && nstep == T.seg_start(sg))
      CUDA_TRY(cudaMemcpyAsync(T.store.p + (size_t)sg * S, W, bytes, cudaMemcpyDeviceToDevice, st), "checkpoint");
    if (plan == 3 && nstep >= nL)
      CUDA_TRY(cudaMemcpyAsync(buf + (size_t)(nstep - nL) * S, W, bytes, cudaMemcpyDeviceToDevice, st), "step start");
    for (int stage = 1; stage <= 5; ++stage) {
      double* slot = nullptr;
      if (plan == 1) slot = T.store.p + ((size_t)nstep * 5 + stage - 1) * S;
      else if (plan == 2 && nstep >= nL && (nstep > nL || stage > 1)) slot = T.p2_input(nSeg - 1, nstep, stage, buf);
      else if (plan == 3 && nstep == nSteps - 1) slot = buf + ((size_t)k + stage - 1) * S;
      if (slot) CUDA_TRY(cudaMemcpyAsync(slot, W, bytes, cudaMemcpyDeviceToDevice, st), "stage checkpoint");
      if (int rc = fwd_stage(ctx, stage, dt, W, K, st)) return rc;
    }
  }
  if (d_U_final) CUDA_TRY(cudaMemcpyAsync(d_U_final, W, bytes, cudaMemcpyDeviceToDevice, st), "copy U_final");
  T.ok = true;
  if (plan_out) *plan_out = plan;
  return DG_OK;
}

int dg_adjoint_reverse(dg_ctx* ctx, double* d_Ubar, double* mu_bar, void* stream) {
  if (int rc = check_ctx(ctx, true)) return rc;
  if (!d_Ubar) { set_error("dg_adjoint_reverse: null argument"); return DG_ERR_ARG; }
  AdjTape& T = ctx->tape;
  if (!T.ok) { set_error("dg_adjoint_reverse: no recorded forward window (dg_adjoint_forward)"); return DG_ERR_ARG; }
  cudaStream_t st = (cudaStream_t)stream;
  const size_t S = T.state, bytes = S * sizeof(double);
  double* Kbar = ctx->K.p;  // the forward K is not needed any more; reused for K_bar
  double* W = ctx->W.p;
  // a second K for the recomputation sweeps
  gxc::DBuf<double> K2;
  if (T.plan != 1 && !K2.alloc(S)) { set_error("cudaMalloc"); return DG_ERR_ALLOC; }
  CUDA_TRY(cudaMemsetAsync(Kbar, 0, bytes, st), "clear K_bar");
  CUDA_TRY(cudaMemsetAsync(ctx->acc.p, 0, sizeof(double), st), "clear mu_bar");
  const double dt = T.dt;
  int rc = DG_OK;
  if (T.plan == 1) {
    for (int nstep = T.nSteps - 1; nstep >= 0 && rc == DG_OK; --nstep)
      for (int stage = 5; stage >= 1 && rc == DG_OK; --stage)
        rc = rev_stage(ctx, stage, dt, T.store.p + ((size_t)nstep * 5 + stage - 1) * S, d_Ubar, Kbar, st);
  } else {
    double* seg = T.store.p;
    double* buf = T.store.p + (size_t)T.nSeg * S;  // plan 2: 5k - 1 stage inputs; plan 3: k step starts + 5 stage inputs
    for (int sg = T.nSeg - 1; sg >= 0 && rc == DG_OK; --sg) {
      const int n0 = T.seg_start(sg), n1 = T.seg_end(sg);
      const bool last = sg == T.nSeg - 1;  // recorded by the forward sweep
      if (!last) {
        CUDA_TRY(cudaMemcpyAsync(W, seg + (size_t)sg * S, bytes, cudaMemcpyDeviceToDevice, st), "restore");
        CUDA_TRY(cudaMemsetAsync(K2.p, 0, bytes, st), "clear");
      }
      for (int nstep = n0; nstep < n1 && rc == DG_OK && !last; ++nstep) {
        if (T.plan == 3)
          CUDA_TRY(cudaMemcpyAsync(buf + (size_t)(nstep - n0) * S, W, bytes, cudaMemcpyDeviceToDevice, st), "step start");
        for (int stage = 1; stage <= 5 && rc == DG_OK; ++stage) {
          if (T.plan == 2 && (nstep > n0 || stage > 1))  // the segment's first input is its start
            CUDA_TRY(cudaMemcpyAsync(T.p2_input(sg, nstep, stage, buf), W, bytes, cudaMemcpyDeviceToDevice, st),
                     "stage input");
          rc = fwd_stage(ctx, stage, dt, W, K2.p, st);
        }
      }
      for (int nstep = n1 - 1; nstep >= n0 && rc == DG_OK; --nstep) {
        const double* X = nullptr;
        if (T.plan == 3) {
          double* sbuf = buf + (size_t)T.k * S;
          if (nstep != T.nSteps - 1) {  // the last step's stage inputs were recorded by the forward sweep
            CUDA_TRY(cudaMemcpyAsync(W, buf + (size_t)(nstep - n0) * S, bytes, cudaMemcpyDeviceToDevice, st),
                     "restore step");
            CUDA_TRY(cudaMemsetAsync(K2.p, 0, bytes, st), "clear");
            for (int stage = 1; stage <= 4 && rc == DG_OK; ++stage) {
              CUDA_TRY(cudaMemcpyAsync(sbuf + (size_t)(stage - 1) * S, W, bytes, cudaMemcpyDeviceToDevice, st),
                       "stage input");
              rc = fwd_stage(ctx, stage, dt, W, K2.p, st);
            }
            CUDA_TRY(cudaMemcpyAsync(sbuf + (size_t)4 * S, W, bytes, cudaMemcpyDeviceToDevice, st), "stage input");
          }
          for (int stage = 5; stage >= 1 && rc == DG_OK; --stage)
            rc = rev_stage(ctx, stage, dt, sbuf + (size_t)(stage - 1) * S, d_Ubar, Kbar, st);
          continue;
        }
        for (int stage = 5; stage >= 1 && rc == DG_OK; --stage) {
          X = T.p2_input(sg, nstep, stage, buf);
          rc = rev_stage(ctx, stage, dt, X, d_Ubar, Kbar, st);
        }
      }
    }
  }
  if (rc != DG_OK) return rc;
  if (mu_bar) {
    CUDA_TRY(cudaMemcpyAsync(mu_bar, ctx->acc.p, sizeof(double), cudaMemcpyDeviceToHost, st), "read mu_bar");
    CUDA_TRY(cudaStreamSynchronize(st), "sync");
  }
  T.ok = false;  // the window's K was overwritten; record again before the next reverse sweep
  return DG_OK;
}

int dg_adjoint_window(dg_ctx* ctx, double t0, double dt, int nSteps, const double* d_U0, size_t budget_bytes,
                      double* J, double* d_dJdU0, double* dJdmu, double* d_U_final, void* stream) {
  if (int rc = check_ctx(ctx, true)) return rc;
  if (!d_U0 || !J || !d_dJdU0) { set_error("dg_adjoint_window: null argument"); return DG_ERR_ARG; }
  cudaStream_t st = (cudaStream_t)stream;
  if (int rc = dg_adjoint_forward(ctx, t0, dt, nSteps, d_U0, d_U_final, budget_bytes, nullptr, stream)) return rc;
  if (int rc = dg_kinetic_energy(ctx, ctx->W.p, J, d_dJdU0, stream)) return rc;
  (void)st;
  return dg_adjoint_reverse(ctx, d_dJdU0, dJdmu, stream);
}

}  // extern "C"
