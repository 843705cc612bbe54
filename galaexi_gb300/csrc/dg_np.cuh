// Launch code for one compile-time node count NP = N+1.  Each dg_np<NP>.cu includes this file
// with GX_NP defined, so the kernels of every degree compile in their own translation unit.
#pragma once
#include "dg_ctx.h"

#ifndef GX_NP
#error "define GX_NP before including dg_np.cuh"
#endif

namespace {

using gxc::PrecData;

#define GX_CUDA_TRY(call, what)                                                   \
  do {                                                                            \
    cudaError_t _e = (call);                                                      \
    if (_e != cudaSuccess) {                                                      \
      gxh::set_error(std::string(what) + ": " + cudaGetErrorString(_e));         \
      return DG_ERR_CUDA;                                                         \
    }                                                                             \
  } while (0)

constexpr int NP = GX_NP;
constexpr int EPB = gx::EPBof<NP>::v;
constexpr int NT = EPB * NP * NP * NP;  // threads per element block

template <typename R, int SPL> constexpr size_t volume_smem() {
  return sizeof(R) * (size_t)EPB * (SPL >= 0 ? 19 + 15 : 15) * NP * NP * NP;
}
template <typename R> constexpr size_t lift_smem() { return sizeof(R) * (size_t)EPB * 20 * NP * NP * NP; }

// opt-in shared memory per block of the current device (227 KB on GB300)
int smem_limit() {
  int dev = 0, lim = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  if (cudaDeviceGetAttribute(&lim, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) return 0;
  return lim;
}

template <typename R, int SPL>
bool vol_fits() {
  return volume_smem<R, SPL>() + sizeof(gx::SBasis<NP, R>) <= (size_t)smem_limit();
}

template <typename R, int SPL, int PAR>
int cfg_vol() {
  if (!vol_fits<R, SPL>()) return DG_OK;  // variant not runnable on this device; rejected at launch
  GX_CUDA_TRY(cudaFuncSetAttribute(gx::k_volume<NP, R, SPL, PAR>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)volume_smem<R, SPL>()),
              "k_volume shared-memory attribute");
  return DG_OK;
}

template <typename R>
int configure() {
  GX_CUDA_TRY(cudaFuncSetAttribute(gx::k_lift<NP, R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)lift_smem<R>()),
              "k_lift shared-memory attribute");
  int rc = cfg_vol<R, -1, 0>() | cfg_vol<R, -1, 1>();
  if constexpr (NP >= 3) {
    rc |= cfg_vol<R, 0, 0>() | cfg_vol<R, 0, 1>() | cfg_vol<R, 1, 0>() | cfg_vol<R, 1, 1>() | cfg_vol<R, 2, 0>() |
          cfg_vol<R, 2, 1>() | cfg_vol<R, 3, 0>() | cfg_vol<R, 3, 1>() | cfg_vol<R, 4, 0>() | cfg_vol<R, 4, 1>();
  }
  return rc ? DG_ERR_CUDA : DG_OK;
}

template <typename R, int SPL>
int vol(dg_ctx* ctx, PrecData<R>& P, const double* U, gx::RKArgs rk, int rkmode, cudaStream_t st) {
  if (!vol_fits<R, SPL>()) {
    gxh::set_error("this N / precision / form needs more shared memory per block than the device offers");
    return DG_ERR_UNSUPPORTED;
  }
  const int grid = (ctx->nElems + EPB - 1) / EPB;
  const gx::DevBasis<R> b = gxc::dev_basis(P, NP);
  const gx::Gas<R> gas = gxc::make_gas<R>(ctx->cfg, ctx->cfg.precision == DG_PRECISION_MIXED ? ctx->pref : 0.);
  const gx::Launch L = gxc::make_launch(ctx);
  if (ctx->cfg.parabolic)
    gx::k_volume<NP, R, SPL, 1><<<grid, NT, volume_smem<R, SPL>(), st>>>(U, P.Pvol.p, P.Gvol.p, P.Met.p, P.Flux.p,
                                                                     ctx->E2S.p, b, gas, L, rk, rkmode);
  else
    gx::k_volume<NP, R, SPL, 0><<<grid, NT, volume_smem<R, SPL>(), st>>>(U, P.Pvol.p, P.Gvol.p, P.Met.p, P.Flux.p,
                                                                     ctx->E2S.p, b, gas, L, rk, rkmode);
  return DG_OK;
}

template <typename R>
int rhs(dg_ctx* ctx, PrecData<R>& P, const double* U, gx::RKArgs rk, int rkmode, cudaStream_t st,
        cudaEvent_t* ev = nullptr) {
  const int grid = (ctx->nElems + EPB - 1) / EPB;
  if (ev) cudaEventRecord(ev[0], st);
  const gx::Launch L = gxc::make_launch(ctx);
  const gx::DevBasis<R> b = gxc::dev_basis(P, NP);
  const gx::Gas<R> gas = gxc::make_gas<R>(ctx->cfg, ctx->cfg.precision == DG_PRECISION_MIXED ? ctx->pref : 0.);
  const gx::DevBasis<double> bd = gxc::dev_basis(ctx->d, NP);  // FP64 face interpolation in both forms
  gx::k_prolong<NP, R><<<grid, NT, 0, st>>>(U, ctx->E2S.p, bd.Lm, bd.Lp, gas, L, P.Pvol.p, P.Uf.p, P.Pf.p);
  ctx->launches++;
  if (ev) cudaEventRecord(ev[1], st);
  if (ctx->cfg.parabolic) {
    gx::k_lift<NP, R><<<grid, NT, lift_smem<R>(), st>>>(P.Pvol.p, P.Met.p, P.Pf.p, P.Fgeo.p, ctx->E2S.p, b, L,
                                                        P.Gvol.p, P.Gf.p);
    ctx->launches++;
  }
  if (ev) cudaEventRecord(ev[2], st);
  {
    const long long nt = (long long)ctx->nSides * NP * NP;
    const int fgrid = (int)((nt + 255) / 256);
    gx::k_face<R><<<fgrid, 256, 0, st>>>(P.Uf.p, P.Pf.p, P.Gf.p, P.Fgeo.p, gas, L, NP * NP, P.Flux.p);
    ctx->launches++;
  }
  if (ev) cudaEventRecord(ev[3], st);
  int vrc = DG_OK;
  switch (ctx->cfg.split_dg) {
    case DG_SPLIT_NONE: vrc = vol<R, -1>(ctx, P, U, rk, rkmode, st); break;
    default:
      if constexpr (NP >= 3) {
        switch (ctx->cfg.split_dg) {
          case DG_SPLIT_SD: vrc = vol<R, 0>(ctx, P, U, rk, rkmode, st); break;
          case DG_SPLIT_MO: vrc = vol<R, 1>(ctx, P, U, rk, rkmode, st); break;
          case DG_SPLIT_DU: vrc = vol<R, 2>(ctx, P, U, rk, rkmode, st); break;
          case DG_SPLIT_KG: vrc = vol<R, 3>(ctx, P, U, rk, rkmode, st); break;
          default: vrc = vol<R, 4>(ctx, P, U, rk, rkmode, st); break;
        }
      } else {
        gxh::set_error("split form needs N >= 2");
        return DG_ERR_UNSUPPORTED;
      }
  }
  if (vrc != DG_OK) return vrc;
  ctx->launches++;
  if (ev) cudaEventRecord(ev[4], st);
  GX_CUDA_TRY(cudaGetLastError(), "kernel launch");
  return DG_OK;
}

int rhs_d(dg_ctx* ctx, const double* U, gx::RKArgs rk, int rkmode, cudaStream_t st) { return rhs<double>(ctx, ctx->d, U, rk, rkmode, st); }
int rhs_f(dg_ctx* ctx, const double* U, gx::RKArgs rk, int rkmode, cudaStream_t st) { return rhs<float>(ctx, ctx->f, U, rk, rkmode, st); }

int stage_events(dg_ctx* ctx, double* U, gx::RKArgs rk, cudaStream_t st, cudaEvent_t* ev) {
  return ctx->cfg.precision == DG_PRECISION_FP64 ? rhs<double>(ctx, ctx->d, U, rk, 1, st, ev)
                                                 : rhs<float>(ctx, ctx->f, U, rk, 1, st, ev);
}

int cfl(dg_ctx* ctx, const double* U, double cflS, double dflS, double kpr, cudaStream_t st) {
  const int threads = ((NP * NP * NP + 31) / 32) * 32;
  gx::k_cfl<NP><<<ctx->nElems, threads, 0, st>>>(U, ctx->MetD.p, ctx->nElems, ctx->cfg.kappa, ctx->cfg.mu0,
                                                 ctx->cfg.parabolic, kpr, cflS, dflS, ctx->red.p, ctx->bad.p);
  ctx->launches++;
  GX_CUDA_TRY(cudaGetLastError(), "k_cfl launch");
  return DG_OK;
}

}  // namespace

#define GX_CAT2(a, b) a##b
#define GX_CAT(a, b) GX_CAT2(a, b)
extern const gxc::NPTable GX_CAT(gx_np_table_, GX_NP) = {configure<double>, configure<float>, rhs_d, rhs_f, cfl, stage_events};
