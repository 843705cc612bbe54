// Launch code for one compile-time node count NP = N+1.  Each dg_np<NP>.cu includes this file
// with GX_NP defined, so the kernels of every degree compile in their own translation unit.
#pragma once
#include "dg_ctx.h"
#include <type_traits>

#include "dg_filter.cuh"

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

template <typename R, int SPL, int PAR> constexpr size_t volume_smem() {
  return sizeof(R) * (size_t)EPB * (gx::vol_stage_slots<NP, R>(SPL, PAR) + (SPL >= 0 ? 15 * gx::vol_line_threads<NP, R>() : 0)) *
         NP * NP * NP;
}
template <typename R> constexpr size_t lift_smem() {
  return sizeof(R) * (size_t)EPB * (gx::lift_ps_slots(NP) + 15 * NP * NP * NP);
}

// opt-in shared memory per block of the current device (227 KB on GB300)
int smem_limit() {
  int dev = 0, lim = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  if (cudaDeviceGetAttribute(&lim, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) return 0;
  return lim;
}

template <typename R, int SPL, int PAR>
bool vol_fits() {
  return volume_smem<R, SPL, PAR>() + sizeof(gx::SBasis<NP, R>) <= (size_t)smem_limit();
}

template <typename R, int SPL, int PAR, typename S = double>
int cfg_vol() {
  if (!vol_fits<R, SPL, PAR>()) return DG_OK;  // variant not runnable on this device; rejected at launch
  GX_CUDA_TRY(cudaFuncSetAttribute(gx::k_volume<NP, R, SPL, PAR, S>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)volume_smem<R, SPL, PAR>()),
              "k_volume shared-memory attribute");
  // the largest shared-memory carve-out, so that two blocks share an SM where their staging fits
  GX_CUDA_TRY(cudaFuncSetAttribute(gx::k_volume<NP, R, SPL, PAR, S>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                   100),
              "k_volume carve-out attribute");
  return DG_OK;
}
// the line-per-thread volume kernel of the mixed split form
template <typename R, int SPL>
int cfg_lines() {
  if constexpr (gx::UseLines<NP, R, SPL>::v) {
    const int b = (int)gx::VolLinesSmem<NP>::bytes;
    GX_CUDA_TRY(cudaFuncSetAttribute(gx::k_volume_lines<NP, SPL, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, b),
                "k_volume_lines shared-memory attribute");
    GX_CUDA_TRY(cudaFuncSetAttribute(gx::k_volume_lines<NP, SPL, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, b),
                "k_volume_lines shared-memory attribute");
    GX_CUDA_TRY(cudaFuncSetAttribute(gx::k_volume_lines<NP, SPL, 0>, cudaFuncAttributePreferredSharedMemoryCarveout, 100),
                "k_volume_lines carve-out attribute");
    GX_CUDA_TRY(cudaFuncSetAttribute(gx::k_volume_lines<NP, SPL, 1>, cudaFuncAttributePreferredSharedMemoryCarveout, 100),
                "k_volume_lines carve-out attribute");
  }
  return DG_OK;
}
template <typename R>
int cfg_lift_lines() {
  if constexpr (gx::UseLiftLines<NP, R>::v)
    GX_CUDA_TRY(cudaFuncSetAttribute(gx::k_lift_lines<NP>, cudaFuncAttributePreferredSharedMemoryCarveout, 100),
                "k_lift_lines carve-out attribute");
  return DG_OK;
}

template <typename R>
int configure() {
  GX_CUDA_TRY(cudaFuncSetAttribute(gx::k_lift<NP, R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)lift_smem<R>()),
              "k_lift shared-memory attribute");
  GX_CUDA_TRY(cudaFuncSetAttribute(gx::k_lift<NP, R, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)lift_smem<R>()),
              "k_lift shared-memory attribute");
  // the largest shared-memory carve-out: at least two lifting blocks per SM
  GX_CUDA_TRY(cudaFuncSetAttribute(gx::k_lift<NP, R>, cudaFuncAttributePreferredSharedMemoryCarveout, 100),
              "k_lift carve-out attribute");
  GX_CUDA_TRY(cudaFuncSetAttribute(gx::k_lift<NP, R, 1>, cudaFuncAttributePreferredSharedMemoryCarveout, 100),
              "k_lift carve-out attribute");
  int rc = cfg_vol<R, -1, 0>() | cfg_vol<R, -1, 1>() | cfg_lift_lines<R>();
  if constexpr (NP >= 3) {
    rc |= cfg_vol<R, 0, 0>() | cfg_vol<R, 0, 1>() | cfg_vol<R, 1, 0>() | cfg_vol<R, 1, 1>() | cfg_vol<R, 2, 0>() |
          cfg_vol<R, 2, 1>() | cfg_vol<R, 3, 0>() | cfg_vol<R, 3, 1>() | cfg_vol<R, 4, 0>() | cfg_vol<R, 4, 1>();
    rc |= cfg_lines<R, 0>() | cfg_lines<R, 3>() | cfg_lines<R, 4>();
  }
  return rc ? DG_ERR_CUDA : DG_OK;
}

template <typename R, int SPL, typename S = double>
int vol(dg_ctx* ctx, PrecData<R>& P, const S* U, gx::RKArgsT<S> rk, int rkmode, const gx::Gas<R>& gas,
        cudaStream_t st) {
  if constexpr (SPL >= 0 && gx::UseLines<NP, R, SPL>::v && std::is_same<S, double>::value) {
    // mixed split form: one thread per 1D line (k_volume_lines)
    gx::LineBasis<NP> lb;
    const float scale = SPL == DG_SPLIT_PI ? 0.125f : 1.f;  // PI: the 1/8 of the pair flux (exact scaling)
    for (int t = 0; t < NP * NP; ++t) {
      lb.dvs[t] = (float)ctx->B.DVS[t] * scale;
      lb.dht[t] = (float)ctx->B.DhatT[t];
    }
    lb.lhm0 = (float)ctx->B.Lhm[0];
    lb.lhpN = (float)ctx->B.Lhp[NP - 1];
    const size_t sm = gx::VolLinesSmem<NP>::bytes;
    auto kern = ctx->cfg.parabolic ? gx::k_volume_lines<NP, SPL, 1> : gx::k_volume_lines<NP, SPL, 0>;
    if (ctx->lines_grid == 0) {
      // persistent: every SM holds as many blocks as fit, each walks its share of the elements
      int dev = 0, nsm = 0, occ = 0;
      GX_CUDA_TRY(cudaGetDevice(&dev), "cudaGetDevice");
      GX_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev), "SM count");
      GX_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, 3 * NP * NP, sm),
                  "k_volume_lines occupancy");
      if (occ < 1) {
        gxh::set_error("k_volume_lines does not fit an SM");
        return DG_ERR_UNSUPPORTED;
      }
      ctx->lines_grid = nsm * occ;
    }
    const int grid = ctx->nElems < ctx->lines_grid ? ctx->nElems : ctx->lines_grid;
    kern<<<grid, 3 * NP * NP, sm, st>>>(P.Pvol.p, P.Gvol.p, P.Met.p, P.Flux.p, ctx->E2S.p, lb, gas, ctx->nElems, rk.Ut,
                                        rk.U, rk.Ut_tmp, rk.mRKA, rk.b_dt, rkmode, ctx->kerr.p);
    return DG_OK;
  }
  if (ctx->cfg.parabolic ? !vol_fits<R, SPL, 1>() : !vol_fits<R, SPL, 0>()) {
    gxh::set_error("this N / precision / form needs more shared memory per block than the device offers");
    return DG_ERR_UNSUPPORTED;
  }
  const int grid = (ctx->nElems + EPB - 1) / EPB;
  const gx::DevBasis<R> b = gxc::dev_basis(P, NP);
  const gx::Launch L = gxc::make_launch(ctx);
  if (ctx->cfg.parabolic)
    gx::k_volume<NP, R, SPL, 1, S><<<grid, NT, volume_smem<R, SPL, 1>(), st>>>(U, P.Pvol.p, P.Gvol.p, P.Met.p,
                                                                           P.Flux.p, ctx->E2S.p, b, gas, L, rk, rkmode);
  else
    gx::k_volume<NP, R, SPL, 0, S><<<grid, NT, volume_smem<R, SPL, 0>(), st>>>(U, P.Pvol.p, P.Gvol.p, P.Met.p,
                                                                           P.Flux.p, ctx->E2S.p, b, gas, L, rk, rkmode);
  return DG_OK;
}

// forward kernels up to (and excluding) the volume kernel: prims + face traces, lifting, face fluxes;
// V0 = 1 lifts without the density gradient (no flux reads it; dg_get_gradients completes it)
template <typename R, typename S = double, int V0 = 0>
void rhs_front(dg_ctx* ctx, PrecData<R>& P, const S* U, const gx::Gas<R>& gas, cudaStream_t st, cudaEvent_t* ev,
               bool face) {
  const int grid = (ctx->nElems + EPB - 1) / EPB;
  gx::Launch L = gxc::make_launch(ctx);
  if constexpr (std::is_same<R, gx::Dual<1>>::value) L.bcref = ctx->bcref_t.p;  // boundary states, zero tangents
  const gx::DevBasis<R> b = gxc::dev_basis(P, NP);
  const gx::DevBasis<double> bd = gxc::dev_basis(ctx->d, NP);  // FP64 face interpolation in every form
  bool persistent = false;
  if constexpr (gx::UseProlongGL<NP, R, S>::v) {
    if (!L.gauss) {
      // mixed form on Gauss-Lobatto nodes: persistent, with the next element's state in flight
      constexpr size_t sm = gx::ProlongGLSmem<NP>::bytes;
      if (ctx->prolong_grid == 0) {
        int dev = 0, nsm = 0, occ = 0;
        if (cudaGetDevice(&dev) == cudaSuccess &&
            cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess &&
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, gx::k_prolong_gl<NP>, NP * NP * NP, sm) == cudaSuccess &&
            occ > 0)
          ctx->prolong_grid = nsm * occ;
        else
          ctx->prolong_grid = ctx->nElems;  // one element per block
      }
      const int pg = ctx->nElems < ctx->prolong_grid ? ctx->nElems : ctx->prolong_grid;
      gx::k_prolong_gl<NP><<<pg, NP * NP * NP, sm, st>>>(U, ctx->E2S.p, gas, ctx->nElems, ctx->nSides, P.Pvol.p,
                                                          P.Uf.p, P.Pf.p, ctx->kerr.p);
      persistent = true;
    }
  }
  if (!persistent)
    gx::k_prolong<NP, R, S><<<grid, NT, 0, st>>>(U, ctx->E2S.p, bd.Lm, bd.Lp, gas, L, P.Pvol.p, P.Uf.p, P.Pf.p);
  ctx->launches++;
  const long long nbc = (long long)ctx->nBCSides * NP * NP;
  if (ctx->cfg.parabolic && nbc > 0) {
    gx::k_bc_lift_ghost<R><<<(int)((nbc + 255) / 256), 256, 0, st>>>(P.Pf.p, P.Fgeo.p, gas, L, NP * NP);
    ctx->launches++;
  }
  if (ev) cudaEventRecord(ev[1], st);
  if (ctx->cfg.parabolic) {
    bool lines = false;
    if constexpr (gx::UseLiftLines<NP, R>::v && V0 == 1 && std::is_same<S, double>::value) {
      // mixed form, Gauss-Lobatto BR1 in strong non-conservative form: one thread per 1D line
      if (!L.gauss && !L.br2 && L.lift_mode == 0) {
        gx::LiftBasis<NP> lb;
        for (int t = 0; t < NP * NP; ++t) lb.D[t] = (float)ctx->B.D[t];
        lb.lhm0 = (float)ctx->B.Lhm[0];
        lb.lhpN = (float)ctx->B.Lhp[NP - 1];
        gx::k_lift_lines<NP><<<ctx->nElems, 3 * NP * NP, 0, st>>>(P.Pvol.p, P.Met.p, P.Pf.p, P.Fgeo.p, ctx->E2S.p, lb,
                                                                  ctx->nElems, ctx->nSides, P.Gvol.p, P.Gf.p);
        lines = true;
      }
    }
    if (!lines)
      gx::k_lift<NP, R, V0><<<grid, NT, lift_smem<R>(), st>>>(P.Pvol.p, P.Met.p, P.Pf.p, P.Fgeo.p, ctx->E2S.p, b, L,
                                                              P.Gvol.p, P.Gf.p);
    ctx->launches++;
  }
  if (ev) cudaEventRecord(ev[2], st);
  if (face) {
    const long long nt = (long long)(ctx->nSides - ctx->nBCSides) * NP * NP;
    if (nt > 0) {
      gx::k_face<R><<<(int)((nt + 127) / 128), 128, 0, st>>>(P.Uf.p, P.Pf.p, P.Gf.p, P.Fgeo.p, gas, L, NP * NP,
                                                               P.Flux.p);
      ctx->launches++;
    }
    if (nbc > 0) {
      gx::k_bc_face<R><<<(int)((nbc + 255) / 256), 256, 0, st>>>(P.Pf.p, P.Gf.p, P.Fgeo.p, gas, L, NP * NP, P.Flux.p);
      ctx->launches++;
    }
  }
  if (ev) cudaEventRecord(ev[3], st);
}

// step 1 of the operator: the solution filter, in place on the FP64 state (dg.f90:330)
inline void filter(dg_ctx* ctx, double* U, cudaStream_t st) {
  if (ctx->cfg.filter_type == DG_FILTER_LAF) {
    gx::LafState S{ctx->laf.p, ctx->laf.p + 5 * (size_t)ctx->nElems, ctx->cfg.laf_alpha, ctx->laf_norm};
    gx::k_filter_laf<NP><<<ctx->nElems, ((NP * NP * NP + 31) / 32) * 32, 0, st>>>(U, ctx->filt.p, ctx->nElems, S);
  } else {
    gx::k_filter<NP><<<(ctx->nElems + EPB - 1) / EPB, NT, 0, st>>>(U, ctx->filt.p, ctx->nElems);
  }
  ctx->launches++;
}

template <typename R>
int rhs(dg_ctx* ctx, PrecData<R>& P, const double* U, gx::RKArgs rk, int rkmode, cudaStream_t st,
        cudaEvent_t* ev = nullptr) {
  if (ev) cudaEventRecord(ev[0], st);
  // the reference filters its module array d_U in place; U is the caller's state array
  if (ctx->cfg.filter_type != DG_FILTER_NONE) filter(ctx, const_cast<double*>(U), st);
  const gx::Gas<R> gas = gxc::make_gas<R>(ctx->cfg, ctx->cfg.precision == DG_PRECISION_MIXED ? ctx->pref : 0.);
  rhs_front<R, double, 1>(ctx, P, U, gas, st, ev, true);
  ctx->grad_rho = false;
  int vrc = DG_OK;
  switch (ctx->cfg.split_dg) {
    case DG_SPLIT_NONE: vrc = vol<R, -1>(ctx, P, U, rk, rkmode, gas, st); break;
    default:
      if constexpr (NP >= 3) {
        switch (ctx->cfg.split_dg) {
          case DG_SPLIT_SD: vrc = vol<R, 0>(ctx, P, U, rk, rkmode, gas, st); break;
          case DG_SPLIT_MO: vrc = vol<R, 1>(ctx, P, U, rk, rkmode, gas, st); break;
          case DG_SPLIT_DU: vrc = vol<R, 2>(ctx, P, U, rk, rkmode, gas, st); break;
          case DG_SPLIT_KG: vrc = vol<R, 3>(ctx, P, U, rk, rkmode, gas, st); break;
          default: vrc = vol<R, 4>(ctx, P, U, rk, rkmode, gas, st); break;
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

// ---- tangent-linear operator: R = S = Dual<1>; mu_dot seeds the viscosity direction
using D1 = gx::Dual<1>;

int configure_t() {
  if (lift_smem<D1>() + sizeof(gx::SBasis<NP, D1>) <= (size_t)smem_limit())
    GX_CUDA_TRY(cudaFuncSetAttribute(gx::k_lift<NP, D1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)lift_smem<D1>()),
                "k_lift shared-memory attribute");
  int rc = cfg_vol<D1, -1, 0, D1>() | cfg_vol<D1, -1, 1, D1>();
  if constexpr (NP >= 3) rc |= cfg_vol<D1, 3, 0, D1>() | cfg_vol<D1, 3, 1, D1>() | cfg_vol<D1, 4, 0, D1>() | cfg_vol<D1, 4, 1, D1>();
  return rc ? DG_ERR_CUDA : DG_OK;
}

int rhs_t(dg_ctx* ctx, const D1* U, gx::RKArgsT<D1> rk, int rkmode, double mu_dot, cudaStream_t st) {
  if (ctx->cfg.parabolic && lift_smem<D1>() + sizeof(gx::SBasis<NP, D1>) > (size_t)smem_limit()) {
    gxh::set_error("tangent-linear lifting needs more shared memory per block than the device offers");
    return DG_ERR_UNSUPPORTED;
  }
  gx::Gas<D1> gas = gxc::make_gas<D1>(ctx->cfg, 0.);
  gas.mu.d[0] = mu_dot;
  gas.lambda.d[0] = mu_dot * ctx->cfg.R * ctx->cfg.kappa / ((ctx->cfg.kappa - 1.) * ctx->cfg.Pr);
  rhs_front<D1, D1>(ctx, ctx->t, U, gas, st, nullptr, true);
  int vrc = DG_OK;
  switch (ctx->cfg.split_dg) {
    case DG_SPLIT_NONE: vrc = vol<D1, -1, D1>(ctx, ctx->t, U, rk, rkmode, gas, st); break;
    case DG_SPLIT_KG:
    case DG_SPLIT_PI:
      if constexpr (NP >= 3) {
        vrc = ctx->cfg.split_dg == DG_SPLIT_KG ? vol<D1, 3, D1>(ctx, ctx->t, U, rk, rkmode, gas, st)
                                               : vol<D1, 4, D1>(ctx, ctx->t, U, rk, rkmode, gas, st);
        break;
      }
      [[fallthrough]];
    default:
      gxh::set_error("tangent-linear operator: split forms PI and KG only");
      return DG_ERR_UNSUPPORTED;
  }
  if (vrc != DG_OK) return vrc;
  ctx->launches++;
  GX_CUDA_TRY(cudaGetLastError(), "kernel launch");
  return DG_OK;
}

// ---- adjoint
constexpr size_t adj_vol_smem() { return sizeof(double) * (size_t)EPB * gx::adj_vol_words<NP>(); }
bool adj_fits() { return adj_vol_smem() + sizeof(gx::SBasis<NP, double>) <= (size_t)smem_limit(); }

template <int SPL, int PAR>
int cfg_adj() {
  if (!adj_fits()) return DG_OK;
  GX_CUDA_TRY(cudaFuncSetAttribute(gx::ka_volume<NP, SPL, PAR>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)adj_vol_smem()),
              "ka_volume shared-memory attribute");
  return DG_OK;
}

int configure_a() {
  int rc = cfg_adj<-1, 0>() | cfg_adj<-1, 1>();
  if constexpr (NP >= 3) rc |= cfg_adj<3, 0>() | cfg_adj<3, 1>() | cfg_adj<4, 0>() | cfg_adj<4, 1>();
  return rc ? DG_ERR_CUDA : DG_OK;
}

template <int SPL>
void adj_vol(dg_ctx* ctx, const double* U, gx::CotSrc cs, const gx::AdjLaunch& AL, double* part, cudaStream_t st) {
  const int grid = (ctx->nElems + EPB - 1) / EPB;
  const gx::DevBasis<double> b = gxc::dev_basis(ctx->d, NP);
  PrecData<double>& P = ctx->d;
  if (ctx->cfg.parabolic)
    gx::ka_volume<NP, SPL, 1><<<grid, NT, adj_vol_smem(), st>>>(cs, U, P.Pvol.p, P.Gvol.p, P.Met.p, P.Fgeo.p, ctx->E2S.p,
                                                               b, AL, ctx->GfB.p, ctx->UBv.p, ctx->JB.p, part);
  else
    gx::ka_volume<NP, SPL, 0><<<grid, NT, adj_vol_smem(), st>>>(cs, U, P.Pvol.p, P.Gvol.p, P.Met.p, P.Fgeo.p, ctx->E2S.p,
                                                               b, AL, ctx->GfB.p, ctx->UBv.p, ctx->JB.p, part);
}

int adj(dg_ctx* ctx, const double* U, gx::CotSrc cs, int mode, double* Uout, double* Ubar, double* Kbar, double b_dt,
        double mRKA, double* acc, cudaStream_t st) {
  if (!adj_fits()) {
    gxh::set_error("adjoint: this N needs more shared memory per block than the device offers");
    return DG_ERR_UNSUPPORTED;
  }
  const dg_config& c = ctx->cfg;
  const gx::Gas<double> gas = gxc::make_gas<double>(c, 0.);
  // the state's primitives, traces and lifted gradients (no flux reads the density gradient)
  rhs_front<double, double, 1>(ctx, ctx->d, U, gas, st, nullptr, false);
  ctx->grad_rho = false;
  gx::AdjLaunch AL;
  AL.nElems = ctx->nElems; AL.nSides = ctx->nSides;
  AL.gauss = c.node_type == DG_NODETYPE_GAUSS ? 1 : 0;
  AL.riemann = c.riemann; AL.split = c.split_dg; AL.parabolic = c.parabolic;
  AL.lift_mode = c.do_conservative_lifting ? 1 : 0;
  AL.mu = c.mu0;
  AL.lamc = c.R * c.kappa / ((c.kappa - 1.) * c.Pr);
  AL.lambda = c.mu0 * AL.lamc;
  AL.inv_mu = c.mu0 > 0. ? 1. / c.mu0 : 0.;
  AL.kappa = c.kappa; AL.sR = 1. / c.R;
  AL.nBCSides = ctx->nBCSides; AL.bctype = ctx->bctype.p; AL.bcstate = ctx->bcstate.p; AL.bcref = ctx->bcref_d.p;
  const gx::DevBasis<double> b = gxc::dev_basis(ctx->d, NP);
  const long long nf = (long long)ctx->nSides * NP * NP;
  const long long nbf = (long long)ctx->nBCSides * NP * NP;  // face nodes of the BC sides (listed first)
  const int fgrid = (int)((nf - nbf + 127) / 128);
  const int bgrid = (int)((nbf + 127) / 128);
  const int vgrid = (ctx->nElems + EPB - 1) / EPB;
  if (fgrid == 0) {
    // no connected sides: nothing for ka_face
  } else if (gx::riemann_vjp_supported_host(c.riemann, c.split_dg))
    gx::ka_face<NP, true><<<fgrid, 128, 0, st>>>(cs, ctx->d.Met.p, ctx->d.Uf.p, ctx->d.Pf.p, ctx->d.Gf.p, ctx->d.Fgeo.p,
                                                 ctx->S2E.p, b, gas, AL, ctx->UfB.p, ctx->GfB.p, ctx->part.p);
  else
    gx::ka_face<NP, false><<<fgrid, 128, 0, st>>>(cs, ctx->d.Met.p, ctx->d.Uf.p, ctx->d.Pf.p, ctx->d.Gf.p, ctx->d.Fgeo.p,
                                                  ctx->S2E.p, b, gas, AL, ctx->UfB.p, ctx->GfB.p, ctx->part.p);
  if (bgrid > 0) {
    gx::ka_bc_face<NP><<<bgrid, 128, 0, st>>>(cs, ctx->d.Met.p, ctx->d.Uf.p, ctx->d.Gf.p, ctx->d.Fgeo.p, ctx->S2E.p, b,
                                              gas, AL, ctx->UfB.p, ctx->GfB.p, ctx->part.p + fgrid + vgrid);
    ctx->launches++;
  }
  switch (c.split_dg) {
    case DG_SPLIT_NONE: adj_vol<-1>(ctx, U, cs, AL, ctx->part.p + fgrid, st); break;
    case DG_SPLIT_KG: if constexpr (NP >= 3) adj_vol<3>(ctx, U, cs, AL, ctx->part.p + fgrid, st); break;
    default: if constexpr (NP >= 3) adj_vol<4>(ctx, U, cs, AL, ctx->part.p + fgrid, st); break;
  }
  gx::k_adj_sum<<<1, 256, 0, st>>>(ctx->part.p, fgrid + vgrid + bgrid, acc);
  if (c.parabolic) {
    if (nf > nbf) {
      gx::ka_jump<<<(int)((nf - nbf + 255) / 256), 256, 0, st>>>(ctx->d.Uf.p, ctx->JB.p, AL, NP * NP, ctx->UfB.p);
      ctx->launches++;
    }
    if (nbf > 0) {
      gx::ka_bc_jump<<<(int)((nbf + 255) / 256), 256, 0, st>>>(ctx->d.Uf.p, ctx->JB.p, ctx->d.Fgeo.p, gas, AL, NP * NP,
                                                              ctx->UfB.p);
      ctx->launches++;
    }
  }
  const long long nn = (long long)ctx->nElems * NP * NP * NP;
  gx::ka_final<NP><<<(int)((nn + 255) / 256), 256, 0, st>>>(ctx->UBv.p, ctx->UfB.p, ctx->E2S.p, b, AL, mode, Uout,
                                                           Ubar, Kbar, b_dt, mRKA);
  ctx->launches += 4;
  GX_CUDA_TRY(cudaGetLastError(), "adjoint kernel launch");
  return DG_OK;
}

// the full lifting (density gradient included) of the primitive state stored by the last operator call
template <typename R>
int relift_p(dg_ctx* ctx, PrecData<R>& P, cudaStream_t st) {
  const int grid = (ctx->nElems + EPB - 1) / EPB;
  gx::k_lift<NP, R, 0><<<grid, NT, lift_smem<R>(), st>>>(P.Pvol.p, P.Met.p, P.Pf.p, P.Fgeo.p, ctx->E2S.p,
                                                         gxc::dev_basis(P, NP), gxc::make_launch(ctx), P.Gvol.p, P.Gf.p);
  ctx->launches++;
  GX_CUDA_TRY(cudaGetLastError(), "k_lift launch");
  return DG_OK;
}
int relift(dg_ctx* ctx, cudaStream_t st) {
  return ctx->cfg.precision == DG_PRECISION_FP64 ? relift_p<double>(ctx, ctx->d, st) : relift_p<float>(ctx, ctx->f, st);
}

int rhs_d(dg_ctx* ctx, const double* U, gx::RKArgs rk, int rkmode, cudaStream_t st) { return rhs<double>(ctx, ctx->d, U, rk, rkmode, st); }
int rhs_f(dg_ctx* ctx, const double* U, gx::RKArgs rk, int rkmode, cudaStream_t st) { return rhs<float>(ctx, ctx->f, U, rk, rkmode, st); }

int stage_events(dg_ctx* ctx, double* U, gx::RKArgs rk, cudaStream_t st, cudaEvent_t* ev) {
  return ctx->cfg.precision == DG_PRECISION_FP64 ? rhs<double>(ctx, ctx->d, U, rk, 1, st, ev)
                                                 : rhs<float>(ctx, ctx->f, U, rk, 1, st, ev);
}

int cfl(dg_ctx* ctx, const double* U, double cflS, double dflS, double kpr, cudaStream_t st) {
  const int threads = ((NP * NP * NP + 31) / 32) * 32;
  (void)kpr;  // folded into the precomputed MetricsVisc
  gx::k_cfl<NP><<<ctx->nElems, threads, 0, st>>>(U, ctx->metd, ctx->cflm.p, ctx->nElems, ctx->cfg.kappa,
                                                 ctx->cfg.mu0, ctx->cfg.parabolic, cflS, dflS, ctx->red.p,
                                                 ctx->bad.p);
  ctx->launches++;
  GX_CUDA_TRY(cudaGetLastError(), "k_cfl launch");
  return DG_OK;
}

}  // namespace

#define GX_CAT2(a, b) a##b
#define GX_CAT(a, b) GX_CAT2(a, b)
extern const gxc::NPTable GX_CAT(gx_np_table_, GX_NP) = {configure<double>, configure<float>, rhs_d, rhs_f, cfl,
                                                         stage_events, configure_t, rhs_t, configure_a, adj, relift};
