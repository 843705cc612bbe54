// Internal definition of the operator context, shared by the C-ABI translation unit and the
// per-degree kernel translation units (dg_np*.cu, one per N+1 so they compile in parallel).
#pragma once
#include <cuda_runtime.h>
#include <string>
#include <vector>

#include "../../include/galaexi_gb300.h"
#include "dg_host.h"
#include "dg_kernels.cuh"
#include "dg_adjoint.cuh"

namespace gxc {

// device buffer, freed when it goes out of scope (or by release())
template <typename T>
struct DBuf {
  T* p = nullptr;
  size_t n = 0;
  DBuf() = default;
  DBuf(const DBuf&) = delete;
  DBuf& operator=(const DBuf&) = delete;
  ~DBuf() { release(); }
  bool alloc(size_t cnt) {
    release();
    if (cnt == 0) return true;
    if (cudaMalloc(&p, cnt * sizeof(T)) != cudaSuccess) { p = nullptr; return false; }
    n = cnt;
    return true;
  }
  void release() { if (p) cudaFree(p); p = nullptr; n = 0; }
};

// device data of one compute precision R
template <typename R>
struct PrecData {
  DBuf<R> basis;  // D, DhatT, DVS (n^2 each), Lm, Lp, Lhm, Lhp (n each)
  DBuf<R> Met, Fgeo, Pvol, Gvol, Uf, Pf, Gf, Flux;
  void release() {
    basis.release(); Met.release(); Fgeo.release(); Pvol.release(); Gvol.release();
    Uf.release(); Pf.release(); Gf.release(); Flux.release();
  }
};

template <typename R>
inline gx::DevBasis<R> dev_basis(const PrecData<R>& P, int n) {
  gx::DevBasis<R> b;
  const R* base = P.basis.p;
  b.D = base;
  b.DhatT = base + n * n;
  b.DVS = base + 2 * n * n;
  b.Lm = base + 3 * n * n;
  b.Lp = b.Lm + n;
  b.Lhm = b.Lp + n;
  b.Lhp = b.Lhm + n;
  return b;
}

template <typename R>
inline gx::Gas<R> make_gas(const dg_config& c, double pref) {
  gx::Gas<R> g;
  g.pref = (R)pref;
  g.prefD = pref;
  g.kappaM1D = c.kappa - 1.;
  g.sRD = 1. / c.R;
  g.kappa = (R)c.kappa;
  g.kappaM1 = (R)(c.kappa - 1.);
  g.sKappaM1 = (R)(1. / (c.kappa - 1.));
  g.R_gas = (R)c.R;
  g.sR = (R)(1. / c.R);
  g.mu = (R)c.mu0;
  g.lambda = (R)(c.mu0 * c.R * c.kappa / ((c.kappa - 1.) * c.Pr));  // THERMAL_CONDUCTIVITY_EOS (eos.h:110)
  return g;
}

}  // namespace gxc

// recorded forward window of the adjoint (checkpoints of dg_adjoint_forward)
struct AdjTape {
  int plan = 0;                 // 1: all stage inputs, 2: segment starts + stage inputs of one segment,
                                // 3: segment starts + step starts of one segment + stage inputs of one step
  int nSteps = 0, k = 0, nSeg = 0;
  int r = 0;                    // steps of the first segment (1..k); the other segments have k steps
  double t0 = 0., dt = 0.;
  gxc::DBuf<double> store;      // checkpoint slots, each one state
  size_t state = 0;             // doubles per state
  bool ok = false;
  int seg_of(int nstep) const { return nstep < r ? 0 : 1 + (nstep - r) / k; }
  int seg_start(int sg) const { return sg == 0 ? 0 : r + (sg - 1) * k; }
  int seg_end(int sg) const { return sg == nSeg - 1 ? nSteps : seg_start(sg + 1); }
  // plan 2: the slot of the input of `stage` of step `nstep` in segment sg; the segment's first input
  // is its start checkpoint, the others fill the segment buffer `buf` (5 k - 1 slots)
  double* p2_input(int sg, int nstep, int stage, double* buf) const {
    const size_t j = (size_t)(nstep - seg_start(sg)) * 5 + stage - 1;
    return j == 0 ? store.p + (size_t)sg * state : buf + (j - 1) * state;
  }
};

struct dg_ctx {
  dg_config cfg;
  int N = 0, n = 0, n2 = 0, n3 = 0;
  int nElems = 0, nSides = 0, nBCSides = 0;
  // boundary sides (the first nBCSides sides): BC type and 0-based reference state per side, and
  // the reference states [state][6] in FP64 and FP32
  gxc::DBuf<int> bctype, bcstate;
  gxc::DBuf<double> bcref_d;
  gxc::DBuf<float> bcref_f;
  gxc::DBuf<gx::Dual<1>> bcref_t;  // the reference states for the tangent-linear kernels (zero tangents)
  bool bc_ok = false;
  gxh::Basis1D B;
  gxc::PrecData<double> d;
  gxc::PrecData<float> f;
  gxc::DBuf<double> MetD;  // FP64 packed metrics [e][10][n3] for the CFL reduction (mixed form only)
  const double* metd = nullptr;  // FP64 packed metrics: d.Met in the FP64 form, MetD in the mixed form
  gxc::DBuf<double> cflm;  // [e][6][n3]: MetricsAdv(1:3), MetricsVisc(1:3) (InitCalctimestep)
  gxc::DBuf<int> E2S;      // [e][6][2]: 0-based side, flip
  gxc::DBuf<double> red;   // dt reduction result (2)
  gxc::DBuf<unsigned long long> bad;
  gxc::DBuf<int> kerr;     // set by a kernel whose bounded wait ran out (read by the synchronising calls)
  long long launches = 0;
  int lines_grid = 0;      // blocks of the persistent line volume kernel (SMs x resident blocks), on first use
  int prolong_grid = 0;    // blocks of the persistent prolongation kernel of the mixed form, on first use
  gxc::DBuf<int> S2E;      // [side][5]: master elem, master local side, slave elem, slave local side, flip (0-based)
  gxc::DBuf<double> wq;    // 1D quadrature weights (n)
  // tangent-linear operator (R = S = Dual<1>), set up on first use
  gxc::PrecData<gx::Dual<1>> t;
  gxc::DBuf<gx::Dual<1>> Ud, Utd;
  bool t_ok = false;
  // adjoint scratch, set up on first use
  gxc::DBuf<double> UfB, GfB, JB, UBv, part, acc, W, K;
  AdjTape tape;
  bool mesh_ok = false;
  bool grad_ok = false;    // Gvol holds the lifted gradients of the last RHS evaluation
  bool grad_rho = false;   // ... including the density gradient (the operator itself skips it)
  double pref = 0.;       // reference pressure of the mixed form (dg_set_pressure_offset)
  // solution filter (FilterType > 0): FilterMat (n x n); LAF: per-element state [5][nElems] followed
  // by the normalised integration weights [e][n3], and normMod
  gxc::DBuf<double> filt, laf;
  double laf_norm = 0.;
};

namespace gxc {

inline gx::Launch make_launch(const dg_ctx* ctx) {
  gx::Launch L;
  L.nElems = ctx->nElems;
  L.nSides = ctx->nSides;
  L.gauss = ctx->cfg.node_type == DG_NODETYPE_GAUSS ? 1 : 0;
  L.riemann = ctx->cfg.riemann;
  L.split = ctx->cfg.split_dg;
  L.parabolic = ctx->cfg.parabolic;
  L.lift_mode = ctx->cfg.do_weak_lifting ? 2 : (ctx->cfg.do_conservative_lifting ? 1 : 0);
  L.br2 = ctx->cfg.lifting == DG_LIFTING_BR2 ? 1 : 0;
  L.eta_br2 = ctx->cfg.eta_br2;
  L.nBCSides = ctx->nBCSides;
  L.bctype = ctx->bctype.p;
  L.bcstate = ctx->bcstate.p;
  L.bcref = ctx->cfg.precision == DG_PRECISION_FP64 ? (const void*)ctx->bcref_d.p : (const void*)ctx->bcref_f.p;
  return L;
}

// entry points of one per-degree translation unit
struct NPTable {
  int (*configure_d)();
  int (*configure_f)();
  int (*rhs_d)(dg_ctx*, const double* U, gx::RKArgs rk, int rkmode, cudaStream_t st);
  int (*rhs_f)(dg_ctx*, const double* U, gx::RKArgs rk, int rkmode, cudaStream_t st);
  int (*cfl)(dg_ctx*, const double* U, double cflS, double dflS, double kpr, cudaStream_t st);
  // one RK-mode stage with an event recorded after each kernel (ev[0..4]); lift may be skipped
  int (*stage_events)(dg_ctx*, double* U, gx::RKArgs rk, cudaStream_t st, cudaEvent_t* ev);
  // tangent-linear operator: the forward kernels on Dual<1> state and data
  int (*configure_t)();
  int (*rhs_t)(dg_ctx*, const gx::Dual<1>* U, gx::RKArgsT<gx::Dual<1>> rk, int rkmode, double mu_dot, cudaStream_t st);
  // adjoint of one RHS evaluation at U with cotangent source cs; mode 0: Uout = dR^T Ut_bar,
  // mode 1: reverse LSERK stage on (Ubar, Kbar); adds <Ut_bar, dR/dmu> to *acc (device)
  int (*configure_a)();
  int (*adj)(dg_ctx*, const double* U, gx::CotSrc cs, int mode, double* Uout, double* Ubar, double* Kbar,
             double b_dt, double mRKA, double* acc, cudaStream_t st);
  // the full lifting of the stored primitive state of the last operator call (with the density gradient)
  int (*relift)(dg_ctx*, cudaStream_t st);
};

}  // namespace gxc

#define GX_DECLARE_NP(NPV) extern const gxc::NPTable gx_np_table_##NPV;
GX_DECLARE_NP(2)
GX_DECLARE_NP(3)
GX_DECLARE_NP(4)
GX_DECLARE_NP(5)
GX_DECLARE_NP(6)
GX_DECLARE_NP(7)
GX_DECLARE_NP(8)
GX_DECLARE_NP(9)
GX_DECLARE_NP(10)
#undef GX_DECLARE_NP
