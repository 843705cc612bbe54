// Host-side set-up of the DGSEM operator: 1D basis, ini keys, mesh and metrics, initial states.
// These replace, for the periodic box meshes this library builds itself, the reference's
// InitInterpolation/InitDGbasis (src/interpolation/interpolation.f90:96-193, src/dg/dg.f90:181-242),
// HOPR mesh + ReadMesh + CalcMetrics (src/mesh/metrics.f90:171-789) and FillIni/ExactFunc
// (src/dg/dg.f90:432-456, idealgas/exactfunc.f90, testcase/taylorgreenvortex/testcase.f90).
#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/galaexi_gb300.h"
#include "dg_host.h"

namespace gxh {

static const double kPi = 3.141592653589793238462643383279502884197;

// ---------------------------------------------------------------------------------------------
// 1D basis
// ---------------------------------------------------------------------------------------------
// Normalised Legendre polynomial L_N and derivative by the three-term recurrence
// (the normalisation sqrt(N+1/2) is the one of basis.f90:232-233).
static void legendre(int N, double x, double& L, double& dL) {
  if (N == 0) { L = 1.; dL = 0.; }
  else if (N == 1) { L = x; dL = 1.; }
  else {
    double lm2 = 1., lm1 = x, dlm1 = 1.;
    for (int k = 2; k <= N; ++k) {
      L = ((double)(2 * k - 1) * x * lm1 - (double)(k - 1) * lm2) / (double)k;
      dL = k * lm1 + x * dlm1;
      lm2 = lm1; lm1 = L; dlm1 = dL;
    }
  }
  const double s = std::sqrt((double)N + 0.5);
  L *= s; dL *= s;
}

// Gauss nodes: roots of L_{N+1} by Newton from Chebyshev-Gauss guesses (cf. basis.f90:417-486)
static void gauss_nodes(int N, double* x, double* w) {
  if (N == 0) { x[0] = 0.; w[0] = 2.; return; }
  if (N == 1) { x[0] = -std::sqrt(1. / 3.); x[1] = -x[0]; w[0] = w[1] = 1.; return; }
  const double h = 2. * std::atan(1.) / (double)(N + 1);
  for (int i = 0; i <= (N + 1) / 2 - 1; ++i) {
    double xi = -std::cos(h * (double)(2 * i + 1)), L, dL;
    for (int it = 0; it <= 10; ++it) {
      legendre(N + 1, xi, L, dL);
      const double dx = -L / dL;
      xi += dx;
      if (std::fabs(dx) < 1.e-15 * std::fabs(xi)) break;
    }
    legendre(N + 1, xi, L, dL);
    x[i] = xi; x[N - i] = -xi;
    w[i] = w[N - i] = (2. * N + 3) / ((1. - xi * xi) * dL * dL);
  }
  if (N % 2 == 0) {
    double L, dL;
    x[N / 2] = 0.;
    legendre(N + 1, 0., L, dL);
    w[N / 2] = (2. * N + 3) / (dL * dL);
  }
}

// q = L_{N+1} - L_{N-1} (unnormalised), its derivative, and L_N (cf. basis.f90:527-556)
static void lobatto_q(int N, double x, double& q, double& dq, double& L) {
  double lm2 = 1., lm1 = x;
  L = x;
  for (int k = 2; k <= N; ++k) {
    L = ((double)(2 * k - 1) * x * lm1 - (double)(k - 1) * lm2) / (double)k;
    lm2 = lm1; lm1 = L;
  }
  q = (double)(2 * N + 1) / (double)(N + 1) * (x * L - lm2);
  dq = (double)(2 * N + 1) * L;
}

// Gauss-Lobatto nodes (cf. basis.f90:567-630)
static void lobatto_nodes(int N, double* x, double* w) {
  x[0] = -1.; x[N] = 1.;
  const double w0 = 2. / (double)(N * (N + 1));
  w[0] = w[N] = w0;
  if (N > 1) {
    const double c1 = kPi / (double)N, c2 = 3. / ((double)(8 * N) * kPi);
    for (int i = 1; i <= (N + 1) / 2 - 1; ++i) {
      double xi = -std::cos(c1 * ((double)i + 0.25) - c2 / ((double)i + 0.25)), q, dq, L;
      for (int it = 0; it <= 10; ++it) {
        lobatto_q(N, xi, q, dq, L);
        const double dx = -q / dq;
        xi += dx;
        if (std::fabs(dx) < 1.e-15 * std::fabs(xi)) break;
      }
      lobatto_q(N, xi, q, dq, L);
      x[i] = xi; x[N - i] = -xi;
      w[i] = w[N - i] = w0 / (L * L);
    }
  }
  if (N % 2 == 0) {
    double q, dq, L;
    x[N / 2] = 0.;
    lobatto_q(N, 0., q, dq, L);
    w[N / 2] = w0 / (L * L);
  }
}

static void bary_weights(int N, const double* x, double* wb) {
  for (int i = 0; i <= N; ++i) wb[i] = 1.;
  for (int i = 1; i <= N; ++i)
    for (int j = 0; j < i; ++j) {
      wb[j] *= (x[j] - x[i]);
      wb[i] *= (x[i] - x[j]);
    }
  for (int i = 0; i <= N; ++i) wb[i] = 1. / wb[i];
}

// D(i,l) = dl_l/dx(x_i), column-major, diagonal by negative row sum (cf. basis.f90:664-690)
static void diff_matrix(int N, const double* x, double* D) {
  const int n = N + 1;
  std::vector<double> wb(n);
  bary_weights(N, x, wb.data());
  for (int t = 0; t < n * n; ++t) D[t] = 0.;
  for (int l = 0; l <= N; ++l)
    for (int i = 0; i <= N; ++i)
      if (l != i) {
        D[i + n * l] = wb[l] / (wb[i] * (x[i] - x[l]));
        D[i + n * i] -= D[i + n * l];
      }
}

// Lagrange polynomials at x0 in barycentric form (cf. basis.f90:720-752)
static void lagrange_at(double x0, int N, const double* x, const double* wb, double* L) {
  const double eps = 2.220446049250313e-16;
  bool hit = false;
  for (int i = 0; i <= N; ++i) {
    L[i] = 0.;
    const double d = std::fabs(x0 - x[i]);
    const bool eq = (x0 == 0. || x[i] == 0.) ? d <= 2. * eps : (d <= eps * std::fabs(x0) && d <= eps * std::fabs(x[i]));
    if (eq) { L[i] = 1.; hit = true; }
  }
  if (hit) return;
  double s = 0.;
  for (int i = 0; i <= N; ++i) { L[i] = wb[i] / (x0 - x[i]); s += L[i]; }
  for (int i = 0; i <= N; ++i) L[i] /= s;
}

void basis_1d(int N, int node_type, Basis1D& B) {
  const int n = N + 1;
  B.N = N;
  B.x.assign(n, 0.); B.w.assign(n, 0.); B.wb.assign(n, 0.);
  if (node_type == DG_NODETYPE_GAUSS) gauss_nodes(N, B.x.data(), B.w.data());
  else if (node_type == DG_NODETYPE_GAUSS_LOBATTO) lobatto_nodes(N, B.x.data(), B.w.data());
  else {  // Chebyshev-Gauss-Lobatto (used for the metric computation)
    for (int i = 0; i <= N; ++i) B.x[i] = -std::cos(i / (double)N * kPi);
    for (int i = 0; i <= N; ++i) B.w[i] = kPi / (double)N;
    B.w[0] *= 0.5; B.w[N] *= 0.5;
  }
  bary_weights(N, B.x.data(), B.wb.data());
  B.D.assign(n * n, 0.);
  diff_matrix(N, B.x.data(), B.D.data());
  B.Lm.assign(n, 0.); B.Lp.assign(n, 0.);
  lagrange_at(-1., N, B.x.data(), B.wb.data(), B.Lm.data());
  lagrange_at(1., N, B.x.data(), B.wb.data(), B.Lp.data());
  // D_hat = -M^{-1} D^T M with M = diag(w): D_hat(i,j) = -(1/w_i) * D(j,i) * w_j ; stored transposed
  B.DhatT.assign(n * n, 0.);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) B.DhatT[j + n * i] = -((1. / B.w[i]) * (D_at(B, j, i) * B.w[j]));
  // DVolSurf = D^T with the surface terms of the strong form folded into the corners (dg.f90:228-234)
  B.DVS.assign(n * n, 0.);
  for (int l = 0; l < n; ++l)
    for (int i = 0; i < n; ++i) B.DVS[l + n * i] = D_at(B, i, l);
  B.DVS[0] += 1.0 / (2.0 * B.w[0]);
  B.DVS[N + n * N] -= 1.0 / (2.0 * B.w[N]);
  B.Lhm.assign(n, 0.); B.Lhp.assign(n, 0.);
  for (int i = 0; i < n; ++i) { B.Lhm[i] = (1. / B.w[i]) * B.Lm[i]; B.Lhp[i] = (1. / B.w[i]) * B.Lp[i]; }
}

// FilterMat of InitFilter (filter.f90:100-222): Vdm_Leg diag(sigma) sVdm_Leg with the modal
// Vandermonde of the normalised Legendre polynomials (buildLegendreVdm, basis.f90:100-160); its
// inverse by Gauss quadrature of the interpolant (the reference's VDM_ANALYTICAL branch, exact for
// N+1 Gauss points).  sigma: cut-off (1 up to NFilter) or Hesthaven's exponential filter (HestFilter,
// filter.f90:231-263).  F(i,l) column-major.
int filter_matrix(const dg_config& c, std::vector<double>& F) {
  const int N = c.N, n = N + 1;
  std::vector<double> sigma(n, 0.);
  if (c.filter_type == DG_FILTER_CUTOFF || c.filter_type == DG_FILTER_LAF) {
    if (c.n_filter < 0 || c.n_filter > N) return -1;
    for (int d = 0; d <= c.n_filter; ++d) sigma[d] = 1.;
  } else if (c.filter_type == DG_FILTER_MODAL) {
    const double alpha = c.hest_filter_param[0], s = c.hest_filter_param[1];
    const double etac = c.hest_filter_param[2] / (double)(N + 1);
    const int cut = (int)c.hest_filter_param[2];
    for (int d = 0; d <= std::min(cut - 1, N); ++d) sigma[d] = 1.;
    if (alpha >= 0.)
      for (int d = std::max(cut, 0); d <= N; ++d) {
        const double eta = (double)(d + 1) / (double)(N + 1);
        sigma[d] = std::exp(-alpha * std::pow((eta - etac) / (1. - etac), s));
      }
  } else {
    return -1;
  }
  Basis1D B, G;
  basis_1d(N, c.node_type, B);
  basis_1d(N, DG_NODETYPE_GAUSS, G);
  std::vector<double> V(n * n), sV(n * n, 0.), Vlag;
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      double L, dL;
      legendre(j, B.x[i], L, dL);
      V[i + n * j] = L;  // Vdm_Leg(i,j) = L_j(x_i)
    }
  vandermonde(N, B.x.data(), B.wb.data(), N, G.x.data(), Vlag);  // Vlag(g,i) = l_i(xGauss_g)
  for (int m = 0; m < n; ++m)
    for (int i = 0; i < n; ++i) {
      double acc = 0.;
      for (int g = 0; g < n; ++g) {
        double L, dL;
        legendre(m, G.x[g], L, dL);
        acc += L * G.w[g] * Vlag[g + n * i];
      }
      sV[m + n * i] = acc;  // sVdm_Leg(m,i)
    }
  F.assign(n * n, 0.);
  for (int i = 0; i < n; ++i)
    for (int l = 0; l < n; ++l) {
      double acc = 0.;
      for (int m = 0; m < n; ++m) acc += V[i + n * m] * sigma[m] * sV[m + n * l];
      F[i + n * l] = acc;
    }
  return 0;
}

// Modal projection from degree N on the nodes x to degree M < N on the points y: keep the Legendre
// modes 0..M of the interpolant (the modal branch of GetVandermonde, interpolation.f90:373-374,
// Vdm_Leg_Out * sVdm_Leg_In(0:M,0:N)).  The modes of the Lagrange basis come from Gauss quadrature
// with N+1 points, exact for the degree-2N products.
void modal_projection(int N, const double* x, const double* wb, int M, const double* y, std::vector<double>& V) {
  Basis1D G;
  basis_1d(N, DG_NODETYPE_GAUSS, G);
  std::vector<double> Vlag;
  vandermonde(N, x, wb, N, G.x.data(), Vlag);  // Vlag(g,i) = l_i(xGauss_g)
  std::vector<double> sV((size_t)(M + 1) * (N + 1), 0.);
  for (int m = 0; m <= M; ++m)
    for (int i = 0; i <= N; ++i) {
      double acc = 0.;
      for (int g = 0; g <= N; ++g) {
        double L, dL;
        legendre(m, G.x[g], L, dL);
        acc += L * G.w[g] * Vlag[g + (N + 1) * i];
      }
      sV[m + (M + 1) * i] = acc;
    }
  V.assign((size_t)(M + 1) * (N + 1), 0.);
  for (int o = 0; o <= M; ++o)
    for (int i = 0; i <= N; ++i) {
      double acc = 0.;
      for (int m = 0; m <= M; ++m) {
        double L, dL;
        legendre(m, y[o], L, dL);
        acc += L * sV[m + (M + 1) * i];
      }
      V[o + (M + 1) * i] = acc;
    }
}

// interpolation matrix V(i,j) = l_j(y_i) from nodes x (degree N) to points y (m+1 points)
void vandermonde(int N, const double* x, const double* wb, int M, const double* y, std::vector<double>& V) {
  V.assign((size_t)(M + 1) * (N + 1), 0.);
  std::vector<double> L(N + 1);
  for (int i = 0; i <= M; ++i) {
    lagrange_at(y[i], N, x, wb, L.data());
    for (int j = 0; j <= N; ++j) V[i + (M + 1) * j] = L[j];
  }
}

}  // namespace gxh

using namespace gxh;

// ---------------------------------------------------------------------------------------------
// thread-local last error (shared with dg_api.cu)
// ---------------------------------------------------------------------------------------------
static thread_local std::string g_last_error;
void gxh::set_error(const std::string& s) { g_last_error = s; }

extern "C" const char* dg_last_error(void) { return g_last_error.c_str(); }

extern "C" void dg_config_default(dg_config* c) {
  std::memset(c, 0, sizeof(*c));
  c->N = 3;
  c->node_type = DG_NODETYPE_GAUSS_LOBATTO;
  c->parabolic = 0;
  c->riemann = DG_RIEMANN_LF;
  c->split_dg = DG_SPLIT_NONE;
  c->lifting = DG_LIFTING_BR1;
  c->do_weak_lifting = 0;
  c->do_conservative_lifting = 0;
  c->eta_br2 = 2.;
  c->kappa = 1.4;       // idealgas/eos.f90:86
  c->R = 287.058;       // idealgas/eos.f90:87
  c->Pr = 0.72;         // idealgas/eos.f90:88
  c->mu0 = 0.;          // idealgas/eos.f90:89
  c->precision = DG_PRECISION_FP64;
  c->filter_type = DG_FILTER_NONE;  // filter.f90:78-79
  c->n_filter = -1;                 // NFilter has no default (required for cut-off / LAF)
  c->hest_filter_param[0] = 36.;    // filter.f90:143
  c->hest_filter_param[1] = 12.;
  c->hest_filter_param[2] = 1.;
  c->laf_alpha = 1.;                // filter.f90:85
}

// "(/a, b, c/)" or "a, b, c" -> up to n doubles
static int parse_real_array(const std::string& v, double* out, int n) {
  std::string s;
  for (char ch : v) s += (ch == '(' || ch == ')' || ch == '/' || ch == ',') ? ' ' : ch;
  size_t pos = 0;
  int k = 0;
  while (k < n) {
    size_t a = s.find_first_not_of(" \t", pos);
    if (a == std::string::npos) break;
    size_t b = s.find_first_of(" \t", a);
    std::string tok = s.substr(a, b == std::string::npos ? std::string::npos : b - a);
    for (auto& ch : tok) if (ch == 'd' || ch == 'D') ch = 'e';  // Fortran exponent
    out[k++] = std::stod(tok);
    if (b == std::string::npos) break;
    pos = b;
  }
  return k;
}

static std::string lower(std::string s) {
  for (auto& ch : s) ch = (char)std::tolower((unsigned char)ch);
  return s;
}
static std::string trim(const std::string& s) {
  size_t a = s.find_first_not_of(" \t\r"), b = s.find_last_not_of(" \t\r");
  return a == std::string::npos ? std::string() : s.substr(a, b - a + 1);
}
static bool parse_bool(const std::string& v, int& out) {
  std::string s = lower(v);
  if (s == "t" || s == ".true." || s == "true" || s == "1" || s == "on") { out = 1; return true; }
  if (s == "f" || s == ".false." || s == "false" || s == "0" || s == "off") { out = 0; return true; }
  return false;
}

extern "C" int dg_config_from_ini(const char* text, dg_config* cfg) {
  if (!text || !cfg) { set_error("dg_config_from_ini: null argument"); return DG_ERR_ARG; }
  std::string all(text);
  size_t pos = 0;
  while (pos <= all.size()) {
    size_t e = all.find('\n', pos);
    if (e == std::string::npos) e = all.size();
    std::string line = all.substr(pos, e - pos);
    pos = e + 1;
    size_t bang = line.find('!');
    if (bang != std::string::npos) line = line.substr(0, bang);
    size_t eq = line.find('=');
    if (eq == std::string::npos) continue;
    std::string key = lower(trim(line.substr(0, eq))), val = trim(line.substr(eq + 1));
    std::string lv = lower(val);
    try {
      if (key == "n") cfg->N = std::stoi(val);
      else if (key == "nodetype") {
        if (lv == "gauss") cfg->node_type = DG_NODETYPE_GAUSS;
        else if (lv == "gauss-lobatto") cfg->node_type = DG_NODETYPE_GAUSS_LOBATTO;
        else { set_error("unknown NodeType " + val); return DG_ERR_ARG; }
      } else if (key == "riemann") {
        // string list of riemann.f90:130-144 (commented-out in GALAEXI, compile-time there)
        static const char* names[] = {"lf", "roe", "roel2", "roeentropyfix", "hll", "hllc", "hlle", "hllem", "avg"};
        int found = -1;
        for (int i = 0; i < 9; ++i) if (lv == names[i]) found = i;
        if (found < 0) { set_error("unknown Riemann " + val); return DG_ERR_ARG; }
        cfg->riemann = found;
      } else if (key == "splitdg") {
        static const char* names[] = {"sd", "mo", "du", "kg", "pi"};
        int found = -2;
        if (lv == "none" || lv == "off" || lv == "weak") found = DG_SPLIT_NONE;
        for (int i = 0; i < 5; ++i) if (lv == names[i]) found = i;
        if (found < -1) { set_error("unknown SplitDG " + val); return DG_ERR_ARG; }
        cfg->split_dg = found;
      } else if (key == "lifting") {
        if (lv == "br1") cfg->lifting = DG_LIFTING_BR1;
        else if (lv == "br2") cfg->lifting = DG_LIFTING_BR2;
        else { set_error("unknown Lifting " + val); return DG_ERR_ARG; }
      } else if (key == "parabolic") {
        int b; if (!parse_bool(val, b)) { set_error("bad Parabolic"); return DG_ERR_ARG; } cfg->parabolic = b;
      } else if (key == "kappa") cfg->kappa = std::stod(val);
      else if (key == "r") cfg->R = std::stod(val);
      else if (key == "pr") cfg->Pr = std::stod(val);
      else if (key == "mu0") cfg->mu0 = std::stod(val);
      else if (key == "etabr2") cfg->eta_br2 = std::stod(val);
      else if (key == "doweaklifting") {
        int b; if (!parse_bool(val, b)) { set_error("bad doWeakLifting"); return DG_ERR_ARG; } cfg->do_weak_lifting = b;
      } else if (key == "doconservativelifting") {
        int b; if (!parse_bool(val, b)) { set_error("bad doConservativeLifting"); return DG_ERR_ARG; }
        cfg->do_conservative_lifting = b;
      } else if (key == "filtertype") {
        static const char* names[] = {"none", "cutoff", "modal", "laf"};
        int found = -1;
        for (int i = 0; i < 4; ++i) if (lv == names[i]) found = i;
        if (found < 0 && !lv.empty() && std::isdigit((unsigned char)lv[0])) found = std::stoi(lv);
        if (found < 0 || found > 3) { set_error("unknown FilterType " + val); return DG_ERR_ARG; }
        cfg->filter_type = found;
      } else if (key == "nfilter") cfg->n_filter = std::stoi(val);
      else if (key == "hestfilterparam") {
        if (parse_real_array(val, cfg->hest_filter_param, 3) != 3) { set_error("HestFilterParam needs 3 values"); return DG_ERR_ARG; }
      } else if (key == "laf_alpha") cfg->laf_alpha = std::stod(val);
      else if (key == "precision") {
        if (lv == "fp64" || lv == "double") cfg->precision = DG_PRECISION_FP64;
        else if (lv == "mixed") cfg->precision = DG_PRECISION_MIXED;
        else { set_error("unknown Precision " + val); return DG_ERR_ARG; }
      }
    } catch (...) {
      set_error("cannot parse value of " + key + ": " + val);
      return DG_ERR_ARG;
    }
  }
  return DG_OK;
}

extern "C" int dg_basis(int N, int node_type, double* xGP, double* wGP, double* wBary, double* L_minus,
                        double* L_plus, double* D, double* D_hat_T, double* L_hat_minus, double* L_hat_plus,
                        double* DVolSurf) {
  if (N < 1 || N > 16 || (node_type != DG_NODETYPE_GAUSS && node_type != DG_NODETYPE_GAUSS_LOBATTO)) {
    set_error("dg_basis: bad N or node type");
    return DG_ERR_ARG;
  }
  Basis1D B;
  basis_1d(N, node_type, B);
  auto cp = [](double* d, const std::vector<double>& s) { if (d) std::memcpy(d, s.data(), s.size() * sizeof(double)); };
  cp(xGP, B.x); cp(wGP, B.w); cp(wBary, B.wb); cp(L_minus, B.Lm); cp(L_plus, B.Lp); cp(D, B.D);
  cp(D_hat_T, B.DhatT); cp(L_hat_minus, B.Lhm); cp(L_hat_plus, B.Lhp); cp(DVolSurf, B.DVS);
  return DG_OK;
}

extern "C" int dg_mesh_cartesian_sizes(int nx, int ny, int nz, int* nElems, int* nSides) {
  if (nx < 1 || ny < 1 || nz < 1) { set_error("mesh: bad element counts"); return DG_ERR_ARG; }
  long long ne = (long long)nx * ny * nz;
  if (ne * 3 > 0x7fffffffLL) { set_error("mesh: too many elements"); return DG_ERR_ARG; }
  if (nElems) *nElems = (int)ne;
  if (nSides) *nSides = (int)(3 * ne);
  return DG_OK;
}

// ---------------------------------------------------------------------------------------------
// Periodic box.  Local side numbering and orientation follow src/flexi.h:98-103 and
// src/mesh/mappings.f90; each element is master (flip 0) of its XI_PLUS, ETA_PLUS and
// ZETA_PLUS sides, and its neighbour's XI_MINUS, ETA_MINUS, ZETA_MINUS sides are the slaves.
// The slave flips (1 for xi/zeta sides, 2 for eta sides) are the ones for which
// SideToVol2(p,q,flip,slave side) lands on the same physical point as the master's (p,q).
// ---------------------------------------------------------------------------------------------
namespace gxh {
enum { ZETA_MINUS = 1, ETA_MINUS = 2, XI_PLUS = 3, ETA_PLUS = 4, XI_MINUS = 5, ZETA_PLUS = 6 };
const int NormalDirs[7] = {0, 3, 2, 1, 2, 1, 3};            // mesh_vars.f90:112 (1-based locSide)
const int TangDirs[7] = {0, 1, 3, 2, 3, 2, 1};              // mesh_vars.f90:114
const double NormalSigns[7] = {0, -1., -1., 1., 1., -1., 1.}; // mesh_vars.f90:118

struct Mapping {
  double x0[3], L[3], amp;
  int nel[3];
  void operator()(int e3[3], const double xi[3], double X[3]) const {
    for (int d = 0; d < 3; ++d) X[d] = x0[d] + ((double)e3[d] + 0.5 * (xi[d] + 1.)) * (L[d] / nel[d]);
    if (amp != 0.) {
      const double s = std::sin(2. * kPi * (X[0] - x0[0]) / L[0]) * std::sin(2. * kPi * (X[1] - x0[1]) / L[1]) *
                       std::sin(2. * kPi * (X[2] - x0[2]) / L[2]);
      for (int d = 0; d < 3; ++d) X[d] += amp * s;
    }
  }
};


// SurfMetricsFromJa (metrics.f90:752-789) for a master side (flip 0) of local side loc: the side
// node (p,q) sits at the volume face coordinates CGNS_SideToVol2(p,q,loc) (mappings.f90:388-425).
void surface_metrics(int N, int loc, const double* JaFace, size_t side, double* nvec, double* t1vec, double* t2vec,
                     double* surfelem) {
  const int n = N + 1, n2 = n * n;
  const int nd = NormalDirs[loc] - 1, td = TangDirs[loc] - 1;
  const double sgn = NormalSigns[loc];
  for (int q = 0; q <= N; ++q)
    for (int p = 0; p <= N; ++p) {
      int a = p, b = q;
      if (loc == XI_MINUS || loc == ZETA_MINUS) { a = q; b = p; }
      else if (loc == ETA_PLUS) a = N - p;
      const double* J = &JaFace[((size_t)(loc - 1) * n2 + a + n * b) * 9];
      const size_t f = (size_t)p + n * (q + (size_t)n * side);
      double se = std::sqrt(J[nd * 3 + 0] * J[nd * 3 + 0] + J[nd * 3 + 1] * J[nd * 3 + 1] + J[nd * 3 + 2] * J[nd * 3 + 2]);
      double nv[3], t1[3], t2[3];
      for (int c = 0; c < 3; ++c) nv[c] = sgn * J[nd * 3 + c] / se;
      const double dot = J[td * 3 + 0] * nv[0] + J[td * 3 + 1] * nv[1] + J[td * 3 + 2] * nv[2];
      for (int c = 0; c < 3; ++c) t1[c] = J[td * 3 + c] - dot * nv[c];
      const double tn = std::sqrt(t1[0] * t1[0] + t1[1] * t1[1] + t1[2] * t1[2]);
      for (int c = 0; c < 3; ++c) t1[c] = t1[c] / tn;
      t2[0] = nv[1] * t1[2] - nv[2] * t1[1];
      t2[1] = nv[2] * t1[0] - nv[0] * t1[2];
      t2[2] = nv[0] * t1[1] - nv[1] * t1[0];
      surfelem[f] = se;
      for (int c = 0; c < 3; ++c) { nvec[c + 3 * f] = nv[c]; t1vec[c + 3 * f] = t1[c]; t2vec[c + 3 * f] = t2[c]; }
    }
}
}  // namespace gxh

extern "C" int dg_mesh_cartesian(int N, int node_type, int NGeo, int nx, int ny, int nz, const double* x0,
                                 const double* x1, double deform_amp, double* node_coords, double* elem_xgp, double* Mf,
                                 double* Mg, double* Mh, double* sJ, double* nvec, double* t1vec, double* t2vec,
                                 double* surfelem, int* E2S, int* S2E) {
  int nElems, nSides;
  if (dg_mesh_cartesian_sizes(nx, ny, nz, &nElems, &nSides) != DG_OK) return DG_ERR_ARG;
  if (N < 1 || N > DG_MAX_N) { set_error("mesh: N out of range"); return DG_ERR_ARG; }
  if (NGeo < 1 || NGeo > DG_MAX_N) { set_error("mesh: NGeo out of range"); return DG_ERR_ARG; }
  if (!Mf || !Mg || !Mh || !sJ || !nvec || !t1vec || !t2vec || !surfelem || !E2S || !S2E) {
    set_error("dg_mesh_cartesian: null argument"); return DG_ERR_ARG;
  }
  const int n = N + 1, n2 = n * n, g = NGeo + 1;
  Basis1D B;
  basis_1d(N, node_type, B);
  Mapping map;
  for (int d = 0; d < 3; ++d) { map.x0[d] = x0[d]; map.L[d] = x1[d] - x0[d]; }
  map.nel[0] = nx; map.nel[1] = ny; map.nel[2] = nz;
  map.amp = deform_amp;
  auto eid = [&](int ix, int iy, int iz) {
    ix = (ix + nx) % nx; iy = (iy + ny) % ny; iz = (iz + nz) % nz;
    return ix + nx * (iy + ny * iz);
  };
  // connectivity (1-based IDs as in the reference's ElemToSide / SideToElem)
  for (int iz = 0; iz < nz; ++iz)
    for (int iy = 0; iy < ny; ++iy)
      for (int ix = 0; ix < nx; ++ix) {
        const int e = eid(ix, iy, iz);
        const int sx = 3 * e, sy = 3 * e + 1, sz = 3 * e + 2;
        const int mx = eid(ix - 1, iy, iz), my = eid(ix, iy - 1, iz), mz = eid(ix, iy, iz - 1);
        auto set = [&](int loc, int side0, int flip, int master) {
          int* p = E2S + 3 * ((loc - 1) + 6 * (size_t)e);
          p[0] = side0 + 1; p[1] = flip; p[2] = master;
        };
        set(XI_PLUS, sx, 0, 1); set(ETA_PLUS, sy, 0, 1); set(ZETA_PLUS, sz, 0, 1);
        set(XI_MINUS, 3 * mx, 1, 0); set(ETA_MINUS, 3 * my + 1, 2, 0); set(ZETA_MINUS, 3 * mz + 2, 1, 0);
      }
  for (int iz = 0; iz < nz; ++iz)
    for (int iy = 0; iy < ny; ++iy)
      for (int ix = 0; ix < nx; ++ix) {
        const int e = eid(ix, iy, iz);
        const int nb[3] = {eid(ix + 1, iy, iz), eid(ix, iy + 1, iz), eid(ix, iy, iz + 1)};
        const int mloc[3] = {XI_PLUS, ETA_PLUS, ZETA_PLUS}, sloc[3] = {XI_MINUS, ETA_MINUS, ZETA_MINUS};
        const int flips[3] = {1, 2, 1};
        for (int d = 0; d < 3; ++d) {
          int* p = S2E + 5 * (size_t)(3 * e + d);
          p[0] = e + 1; p[1] = nb[d] + 1; p[2] = mloc[d]; p[3] = sloc[d]; p[4] = flips[d];
        }
      }
  // element node coordinates on NGeo+1 equidistant points per direction, as a HOPR file holds them;
  // the displacement moves these nodes (as the reference's meshdeform does, mesh.f90:224-234)
  std::vector<double> nodes((size_t)3 * g * g * g * nElems);
  for (int e = 0; e < nElems; ++e) {
    int e3[3] = {e % nx, (e / nx) % ny, e / (nx * ny)};
    for (int k = 0; k < g; ++k)
      for (int j = 0; j < g; ++j)
        for (int i = 0; i < g; ++i) {
          const double xi[3] = {2. * (double)i / (double)NGeo - 1., 2. * (double)j / (double)NGeo - 1.,
                                2. * (double)k / (double)NGeo - 1.};
          map(e3, xi, &nodes[3 * vidx(g, i, j, k, e)]);
        }
  }
  if (node_coords) std::memcpy(node_coords, nodes.data(), nodes.size() * sizeof(double));
  if (deform_amp != 0.) {
    // curved: BuildCoords + CalcMetrics + CalcSurfMetrics of the reference on the node coordinates
    const int bad = metrics_from_nodes(N, node_type, NGeo, nElems, nodes.data(), E2S, elem_xgp, Mf, Mg, Mh, sJ, nvec,
                                       t1vec, t2vec, surfelem);
    if (bad != 0) { set_error("mesh: the displacement folds elements (bad Jacobian)"); return DG_ERR_ARG; }
    return DG_OK;
  }
  // affine: the exact mapping at the solution nodes and constant metric terms
  if (elem_xgp)
    for (int e = 0; e < nElems; ++e) {
      int e3[3] = {e % nx, (e / nx) % ny, e / (nx * ny)};
      for (int k = 0; k <= N; ++k)
        for (int j = 0; j <= N; ++j)
          for (int i = 0; i <= N; ++i) {
            const double xi[3] = {B.x[i], B.x[j], B.x[k]};
            map(e3, xi, &elem_xgp[3 * vidx(n, i, j, k, e)]);
          }
    }
  const double h[3] = {map.L[0] / nx, map.L[1] / ny, map.L[2] / nz};
  const double Ja[3] = {0.25 * h[1] * h[2], 0.25 * h[0] * h[2], 0.25 * h[0] * h[1]};
  const double s = 8. / (h[0] * h[1] * h[2]);
  for (size_t t = 0; t < (size_t)nElems * n * n2; ++t) {
    for (int d = 0; d < 3; ++d) {
      Mf[d + 3 * t] = d == 0 ? Ja[0] : 0.;
      Mg[d + 3 * t] = d == 1 ? Ja[1] : 0.;
      Mh[d + 3 * t] = d == 2 ? Ja[2] : 0.;
    }
    sJ[t] = s;
  }
  // SurfMetricsFromJa (metrics.f90:752-789) on the master sides (every element is master of its
  // three plus sides) from the constant face metric terms
  std::vector<double> JaFace((size_t)6 * n2 * 9, 0.);
  for (size_t t = 0; t < (size_t)6 * n2; ++t)
    for (int nn = 0; nn < 3; ++nn)
      for (int dd = 0; dd < 3; ++dd) JaFace[t * 9 + nn * 3 + dd] = (nn == dd) ? Ja[nn] : 0.;
  for (int e = 0; e < nElems; ++e) {
    const int locs[3] = {XI_PLUS, ETA_PLUS, ZETA_PLUS};
    for (int d = 0; d < 3; ++d) surface_metrics(N, locs[d], JaFace.data(), (size_t)(3 * e + d), nvec, t1vec, t2vec, surfelem);
  }
  return DG_OK;
}

// ---------------------------------------------------------------------------------------------
// Initial states
// ---------------------------------------------------------------------------------------------
static void prim_to_cons(const double prim[5], double kappa, double* cons) {
  // PrimToCons (idealgas/eos.f90:467-489)
  cons[0] = prim[0];
  cons[1] = prim[1] * prim[0];
  cons[2] = prim[2] * prim[0];
  cons[3] = prim[3] * prim[0];
  cons[4] = prim[4] / (kappa - 1.) + 0.5 * (cons[1] * prim[1] + cons[2] * prim[2] + cons[3] * prim[3]);
}

extern "C" int dg_fill_ini(int exactfunc, const double* prm, int nprm, long long nNodes, const double* xgp, double kappa,
                           double R, double t, double* U) {
  if (!xgp || !U || nNodes < 0) { set_error("dg_fill_ini: null argument"); return DG_ERR_ARG; }
  for (long long m = 0; m < nNodes; ++m) {
    const double* x = xgp + 3 * m;
    double prim[5];
    if (exactfunc == DG_EXACTFUNC_CONST) {
      if (nprm < 5) { set_error("dg_fill_ini: constant state needs 5 parameters"); return DG_ERR_ARG; }
      for (int c = 0; c < 5; ++c) prim[c] = prm[c];
    } else if (exactfunc == DG_EXACTFUNC_SHU_VORTEX) {
      // exactfunc.f90:482-502: RefState(5), IniCenter(3), IniAxis(3), IniAmplitude, IniHalfwidth
      if (nprm < 13) { set_error("dg_fill_ini: Shu vortex needs 13 parameters"); return DG_ERR_ARG; }
      for (int c = 0; c < 5; ++c) prim[c] = prm[c];
      const double vel[3] = {prm[1], prm[2], prm[3]};
      const double RT = prim[4] / prim[0];
      double cent[3];
      for (int d = 0; d < 3; ++d) cent[d] = x[d] - (prm[5 + d] + vel[d] * t);
      const double* ax = prm + 8;
      double cr[3] = {ax[1] * cent[2] - ax[2] * cent[1], ax[2] * cent[0] - ax[0] * cent[2], ax[0] * cent[1] - ax[1] * cent[0]};
      for (int d = 0; d < 3; ++d) cr[d] = cr[d] / prm[12];
      const double r2 = cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2];
      const double du = prm[11] / (2. * kPi) * std::exp(0.5 * (1. - r2));
      const double km1 = kappa - 1.;
      const double dTemp = -km1 / (2. * kappa * RT) * du * du;
      prim[0] = prim[0] * std::pow(1. + dTemp, 1. * (1. / km1));
      for (int d = 0; d < 3; ++d) prim[1 + d] = prim[1 + d] + du * cr[d];
      prim[4] = prim[4] * std::pow(1. + dTemp, kappa / km1);
    } else if (exactfunc == DG_EXACTFUNC_TGV) {
      // testcase/taylorgreenvortex/testcase.f90:145-149, 241-256: rho0, U0, Ma0, IniConstDens
      if (nprm < 4) { set_error("dg_fill_ini: TGV needs 4 parameters"); return DG_ERR_ARG; }
      const double rho0 = prm[0], U0 = prm[1], Ma0 = prm[2];
      const double p0 = (U0 / Ma0) * (U0 / Ma0) / kappa * rho0;
      const double T0 = p0 / (rho0 * R);
      prim[1] = U0 * std::sin(x[0]) * std::cos(x[1]) * std::cos(x[2]);
      prim[2] = -U0 * std::cos(x[0]) * std::sin(x[1]) * std::cos(x[2]);
      prim[3] = 0.;
      prim[4] = p0 + (rho0 * U0 * U0) / 16. *
                         (std::cos(2 * x[0]) * std::cos(2. * x[2]) + 2. * std::cos(2. * x[1]) + 2. * std::cos(2. * x[0]) +
                          std::cos(2 * x[1]) * std::cos(2. * x[2]));
      if (prm[3] != 0.) prim[0] = rho0;
      else prim[0] = prim[4] / (T0 * R);
    } else {
      set_error("dg_fill_ini: unknown exact function");
      return DG_ERR_ARG;
    }
    prim_to_cons(prim, kappa, U + 5 * m);
  }
  return DG_OK;
}
