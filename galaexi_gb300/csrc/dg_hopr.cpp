// HOPR mesh files (HDF5) -> the reference's mesh arrays.
//
// Follows ReadMesh (src/mesh/mesh_readin.f90:204-470) for the connectivity: ElemInfo rows
// (type, zone, first/last side index, first/last node index) and SideInfo rows (type, ±global side
// ID, neighbour element, flip, BC index); a positive side ID marks the oriented (master, flip 0)
// side, a negative one the slave with flip = SideInfo flip mod 10; sides on periodic BCs (BC type 1)
// are connected like inner sides, the other BC sides have no neighbour.  Geometry follows
// BuildCoords / CalcMetrics (src/mesh/metrics.f90:85-160, 171-560): the equidistant NGeo node
// coordinates are interpolated to the Chebyshev-Gauss-Lobatto points of degree N, the metric terms
// are formed in curl form there and interpolated to the solution nodes; the side vectors come from
// the master element (SurfMetricsFromJa, metrics.f90:752-789).  Side numbering: BC sides first
// (1..nBCSides), then the connected sides in order of first appearance.  Mortar meshes are not
// supported.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "../../include/galaexi_gb300.h"
#include "dg_hdf5.h"
#include "dg_host.h"

using gxh::set_error;

namespace {

struct Hopr {
  int nElems = 0, NGeo = 0, nBCs = 0;
  std::vector<long long> elemInfo, sideInfo, bcType;  // (nElems,6), (nSideRows,5), (nBCs,4)
  std::vector<double> nodes;                          // (nElems*(NGeo+1)^3, 3)
  // per element side (e*6 + ls-1): local side ID (0-based), flip, master flag, BC index (1-based, 0 if none)
  std::vector<int> side, flip, master, bc;
  int nSides = 0, nBCSides = 0;
};

bool read_hopr(const char* path, Hopr& H, bool with_nodes) {
  gxh5::File f;
  std::string err;
  if (!path || !f.open(path, err)) { set_error(path ? err : "null path"); return false; }
  gxh5::Array a;
  if (!f.attribute("Ngeo", a, err)) { set_error(err); return false; }
  H.NGeo = (int)a.as_int()[0];
  if (!f.dataset("ElemInfo", a, err)) { set_error(err); return false; }
  if (a.dims.size() != 2 || a.dims[1] != 6) { set_error("ElemInfo must be (nElems,6)"); return false; }
  H.nElems = (int)a.dims[0];
  H.elemInfo = a.as_int();
  if (!f.dataset("SideInfo", a, err)) { set_error(err); return false; }
  if (a.dims.size() != 2 || a.dims[1] != 5) { set_error("SideInfo must be (nSides,5)"); return false; }
  H.sideInfo = a.as_int();
  const long long nSideRows = (long long)a.dims[0];
  if (f.has_dataset("BCType")) {
    if (!f.dataset("BCType", a, err)) { set_error(err); return false; }
    H.bcType = a.as_int();
    H.nBCs = (int)a.dims[0];
  }
  if (with_nodes) {
    if (!f.dataset("NodeCoords", a, err)) { set_error(err); return false; }
    H.nodes = a.as_double();
  }
  const int ng = H.NGeo + 1, ng3 = ng * ng * ng;
  if (H.NGeo < 1 || H.nElems < 1) { set_error("HOPR mesh: bad NGeo or nElems"); return false; }
  if (with_nodes && H.nodes.size() != (size_t)H.nElems * ng3 * 3) {
    set_error("HOPR mesh: NodeCoords does not hold (NGeo+1)^3 nodes per element"); return false;
  }
  // connectivity
  H.side.assign((size_t)H.nElems * 6, -1);
  H.flip.assign((size_t)H.nElems * 6, 0);
  H.master.assign((size_t)H.nElems * 6, 0);
  H.bc.assign((size_t)H.nElems * 6, 0);
  std::map<long long, int> inner;
  std::vector<std::pair<int, int>> bcsides;  // (element side slot, BC index)
  for (int e = 0; e < H.nElems; ++e) {
    const long long* ei = &H.elemInfo[(size_t)e * 6];
    if (ei[5] - ei[4] != ng3) { set_error("HOPR mesh: only hexahedra with (NGeo+1)^3 nodes are supported"); return false; }
    if (ei[3] - ei[2] != 6) { set_error("HOPR mesh: mortar sides are not supported"); return false; }
    for (int ls = 1; ls <= 6; ++ls) {
      const long long r = ei[2] + ls - 1;
      if (r < 0 || r >= nSideRows) { set_error("HOPR mesh: SideInfo index out of range"); return false; }
      const long long* si = &H.sideInfo[(size_t)r * 5];
      if (si[0] < 0 || si[2] < 0) { set_error("HOPR mesh: mortar sides are not supported"); return false; }
      const long long gid = si[1], nb = si[2], bci = si[4];
      const size_t slot = (size_t)e * 6 + ls - 1;
      bool isBC = false;
      if (bci != 0) {
        if (bci < 1 || bci > H.nBCs) { set_error("HOPR mesh: BC index out of range"); return false; }
        const long long type = H.bcType[(size_t)(bci - 1) * 4];
        isBC = type != 1 && type != 100;  // periodic (1) and inner (100) BCs are connected sides
      }
      H.bc[slot] = (int)bci;
      if (isBC || nb == 0) {
        if (!isBC) { set_error("HOPR mesh: side without neighbour and without BC"); return false; }
        bcsides.push_back({(int)slot, (int)bci});
        H.flip[slot] = 0;
        H.master[slot] = 1;
        continue;
      }
      const long long key = gid < 0 ? -gid : gid;
      auto it = inner.find(key);
      int id;
      if (it == inner.end()) { id = (int)inner.size(); inner[key] = id; }
      else id = it->second;
      H.side[slot] = id;
      H.flip[slot] = gid > 0 ? 0 : (int)(si[3] % 10);
      H.master[slot] = gid > 0 ? 1 : 0;
      if (gid < 0 && (H.flip[slot] < 1 || H.flip[slot] > 4)) { set_error("HOPR mesh: bad flip of a slave side"); return false; }
    }
  }
  H.nBCSides = (int)bcsides.size();
  std::vector<char> bcslot(H.side.size(), 0);
  for (int b = 0; b < H.nBCSides; ++b) {
    H.side[bcsides[b].first] = b;
    bcslot[bcsides[b].first] = 1;
  }
  for (size_t s = 0; s < H.side.size(); ++s)
    if (!bcslot[s]) H.side[s] += H.nBCSides;  // connected sides are numbered after the BC sides
  H.nSides = H.nBCSides + (int)inner.size();
  // every connected side: one master, one slave
  std::vector<int> cnt((size_t)H.nSides * 2, 0);
  for (size_t s = 0; s < H.side.size(); ++s) cnt[(size_t)H.side[s] * 2 + (H.master[s] ? 0 : 1)]++;
  for (int sd = 0; sd < H.nSides; ++sd) {
    const bool bcside = sd < H.nBCSides;
    if (cnt[(size_t)sd * 2] != 1 || cnt[(size_t)sd * 2 + 1] != (bcside ? 0 : 1)) {
      set_error("HOPR mesh: a side lacks its master or slave element"); return false;
    }
  }
  return true;
}


// 1D operator set for the metric terms
struct Ops1D {
  int N = 0;
  std::vector<double> x, wb, D;  // nodes, barycentric weights, D(i,l) column-major
};
Ops1D ops_for(int N, int node_type) {
  gxh::Basis1D B;
  gxh::basis_1d(N, node_type, B);
  Ops1D o;
  o.N = N; o.x = B.x; o.wb = B.wb; o.D = B.D;
  return o;
}
std::vector<double> vdm(const Ops1D& from, const Ops1D& to) {
  std::vector<double> V;
  gxh::vandermonde(from.N, from.x.data(), from.wb.data(), to.N, to.x.data(), V);
  return V;
}

// ChangeBasis3D (changebasis.f90): nv components per node, V (0:mo,0:mi) column-major; the three
// directions are applied xi, eta, zeta with the input index running innermost
void change_basis_3d(int nv, int mi, int mo, const std::vector<double>& V, const double* in, double* out) {
  const int ni = mi + 1, no = mo + 1;
  std::vector<double> b1((size_t)nv * no * ni * ni, 0.), b2((size_t)nv * no * no * ni, 0.);
  for (int k = 0; k < ni; ++k) for (int j = 0; j < ni; ++j) for (int i = 0; i < ni; ++i)
    for (int io = 0; io < no; ++io)
      for (int c = 0; c < nv; ++c)
        b1[c + nv * (io + no * (j + ni * k))] += V[io + no * i] * in[c + nv * (i + ni * (j + ni * k))];
  for (int k = 0; k < ni; ++k) for (int j = 0; j < ni; ++j) for (int io = 0; io < no; ++io)
    for (int jo = 0; jo < no; ++jo)
      for (int c = 0; c < nv; ++c)
        b2[c + nv * (io + no * (jo + no * k))] += V[jo + no * j] * b1[c + nv * (io + no * (j + ni * k))];
  for (size_t t = 0; t < (size_t)nv * no * no * no; ++t) out[t] = 0.;
  for (int k = 0; k < ni; ++k) for (int jo = 0; jo < no; ++jo) for (int io = 0; io < no; ++io)
    for (int ko = 0; ko < no; ++ko)
      for (int c = 0; c < nv; ++c)
        out[c + nv * (io + no * (jo + no * ko))] += V[ko + no * k] * b2[c + nv * (io + no * (jo + no * k))];
}
// ChangeBasis2D on a face plane (nv components)
void change_basis_2d(int nv, int m, const std::vector<double>& V, const double* in, double* out) {
  const int n = m + 1;
  std::vector<double> b1((size_t)nv * n * n, 0.);
  for (int j = 0; j < n; ++j) for (int i = 0; i < n; ++i)
    for (int io = 0; io < n; ++io)
      for (int c = 0; c < nv; ++c) b1[c + nv * (io + n * j)] += V[io + n * i] * in[c + nv * (i + n * j)];
  for (size_t t = 0; t < (size_t)nv * n * n; ++t) out[t] = 0.;
  for (int j = 0; j < n; ++j) for (int io = 0; io < n; ++io)
    for (int jo = 0; jo < n; ++jo)
      for (int c = 0; c < nv; ++c) out[c + nv * (io + n * jo)] += V[jo + n * j] * b1[c + nv * (io + n * j)];
}

// CalcMetrics (metrics.f90:171-560, curl form, N >= NGeo or N < NGeo) for one element from its
// equidistant NGeo node coordinates; writes Elem_xGP (BuildCoords, metrics.f90:85-160), the metric
// terms and sJ at the solution nodes, and JaCL_N (3 x 3 per CL node) for the surface metrics.
struct MetricOps {
  int N, NGeo, NGeoRef;
  Ops1D clN, clG, eqG;
  std::vector<double> V_eq_clG, V_clG_clN, V_clG_ref, V_ref_N, V_clN_N, V_eq_N;
  MetricOps(int N_, int NGeo_, int node_type) : N(N_), NGeo(NGeo_), NGeoRef(3 * NGeo_) {
    clN = ops_for(N, 99);
    clG = ops_for(NGeo, 99);
    eqG.N = NGeo;
    eqG.x.resize(NGeo + 1);
    eqG.wb.resize(NGeo + 1);
    for (int k = 0; k <= NGeo; ++k) eqG.x[k] = -1. + 2. * k / NGeo;
    for (int k = 0; k <= NGeo; ++k) {
      double pr = 1.;
      for (int j = 0; j <= NGeo; ++j)
        if (j != k) pr *= eqG.x[k] - eqG.x[j];
      eqG.wb[k] = 1. / pr;
    }
    const Ops1D ref = ops_for(NGeoRef, node_type), sol = ops_for(N, node_type);
    V_eq_clG = vdm(eqG, clG);
    V_clG_clN = vdm(clG, clN);
    V_clG_ref = vdm(clG, ref);
    // the Jacobian of degree 3 NGeo to the solution nodes: modal projection for N < NGeoRef (the
    // modal Vandermonde of metrics.f90:289, which keeps the element volume), interpolation otherwise
    if (N < NGeoRef) gxh::modal_projection(NGeoRef, ref.x.data(), ref.wb.data(), N, sol.x.data(), V_ref_N);
    else V_ref_N = vdm(ref, sol);
    V_clN_N = vdm(clN, sol);
    // BuildCoords: Vdm_EQNGeo_CLN then MATMUL(Vdm_CLN_N, .) -> EQ(NGeo) -> solution nodes
    const std::vector<double> V_eq_clN = vdm(eqG, clN);
    const int n = N + 1, g = NGeo + 1;
    V_eq_N.assign((size_t)n * g, 0.);
    for (int c = 0; c < g; ++c)
      for (int r = 0; r < n; ++r) {
        double sacc = 0.;
        for (int m = 0; m < n; ++m) sacc += V_clN_N[r + n * m] * V_eq_clN[m + n * c];
        V_eq_N[r + n * c] = sacc;
      }
  }
};

int flexi_metrics(const MetricOps& O, const double* nodes, int e, double* elem_xgp, double* Mf, double* Mg,
                  double* Mh, double* sJ, std::vector<double>& JaCL) {
  const int N = O.N, NGeo = O.NGeo, n = N + 1, g = NGeo + 1, n3 = n * n * n, g3 = g * g * g, r = O.NGeoRef + 1;
  std::vector<double> XG(3 * g3), XN(3 * n3), dXG(9 * g3), dXN(9 * n3), tmpG(3 * g3), tmpN(3 * n3);
  change_basis_3d(3, NGeo, NGeo, O.V_eq_clG, nodes, XG.data());
  change_basis_3d(3, NGeo, N, O.V_clG_clN, XG.data(), XN.data());
  if (elem_xgp) change_basis_3d(3, NGeo, N, O.V_eq_N, nodes, elem_xgp + (size_t)3 * n3 * e);
  // dXCL_NGeo(dd, nn): d X_nn / d xi_dd on the CL(NGeo) points
  auto GI = [&](int i, int j, int k) { return (size_t)i + g * (j + (size_t)g * k); };
  for (int k = 0; k < g; ++k) for (int j = 0; j < g; ++j) for (int i = 0; i < g; ++i) {
    double* d = &dXG[9 * GI(i, j, k)];
    for (int t = 0; t < 9; ++t) d[t] = 0.;
    for (int ll = 0; ll < g; ++ll)
      for (int nn = 0; nn < 3; ++nn) {
        d[0 * 3 + nn] += O.clG.D[i + g * ll] * XG[nn + 3 * GI(ll, j, k)];
        d[1 * 3 + nn] += O.clG.D[j + g * ll] * XG[nn + 3 * GI(i, ll, k)];
        d[2 * 3 + nn] += O.clG.D[k + g * ll] * XG[nn + 3 * GI(i, j, ll)];
      }
  }
  // Jacobian on NGeoRef = 3 NGeo nodes, interpolated to the solution nodes (exact)
  std::vector<double> dXR((size_t)9 * r * r * r), det((size_t)r * r * r), detN(n3);
  for (int nn = 0; nn < 3; ++nn) {
    // the slice dXCL_NGeo(1:3, nn): the three direction derivatives of coordinate nn
    for (size_t t = 0; t < (size_t)g3; ++t)
      for (int dd = 0; dd < 3; ++dd) tmpG[3 * t + dd] = dXG[9 * t + dd * 3 + nn];
    std::vector<double> outR((size_t)3 * r * r * r);
    change_basis_3d(3, NGeo, O.NGeoRef, O.V_clG_ref, tmpG.data(), outR.data());
    for (size_t t = 0; t < (size_t)r * r * r; ++t)
      for (int dd = 0; dd < 3; ++dd) dXR[9 * t + dd * 3 + nn] = outR[3 * t + dd];
  }
  for (size_t t = 0; t < (size_t)r * r * r; ++t) {
    const double* a = &dXR[9 * t];  // a[dd*3+nn] = dX(dd+1, nn+1)
    auto X = [&](int dd, int nn) { return a[(dd - 1) * 3 + (nn - 1)]; };
    det[t] = 0. + X(1, 1) * (X(2, 2) * X(3, 3) - X(3, 2) * X(2, 3)) + X(2, 1) * (X(3, 2) * X(1, 3) - X(1, 2) * X(3, 3)) +
             X(3, 1) * (X(1, 2) * X(2, 3) - X(2, 2) * X(1, 3));
  }
  change_basis_3d(1, O.NGeoRef, N, O.V_ref_N, det.data(), detN.data());
  // scaled-Jacobian check of metrics.f90:340-353 (the reference aborts below 0.01)
  int bad = 0;
  const double mx = *std::max_element(detN.begin(), detN.end());
  for (int t = 0; t < n3; ++t) {
    sJ[(size_t)e * n3 + t] = 1. / detN[t];
    if (!(detN[t] > 0.)) bad = -1;
    else if (bad >= 0 && detN[t] / mx < 0.01) bad++;
  }
  // dXCL_N: interpolated from NGeo (N >= NGeo) or differentiated on CL(N)
  auto NI = [&](int i, int j, int k) { return (size_t)i + n * (j + (size_t)n * k); };
  if (N >= NGeo) {
    for (int nn = 0; nn < 3; ++nn) {
      for (size_t t = 0; t < (size_t)g3; ++t)
        for (int dd = 0; dd < 3; ++dd) tmpG[3 * t + dd] = dXG[9 * t + dd * 3 + nn];
      change_basis_3d(3, NGeo, N, O.V_clG_clN, tmpG.data(), tmpN.data());
      for (int t = 0; t < n3; ++t)
        for (int dd = 0; dd < 3; ++dd) dXN[9 * t + dd * 3 + nn] = tmpN[3 * t + dd];
    }
  } else {
    for (int k = 0; k < n; ++k) for (int j = 0; j < n; ++j) for (int i = 0; i < n; ++i) {
      double* d = &dXN[9 * NI(i, j, k)];
      for (int t = 0; t < 9; ++t) d[t] = 0.;
      for (int ll = 0; ll < n; ++ll)
        for (int nn = 0; nn < 3; ++nn) {
          d[0 * 3 + nn] += O.clN.D[i + n * ll] * XN[nn + 3 * NI(ll, j, k)];
          d[1 * 3 + nn] += O.clN.D[j + n * ll] * XN[nn + 3 * NI(i, ll, k)];
          d[2 * 3 + nn] += O.clN.D[k + n * ll] * XN[nn + 3 * NI(i, j, ll)];
        }
    }
  }
  // curl form: R(dd, nn), then JaCL(dd, nn)
  std::vector<double> R((size_t)9 * n3);
  for (int t = 0; t < n3; ++t) {
    const double* x = &XN[3 * t];
    const double* d = &dXN[9 * t];
    for (int dd = 0; dd < 3; ++dd) {
      R[9 * t + dd * 3 + 0] = 0.5 * (x[2] * d[dd * 3 + 1] - x[1] * d[dd * 3 + 2]);
      R[9 * t + dd * 3 + 1] = 0.5 * (x[0] * d[dd * 3 + 2] - x[2] * d[dd * 3 + 0]);
      R[9 * t + dd * 3 + 2] = 0.5 * (x[1] * d[dd * 3 + 0] - x[0] * d[dd * 3 + 1]);
    }
  }
  JaCL.assign((size_t)9 * n3, 0.);
  for (int k = 0; k < n; ++k) for (int j = 0; j < n; ++j) for (int i = 0; i < n; ++i) {
    double* J = &JaCL[9 * NI(i, j, k)];
    for (int q = 0; q < n; ++q)
      for (int nn = 0; nn < 3; ++nn) {
        J[0 * 3 + nn] = J[0 * 3 + nn] - O.clN.D[j + n * q] * R[9 * NI(i, q, k) + 2 * 3 + nn];
        J[1 * 3 + nn] = J[1 * 3 + nn] - O.clN.D[k + n * q] * R[9 * NI(i, j, q) + 0 * 3 + nn];
        J[2 * 3 + nn] = J[2 * 3 + nn] - O.clN.D[i + n * q] * R[9 * NI(q, j, k) + 1 * 3 + nn];
      }
    for (int q = 0; q < n; ++q)
      for (int nn = 0; nn < 3; ++nn) {
        J[0 * 3 + nn] = J[0 * 3 + nn] + O.clN.D[k + n * q] * R[9 * NI(i, j, q) + 1 * 3 + nn];
        J[1 * 3 + nn] = J[1 * 3 + nn] + O.clN.D[i + n * q] * R[9 * NI(q, j, k) + 2 * 3 + nn];
        J[2 * 3 + nn] = J[2 * 3 + nn] + O.clN.D[j + n * q] * R[9 * NI(i, q, k) + 0 * 3 + nn];
      }
  }
  // Metrics_f/g/hTilde = Vdm_CLN_N applied to JaCL_N(dd, 1:3)
  double* outs[3] = {Mf, Mg, Mh};
  for (int dd = 0; dd < 3; ++dd) {
    for (int t = 0; t < n3; ++t)
      for (int nn = 0; nn < 3; ++nn) tmpN[3 * t + nn] = JaCL[9 * t + dd * 3 + nn];
    change_basis_3d(3, N, N, O.V_clN_N, tmpN.data(), outs[dd] + (size_t)3 * n3 * e);
  }
  return bad;
}

// CalcSurfMetrics (metrics.f90:596-750) for one master side: JaCL_N on the face plane, ChangeBasis2D
// to the solution nodes, SideToVol2(p,q,0,locSide), SurfMetricsFromJa
void flexi_surface(const MetricOps& O, const std::vector<double>& JaCL, int loc, size_t side, double* nvec,
                   double* t1vec, double* t2vec, double* surfelem) {
  const int N = O.N, n = N + 1, n2 = n * n;
  auto NI = [&](int i, int j, int k) { return (size_t)i + n * (j + (size_t)n * k); };
  std::vector<double> face((size_t)9 * n2), plane((size_t)3 * n2), tmp((size_t)3 * n2);
  const int pl = (loc == 5 || loc == 2 || loc == 1) ? 0 : N;  // XI_MINUS, ETA_MINUS, ZETA_MINUS
  std::vector<double> JaFace((size_t)6 * n2 * 9, 0.);
  for (int dd = 0; dd < 3; ++dd) {
    for (int b = 0; b < n; ++b)
      for (int a = 0; a < n; ++a) {
        size_t src;
        if (loc == 5 || loc == 3) src = NI(pl, a, b);
        else if (loc == 2 || loc == 4) src = NI(a, pl, b);
        else src = NI(a, b, pl);
        for (int nn = 0; nn < 3; ++nn) plane[3 * (a + n * b) + nn] = JaCL[9 * src + dd * 3 + nn];
      }
    change_basis_2d(3, N, O.V_clN_N, plane.data(), tmp.data());
    for (int b = 0; b < n; ++b)
      for (int a = 0; a < n; ++a)
        for (int nn = 0; nn < 3; ++nn) JaFace[((size_t)(loc - 1) * n2 + a + n * b) * 9 + dd * 3 + nn] = tmp[3 * (a + n * b) + nn];
  }
  gxh::surface_metrics(N, loc, JaFace.data(), side, nvec, t1vec, t2vec, surfelem);
}
}  // namespace

int gxh::metrics_from_nodes(int N, int node_type, int NGeo, int nElems, const double* nodes, const int* E2S,
                            double* elem_xgp, double* Mf, double* Mg, double* Mh, double* sJ, double* nvec,
                            double* t1vec, double* t2vec, double* surfelem) {
  const MetricOps O(N, NGeo, node_type);
  const size_t ng3 = (size_t)(NGeo + 1) * (NGeo + 1) * (NGeo + 1);
  std::vector<double> JaCL;
  int bad = 0;
  for (int e = 0; e < nElems; ++e) {
    const int b = flexi_metrics(O, nodes + ng3 * 3 * e, e, elem_xgp, Mf, Mg, Mh, sJ, JaCL);
    if (b < 0 || bad < 0) bad = -1;
    else bad += b;
    for (int ls = 1; ls <= 6; ++ls) {
      const int* p = E2S + 3 * ((size_t)e * 6 + ls - 1);
      if (p[1] == 0) flexi_surface(O, JaCL, ls, (size_t)(p[0] - 1), nvec, t1vec, t2vec, surfelem);
    }
  }
  return bad;
}

extern "C" int dg_mesh_hopr_sizes(const char* path, int* nElems, int* nSides, int* nBCSides, int* NGeo) {
  if (!nElems || !nSides || !nBCSides || !NGeo) { set_error("dg_mesh_hopr_sizes: null argument"); return DG_ERR_ARG; }
  Hopr H;
  if (!read_hopr(path, H, false)) return DG_ERR_ARG;
  *nElems = H.nElems;
  *nSides = H.nSides;
  *nBCSides = H.nBCSides;
  *NGeo = H.NGeo;
  return DG_OK;
}

extern "C" int dg_h5_read(const char* path, const char* name, int attribute, int* ndims, long long* dims, double* out,
                          long long cap, char* str, int str_len) {
  if (!path || !name || !ndims || !dims) { set_error("dg_h5_read: null argument"); return DG_ERR_ARG; }
  gxh5::File f;
  std::string err;
  if (!f.open(path, err)) { set_error(err); return DG_ERR_ARG; }
  gxh5::Array a;
  if (!(attribute ? f.attribute(name, a, err) : f.dataset(name, a, err))) { set_error(err); return DG_ERR_ARG; }
  if (a.dims.size() > 8) { set_error("dg_h5_read: more than 8 dimensions"); return DG_ERR_UNSUPPORTED; }
  *ndims = (int)a.dims.size();
  for (size_t d = 0; d < a.dims.size(); ++d) dims[d] = (long long)a.dims[d];
  if (a.cls == 3) {
    if (str && str_len > 1) {
      const std::vector<std::string> v = a.as_strings();
      std::memset(str, 0, str_len);
      if (!v.empty()) std::memcpy(str, v[0].data(), std::min((size_t)str_len - 1, v[0].size()));
    }
    return DG_OK;
  }
  if (out) {
    if ((unsigned long long)cap < a.count()) { set_error("dg_h5_read: output too small"); return DG_ERR_ARG; }
    const std::vector<double> v = a.as_double();
    std::memcpy(out, v.data(), v.size() * sizeof(double));
  }
  return DG_OK;
}

extern "C" int dg_write_state(const char* path, const char* project, const char* mesh_file, int N,
                              const char* node_type, double time, int nElems, const double* U) {
  if (!path || !project || !mesh_file || !node_type || !U || N < 1 || nElems < 1) {
    set_error("dg_write_state: bad argument"); return DG_ERR_ARG;
  }
  const uint64_t n = (uint64_t)N + 1;
  gxh5::Writer w;
  // the attributes of GenerateFileSkeleton / WriteHeader (io_hdf5/hdf5_output.f90:744-870, 941-961)
  w.attr_string("Program", "GALAEXI-GB300");
  w.attr_string("File_Type", "State");
  w.attr_string("Project_Name", project);
  w.attr_double("File_Version", {0.1});
  w.attr_strings("VarNames", {"Density", "MomentumX", "MomentumY", "MomentumZ", "EnergyStagnationDensity"}, 255);
  w.attr_int("N", {N});
  w.attr_int("Dimension", {3});
  w.attr_double("Time", {time});
  w.attr_string("MeshFile", mesh_file);
  std::string base(path);
  const size_t slash = base.find_last_of('/');
  if (slash != std::string::npos) base = base.substr(slash + 1);
  w.attr_string("NextFile", base);
  w.attr_string("NodeType", node_type);
  // DG_Solution(nVar, 0:N, 0:N, 0:N, nElems) in Fortran order = (nElems, k, j, i, nVar) in HDF5 order
  w.dataset_double("DG_Solution", {(uint64_t)nElems, n, n, n, 5}, U);
  std::string err;
  if (!w.write(path, err)) { set_error(err); return DG_ERR_ARG; }
  return DG_OK;
}

extern "C" int dg_mesh_hopr_bcs(const char* path, int* nBCs, char* names, int name_len, int* bc_type) {
  if (!path || !nBCs) { set_error("dg_mesh_hopr_bcs: null argument"); return DG_ERR_ARG; }
  gxh5::File f;
  std::string err;
  if (!f.open(path, err)) { set_error(err); return DG_ERR_ARG; }
  *nBCs = 0;
  if (!f.has_dataset("BCType")) return DG_OK;
  gxh5::Array t, nm;
  if (!f.dataset("BCType", t, err) || !f.dataset("BCNames", nm, err)) { set_error(err); return DG_ERR_ARG; }
  if (t.dims.size() != 2 || t.dims[1] != 4) { set_error("BCType must be (nBCs,4)"); return DG_ERR_ARG; }
  const std::vector<std::string> bn = nm.as_strings();
  if (bn.size() != t.dims[0]) { set_error("BCNames and BCType differ in length"); return DG_ERR_ARG; }
  *nBCs = (int)t.dims[0];
  if (bc_type) {
    const std::vector<long long> v = t.as_int();
    for (size_t i = 0; i < v.size(); ++i) bc_type[i] = (int)v[i];
  }
  if (names) {
    if (name_len < 2) { set_error("dg_mesh_hopr_bcs: name_len too small"); return DG_ERR_ARG; }
    for (int b = 0; b < *nBCs; ++b) {
      // names are fixed-length, blank padded: trimmed as Fortran TRIM does
      std::string x = bn[b];
      while (!x.empty() && (x.back() == ' ' || x.back() == '\0')) x.pop_back();
      char* dst = names + (size_t)b * name_len;
      std::memset(dst, 0, name_len);
      std::memcpy(dst, x.data(), std::min((size_t)name_len - 1, x.size()));
    }
  }
  return DG_OK;
}

extern "C" int dg_mesh_hopr(const char* path, int N, int node_type, double* elem_xgp, double* Mf, double* Mg, double* Mh,
                            double* sJ, double* nvec, double* t1vec, double* t2vec, double* surfelem, int* E2S, int* S2E,
                            int* BCIndex) {
  if (N < 1 || N > DG_MAX_N) { set_error("mesh: N out of range"); return DG_ERR_ARG; }
  if (!Mf || !Mg || !Mh || !sJ || !nvec || !t1vec || !t2vec || !surfelem || !E2S || !S2E) {
    set_error("dg_mesh_hopr: null argument"); return DG_ERR_ARG;
  }
  Hopr H;
  if (!read_hopr(path, H, true)) return DG_ERR_ARG;
  // ElemToSide(3,6,nElems): side (1-based), flip, master flag; SideToElem(5,nSides)
  for (int s = 0; s < H.nSides; ++s)
    for (int c = 0; c < 5; ++c) S2E[(size_t)s * 5 + c] = c >= 2 ? 0 : -1;
  for (int e = 0; e < H.nElems; ++e)
    for (int ls = 1; ls <= 6; ++ls) {
      const size_t slot = (size_t)e * 6 + ls - 1;
      int* p = E2S + 3 * slot;
      const int sd = H.side[slot];
      p[0] = sd + 1; p[1] = H.flip[slot]; p[2] = H.master[slot];
      int* q = S2E + 5 * (size_t)sd;
      if (H.master[slot]) { q[0] = e + 1; q[2] = ls; }
      else { q[1] = e + 1; q[3] = ls; q[4] = H.flip[slot]; }
      if (BCIndex && sd < H.nBCSides) BCIndex[sd] = H.bc[slot];
    }
  for (int s = 0; s < H.nSides; ++s) {
    int* q = S2E + 5 * (size_t)s;
    if (q[1] < 0) q[1] = 0;  // BC side: no neighbour
  }
  // geometry: CalcMetrics / CalcSurfMetrics / BuildCoords of the reference, element by element
  const int bad = gxh::metrics_from_nodes(N, node_type, H.NGeo, H.nElems, H.nodes.data(), E2S, elem_xgp, Mf, Mg, Mh, sJ,
                                          nvec, t1vec, t2vec, surfelem);
  if (bad != 0) {
    set_error(bad < 0 ? "HOPR mesh: negative Jacobian" : "HOPR mesh: scaled Jacobian below 0.01");
    return DG_ERR_ARG;
  }
  return DG_OK;
}
