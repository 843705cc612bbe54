// Internal host helpers shared by the host set-up code and the CUDA context code.
#pragma once
#include <string>
#include <vector>

#include "../../include/galaexi_gb300.h"

namespace gxh {

// 1D basis of degree N on one node set (column-major (0:N,0:N) matrices)
struct Basis1D {
  int N = 0;
  std::vector<double> x, w, wb;     // nodes, quadrature weights, barycentric weights
  std::vector<double> D;            // D(i,l) = l_l'(x_i)
  std::vector<double> DhatT;        // D_hat^T(l,i), D_hat = -M^{-1} D^T M
  std::vector<double> DVS;          // DVolSurf(l,i)
  std::vector<double> Lm, Lp;       // l_j(-1), l_j(+1)
  std::vector<double> Lhm, Lhp;     // M^{-1} L_minus, M^{-1} L_plus
};
inline double D_at(const Basis1D& B, int i, int l) { return B.D[i + (B.N + 1) * l]; }

void basis_1d(int N, int node_type, Basis1D& B);
// FilterMat (0:N,0:N) of the configured filter type (column-major); -1 if the configuration is invalid
int filter_matrix(const dg_config& c, std::vector<double>& F);
void set_error(const std::string& s);

// Lagrange interpolation matrix V(j,i) = l_i(y_j) from the N+1 nodes x (barycentric weights wb) to
// the M+1 points y, column-major (0:M, 0:N)
void vandermonde(int N, const double* x, const double* wb, int M, const double* y, std::vector<double>& V);
inline size_t vidx(int n, int i, int j, int k, int e) { return (size_t)i + n * (j + n * (k + (size_t)n * e)); }
// modal projection (Legendre modes 0..M) from degree N on the nodes x to degree M < N on the points y,
// column-major (0:M, 0:N)
void modal_projection(int N, const double* x, const double* wb, int M, const double* y, std::vector<double>& V);
// BuildCoords + CalcMetrics + CalcSurfMetrics (dg_hopr.cpp) from the equidistant element node coordinates
// nodes (3,0:NGeo,0:NGeo,0:NGeo,nElems) and ElemToSide (3,6,nElems, 1-based side IDs); the master
// sides (flip 0) receive the side vectors.  elem_xgp may be null.  Returns the count of solution nodes
// with a scaled Jacobian below 0.01, or -1 for a non-positive Jacobian.
int metrics_from_nodes(int N, int node_type, int NGeo, int nElems, const double* nodes, const int* E2S,
                       double* elem_xgp, double* Mf, double* Mg, double* Mh, double* sJ, double* nvec,
                       double* t1vec, double* t2vec, double* surfelem);
// normal, tangents and surface element of a master side from the element's face metric terms
void surface_metrics(int N, int loc, const double* JaFace, size_t side, double* nvec, double* t1vec, double* t2vec,
                     double* surfelem);

}  // namespace gxh
