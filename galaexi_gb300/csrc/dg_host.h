// Internal host helpers shared by the host set-up code and the CUDA context code.
#pragma once
#include <string>
#include <vector>

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
void set_error(const std::string& s);

}  // namespace gxh
