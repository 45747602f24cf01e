// TEST INFRASTRUCTURE ONLY -- part of the CPU oracle (restatement of FLEXI v25.10) used by tests/,
// __graft_entry__.smoke() and bench.py's cpu_baseline leg as the checker. Never linked into the product.
//
// Polynomial basis of the DGSEM: nodes, weights, barycentric weights, Lagrange polynomials,
// Vandermonde matrices (nodal and modal), derivative matrices.
// Restates src/interpolation/basis.f90 and src/interpolation/interpolation.f90 (FLEXI v25.10).
#pragma once
#include <cmath>
#include <vector>
#include <stdexcept>
#include <string>

namespace orc {

enum NodeTypeId { NT_GAUSS = 1, NT_GL = 2, NT_CL = 3, NT_VISU = 4 };

// basis.f90:LegendrePolynomialAndDerivative -- normalised Legendre polynomial L_N(x)*sqrt(N+1/2) and derivative.
inline void legendre_poly_and_deriv(int N, double x, double& L, double& Lder) {
  if (N == 0) { L = 1.; Lder = 0.; }
  else if (N == 1) { L = x; Lder = 1.; }
  else {
    double Lm2 = 1., Lm1 = x, Ldm2 = 0., Ldm1 = 1.;
    for (int iL = 2; iL <= N; ++iL) {
      L = ((2. * iL - 1.) * x * Lm1 - (iL - 1.) * Lm2) / (double)iL;
      Lder = iL * Lm1 + x * Ldm1;
      Lm2 = Lm1; Lm1 = L; Ldm2 = Ldm1; Ldm1 = Lder;
    }
  }
  L *= std::sqrt(N + 0.5);
  Lder *= std::sqrt(N + 0.5);
}

// basis.f90:qAndLEvaluation -- q = L_{N+1}-L_{N-1}, q', L_N (unnormalised), for Gauss-Lobatto nodes.
inline void q_and_l(int N, double x, double& q, double& qder, double& L) {
  double Lm2 = 1., Lm1 = x;
  for (int iL = 2; iL <= N; ++iL) {
    L = ((2. * iL - 1.) * x * Lm1 - (iL - 1.) * Lm2) / (double)iL;
    Lm2 = Lm1; Lm1 = L;
  }
  q = (2. * N + 1.) / (N + 1.) * (x * L - Lm2);
  qder = (2. * N + 1.) * L;
}

// basis.f90:LegendreGaussNodesAndWeights (Newton on L_{N+1}, Chebyshev initial guess)
inline void gauss_nodes(int N, double* x, double* w) {
  if (N == 0) { x[0] = 0.; w[0] = 2.; return; }
  if (N == 1) { x[0] = -std::sqrt(1. / 3.); x[1] = -x[0]; w[0] = w[1] = 1.; return; }
  const double cheb = 2. * std::atan(1.) / (double)(N + 1);
  for (int i = 0; i <= (N + 1) / 2 - 1; ++i) {
    x[i] = -std::cos(cheb * (2 * i + 1));
    double L, Ld;
    for (int it = 0; it <= 10; ++it) {
      legendre_poly_and_deriv(N + 1, x[i], L, Ld);
      double dx = -L / Ld;
      x[i] += dx;
      if (std::fabs(dx) < 1e-15 * std::fabs(x[i])) break;
    }
    legendre_poly_and_deriv(N + 1, x[i], L, Ld);
    x[N - i] = -x[i];
    w[i] = (2. * N + 3.) / ((1. - x[i] * x[i]) * Ld * Ld);
    w[N - i] = w[i];
  }
  if (N % 2 == 0) {
    double L, Ld;
    x[N / 2] = 0.;
    legendre_poly_and_deriv(N + 1, 0., L, Ld);
    w[N / 2] = (2. * N + 3.) / (Ld * Ld);
  }
}

// basis.f90:LegGaussLobNodesAndWeights
inline void gl_nodes(int N, double* x, double* w) {
  x[0] = -1.; x[N] = 1.;
  w[0] = 2. / (double)(N * (N + 1)); w[N] = w[0];
  if (N > 1) {
    const double c1 = M_PI / (double)N, c2 = 3. / ((double)(8 * N) * M_PI);
    for (int i = 1; i <= (N + 1) / 2 - 1; ++i) {
      x[i] = -std::cos(c1 * (i + 0.25) - c2 / (i + 0.25));
      double q, qd, L;
      for (int it = 0; it <= 10; ++it) {
        q_and_l(N, x[i], q, qd, L);
        double dx = -q / qd;
        x[i] += dx;
        if (std::fabs(dx) < 1e-15 * std::fabs(x[i])) break;
      }
      q_and_l(N, x[i], q, qd, L);
      x[N - i] = -x[i];
      w[i] = w[0] / (L * L);
      w[N - i] = w[i];
    }
  }
  if (N % 2 == 0) {
    double q, qd, L;
    x[N / 2] = 0.;
    q_and_l(N, 0., q, qd, L);
    w[N / 2] = w[0] / (L * L);
  }
}

// basis.f90:ChebyGaussLobNodesAndWeights
inline void cl_nodes(int N, double* x, double* w) {
  for (int i = 0; i <= N; ++i) { x[i] = -std::cos(i / (double)N * M_PI); w[i] = M_PI / (double)N; }
  w[0] *= 0.5; w[N] *= 0.5;
}

// interpolation.f90:GetNodesAndWeights, 'visu' branch (equidistant)
inline void visu_nodes(int N, double* x, double* w) {
  for (int i = 0; i <= N; ++i) { x[i] = 2. * i / (double)N - 1.; w[i] = 2. / (double)N; }
  w[0] *= 0.5; w[N] *= 0.5;
}

// basis.f90:BarycentricWeights
inline void barycentric_weights(int N, const double* x, double* wb) {
  for (int i = 0; i <= N; ++i) wb[i] = 1.;
  for (int i = 1; i <= N; ++i)
    for (int j = 0; j <= i - 1; ++j) { wb[j] *= (x[j] - x[i]); wb[i] *= (x[i] - x[j]); }
  for (int i = 0; i <= N; ++i) wb[i] = 1. / wb[i];
}

// interpolation.f90:GetNodesAndWeights
inline void nodes_and_weights(int N, int type, double* x, double* w, double* wb) {
  std::vector<double> wt(N + 1);
  double* ww = w ? w : wt.data();
  switch (type) {
    case NT_GAUSS: gauss_nodes(N, x, ww); break;
    case NT_GL: gl_nodes(N, x, ww); break;
    case NT_CL: cl_nodes(N, x, ww); break;
    case NT_VISU: visu_nodes(N, x, ww); break;
    default: throw std::runtime_error("unknown node type");
  }
  if (wb) barycentric_weights(N, x, wb);
}

// basis.f90:PolynomialDerivativeMatrix ; D is (N+1)x(N+1), D[i*(N+1)+l] = D(i,l)
inline void derivative_matrix(int N, const double* x, double* D) {
  std::vector<double> wb(N + 1);
  barycentric_weights(N, x, wb.data());
  const int n = N + 1;
  for (int i = 0; i < n * n; ++i) D[i] = 0.;
  for (int l = 0; l <= N; ++l)
    for (int i = 0; i <= N; ++i)
      if (l != i) {
        D[i * n + l] = wb[l] / (wb[i] * (x[i] - x[l]));
        D[i * n + i] -= D[i * n + l];
      }
}

// basis.f90:ALMOSTEQUAL with PP_RealTolerance = EPSILON(1.d0)
inline bool almost_equal(double x, double y) {
  const double tol = 2.220446049250313e-16;
  if (x == 0. || y == 0.) return std::fabs(x - y) <= 2. * tol;
  return std::fabs(x - y) <= tol * std::fabs(x) && std::fabs(x - y) <= tol * std::fabs(y);
}

// basis.f90:LagrangeInterpolationPolys (barycentric form)
inline void lagrange_polys(double x, int N, const double* xGP, const double* wb, double* L) {
  bool eq = false;
  for (int i = 0; i <= N; ++i) {
    L[i] = 0.;
    if (almost_equal(x, xGP[i])) { L[i] = 1.; eq = true; }
  }
  if (eq) return;
  double s = 0.;
  for (int i = 0; i <= N; ++i) { L[i] = wb[i] / (x - xGP[i]); s += L[i]; }
  for (int i = 0; i <= N; ++i) L[i] /= s;
}

// basis.f90:InitializeVandermonde; Vdm is (Nout+1)x(Nin+1) row-major: Vdm[o*(Nin+1)+i]
inline std::vector<double> init_vandermonde(int Nin, int Nout, const double* wbIn, const double* xIn, const double* xOut) {
  std::vector<double> V((Nout + 1) * (Nin + 1));
  for (int o = 0; o <= Nout; ++o) lagrange_polys(xOut[o], Nin, xIn, wbIn, &V[o * (Nin + 1)]);
  return V;
}

// Gauss-Jordan inverse with partial pivoting (stands in for the LAPACK call in globals/lapack.f90)
inline std::vector<double> mat_inverse(const std::vector<double>& A, int n) {
  std::vector<double> a(A), inv(n * n, 0.);
  for (int i = 0; i < n; ++i) inv[i * n + i] = 1.;
  for (int c = 0; c < n; ++c) {
    int p = c;
    for (int r = c + 1; r < n; ++r) if (std::fabs(a[r * n + c]) > std::fabs(a[p * n + c])) p = r;
    if (p != c) for (int k = 0; k < n; ++k) { std::swap(a[p * n + k], a[c * n + k]); std::swap(inv[p * n + k], inv[c * n + k]); }
    double d = a[c * n + c];
    for (int k = 0; k < n; ++k) { a[c * n + k] /= d; inv[c * n + k] /= d; }
    for (int r = 0; r < n; ++r) if (r != c) {
      double f = a[r * n + c];
      if (f != 0.) for (int k = 0; k < n; ++k) { a[r * n + k] -= f * a[c * n + k]; inv[r * n + k] -= f * inv[c * n + k]; }
    }
  }
  return inv;
}

// basis.f90:buildLegendreVdm -- Vdm_Leg(i,j) = L_j(xi_i), sVdm_Leg = inverse
inline void legendre_vdm(int N, const double* xi, std::vector<double>& V, std::vector<double>& sV) {
  const int n = N + 1;
  V.assign(n * n, 0.);
  for (int i = 0; i < n; ++i) for (int j = 0; j < n; ++j) { double d; legendre_poly_and_deriv(j, xi[i], V[i * n + j], d); }
  sV = mat_inverse(V, n);
}

// interpolation.f90:GetVandermonde (Vdm_In_Out only); returns (Nout+1)x(Nin+1)
inline std::vector<double> get_vandermonde(int Nin, int typeIn, int Nout, int typeOut, bool modal) {
  std::vector<double> V((Nout + 1) * (Nin + 1), 0.);
  if (typeIn == typeOut && Nin == Nout) {
    for (int i = 0; i <= Nin; ++i) V[i * (Nin + 1) + i] = 1.;
    return V;
  }
  std::vector<double> xi(Nin + 1), wb(Nin + 1), xo(Nout + 1);
  nodes_and_weights(Nin, typeIn, xi.data(), nullptr, wb.data());
  nodes_and_weights(Nout, typeOut, xo.data(), nullptr, nullptr);
  if (Nout < Nin && modal) {
    std::vector<double> VLi, sVLi, VLo, sVLo;
    legendre_vdm(Nin, xi.data(), VLi, sVLi);
    legendre_vdm(Nout, xo.data(), VLo, sVLo);
    // Vdm_In_Out = Vdm_Leg_Out(0:Nout,0:Nout) * sVdm_Leg_In(0:Nout,0:Nin)
    for (int o = 0; o <= Nout; ++o)
      for (int i = 0; i <= Nin; ++i) {
        double s = 0.;
        for (int m = 0; m <= Nout; ++m) s += VLo[o * (Nout + 1) + m] * sVLi[m * (Nin + 1) + i];
        V[o * (Nin + 1) + i] = s;
      }
    return V;
  }
  return init_vandermonde(Nin, Nout, wb.data(), xi.data(), xo.data());
}

inline std::vector<double> get_derivative_matrix(int N, int type) {
  std::vector<double> x(N + 1), D((N + 1) * (N + 1));
  nodes_and_weights(N, type, x.data(), nullptr, nullptr);
  derivative_matrix(N, x.data(), D.data());
  return D;
}

// DG building blocks of dg.f90:InitDGBasis (weak and split forms) + L_Minus/L_Plus of interpolation.f90:InitInterpolationBasis
struct DGBasis {
  int N = 0, n = 0, nodeType = NT_GAUSS;
  std::vector<double> xGP, wGP, wBary, Lm, Lp, LhatM, LhatP;
  std::vector<double> D, D_T, Dhat, Dhat_T, DVolSurf;  // n*n row-major, X[i*n+l] = X(i,l) in Fortran indices (0-based)
  void init(int N_, int nt) {
    N = N_; n = N + 1; nodeType = nt;
    xGP.resize(n); wGP.resize(n); wBary.resize(n); Lm.resize(n); Lp.resize(n); LhatM.resize(n); LhatP.resize(n);
    nodes_and_weights(N, nt, xGP.data(), wGP.data(), wBary.data());
    lagrange_polys(1., N, xGP.data(), wBary.data(), Lp.data());
    lagrange_polys(-1., N, xGP.data(), wBary.data(), Lm.data());
    D.resize(n * n); derivative_matrix(N, xGP.data(), D.data());
    D_T.resize(n * n); Dhat.resize(n * n); Dhat_T.resize(n * n); DVolSurf.resize(n * n);
    for (int i = 0; i < n; ++i) for (int l = 0; l < n; ++l) D_T[i * n + l] = D[l * n + i];
    // D_Hat = -Minv * D^T * M (M diagonal with wGP)
    for (int i = 0; i < n; ++i) for (int l = 0; l < n; ++l) Dhat[i * n + l] = -(1. / wGP[i]) * D[l * n + i] * wGP[l];
    for (int i = 0; i < n; ++i) for (int l = 0; l < n; ++l) Dhat_T[i * n + l] = Dhat[l * n + i];
    if (nt == NT_GL) {
      DVolSurf = D_T;
      DVolSurf[0] += 1.0 / (2.0 * wGP[0]);
      DVolSurf[N * n + N] -= 1.0 / (2.0 * wGP[N]);
    } else {
      // S = D - 1/2 * Minv * Vf^T B Vf ; Vf rows = L_Minus, L_Plus ; B = diag(-1,1); then transpose
      std::vector<double> S(n * n);
      for (int i = 0; i < n; ++i) for (int l = 0; l < n; ++l)
        S[i * n + l] = D[i * n + l] - 0.5 * (1. / wGP[i]) * (-Lm[i] * Lm[l] + Lp[i] * Lp[l]);
      for (int i = 0; i < n; ++i) for (int l = 0; l < n; ++l) DVolSurf[i * n + l] = S[l * n + i];
    }
    for (int i = 0; i < n; ++i) { LhatP[i] = Lp[i] / wGP[i]; LhatM[i] = Lm[i] / wGP[i]; }
  }
};

}  // namespace orc
