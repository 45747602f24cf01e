// flexi_gb300 -- host-side 1D polynomial toolbox used at set-up: Legendre-Gauss, Legendre-Gauss-Lobatto,
// Chebyshev-Gauss-Lobatto and equidistant node sets, barycentric Lagrange interpolation, nodal and
// modal (Legendre) Vandermonde matrices, derivative matrices. The node sets, their normalisation and
// the Newton iterations follow FLEXI's src/interpolation/basis.f90 (LegendreGaussNodesAndWeights :370,
// LegGaussLobNodesAndWeights :521, PolynomialDerivativeMatrix :619, LagrangeInterpolationPolys :679)
// and interpolation.f90:GetVandermonde :293 so that set-up matrices agree with the reference to
// round-off.
#pragma once
#include <cmath>
#include <stdexcept>
#include <vector>

namespace fgh {

enum Nodes { GAUSS = 1, LOBATTO = 2, CHEBLOB = 3, EQUI = 4 };

using Vec = std::vector<double>;

// small dense row-major matrix
struct Mat {
  int r = 0, c = 0;
  Vec a;
  Mat() = default;
  Mat(int r_, int c_, double v = 0.) : r(r_), c(c_), a((size_t)r_ * c_, v) {}
  double& operator()(int i, int j) { return a[(size_t)i * c + j]; }
  double operator()(int i, int j) const { return a[(size_t)i * c + j]; }
};
inline Mat matmul(const Mat& A, const Mat& B) {
  Mat C(A.r, B.c);
  for (int i = 0; i < A.r; ++i)
    for (int k = 0; k < A.c; ++k) {
      const double x = A(i, k);
      for (int j = 0; j < B.c; ++j) C(i, j) += x * B(k, j);
    }
  return C;
}

// Legendre polynomial of degree m at x, scaled by sqrt(m+1/2), and its derivative
inline void legendre(int m, double x, double& L, double& dL) {
  double l0 = 1., l1 = x, d1 = 1.;
  if (m == 0) { L = 1.; dL = 0.; }
  else if (m == 1) { L = x; dL = 1.; }
  else {
    for (int k = 2; k <= m; ++k) {
      const double lk = ((2. * k - 1.) * x * l1 - (k - 1.) * l0) / k;
      const double dk = k * l1 + x * d1;
      l0 = l1; l1 = lk; d1 = dk;
    }
    L = l1; dL = d1;
  }
  const double s = std::sqrt(m + 0.5);
  L *= s; dL *= s;
}

inline void nodes(int N, int type, Vec& x, Vec& w) {
  x.assign(N + 1, 0.); w.assign(N + 1, 0.);
  if (type == GAUSS) {
    if (N == 0) { w[0] = 2.; return; }
    if (N == 1) { x[0] = -std::sqrt(1. / 3.); x[1] = -x[0]; w[0] = w[1] = 1.; return; }
    const double h = 2. * std::atan(1.) / (N + 1);
    for (int i = 0; i <= (N + 1) / 2 - 1; ++i) {
      double xi = -std::cos(h * (2 * i + 1)), L, dL;
      for (int it = 0; it <= 10; ++it) {
        legendre(N + 1, xi, L, dL);
        const double dx = -L / dL;
        xi += dx;
        if (std::fabs(dx) < 1e-15 * std::fabs(xi)) break;
      }
      legendre(N + 1, xi, L, dL);
      x[i] = xi; x[N - i] = -xi;
      w[i] = w[N - i] = (2. * N + 3.) / ((1. - xi * xi) * dL * dL);
    }
    if (N % 2 == 0) { double L, dL; legendre(N + 1, 0., L, dL); x[N / 2] = 0.; w[N / 2] = (2. * N + 3.) / (dL * dL); }
  } else if (type == LOBATTO) {
    x[0] = -1.; x[N] = 1.; w[0] = w[N] = 2. / (N * (N + 1.));
    // q = L_{N+1} - L_{N-1} (unscaled), its roots are the inner LGL nodes
    auto qeval = [N](double xx, double& q, double& dq, double& LN) {
      double l0 = 1., l1 = xx;
      for (int k = 2; k <= N; ++k) { const double lk = ((2. * k - 1.) * xx * l1 - (k - 1.) * l0) / k; l0 = l1; l1 = lk; }
      LN = l1;
      q = (2. * N + 1.) / (N + 1.) * (xx * l1 - l0);
      dq = (2. * N + 1.) * l1;
    };
    for (int i = 1; i <= (N + 1) / 2 - 1; ++i) {
      double xi = -std::cos(M_PI / N * (i + 0.25) - 3. / (8. * N * M_PI) / (i + 0.25)), q, dq, LN;
      for (int it = 0; it <= 10; ++it) {
        qeval(xi, q, dq, LN);
        const double dx = -q / dq;
        xi += dx;
        if (std::fabs(dx) < 1e-15 * std::fabs(xi)) break;
      }
      qeval(xi, q, dq, LN);
      x[i] = xi; x[N - i] = -xi;
      w[i] = w[N - i] = w[0] / (LN * LN);
    }
    if (N % 2 == 0) { double q, dq, LN; qeval(0., q, dq, LN); x[N / 2] = 0.; w[N / 2] = w[0] / (LN * LN); }
  } else if (type == CHEBLOB) {
    for (int i = 0; i <= N; ++i) { x[i] = -std::cos(i / (double)N * M_PI); w[i] = M_PI / N; }
    w[0] *= 0.5; w[N] *= 0.5;
  } else if (type == EQUI) {
    for (int i = 0; i <= N; ++i) { x[i] = 2. * i / (double)N - 1.; w[i] = 2. / N; }
    w[0] *= 0.5; w[N] *= 0.5;
  } else throw std::runtime_error("unknown node type");
}

inline Vec bary_weights(const Vec& x) {
  const int n = (int)x.size();
  Vec wb(n, 1.);
  for (int i = 1; i < n; ++i)
    for (int j = 0; j < i; ++j) { wb[j] *= (x[j] - x[i]); wb[i] *= (x[i] - x[j]); }
  for (double& v : wb) v = 1. / v;
  return wb;
}

// values of the Lagrange polynomials of the nodes x at the point xp
inline Vec lagrange_at(double xp, const Vec& x, const Vec& wb) {
  const int n = (int)x.size();
  Vec L(n, 0.);
  const double eps = 2.220446049250313e-16;
  bool hit = false;
  for (int i = 0; i < n; ++i) {
    const double a = xp, b = x[i];
    const bool eq = (a == 0. || b == 0.) ? std::fabs(a - b) <= 2. * eps
                                         : (std::fabs(a - b) <= eps * std::fabs(a) && std::fabs(a - b) <= eps * std::fabs(b));
    if (eq) { L[i] = 1.; hit = true; }
  }
  if (hit) return L;
  double s = 0.;
  for (int i = 0; i < n; ++i) { L[i] = wb[i] / (xp - x[i]); s += L[i]; }
  for (double& v : L) v /= s;
  return L;
}

// interpolation matrix from nodes xin to points xout: (nout x nin)
inline Mat interp_matrix(const Vec& xin, const Vec& xout) {
  const Vec wb = bary_weights(xin);
  Mat V((int)xout.size(), (int)xin.size());
  for (int o = 0; o < V.r; ++o) {
    const Vec L = lagrange_at(xout[o], xin, wb);
    for (int i = 0; i < V.c; ++i) V(o, i) = L[i];
  }
  return V;
}

inline Mat inverse(const Mat& A) {
  const int n = A.r;
  Mat a = A, inv(n, n);
  for (int i = 0; i < n; ++i) inv(i, i) = 1.;
  for (int c = 0; c < n; ++c) {
    int p = c;
    for (int r = c + 1; r < n; ++r) if (std::fabs(a(r, c)) > std::fabs(a(p, c))) p = r;
    if (p != c) for (int k = 0; k < n; ++k) { std::swap(a(p, k), a(c, k)); std::swap(inv(p, k), inv(c, k)); }
    const double dinv = 1. / a(c, c);
    for (int k = 0; k < n; ++k) { a(c, k) *= dinv; inv(c, k) *= dinv; }
    for (int r = 0; r < n; ++r) if (r != c) {
      const double f = a(r, c);
      if (f != 0.) for (int k = 0; k < n; ++k) { a(r, k) -= f * a(c, k); inv(r, k) -= f * inv(c, k); }
    }
  }
  return inv;
}

// Vandermonde matrix from (Nin, typeIn) to (Nout, typeOut). With modal=true and Nout < Nin the map is the
// L2 projection through the Legendre modes (a cut-off), otherwise plain interpolation.
inline Mat vandermonde(int Nin, int typeIn, int Nout, int typeOut, bool modal) {
  if (Nin == Nout && typeIn == typeOut) { Mat I(Nin + 1, Nin + 1); for (int i = 0; i <= Nin; ++i) I(i, i) = 1.; return I; }
  Vec xi, wi, xo, wo;
  nodes(Nin, typeIn, xi, wi);
  nodes(Nout, typeOut, xo, wo);
  if (modal && Nout < Nin) {
    Mat Vin(Nin + 1, Nin + 1), Vout(Nout + 1, Nout + 1);
    double dL;
    for (int i = 0; i <= Nin; ++i) for (int m = 0; m <= Nin; ++m) legendre(m, xi[i], Vin(i, m), dL);
    for (int i = 0; i <= Nout; ++i) for (int m = 0; m <= Nout; ++m) legendre(m, xo[i], Vout(i, m), dL);
    const Mat sVin = inverse(Vin);  // nodal -> modal
    Mat cut(Nout + 1, Nin + 1);
    for (int m = 0; m <= Nout; ++m) for (int i = 0; i <= Nin; ++i) cut(m, i) = sVin(m, i);
    return matmul(Vout, cut);
  }
  return interp_matrix(xi, xo);
}

// derivative matrix D(i,l) = l_l'(x_i), barycentric form with the negative-sum trick for the diagonal
inline Mat diff_matrix(const Vec& x) {
  const int n = (int)x.size();
  const Vec wb = bary_weights(x);
  Mat D(n, n);
  for (int l = 0; l < n; ++l)
    for (int i = 0; i < n; ++i)
      if (l != i) { D(i, l) = wb[l] / (wb[i] * (x[i] - x[l])); D(i, i) -= D(i, l); }
  return D;
}
inline Mat diff_matrix(int N, int type) { Vec x, w; nodes(N, type, x, w); return diff_matrix(x); }

}  // namespace fgh
