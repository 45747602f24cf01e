// flexi_gb300 -- host-side mesh preparation (see fg_mesh.hpp).
#include "fg_mesh.hpp"
#include <algorithm>
#include <array>
#include <cstring>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace fgh {

namespace {

enum { ZM = 1, EM = 2, XP = 3, EP = 4, XM = 5, ZP = 6 };  // FLEXI local side ids

// mappings.f90: Flip_S2M / CGNS_SideToVol2
void flip_map(int N, int p, int q, int flip, int& a, int& b) {
  switch (flip) {
    case 0: a = p; b = q; break;
    case 1: a = q; b = p; break;
    case 2: a = N - p; b = q; break;
    case 3: a = N - q; b = N - p; break;
    default: a = p; b = N - q;
  }
}
void s2v2(int N, int p, int q, int flip, int ls, int& a, int& b) {
  int x, y;
  flip_map(N, p, q, flip, x, y);
  switch (ls) {
    case XM: case ZM: a = y; b = x; break;
    case EP: a = N - x; b = y; break;
    default: a = x; b = y;
  }
}
// node (i,j,k) of face coordinate (a,b) at volume index l along the face normal
inline void face_ijk(int ls, int a, int b, int l, int& i, int& j, int& k) {
  if (ls == XM || ls == XP) { i = l; j = a; k = b; }
  else if (ls == EM || ls == EP) { i = a; j = l; k = b; }
  else { i = a; j = b; k = l; }
}
inline bool minus_side(int ls) { return ls == XM || ls == EM || ls == ZM; }
// normal direction (0-based) and first tangential direction of a local side, mesh_vars.f90:105-111
const int kNormalDir[7] = {0, 2, 1, 0, 1, 0, 2};
const int kTangDir[7] = {0, 0, 2, 1, 2, 1, 0};
const double kNormalSign[7] = {0., -1., -1., 1., 1., -1., 1.};

// applies V (no x ni) along all three directions of a component-major array X[c][k][j][i] (ni^3 per component)
void tensor3(const Mat& V, const double* in, double* out, int nc) {
  const int ni = V.c, no = V.r;
  std::vector<double> t1((size_t)ni * ni * no), t2((size_t)ni * no * no);
  for (int c = 0; c < nc; ++c) {
    const double* X = in + (size_t)c * ni * ni * ni;
    double* Y = out + (size_t)c * no * no * no;
    for (int kj = 0; kj < ni * ni; ++kj)
      for (int a = 0; a < no; ++a) {
        double s = 0.;
        for (int i = 0; i < ni; ++i) s += V(a, i) * X[(size_t)kj * ni + i];
        t1[(size_t)kj * no + a] = s;
      }
    for (int k = 0; k < ni; ++k)
      for (int b = 0; b < no; ++b)
        for (int a = 0; a < no; ++a) {
          double s = 0.;
          for (int j = 0; j < ni; ++j) s += V(b, j) * t1[((size_t)k * ni + j) * no + a];
          t2[((size_t)k * no + b) * no + a] = s;
        }
    for (int cc = 0; cc < no; ++cc)
      for (int ba = 0; ba < no * no; ++ba) {
        double s = 0.;
        for (int k = 0; k < ni; ++k) s += V(cc, k) * t2[(size_t)k * no * no + ba];
        Y[(size_t)cc * no * no + ba] = s;
      }
  }
}
// 2D version on X[c][b][a]
void tensor2(const Mat& V, const double* in, double* out, int nc) {
  const int ni = V.c, no = V.r;
  std::vector<double> t1((size_t)ni * no);
  for (int c = 0; c < nc; ++c) {
    const double* X = in + (size_t)c * ni * ni;
    double* Y = out + (size_t)c * no * no;
    for (int j = 0; j < ni; ++j)
      for (int a = 0; a < no; ++a) {
        double s = 0.;
        for (int i = 0; i < ni; ++i) s += V(a, i) * X[(size_t)j * ni + i];
        t1[(size_t)j * no + a] = s;
      }
    for (int b = 0; b < no; ++b)
      for (int a = 0; a < no; ++a) {
        double s = 0.;
        for (int j = 0; j < ni; ++j) s += V(b, j) * t1[(size_t)j * no + a];
        Y[(size_t)b * no + a] = s;
      }
  }
}
// derivative along direction dir of X[c][k][j][i] with the (n x n) matrix D(i,l)
void deriv3(const Mat& D, const double* X, double* out, int dir) {
  const int n = D.r;
  for (int k = 0; k < n; ++k)
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        double s = 0.;
        for (int l = 0; l < n; ++l) {
          const int x = dir == 0 ? l + n * (j + n * k) : (dir == 1 ? i + n * (l + n * k) : i + n * (j + n * l));
          s += D(dir == 0 ? i : (dir == 1 ? j : k), l) * X[x];
        }
        out[i + n * (j + n * k)] = s;
      }
}

// metrics.f90:SurfMetricsFromJa at one side point: unit normal (sign of local side ls), tangents and surface
// element from the normal row jn and the tangential row jt of the face metrics; G = field 0 of the point
// in a [10][n2] side block
void surf_point(const double* jn, const double* jt, int ls, double* G, int n2) {
  const double se = std::sqrt(jn[0] * jn[0] + jn[1] * jn[1] + jn[2] * jn[2]);
  double nv[3], t1[3], t2[3];
  for (int c = 0; c < 3; ++c) nv[c] = kNormalSign[ls] * jn[c] / se;
  const double dt = jt[0] * nv[0] + jt[1] * nv[1] + jt[2] * nv[2];
  for (int c = 0; c < 3; ++c) t1[c] = jt[c] - dt * nv[c];
  const double tl = std::sqrt(t1[0] * t1[0] + t1[1] * t1[1] + t1[2] * t1[2]);
  for (int c = 0; c < 3; ++c) t1[c] /= tl;
  t2[0] = nv[1] * t1[2] - nv[2] * t1[1];
  t2[1] = nv[2] * t1[0] - nv[0] * t1[2];
  t2[2] = nv[0] * t1[1] - nv[1] * t1[0];
  for (int c = 0; c < 3; ++c) { G[c * n2] = nv[c]; G[(3 + c) * n2] = t1[c]; G[(6 + c) * n2] = t2[c]; }
  G[9 * n2] = se;
}

}  // namespace

void build_from_raw(const RawMesh& R, int N, int nodeType, HostMesh& M) {
  const int nE = R.nElems, NG = R.NGeo, ng = NG + 1, n = N + 1, n2 = n * n, n3 = n2 * n;
  M.N = N; M.n = n; M.nodeType = nodeType; M.nElems = nE;
  auto nb = [&](int c, int ls, int e) { return R.elemNb[((size_t)e * 6 + (ls - 1)) * 3 + c]; };
  auto X = [&](int d, int i, int j, int k, int e) { return R.nodeCoords[((((size_t)e * ng + k) * ng + j) * ng + i) * 3 + d]; };

  // ---------------- sides: BC | conforming inner | small mortar | big mortar ----------------
  struct SideRec { int e, ls, ne, nls, bc; };
  std::vector<SideRec> bcs, inner;
  int nMortarSides = 0;  // element sides with neighbour -1 (big and small mortar sides)
  for (int e = 0; e < nE; ++e)
    for (int ls = 1; ls <= 6; ++ls) {
      const int ne = nb(0, ls, e);
      if (ne == 0) { bcs.push_back({e, ls, -1, 0, nb(2, ls, e)}); continue; }
      if (ne == -1) { ++nMortarSides; continue; }
      if (ne < 0 || ne > nE) throw std::runtime_error("neighbour element out of range");
      const int oe = ne - 1, ols = nb(1, ls, e);
      if (e < oe || (e == oe && ls < ols)) inner.push_back({e, ls, oe, ols, 0});
    }
  const int nMo = R.nMortars;
  int nSmall = 0;
  for (int m = 0; m < nMo; ++m) {
    const int type = R.mortars[(size_t)m * 15 + 2];
    if (type < 1 || type > 3) throw std::runtime_error("mortar type must be 1, 2 or 3");
    nSmall += type == 1 ? 4 : 2;
  }
  if (nMortarSides != nMo + nSmall) throw std::runtime_error("mortar sides (neighbour -1) do not match the Mortars table");
  M.nBCSides = (int)bcs.size();
  M.nFluxSides = M.nBCSides + (int)inner.size();
  M.nMortars = nMo;
  M.flexiSide.clear();
  M.nSides = M.nFluxSides + nSmall + nMo;
  M.sideElem.assign((size_t)M.nSides * 4, -1);
  M.elemSide.assign((size_t)nE * 6, 0);
  M.bcType.assign(M.nBCSides, 0);
  M.bcTwall.assign(M.nBCSides, 0.);
  for (int s = 0; s < M.nBCSides; ++s) {
    const SideRec& r = bcs[s];
    M.sideElem[s * 4 + 0] = r.e; M.sideElem[s * 4 + 1] = r.ls; M.sideElem[s * 4 + 2] = -1; M.sideElem[s * 4 + 3] = 0;
    M.elemSide[r.e * 6 + r.ls - 1] = 8 * s;
    if (r.bc < 1 || r.bc > R.nBCs) throw std::runtime_error("boundary side without a valid BC index");
    const int bt = R.boundaryType[(r.bc - 1) * 2 + 0], bs = R.boundaryType[(r.bc - 1) * 2 + 1];
    if (bt != 3 && bt != 4) throw std::runtime_error("only no-slip wall boundaries (types 3, 4) and periodic connections are supported");
    M.bcType[s] = bt;
    if (bt == 4) {
      if (bs < 1 || bs > R.nRefStates) throw std::runtime_error("isothermal wall needs a RefState");
      M.bcTwall[s] = R.refStatePrim[(bs - 1) * 6 + 5];
    }
  }
  // orientation of the slave: the flip that makes the four corner nodes coincide up to one translation
  auto corner = [&](int e, int ls, int p, int q, double* x) {
    int a, b, i, j, k;
    s2v2(NG, p, q, 0, ls, a, b);
    face_ijk(ls, a, b, minus_side(ls) ? 0 : NG, i, j, k);
    for (int d = 0; d < 3; ++d) x[d] = X(d, i, j, k, e);
  };
  // flip of the slave face (ne, nls) whose corners coincide with the master corners xm[c] (c = p + 2q over
  // the side's corner nodes) up to one constant (periodic) shift; -1 if none does
  auto match_flip = [&](const double (*xm)[3], int ne, int nls) {
    for (int f = 1; f <= 4; ++f) {
      bool ok = true;
      double sh[3] = {0., 0., 0.};
      for (int c = 0; c < 4 && ok; ++c) {
        const int p = (c & 1) ? NG : 0, q = (c & 2) ? NG : 0;
        double xs[3];
        int pa, qa;
        flip_map(NG, p, q, f, pa, qa);
        corner(ne, nls, pa, qa, xs);
        for (int dd = 0; dd < 3; ++dd) {
          const double dv = xs[dd] - xm[c][dd];
          if (c == 0) sh[dd] = dv;
          else if (std::fabs(dv - sh[dd]) > 1e-9 * (1. + std::fabs(sh[dd]))) ok = false;
        }
      }
      if (ok) return f;
    }
    return -1;
  };
  for (size_t t = 0; t < inner.size(); ++t) {
    const SideRec& r = inner[t];
    const int s = M.nBCSides + (int)t;
    double xm[4][3];
    for (int c = 0; c < 4; ++c) corner(r.e, r.ls, (c & 1) ? NG : 0, (c & 2) ? NG : 0, xm[c]);
    const int found = match_flip(xm, r.ne, r.nls);
    if (found < 0) throw std::runtime_error("neighbouring faces do not match geometrically");
    M.sideElem[s * 4 + 0] = r.e; M.sideElem[s * 4 + 1] = r.ls; M.sideElem[s * 4 + 2] = r.ne; M.sideElem[s * 4 + 3] = 8 * r.nls + found;
    M.elemSide[r.e * 6 + r.ls - 1] = 8 * s;
    M.elemSide[r.ne * 6 + r.nls - 1] = 8 * s + found;
  }
  // mortar sides (mesh_readin.f90 / prepare_mesh.f90: MortarType, MortarInfo). The big side has the big
  // element as master and no slave. Small side im covers quadrant (iNb, jNb) of the big side in its master
  // orientation; its master slot is filled from the big side (U_Mortar), so its master element is the big
  // element (viscosity, instance) and the small element is the slave, flip from the quadrant corners.
  M.mortarInfo.assign((size_t)6 * nMo, -1);
  {
    const int firstBig = M.nSides - nMo;
    Vec xe(ng);
    for (int a = 0; a < ng; ++a) xe[a] = -1. + 2. * a / NG;
    const Vec wbe = bary_weights(xe);
    std::vector<char> used((size_t)6 * nE, 0);
    auto take = [&](int e, int ls) {
      if (e < 0 || e >= nE || ls < 1 || ls > 6 || nb(0, ls, e) != -1 || used[(size_t)e * 6 + ls - 1])
        throw std::runtime_error("mortar table names a side that is not an unused mortar side");
      used[(size_t)e * 6 + ls - 1] = 1;
    };
    int s = M.nFluxSides;
    for (int m = 0; m < nMo; ++m) {
      const int* r = &R.mortars[(size_t)m * 15];
      const int be = r[0] - 1, bls = r[1], type = r[2], nm = type == 1 ? 4 : 2, sb = firstBig + m;
      take(be, bls);
      M.sideElem[sb * 4 + 0] = be; M.sideElem[sb * 4 + 1] = bls; M.sideElem[sb * 4 + 2] = -1; M.sideElem[sb * 4 + 3] = 0;
      M.elemSide[be * 6 + bls - 1] = 8 * sb;
      M.mortarInfo[(size_t)m * 6 + 0] = type;
      M.mortarInfo[(size_t)m * 6 + 1] = sb;
      for (int im = 0; im < nm; ++im, ++s) {
        const int se = r[3 + 3 * im] - 1, sls = r[4 + 3 * im];
        take(se, sls);
        const int iNb = type == 1 ? im % 2 : (type == 3 ? im : -1), jNb = type == 1 ? im / 2 : (type == 2 ? im : -1);
        double xm[4][3];
        for (int c = 0; c < 4; ++c) {
          const double xi = iNb < 0 ? ((c & 1) ? 1. : -1.) : ((c & 1) ? (iNb ? 1. : 0.) : (iNb ? 0. : -1.));
          const double eta = jNb < 0 ? ((c & 2) ? 1. : -1.) : ((c & 2) ? (jNb ? 1. : 0.) : (jNb ? 0. : -1.));
          const Vec La = lagrange_at(xi, xe, wbe), Lb = lagrange_at(eta, xe, wbe);
          for (int dd = 0; dd < 3; ++dd) xm[c][dd] = 0.;
          for (int b = 0; b < ng; ++b)
            for (int a = 0; a < ng; ++a) {
              double x[3];
              corner(be, bls, a, b, x);
              for (int dd = 0; dd < 3; ++dd) xm[c][dd] += La[a] * Lb[b] * x[dd];
            }
        }
        const int f = match_flip(xm, se, sls);
        if (f < 0) throw std::runtime_error("mortar: small face does not match its part of the big face");
        M.sideElem[s * 4 + 0] = be; M.sideElem[s * 4 + 1] = bls; M.sideElem[s * 4 + 2] = se; M.sideElem[s * 4 + 3] = 8 * sls + f;
        M.elemSide[se * 6 + sls - 1] = 8 * s + f;
        M.mortarInfo[(size_t)m * 6 + 2 + im] = s;
      }
    }
  }
  // instances
  M.elemInst.assign(nE, 0);
  if (R.elemInst) for (int e = 0; e < nE; ++e) M.elemInst[e] = R.elemInst[e];
  M.sideInst.assign(M.nSides, 0);
  for (int s = 0; s < M.nSides; ++s) M.sideInst[s] = M.elemInst[M.sideElem[s * 4]];

  // ---------------- metrics (curl form, metrics.f90:CalcMetrics) ----------------
  const int NGeoRef = 3 * NG, nr = NGeoRef + 1;
  const Mat V_EQ_CL = vandermonde(NG, EQUI, NG, CHEBLOB, false);
  const Mat V_CLNG_CLN = vandermonde(NG, CHEBLOB, N, CHEBLOB, false);
  const Mat D_CLNG = diff_matrix(NG, CHEBLOB);
  const Mat V_CLNG_Ref = vandermonde(NG, CHEBLOB, NGeoRef, nodeType, false);
  const Mat V_Ref_N = vandermonde(NGeoRef, nodeType, N, nodeType, true);
  const Mat D_CLN = diff_matrix(N, CHEBLOB);
  const Mat V_CLN_N = vandermonde(N, CHEBLOB, N, nodeType, false);
  const Mat V_EQ_N = matmul(V_CLN_N, vandermonde(NG, EQUI, N, CHEBLOB, false));
  M.metr.assign((size_t)nE * 9 * n3, 0.);
  M.sJ.assign((size_t)nE * n3, 0.);
  M.elemX.assign((size_t)nE * 3 * n3, 0.);
  M.geo.assign((size_t)M.nSides * 10 * n2, 0.);
  M.faceJa.assign((size_t)nE * 6 * 3 * n2, 0.);
  // mortar.f90:InitMortar interpolation to the two halves, MI[h](p, l) = L_l(0.5 (x_p -/+ 1))
  Mat MI[2];
  {
    Vec x, w, x1, x2;
    nodes(N, nodeType, x, w);
    for (double v : x) { x1.push_back(0.5 * (v - 1.)); x2.push_back(0.5 * (v + 1.)); }
    MI[0] = interp_matrix(x, x1);
    MI[1] = interp_matrix(x, x2);
  }
  std::string err;
#pragma omp parallel
  {
    std::vector<double> nc((size_t)3 * ng * ng * ng), xcl_ng(nc.size()), xcl_n((size_t)3 * n3), dng((size_t)9 * ng * ng * ng),
        dref((size_t)9 * nr * nr * nr), detRef((size_t)nr * nr * nr), detN(n3), dn((size_t)9 * n3), Rc((size_t)9 * n3), Ja((size_t)9 * n3),
        tmp(n3), tmp2((size_t)3 * n2), tmp3((size_t)3 * n2), ja_out((size_t)3 * n3), sjn((size_t)3 * n2), sjt((size_t)3 * n2);
#pragma omp for schedule(dynamic, 16)
    for (int e = 0; e < nE; ++e) {
      // component-major copy of the element's node coordinates
      for (int d = 0; d < 3; ++d)
        for (int k = 0; k < ng; ++k) for (int j = 0; j < ng; ++j) for (int i = 0; i < ng; ++i)
          nc[(size_t)d * ng * ng * ng + (k * ng + j) * ng + i] = X(d, i, j, k, e);
      tensor3(V_EQ_CL, nc.data(), xcl_ng.data(), 3);
      tensor3(V_CLNG_CLN, xcl_ng.data(), xcl_n.data(), 3);
      tensor3(V_EQ_N, nc.data(), &M.elemX[(size_t)e * 3 * n3], 3);
      // dXCL_NGeo(dir,comp): stored [3*dir+comp][pts]
      const int ng3 = ng * ng * ng;
      for (int dir = 0; dir < 3; ++dir)
        for (int c = 0; c < 3; ++c) deriv3(D_CLNG, &xcl_ng[(size_t)c * ng3], &dng[(size_t)(3 * dir + c) * ng3], dir);
      tensor3(V_CLNG_Ref, dng.data(), dref.data(), 9);
      const int nr3 = nr * nr * nr;
      for (int x = 0; x < nr3; ++x) {
        auto J = [&](int dir, int c) { return dref[(size_t)(3 * dir + c) * nr3 + x]; };
        detRef[x] = J(0, 0) * (J(1, 1) * J(2, 2) - J(2, 1) * J(1, 2)) + J(1, 0) * (J(2, 1) * J(0, 2) - J(0, 1) * J(2, 2)) +
                    J(2, 0) * (J(0, 1) * J(1, 2) - J(1, 1) * J(0, 2));
      }
      tensor3(V_Ref_N, detRef.data(), detN.data(), 1);
      bool bad = false;
      for (int x = 0; x < n3; ++x) { M.sJ[(size_t)e * n3 + x] = 1. / detN[x]; if (!(detN[x] > 0.)) bad = true; }
      if (bad) {
#pragma omp critical
        err = "negative or zero Jacobian in element " + std::to_string(e + 1);
      }
      if (N >= NG) tensor3(V_CLNG_CLN, dng.data(), dn.data(), 9);
      else
        for (int dir = 0; dir < 3; ++dir)
          for (int c = 0; c < 3; ++c) deriv3(D_CLN, &xcl_n[(size_t)c * n3], &dn[(size_t)(3 * dir + c) * n3], dir);
      // R(dir, comp) = 1/2 (X_b dX_c/d(dir) - X_c dX_b/d(dir)) for the cyclic (comp,b,c)
      for (int x = 0; x < n3; ++x) {
        const double x0 = xcl_n[x], x1 = xcl_n[n3 + x], x2 = xcl_n[2 * n3 + x];
        for (int dir = 0; dir < 3; ++dir) {
          const double d0 = dn[(size_t)(3 * dir + 0) * n3 + x], d1 = dn[(size_t)(3 * dir + 1) * n3 + x], d2 = dn[(size_t)(3 * dir + 2) * n3 + x];
          Rc[(size_t)(3 * dir + 0) * n3 + x] = 0.5 * (x2 * d1 - x1 * d2);
          Rc[(size_t)(3 * dir + 1) * n3 + x] = 0.5 * (x0 * d2 - x2 * d0);
          Rc[(size_t)(3 * dir + 2) * n3 + x] = 0.5 * (x1 * d0 - x0 * d1);
        }
      }
      // Ja(m,c) = d/d(xi_{m+1}) R(m+2, c) - d/d(xi_{m+2}) R(m+1, c)   (cyclic m), curl form
      std::fill(Ja.begin(), Ja.end(), 0.);
      for (int m = 0; m < 3; ++m) {
        const int d1 = (m + 1) % 3, d2 = (m + 2) % 3;
        for (int c = 0; c < 3; ++c) {
          deriv3(D_CLN, &Rc[(size_t)(3 * d2 + c) * n3], tmp.data(), d1);
          for (int x = 0; x < n3; ++x) Ja[(size_t)(3 * m + c) * n3 + x] -= tmp[x];
          deriv3(D_CLN, &Rc[(size_t)(3 * d1 + c) * n3], tmp.data(), d2);
          for (int x = 0; x < n3; ++x) Ja[(size_t)(3 * m + c) * n3 + x] += tmp[x];
        }
      }
      tensor3(V_CLN_N, Ja.data(), &M.metr[(size_t)e * 9 * n3], 9);
      // surface metrics (metrics.f90:CalcSurfMetrics/SurfMetricsFromJa): the normal row of every side of the
      // element (Ja_Face / Ja_slave), the normal vectors and surface elements of the sides it is master of
      for (int ls = 1; ls <= 6; ++ls) {
        const int code = M.elemSide[e * 6 + ls - 1];
        const int s = code >> 3;
        const int lf = minus_side(ls) ? 0 : N;
        const int nd = kNormalDir[ls], td = kTangDir[ls];
        // Ja rows nd and td on the face (CL points), interpolated to the solution nodes
        for (int row = 0; row < 2; ++row) {
          if (row == 1) {
            std::copy(tmp3.begin(), tmp3.end(), M.faceJa.begin() + ((size_t)e * 6 + ls - 1) * 3 * n2);
            if ((code & 7) != 0) break;
          }
          const int mrow = row == 0 ? nd : td;
          for (int c = 0; c < 3; ++c)
            for (int b = 0; b < n; ++b) for (int a = 0; a < n; ++a) {
              int i, j, k;
              face_ijk(ls, a, b, lf, i, j, k);
              tmp2[(size_t)c * n2 + b * n + a] = Ja[(size_t)(3 * mrow + c) * n3 + i + n * (j + n * k)];
            }
          tensor2(V_CLN_N, tmp2.data(), row == 0 ? tmp3.data() : ja_out.data(), 3);
        }
        if ((code & 7) != 0) continue;
        // normal and tangential rows in side coordinates (p + n q, master orientation)
        for (int q = 0; q < n; ++q) for (int p = 0; p < n; ++p) {
          int a, b;
          s2v2(N, p, q, 0, ls, a, b);
          const int o = b * n + a;
          for (int c = 0; c < 3; ++c) { sjn[(size_t)c * n2 + q * n + p] = tmp3[(size_t)c * n2 + o]; sjt[(size_t)c * n2 + q * n + p] = ja_out[(size_t)c * n2 + o]; }
        }
        for (int pq = 0; pq < n2; ++pq) {
          const double jn[3] = {sjn[pq], sjn[n2 + pq], sjn[2 * n2 + pq]};
          const double jt[3] = {sjt[pq], sjt[n2 + pq], sjt[2 * n2 + pq]};
          surf_point(jn, jt, ls, &M.geo[(size_t)s * 10 * n2 + pq], n2);
        }
        // mortar_metrics.f90:Mortar_CalcSurfMetrics: each small side's rows are the big side's interpolated to
        // its part and halved per split direction
        const int mb = s - (M.nSides - M.nMortars);
        if (mb < 0) continue;
        const int type = M.mortarInfo[(size_t)mb * 6];
        for (int im = 0; im < (type == 1 ? 4 : 2); ++im) {
          const int iNb = type == 1 ? im % 2 : (type == 3 ? im : -1), jNb = type == 1 ? im / 2 : (type == 2 ? im : -1);
          const int ss = M.mortarInfo[(size_t)mb * 6 + 2 + im];
          for (int q = 0; q < n; ++q) for (int p = 0; p < n; ++p) {
            double jn[3] = {0., 0., 0.}, jt[3] = {0., 0., 0.};
            for (int b = 0; b < n; ++b) {
              const double wq = jNb < 0 ? (b == q ? 1. : 0.) : 0.5 * MI[jNb](q, b);
              if (wq == 0.) continue;
              for (int a = 0; a < n; ++a) {
                const double w = wq * (iNb < 0 ? (a == p ? 1. : 0.) : 0.5 * MI[iNb](p, a));
                if (w == 0.) continue;
                for (int c = 0; c < 3; ++c) { jn[c] += w * sjn[(size_t)c * n2 + b * n + a]; jt[c] += w * sjt[(size_t)c * n2 + b * n + a]; }
              }
            }
            surf_point(jn, jt, ls, &M.geo[(size_t)ss * 10 * n2 + q * n + p], n2);
          }
        }
      }
    }
  }
  if (!err.empty()) throw std::runtime_error(err);
}

void build_from_flexi(int N, int nodeType, int nElems, int nSides, int nBCSides, const int* SideToElem, const int* ElemToSide, const int* BC,
                      int nBCs, const int* BoundaryType, int nRefStates, const double* RefStatePrim, const double* Mf, const double* Mg,
                      const double* Mh, const double* sJ, const double* NormVec, const double* TangVec1, const double* TangVec2,
                      const double* SurfElem, int nMortars, const int* MortarType, const int* MortarInfo, HostMesh& M) {
  const int n = N + 1, n2 = n * n, n3 = n2 * n;
  M.N = N; M.n = n; M.nodeType = nodeType; M.nElems = nElems; M.nSides = nSides; M.nBCSides = nBCSides;
  if (nMortars < 0 || (nMortars > 0 && (!MortarType || !MortarInfo))) throw std::runtime_error("invalid mortar arrays");
  // side order of the library: BC | conforming inner | small mortar | big mortar. FLEXI's big mortar sides
  // carry MortarType(1,SideID) > 0 and the small sides of mortar MortarType(2,SideID) in MortarInfo
  // (mesh_vars.f90:158-159); a small side has no master element (its data come from the big side).
  std::vector<int> newId(nSides, -1), order;
  order.reserve(nSides);
  std::vector<int> bigOf(nMortars, -1);
  for (int s = 0; s < nSides; ++s) {
    const int type = nMortars ? MortarType[(size_t)s * 2] : 0;
    if (type < 0 || type > 3) throw std::runtime_error("MortarType must be 0..3 (no MPI mortars)");
    if (type > 0) {
      const int m = MortarType[(size_t)s * 2 + 1] - 1;
      if (m < 0 || m >= nMortars || bigOf[m] >= 0) throw std::runtime_error("invalid mortar index in MortarType");
      bigOf[m] = s;
    }
  }
  for (int m = 0; m < nMortars; ++m) if (bigOf[m] < 0) throw std::runtime_error("mortar without big side");
  std::vector<char> isSmall(nSides, 0);
  for (int m = 0; m < nMortars; ++m) {
    const int nm = MortarType[(size_t)bigOf[m] * 2] == 1 ? 4 : 2;
    for (int im = 0; im < nm; ++im) {
      const int ss = MortarInfo[((size_t)m * 4 + im) * 2] - 1;
      if (ss < nBCSides || ss >= nSides || isSmall[ss] || SideToElem[(size_t)ss * 5] > 0 || SideToElem[(size_t)ss * 5 + 1] <= 0)
        throw std::runtime_error("MortarInfo names a side that is not a small mortar side");
      isSmall[ss] = 1;
    }
  }
  for (int s = 0; s < nSides; ++s)
    if (!isSmall[s] && !(nMortars && MortarType[(size_t)s * 2] > 0)) order.push_back(s);
  M.nFluxSides = (int)order.size();
  M.nMortars = nMortars;
  for (int m = 0; m < nMortars; ++m) {
    const int nm = MortarType[(size_t)bigOf[m] * 2] == 1 ? 4 : 2;
    for (int im = 0; im < nm; ++im) order.push_back(MortarInfo[((size_t)m * 4 + im) * 2] - 1);
  }
  for (int m = 0; m < nMortars; ++m) order.push_back(bigOf[m]);
  if ((int)order.size() != nSides) throw std::runtime_error("small mortar sides counted twice or missing");
  for (int t = 0; t < nSides; ++t) newId[order[t]] = t;
  M.flexiSide = order;
  M.mortarInfo.assign((size_t)6 * nMortars, -1);
  M.sideElem.assign((size_t)nSides * 4, -1);
  M.elemSide.assign((size_t)nElems * 6, -1);
  for (int t = 0; t < nSides; ++t) {
    const int s = order[t];
    const int* r = &SideToElem[(size_t)s * 5];
    if (isSmall[s]) continue;  // below, with its mortar
    if (r[0] <= 0) throw std::runtime_error("side without master element (MPI sides are not supported)");
    M.sideElem[t * 4 + 0] = r[0] - 1; M.sideElem[t * 4 + 1] = r[2];
    if (r[1] > 0) { M.sideElem[t * 4 + 2] = r[1] - 1; M.sideElem[t * 4 + 3] = 8 * r[3] + r[4]; }
    else if (s >= nBCSides && !(nMortars && MortarType[(size_t)s * 2] > 0)) throw std::runtime_error("inner side without slave element");
  }
  for (int m = 0; m < nMortars; ++m) {
    const int sb = bigOf[m], type = MortarType[(size_t)sb * 2], nm = type == 1 ? 4 : 2;
    const int* rb = &SideToElem[(size_t)sb * 5];
    M.mortarInfo[(size_t)m * 6 + 0] = type;
    M.mortarInfo[(size_t)m * 6 + 1] = newId[sb];
    for (int im = 0; im < nm; ++im) {
      const int ss = MortarInfo[((size_t)m * 4 + im) * 2] - 1, t = newId[ss];
      const int* r = &SideToElem[(size_t)ss * 5];
      M.sideElem[t * 4 + 0] = rb[0] - 1; M.sideElem[t * 4 + 1] = rb[2];
      M.sideElem[t * 4 + 2] = r[1] - 1; M.sideElem[t * 4 + 3] = 8 * r[3] + r[4];
      M.mortarInfo[(size_t)m * 6 + 2 + im] = t;
    }
  }
  for (int e = 0; e < nElems; ++e)
    for (int ls = 1; ls <= 6; ++ls) {
      const int sid = ElemToSide[((size_t)e * 6 + ls - 1) * 2] - 1, flip = ElemToSide[((size_t)e * 6 + ls - 1) * 2 + 1];
      if (sid < 0 || sid >= nSides) throw std::runtime_error("invalid ElemToSide");
      M.elemSide[e * 6 + ls - 1] = 8 * newId[sid] + flip;
    }
  M.bcType.assign(nBCSides, 0);
  M.bcTwall.assign(nBCSides, 0.);
  for (int s = 0; s < nBCSides; ++s) {
    const int bi = BC[s];
    if (bi < 1 || bi > nBCs) throw std::runtime_error("invalid BC index");
    const int bt = BoundaryType[(bi - 1) * 2], bs = BoundaryType[(bi - 1) * 2 + 1];
    if (bt != 3 && bt != 4) throw std::runtime_error("only no-slip wall boundaries (types 3, 4) are supported");
    M.bcType[s] = bt;
    if (bt == 4) {
      if (bs < 1 || bs > nRefStates) throw std::runtime_error("isothermal wall needs a RefState");
      M.bcTwall[s] = RefStatePrim[(bs - 1) * 6 + 5];
    }
  }
  M.elemInst.assign(nElems, 0);
  M.sideInst.assign(nSides, 0);
  M.metr.assign((size_t)nElems * 9 * n3, 0.);
  M.sJ.assign((size_t)nElems * n3, 0.);
  for (int e = 0; e < nElems; ++e)
    for (int x = 0; x < n3; ++x) {
      const size_t g = (size_t)e * n3 + x;
      for (int c = 0; c < 3; ++c) {
        M.metr[((size_t)e * 9 + c) * n3 + x] = Mf[g * 3 + c];
        M.metr[((size_t)e * 9 + 3 + c) * n3 + x] = Mg[g * 3 + c];
        M.metr[((size_t)e * 9 + 6 + c) * n3 + x] = Mh[g * 3 + c];
      }
      M.sJ[g] = sJ[g];
    }
  M.geo.assign((size_t)nSides * 10 * n2, 0.);
  for (int t = 0; t < nSides; ++t)
    for (int pq = 0; pq < n2; ++pq) {
      const size_t g = (size_t)order[t] * n2 + pq;
      double* G = &M.geo[(size_t)t * 10 * n2 + pq];
      for (int c = 0; c < 3; ++c) { G[c * n2] = NormVec[g * 3 + c]; G[(3 + c) * n2] = TangVec1[g * 3 + c]; G[(6 + c) * n2] = TangVec2[g * 3 + c]; }
      G[9 * n2] = SurfElem[g];
    }
  // face metrics of every element side: the normal-direction volume metrics evaluated at the face (GL: the
  // face node; Gauss: interpolated with L(-1) / L(+1)); equal to FLEXI's Ja_Face / Ja_slave up to round-off
  // (fg_set_face_metrics can hand over FLEXI's own arrays instead)
  {
    Vec x, w;
    nodes(N, nodeType, x, w);
    const Vec wb = bary_weights(x);
    const Vec Lm = lagrange_at(-1.0, x, wb), Lp = lagrange_at(1.0, x, wb);
    M.faceJa.assign((size_t)nElems * 6 * 3 * n2, 0.);
    for (int e = 0; e < nElems; ++e)
      for (int ls = 1; ls <= 6; ++ls) {
        const int nd = kNormalDir[ls];
        const Vec& L = minus_side(ls) ? Lm : Lp;
        for (int c = 0; c < 3; ++c)
          for (int b = 0; b < n; ++b) for (int a = 0; a < n; ++a) {
            double acc = 0.;
            for (int l = 0; l < n; ++l) {
              int i, j, k;
              face_ijk(ls, a, b, l, i, j, k);
              acc += L[l] * M.metr[((size_t)e * 9 + 3 * nd + c) * n3 + i + n * (j + n * k)];
            }
            M.faceJa[(((size_t)e * 6 + ls - 1) * 3 + c) * n2 + b * n + a] = acc;
          }
      }
  }
  M.elemX.clear();
}

void finish_mesh(HostMesh& M, double kappa, double Pr) {
  const int n = M.n, n3 = n * n * n;
  Vec x, w;
  nodes(M.N, M.nodeType, x, w);
  M.wVol.assign(n3, 0.);
  for (int k = 0; k < n; ++k) for (int j = 0; j < n; ++j) for (int i = 0; i < n; ++i) M.wVol[i + n * (j + n * k)] = w[i] * w[j] * w[k];
  M.nInst = 1;
  for (int v : M.elemInst) M.nInst = std::max(M.nInst, v + 1);
  M.instVol.assign(M.nInst, 0.);
  for (int e = 0; e < M.nElems; ++e)
    for (int q = 0; q < n3; ++q) M.instVol[M.elemInst[e]] += M.wVol[q] / M.sJ[(size_t)e * n3 + q];
  // calctimestep.f90:InitCalctimestep
  const double kspr = std::max(4. / 3., kappa / Pr);
  M.metAdv.assign((size_t)M.nElems * 3 * n3, 0.);
  M.metVisc.assign((size_t)M.nElems * 3 * n3, 0.);
  for (int e = 0; e < M.nElems; ++e)
    for (int q = 0; q < n3; ++q) {
      const double sj = M.sJ[(size_t)e * n3 + q];
      for (int d = 0; d < 3; ++d) {
        const double m0 = M.metr[((size_t)e * 9 + 3 * d) * n3 + q], m1 = M.metr[((size_t)e * 9 + 3 * d + 1) * n3 + q],
                     m2 = M.metr[((size_t)e * 9 + 3 * d + 2) * n3 + q];
        M.metAdv[((size_t)e * 3 + d) * n3 + q] = sj * std::sqrt(m0 * m0 + m1 * m1 + m2 * m2);
        M.metVisc[((size_t)e * 3 + d) * n3 + q] = kspr * ((m0 * sj) * (m0 * sj) + (m1 * sj) * (m1 * sj) + (m2 * sj) * (m2 * sj));
      }
    }
}

}  // namespace fgh
