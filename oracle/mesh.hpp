// TEST INFRASTRUCTURE ONLY -- part of the CPU oracle (restatement of FLEXI v25.10); see basis.hpp.
//
// Face orientation maps (src/mesh/mappings.f90), side numbering and SideToElem/ElemToSide
// (src/mesh/prepare_mesh.f90:fillMeshInfo, src/mesh/mesh_readin.f90 flips), curl-form volume metrics,
// Jacobian and surface metrics (src/mesh/metrics.f90:CalcMetrics/CalcSurfMetrics/SurfMetricsFromJa),
// and solution-point coordinates (metrics.f90:BuildCoords).
#pragma once
#include "basis.hpp"
#include <array>
#include <algorithm>

namespace orc {

// local side ids, src/flexi.h:90-95
enum { ZETA_MINUS = 1, ETA_MINUS = 2, XI_PLUS = 3, ETA_PLUS = 4, XI_MINUS = 5, ZETA_PLUS = 6 };
// src/mesh/mesh_vars.f90:105-111
static const int NormalDirs[7] = {0, 3, 2, 1, 2, 1, 3};
static const int TangDirs[7] = {0, 1, 3, 2, 3, 2, 1};
static const double NormalSigns[7] = {0., -1., -1., 1., 1., -1., 1.};

// mappings.f90:Flip_S2M (3D)
inline std::array<int, 2> flip_s2m(int N, int p, int q, int flip) {
  switch (flip) {
    case 0: return {p, q};
    case 1: return {q, p};
    case 2: return {N - p, q};
    case 3: return {N - q, N - p};
    default: return {p, N - q};
  }
}
// mappings.f90:CGNS_SideToVol2 (3D)
inline std::array<int, 2> cgns_side_to_vol2(int N, int p, int q, int locSide) {
  switch (locSide) {
    case XI_MINUS: return {q, p};
    case XI_PLUS: return {p, q};
    case ETA_MINUS: return {p, q};
    case ETA_PLUS: return {N - p, q};
    case ZETA_MINUS: return {q, p};
    default: return {p, q};  // ZETA_PLUS
  }
}
// mappings.f90:CGNS_SideToVol (3D)
inline std::array<int, 3> cgns_side_to_vol(int N, int l, int p, int q, int locSide) {
  switch (locSide) {
    case XI_MINUS: return {l, q, p};
    case XI_PLUS: return {N - l, p, q};
    case ETA_MINUS: return {p, l, q};
    case ETA_PLUS: return {N - p, N - l, q};
    case ZETA_MINUS: return {q, p, l};
    default: return {p, q, N - l};  // ZETA_PLUS
  }
}
// mappings.f90:SideToVol2 / SideToVol
inline std::array<int, 2> side_to_vol2(int N, int p, int q, int flip, int locSide) {
  auto pq = flip_s2m(N, p, q, flip);
  return cgns_side_to_vol2(N, pq[0], pq[1], locSide);
}
inline std::array<int, 3> side_to_vol(int N, int l, int p, int q, int flip, int locSide) {
  auto pq = flip_s2m(N, p, q, flip);
  return cgns_side_to_vol(N, l, pq[0], pq[1], locSide);
}

// Face nodes of a volume array: for a local side, face array index (a,b) in "volume order" as used by
// prolongtoface.t90:EvalElemFaceG/GL (XI sides -> (j,k), ETA -> (i,k), ZETA -> (i,j)) and the normal index.
inline void face_vol_index(int locSide, int a, int b, int l, int N, int& i, int& j, int& k) {
  // l = index along the normal direction counted in the volume (0..N)
  switch (locSide) {
    case XI_MINUS: case XI_PLUS: i = l; j = a; k = b; break;
    case ETA_MINUS: case ETA_PLUS: i = a; j = l; k = b; break;
    default: i = a; j = b; k = l; break;
  }
  (void)N;
}

struct MeshInput {
  int nElems = 0, NGeo = 1;
  std::vector<double> NodeCoords;  // Fortran (3,0:NGeo,0:NGeo,0:NGeo,nElems)
  std::vector<int> ElemNb;         // (3,6,nElems): nbElem(1-based,0=none), nbLocSide, BCIndex(1-based,0=none)
  int nBCs = 0;
  std::vector<int> BoundaryType;   // (2,nBCs): type, state
  std::vector<double> RefStatePrim;  // (6,nRefStates)
  // mortar interfaces, 15 per mortar: big element (1-based), its local side, mortar type (1: 1->4, 2: 1->2 in
  // eta, 3: 1->2 in xi), then for the 2 or 4 small sides: small element (1-based), its local side, unused;
  // the ElemNb entries of these element sides are -1
  std::vector<int> Mortars;
};

// Processed mesh: everything MOD_Mesh_Vars provides to the DG operator.
struct Mesh {
  int N = 0, n = 0, NGeo = 1, nElems = 0, nSides = 0, nBCSides = 0, nInnerSides = 0;
  int firstInnerSide = 0, lastInnerSide = 0;
  std::vector<int> SideToElem;  // (5,nSides) 1-based entries as in FLEXI, -1 if none
  std::vector<int> ElemToSide;  // (2,6,nElems)
  std::vector<int> BC;          // (nBCSides) -> BC index (1-based)
  // mortars (mesh_vars.f90): MortarType(2,nSides) = type, mortar index (1-based) of a big mortar side;
  // MortarInfo(2,4,nMortars) = small SideID (1-based), flip (0: the big element is master)
  int nMortars = 0;
  std::vector<int> MortarType, MortarInfo;
  std::vector<int> BoundaryType;  // (2,nBCs)
  std::vector<double> RefStatePrim;
  std::vector<double> Mf, Mg, Mh;  // Metrics_f/g/hTilde (3,0:N,0:N,0:N,nElems)
  std::vector<double> sJ;          // (0:N,0:N,0:N,nElems)
  std::vector<double> NormVec, TangVec1, TangVec2, Face_xGP;  // (3,0:N,0:N,nSides)
  // row NormalDir of the face metrics Ja_Face (master, flip 0) and Ja_slave (slave, its own flip), in side
  // orientation (3,0:N,0:N,nSides): used by the split-Gauss surface integral (surfint.t90:90-140)
  std::vector<double> JaN_master, JaN_slave;
  // Jacobian determinant on the NGeoRef = 3 NGeo points of the solution node type (metrics.f90, DetJac_Ref),
  // (0:NGeoRef,0:NGeoRef,0:NGeoRef,nElems): the conservative cut-off of overintegration.f90 projects it
  std::vector<double> DetJac_Ref;
  int NGeoRef = 0;
  std::vector<double> SurfElem;    // (0:N,0:N,nSides)
  std::vector<double> Elem_xGP;    // (3,0:N,0:N,0:N,nElems)
  double Vol = 0.;
  std::vector<double> wGPVol;
  size_t vidx(int i, int j, int k, int e) const { return (((size_t)e * n + k) * n + j) * n + i; }
  size_t sidx(int p, int q, int s) const { return ((size_t)s * n + q) * n + p; }
};

// ChangeBasis3D: Xout(nv, 0:No^3) = Vdm (No+1 x Ni+1) applied in all three directions to Xin(nv, 0:Ni^3)
inline void change_basis_3d(int nv, int Ni, int No, const std::vector<double>& V, const double* Xin, double* Xout) {
  const int ni = Ni + 1, no = No + 1;
  std::vector<double> t1((size_t)nv * no * ni * ni, 0.), t2((size_t)nv * no * no * ni, 0.);
  for (int k = 0; k < ni; ++k) for (int j = 0; j < ni; ++j) for (int a = 0; a < no; ++a)
    for (int i = 0; i < ni; ++i) { double v = V[a * ni + i];
      for (int c = 0; c < nv; ++c) t1[(((size_t)k * ni + j) * no + a) * nv + c] += v * Xin[(((size_t)k * ni + j) * ni + i) * nv + c]; }
  for (int k = 0; k < ni; ++k) for (int b = 0; b < no; ++b) for (int j = 0; j < ni; ++j) { double v = V[b * ni + j];
    for (int a = 0; a < no; ++a) for (int c = 0; c < nv; ++c)
      t2[(((size_t)k * no + b) * no + a) * nv + c] += v * t1[(((size_t)k * ni + j) * no + a) * nv + c]; }
  for (size_t x = 0; x < (size_t)nv * no * no * no; ++x) Xout[x] = 0.;
  for (int cc = 0; cc < no; ++cc) for (int k = 0; k < ni; ++k) { double v = V[cc * ni + k];
    for (int b = 0; b < no; ++b) for (int a = 0; a < no; ++a) for (int c = 0; c < nv; ++c)
      Xout[(((size_t)cc * no + b) * no + a) * nv + c] += v * t2[(((size_t)k * no + b) * no + a) * nv + c]; }
}
// ChangeBasisSurf: 2D version
inline void change_basis_2d(int nv, int Ni, int No, const std::vector<double>& V, const double* Xin, double* Xout) {
  const int ni = Ni + 1, no = No + 1;
  std::vector<double> t1((size_t)nv * no * ni, 0.);
  for (int j = 0; j < ni; ++j) for (int a = 0; a < no; ++a) for (int i = 0; i < ni; ++i) { double v = V[a * ni + i];
    for (int c = 0; c < nv; ++c) t1[((size_t)j * no + a) * nv + c] += v * Xin[((size_t)j * ni + i) * nv + c]; }
  for (size_t x = 0; x < (size_t)nv * no * no; ++x) Xout[x] = 0.;
  for (int b = 0; b < no; ++b) for (int j = 0; j < ni; ++j) { double v = V[b * ni + j];
    for (int a = 0; a < no; ++a) for (int c = 0; c < nv; ++c) Xout[((size_t)b * no + a) * nv + c] += v * t1[((size_t)j * no + a) * nv + c]; }
}

// Builds sides, orientation flips, metrics. N: polynomial degree, nodeType: NT_GAUSS / NT_GL.
inline void build_mesh(const MeshInput& in, int N, int nodeType, Mesh& M) {
  M.N = N; M.n = N + 1; M.NGeo = in.NGeo; M.nElems = in.nElems;
  M.BoundaryType = in.BoundaryType; M.RefStatePrim = in.RefStatePrim;
  const int nE = in.nElems, NG = in.NGeo, ng = NG + 1, n = N + 1;
  auto nc = [&](int d, int i, int j, int k, int e) { return in.NodeCoords[((((size_t)e * ng + k) * ng + j) * ng + i) * 3 + d]; };
  auto nb = [&](int c, int ls, int e) { return in.ElemNb[((size_t)e * 6 + (ls - 1)) * 3 + c]; };

  // ---- sides: BC sides, big mortar sides, inner sides, small mortar sides (no MPI sides) ----
  std::vector<int> sideOf(6 * nE, -1), flipOf(6 * nE, 0);
  struct S { int e, ls, nbe, nbls, bc; };
  std::vector<S> bcs, inner;
  for (int e = 0; e < nE; ++e)
    for (int ls = 1; ls <= 6; ++ls) {
      int ne = nb(0, ls, e), nls = nb(1, ls, e), bci = nb(2, ls, e);
      if (ne < 0) continue;  // mortar
      if (ne == 0) { bcs.push_back({e, ls, -1, -1, bci}); continue; }
      int oe = ne - 1;
      // master = element with smaller id (same element: smaller local side id)
      bool iAmMaster = (e < oe) || (e == oe && ls < nls);
      if (iAmMaster) inner.push_back({e, ls, oe, nls, 0});
    }
  const int nMo = (int)in.Mortars.size() / 15;
  int nSmall = 0;
  for (int m = 0; m < nMo; ++m) nSmall += in.Mortars[(size_t)m * 15 + 2] == 1 ? 4 : 2;
  M.nMortars = nMo;
  M.nBCSides = (int)bcs.size(); M.nInnerSides = (int)inner.size() + nSmall;
  M.nSides = M.nBCSides + nMo + M.nInnerSides;
  M.firstInnerSide = M.nBCSides + nMo + 1; M.lastInnerSide = M.nSides;
  M.SideToElem.assign(5 * M.nSides, -1);
  M.ElemToSide.assign(2 * 6 * nE, 0);
  M.BC.assign(M.nBCSides, 0);
  M.MortarType.assign(2 * M.nSides, 0);
  M.MortarInfo.assign(2 * 4 * nMo, 0);
  auto s2e = [&](int c, int s) -> int& { return M.SideToElem[(size_t)s * 5 + c]; };
  auto e2s = [&](int c, int ls, int e) -> int& { return M.ElemToSide[((size_t)e * 6 + (ls - 1)) * 2 + c]; };
  for (int s = 0; s < M.nBCSides; ++s) {
    const S& b = bcs[s];
    s2e(0, s) = b.e + 1; s2e(1, s) = -1; s2e(2, s) = b.ls; s2e(3, s) = -1; s2e(4, s) = 0;
    e2s(0, b.ls, b.e) = s + 1; e2s(1, b.ls, b.e) = 0;
    M.BC[s] = b.bc;
  }
  // geometric flip: corner nodes of the master face must coincide (up to one constant periodic shift) with the slave's
  auto face_node = [&](int e, int ls, int p, int q, double* x) {
    // node (p,q) of the side in CGNS side coordinates at degree NGeo, flip 0
    auto ij = cgns_side_to_vol2(NG, p, q, ls);
    int i, j, k; int l = (ls == XI_MINUS || ls == ETA_MINUS || ls == ZETA_MINUS) ? 0 : NG;
    face_vol_index(ls, ij[0], ij[1], l, NG, i, j, k);
    for (int d = 0; d < 3; ++d) x[d] = nc(d, i, j, k, e);
  };
  // flip of the slave whose face corners match the master corners xm(c) (c = p + 2q over the NGeo corners)
  auto match_flip = [&](const double (*xm)[3], int nbe, int nbls) {
    for (int f = 1; f <= 4; ++f) {
      double shift[3]; bool ok = true;
      for (int c = 0; c < 4 && ok; ++c) {
        const int p = (c & 1) ? NG : 0, q = (c & 2) ? NG : 0;
        double xs[3];
        auto ab = flip_s2m(NG, p, q, f);
        face_node(nbe, nbls, ab[0], ab[1], xs);
        double d[3] = {xs[0] - xm[c][0], xs[1] - xm[c][1], xs[2] - xm[c][2]};
        if (c == 0) { for (int k = 0; k < 3; ++k) shift[k] = d[k]; }
        else for (int k = 0; k < 3; ++k) if (std::fabs(d[k] - shift[k]) > 1e-9 * (1. + std::fabs(shift[k]))) ok = false;
      }
      if (ok) return f;
    }
    return -1;
  };
  // big mortar sides: master = the big element, no slave (prepare_mesh.f90, MortarType)
  const int firstBig = M.nBCSides;
  for (int m = 0; m < nMo; ++m) {
    const int* r = &in.Mortars[(size_t)m * 15];
    const int s = firstBig + m;
    s2e(0, s) = r[0]; s2e(1, s) = -1; s2e(2, s) = r[1]; s2e(3, s) = -1; s2e(4, s) = 0;
    e2s(0, r[1], r[0] - 1) = s + 1; e2s(1, r[1], r[0] - 1) = 0;
    M.MortarType[(size_t)s * 2 + 0] = r[2]; M.MortarType[(size_t)s * 2 + 1] = m + 1;
  }
  for (int t = 0; t < (int)inner.size(); ++t) {
    const S& si = inner[t];
    const int s = firstBig + nMo + t;
    double xm[4][3];
    for (int c = 0; c < 4; ++c) face_node(si.e, si.ls, (c & 1) ? NG : 0, (c & 2) ? NG : 0, xm[c]);
    const int best = match_flip(xm, si.nbe, si.nbls);
    if (best < 0) throw std::runtime_error("could not determine side flip");
    s2e(0, s) = si.e + 1; s2e(1, s) = si.nbe + 1; s2e(2, s) = si.ls; s2e(3, s) = si.nbls; s2e(4, s) = best;
    e2s(0, si.ls, si.e) = s + 1; e2s(1, si.ls, si.e) = 0;
    e2s(0, si.nbls, si.nbe) = s + 1; e2s(1, si.nbls, si.nbe) = best;
  }
  // small mortar sides: no master element (its data come from the big side, U_Mortar), the small element is
  // the slave; orientation of the big side's quadrant, flip found from the quadrant corners
  {
    int s = firstBig + nMo + (int)inner.size();
    std::vector<double> Leq(ng);
    std::vector<double> xe(ng);
    for (int a = 0; a < ng; ++a) xe[a] = NG == 0 ? 0. : -1. + 2. * a / NG;
    auto lag = [&](double x, std::vector<double>& L) {
      for (int a = 0; a < ng; ++a) {
        double v = 1.;
        for (int b = 0; b < ng; ++b) if (b != a) v *= (x - xe[b]) / (xe[a] - xe[b]);
        L[a] = v;
      }
    };
    std::vector<double> La(ng), Lb(ng);
    for (int m = 0; m < nMo; ++m) {
      const int* r = &in.Mortars[(size_t)m * 15];
      const int be = r[0] - 1, bls = r[1], type = r[2], nm = type == 1 ? 4 : 2;
      for (int im = 0; im < nm; ++im, ++s) {
        const int se = r[3 + 3 * im] - 1, sls = r[4 + 3 * im];
        // quadrant of the big side (p: xi, q: eta of the side) covered by small side im
        const int iNb = type == 1 ? im % 2 : (type == 3 ? im : -1), jNb = type == 1 ? im / 2 : (type == 2 ? im : -1);
        double xm[4][3];
        for (int c = 0; c < 4; ++c) {
          const double xi = iNb < 0 ? ((c & 1) ? 1. : -1.) : ((c & 1) ? (iNb ? 1. : 0.) : (iNb ? 0. : -1.));
          const double eta = jNb < 0 ? ((c & 2) ? 1. : -1.) : ((c & 2) ? (jNb ? 1. : 0.) : (jNb ? 0. : -1.));
          lag(xi, La); lag(eta, Lb);
          for (int d = 0; d < 3; ++d) xm[c][d] = 0.;
          for (int b = 0; b < ng; ++b) for (int a = 0; a < ng; ++a) {
            double x[3];
            face_node(be, bls, a, b, x);
            for (int d = 0; d < 3; ++d) xm[c][d] += La[a] * Lb[b] * x[d];
          }
        }
        const int f = match_flip(xm, se, sls);
        if (f < 0) throw std::runtime_error("mortar: small face does not match its quadrant of the big face");
        s2e(0, s) = -1; s2e(1, s) = se + 1; s2e(2, s) = -1; s2e(3, s) = sls; s2e(4, s) = f;
        e2s(0, sls, se) = s + 1; e2s(1, sls, se) = f;
        M.MortarInfo[((size_t)m * 4 + im) * 2 + 0] = s + 1;
        M.MortarInfo[((size_t)m * 4 + im) * 2 + 1] = 0;
      }
    }
  }

  // ---- metrics: metrics.f90:CalcMetrics (curl form, no tree) ----
  const int NGeoRef = 3 * NG;
  auto V_EQ_CL = get_vandermonde(NG, NT_VISU, NG, NT_CL, false);
  auto V_CLNG_CLN = get_vandermonde(NG, NT_CL, N, NT_CL, false);
  auto DCL_NG = get_derivative_matrix(NG, NT_CL);
  auto V_CLNG_Ref = get_vandermonde(NG, NT_CL, NGeoRef, nodeType, false);
  auto V_Ref_N = get_vandermonde(NGeoRef, nodeType, N, nodeType, true);
  auto DCL_N = get_derivative_matrix(N, NT_CL);
  auto V_CLN_N = get_vandermonde(N, NT_CL, N, nodeType, false);
  // Elem_xGP via BuildCoords: Vdm = Vdm_CLN_N * Vdm_EQNGeo_CLN
  auto V_EQ_CLN = get_vandermonde(NG, NT_VISU, N, NT_CL, false);
  std::vector<double> V_EQ_N((size_t)n * ng, 0.);
  for (int a = 0; a < n; ++a) for (int b = 0; b < ng; ++b) { double s = 0.; for (int m = 0; m < n; ++m) s += V_CLN_N[a * n + m] * V_EQ_CLN[m * ng + b]; V_EQ_N[a * ng + b] = s; }

  const size_t nv3 = (size_t)n * n * n;
  M.Mf.assign(3 * nv3 * nE, 0.); M.Mg.assign(3 * nv3 * nE, 0.); M.Mh.assign(3 * nv3 * nE, 0.);
  M.sJ.assign(nv3 * nE, 0.); M.Elem_xGP.assign(3 * nv3 * nE, 0.);
  const size_t nsp = (size_t)n * n;
  M.NormVec.assign(3 * nsp * M.nSides, 0.); M.TangVec1 = M.NormVec; M.TangVec2 = M.NormVec; M.Face_xGP = M.NormVec;
  M.JaN_master = M.NormVec; M.JaN_slave = M.NormVec;
  M.SurfElem.assign(nsp * M.nSides, 0.);
  const int nr = NGeoRef + 1;
  M.NGeoRef = NGeoRef;
  M.DetJac_Ref.assign((size_t)nr * nr * nr * nE, 0.);

  for (int e = 0; e < nE; ++e) {
    const double* NC = &in.NodeCoords[(size_t)e * ng * ng * ng * 3];
    std::vector<double> XCL_NG((size_t)ng * ng * ng * 3), XCL_N(nv3 * 3);
    change_basis_3d(3, NG, NG, V_EQ_CL, NC, XCL_NG.data());
    change_basis_3d(3, NG, N, V_CLNG_CLN, XCL_NG.data(), XCL_N.data());
    change_basis_3d(3, NG, N, V_EQ_N, NC, &M.Elem_xGP[(size_t)e * nv3 * 3]);
    // dXCL_NGeo(dir, comp, i,j,k): stored as [(k,j,i)][dir*3+comp]
    std::vector<double> dX_NG((size_t)ng * ng * ng * 9, 0.);
    for (int k = 0; k < ng; ++k) for (int j = 0; j < ng; ++j) for (int i = 0; i < ng; ++i) {
      double* o = &dX_NG[(((size_t)k * ng + j) * ng + i) * 9];
      for (int ll = 0; ll < ng; ++ll) for (int c = 0; c < 3; ++c) {
        o[0 * 3 + c] += DCL_NG[i * ng + ll] * XCL_NG[(((size_t)k * ng + j) * ng + ll) * 3 + c];
        o[1 * 3 + c] += DCL_NG[j * ng + ll] * XCL_NG[(((size_t)k * ng + ll) * ng + i) * 3 + c];
        o[2 * 3 + c] += DCL_NG[k * ng + ll] * XCL_NG[(((size_t)ll * ng + j) * ng + i) * 3 + c];
      }
    }
    // dX_NGeoRef = ChangeBasis(dXCL_NGeo), detJac on NGeoRef
    std::vector<double> dX_Ref((size_t)nr * nr * nr * 9);
    change_basis_3d(9, NG, NGeoRef, V_CLNG_Ref, dX_NG.data(), dX_Ref.data());
    std::vector<double> detRef((size_t)nr * nr * nr), detN(nv3);
    for (size_t x = 0; x < (size_t)nr * nr * nr; ++x) {
      const double* d = &dX_Ref[x * 9];
      auto dd = [&](int a, int b) { return d[(a - 1) * 3 + (b - 1)]; };
      detRef[x] = dd(1, 1) * (dd(2, 2) * dd(3, 3) - dd(3, 2) * dd(2, 3)) + dd(2, 1) * (dd(3, 2) * dd(1, 3) - dd(1, 2) * dd(3, 3)) +
                  dd(3, 1) * (dd(1, 2) * dd(2, 3) - dd(2, 2) * dd(1, 3));
    }
    change_basis_3d(1, NGeoRef, N, V_Ref_N, detRef.data(), detN.data());
    std::copy(detRef.begin(), detRef.end(), M.DetJac_Ref.begin() + (size_t)e * nr * nr * nr);
    for (size_t x = 0; x < nv3; ++x) M.sJ[(size_t)e * nv3 + x] = 1. / detN[x];
    // dXCL_N
    std::vector<double> dX_N(nv3 * 9, 0.);
    if (N >= NG) change_basis_3d(9, NG, N, V_CLNG_CLN, dX_NG.data(), dX_N.data());
    else {
      for (int k = 0; k < n; ++k) for (int j = 0; j < n; ++j) for (int i = 0; i < n; ++i) {
        double* o = &dX_N[(((size_t)k * n + j) * n + i) * 9];
        for (int ll = 0; ll < n; ++ll) for (int c = 0; c < 3; ++c) {
          o[0 * 3 + c] += DCL_N[i * n + ll] * XCL_N[(((size_t)k * n + j) * n + ll) * 3 + c];
          o[1 * 3 + c] += DCL_N[j * n + ll] * XCL_N[(((size_t)k * n + ll) * n + i) * 3 + c];
          o[2 * 3 + c] += DCL_N[k * n + ll] * XCL_N[(((size_t)ll * n + j) * n + i) * 3 + c];
        }
      }
    }
    // curl metrics: R_CL_N(dir, comp), JaCL_N(dd, comp)
    std::vector<double> R(nv3 * 9), Ja(nv3 * 9, 0.);
    for (size_t x = 0; x < nv3; ++x) {
      const double* X = &XCL_N[x * 3]; const double* d = &dX_N[x * 9];
      for (int dir = 0; dir < 3; ++dir) {
        R[x * 9 + dir * 3 + 0] = 0.5 * (X[2] * d[dir * 3 + 1] - X[1] * d[dir * 3 + 2]);
        R[x * 9 + dir * 3 + 1] = 0.5 * (X[0] * d[dir * 3 + 2] - X[2] * d[dir * 3 + 0]);
        R[x * 9 + dir * 3 + 2] = 0.5 * (X[1] * d[dir * 3 + 0] - X[0] * d[dir * 3 + 1]);
      }
    }
    auto Rv = [&](int dir, int comp, int i, int j, int k) { return R[(((size_t)k * n + j) * n + i) * 9 + dir * 3 + comp]; };
    for (int k = 0; k < n; ++k) for (int j = 0; j < n; ++j) for (int i = 0; i < n; ++i) {
      double* J = &Ja[(((size_t)k * n + j) * n + i) * 9];
      for (int c = 0; c < 3; ++c) {
        for (int q = 0; q < n; ++q) {
          J[0 * 3 + c] -= DCL_N[j * n + q] * Rv(2, c, i, q, k);
          J[1 * 3 + c] -= DCL_N[k * n + q] * Rv(0, c, i, j, q);
          J[2 * 3 + c] -= DCL_N[i * n + q] * Rv(1, c, q, j, k);
        }
        for (int q = 0; q < n; ++q) {
          J[0 * 3 + c] += DCL_N[k * n + q] * Rv(1, c, i, j, q);
          J[1 * 3 + c] += DCL_N[i * n + q] * Rv(2, c, q, j, k);
          J[2 * 3 + c] += DCL_N[j * n + q] * Rv(0, c, i, q, k);
        }
      }
    }
    // volume metrics: ChangeBasis(Vdm_CLN_N, JaCL_N(dd,:))
    for (int dd = 0; dd < 3; ++dd) {
      std::vector<double> tin(nv3 * 3), tout(nv3 * 3);
      for (size_t x = 0; x < nv3; ++x) for (int c = 0; c < 3; ++c) tin[x * 3 + c] = Ja[x * 9 + dd * 3 + c];
      change_basis_3d(3, N, N, V_CLN_N, tin.data(), tout.data());
      std::vector<double>& Mx = dd == 0 ? M.Mf : (dd == 1 ? M.Mg : M.Mh);
      std::copy(tout.begin(), tout.end(), Mx.begin() + (size_t)e * nv3 * 3);
    }
    // surface metrics: CalcSurfMetrics (only for flip==0 sides: master/BC)
    for (int ls = 1; ls <= 6; ++ls) {
      int flip = e2s(1, ls, e), SideID = e2s(0, ls, e) - 1;
      int lface = (ls == XI_MINUS || ls == ETA_MINUS || ls == ZETA_MINUS) ? 0 : N;
      if (flip == 0) {
        std::vector<double> tmp(nsp * 3), tmp2(nsp * 3);
        for (int b = 0; b < n; ++b) for (int a = 0; a < n; ++a) {
          int i, j, k; face_vol_index(ls, a, b, lface, N, i, j, k);
          for (int c = 0; c < 3; ++c) tmp[((size_t)b * n + a) * 3 + c] = XCL_N[(((size_t)k * n + j) * n + i) * 3 + c];
        }
        change_basis_2d(3, N, N, V_CLN_N, tmp.data(), tmp2.data());
        for (int q = 0; q < n; ++q) for (int p = 0; p < n; ++p) {
          auto pq = side_to_vol2(N, p, q, 0, ls);
          for (int c = 0; c < 3; ++c) M.Face_xGP[M.sidx(p, q, SideID) * 3 + c] = tmp2[((size_t)pq[1] * n + pq[0]) * 3 + c];
        }
      }
      std::vector<double> JaF(nsp * 9);
      for (int dd = 0; dd < 3; ++dd) {
        std::vector<double> tmp(nsp * 3), tmp2(nsp * 3);
        for (int b = 0; b < n; ++b) for (int a = 0; a < n; ++a) {
          int i, j, k; face_vol_index(ls, a, b, lface, N, i, j, k);
          for (int c = 0; c < 3; ++c) tmp[((size_t)b * n + a) * 3 + c] = Ja[(((size_t)k * n + j) * n + i) * 9 + dd * 3 + c];
        }
        change_basis_2d(3, N, N, V_CLN_N, tmp.data(), tmp2.data());
        for (int q = 0; q < n; ++q) for (int p = 0; p < n; ++p) {
          auto pq = side_to_vol2(N, p, q, flip, ls);
          for (int c = 0; c < 3; ++c) JaF[((size_t)q * n + p) * 9 + dd * 3 + c] = tmp2[((size_t)pq[1] * n + pq[0]) * 3 + c];
        }
      }
      int nd = NormalDirs[ls] - 1, td = TangDirs[ls] - 1; double ns = NormalSigns[ls];
      // Ja_Face / Ja_slave (metrics.f90:704-705), row nd only
      std::vector<double>& JaN = flip == 0 ? M.JaN_master : M.JaN_slave;
      for (int q = 0; q < n; ++q) for (int p = 0; p < n; ++p)
        for (int c = 0; c < 3; ++c) JaN[M.sidx(p, q, SideID) * 3 + c] = JaF[((size_t)q * n + p) * 9 + nd * 3 + c];
      if (flip != 0) continue;
      // SurfMetricsFromJa
      auto surf_metrics = [&](const std::vector<double>& JaF, int SideID) {
      for (int q = 0; q < n; ++q) for (int p = 0; p < n; ++p) {
        const double* J = &JaF[((size_t)q * n + p) * 9];
        size_t si = M.sidx(p, q, SideID);
        double se = std::sqrt(J[nd * 3 + 0] * J[nd * 3 + 0] + J[nd * 3 + 1] * J[nd * 3 + 1] + J[nd * 3 + 2] * J[nd * 3 + 2]);
        M.SurfElem[si] = se;
        double nv[3], t1[3], t2[3];
        for (int c = 0; c < 3; ++c) nv[c] = ns * J[nd * 3 + c] / se;
        double dt = J[td * 3 + 0] * nv[0] + J[td * 3 + 1] * nv[1] + J[td * 3 + 2] * nv[2];
        for (int c = 0; c < 3; ++c) t1[c] = J[td * 3 + c] - dt * nv[c];
        double tl = std::sqrt(t1[0] * t1[0] + t1[1] * t1[1] + t1[2] * t1[2]);
        for (int c = 0; c < 3; ++c) t1[c] /= tl;
        t2[0] = nv[1] * t1[2] - nv[2] * t1[1];
        t2[1] = nv[2] * t1[0] - nv[0] * t1[2];
        t2[2] = nv[0] * t1[1] - nv[1] * t1[0];
        for (int c = 0; c < 3; ++c) { M.NormVec[si * 3 + c] = nv[c]; M.TangVec1[si * 3 + c] = t1[c]; M.TangVec2[si * 3 + c] = t2[c]; }
      }
      };
      surf_metrics(JaF, SideID);
      // mortar_metrics.f90:Mortar_CalcSurfMetrics -- small sides: the big side's Ja interpolated to each
      // quadrant and halved per split direction, coordinates interpolated
      const int mtype = M.MortarType[(size_t)SideID * 2];
      if (mtype > 0) {
        const int m = M.MortarType[(size_t)SideID * 2 + 1] - 1;
        std::vector<double> M01(nsp), M02(nsp);  // (out, in): L_in(0.5 (xi_out -/+ 1))
        {
          DGBasis Bm; Bm.init(N, nodeType);
          for (int o = 0; o < n; ++o) {
            std::vector<double> L1(n), L2(n);
            lagrange_polys(0.5 * (Bm.xGP[o] - 1.), N, Bm.xGP.data(), Bm.wBary.data(), L1.data());
            lagrange_polys(0.5 * (Bm.xGP[o] + 1.), N, Bm.xGP.data(), Bm.wBary.data(), L2.data());
            for (int l = 0; l < n; ++l) { M01[(size_t)o * n + l] = L1[l]; M02[(size_t)o * n + l] = L2[l]; }
          }
        }
        const int nm = mtype == 1 ? 4 : 2;
        std::vector<double> xF((size_t)nsp * 3);
        for (int q = 0; q < n; ++q) for (int p = 0; p < n; ++p)
          for (int c = 0; c < 3; ++c) xF[((size_t)q * n + p) * 3 + c] = M.Face_xGP[M.sidx(p, q, SideID) * 3 + c];
        for (int im = 0; im < nm; ++im) {
          const int iNb = mtype == 1 ? im % 2 : (mtype == 3 ? im : -1), jNb = mtype == 1 ? im / 2 : (mtype == 2 ? im : -1);
          const std::vector<double>* Mp = iNb < 0 ? nullptr : (iNb ? &M02 : &M01);
          const std::vector<double>* Mq = jNb < 0 ? nullptr : (jNb ? &M02 : &M01);
          std::vector<double> Js((size_t)nsp * 9), xs((size_t)nsp * 3);
          for (int q = 0; q < n; ++q) for (int p = 0; p < n; ++p) {
            for (int c = 0; c < 9; ++c) {
              double acc = 0.;
              for (int b = 0; b < n; ++b) for (int a = 0; a < n; ++a) {
                const double wp = Mp ? 0.5 * (*Mp)[(size_t)p * n + a] : (a == p ? 1. : 0.);
                const double wq = Mq ? 0.5 * (*Mq)[(size_t)q * n + b] : (b == q ? 1. : 0.);
                if (wp != 0. && wq != 0.) acc += wp * wq * JaF[((size_t)b * n + a) * 9 + c];
              }
              Js[((size_t)q * n + p) * 9 + c] = acc;
            }
            for (int c = 0; c < 3; ++c) {
              double acc = 0.;
              for (int b = 0; b < n; ++b) for (int a = 0; a < n; ++a) {
                const double wp = Mp ? (*Mp)[(size_t)p * n + a] : (a == p ? 1. : 0.);
                const double wq = Mq ? (*Mq)[(size_t)q * n + b] : (b == q ? 1. : 0.);
                if (wp != 0. && wq != 0.) acc += wp * wq * xF[((size_t)b * n + a) * 3 + c];
              }
              xs[((size_t)q * n + p) * 3 + c] = acc;
            }
          }
          const int small = M.MortarInfo[((size_t)m * 4 + im) * 2] - 1;
          surf_metrics(Js, small);
          for (int q = 0; q < n; ++q) for (int p = 0; p < n; ++p) {
            for (int c = 0; c < 3; ++c) M.Face_xGP[M.sidx(p, q, small) * 3 + c] = xs[((size_t)q * n + p) * 3 + c];
            for (int c = 0; c < 3; ++c) M.JaN_master[M.sidx(p, q, small) * 3 + c] = Js[((size_t)q * n + p) * 9 + nd * 3 + c];
          }
        }
      }
    }
  }
  // analyze.f90:InitAnalyze -- wGPVol and domain volume
  DGBasis B; B.init(N, nodeType);
  M.wGPVol.resize(nv3);
  for (int k = 0; k < n; ++k) for (int j = 0; j < n; ++j) for (int i = 0; i < n; ++i)
    M.wGPVol[((size_t)k * n + j) * n + i] = B.wGP[i] * B.wGP[j] * B.wGP[k];
  double vol = 0.;
  for (int e = 0; e < nE; ++e) for (size_t x = 0; x < nv3; ++x) vol += M.wGPVol[x] / M.sJ[(size_t)e * nv3 + x];
  M.Vol = vol;
}

}  // namespace orc
