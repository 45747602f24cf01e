// TEST INFRASTRUCTURE ONLY -- C interface of the CPU oracle (restatement of FLEXI v25.10).
// Loaded by tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg through ctypes, as the
// checker and as the timed CPU baseline. Never linked into, or called by, the product library.
#include "dg.hpp"
#include <cstring>
#include <limits>
#include <memory>

using namespace orc;

extern "C" {

struct orc_config {
  int N, nodeType, riemann, riemannBC, lifting, weakLifting, consLifting, splitDG;
  double etaBR2, etaBR2_wall, kappa, R, Pr, mu0, CFLScale, DFLScale;
  int doTCSource;
  double dpdx;
  int overintType, NUnder;
  int iniExactFunc;
  double advVel[3], iniFrequency, iniAmplitude;
  int timeDisc;
  double riemannPhi;
};

static Config to_cfg(const orc_config* c) {
  Config C;
  C.N = c->N; C.nodeType = c->nodeType; C.riemann = c->riemann; C.riemannBC = c->riemannBC;
  C.lifting = c->lifting; C.weakLifting = c->weakLifting; C.consLifting = c->consLifting; C.splitDG = c->splitDG;
  C.etaBR2 = c->etaBR2; C.etaBR2_wall = c->etaBR2_wall; C.kappa = c->kappa; C.R = c->R; C.Pr = c->Pr; C.mu0 = c->mu0;
  C.CFLScale = c->CFLScale; C.DFLScale = c->DFLScale; C.doTCSource = c->doTCSource; C.dpdx = c->dpdx;
  C.overintType = c->overintType; C.NUnder = c->NUnder;
  C.timeDisc = c->timeDisc;
  C.iniExactFunc = c->iniExactFunc;
  for (int d = 0; d < 3; ++d) C.advVel[d] = c->advVel[d];
  C.iniFrequency = c->iniFrequency; C.iniAmplitude = c->iniAmplitude;
  C.riemannPhi = c->riemannPhi;
  return C;
}


struct OrcHandle {
  DG<double> dg;
  MeshInput mi;
  Config cfg;
  std::unique_ptr<DG<DD>> dgd;  // dual-number instance for exact Jacobian-vector products (built on first use)
  std::string err;
};

static thread_local std::string g_err;
const char* orc_last_error() { return g_err.c_str(); }

void* orc_create(const orc_config* cfg, int nElems, int NGeo, const double* NodeCoords, const int* ElemNb, int nBCs,
                 const int* BoundaryType, int nRefStates, const double* RefStatePrim, int nMortars, const int* Mortars) {
  try {
    auto* h = new OrcHandle();
    MeshInput& mi = h->mi;
    if (nMortars > 0) mi.Mortars.assign(Mortars, Mortars + (size_t)15 * nMortars);
    mi.nElems = nElems; mi.NGeo = NGeo; mi.nBCs = nBCs;
    size_t nnc = (size_t)3 * (NGeo + 1) * (NGeo + 1) * (NGeo + 1) * nElems;
    mi.NodeCoords.assign(NodeCoords, NodeCoords + nnc);
    mi.ElemNb.assign(ElemNb, ElemNb + (size_t)18 * nElems);
    if (nBCs > 0) mi.BoundaryType.assign(BoundaryType, BoundaryType + 2 * nBCs);
    if (nRefStates > 0) mi.RefStatePrim.assign(RefStatePrim, RefStatePrim + 6 * nRefStates);
    h->cfg = to_cfg(cfg);
    h->dg.init(h->cfg, mi);
    return h;
  } catch (std::exception& e) { g_err = e.what(); return nullptr; }
}
void orc_destroy(void* h) { delete (OrcHandle*)h; }
void orc_set_threads(int n) {
#ifdef _OPENMP
  omp_set_num_threads(n);
#else
  (void)n;
#endif
}
int orc_max_threads() {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

// sizes: nElems, nSides, nBCSides, N
void orc_sizes(void* hp, int* out) {
  auto& d = ((OrcHandle*)hp)->dg;
  out[0] = d.nE; out[1] = d.nS; out[2] = d.M.nBCSides; out[3] = d.N;
}
void orc_set_state(void* hp, const double* U) { auto& d = ((OrcHandle*)hp)->dg; std::memcpy(d.U.data(), U, d.U.size() * 8); }
void orc_get_state(void* hp, double* U) { auto& d = ((OrcHandle*)hp)->dg; std::memcpy(U, d.U.data(), d.U.size() * 8); }
int orc_time_derivative(void* hp, double t, double* Ut) {
  auto* h = (OrcHandle*)hp;
  try { h->dg.time_derivative(t); } catch (std::exception& e) { g_err = e.what(); return 1; }
  if (Ut) std::memcpy(Ut, h->dg.Ut.data(), h->dg.Ut.size() * 8);
  return 0;
}
// one TimeDisc iteration body: CalcForcing (if channel source) then TimeStepByLSERKW2
int orc_timestep(void* hp, double* t, double dt) {
  auto* h = (OrcHandle*)hp;
  try {
    if (h->dg.C.doTCSource) h->dg.calc_forcing();
    h->dg.timestep_lserkw2(*t, dt);
  } catch (std::exception& e) { g_err = e.what(); return 1; }
  return 0;
}
double orc_calc_timestep(void* hp, int* err) { return ((OrcHandle*)hp)->dg.calc_timestep(*err); }
// timedisc.f90:115-123: overintegration of the state before the first time step
void orc_overintegrate_state(void* hp) { ((OrcHandle*)hp)->dg.overintegrate_state(); }

// additional per-node x-momentum body force, layout of U without the variable index (NULL: none)
void orc_set_force_field(void* hp, const double* F) {
  auto& d = ((OrcHandle*)hp)->dg;
  if (F) d.forceField.assign(F, F + d.U.size() / 5); else d.forceField.clear();
}

// per-element viscosity multiplier (NULL: all ones)
void orc_set_mu_scale(void* hp, const double* s) {
  auto& d = ((OrcHandle*)hp)->dg;
  if (s) d.muScale.assign(s, s + d.nE); else d.muScale.clear();
}

// exact J V of DGTimeDerivative_weakForm at the current state, by the dual-number instantiation
int orc_jvp(void* hp, const double* V, double* JV) {
  auto* h = (OrcHandle*)hp;
  try {
    if (!h->dgd) { h->dgd.reset(new DG<DD>()); h->dgd->init(h->cfg, h->mi); }
    DG<DD>& dd = *h->dgd;
    const DG<double>& d = h->dg;
    dd.muScale = d.muScale;
    dd.BulkVel = d.BulkVel;
    dd.forceField.assign(d.forceField.begin(), d.forceField.end());
    for (size_t i = 0; i < d.U.size(); ++i) dd.U[i] = DD(d.U[i], V[i]);
    dd.time_derivative(0.);
    for (size_t i = 0; i < d.U.size(); ++i) JV[i] = dd.Ut[i].d;
    return 0;
  } catch (std::exception& e) { g_err = e.what(); return 1; }
}

// exact tangent of nSteps LSERK steps of fixed dt from the current state (dual numbers):
// JV = dU(t_end)/dU(t_0) V + dU(t_end)/d(viscosity multipliers) dScale (either direction may be NULL);
// the state of the double instance is not changed
int orc_jvp_solve(void* hp, const double* V, const double* dScale, const double* dForce, int nSteps, double dt, double* JV) {
  auto* h = (OrcHandle*)hp;
  try {
    if (!h->dgd) { h->dgd.reset(new DG<DD>()); h->dgd->init(h->cfg, h->mi); }
    DG<DD>& dd = *h->dgd;
    const DG<double>& d = h->dg;
    dd.muScale = d.muScale;
    dd.muScaleR.clear();
    if (dScale)
      for (int e = 0; e < d.nE; ++e) dd.muScaleR.push_back(DD(d.muScale.empty() ? 1.0 : d.muScale[e], dScale[e]));
    dd.BulkVel = d.BulkVel;
    dd.forceField.clear();
    if (dForce || !d.forceField.empty())
      for (size_t i = 0; i < d.U.size() / 5; ++i) dd.forceField.push_back(DD(d.forceField.empty() ? 0. : d.forceField[i], dForce ? dForce[i] : 0.));
    for (size_t i = 0; i < d.U.size(); ++i) dd.U[i] = DD(d.U[i], V ? V[i] : 0.);
    double t = 0.;
    for (int s = 0; s < nSteps; ++s) {
      if (dd.C.doTCSource) dd.calc_forcing();
      dd.timestep_lserkw2(t, dt);
    }
    for (size_t i = 0; i < d.U.size(); ++i) JV[i] = dd.U[i].d;
    dd.muScaleR.clear();
    dd.forceField.clear();
    return 0;
  } catch (std::exception& e) { g_err = e.what(); return 1; }
}

// matrix-free finite-difference J V as the reference's implicit solver forms it (implicit.f90:MatrixVector,
// step size of InitImplicit): FD_Order 1 or 2, Eps_Method 1 (Qin, Ludlow, Shaw) or 2 (Knoll, Keyes)
int orc_fd_jvp(void* hp, const double* V, int fdOrder, int epsMethod, double scaleps, double* JV) {
  auto* h = (OrcHandle*)hp;
  DG<double>& d = h->dg;
  try {
    const size_t nTot = d.U.size();
    const std::vector<double> Xk = d.U;
    double Vabs = 0., normXk = 0.;
    for (size_t i = 0; i < nTot; ++i) Vabs += V[i] * V[i];
    if (epsMethod == 2) { for (size_t i = 0; i < nTot; ++i) normXk += Xk[i] * Xk[i]; normXk = std::sqrt(normXk); }
    const double mach = std::numeric_limits<double>::epsilon();
    const double rEps0 = fdOrder == 1 ? scaleps * std::sqrt(mach) : std::pow(scaleps * scaleps * 0.5 * mach, 1. / 3.);
    double eps = rEps0 / std::sqrt(Vabs);
    if (epsMethod == 2) eps *= std::sqrt(1. + normXk);
    d.time_derivative(0.);
    const std::vector<double> R0 = d.Ut;
    for (size_t i = 0; i < nTot; ++i) d.U[i] = Xk[i] + eps * V[i];
    d.time_derivative(0.);
    if (fdOrder == 1) {
      for (size_t i = 0; i < nTot; ++i) JV[i] = (d.Ut[i] - R0[i]) / eps;
    } else {
      const std::vector<double> Rp = d.Ut;
      for (size_t i = 0; i < nTot; ++i) d.U[i] = Xk[i] - eps * V[i];
      d.time_derivative(0.);
      for (size_t i = 0; i < nTot; ++i) JV[i] = (Rp[i] - d.Ut[i]) / (2. * eps);
    }
    d.U = Xk;
    return 0;
  } catch (std::exception& e) { g_err = e.what(); return 1; }
}
// point-wise fluxes of the restated reference with the handle's configuration, for the CPU tests of the GPU's point
// functions: riemann.f90:Riemann_Point's solver call on extended rotated states UE(11) (0..4 cons, 5 srho, 6..8 vel,
// 9 p, 10 T), and splitflux.f90's two-point volume flux (U(5), UPrim(6), metric vectors(3) of both nodes)
void orc_point_riemann(void* hp, int solver, const double* L, const double* R, double* F) {
  ((OrcHandle*)hp)->dg.riemann_point(solver, L, R, F);
}
void orc_point_split_volume(void* hp, const double* uR, const double* pR, const double* u, const double* p, const double* mR, const double* m,
                            double* F) {
  ((OrcHandle*)hp)->dg.split_volume_flux(uR, pR, u, p, mR, m, F);
}
double orc_bulk_velocity(void* hp) { auto& d = ((OrcHandle*)hp)->dg; d.calc_forcing(); return val(d.BulkVel); }
void orc_set_bulk_velocity(void* hp, double bv) { ((OrcHandle*)hp)->dg.BulkVel = bv; }

// mesh arrays for comparison and for the drop-in (fg_set_mesh) path
// which: 0 Mf,1 Mg,2 Mh,3 sJ,4 NormVec,5 TangVec1,6 TangVec2,7 SurfElem,8 Face_xGP,9 Elem_xGP,10 wGPVol,11 Vol
long long orc_mesh_array(void* hp, int which, double* out) {
  auto& M = ((OrcHandle*)hp)->dg.M;
  const std::vector<double>* a = nullptr;
  switch (which) {
    case 0: a = &M.Mf; break; case 1: a = &M.Mg; break; case 2: a = &M.Mh; break; case 3: a = &M.sJ; break;
    case 4: a = &M.NormVec; break; case 5: a = &M.TangVec1; break; case 6: a = &M.TangVec2; break;
    case 7: a = &M.SurfElem; break; case 8: a = &M.Face_xGP; break; case 9: a = &M.Elem_xGP; break;
    case 10: a = &M.wGPVol; break;
    case 12: a = &M.JaN_master; break; case 13: a = &M.JaN_slave; break;
    case 11: if (out) out[0] = M.Vol; return 1;
    default: return -1;
  }
  if (out) std::memcpy(out, a->data(), a->size() * 8);
  return (long long)a->size();
}
// which: 0 SideToElem(5,nSides), 1 ElemToSide(2,6,nElems), 2 BC(nBCSides)
long long orc_mesh_iarray(void* hp, int which, int* out) {
  auto& M = ((OrcHandle*)hp)->dg.M;
  const std::vector<int>* a = which == 0 ? &M.SideToElem
                              : which == 1 ? &M.ElemToSide
                              : which == 2 ? &M.BC
                              : which == 3 ? &M.MortarType
                                           : &M.MortarInfo;
  if (out) std::memcpy(out, a->data(), a->size() * 4);
  return (long long)a->size();
}
// lifted gradients of the last time derivative: which 0/1/2 = x/y/z, (4,0:N,0:N,0:N,nElems)
void orc_get_gradients(void* hp, int which, double* out) {
  auto& d = ((OrcHandle*)hp)->dg;
  auto& g = which == 0 ? d.gradUx : (which == 1 ? d.gradUy : d.gradUz);
  std::memcpy(out, g.data(), g.size() * 8);
}

// the oracle's low-storage scheme tables: stages, RKA(2..s), RKb(1..s), RKc(2..s) (1-based, length 21)
int orc_lserk_table(int code, int* stages, double* A, double* b, double* c) {
  const LserkTable* t = lserk_table(code);
  if (!t) return 1;
  *stages = t->stages;
  for (int s = 0; s < 21; ++s) { A[s] = t->A[s]; b[s] = t->b[s]; c[s] = t->c[s]; }
  return 0;
}

// algorithmic flops of one right-hand side evaluation (flop-counting scalar), divided by the DOF count
double orc_flops_per_dof_stage(void* hp) {
  auto* h = (OrcHandle*)hp;
  DG<FD> f;
  f.init(h->dg.C, h->mi);
  for (size_t x = 0; x < f.U.size(); ++x) f.U[x] = FD(h->dg.U[x]);
  f.BulkVel = h->dg.BulkVel;
  long long c0 = flop_counter();
  f.time_derivative(0.);
  // LSERK update per stage: Ut_tmp = Ut - A*Ut_tmp (2 flops), U += b dt Ut_tmp (2 flops), per variable
  long long rhs = flop_counter() - c0;
  double ndof = (double)f.nE * f.n * f.n * f.n;
  return (double)rhs / ndof + 4. * 5.;
}

// algorithmic flops per DOF of one stage, split like the GPU kernel classes:
// out[0] ConsToPrim+ProlongToFace(+face ConsToPrim), out[1] lifting, out[2] FillFlux (Riemann+viscous+BC),
// out[3] volume integral + surface integral + sign/source/Jacobian + LSERK register update, out[4] total
void orc_flops_breakdown(void* hp, double* out) {
  auto* h = (OrcHandle*)hp;
  DG<FD> f;
  f.init(h->dg.C, h->mi);
  for (size_t x = 0; x < f.U.size(); ++x) f.U[x] = FD(h->dg.U[x]);
  f.BulkVel = h->dg.BulkVel;
  f.time_derivative(0.);
  const double ndof = (double)f.nE * f.n * f.n * f.n;
  const long long* p = f.phase;
  out[0] = (p[1] - p[0]) / ndof;
  out[1] = (p[2] - p[1]) / ndof;
  out[2] = (p[4] - p[3]) / ndof;
  out[3] = ((p[3] - p[2]) + (p[5] - p[4])) / ndof + 4. * 5.;
  out[4] = out[0] + out[1] + out[2] + out[3];
}

// --------------------------------------------------------------------------------------------
// unit-test level restatements (unitTests/ProlongToFace.f90, unitTests/SurfInt.f90)
// --------------------------------------------------------------------------------------------
void orc_nodes_and_weights(int N, int type, double* x, double* w, double* wb) { nodes_and_weights(N, type, x, w, wb); }
void orc_derivative_matrix(int N, int type, double* D) {
  auto d = get_derivative_matrix(N, type);
  // return in Fortran order D(i,l) -> D[l*(N+1)+i]
  for (int i = 0; i <= N; ++i) for (int l = 0; l <= N; ++l) D[l * (N + 1) + i] = d[i * (N + 1) + l];
}
// S2V2 (2,0:N,0:N,0:4,1:6) and S2V (3,0:N,0:N,0:N,0:4,1:6) tables in Fortran order
void orc_mappings(int N, int* S2V2, int* S2V) {
  const int n = N + 1;
  for (int s = 1; s <= 6; ++s) for (int f = 0; f <= 4; ++f) for (int q = 0; q < n; ++q) for (int p = 0; p < n; ++p) {
    auto a = side_to_vol2(N, p, q, f, s);
    size_t o = ((((size_t)(s - 1) * 5 + f) * n + q) * n + p) * 2;
    S2V2[o] = a[0]; S2V2[o + 1] = a[1];
    for (int l = 0; l < n; ++l) {
      auto b = side_to_vol(N, l, p, q, f, s);
      size_t o3 = (((((size_t)(s - 1) * 5 + f) * n + q) * n + p) * n + l) * 3;
      S2V[o3] = b[0]; S2V[o3 + 1] = b[1]; S2V[o3 + 2] = b[2];
    }
  }
}
// ProlongToFace of one scalar field on the unit-test element: Uvol(0:N,0:N,0:N) -> Uface_master(0:N,0:N,nSides)
void orc_prolong_unittest(int N, int nodeType, int nSides, const int* SideToElem, const int* S2V2, const double* Lm, const double* Lp,
                          const double* Uvol, double* Um) {
  const int n = N + 1;
  for (int s = 0; s < nSides; ++s) {
    int e = SideToElem[s * 5 + 0];
    if (e <= 0) continue;
    int ls = SideToElem[s * 5 + 2];
    std::vector<double> Uf(n * n);
    for (int b = 0; b < n; ++b) for (int a = 0; a < n; ++a) {
      int i, j, k;
      if (nodeType == NT_GL) {
        int l = (ls == XI_MINUS || ls == ETA_MINUS || ls == ZETA_MINUS) ? 0 : N;
        face_vol_index(ls, a, b, l, N, i, j, k);
        Uf[b * n + a] = Uvol[((size_t)k * n + j) * n + i];
      } else {
        const double* L = (ls == XI_MINUS || ls == ETA_MINUS || ls == ZETA_MINUS) ? Lm : Lp;
        face_vol_index(ls, a, b, 0, N, i, j, k);
        double acc = Uvol[((size_t)k * n + j) * n + i] * L[0];
        for (int l = 1; l <= N; ++l) { face_vol_index(ls, a, b, l, N, i, j, k); acc += Uvol[((size_t)k * n + j) * n + i] * L[l]; }
        Uf[b * n + a] = acc;
      }
    }
    for (int q = 0; q < n; ++q) for (int p = 0; p < n; ++p) {
      size_t o = ((((size_t)(ls - 1) * 5 + 0) * n + q) * n + p) * 2;
      Um[((size_t)s * n + q) * n + p] = Uf[S2V2[o + 1] * n + S2V2[o]];
    }
  }
}
// SurfInt of one scalar flux field on the unit-test element (Flux_master = Flux_slave = Flux)
void orc_surfint_unittest(int N, int nodeType, int nSides, const int* SideToElem, const int* S2V2, const double* LhM, const double* LhP,
                          const double* Flux, double* Ut) {
  const int n = N + 1;
  for (size_t x = 0; x < (size_t)n * n * n; ++x) Ut[x] = 0.;
  auto dosurf = [&](const std::vector<double>& FT, int ls) {
    bool minus = (ls == XI_MINUS || ls == ETA_MINUS || ls == ZETA_MINUS);
    for (int b = 0; b < n; ++b) for (int a = 0; a < n; ++a) {
      if (nodeType == NT_GL) {
        int l = minus ? 0 : N; double Lh = minus ? LhM[0] : LhP[N];
        int i, j, k; face_vol_index(ls, a, b, l, N, i, j, k);
        Ut[((size_t)k * n + j) * n + i] += FT[b * n + a] * Lh;
      } else {
        const double* Lh = minus ? LhM : LhP;
        for (int l = 0; l <= N; ++l) { int i, j, k; face_vol_index(ls, a, b, l, N, i, j, k); Ut[((size_t)k * n + j) * n + i] += FT[b * n + a] * Lh[l]; }
      }
    }
  };
  for (int s = 0; s < nSides; ++s) {
    int e = SideToElem[s * 5 + 0], ne = SideToElem[s * 5 + 1];
    std::vector<double> FT(n * n);
    if (e > 0) {
      int ls = SideToElem[s * 5 + 2];
      for (int q = 0; q < n; ++q) for (int p = 0; p < n; ++p) {
        size_t o = ((((size_t)(ls - 1) * 5 + 0) * n + q) * n + p) * 2;
        FT[S2V2[o + 1] * n + S2V2[o]] = Flux[((size_t)s * n + q) * n + p];
      }
      dosurf(FT, ls);
    }
    if (ne > 0) {
      int nls = SideToElem[s * 5 + 3], flip = SideToElem[s * 5 + 4];
      for (int q = 0; q < n; ++q) for (int p = 0; p < n; ++p) {
        size_t o = ((((size_t)(nls - 1) * 5 + flip) * n + q) * n + p) * 2;
        FT[S2V2[o + 1] * n + S2V2[o]] = -Flux[((size_t)s * n + q) * n + p];
      }
      dosurf(FT, nls);
    }
  }
}

// SurfInt with SPLIT_DG on Gauss nodes for the unit-test element as the reference's unit test sets it up
// (unitTests/SurfInt.f90:130-150): U, UPrim, U_master, UPrim_master, metrics and face metrics all 1,
// SplitVolumeFluxSD; Flux_master = Flux_slave = Flux in every variable. Returns Ut of the first variable.
void orc_surfint_split_unittest(int N, int nSides, const int* SideToElem, const double* Lm, const double* Lp, const double* LhM,
                                const double* LhP, const double* Flux, double* Ut1) {
  const int n = N + 1;
  const size_t n3 = (size_t)n * n * n, n2 = (size_t)n * n;
  DGBasis B;
  B.init(N, NT_GAUSS);
  for (int l = 0; l < n; ++l) { B.Lm[l] = Lm[l]; B.Lp[l] = Lp[l]; B.LhatM[l] = LhM[l]; B.LhatP[l] = LhP[l]; }
  std::vector<double> Ut(5 * n3, 0.), Fside(5 * n2);
  const double ones[6] = {1., 1., 1., 1., 1., 1.};
  auto vol = [&](int, int, int, const double*& u, const double*& up, const double*& m) { u = ones; up = ones; m = ones; };
  auto face = [&](int, int, const double*& u, const double*& up, const double*& ja) { u = ones; up = ones; ja = ones; };
  for (int s = 0; s < nSides; ++s) {
    const int e = SideToElem[s * 5 + 0], ne = SideToElem[s * 5 + 1];
    if (e > 0) {
      for (size_t x = 0; x < n2; ++x) for (int v = 0; v < 5; ++v) Fside[x * 5 + v] = Flux[(size_t)s * n2 + x];
      split_gauss_surf_side<double>(SPLIT_SD, N, SideToElem[s * 5 + 2], 0, B, Fside.data(), vol, face, Ut.data());
    }
    if (ne > 0) {
      for (size_t x = 0; x < n2; ++x) for (int v = 0; v < 5; ++v) Fside[x * 5 + v] = -Flux[(size_t)s * n2 + x];
      split_gauss_surf_side<double>(SPLIT_SD, N, SideToElem[s * 5 + 3], SideToElem[s * 5 + 4], B, Fside.data(), vol, face, Ut.data());
    }
  }
  for (size_t x = 0; x < n3; ++x) Ut1[x] = Ut[x * 5];
}

// --------------------------------------------------------------------------------------------
// Taylor-Green vortex: taylorgreenvortex/testcase.f90:ExactFuncTestcase and AnalyzeTestcase
// --------------------------------------------------------------------------------------------
void orc_tgv_exact(int nPts, const double* x, double Ma, double kappa, double R, int iniConstDens, double* U) {
  const double rho0 = 1., U0 = 1.;
  double p0 = (U0 / Ma) * (U0 / Ma) / kappa * rho0;
  double T0 = p0 / (rho0 * R);
  for (int i = 0; i < nPts; ++i) {
    const double* X = &x[i * 3];
    double prim[6];
    prim[1] = U0 * std::sin(X[0]) * std::cos(X[1]) * std::cos(X[2]);
    prim[2] = -U0 * std::cos(X[0]) * std::sin(X[1]) * std::cos(X[2]);
    prim[3] = 0.;
    prim[4] = p0 + (rho0 * U0 * U0) / 16. * (std::cos(2 * X[0]) * std::cos(2. * X[2]) + 2. * std::cos(2. * X[1]) + 2. * std::cos(2. * X[0]) +
                                              std::cos(2 * X[1]) * std::cos(2. * X[2]));
    if (iniConstDens) { prim[0] = rho0; prim[5] = prim[4] / (prim[0] * R); }
    else { prim[5] = T0; prim[0] = prim[4] / (prim[5] * R); }
    double* u = &U[i * 5];
    u[0] = prim[0]; u[1] = prim[1] * prim[0]; u[2] = prim[2] * prim[0]; u[3] = prim[3] * prim[0];
    u[4] = 1. / (kappa - 1.) * prim[4] + 0.5 * (u[1] * prim[1] + u[2] * prim[2] + u[3] * prim[3]);
  }
}

// TGV analysis (15 columns) of state U and lifted velocity gradients (gradU*: (4,0:N,0:N,0:N,nElems)),
// integrated at NAnalyze Gauss-Lobatto points. Needs only sJ and the basis, so it takes them directly.
void orc_tgv_analysis(int N, int nodeType, int nElems, const double* sJ, const double* U, const double* gx, const double* gy,
                      const double* gz, int NAnalyze, double kappa, double R, double mu0, double* out) {
  const int n = N + 1, na = NAnalyze + 1;
  DGBasis B; B.init(N, nodeType);
  std::vector<double> xa(na), wa(na);
  nodes_and_weights(NAnalyze, NT_GL, xa.data(), wa.data(), nullptr);
  auto V = init_vandermonde(N, NAnalyze, B.wBary.data(), B.xGP.data(), xa.data());
  double Vol = 0.;
  for (int e = 0; e < nElems; ++e) for (int k = 0; k < n; ++k) for (int j = 0; j < n; ++j) for (int i = 0; i < n; ++i)
    Vol += B.wGP[i] * B.wGP[j] * B.wGP[k] / sJ[(((size_t)e * n + k) * n + j) * n + i];
  double Ekin = 0, Ekc = 0, Tm = 0, Ent = 0, DRu = 0, DRS = 0, DRSd = 0, DRp = 0, EDS = 0, EDD = 0, Enst = 0, vmax = 0;
  const double sKM1 = 1. / (kappa - 1.), rho0 = 1.;
  std::vector<double> sJa((size_t)na * na * na), Ua((size_t)na * na * na * 5), Gx((size_t)na * na * na * 3), Gy(Gx.size()), Gz(Gx.size());
  std::vector<double> tmp3((size_t)n * n * n * 3);
  for (int e = 0; e < nElems; ++e) {
    change_basis_3d(1, N, NAnalyze, V, &sJ[(size_t)e * n * n * n], sJa.data());
    change_basis_3d(5, N, NAnalyze, V, &U[(size_t)e * n * n * n * 5], Ua.data());
    const double* gs[3] = {gx, gy, gz};
    std::vector<double>* Go[3] = {&Gx, &Gy, &Gz};
    for (int d = 0; d < 3; ++d) {
      for (size_t x = 0; x < (size_t)n * n * n; ++x) for (int c = 0; c < 3; ++c) tmp3[x * 3 + c] = gs[d][((size_t)e * n * n * n + x) * 4 + c];
      change_basis_3d(3, N, NAnalyze, V, tmp3.data(), Go[d]->data());
    }
    for (int k = 0; k < na; ++k) for (int j = 0; j < na; ++j) for (int i = 0; i < na; ++i) {
      size_t x = ((size_t)k * na + j) * na + i;
      const double* u = &Ua[x * 5];
      double rho = u[0], s = 1. / rho, vel[3] = {u[1] * s, u[2] * s, u[3] * s};
      double p = (kappa - 1.) * (u[4] - 0.5 * (u[1] * vel[0] + u[2] * vel[1] + u[3] * vel[2]));
      double T = p * s / R;
      double G[3][3];  // GradVel(:,1)=GradVelx etc: G[a][b] = d vel_a / d x_b
      for (int a = 0; a < 3; ++a) { G[a][0] = Gx[x * 3 + a]; G[a][1] = Gy[x * 3 + a]; G[a][2] = Gz[x * 3 + a]; }
      double divU = G[0][0] + G[1][1] + G[2][2];
      double S[3][3], Sd[3][3];
      for (int a = 0; a < 3; ++a) for (int b = 0; b < 3; ++b) { S[a][b] = 0.5 * (G[a][b] + G[b][a]); Sd[a][b] = S[a][b]; }
      for (int a = 0; a < 3; ++a) Sd[a][a] -= 1. / 3. * divU;
      double w[3] = {G[2][1] - G[1][2], G[0][2] - G[2][0], G[1][0] - G[0][1]};
      double w2 = w[0] * w[0] + w[1] * w[1] + w[2] * w[2];
      vmax = std::max(vmax, std::sqrt(w2));
      double IF = wa[i] * wa[j] * wa[k] / sJa[x];
      double v2 = vel[0] * vel[0] + vel[1] * vel[1] + vel[2] * vel[2];
      Tm += IF * T;
      Ent += IF * (-sKM1) * rho * (std::log(p) - kappa * std::log(rho));
      Ekin += IF * 0.5 * v2;
      Ekc += IF * 0.5 * rho * v2;
      Enst += IF * 0.5 * rho * w2;
      double sG = 0, sS = 0, sSd = 0;
      for (int a = 0; a < 3; ++a) for (int b = 0; b < 3; ++b) { sG += G[a][b] * G[a][b]; sS += S[a][b] * S[a][b]; sSd += Sd[a][b] * Sd[a][b]; }
      DRu += IF * sG; DRS += IF * sS; DRSd += IF * sSd; DRp += IF * p * divU;
      EDS += IF * mu0 * w2; EDD += IF * mu0 * divU * divU;
    }
  }
  Ekin /= Vol; Ekc = Ekc / Vol / rho0; Tm /= Vol; Ent /= Vol;
  Enst = Enst / (rho0 * Vol); DRu = DRu * mu0 / Vol; DRS = DRS * 2. * mu0 / (rho0 * Vol); DRSd = DRSd * 2. * mu0 / (rho0 * Vol);
  DRp = -DRp / (rho0 * Vol); EDS = EDS / Vol; EDD = EDD * 4. / 3. / Vol;
  double up = std::sqrt(2. / 3. * Ekin);
  double r[15] = {DRS, DRSd + DRp, Ekin, Ekc, Enst, DRu, DRS, DRSd, DRp, vmax, Tm, up, Ent, EDS, EDD};
  for (int c = 0; c < 15; ++c) out[c] = r[c];
}

}  // extern "C"
