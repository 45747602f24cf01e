// flexi_gb300 -- device data layout and point-wise physics of the DGSEM Navier-Stokes operator.
//
// Everything is FP64. GB300's FP64 pipe (a pure DFMA stream attains 0.53 T instr/s, 1.06 TFLOP/s) is ~70x slower than
// its FP32 pipe and ~30x below what this operator needs to be HBM-bound, so the kernels are organised to
// minimise FP64 instructions: reciprocals are formed once and reused, constant factors are folded, face
// values are computed once per side and read by both neighbours, and integer/shared-memory work (which
// is essentially free next to FP64) replaces recomputation wherever possible.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#define FG_MAXN 12  // maximum number of nodes per direction (N <= 11)

namespace fg {

// local side ids of FLEXI (src/flexi.h:90-95)
enum { ZETA_MINUS = 1, ETA_MINUS = 2, XI_PLUS = 3, ETA_PLUS = 4, XI_MINUS = 5, ZETA_PLUS = 6 };
// riemann.f90:44-58 and splitflux.f90:63-69
enum { RIEMANN_LF = 1, RIEMANN_HLLC = 2, RIEMANN_ROE = 3, RIEMANN_ROEL2 = 32, RIEMANN_ROEENTROPYFIX = 33, RIEMANN_ROEENTROPYGSHOCKFIX = 34,
       RIEMANN_HLL = 4, RIEMANN_HLLE = 5, RIEMANN_HLLEM = 6, RIEMANN_CH = 7, RIEMANN_IR = 8, RIEMANN_AVERAGE = 0 };
enum { SPLIT_SD = 0, SPLIT_MO = 1, SPLIT_DU = 2, SPLIT_KG = 3, SPLIT_PI = 4, SPLIT_CH = 5, SPLIT_IR = 6 };
enum { NODE_GAUSS = 1, NODE_GL = 2 };

// face state fields, stored [side][field][p + n*q] for the master and for the slave (in master orientation)
enum { FS_RHO = 0, FS_E, FS_U, FS_V, FS_W, FS_P, FS_T, FS_SRHO, FS_NF };
// volume primitive fields, stored [elem][field][node]
enum { VP_SRHO = 0, VP_U, VP_V, VP_W, VP_P, VP_T, VP_NF };
// face geometry, stored [side][field][p + n*q]
enum { FG_NX = 0, FG_NY, FG_NZ, FG_T1X, FG_T1Y, FG_T1Z, FG_T2X, FG_T2Y, FG_T2Z, FG_SURF, FG_NF };

// Operator constants passed by value (they live in the kernel-parameter constant bank).
struct Basis {
  int N, n, nodeType, splitDG;
  int riemann, riemannBC, lifting, weakLifting;
  double D_T[FG_MAXN * FG_MAXN];     // D_T[l*n+i] = D(i,l)
  double Dhat_T[FG_MAXN * FG_MAXN];  // Dhat_T[l*n+i] = D_Hat_T(l,i)
  double DVS[FG_MAXN * FG_MAXN];     // DVS[l*n+i] = DVolSurf(l,i)
  double Lm[FG_MAXN], Lp[FG_MAXN], LhM[FG_MAXN], LhP[FG_MAXN];
  double kappa, kappaM1, sKappaM1, Rgas, sR, lambdaFac, etaBR2, etaBR2_wall;
  double kappaFac, sKappaP1;
  double logEntC, kappa_kappaM1;  // ln((kappa-1)^(1/(kappa-1))), kappa/(kappa-1): eos.f90:EntropyToCons
  double riemannPhi;              // RiemannPhiFactor of RoeEntropyGShockFix
  // even-odd form of D (eoD) and D_Hat (eoDh), row a = node a of a line, 8 columns: for a < n/2 the
  // coefficients 1/2 (M(a,l) + M(a,N-l)) (l < n/2) on the sums s_l = u_l + u_{N-l}; for a past the middle
  // 1/2 (M(N-a,l) - M(N-a,N-l)) on the differences d_l = u_l - u_{N-l}; for the middle node of odd n M(m,l) on d_l;
  // column n/2: M(a,m) (odd n, a < n/2), column n/2+1: the sign (+1, -1, 0 middle) that combines a lane's sum
  // with its mirror lane's (eo_line_derivative)
  double eoD[FG_MAXN * 8];
  double eoDh[FG_MAXN * 8];
};

// Basis::eoD and eoDh from D_T and Dhat_T (both must be filled): D(i,l) = D_T[l*n+i], D_Hat(i,l) = Dhat_T[l*n+i].
inline void fill_even_odd(Basis& B) {
  const int n = B.n, N = n - 1, h = n / 2, m = N / 2;
  auto fill = [&](double* T, const double* MT) {
    auto M = [&](int i, int l) { return MT[l * n + i]; };
    for (int a = 0; a < n; ++a) {
      double* r = T + a * 8;
      for (int c = 0; c < 8; ++c) r[c] = 0.;
      if (a < h) {
        for (int c = 0; c < h; ++c) r[c] = 0.5 * (M(a, c) + M(a, N - c));
        r[h] = (n % 2) ? M(a, m) : 0.;
        r[h + 1] = 1.;
      } else if (n % 2 && a == m) {
        for (int c = 0; c < h; ++c) r[c] = M(m, c);
      } else {
        for (int c = 0; c < h; ++c) r[c] = 0.5 * (M(N - a, c) - M(N - a, N - c));
        r[h + 1] = -1.;
      }
    }
  };
  fill(B.eoD, B.D_T);
  fill(B.eoDh, B.Dhat_T);
}

// Device arrays of one solver handle (all sizes in units of doubles / ints).
struct Dev {
  int nElems, nSides, nBCSides, nInst;
  // elements
  double* U;       // [e][5][n3]
  double* Ut;      // [e][5][n3] time derivative (RK register source)
  double* Ut_tmp;  // [e][5][n3] LSERK register
  double* prim;    // [e][VP_NF][n3]
  double* grad;    // [e][12][n3]: index 4*dir + var, var = (u,v,w,T)
  double* metr;    // [e][9][n3]: Metrics_fTilde(3), Metrics_gTilde(3), Metrics_hTilde(3)
  double* metrJ;   // [e][9][n3]: metr times sJ (null: the kernels form the products)
  double* sJ;      // [e][n3]
  int* elemSide;   // [e][6]: 8*sideID + flip (flip 0 => this element is the master)
  int* elemInst;   // [e]
  // sides
  double* faceM;   // [s][FS_NF][n2]
  double* faceS;   // [s][FS_NF][n2]
  double* gradM;   // [s][12][n2]
  double* gradS;   // [s][12][n2]
  double* faceJa;  // [e][6][3][n2]: normal row of the element's own face metrics (split form on Gauss nodes; else null)
  double* geo;     // [s][FG_NF][n2]
  double* flux;    // [s][5][n2] numerical flux times SurfElem, master orientation
  int* sideElem;   // [s][4]: master elem, master locSide, slave elem (-1: BC side), 8*slave locSide + flip
  int* sideInst;   // [s]
  int* bcType;     // [nBCSides]
  double* bcTwall; // [nBCSides]
  // per instance
  double* mu0;     // [nInst]
  double* dt;      // [nInst]
  double* bulkVel; // [nInst]
  double* dpdx;    // [nInst] (0 when no body force)
  double* muScale; // [nElems] viscosity multiplier of each element (null: 1)
  double* forceField;  // [e][n3] additional x-momentum body force per node, energy source F * bulkVel (null: none)
  // source of an exact function (exactfunc.f90:CalcSource; null: none): srcPar = (omega, a, tmp(1:6)) of
  // IniExactFunc 4, elemX [e][3][n3] the solution points, tStage [nInst] the time of the current RK stage,
  // tStep [nInst] the time at the start of the current step
  const double* srcPar;
  const double* elemX;
  double* tStage;
  double* tStep;
  double* scratch;  // element kernels whose per-element arrays exceed shared memory (lines of 9..12 nodes):
                    // [block][scratchStride] (null otherwise)
  long long scratchStride;
  // mortar interfaces (mortar.f90): sides are ordered BC | conforming inner | small mortar | big mortar;
  // k_flux handles the first nFluxSides, the mortar kernels the rest
  int nFluxSides, nMortars;
  double* mortarLift;  // [m][12][n2] BR1 lifting flux times normal (4*dir + var) projected onto big side m
  int* err;        // [1] sticky error word
  double* dtElem;  // [2][nElems] convective and viscous element time-step limits of the last CALCTIMESTEP
  const int* dtSkip;  // [nInst] nonzero: the instance needs no CALCTIMESTEP in this step (null: every instance does)
  // element range of one volume-kernel launch: elements volBegin .. volBegin + volCount - 1 (volCount 0: all);
  // volBegin is a multiple of the kernel's elements per CTA
  int volBegin, volCount;
};

// Overintegration (overintegration.f90): type 1 the modal cut-off filter F = Vdm_Leg diag(1..1,0..0) sVdm_Leg
// on J u_t; type 2 the conservative cut-off (project J u_t to NUnder, times 1/J on NUnder, back to N).
struct OverintDev {
  int type, nu;         // 0/1/2, NUnder + 1
  const double* F;      // [n][n]: F[i*n+l] = OverintegrationMat(i,l)
  const double* VNU;    // [nu][n]: Vdm_N_NUnder(iU,i)
  const double* VUN;    // [n][nu]: Vdm_NUnder_N(i,iU)
  const double* sJNU;   // [e][nu^3]: 1/J on the NUnder nodes
};

// Mortar operators and table (mortar.f90:InitMortar, fillmortar.t90), passed to the mortar kernels only.
// Big mortar side m is side nSides - nMortars + m, its small sides are listed in info.
struct MortarDev {
  const int* info;                // [m][6]: type (1: 1->4, 2: 1->2 in eta, 3: 1->2 in xi), big side, small sides (-1: unused)
  double M01[FG_MAXN * FG_MAXN];  // [l*n+p] = M_0_1(l,p): big-side node l -> small-side node p, first half
  double M02[FG_MAXN * FG_MAXN];  // second half
  double M10[FG_MAXN * FG_MAXN];  // [l*n+p] = M_1_0(l,p): small-side node l (first half) -> big-side node p (L2 projection)
  double M20[FG_MAXN * FG_MAXN];  // second half
};

// viscosity of element e: its instance's mu0 times its multiplier
__host__ __device__ inline double elem_mu(const Dev& d, int e) {
  const double m = d.mu0[d.elemInst[e]];
  return d.muScale ? m * d.muScale[e] : m;
}

// ------------------------------------------------------------------------------------------------------
// orientation maps (mappings.f90: Flip_S2M, CGNS_SideToVol2) -- integer work, free next to FP64
// ------------------------------------------------------------------------------------------------------
__host__ __device__ inline void flip_s2m(int N, int p, int q, int flip, int& a, int& b) {
  switch (flip) {
    case 0: a = p; b = q; break;
    case 1: a = q; b = p; break;
    case 2: a = N - p; b = q; break;
    case 3: a = N - q; b = N - p; break;
    default: a = p; b = N - q; break;
  }
}
__host__ __device__ inline void side_to_vol2(int N, int p, int q, int flip, int ls, int& a, int& b) {
  int x, y;
  flip_s2m(N, p, q, flip, x, y);
  switch (ls) {
    case XI_MINUS: a = y; b = x; break;
    case XI_PLUS: a = x; b = y; break;
    case ETA_MINUS: a = x; b = y; break;
    case ETA_PLUS: a = N - x; b = y; break;
    case ZETA_MINUS: a = y; b = x; break;
    default: a = x; b = y; break;
  }
}
// node index of face coordinate (a,b) at normal distance l counted in volume index order
__host__ __device__ inline int face_node(int ls, int a, int b, int l, int n) {
  switch (ls) {
    case XI_MINUS: case XI_PLUS: return l + n * (a + n * b);
    case ETA_MINUS: case ETA_PLUS: return a + n * (l + n * b);
    default: return a + n * (b + n * l);
  }
}
__host__ __device__ inline bool side_is_minus(int ls) { return ls == XI_MINUS || ls == ETA_MINUS || ls == ZETA_MINUS; }
__host__ __device__ inline int side_dir(int ls) {  // 0 xi, 1 eta, 2 zeta
  return (ls == XI_MINUS || ls == XI_PLUS) ? 0 : ((ls == ETA_MINUS || ls == ETA_PLUS) ? 1 : 2);
}

// ------------------------------------------------------------------------------------------------------
// point-wise physics
// ------------------------------------------------------------------------------------------------------
// Viscous flux (flux.f90:EvalDiffFlux3D_Point, stored with the minus sign), contracted with a direction
// vector m: F = m1*f + m2*g + m3*h. g[4*d+v] = d/dx_d of (u,v,w,T). Returns F[1..4] (F[0] = 0).
__host__ __device__ __forceinline__ void visc_flux_dir(double mu, double lam, double u, double v, double w, const double* g,
                                              double m1, double m2, double m3, double* F) {
  // tau terms (s43 = 4/3, s23 = 2/3): tau_xx = mu*(4/3 ux - 2/3 (vy + wz)) = mu*(2 ux - 2/3 div)
  const double div = g[0] + g[5] + g[10];
  const double mdiv = (2.0 / 3.0) * div;
  const double txx = mu * (2.0 * g[0] - mdiv);
  const double tyy = mu * (2.0 * g[5] - mdiv);
  const double tzz = mu * (2.0 * g[10] - mdiv);
  const double txy = mu * (g[4] + g[1]);
  const double txz = mu * (g[8] + g[2]);
  const double tyz = mu * (g[9] + g[6]);
  // row of tau contracted with m
  const double a1 = txx * m1 + txy * m2 + txz * m3;
  const double a2 = txy * m1 + tyy * m2 + tyz * m3;
  const double a3 = txz * m1 + tyz * m2 + tzz * m3;
  const double qn = g[3] * m1 + g[7] * m2 + g[11] * m3;
  F[1] = -a1;
  F[2] = -a2;
  F[3] = -a3;
  F[4] = -(a1 * u + a2 * v + a3 * w) - lam * qn;
}

// The same flux in three directions of one node: the stress tensor formed once (tau = txx, tyy, tzz, txy,
// txz, tyz), then contracted with each direction vector.
__host__ __device__ __forceinline__ void visc_tau(double mu, const double* g, double* tau) {
  const double mdiv = (2.0 / 3.0) * (g[0] + g[5] + g[10]);
  tau[0] = mu * (2.0 * g[0] - mdiv);
  tau[1] = mu * (2.0 * g[5] - mdiv);
  tau[2] = mu * (2.0 * g[10] - mdiv);
  tau[3] = mu * (g[4] + g[1]);
  tau[4] = mu * (g[8] + g[2]);
  tau[5] = mu * (g[9] + g[6]);
}
__host__ __device__ __forceinline__ void visc_flux_tau(const double* tau, double lam, double u, double v, double w, const double* g,
                                                       double m1, double m2, double m3, double* F) {
  const double a1 = tau[0] * m1 + tau[3] * m2 + tau[4] * m3;
  const double a2 = tau[3] * m1 + tau[1] * m2 + tau[5] * m3;
  const double a3 = tau[4] * m1 + tau[5] * m2 + tau[2] * m3;
  const double qn = g[3] * m1 + g[7] * m2 + g[11] * m3;
  F[1] = -a1;
  F[2] = -a2;
  F[3] = -a3;
  F[4] = -(a1 * u + a2 * v + a3 * w) - lam * qn;
}

// Rotated extended state (riemann.f90:Riemann_Point): rho, srho, E, p, vn, vt1, vt2.
struct RotState {
  double rho, srho, E, p, v1, v2, v3;
};

// splitflux.f90:GetLogMean (Ismail and Roe): (a + b) / g, g = log(chi) / f or its series 2 + 2/3 u + 2/5 u^2 + 2/7 u^3
// (u = f^2) for |f| < 0.1, chi = a / b, f = (chi - 1) / (chi + 1)
__host__ __device__ __forceinline__ double log_mean(double a, double b) {
  const double chi = a / b;
  const double f = (chi - 1.0) / (chi + 1.0);
  double g;
  if (fabs(f) < 0.1) {
    const double u = f * f;
    g = 2.0 + u * ((2.0 / 3.0) + u * (0.4 + u * (2.0 / 7.0)));
  } else {
    g = log(chi) / f;
  }
  return (a + b) / g;
}

// Central split surface flux (splitflux.f90:SplitSurfaceFlux*) on rotated states: SD, MO, DU, KG, PI, CH, IR.
__host__ __device__ __forceinline__ void split_surface_flux_more(int splitDG, const Basis& B, const RotState& L, const RotState& R,
                                                                 double* F) {
  const double mL = L.rho * L.v1, mR = R.rho * R.v1;
  if (splitDG == SPLIT_MO) {
    const double rhoepL = L.E - 0.5 * L.rho * (L.v1 * L.v1 + L.v2 * L.v2 + L.v3 * L.v3) + L.p;
    const double rhoepR = R.E - 0.5 * R.rho * (R.v1 * R.v1 + R.v2 * R.v2 + R.v3 * R.v3) + R.p;
    const double ms = mL + mR;
    F[0] = 0.5 * ms;
    F[1] = 0.25 * ms * (L.v1 + R.v1) + 0.5 * (L.p + R.p);
    F[2] = 0.25 * ms * (L.v2 + R.v2);
    F[3] = 0.25 * ms * (L.v3 + R.v3);
    // {rho u v_k}{v_k} - 1/2 {rho u v_k^2} summed over k = 1/4 (mL + mR) ... as (mL vL.vR + mR vL.vR) / 4
    const double vv = L.v1 * R.v1 + L.v2 * R.v2 + L.v3 * R.v3;
    F[4] = 0.5 * (rhoepL * L.v1 + rhoepR * R.v1) + 0.25 * ms * vv;
  } else if (splitDG == SPLIT_DU) {
    const double us = L.v1 + R.v1;
    F[0] = 0.25 * (L.rho + R.rho) * us;
    F[1] = 0.25 * (mL + mR) * us + 0.5 * (L.p + R.p);
    F[2] = 0.25 * (L.rho * L.v2 + R.rho * R.v2) * us;
    F[3] = 0.25 * (L.rho * L.v3 + R.rho * R.v3) * us;
    F[4] = 0.25 * (L.E + R.E + L.p + R.p) * us;
  } else if (splitDG == SPLIT_KG) {
    const double rs = L.rho + R.rho, us = L.v1 + R.v1;
    const double b = 0.125 * rs * us;
    F[0] = 0.25 * rs * us;
    F[1] = b * us + 0.5 * (L.p + R.p);
    F[2] = b * (L.v2 + R.v2);
    F[3] = b * (L.v3 + R.v3);
    F[4] = b * (L.E * L.srho + R.E * R.srho) + 0.25 * (L.p + R.p) * us;
  } else if (splitDG == SPLIT_CH) {
    const double bL = 0.5 * L.rho / L.p, bR = 0.5 * R.rho / R.p;
    const double rhoLog = log_mean(L.rho, R.rho), betaLog = log_mean(bL, bR);
    const double pHat = 0.5 * (L.rho + R.rho) / (bL + bR);
    const double H = 0.5 * B.sKappaM1 / betaLog + pHat / rhoLog + 0.5 * (L.v1 * R.v1 + L.v2 * R.v2 + L.v3 * R.v3);
    F[0] = rhoLog * 0.5 * (L.v1 + R.v1);
    F[1] = F[0] * 0.5 * (L.v1 + R.v1) + pHat;
    F[2] = F[0] * 0.5 * (L.v2 + R.v2);
    F[3] = F[0] * 0.5 * (L.v3 + R.v3);
    F[4] = F[0] * H;
  } else {  // IR
    const double zL1 = sqrt(L.rho / L.p), zL5 = sqrt(L.rho * L.p), zR1 = sqrt(R.rho / R.p), zR5 = sqrt(R.rho * R.p);
    const double z1Log = log_mean(zL1, zR1), z5Log = log_mean(zL5, zR5);
    const double z1s = zL1 + zR1;  // 2 z1Mean
    const double rhoHat = 0.5 * z1s * z5Log;
    const double pHat = (zL5 + zR5) / z1s;
    const double p2Hat = 0.5 / B.kappa * ((B.kappa + 1.0) * z5Log / z1Log + B.kappaM1 * pHat);
    const double uHat = (zL1 * L.v1 + zR1 * R.v1) / z1s, vHat = (zL1 * L.v2 + zR1 * R.v2) / z1s, wHat = (zL1 * L.v3 + zR1 * R.v3) / z1s;
    const double hHat = B.kappa * p2Hat / (rhoHat * B.kappaM1) + 0.5 * (uHat * uHat + vHat * vHat + wHat * wHat);
    F[0] = rhoHat * uHat;
    F[1] = F[0] * uHat + pHat;
    F[2] = F[0] * vHat;
    F[3] = F[0] * wHat;
    F[4] = F[0] * hHat;
  }
}

// Central split surface flux (splitflux.f90:SplitSurfaceFluxPI / SD) on rotated states.
__host__ __device__ __forceinline__ void split_surface_flux(int splitDG, const RotState& L, const RotState& R, double HL, double HR, double* F) {
  if (splitDG == 4) {
    const double rs = L.rho + R.rho, us = L.v1 + R.v1;
    const double a = rs * us;
    const double b = 0.125 * a;
    F[0] = 0.25 * a;
    F[1] = b * us + 0.5 * (L.p + R.p);
    F[2] = b * (L.v2 + R.v2);
    F[3] = b * (L.v3 + R.v3);
    F[4] = b * (HL + HR);
  } else {  // SD: 0.5*(F_L+F_R)
    const double mL = L.rho * L.v1, mR = R.rho * R.v1;
    F[0] = 0.5 * (mL + mR);
    F[1] = 0.5 * (mL * L.v1 + L.p + mR * R.v1 + R.p);
    F[2] = 0.5 * (mL * L.v2 + mR * R.v2);
    F[3] = 0.5 * (mL * L.v3 + mR * R.v3);
    F[4] = 0.5 * ((L.E + L.p) * L.v1 + (R.E + R.p) * R.v1);
  }
}

__host__ __device__ __forceinline__ void euler_flux_1d(const RotState& S, double* F) {
  const double m = S.rho * S.v1;
  F[0] = m;
  F[1] = m * S.v1 + S.p;
  F[2] = m * S.v2;
  F[3] = m * S.v3;
  F[4] = (S.E + S.p) * S.v1;
}

// central flux of the split form for any SplitDG (GEN) or for PI / SD only
template <bool GEN>
__host__ __device__ __forceinline__ void central_flux(int splitDG, const Basis& B, const RotState& L, const RotState& R, double HL, double HR,
                                                      double* F) {
  if (GEN && splitDG != SPLIT_PI && splitDG != SPLIT_SD) split_surface_flux_more(splitDG, B, L, R, F);
  else split_surface_flux(splitDG, L, R, HL, HR, F);
}

// Riemann solvers of riemann.f90 (LF :558, HLLC :594, Roe :668, RoeEntropyFix :748) on rotated states.
// split != 0: central part from the split surface flux (SPLIT_DG builds), as the reference does; GEN: any SplitDG.
template <bool GEN = false>
__host__ __device__ __forceinline__ void riemann_rotated(int solver, int splitDG, const Basis& B, const RotState& L, const RotState& R, double* F) {
  const bool split = splitDG >= 0;
  const double HL = (L.E + L.p) * L.srho, HR = (R.E + R.p) * R.srho;
  if (solver == RIEMANN_LF) {
    const double cL = sqrt(B.kappa * L.p * L.srho), cR = sqrt(B.kappa * R.p * R.srho);
    const double lmax = fmax(fabs(R.v1), fabs(L.v1)) + fmax(cL, cR);
    const double dU[5] = {R.rho - L.rho, R.rho * R.v1 - L.rho * L.v1, R.rho * R.v2 - L.rho * L.v2, R.rho * R.v3 - L.rho * L.v3, R.E - L.E};
    if (!split) {
      double FL[5], FR[5];
      euler_flux_1d(L, FL); euler_flux_1d(R, FR);
#pragma unroll
      for (int v = 0; v < 5; ++v) F[v] = 0.5 * ((FL[v] + FR[v]) - lmax * dU[v]);
    } else {
      central_flux<GEN>(splitDG, B, L, R, HL, HR, F);
      const double h = 0.5 * lmax;
#pragma unroll
      for (int v = 0; v < 5; ++v) F[v] = F[v] - h * dU[v];
    }
    return;
  }
  const double sqL = sqrt(L.rho), sqR = sqrt(R.rho);
  const double ssq = 1.0 / (sqL + sqR);
  const double r1v = (sqR * R.v1 + sqL * L.v1) * ssq;
  const double r2v = (sqR * R.v2 + sqL * L.v2) * ssq;
  const double r3v = (sqR * R.v3 + sqL * L.v3) * ssq;
  const double rH = (sqR * HR + sqL * HL) * ssq;
  const double absVel = r1v * r1v + r2v * r2v + r3v * r3v;
  const double rc = sqrt(B.kappaM1 * (rH - 0.5 * absVel));
  if (solver == RIEMANN_HLLC) {
    // the side X whose flux (and, subsonic, whose star state) the interface takes is selected first, so
    // that a warp evaluates one Euler flux and one star state whatever mix of sides its points take
    const double Ssl = r1v - rc, Ssr = r1v + rc;
    const bool supL = Ssl >= 0.0, supR = !supL && Ssr <= 0.0;
    const double sMuL = Ssl - L.v1, sMuR = Ssr - R.v1;
    const double mL = L.rho * L.v1, mR = R.rho * R.v1;
    double SStar = 0.0;
    if (!supL && !supR) SStar = (R.p - L.p + mL * sMuL - mR * sMuR) / (L.rho * sMuL - R.rho * sMuR);
    const bool useL = supL || (!supR && SStar >= 0.0);  // subsonic: Ssl < 0, the left star state for SStar >= 0
    const RotState& X = useL ? L : R;
    double FX[5];
    euler_flux_1d(X, FX);
    if (supL || supR) {
#pragma unroll
      for (int v = 0; v < 5; ++v) F[v] = FX[v];
    } else {
      const double S = useL ? Ssl : Ssr, sMu = useL ? sMuL : sMuR, m = useL ? mL : mR;
      const double EStar = X.E * X.srho + (SStar - X.v1) * (SStar + X.p * X.srho / sMu);
      const double fac = X.rho * sMu / (S - SStar);
      const double Us[5] = {fac, fac * SStar, fac * X.v2, fac * X.v3, fac * EStar};
      const double Uc[5] = {X.rho, m, X.rho * X.v2, X.rho * X.v3, X.E};
#pragma unroll
      for (int v = 0; v < 5; ++v) F[v] = FX[v] + S * (Us[v] - Uc[v]);
    }
    return;
  }
  // Roe-type: eigenvalues a, strengths Alpha, eigenvectors r1..r5
  double a0 = r1v - rc, a1 = r1v, a4 = r1v + rc;
  double A0, A1, A2, A3, A4;
  double e0, e1, e4;  // |a| after the optional entropy fix (a1 = a2 = a3)
  if (solver == RIEMANN_ROE) {
    const double d0 = R.rho - L.rho;
    const double d1 = R.rho * R.v1 - L.rho * L.v1;
    const double d2 = R.rho * R.v2 - L.rho * L.v2;
    const double d3 = R.rho * R.v3 - L.rho * L.v3;
    const double d4 = R.E - L.E;
    A2 = d2 - r2v * d0;
    A3 = d3 - r3v * d0;
    const double d5 = d4 - A2 * r2v - A3 * r3v;
    const double src = 1.0 / rc;
    A1 = B.kappaM1 * (src * src) * (d0 * (rH - r1v * r1v) - d5 + r1v * d1);
    A0 = 0.5 * src * (d0 * (r1v + rc) - d1 - rc * A1);
    A4 = d0 - A0 - A1;
    e0 = fabs(a0); e1 = fabs(a1); e4 = fabs(a4);
  } else {  // RoeEntropyFix
    const double cL = sqrt(B.kappa * L.p * L.srho), cR = sqrt(B.kappa * R.p * R.srho);
    const double RoeDens = sqL * sqR;
    const double dr = R.rho - L.rho, du = R.v1 - L.v1, dv = R.v2 - L.v2, dw = R.v3 - L.v3, dp = R.p - L.p;
    const double tmp = 0.5 / (rc * rc);
    const double rdc = RoeDens * rc * du;
    A0 = tmp * (dp - rdc);
    A1 = dr - dp * (2.0 * tmp);
    A2 = RoeDens * dv;
    A3 = RoeDens * dw;
    A4 = tmp * (dp + rdc);
    // Harten-Hyman entropy fix
    auto fix = [](double a, double al, double ar) {
      const double da = fmax(0.0, fmax(a - al, ar - a));
      const double aa = fabs(a);
      double e = aa;
      if (aa < da) e = 0.5 * (a * a / da + da);  // a branch: the division only where the fix applies
      return e;
    };
    e0 = fix(a0, L.v1 - cL, R.v1 - cR);
    e1 = fix(a1, L.v1, R.v1);
    e4 = fix(a4, L.v1 + cL, R.v1 + cR);
  }
  // dissipation D = sum_k Alpha_k |a_k| r_k
  const double w0 = A0 * e0, w1 = A1 * e1, w2 = A2 * e1, w3 = A3 * e1, w4 = A4 * e4;
  double D[5];
  D[0] = w0 + w1 + w4;
  D[1] = w0 * a0 + w1 * r1v + w4 * a4;
  D[2] = (w0 + w1 + w4) * r2v + w2;
  D[3] = (w0 + w1 + w4) * r3v + w3;
  D[4] = w0 * (rH - r1v * rc) + w1 * (0.5 * absVel) + w2 * r2v + w3 * r3v + w4 * (rH + r1v * rc);
  if (!split) {
    double FL[5], FR[5];
    euler_flux_1d(L, FL); euler_flux_1d(R, FR);
#pragma unroll
    for (int v = 0; v < 5; ++v) F[v] = 0.5 * ((FL[v] + FR[v]) - D[v]);
  } else {
    central_flux<GEN>(splitDG, B, L, R, HL, HR, F);
#pragma unroll
    for (int v = 0; v < 5; ++v) F[v] = F[v] - 0.5 * D[v];
  }
}

// The other Riemann solvers of riemann.f90 -- RoeL2 (:983), RoeEntropyGShockFix (:866), HLL (:1067), HLLE (:1119),
// HLLEM (:1170), and with the split form the flux average (:1236), CH (:1261) and IR (:1315) -- and every solver with
// the split fluxes MO, DU, KG, CH, IR, on rotated states.
__host__ __device__ inline void riemann_rotated_more(int solver, int splitDG, const Basis& B, const RotState& L, const RotState& R, double* F) {
  if (solver == RIEMANN_LF || solver == RIEMANN_HLLC || solver == RIEMANN_ROE || solver == RIEMANN_ROEENTROPYFIX) {
    riemann_rotated<true>(solver, splitDG, B, L, R, F);
    return;
  }
  const bool split = splitDG >= 0;
  const double HL = (L.E + L.p) * L.srho, HR = (R.E + R.p) * R.srho;
  if (solver == RIEMANN_AVERAGE) {
    central_flux<true>(splitDG, B, L, R, HL, HR, F);
    return;
  }
  const double cL = sqrt(B.kappa * L.p * L.srho), cR = sqrt(B.kappa * R.p * R.srho);
  if (solver == RIEMANN_CH) {
    const double lmax = fmax(fabs(R.v1), fabs(L.v1)) + fmax(cL, cR);
    const double rhoMean = 0.5 * (L.rho + R.rho);
    const double bL = 0.5 * L.rho / L.p, bR = 0.5 * R.rho / R.p;
    const double betaLog = log_mean(bL, bR);
    central_flux<true>(splitDG, B, L, R, HL, HR, F);
    const double h = 0.5 * lmax;
    const double dU[4] = {R.rho - L.rho, R.rho * R.v1 - L.rho * L.v1, R.rho * R.v2 - L.rho * L.v2, R.rho * R.v3 - L.rho * L.v3};
#pragma unroll
    for (int v = 0; v < 4; ++v) F[v] -= h * dU[v];
    F[4] -= h * (dU[0] * (0.5 * B.sKappaM1 / betaLog + 0.5 * (R.v1 * L.v1 + R.v2 * L.v2 + R.v3 * L.v3)) +
                 rhoMean * (0.5 * (L.v1 + R.v1) * (R.v1 - L.v1) + 0.5 * (L.v2 + R.v2) * (R.v2 - L.v2) + 0.5 * (L.v3 + R.v3) * (R.v3 - L.v3)) +
                 0.5 * rhoMean * B.sKappaM1 * (1.0 / bR - 1.0 / bL));
    return;
  }
  if (solver == RIEMANN_IR) {
    const double sR = log(R.p) - B.kappa * log(R.rho), sL = log(L.p) - B.kappa * log(L.rho);
    const double rpR = R.rho / R.p, rpL = L.rho / L.p;
    double vJ[5];
    vJ[0] = ((B.kappa - sR) - (B.kappa - sL)) * B.sKappaM1 - 0.5 * (rpR * (R.v1 * R.v1 + R.v2 * R.v2 + R.v3 * R.v3) -
                                                                    rpL * (L.v1 * L.v1 + L.v2 * L.v2 + L.v3 * L.v3));
    vJ[1] = rpR * R.v1 - rpL * L.v1;
    vJ[2] = rpR * R.v2 - rpL * L.v2;
    vJ[3] = rpR * R.v3 - rpL * L.v3;
    vJ[4] = rpL - rpR;
    const double zL1 = sqrt(rpL), zL5 = sqrt(L.rho * L.p), zR1 = sqrt(rpR), zR5 = sqrt(R.rho * R.p);
    const double z1Log = log_mean(zL1, zR1), z5Log = log_mean(zL5, zR5);
    const double z1s = zL1 + zR1;
    const double rhoHat = 0.5 * z1s * z5Log;
    const double uH = (zL1 * L.v1 + zR1 * R.v1) / z1s, vH = (zL1 * L.v2 + zR1 * R.v2) / z1s, wH = (zL1 * L.v3 + zR1 * R.v3) / z1s;
    const double pHat = (zL5 + zR5) / z1s;
    const double p2Hat = 0.5 / B.kappa * ((B.kappa + 1.0) * z5Log / z1Log + B.kappaM1 * pHat);
    const double aH = sqrt(B.kappa * p2Hat / rhoHat);
    const double ek = 0.5 * (uH * uH + vH * vH + wH * wH);
    const double hH = B.kappa * p2Hat / (rhoHat * B.kappaM1) + ek;
    // R = [r1 .. r5] (columns): r1 = (1, u-a, v, w, h-ua), r2 = (1, u, v, w, ek), r3 = e3 + v e5, r4 = e4 + w e5,
    // r5 = (1, u+a, v, w, h+ua); dissipation R diag(D) R^T vJump
    const double c0 = vJ[0] + (uH - aH) * vJ[1] + vH * vJ[2] + wH * vJ[3] + (hH - uH * aH) * vJ[4];
    const double c1 = vJ[0] + uH * vJ[1] + vH * vJ[2] + wH * vJ[3] + ek * vJ[4];
    const double c2 = vJ[2] + vH * vJ[4];
    const double c3 = vJ[3] + wH * vJ[4];
    const double c4 = vJ[0] + (uH + aH) * vJ[1] + vH * vJ[2] + wH * vJ[3] + (hH + uH * aH) * vJ[4];
    const double d0 = 0.5 * fabs(uH - aH) * rhoHat / B.kappa * c0;
    const double d1 = fabs(uH) * (B.kappaM1 / B.kappa) * rhoHat * c1;
    const double d2 = fabs(uH) * pHat * c2;
    const double d3 = fabs(uH) * pHat * c3;
    const double d4 = 0.5 * fabs(uH + aH) * rhoHat / B.kappa * c4;
    const double sum014 = d0 + d1 + d4;
    double Dd[5];
    Dd[0] = sum014;
    Dd[1] = (uH - aH) * d0 + uH * d1 + (uH + aH) * d4;
    Dd[2] = vH * sum014 + d2;
    Dd[3] = wH * sum014 + d3;
    Dd[4] = (hH - uH * aH) * d0 + ek * d1 + vH * d2 + wH * d3 + (hH + uH * aH) * d4;
    central_flux<true>(splitDG, B, L, R, HL, HR, F);
#pragma unroll
    for (int v = 0; v < 5; ++v) F[v] -= 0.5 * Dd[v];
    return;
  }
  double FL[5], FR[5];
  euler_flux_1d(L, FL);
  euler_flux_1d(R, FR);
  const double sqL = sqrt(L.rho), sqR = sqrt(R.rho);
  const double ssq = 1.0 / (sqL + sqR);
  const double r1v = (sqR * R.v1 + sqL * L.v1) * ssq;
  const double r2v = (sqR * R.v2 + sqL * L.v2) * ssq;
  const double r3v = (sqR * R.v3 + sqL * L.v3) * ssq;
  const double rH = (sqR * HR + sqL * HL) * ssq;
  const double absVel = r1v * r1v + r2v * r2v + r3v * r3v;
  const double rc = sqrt(B.kappaM1 * (rH - 0.5 * absVel));
  const double dU[5] = {R.rho - L.rho, R.rho * R.v1 - L.rho * L.v1, R.rho * R.v2 - L.rho * L.v2, R.rho * R.v3 - L.rho * L.v3, R.E - L.E};
  if (solver == RIEMANN_HLL || solver == RIEMANN_HLLE || solver == RIEMANN_HLLEM) {
    double Ssl = r1v - rc, Ssr = r1v + rc;
    if (solver != RIEMANN_HLL) {
      const double beta = sqrt(0.5 * B.kappaM1 / B.kappa);
      Ssl = fmin(fmin(Ssl, L.v1 - beta * cL), 0.0);
      Ssr = fmax(fmax(Ssr, R.v1 + beta * cR), 0.0);
    }
    if (Ssl >= 0.0) {
#pragma unroll
      for (int v = 0; v < 5; ++v) F[v] = FL[v];
    } else if (Ssr <= 0.0) {
#pragma unroll
      for (int v = 0; v < 5; ++v) F[v] = FR[v];
    } else {
      double J[5] = {dU[0], dU[1], dU[2], dU[3], dU[4]};
      if (solver == RIEMANN_HLLEM) {
        const double RoeDens = sqL * sqR;
        const double delta = rc / (rc + fabs(0.5 * (Ssl + Ssr)));
        const double A2 = (R.rho - L.rho) - (R.p - L.p) / (rc * rc);
        const double A3 = RoeDens * (R.v2 - L.v2), A4 = RoeDens * (R.v3 - L.v3);
        J[0] -= delta * A2;
        J[1] -= delta * r1v * A2;
        J[2] -= delta * (r2v * A2 + A3);
        J[3] -= delta * (r3v * A2 + A4);
        J[4] -= delta * (0.5 * absVel * A2 + r2v * A3 + r3v * A4);
      }
      const double sd = 1.0 / (Ssr - Ssl), ss = Ssl * Ssr;
#pragma unroll
      for (int v = 0; v < 5; ++v) F[v] = (Ssr * FL[v] - Ssl * FR[v] + ss * J[v]) * sd;
    }
    return;
  }
  // RoeL2 / RoeEntropyGShockFix: Roe-type dissipation sum_k Alpha_k |a_k| r_k
  double a0 = r1v - rc, a1 = r1v, a4 = r1v + rc;
  double A0, A1, A2, A3, A4, e0, e1, e4;
  if (solver == RIEMANN_ROEL2) {
    const double d5 = dU[4] - (dU[2] - r2v * dU[0]) * r2v - (dU[3] - r3v * dU[0]) * r3v;
    const double Ma = sqrt(absVel) / (rc * sqrt(B.kappa));
    const double d1 = dU[1] * Ma, d2 = dU[2] * Ma, d3 = dU[3] * Ma;
    A2 = d2 - r2v * dU[0];
    A3 = d3 - r3v * dU[0];
    A1 = B.kappaM1 / (rc * rc) * (dU[0] * (rH - r1v * r1v) - d5 + r1v * d1);
    A0 = 0.5 / rc * (dU[0] * (r1v + rc) - d1 - rc * A1);
    A4 = dU[0] - A0 - A1;
    e0 = fabs(a0); e1 = fabs(a1); e4 = fabs(a4);
  } else {  // RoeEntropyGShockFix
    const double am = (r1v < 0.0 ? -1.0 : 1.0) * fmax(rc / B.riemannPhi, fabs(r1v));
    a0 = am - rc; a1 = am; a4 = am + rc;
    const double RoeDens = sqL * sqR;
    const double dr = R.rho - L.rho, du = R.v1 - L.v1, dv = R.v2 - L.v2, dw = R.v3 - L.v3, dp = R.p - L.p;
    const double tmp = 0.5 / (rc * rc);
    A0 = tmp * (dp - RoeDens * rc * du);
    A1 = dr - dp * (2.0 * tmp);
    A2 = RoeDens * dv;
    A3 = RoeDens * dw;
    A4 = tmp * (dp + RoeDens * rc * du);
    auto fix = [](double a, double al, double ar) {
      const double da = fmax(0.0, fmax(a - al, ar - a));
      return fabs(a) < da ? 0.5 * (a * a / da + da) : fabs(a);
    };
    e0 = fix(a0, L.v1 - cL, R.v1 - cR);
    e1 = fix(a1, L.v1, R.v1);
    e4 = fix(a4, L.v1 + cL, R.v1 + cR);
  }
  const double w0 = A0 * e0, w1 = A1 * e1, w2 = A2 * e1, w3 = A3 * e1, w4 = A4 * e4;
  double D[5];
  D[0] = w0 + w1 + w4;
  D[1] = w0 * a0 + w1 * r1v + w4 * a4;
  D[2] = (w0 + w1 + w4) * r2v + w2;
  D[3] = (w0 + w1 + w4) * r3v + w3;
  D[4] = w0 * (rH - r1v * rc) + w1 * (0.5 * absVel) + w2 * r2v + w3 * r3v + w4 * (rH + r1v * rc);
  if (!split) {
#pragma unroll
    for (int v = 0; v < 5; ++v) F[v] = 0.5 * ((FL[v] + FR[v]) - D[v]);
  } else {
    central_flux<true>(splitDG, B, L, R, HL, HR, F);
#pragma unroll
    for (int v = 0; v < 5; ++v) F[v] = F[v] - 0.5 * D[v];
  }
}

// eos.f90:PRESSURE_RIEMANN on the rotated boundary state (v1 = normal velocity)
__host__ __device__ __forceinline__ double pressure_riemann(const Basis& B, double rho, double vn, double p) {
  if (vn <= 0.0) {
    const double base = fmax(0.0001, 1.0 + 0.5 * B.kappaM1 * vn / sqrt(B.kappa * p / rho));
    return p * pow(base, B.kappaFac);
  }
  const double ar = 2.0 * B.sKappaP1 / rho;
  const double br = B.kappaM1 * B.sKappaP1 * p;
  return p + vn / ar * 0.5 * (vn + sqrt(vn * vn + 4.0 * ar * (p + br)));
}

// Two-point volume fluxes of the split form in contravariant form (split kernels; the point harness checks them on
// the CPU): SplitVolumeFluxPI / SD and, for the other kinds, their per-node inputs, constant factors and pair flux.
__host__ __device__ __forceinline__ void split_pair_flux(bool pi, double ra, double ua, double va, double wa, double pa, double ha, double rb,
                                                double ub, double vb, double wb, double pb, double hb, double ms0, double ms1,
                                                double ms2, double* G) {
  if (pi) {
    const double rs = ra + rb, us = ua + ub, vs = va + vb, ws = wa + wb, ps4 = pa + pb, hs = ha + hb;
    const double qs = us * ms0 + vs * ms1 + ws * ms2;
    const double A = rs * qs;
    G[0] = A;
    G[1] = fma(A, us, ps4 * ms0);
    G[2] = fma(A, vs, ps4 * ms1);
    G[3] = fma(A, ws, ps4 * ms2);
    G[4] = A * hs;
  } else {
    const double qa = ua * ms0 + va * ms1 + wa * ms2, qb = ub * ms0 + vb * ms1 + wb * ms2;
    const double mqa = ra * qa, mqb = rb * qb;
    G[0] = mqa + mqb;
    G[1] = fma(mqa, ua, mqb * ub) + (pa + pb) * ms0;
    G[2] = fma(mqa, va, mqb * vb) + (pa + pb) * ms1;
    G[3] = fma(mqa, wa, mqb * wb) + (pa + pb) * ms2;
    G[4] = fma(ha, qa, hb * qb);
  }
}

// The other two-point volume fluxes of splitflux.f90 (MO :445, DU :225, KG :327, CH :703, IR :822) in the same
// contravariant form, on the per-node inputs of split_node_inputs (q0, u, v, w, q4, q5); the constant factors of
// split_factors are applied by the kernels' pre-scaled coefficients. IR carries no factor 2, as in the reference.
__host__ __device__ __forceinline__ void split_node_inputs(int sd, double rho, double u, double v, double w, double p, double E, double srho, double& q0,
                                                  double& q4, double& q5) {
  q0 = rho;
  switch (sd) {
    case SPLIT_PI: q4 = 4.0 * p; q5 = (E + p) * srho; break;
    case SPLIT_DU: q4 = 2.0 * p; q5 = E + p; break;
    case SPLIT_KG: q4 = 4.0 * p; q5 = E * srho; break;
    case SPLIT_MO: q4 = 2.0 * p; q5 = 2.0 * (E - 0.5 * rho * (u * u + v * v + w * w) + p); break;
    case SPLIT_CH: q4 = 0.5 * rho / p; q5 = 0.; break;
    case SPLIT_IR: q0 = sqrt(rho / p); q4 = sqrt(rho * p); q5 = 0.; break;
    default: q4 = p; q5 = E + p; break;  // SD
  }
}
__host__ __device__ __forceinline__ void split_factors(int sd, double& f0, double& f1) {
  switch (sd) {
    case SPLIT_PI: f0 = 0.25; f1 = 0.125; break;
    case SPLIT_DU: f0 = 0.25; f1 = 0.25; break;
    case SPLIT_KG: f0 = 0.25; f1 = 0.125; break;
    case SPLIT_MO: f0 = 0.5; f1 = 0.25; break;
    default: f0 = 0.5; f1 = 0.5; break;  // SD, CH, IR
  }
}
__host__ __device__ __forceinline__ void split_pair_flux_gen(int sd, const Basis& B, double ra, double ua, double va, double wa, double pa, double ha,
                                                    double rb, double ub, double vb, double wb, double pb, double hb, double ms0, double ms1,
                                                    double ms2, double* G) {
  if (sd == SPLIT_PI || sd == SPLIT_SD) {
    split_pair_flux(sd == SPLIT_PI, ra, ua, va, wa, pa, ha, rb, ub, vb, wb, pb, hb, ms0, ms1, ms2, G);
    return;
  }
  const double us = ua + ub, vs = va + vb, ws = wa + wb;
  const double qs = us * ms0 + vs * ms1 + ws * ms2;
  if (sd == SPLIT_DU) {
    const double ps = pa + pb;
    G[0] = (ra + rb) * qs;
    G[1] = fma(ra * ua + rb * ub, qs, ps * ms0);
    G[2] = fma(ra * va + rb * vb, qs, ps * ms1);
    G[3] = fma(ra * wa + rb * wb, qs, ps * ms2);
    G[4] = (ha + hb) * qs;
  } else if (sd == SPLIT_KG) {
    const double A = (ra + rb) * qs, ps = pa + pb;
    G[0] = A;
    G[1] = fma(A, us, ps * ms0);
    G[2] = fma(A, vs, ps * ms1);
    G[3] = fma(A, ws, ps * ms2);
    G[4] = fma(A, ha + hb, 0.5 * ps * qs);
  } else if (sd == SPLIT_MO) {
    const double qa = ua * ms0 + va * ms1 + wa * ms2, qb = ub * ms0 + vb * ms1 + wb * ms2;
    const double mq = ra * qa + rb * qb, ps = pa + pb;
    G[0] = mq;
    G[1] = fma(mq, us, ps * ms0);
    G[2] = fma(mq, vs, ps * ms1);
    G[3] = fma(mq, ws, ps * ms2);
    G[4] = fma(ha, qa, fma(hb, qb, mq * (ua * ub + va * vb + wa * wb)));
  } else if (sd == SPLIT_CH) {
    const double rhoLog = log_mean(ra, rb), betaLog = log_mean(pa, pb);
    const double pHat = 0.5 * (ra + rb) / (pa + pb);
    const double H = 0.5 * B.sKappaM1 / betaLog + pHat / rhoLog + 0.5 * (ua * ub + va * vb + wa * wb);
    const double A = rhoLog * qs, hA = 0.5 * A, p2 = 2.0 * pHat;
    G[0] = A;
    G[1] = fma(hA, us, p2 * ms0);
    G[2] = fma(hA, vs, p2 * ms1);
    G[3] = fma(hA, ws, p2 * ms2);
    G[4] = A * H;
  } else {  // IR: q0 = sqrt(rho/p), q4 = sqrt(rho p)
    const double z1Log = log_mean(ra, rb), z5Log = log_mean(pa, pb);
    const double z1s = ra + rb;
    const double rhoHat = 0.5 * z1s * z5Log;
    const double pHat = (pa + pb) / z1s;
    const double p2Hat = 0.5 / B.kappa * ((B.kappa + 1.0) * z5Log / z1Log + B.kappaM1 * pHat);
    const double uH = (ra * ua + rb * ub) / z1s, vH = (ra * va + rb * vb) / z1s, wH = (ra * wa + rb * wb) / z1s;
    const double hH = B.kappa * p2Hat / (rhoHat * B.kappaM1) + 0.5 * (uH * uH + vH * vH + wH * wH);
    const double A = rhoHat * (uH * ms0 + vH * ms1 + wH * ms2);
    G[0] = A;
    G[1] = fma(A, uH, pHat * ms0);
    G[2] = fma(A, vH, pHat * ms1);
    G[3] = fma(A, wH, pHat * ms2);
    G[4] = A * hH;
  }
}
__device__ __forceinline__ void set_error(int* err, int code) { atomicCAS(err, 0, code); }

}  // namespace fg
