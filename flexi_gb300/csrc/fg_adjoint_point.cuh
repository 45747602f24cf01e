// flexi_gb300 -- reverse-mode (vector-Jacobian) counterparts of the point-wise physics of fg_common.cuh.
//
// Each *_adj function takes the inputs of its forward function and the cotangent of its outputs and
// ADDS the cotangent of every input to the caller's accumulators (x_bar += J^T y_bar). They retrace the
// forward function's own operations, so that they are the exact transposed Jacobians of the code that
// runs forward, including its branch choices (entropy fix, max/abs, pressure clamp). At a tie of a max
// the forward's choice (the first argument of fmax when both are equal) gets the derivative.
#pragma once
#include "fg_common.cuh"

namespace fg {

#define FG_HD __host__ __device__ __forceinline__

FG_HD double sgn1(double x) { return x >= 0.0 ? 1.0 : -1.0; }

// log_mean transposed (splitflux.f90:GetLogMean, the branch the forward took): given the bar Lb of the mean of a and b,
// adds the bars of a and b
FG_HD void log_mean_adj(double a, double b, double Lb, double& ab, double& bb) {
  const double chi = a / b;
  const double f = (chi - 1.0) / (chi + 1.0);
  double g, gu = 0.0;  // g and, on the series branch, dg/du
  const bool series = fabs(f) < 0.1;
  const double u = f * f;
  if (series) {
    g = 2.0 + u * ((2.0 / 3.0) + u * (0.4 + u * (2.0 / 7.0)));
    gu = (2.0 / 3.0) + u * (0.8 + u * (6.0 / 7.0));
  } else {
    g = log(chi) / f;
  }
  const double sb = Lb / g;                // bar of a + b
  const double gb = -Lb * (a + b) / (g * g);
  double fb = 0.0, chib = 0.0;
  if (series) {
    fb = gb * gu * 2.0 * f;
  } else {
    chib = gb / (chi * f);
    fb = -gb * log(chi) / (f * f);
  }
  chib += fb * 2.0 / ((chi + 1.0) * (chi + 1.0));
  ab += sb + chib / b;
  bb += sb - chib * a / (b * b);
}

// eos.f90:ConsToPrim: (rho, m, E) -> (1/rho, v, p, T). Given the bars of 1/rho, v (3), p, T and direct bars
// of rho and E (face states store both), accumulates the conservative bars into Ub[5].
FG_HD void cons_to_prim_adj(const Basis& B, const double* U, double sb, double ub, double vb, double wb, double pb, double Tb,
                            double rhob, double Eb, double* Ub) {
  const double srho = 1.0 / U[0];
  const double vx = U[1] * srho, vy = U[2] * srho, vz = U[3] * srho;
  const double p = B.kappaM1 * (U[4] - 0.5 * (U[1] * vx + U[2] * vy + U[3] * vz));
  // T = p * srho * sR
  pb += Tb * srho * B.sR;
  sb += Tb * p * B.sR;
  // p = kappaM1 * (E - 1/2 (m . v))
  const double kp = B.kappaM1 * pb;
  Eb += kp;
  double mb1 = -0.5 * kp * vx, mb2 = -0.5 * kp * vy, mb3 = -0.5 * kp * vz;
  ub -= 0.5 * kp * U[1];
  vb -= 0.5 * kp * U[2];
  wb -= 0.5 * kp * U[3];
  // v = m * srho
  mb1 += ub * srho; mb2 += vb * srho; mb3 += wb * srho;
  sb += ub * U[1] + vb * U[2] + wb * U[3];
  // srho = 1 / rho
  rhob -= sb * srho * srho;
  Ub[0] += rhob; Ub[1] += mb1; Ub[2] += mb2; Ub[3] += mb3; Ub[4] += Eb;
}

// visc_flux_dir: F[1..4] of the viscous flux contracted with (m1, m2, m3). Fb[1..4] given; adds to the
// velocity bars (ub, vb, wb), the gradient bars gb[12] and the viscosity bar mub (lam = mu * lamFac).
FG_HD void visc_flux_dir_adj(double mu, double lamFac, double u, double v, double w, const double* g, double m1, double m2, double m3,
                             const double* Fb, double& ub, double& vb, double& wb, double* gb, double& mub) {
  const double lam = mu * lamFac;
  const double div = g[0] + g[5] + g[10];
  const double mdiv = (2.0 / 3.0) * div;
  const double sxx = 2.0 * g[0] - mdiv, syy = 2.0 * g[5] - mdiv, szz = 2.0 * g[10] - mdiv;
  const double sxy = g[4] + g[1], sxz = g[8] + g[2], syz = g[9] + g[6];
  const double txx = mu * sxx, tyy = mu * syy, tzz = mu * szz, txy = mu * sxy, txz = mu * sxz, tyz = mu * syz;
  const double a1 = txx * m1 + txy * m2 + txz * m3;
  const double a2 = txy * m1 + tyy * m2 + tyz * m3;
  const double a3 = txz * m1 + tyz * m2 + tzz * m3;
  const double qn = g[3] * m1 + g[7] * m2 + g[11] * m3;
  // F1 = -a1, F2 = -a2, F3 = -a3, F4 = -(a1 u + a2 v + a3 w) - lam qn
  const double a1b = -Fb[1] - Fb[4] * u, a2b = -Fb[2] - Fb[4] * v, a3b = -Fb[3] - Fb[4] * w;
  ub -= Fb[4] * a1; vb -= Fb[4] * a2; wb -= Fb[4] * a3;
  const double lamb = -Fb[4] * qn, qnb = -Fb[4] * lam;
  gb[3] += qnb * m1; gb[7] += qnb * m2; gb[11] += qnb * m3;
  const double txxb = a1b * m1, tyyb = a2b * m2, tzzb = a3b * m3;
  const double txyb = a1b * m2 + a2b * m1, txzb = a1b * m3 + a3b * m1, tyzb = a2b * m3 + a3b * m2;
  mub += txxb * sxx + tyyb * syy + tzzb * szz + txyb * sxy + txzb * sxz + tyzb * syz + lamb * lamFac;
  const double sxxb = mu * txxb, syyb = mu * tyyb, szzb = mu * tzzb;
  const double divb = -(2.0 / 3.0) * (sxxb + syyb + szzb);
  gb[0] += 2.0 * sxxb + divb; gb[5] += 2.0 * syyb + divb; gb[10] += 2.0 * szzb + divb;
  gb[4] += mu * txyb; gb[1] += mu * txyb;
  gb[8] += mu * txzb; gb[2] += mu * txzb;
  gb[9] += mu * tyzb; gb[6] += mu * tyzb;
}

// Physical viscous fluxes f, g, h (flux.f90:EvalDiffFlux3D_Point, components 1..4 of each, with the minus
// sign) at one node: given their bars fb, gb_, hb (index 1..4 used), adds the velocity bars, the gradient
// bars and the viscosity bar (lam = mu * lamFac).
FG_HD void visc_flux_phys_adj(double mu, double lamFac, double u, double v, double w, const double* g, const double* fb, const double* gyb,
                              const double* hb, double& ub, double& vb, double& wb, double* gb, double& mub) {
  const double lam = mu * lamFac;
  const double div = g[0] + g[5] + g[10];
  const double mdiv = (2.0 / 3.0) * div;
  const double sxx = 2.0 * g[0] - mdiv, syy = 2.0 * g[5] - mdiv, szz = 2.0 * g[10] - mdiv;
  const double sxy = g[4] + g[1], sxz = g[8] + g[2], syz = g[9] + g[6];
  const double txx = mu * sxx, tyy = mu * syy, tzz = mu * szz, txy = mu * sxy, txz = mu * sxz, tyz = mu * syz;
  // f = (-txx, -txy, -txz, -(txx u + txy v + txz w) - lam Tx), g = (-txy, -tyy, -tyz, ...), h = (-txz, -tyz, -tzz, ...)
  const double txxb = -fb[1] - fb[4] * u;
  const double tyyb = -gyb[2] - gyb[4] * v;
  const double tzzb = -hb[3] - hb[4] * w;
  const double txyb = -fb[2] - gyb[1] - fb[4] * v - gyb[4] * u;
  const double txzb = -fb[3] - hb[1] - fb[4] * w - hb[4] * u;
  const double tyzb = -gyb[3] - hb[2] - gyb[4] * w - hb[4] * v;
  ub -= fb[4] * txx + gyb[4] * txy + hb[4] * txz;
  vb -= fb[4] * txy + gyb[4] * tyy + hb[4] * tyz;
  wb -= fb[4] * txz + gyb[4] * tyz + hb[4] * tzz;
  const double lamb = -(fb[4] * g[3] + gyb[4] * g[7] + hb[4] * g[11]);
  gb[3] -= fb[4] * lam; gb[7] -= gyb[4] * lam; gb[11] -= hb[4] * lam;
  mub += txxb * sxx + tyyb * syy + tzzb * szz + txyb * sxy + txzb * sxz + tyzb * syz + lamb * lamFac;
  const double sxxb = mu * txxb, syyb = mu * tyyb, szzb = mu * tzzb;
  const double divb = -(2.0 / 3.0) * (sxxb + syyb + szzb);
  gb[0] += 2.0 * sxxb + divb; gb[5] += 2.0 * syyb + divb; gb[10] += 2.0 * szzb + divb;
  gb[4] += mu * txyb; gb[1] += mu * txyb;
  gb[8] += mu * txzb; gb[2] += mu * txzb;
  gb[9] += mu * tyzb; gb[6] += mu * tyzb;
}

FG_HD void rot_zero(RotState& S) { S.rho = S.srho = S.E = S.p = S.v1 = S.v2 = S.v3 = 0.0; }

FG_HD void euler_flux_1d_adj(const RotState& S, const double* Fb, RotState& Sb) {
  const double m = S.rho * S.v1;
  const double mb = Fb[0] + Fb[1] * S.v1 + Fb[2] * S.v2 + Fb[3] * S.v3;
  Sb.v1 += Fb[1] * m + Fb[4] * (S.E + S.p) + mb * S.rho;
  Sb.p += Fb[1] + Fb[4] * S.v1;
  Sb.v2 += Fb[2] * m;
  Sb.v3 += Fb[3] * m;
  Sb.E += Fb[4] * S.v1;
  Sb.rho += mb * S.v1;
}

// H = (E + p) * srho
FG_HD void enthalpy_adj(const RotState& S, double Hb, RotState& Sb) {
  Sb.E += Hb * S.srho;
  Sb.p += Hb * S.srho;
  Sb.srho += Hb * (S.E + S.p);
}

FG_HD void split_surface_flux_adj(int splitDG, const RotState& L, const RotState& R, double HL, double HR, const double* Fb, RotState& Lb,
                                  RotState& Rb, double& HLb, double& HRb) {
  if (splitDG == 4) {
    const double rs = L.rho + R.rho, us = L.v1 + R.v1;
    const double a = rs * us;
    const double b = 0.125 * a;
    const double v2s = L.v2 + R.v2, v3s = L.v3 + R.v3, Hs = HL + HR;
    const double bb = Fb[1] * us + Fb[2] * v2s + Fb[3] * v3s + Fb[4] * Hs;
    const double ab = 0.25 * Fb[0] + 0.125 * bb;
    const double usb = Fb[1] * b + ab * rs;
    const double rsb = ab * us;
    Lb.rho += rsb; Rb.rho += rsb;
    Lb.v1 += usb; Rb.v1 += usb;
    Lb.p += 0.5 * Fb[1]; Rb.p += 0.5 * Fb[1];
    Lb.v2 += Fb[2] * b; Rb.v2 += Fb[2] * b;
    Lb.v3 += Fb[3] * b; Rb.v3 += Fb[3] * b;
    HLb += Fb[4] * b; HRb += Fb[4] * b;
  } else {  // SD
    const double mL = L.rho * L.v1, mR = R.rho * R.v1;
    // F0 = (mL+mR)/2; F1 = (mL vL + pL + mR vR + pR)/2; F2 = (mL v2L + mR v2R)/2; F3 ...; F4 = ((EL+pL) v1L + (ER+pR) v1R)/2
    const double mLb = 0.5 * (Fb[0] + Fb[1] * L.v1 + Fb[2] * L.v2 + Fb[3] * L.v3);
    const double mRb = 0.5 * (Fb[0] + Fb[1] * R.v1 + Fb[2] * R.v2 + Fb[3] * R.v3);
    Lb.v1 += 0.5 * Fb[1] * mL + 0.5 * Fb[4] * (L.E + L.p) + mLb * L.rho;
    Rb.v1 += 0.5 * Fb[1] * mR + 0.5 * Fb[4] * (R.E + R.p) + mRb * R.rho;
    Lb.p += 0.5 * Fb[1] + 0.5 * Fb[4] * L.v1;
    Rb.p += 0.5 * Fb[1] + 0.5 * Fb[4] * R.v1;
    Lb.v2 += 0.5 * Fb[2] * mL; Rb.v2 += 0.5 * Fb[2] * mR;
    Lb.v3 += 0.5 * Fb[3] * mL; Rb.v3 += 0.5 * Fb[3] * mR;
    Lb.E += 0.5 * Fb[4] * L.v1; Rb.E += 0.5 * Fb[4] * R.v1;
    Lb.rho += mLb * L.v1; Rb.rho += mRb * R.v1;
  }
}

// Harten-Hyman entropy fix of RoeEntropyFix: e = fix(a, al, ar); adds the bars of a, al, ar.
FG_HD void entropy_fix_adj(double a, double al, double ar, double eb, double& abar, double& alb, double& arb) {
  const double x = a - al, y = ar - a;
  const double da = fmax(0.0, fmax(x, y));
  const double aa = fabs(a);
  double dab = 0.0;
  if (aa < da) {
    abar += eb * (a / da);
    dab = eb * 0.5 * (1.0 - (a * a) / (da * da));
  } else {
    abar += eb * sgn1(a);
  }
  if (dab != 0.0 && da > 0.0) {
    if (x >= y) { abar += dab; alb -= dab; }
    else { arb += dab; abar -= dab; }
  }
}

// Transposed Jacobian of the HLLC flux of riemann_rotated (riemann.f90:594-663, Roe-Einfeldt wave speeds;
// its split and non-split forms are the same): Fb[5] given, adds to the bars of both rotated states,
// retracing the forward's branch (supersonic left / right, left or right star state).
FG_HD void hllc_adj(const Basis& B, const RotState& L, const RotState& R, const double* Fb, RotState& Lb, RotState& Rb) {
  const double HL = (L.E + L.p) * L.srho, HR = (R.E + R.p) * R.srho;
  const double sqL = sqrt(L.rho), sqR = sqrt(R.rho);
  const double ssq = 1.0 / (sqL + sqR);
  const double r1v = (sqR * R.v1 + sqL * L.v1) * ssq;
  const double r2v = (sqR * R.v2 + sqL * L.v2) * ssq;
  const double r3v = (sqR * R.v3 + sqL * L.v3) * ssq;
  const double rH = (sqR * HR + sqL * HL) * ssq;
  const double absVel = r1v * r1v + r2v * r2v + r3v * r3v;
  const double rc = sqrt(B.kappaM1 * (rH - 0.5 * absVel));
  const double Ssl = r1v - rc, Ssr = r1v + rc;
  if (Ssl >= 0.0) { euler_flux_1d_adj(L, Fb, Lb); return; }
  if (Ssr <= 0.0) { euler_flux_1d_adj(R, Fb, Rb); return; }
  const double sMuL = Ssl - L.v1, sMuR = Ssr - R.v1;
  const double mL = L.rho * L.v1, mR = R.rho * R.v1;
  const double num = R.p - L.p + mL * sMuL - mR * sMuR, den = L.rho * sMuL - R.rho * sMuR;
  const double SStar = num / den;
  double Sslb = 0, Ssrb = 0, SStarb = 0, sMuLb = 0, sMuRb = 0, mLb = 0, mRb = 0;
  // star state of side X (left: sign s = Ssl, right: Ssr): F = F_X + S (Us - Uc)
  auto star = [&](const RotState& X, RotState& Xb, double S, double sMu, double m, double& Sb, double& sMub, double& mb) {
    euler_flux_1d_adj(X, Fb, Xb);
    const double Z = X.p * X.srho / sMu;
    const double EStar = X.E * X.srho + (SStar - X.v1) * (SStar + Z);
    const double d = S - SStar;
    const double fac = X.rho * sMu / d;
    const double Us[5] = {fac, fac * SStar, fac * X.v2, fac * X.v3, fac * EStar};
    const double Uc[5] = {X.rho, m, X.rho * X.v2, X.rho * X.v3, X.E};
    for (int v = 0; v < 5; ++v) Sb += Fb[v] * (Us[v] - Uc[v]);
    // Uc
    Xb.rho -= S * (Fb[0] + Fb[2] * X.v2 + Fb[3] * X.v3);
    mb -= S * Fb[1];
    Xb.v2 -= S * Fb[2] * X.rho;
    Xb.v3 -= S * Fb[3] * X.rho;
    Xb.E -= S * Fb[4];
    // Us
    const double facb = S * (Fb[0] + Fb[1] * SStar + Fb[2] * X.v2 + Fb[3] * X.v3 + Fb[4] * EStar);
    SStarb += S * Fb[1] * fac;
    Xb.v2 += S * Fb[2] * fac;
    Xb.v3 += S * Fb[3] * fac;
    const double EStarb = S * Fb[4] * fac;
    // fac = X.rho sMu / d
    const double qb = facb / d, db = -facb * fac / d;
    Xb.rho += qb * sMu; sMub += qb * X.rho;
    Sb += db; SStarb -= db;
    // EStar = X.E X.srho + (SStar - X.v1) (SStar + Z), Z = X.p X.srho / sMu
    Xb.E += EStarb * X.srho; Xb.srho += EStarb * X.E;
    const double Xdb = EStarb * (SStar + Z), Ydb = EStarb * (SStar - X.v1);
    SStarb += Xdb + Ydb; Xb.v1 -= Xdb;
    Xb.p += Ydb * X.srho / sMu; Xb.srho += Ydb * X.p / sMu; sMub -= Ydb * Z / sMu;
  };
  if (Ssl <= 0.0 && SStar >= 0.0) star(L, Lb, Ssl, sMuL, mL, Sslb, sMuLb, mLb);
  else star(R, Rb, Ssr, sMuR, mR, Ssrb, sMuRb, mRb);
  // SStar = num / den
  const double numb = SStarb / den, denb = -SStarb * SStar / den;
  Rb.p += numb; Lb.p -= numb;
  mLb += numb * sMuL; sMuLb += numb * mL; mRb -= numb * sMuR; sMuRb -= numb * mR;
  Lb.rho += denb * sMuL; sMuLb += denb * L.rho; Rb.rho -= denb * sMuR; sMuRb -= denb * R.rho;
  Lb.rho += mLb * L.v1; Lb.v1 += mLb * L.rho; Rb.rho += mRb * R.v1; Rb.v1 += mRb * R.rho;
  Sslb += sMuLb; Lb.v1 -= sMuLb; Ssrb += sMuRb; Rb.v1 -= sMuRb;
  // wave speeds from the Roe averages
  double r1vb = Sslb + Ssrb, rcb = Ssrb - Sslb, r2vb = 0, r3vb = 0, rHb = 0, absb = 0, HLb = 0, HRb = 0;
  const double Zb = rcb / (2.0 * rc);
  rHb += B.kappaM1 * Zb;
  absb -= 0.5 * B.kappaM1 * Zb;
  r1vb += 2.0 * r1v * absb; r2vb += 2.0 * r2v * absb; r3vb += 2.0 * r3v * absb;
  const double ssqb = rHb * (sqR * HR + sqL * HL) + r1vb * (sqR * R.v1 + sqL * L.v1) + r2vb * (sqR * R.v2 + sqL * L.v2) +
                      r3vb * (sqR * R.v3 + sqL * L.v3);
  double sqRb = (rHb * HR + r1vb * R.v1 + r2vb * R.v2 + r3vb * R.v3) * ssq;
  double sqLb = (rHb * HL + r1vb * L.v1 + r2vb * L.v2 + r3vb * L.v3) * ssq;
  HRb += rHb * sqR * ssq; HLb += rHb * sqL * ssq;
  Rb.v1 += r1vb * sqR * ssq; Lb.v1 += r1vb * sqL * ssq;
  Rb.v2 += r2vb * sqR * ssq; Lb.v2 += r2vb * sqL * ssq;
  Rb.v3 += r3vb * sqR * ssq; Lb.v3 += r3vb * sqL * ssq;
  sqLb -= ssqb * ssq * ssq; sqRb -= ssqb * ssq * ssq;
  Lb.rho += sqLb / (2.0 * sqL); Rb.rho += sqRb / (2.0 * sqR);
  enthalpy_adj(L, HLb, Lb);
  enthalpy_adj(R, HRb, Rb);
}

// Transposed Jacobian of riemann_rotated (LF, HLLC, Roe, RoeEntropyFix; split or not): Fb[5] given, adds to the
// bars of both rotated states (all seven fields of each are independent inputs).
FG_HD void riemann_rotated_adj(int solver, int splitDG, const Basis& B, const RotState& L, const RotState& R, const double* Fb, RotState& Lb,
                               RotState& Rb) {
  if (solver == RIEMANN_HLLC) { hllc_adj(B, L, R, Fb, Lb, Rb); return; }
  const bool split = splitDG >= 0;
  const double HL = (L.E + L.p) * L.srho, HR = (R.E + R.p) * R.srho;
  double HLb = 0.0, HRb = 0.0;
  double Db[5];  // bar of the dissipation term (F = central - 1/2 D, or -1/2 lmax dU)
  if (!split) {
    double Fh[5];
    for (int v = 0; v < 5; ++v) Fh[v] = 0.5 * Fb[v];
    euler_flux_1d_adj(L, Fh, Lb);
    euler_flux_1d_adj(R, Fh, Rb);
  } else {
    split_surface_flux_adj(splitDG, L, R, HL, HR, Fb, Lb, Rb, HLb, HRb);
  }
  for (int v = 0; v < 5; ++v) Db[v] = -0.5 * Fb[v];
  if (solver == RIEMANN_LF) {
    const double cL = sqrt(B.kappa * L.p * L.srho), cR = sqrt(B.kappa * R.p * R.srho);
    const double aL = fabs(L.v1), aR = fabs(R.v1);
    const double lmax = fmax(aR, aL) + fmax(cL, cR);
    const double dU[5] = {R.rho - L.rho, R.rho * R.v1 - L.rho * L.v1, R.rho * R.v2 - L.rho * L.v2, R.rho * R.v3 - L.rho * L.v3, R.E - L.E};
    double lb = 0.0;
    for (int v = 0; v < 5; ++v) lb += Db[v] * dU[v];
    double dUb[5];
    for (int v = 0; v < 5; ++v) dUb[v] = Db[v] * lmax;
    if (aR >= aL) Rb.v1 += lb * sgn1(R.v1); else Lb.v1 += lb * sgn1(L.v1);
    if (cL >= cR) {
      Lb.p += lb * B.kappa * L.srho / (2.0 * cL);
      Lb.srho += lb * B.kappa * L.p / (2.0 * cL);
    } else {
      Rb.p += lb * B.kappa * R.srho / (2.0 * cR);
      Rb.srho += lb * B.kappa * R.p / (2.0 * cR);
    }
    Rb.rho += dUb[0] + dUb[1] * R.v1 + dUb[2] * R.v2 + dUb[3] * R.v3;
    Lb.rho -= dUb[0] + dUb[1] * L.v1 + dUb[2] * L.v2 + dUb[3] * L.v3;
    Rb.v1 += dUb[1] * R.rho; Lb.v1 -= dUb[1] * L.rho;
    Rb.v2 += dUb[2] * R.rho; Lb.v2 -= dUb[2] * L.rho;
    Rb.v3 += dUb[3] * R.rho; Lb.v3 -= dUb[3] * L.rho;
    Rb.E += dUb[4]; Lb.E -= dUb[4];
    enthalpy_adj(L, HLb, Lb);
    enthalpy_adj(R, HRb, Rb);
    return;
  }
  // Roe averages
  const double sqL = sqrt(L.rho), sqR = sqrt(R.rho);
  const double ssq = 1.0 / (sqL + sqR);
  const double r1v = (sqR * R.v1 + sqL * L.v1) * ssq;
  const double r2v = (sqR * R.v2 + sqL * L.v2) * ssq;
  const double r3v = (sqR * R.v3 + sqL * L.v3) * ssq;
  const double rH = (sqR * HR + sqL * HL) * ssq;
  const double absVel = r1v * r1v + r2v * r2v + r3v * r3v;
  const double rc = sqrt(B.kappaM1 * (rH - 0.5 * absVel));
  const double a0 = r1v - rc, a1 = r1v, a4 = r1v + rc;
  // forward: strengths and |eigenvalues|
  double A0, A1, A2, A3, A4, e0, e1, e4;
  // Roe intermediates
  double d0 = 0, d1 = 0, d2 = 0, d3 = 0, d4 = 0, d5 = 0, src = 0;
  // RoeEntropyFix intermediates
  double cL = 0, cR = 0, RoeDens = 0, dr = 0, du = 0, dv = 0, dw = 0, dp = 0, tmp = 0, rdc = 0;
  if (solver == RIEMANN_ROE) {
    d0 = R.rho - L.rho;
    d1 = R.rho * R.v1 - L.rho * L.v1;
    d2 = R.rho * R.v2 - L.rho * L.v2;
    d3 = R.rho * R.v3 - L.rho * L.v3;
    d4 = R.E - L.E;
    A2 = d2 - r2v * d0;
    A3 = d3 - r3v * d0;
    d5 = d4 - A2 * r2v - A3 * r3v;
    src = 1.0 / rc;
    A1 = B.kappaM1 * (src * src) * (d0 * (rH - r1v * r1v) - d5 + r1v * d1);
    A0 = 0.5 * src * (d0 * (r1v + rc) - d1 - rc * A1);
    A4 = d0 - A0 - A1;
    e0 = fabs(a0); e1 = fabs(a1); e4 = fabs(a4);
  } else {
    cL = sqrt(B.kappa * L.p * L.srho); cR = sqrt(B.kappa * R.p * R.srho);
    RoeDens = sqL * sqR;
    dr = R.rho - L.rho; du = R.v1 - L.v1; dv = R.v2 - L.v2; dw = R.v3 - L.v3; dp = R.p - L.p;
    tmp = 0.5 / (rc * rc);
    rdc = RoeDens * rc * du;
    A0 = tmp * (dp - rdc);
    A1 = dr - dp * (2.0 * tmp);
    A2 = RoeDens * dv;
    A3 = RoeDens * dw;
    A4 = tmp * (dp + rdc);
    auto fix = [](double a, double al, double ar) {
      const double da = fmax(0.0, fmax(a - al, ar - a));
      const double aa = fabs(a);
      return (aa < da) ? 0.5 * (a * a / da + da) : aa;
    };
    e0 = fix(a0, L.v1 - cL, R.v1 - cR);
    e1 = fix(a1, L.v1, R.v1);
    e4 = fix(a4, L.v1 + cL, R.v1 + cR);
  }
  const double w0 = A0 * e0, w1 = A1 * e1, w2 = A2 * e1, w3 = A3 * e1, w4 = A4 * e4;
  const double Ssum = w0 + w1 + w4;
  // reverse of D
  double w0b = 0, w1b = 0, w2b = 0, w3b = 0, w4b = 0, a0b = 0, a1b = 0, a4b = 0, r1vb = 0, r2vb = 0, r3vb = 0, rHb = 0, rcb = 0, absb = 0;
  double Sb = Db[0];
  w0b += Db[1] * a0; a0b += Db[1] * w0; w1b += Db[1] * r1v; r1vb += Db[1] * w1; w4b += Db[1] * a4; a4b += Db[1] * w4;
  Sb += Db[2] * r2v; r2vb += Db[2] * Ssum; w2b += Db[2];
  Sb += Db[3] * r3v; r3vb += Db[3] * Ssum; w3b += Db[3];
  w0b += Db[4] * (rH - r1v * rc); rHb += Db[4] * (w0 + w4); r1vb += Db[4] * rc * (w4 - w0); rcb += Db[4] * r1v * (w4 - w0);
  w1b += Db[4] * (0.5 * absVel); absb += Db[4] * 0.5 * w1;
  w2b += Db[4] * r2v; r2vb += Db[4] * w2; w3b += Db[4] * r3v; r3vb += Db[4] * w3;
  w4b += Db[4] * (rH + r1v * rc);
  w0b += Sb; w1b += Sb; w4b += Sb;
  double A0b = w0b * e0, A1b = w1b * e1, A2b = w2b * e1, A3b = w3b * e1, A4b = w4b * e4;
  const double e0b = w0b * A0, e1b = w1b * A1 + w2b * A2 + w3b * A3, e4b = w4b * A4;
  if (solver == RIEMANN_ROE) {
    a0b += e0b * sgn1(a0); a1b += e1b * sgn1(a1); a4b += e4b * sgn1(a4);
    double d0b = 0, d1b = 0, d2b = 0, d3b = 0, d4b = 0, d5b = 0, srcb = 0;
    // A4 = d0 - A0 - A1
    d0b += A4b; A0b -= A4b; A1b -= A4b;
    // A0 = 1/2 src X, X = d0 (r1v + rc) - d1 - rc A1
    const double X = d0 * (r1v + rc) - d1 - rc * A1;
    srcb += A0b * 0.5 * X;
    const double Xb = A0b * 0.5 * src;
    d0b += Xb * (r1v + rc); r1vb += Xb * d0; rcb += Xb * (d0 - A1); d1b -= Xb; A1b -= Xb * rc;
    // A1 = kappaM1 src^2 Y, Y = d0 (rH - r1v^2) - d5 + r1v d1
    const double Y = d0 * (rH - r1v * r1v) - d5 + r1v * d1;
    srcb += A1b * B.kappaM1 * 2.0 * src * Y;
    const double Yb = A1b * B.kappaM1 * src * src;
    d0b += Yb * (rH - r1v * r1v); rHb += Yb * d0; r1vb += Yb * (d1 - 2.0 * r1v * d0); d5b -= Yb; d1b += Yb * r1v;
    rcb -= srcb * src * src;
    // d5 = d4 - A2 r2v - A3 r3v
    d4b += d5b; A2b -= d5b * r2v; r2vb -= d5b * A2; A3b -= d5b * r3v; r3vb -= d5b * A3;
    // A2 = d2 - r2v d0, A3 = d3 - r3v d0
    d2b += A2b; r2vb -= A2b * d0; d0b -= A2b * r2v;
    d3b += A3b; r3vb -= A3b * d0; d0b -= A3b * r3v;
    // differences
    Rb.rho += d0b + d1b * R.v1 + d2b * R.v2 + d3b * R.v3;
    Lb.rho -= d0b + d1b * L.v1 + d2b * L.v2 + d3b * L.v3;
    Rb.v1 += d1b * R.rho; Lb.v1 -= d1b * L.rho;
    Rb.v2 += d2b * R.rho; Lb.v2 -= d2b * L.rho;
    Rb.v3 += d3b * R.rho; Lb.v3 -= d3b * L.rho;
    Rb.E += d4b; Lb.E -= d4b;
  } else {
    double alb = 0, arb = 0;
    double cLb = 0, cRb = 0;
    entropy_fix_adj(a0, L.v1 - cL, R.v1 - cR, e0b, a0b, alb, arb);
    Lb.v1 += alb; cLb -= alb; Rb.v1 += arb; cRb -= arb;
    alb = arb = 0;
    entropy_fix_adj(a1, L.v1, R.v1, e1b, a1b, alb, arb);
    Lb.v1 += alb; Rb.v1 += arb;
    alb = arb = 0;
    entropy_fix_adj(a4, L.v1 + cL, R.v1 + cR, e4b, a4b, alb, arb);
    Lb.v1 += alb; cLb += alb; Rb.v1 += arb; cRb += arb;
    // strengths
    const double tmpb = A0b * (dp - rdc) - 2.0 * A1b * dp + A4b * (dp + rdc);
    const double dpb = (A0b - 2.0 * A1b + A4b) * tmp;
    const double rdcb = (A4b - A0b) * tmp;
    const double drb = A1b;
    const double RoeDensb = A2b * dv + A3b * dw + rdcb * rc * du;
    const double dvb = A2b * RoeDens, dwb = A3b * RoeDens;
    rcb += rdcb * RoeDens * du - tmpb / (rc * rc * rc);
    const double dub = rdcb * RoeDens * rc;
    Rb.rho += drb; Lb.rho -= drb;
    Rb.v1 += dub; Lb.v1 -= dub;
    Rb.v2 += dvb; Lb.v2 -= dvb;
    Rb.v3 += dwb; Lb.v3 -= dwb;
    Rb.p += dpb; Lb.p -= dpb;
    // RoeDens = sqL sqR handled with the Roe averages below through sqLb/sqRb
    // c = sqrt(kappa p srho)
    Lb.p += cLb * B.kappa * L.srho / (2.0 * cL); Lb.srho += cLb * B.kappa * L.p / (2.0 * cL);
    Rb.p += cRb * B.kappa * R.srho / (2.0 * cR); Rb.srho += cRb * B.kappa * R.p / (2.0 * cR);
    // stash RoeDens bar into the square-root bars
    // (applied below)
    HLb += 0.0;
    // eigenvalue bars
    r1vb += a0b + a1b + a4b;
    rcb += a4b - a0b;
    // Roe averages reverse (shared with Roe), plus RoeDens
    double ssqb = 0, sqLb = RoeDensb * sqR, sqRb = RoeDensb * sqL;
    const double Zb = rcb / (2.0 * rc);
    rHb += B.kappaM1 * Zb;
    absb -= 0.5 * B.kappaM1 * Zb;
    r1vb += 2.0 * r1v * absb; r2vb += 2.0 * r2v * absb; r3vb += 2.0 * r3v * absb;
    ssqb += rHb * (sqR * HR + sqL * HL) + r1vb * (sqR * R.v1 + sqL * L.v1) + r2vb * (sqR * R.v2 + sqL * L.v2) + r3vb * (sqR * R.v3 + sqL * L.v3);
    sqRb += (rHb * HR + r1vb * R.v1 + r2vb * R.v2 + r3vb * R.v3) * ssq;
    sqLb += (rHb * HL + r1vb * L.v1 + r2vb * L.v2 + r3vb * L.v3) * ssq;
    HRb += rHb * sqR * ssq; HLb += rHb * sqL * ssq;
    Rb.v1 += r1vb * sqR * ssq; Lb.v1 += r1vb * sqL * ssq;
    Rb.v2 += r2vb * sqR * ssq; Lb.v2 += r2vb * sqL * ssq;
    Rb.v3 += r3vb * sqR * ssq; Lb.v3 += r3vb * sqL * ssq;
    sqLb -= ssqb * ssq * ssq; sqRb -= ssqb * ssq * ssq;
    Lb.rho += sqLb / (2.0 * sqL); Rb.rho += sqRb / (2.0 * sqR);
    enthalpy_adj(L, HLb, Lb);
    enthalpy_adj(R, HRb, Rb);
    return;
  }
  // Roe: eigenvalue bars and Roe averages reverse
  r1vb += a0b + a1b + a4b;
  rcb += a4b - a0b;
  double ssqb = 0, sqLb = 0, sqRb = 0;
  const double Zb = rcb / (2.0 * rc);
  rHb += B.kappaM1 * Zb;
  absb -= 0.5 * B.kappaM1 * Zb;
  r1vb += 2.0 * r1v * absb; r2vb += 2.0 * r2v * absb; r3vb += 2.0 * r3v * absb;
  ssqb += rHb * (sqR * HR + sqL * HL) + r1vb * (sqR * R.v1 + sqL * L.v1) + r2vb * (sqR * R.v2 + sqL * L.v2) + r3vb * (sqR * R.v3 + sqL * L.v3);
  sqRb += (rHb * HR + r1vb * R.v1 + r2vb * R.v2 + r3vb * R.v3) * ssq;
  sqLb += (rHb * HL + r1vb * L.v1 + r2vb * L.v2 + r3vb * L.v3) * ssq;
  HRb += rHb * sqR * ssq; HLb += rHb * sqL * ssq;
  Rb.v1 += r1vb * sqR * ssq; Lb.v1 += r1vb * sqL * ssq;
  Rb.v2 += r2vb * sqR * ssq; Lb.v2 += r2vb * sqL * ssq;
  Rb.v3 += r3vb * sqR * ssq; Lb.v3 += r3vb * sqL * ssq;
  sqLb -= ssqb * ssq * ssq; sqRb -= ssqb * ssq * ssq;
  Lb.rho += sqLb / (2.0 * sqL); Rb.rho += sqRb / (2.0 * sqR);
  enthalpy_adj(L, HLb, Lb);
  enthalpy_adj(R, HRb, Rb);
}

// ---- the split fluxes MO, DU and KG (splitflux.f90: SplitVolumeFluxMO :445, DU :225, KG :327 and their surface forms) ----

// IR's means of two states (splitflux.f90:SplitSurfaceFluxIR, riemann.f90:Riemann_IR): z1 = sqrt(rho/p), z5 = sqrt(rho p)
struct IRMeans {
  double zL1, zL5, zR1, zR5, z1Log, z5Log, z1s, rhoHat, pHat, p2Hat, uH, vH, wH;
};
FG_HD IRMeans ir_means(const Basis& B, const RotState& L, const RotState& R) {
  IRMeans m;
  m.zL1 = sqrt(L.rho / L.p); m.zL5 = sqrt(L.rho * L.p); m.zR1 = sqrt(R.rho / R.p); m.zR5 = sqrt(R.rho * R.p);
  m.z1Log = log_mean(m.zL1, m.zR1); m.z5Log = log_mean(m.zL5, m.zR5);
  m.z1s = m.zL1 + m.zR1;
  m.rhoHat = 0.5 * m.z1s * m.z5Log;
  m.pHat = (m.zL5 + m.zR5) / m.z1s;
  m.p2Hat = 0.5 / B.kappa * ((B.kappa + 1.0) * m.z5Log / m.z1Log + B.kappaM1 * m.pHat);
  m.uH = (m.zL1 * L.v1 + m.zR1 * R.v1) / m.z1s;
  m.vH = (m.zL1 * L.v2 + m.zR1 * R.v2) / m.z1s;
  m.wH = (m.zL1 * L.v3 + m.zR1 * R.v3) / m.z1s;
  return m;
}
// the means transposed: given the bars of rhoHat, pHat, p2Hat, uH, vH, wH, adds to both states' bars
FG_HD void ir_means_adj(const Basis& B, const RotState& L, const RotState& R, const IRMeans& m, double rhoHatb, double pHatb, double p2Hatb,
                        double uHb, double vHb, double wHb, RotState& Lb, RotState& Rb) {
  double z5Logb = p2Hatb * 0.5 / B.kappa * (B.kappa + 1.0) / m.z1Log;
  const double z1Logb = -p2Hatb * 0.5 / B.kappa * (B.kappa + 1.0) * m.z5Log / (m.z1Log * m.z1Log);
  pHatb += p2Hatb * 0.5 * B.kappaM1 / B.kappa;
  double zL1b = 0.0, zR1b = 0.0, zL5b = pHatb / m.z1s, zR5b = pHatb / m.z1s;
  double z1sb = -pHatb * m.pHat / m.z1s;
  zL1b += (uHb * L.v1 + vHb * L.v2 + wHb * L.v3) / m.z1s;
  zR1b += (uHb * R.v1 + vHb * R.v2 + wHb * R.v3) / m.z1s;
  Lb.v1 += uHb * m.zL1 / m.z1s; Rb.v1 += uHb * m.zR1 / m.z1s;
  Lb.v2 += vHb * m.zL1 / m.z1s; Rb.v2 += vHb * m.zR1 / m.z1s;
  Lb.v3 += wHb * m.zL1 / m.z1s; Rb.v3 += wHb * m.zR1 / m.z1s;
  z1sb -= (uHb * m.uH + vHb * m.vH + wHb * m.wH) / m.z1s;
  z1sb += rhoHatb * 0.5 * m.z5Log;
  z5Logb += rhoHatb * 0.5 * m.z1s;
  zL1b += z1sb; zR1b += z1sb;
  log_mean_adj(m.zL1, m.zR1, z1Logb, zL1b, zR1b);
  log_mean_adj(m.zL5, m.zR5, z5Logb, zL5b, zR5b);
  // z1 = sqrt(rho / p), z5 = sqrt(rho p)
  Lb.rho += zL1b * m.zL1 / (2.0 * L.rho) + zL5b * m.zL5 / (2.0 * L.rho);
  Lb.p += -zL1b * m.zL1 / (2.0 * L.p) + zL5b * m.zL5 / (2.0 * L.p);
  Rb.rho += zR1b * m.zR1 / (2.0 * R.rho) + zR5b * m.zR5 / (2.0 * R.rho);
  Rb.p += -zR1b * m.zR1 / (2.0 * R.p) + zR5b * m.zR5 / (2.0 * R.p);
}

// split_surface_flux_more transposed for MO, DU, KG, CH, IR on rotated states: Fb[5] given, adds to both states' bars
FG_HD void split_surface_flux_more_adj(int sd, const Basis& B, const RotState& L, const RotState& R, const double* Fb, RotState& Lb,
                                       RotState& Rb) {
  if (sd == SPLIT_CH) {
    const double bL = 0.5 * L.rho / L.p, bR = 0.5 * R.rho / R.p;
    const double rhoLog = log_mean(L.rho, R.rho), betaLog = log_mean(bL, bR);
    const double pHat = 0.5 * (L.rho + R.rho) / (bL + bR);
    const double H = 0.5 * B.sKappaM1 / betaLog + pHat / rhoLog + 0.5 * (L.v1 * R.v1 + L.v2 * R.v2 + L.v3 * R.v3);
    const double us = L.v1 + R.v1;
    const double F0 = rhoLog * 0.5 * us;
    const double F0b = Fb[0] + Fb[1] * 0.5 * us + Fb[2] * 0.5 * (L.v2 + R.v2) + Fb[3] * 0.5 * (L.v3 + R.v3) + Fb[4] * H;
    const double usb = Fb[1] * F0 * 0.5 + F0b * rhoLog * 0.5;
    Lb.v1 += usb; Rb.v1 += usb;
    Lb.v2 += Fb[2] * F0 * 0.5; Rb.v2 += Fb[2] * F0 * 0.5;
    Lb.v3 += Fb[3] * F0 * 0.5; Rb.v3 += Fb[3] * F0 * 0.5;
    const double Hb = Fb[4] * F0;
    const double pHatb = Fb[1] + Hb / rhoLog;
    const double rhoLogb = F0b * 0.5 * us - Hb * pHat / (rhoLog * rhoLog);
    const double betaLogb = -Hb * 0.5 * B.sKappaM1 / (betaLog * betaLog);
    Lb.v1 += 0.5 * Hb * R.v1; Rb.v1 += 0.5 * Hb * L.v1;
    Lb.v2 += 0.5 * Hb * R.v2; Rb.v2 += 0.5 * Hb * L.v2;
    Lb.v3 += 0.5 * Hb * R.v3; Rb.v3 += 0.5 * Hb * L.v3;
    Lb.rho += pHatb * 0.5 / (bL + bR); Rb.rho += pHatb * 0.5 / (bL + bR);
    double bLb = -pHatb * pHat / (bL + bR), bRb = bLb;
    log_mean_adj(L.rho, R.rho, rhoLogb, Lb.rho, Rb.rho);
    log_mean_adj(bL, bR, betaLogb, bLb, bRb);
    Lb.rho += bLb * 0.5 / L.p; Lb.p -= bLb * 0.5 * L.rho / (L.p * L.p);
    Rb.rho += bRb * 0.5 / R.p; Rb.p -= bRb * 0.5 * R.rho / (R.p * R.p);
    return;
  }
  if (sd == SPLIT_IR) {
    const IRMeans m = ir_means(B, L, R);
    const double hH = B.kappa * m.p2Hat / (m.rhoHat * B.kappaM1) + 0.5 * (m.uH * m.uH + m.vH * m.vH + m.wH * m.wH);
    const double F0 = m.rhoHat * m.uH;
    const double F0b = Fb[0] + Fb[1] * m.uH + Fb[2] * m.vH + Fb[3] * m.wH + Fb[4] * hH;
    const double hHb = Fb[4] * F0;
    const double uHb = Fb[1] * F0 + F0b * m.rhoHat + hHb * m.uH;
    const double vHb = Fb[2] * F0 + hHb * m.vH, wHb = Fb[3] * F0 + hHb * m.wH;
    const double p2Hatb = hHb * B.kappa / (m.rhoHat * B.kappaM1);
    const double rhoHatb = F0b * m.uH - hHb * B.kappa * m.p2Hat / (m.rhoHat * m.rhoHat * B.kappaM1);
    ir_means_adj(B, L, R, m, rhoHatb, Fb[1], p2Hatb, uHb, vHb, wHb, Lb, Rb);
    return;
  }
  if (sd == SPLIT_DU) {
    const double us = L.v1 + R.v1;
    const double mL = L.rho * L.v1, mR = R.rho * R.v1;
    const double usb = 0.25 * (Fb[0] * (L.rho + R.rho) + Fb[1] * (mL + mR) + Fb[2] * (L.rho * L.v2 + R.rho * R.v2) +
                               Fb[3] * (L.rho * L.v3 + R.rho * R.v3) + Fb[4] * (L.E + R.E + L.p + R.p));
    const double q = 0.25 * us;
    Lb.rho += q * (Fb[0] + Fb[1] * L.v1 + Fb[2] * L.v2 + Fb[3] * L.v3);
    Rb.rho += q * (Fb[0] + Fb[1] * R.v1 + Fb[2] * R.v2 + Fb[3] * R.v3);
    Lb.v1 += q * Fb[1] * L.rho + usb; Rb.v1 += q * Fb[1] * R.rho + usb;
    Lb.v2 += q * Fb[2] * L.rho; Rb.v2 += q * Fb[2] * R.rho;
    Lb.v3 += q * Fb[3] * L.rho; Rb.v3 += q * Fb[3] * R.rho;
    Lb.p += 0.5 * Fb[1] + q * Fb[4]; Rb.p += 0.5 * Fb[1] + q * Fb[4];
    Lb.E += q * Fb[4]; Rb.E += q * Fb[4];
  } else if (sd == SPLIT_KG) {
    const double rs = L.rho + R.rho, us = L.v1 + R.v1, b = 0.125 * rs * us;
    const double eL = L.E * L.srho, eR = R.E * R.srho;
    const double bb = Fb[1] * us + Fb[2] * (L.v2 + R.v2) + Fb[3] * (L.v3 + R.v3) + Fb[4] * (eL + eR);
    const double rsb = 0.25 * Fb[0] * us + 0.125 * bb * us;
    const double usb = 0.25 * Fb[0] * rs + Fb[1] * b + 0.125 * bb * rs + 0.25 * Fb[4] * (L.p + R.p);
    Lb.rho += rsb; Rb.rho += rsb;
    Lb.v1 += usb; Rb.v1 += usb;
    Lb.v2 += Fb[2] * b; Rb.v2 += Fb[2] * b;
    Lb.v3 += Fb[3] * b; Rb.v3 += Fb[3] * b;
    Lb.E += Fb[4] * b * L.srho; Lb.srho += Fb[4] * b * L.E;
    Rb.E += Fb[4] * b * R.srho; Rb.srho += Fb[4] * b * R.E;
    Lb.p += 0.5 * Fb[1] + 0.25 * Fb[4] * us; Rb.p += 0.5 * Fb[1] + 0.25 * Fb[4] * us;
  } else {  // MO
    const double mL = L.rho * L.v1, mR = R.rho * R.v1, ms = mL + mR;
    const double kL = L.v1 * L.v1 + L.v2 * L.v2 + L.v3 * L.v3, kR = R.v1 * R.v1 + R.v2 * R.v2 + R.v3 * R.v3;
    const double rhoepL = L.E - 0.5 * L.rho * kL + L.p, rhoepR = R.E - 0.5 * R.rho * kR + R.p;
    const double vv = L.v1 * R.v1 + L.v2 * R.v2 + L.v3 * R.v3;
    const double msb = 0.5 * Fb[0] + 0.25 * (Fb[1] * (L.v1 + R.v1) + Fb[2] * (L.v2 + R.v2) + Fb[3] * (L.v3 + R.v3) + Fb[4] * vv);
    const double q = 0.25 * ms;
    Lb.v1 += q * Fb[1]; Rb.v1 += q * Fb[1];
    Lb.v2 += q * Fb[2]; Rb.v2 += q * Fb[2];
    Lb.v3 += q * Fb[3]; Rb.v3 += q * Fb[3];
    Lb.p += 0.5 * Fb[1]; Rb.p += 0.5 * Fb[1];
    const double vvb = q * Fb[4];
    Lb.v1 += vvb * R.v1; Rb.v1 += vvb * L.v1;
    Lb.v2 += vvb * R.v2; Rb.v2 += vvb * L.v2;
    Lb.v3 += vvb * R.v3; Rb.v3 += vvb * L.v3;
    // F4's (rho e + p) v1 / 2 terms, rho e + p = E - rho |v|^2 / 2 + p
    const double eLb = 0.5 * Fb[4] * L.v1, eRb = 0.5 * Fb[4] * R.v1;
    Lb.v1 += 0.5 * Fb[4] * rhoepL; Rb.v1 += 0.5 * Fb[4] * rhoepR;
    Lb.E += eLb; Lb.p += eLb; Lb.rho -= 0.5 * eLb * kL;
    Lb.v1 -= eLb * L.rho * L.v1; Lb.v2 -= eLb * L.rho * L.v2; Lb.v3 -= eLb * L.rho * L.v3;
    Rb.E += eRb; Rb.p += eRb; Rb.rho -= 0.5 * eRb * kR;
    Rb.v1 -= eRb * R.rho * R.v1; Rb.v2 -= eRb * R.rho * R.v2; Rb.v3 -= eRb * R.rho * R.v3;
    // ms = rho_L v1_L + rho_R v1_R
    Lb.rho += msb * L.v1; Lb.v1 += msb * L.rho;
    Rb.rho += msb * R.v1; Rb.v1 += msb * R.rho;
  }
}

// the split form's central surface flux transposed: PI / SD (split_surface_flux_adj) or MO, DU, KG, CH, IR
FG_HD void central_flux_adj(int sd, const Basis& B, const RotState& L, const RotState& R, double HL, double HR, const double* Fb, RotState& Lb,
                            RotState& Rb, double& HLb, double& HRb) {
  if (sd == SPLIT_PI || sd == SPLIT_SD) split_surface_flux_adj(sd, L, R, HL, HR, Fb, Lb, Rb, HLb, HRb);
  else split_surface_flux_more_adj(sd, B, L, R, Fb, Lb, Rb);
}

// ---- the Riemann solvers of riemann_rotated_more: HLL, HLLE, HLLEM, RoeL2, RoeEntropyGShockFix, the flux average ----

// transposed Roe averages (square-root-density weights of v1..v3 and H; rc = sqrt(kappaM1 (rH - absVel/2)), absVel =
// r1v^2 + r2v^2 + r3v^2): given the bars of the averages, of rc and absVel, and of the square roots of the densities,
// adds to the states' bars and to the enthalpy bars HLb, HRb (the caller applies enthalpy_adj)
FG_HD void roe_average_adj(const Basis& B, const RotState& L, const RotState& R, double HL, double HR, double sqL, double sqR, double ssq,
                           double r1v, double r2v, double r3v, double rc, double r1vb, double r2vb, double r3vb, double rHb, double rcb,
                           double absb, double sqLb, double sqRb, RotState& Lb, RotState& Rb, double& HLb, double& HRb) {
  const double Zb = rcb / (2.0 * rc);
  rHb += B.kappaM1 * Zb;
  absb -= 0.5 * B.kappaM1 * Zb;
  r1vb += 2.0 * r1v * absb; r2vb += 2.0 * r2v * absb; r3vb += 2.0 * r3v * absb;
  const double ssqb = rHb * (sqR * HR + sqL * HL) + r1vb * (sqR * R.v1 + sqL * L.v1) + r2vb * (sqR * R.v2 + sqL * L.v2) +
                      r3vb * (sqR * R.v3 + sqL * L.v3);
  sqRb += (rHb * HR + r1vb * R.v1 + r2vb * R.v2 + r3vb * R.v3) * ssq;
  sqLb += (rHb * HL + r1vb * L.v1 + r2vb * L.v2 + r3vb * L.v3) * ssq;
  HRb += rHb * sqR * ssq; HLb += rHb * sqL * ssq;
  Rb.v1 += r1vb * sqR * ssq; Lb.v1 += r1vb * sqL * ssq;
  Rb.v2 += r2vb * sqR * ssq; Lb.v2 += r2vb * sqL * ssq;
  Rb.v3 += r3vb * sqR * ssq; Lb.v3 += r3vb * sqL * ssq;
  sqLb -= ssqb * ssq * ssq; sqRb -= ssqb * ssq * ssq;
  Lb.rho += sqLb / (2.0 * sqL); Rb.rho += sqRb / (2.0 * sqR);
}

// c = sqrt(kappa p srho): adds the bars of p and srho for the bar of c
FG_HD void sound_speed_adj(const Basis& B, const RotState& S, double c, double cb, RotState& Sb) {
  Sb.p += cb * B.kappa * S.srho / (2.0 * c);
  Sb.srho += cb * B.kappa * S.p / (2.0 * c);
}

// dU = U_R - U_L of the conservative variables (rho, rho v1, rho v2, rho v3, E): adds the states' bars for dUb[5]
FG_HD void jump_adj(const RotState& L, const RotState& R, const double* dUb, RotState& Lb, RotState& Rb) {
  Rb.rho += dUb[0] + dUb[1] * R.v1 + dUb[2] * R.v2 + dUb[3] * R.v3;
  Lb.rho -= dUb[0] + dUb[1] * L.v1 + dUb[2] * L.v2 + dUb[3] * L.v3;
  Rb.v1 += dUb[1] * R.rho; Lb.v1 -= dUb[1] * L.rho;
  Rb.v2 += dUb[2] * R.rho; Lb.v2 -= dUb[2] * L.rho;
  Rb.v3 += dUb[3] * R.rho; Lb.v3 -= dUb[3] * L.rho;
  Rb.E += dUb[4]; Lb.E -= dUb[4];
}

// bars of the Roe-type dissipation D = sum_k A_k e_k r_k (w_k = A_k e_k; a0, a4 the outer eigenvalues in D[1], r1v the
// averaged normal velocity in the other rows): given Db[5], sets the bars of A0..A4, e0, e1, e4, a0, a4 and adds those of
// r1v, r2v, r3v, rH, rc and absVel
struct RoeDissBars {
  double A[5], e0, e1, e4, a0, a4;
};
FG_HD void roe_dissipation_adj(const double* Db, const double* A, double e0, double e1, double e4, double a0, double a4, double r1v, double r2v,
                               double r3v, double rH, double rc, double absVel, RoeDissBars& o, double& r1vb, double& r2vb, double& r3vb,
                               double& rHb, double& rcb, double& absb) {
  const double w0 = A[0] * e0, w1 = A[1] * e1, w2 = A[2] * e1, w3 = A[3] * e1, w4 = A[4] * e4;
  const double S = w0 + w1 + w4;
  double w0b = 0, w1b = 0, w2b = 0, w3b = 0, w4b = 0;
  double Sb = Db[0];
  w0b += Db[1] * a0; o.a0 = Db[1] * w0; w1b += Db[1] * r1v; r1vb += Db[1] * w1; w4b += Db[1] * a4; o.a4 = Db[1] * w4;
  Sb += Db[2] * r2v; r2vb += Db[2] * S; w2b += Db[2];
  Sb += Db[3] * r3v; r3vb += Db[3] * S; w3b += Db[3];
  w0b += Db[4] * (rH - r1v * rc); rHb += Db[4] * (w0 + w4); r1vb += Db[4] * rc * (w4 - w0); rcb += Db[4] * r1v * (w4 - w0);
  w1b += Db[4] * (0.5 * absVel); absb += Db[4] * 0.5 * w1;
  w2b += Db[4] * r2v; r2vb += Db[4] * w2; w3b += Db[4] * r3v; r3vb += Db[4] * w3;
  w4b += Db[4] * (rH + r1v * rc);
  w0b += Sb; w1b += Sb; w4b += Sb;
  o.A[0] = w0b * e0; o.A[1] = w1b * e1; o.A[2] = w2b * e1; o.A[3] = w3b * e1; o.A[4] = w4b * e4;
  o.e0 = w0b * A[0]; o.e1 = w1b * A[1] + w2b * A[2] + w3b * A[3]; o.e4 = w4b * A[4];
}

// Transposed Jacobian of riemann_rotated_more for HLL, HLLE, HLLEM (riemann.f90:1067-1235), RoeL2 (:983) and
// RoeEntropyGShockFix (:866) with the weak form or any split form, of the split form's flux average (:1236), CH (:1261) and
// IR (:1315) surface fluxes, and of LF, HLLC, Roe and RoeEntropyFix (riemann_rotated_adj) with MO, DU, KG, CH, IR. Fb[5]
// given, adds to the bars of both rotated states.
FG_HD void riemann_rotated_more_adj(int solver, int splitDG, const Basis& B, const RotState& L, const RotState& R, const double* Fb,
                                    RotState& Lb, RotState& Rb) {
  if (solver == RIEMANN_LF || solver == RIEMANN_HLLC || solver == RIEMANN_ROE || solver == RIEMANN_ROEENTROPYFIX) {
    if (splitDG >= 0 && splitDG != SPLIT_PI && splitDG != SPLIT_SD && solver != RIEMANN_HLLC) {
      // central part MO / DU / KG: F = central - dissipation/2, the weak form's F = (F_L + F_R)/2 - the same dissipation/2,
      // so the transpose is the weak form's, minus that of (F_L + F_R)/2, plus that of the central flux (HLLC has no
      // central part)
      riemann_rotated_adj(solver, -1, B, L, R, Fb, Lb, Rb);
      double Fh[5];
      for (int v = 0; v < 5; ++v) Fh[v] = -0.5 * Fb[v];
      euler_flux_1d_adj(L, Fh, Lb);
      euler_flux_1d_adj(R, Fh, Rb);
      split_surface_flux_more_adj(splitDG, B, L, R, Fb, Lb, Rb);
      return;
    }
    riemann_rotated_adj(solver, splitDG, B, L, R, Fb, Lb, Rb);
    return;
  }
  const bool split = splitDG >= 0;
  const double HL = (L.E + L.p) * L.srho, HR = (R.E + R.p) * R.srho;
  double HLb = 0.0, HRb = 0.0;
  if (solver == RIEMANN_AVERAGE) {
    central_flux_adj(splitDG, B, L, R, HL, HR, Fb, Lb, Rb, HLb, HRb);
    enthalpy_adj(L, HLb, Lb);
    enthalpy_adj(R, HRb, Rb);
    return;
  }
  const double cL = sqrt(B.kappa * L.p * L.srho), cR = sqrt(B.kappa * R.p * R.srho);
  if (solver == RIEMANN_CH) {
    // F = central - (lmax / 2) (dU_0..3, X4), X4 = drho T1 + rhoMean T2 + rhoMean sKappaM1 (1/bR - 1/bL) / 2,
    // T1 = sKappaM1 / (2 betaLog) + vL . vR / 2, T2 = (|vR|^2 - |vL|^2) / 2, b = rho / (2p)
    central_flux_adj(splitDG, B, L, R, HL, HR, Fb, Lb, Rb, HLb, HRb);
    const double aL = fabs(L.v1), aR = fabs(R.v1);
    const double lmax = fmax(aR, aL) + fmax(cL, cR), h = 0.5 * lmax;
    const double rhoMean = 0.5 * (L.rho + R.rho);
    const double bL = 0.5 * L.rho / L.p, bR = 0.5 * R.rho / R.p;
    const double betaLog = log_mean(bL, bR);
    const double dU[4] = {R.rho - L.rho, R.rho * R.v1 - L.rho * L.v1, R.rho * R.v2 - L.rho * L.v2, R.rho * R.v3 - L.rho * L.v3};
    const double T1 = 0.5 * B.sKappaM1 / betaLog + 0.5 * (R.v1 * L.v1 + R.v2 * L.v2 + R.v3 * L.v3);
    const double T2 = 0.5 * (L.v1 + R.v1) * (R.v1 - L.v1) + 0.5 * (L.v2 + R.v2) * (R.v2 - L.v2) + 0.5 * (L.v3 + R.v3) * (R.v3 - L.v3);
    const double X4 = dU[0] * T1 + rhoMean * T2 + 0.5 * rhoMean * B.sKappaM1 * (1.0 / bR - 1.0 / bL);
    double hb = 0.0, dUb[5] = {0., 0., 0., 0., 0.};
    for (int v = 0; v < 4; ++v) { hb -= Fb[v] * dU[v]; dUb[v] = -h * Fb[v]; }
    hb -= Fb[4] * X4;
    const double X4b = -h * Fb[4];
    dUb[0] += X4b * T1;
    const double T1b = X4b * dU[0], T2b = X4b * rhoMean;
    const double rhoMeanb = X4b * (T2 + 0.5 * B.sKappaM1 * (1.0 / bR - 1.0 / bL));
    double bLb = X4b * 0.5 * rhoMean * B.sKappaM1 / (bL * bL), bRb = -X4b * 0.5 * rhoMean * B.sKappaM1 / (bR * bR);
    const double betaLogb = -T1b * 0.5 * B.sKappaM1 / (betaLog * betaLog);
    Rb.v1 += 0.5 * T1b * L.v1 + T2b * R.v1; Lb.v1 += 0.5 * T1b * R.v1 - T2b * L.v1;
    Rb.v2 += 0.5 * T1b * L.v2 + T2b * R.v2; Lb.v2 += 0.5 * T1b * R.v2 - T2b * L.v2;
    Rb.v3 += 0.5 * T1b * L.v3 + T2b * R.v3; Lb.v3 += 0.5 * T1b * R.v3 - T2b * L.v3;
    log_mean_adj(bL, bR, betaLogb, bLb, bRb);
    Lb.rho += bLb * 0.5 / L.p + 0.5 * rhoMeanb; Lb.p -= bLb * 0.5 * L.rho / (L.p * L.p);
    Rb.rho += bRb * 0.5 / R.p + 0.5 * rhoMeanb; Rb.p -= bRb * 0.5 * R.rho / (R.p * R.p);
    jump_adj(L, R, dUb, Lb, Rb);
    const double lb = 0.5 * hb;
    if (aR >= aL) Rb.v1 += lb * sgn1(R.v1); else Lb.v1 += lb * sgn1(L.v1);
    if (cL >= cR) sound_speed_adj(B, L, cL, lb, Lb); else sound_speed_adj(B, R, cR, lb, Rb);
    enthalpy_adj(L, HLb, Lb);
    enthalpy_adj(R, HRb, Rb);
    return;
  }
  if (solver == RIEMANN_IR) {
    // F = central - Dd/2, Dd = R |Lambda| T R^T vJ with the jump vJ of the entropy variables and the eigenvectors at IR's means
    central_flux_adj(splitDG, B, L, R, HL, HR, Fb, Lb, Rb, HLb, HRb);
    const double sR = log(R.p) - B.kappa * log(R.rho), sL = log(L.p) - B.kappa * log(L.rho);
    const double rpR = R.rho / R.p, rpL = L.rho / L.p;
    const double kR = R.v1 * R.v1 + R.v2 * R.v2 + R.v3 * R.v3, kL = L.v1 * L.v1 + L.v2 * L.v2 + L.v3 * L.v3;
    double vJ[5];
    vJ[0] = ((B.kappa - sR) - (B.kappa - sL)) * B.sKappaM1 - 0.5 * (rpR * kR - rpL * kL);
    vJ[1] = rpR * R.v1 - rpL * L.v1;
    vJ[2] = rpR * R.v2 - rpL * L.v2;
    vJ[3] = rpR * R.v3 - rpL * L.v3;
    vJ[4] = rpL - rpR;
    const IRMeans m = ir_means(B, L, R);
    const double uH = m.uH, vH = m.vH, wH = m.wH, rhoHat = m.rhoHat, pHat = m.pHat, p2Hat = m.p2Hat;
    const double aH = sqrt(B.kappa * p2Hat / rhoHat);
    const double ek = 0.5 * (uH * uH + vH * vH + wH * wH);
    const double hH = B.kappa * p2Hat / (rhoHat * B.kappaM1) + ek;
    const double c0 = vJ[0] + (uH - aH) * vJ[1] + vH * vJ[2] + wH * vJ[3] + (hH - uH * aH) * vJ[4];
    const double c1 = vJ[0] + uH * vJ[1] + vH * vJ[2] + wH * vJ[3] + ek * vJ[4];
    const double c2 = vJ[2] + vH * vJ[4];
    const double c3 = vJ[3] + wH * vJ[4];
    const double c4 = vJ[0] + (uH + aH) * vJ[1] + vH * vJ[2] + wH * vJ[3] + (hH + uH * aH) * vJ[4];
    const double am = uH - aH, ap = uH + aH;
    const double Am = fabs(am), Ap = fabs(ap), Au = fabs(uH);
    const double d0 = 0.5 * Am * rhoHat / B.kappa * c0;
    const double d1 = Au * (B.kappaM1 / B.kappa) * rhoHat * c1;
    const double d2 = Au * pHat * c2;
    const double d3 = Au * pHat * c3;
    const double d4 = 0.5 * Ap * rhoHat / B.kappa * c4;
    const double sum014 = d0 + d1 + d4;
    double Ddb[5];
    for (int v = 0; v < 5; ++v) Ddb[v] = -0.5 * Fb[v];
    // Dd0 = sum014, Dd1 = (uH - aH) d0 + uH d1 + (uH + aH) d4, Dd2 = vH sum014 + d2, Dd3 = wH sum014 + d3,
    // Dd4 = (hH - uH aH) d0 + ek d1 + vH d2 + wH d3 + (hH + uH aH) d4
    const double sumb = Ddb[0] + Ddb[2] * vH + Ddb[3] * wH;
    const double d0b = sumb + Ddb[1] * am + Ddb[4] * (hH - uH * aH);
    const double d1b = sumb + Ddb[1] * uH + Ddb[4] * ek;
    const double d4b = sumb + Ddb[1] * ap + Ddb[4] * (hH + uH * aH);
    const double d2b = Ddb[2] + Ddb[4] * vH, d3b = Ddb[3] + Ddb[4] * wH;
    double uHb = Ddb[1] * (d0 + d1 + d4) + Ddb[4] * aH * (d4 - d0);
    double aHb = Ddb[1] * (d4 - d0) + Ddb[4] * uH * (d4 - d0);
    double vHb = Ddb[2] * sum014 + Ddb[4] * d2;
    double wHb = Ddb[3] * sum014 + Ddb[4] * d3;
    double hHb = Ddb[4] * (d0 + d4);
    double ekb = Ddb[4] * d1;
    // d_k
    const double Amb = d0b * 0.5 * rhoHat / B.kappa * c0, Apb = d4b * 0.5 * rhoHat / B.kappa * c4;
    const double Aub = d1b * (B.kappaM1 / B.kappa) * rhoHat * c1 + (d2b * c2 + d3b * c3) * pHat;
    double rhoHatb = d0b * 0.5 * Am / B.kappa * c0 + d1b * Au * (B.kappaM1 / B.kappa) * c1 + d4b * 0.5 * Ap / B.kappa * c4;
    double pHatb = Au * (d2b * c2 + d3b * c3);
    const double c0b = d0b * 0.5 * Am * rhoHat / B.kappa, c1b = d1b * Au * (B.kappaM1 / B.kappa) * rhoHat;
    const double c2b = d2b * Au * pHat, c3b = d3b * Au * pHat, c4b = d4b * 0.5 * Ap * rhoHat / B.kappa;
    const double amb = Amb * sgn1(am), apb = Apb * sgn1(ap);
    uHb += amb + apb + Aub * sgn1(uH);
    aHb += apb - amb;
    // c_k
    double vJb[5];
    vJb[0] = c0b + c1b + c4b;
    vJb[1] = c0b * am + c1b * uH + c4b * ap;
    vJb[2] = c0b * vH + c1b * vH + c2b + c4b * vH;
    vJb[3] = c0b * wH + c1b * wH + c3b + c4b * wH;
    vJb[4] = c0b * (hH - uH * aH) + c1b * ek + c2b * vH + c3b * wH + c4b * (hH + uH * aH);
    uHb += c0b * (vJ[1] - aH * vJ[4]) + c1b * vJ[1] + c4b * (vJ[1] + aH * vJ[4]);
    aHb += c0b * (-vJ[1] - uH * vJ[4]) + c4b * (vJ[1] + uH * vJ[4]);
    vHb += (c0b + c1b + c4b) * vJ[2] + c2b * vJ[4];
    wHb += (c0b + c1b + c4b) * vJ[3] + c3b * vJ[4];
    hHb += (c0b + c4b) * vJ[4];
    ekb += c1b * vJ[4];
    // hH = kappa p2Hat / (rhoHat kappaM1) + ek, ek = |uH|^2 / 2, aH = sqrt(kappa p2Hat / rhoHat)
    double p2Hatb = hHb * B.kappa / (rhoHat * B.kappaM1);
    rhoHatb -= hHb * B.kappa * p2Hat / (rhoHat * rhoHat * B.kappaM1);
    ekb += hHb;
    uHb += ekb * uH; vHb += ekb * vH; wHb += ekb * wH;
    const double rb = aHb / (2.0 * aH);
    p2Hatb += rb * B.kappa / rhoHat;
    rhoHatb -= rb * B.kappa * p2Hat / (rhoHat * rhoHat);
    ir_means_adj(B, L, R, m, rhoHatb, pHatb, p2Hatb, uHb, vHb, wHb, Lb, Rb);
    // vJ
    const double sLb = vJb[0] * B.sKappaM1, sRb = -vJb[0] * B.sKappaM1;
    const double rpRb = -0.5 * vJb[0] * kR + vJb[1] * R.v1 + vJb[2] * R.v2 + vJb[3] * R.v3 - vJb[4];
    const double rpLb = 0.5 * vJb[0] * kL - vJb[1] * L.v1 - vJb[2] * L.v2 - vJb[3] * L.v3 + vJb[4];
    Rb.v1 += -vJb[0] * rpR * R.v1 + vJb[1] * rpR; Lb.v1 += vJb[0] * rpL * L.v1 - vJb[1] * rpL;
    Rb.v2 += -vJb[0] * rpR * R.v2 + vJb[2] * rpR; Lb.v2 += vJb[0] * rpL * L.v2 - vJb[2] * rpL;
    Rb.v3 += -vJb[0] * rpR * R.v3 + vJb[3] * rpR; Lb.v3 += vJb[0] * rpL * L.v3 - vJb[3] * rpL;
    // s = ln p - kappa ln rho, rp = rho / p
    Rb.p += sRb / R.p - rpRb * R.rho / (R.p * R.p); Rb.rho += -sRb * B.kappa / R.rho + rpRb / R.p;
    Lb.p += sLb / L.p - rpLb * L.rho / (L.p * L.p); Lb.rho += -sLb * B.kappa / L.rho + rpLb / L.p;
    enthalpy_adj(L, HLb, Lb);
    enthalpy_adj(R, HRb, Rb);
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
  double r1vb = 0, r2vb = 0, r3vb = 0, rHb = 0, rcb = 0, absb = 0, sqLb = 0, sqRb = 0, cLb = 0, cRb = 0;
  double dUb[5] = {0, 0, 0, 0, 0};
  if (solver == RIEMANN_HLL || solver == RIEMANN_HLLE || solver == RIEMANN_HLLEM) {
    // signal speeds and which argument of each min / max the forward took
    const double Ssl0 = r1v - rc, Ssr0 = r1v + rc;
    double Ssl = Ssl0, Ssr = Ssr0, xl = 0.0, xr = 0.0, beta = 0.0;
    bool lRoe = true, rRoe = true;
    if (solver != RIEMANN_HLL) {
      beta = sqrt(0.5 * B.kappaM1 / B.kappa);
      xl = L.v1 - beta * cL;
      xr = R.v1 + beta * cR;
      lRoe = !(xl < Ssl0);
      rRoe = !(xr > Ssr0);
      Ssl = fmin(fmin(Ssl0, xl), 0.0);
      Ssr = fmax(fmax(Ssr0, xr), 0.0);
    }
    if (Ssl >= 0.0) { euler_flux_1d_adj(L, Fb, Lb); return; }
    if (Ssr <= 0.0) { euler_flux_1d_adj(R, Fb, Rb); return; }
    // F = (Ssr FL - Ssl FR + Ssl Ssr J) / (Ssr - Ssl), J = dU (HLLEM: minus the anti-diffusion of the contact and shear waves)
    double J[5] = {dU[0], dU[1], dU[2], dU[3], dU[4]};
    double delta = 0, A2 = 0, A3 = 0, A4 = 0, RoeDens = 0, K[5] = {0, 0, 0, 0, 0};
    if (solver == RIEMANN_HLLEM) {
      RoeDens = sqL * sqR;
      delta = rc / (rc + fabs(0.5 * (Ssl + Ssr)));
      A2 = (R.rho - L.rho) - (R.p - L.p) / (rc * rc);
      A3 = RoeDens * (R.v2 - L.v2);
      A4 = RoeDens * (R.v3 - L.v3);
      K[0] = A2; K[1] = r1v * A2; K[2] = r2v * A2 + A3; K[3] = r3v * A2 + A4; K[4] = 0.5 * absVel * A2 + r2v * A3 + r3v * A4;
      for (int v = 0; v < 5; ++v) J[v] -= delta * K[v];
    }
    const double sd = 1.0 / (Ssr - Ssl), ss = Ssl * Ssr;
    double FLb[5], FRb[5], Jb[5], sdb = 0, ssb = 0, Sslb = 0, Ssrb = 0;
    for (int v = 0; v < 5; ++v) {
      FLb[v] = Fb[v] * Ssr * sd;
      FRb[v] = -Fb[v] * Ssl * sd;
      Jb[v] = Fb[v] * ss * sd;
      sdb += Fb[v] * (Ssr * FL[v] - Ssl * FR[v] + ss * J[v]);
      ssb += Fb[v] * J[v] * sd;
      Ssrb += Fb[v] * FL[v] * sd;
      Sslb -= Fb[v] * FR[v] * sd;
    }
    Ssrb += ssb * Ssl - sdb * sd * sd;
    Sslb += ssb * Ssr + sdb * sd * sd;
    euler_flux_1d_adj(L, FLb, Lb);
    euler_flux_1d_adj(R, FRb, Rb);
    for (int v = 0; v < 5; ++v) dUb[v] += Jb[v];
    if (solver == RIEMANN_HLLEM) {
      double Kb[5], deltab = 0;
      for (int v = 0; v < 5; ++v) { Kb[v] = -delta * Jb[v]; deltab -= Jb[v] * K[v]; }
      const double A2b = Kb[0] + Kb[1] * r1v + Kb[2] * r2v + Kb[3] * r3v + Kb[4] * 0.5 * absVel;
      const double A3b = Kb[2] + Kb[4] * r2v, A4b = Kb[3] + Kb[4] * r3v;
      r1vb += Kb[1] * A2; r2vb += Kb[2] * A2 + Kb[4] * A3; r3vb += Kb[3] * A2 + Kb[4] * A4; absb += Kb[4] * 0.5 * A2;
      // delta = rc / (rc + |m|), m = (Ssl + Ssr) / 2
      const double m = 0.5 * (Ssl + Ssr), q = rc + fabs(m);
      rcb += deltab * fabs(m) / (q * q);
      const double mb = -deltab * rc / (q * q) * sgn1(m);
      Sslb += 0.5 * mb; Ssrb += 0.5 * mb;
      // A2 = drho - dp / rc^2, A3 = RoeDens dv2, A4 = RoeDens dv3, RoeDens = sqL sqR
      const double dp = R.p - L.p;
      Rb.rho += A2b; Lb.rho -= A2b;
      Rb.p -= A2b / (rc * rc); Lb.p += A2b / (rc * rc);
      rcb += A2b * 2.0 * dp / (rc * rc * rc);
      const double RoeDensb = A3b * (R.v2 - L.v2) + A4b * (R.v3 - L.v3);
      Rb.v2 += A3b * RoeDens; Lb.v2 -= A3b * RoeDens;
      Rb.v3 += A4b * RoeDens; Lb.v3 -= A4b * RoeDens;
      sqLb += RoeDensb * sqR; sqRb += RoeDensb * sqL;
    }
    jump_adj(L, R, dUb, Lb, Rb);
    // signal speeds (in the subsonic case neither min nor max took 0)
    if (lRoe) { r1vb += Sslb; rcb -= Sslb; } else { Lb.v1 += Sslb; cLb -= beta * Sslb; }
    if (rRoe) { r1vb += Ssrb; rcb += Ssrb; } else { Rb.v1 += Ssrb; cRb += beta * Ssrb; }
    sound_speed_adj(B, L, cL, cLb, Lb);
    sound_speed_adj(B, R, cR, cRb, Rb);
    roe_average_adj(B, L, R, HL, HR, sqL, sqR, ssq, r1v, r2v, r3v, rc, r1vb, r2vb, r3vb, rHb, rcb, absb, sqLb, sqRb, Lb, Rb, HLb, HRb);
    enthalpy_adj(L, HLb, Lb);
    enthalpy_adj(R, HRb, Rb);
    return;
  }
  // RoeL2 / RoeEntropyGShockFix: F = central - D/2 with the Roe-type dissipation D
  if (!split) {
    double Fh[5];
    for (int v = 0; v < 5; ++v) Fh[v] = 0.5 * Fb[v];
    euler_flux_1d_adj(L, Fh, Lb);
    euler_flux_1d_adj(R, Fh, Rb);
  } else {
    central_flux_adj(splitDG, B, L, R, HL, HR, Fb, Lb, Rb, HLb, HRb);
  }
  double Db[5];
  for (int v = 0; v < 5; ++v) Db[v] = -0.5 * Fb[v];
  RoeDissBars o;
  if (solver == RIEMANN_ROEL2) {
    const double a0 = r1v - rc, a1 = r1v, a4 = r1v + rc;
    const double P2 = dU[2] - r2v * dU[0], P3 = dU[3] - r3v * dU[0];
    const double d5 = dU[4] - P2 * r2v - P3 * r3v;
    const double sa = sqrt(absVel), sk = sqrt(B.kappa);
    const double Ma = sa / (rc * sk);
    const double d1 = dU[1] * Ma, d2 = dU[2] * Ma, d3 = dU[3] * Ma;
    const double src = 1.0 / rc;
    double A[5];
    A[2] = d2 - r2v * dU[0];
    A[3] = d3 - r3v * dU[0];
    const double Y = dU[0] * (rH - r1v * r1v) - d5 + r1v * d1;
    A[1] = B.kappaM1 * (src * src) * Y;
    const double X = dU[0] * (r1v + rc) - d1 - rc * A[1];
    A[0] = 0.5 * src * X;
    A[4] = dU[0] - A[0] - A[1];
    const double e0 = fabs(a0), e1 = fabs(a1), e4 = fabs(a4);
    roe_dissipation_adj(Db, A, e0, e1, e4, a0, a4, r1v, r2v, r3v, rH, rc, absVel, o, r1vb, r2vb, r3vb, rHb, rcb, absb);
    double a0b = o.a0 + o.e0 * sgn1(a0), a1b = o.e1 * sgn1(a1), a4b = o.a4 + o.e4 * sgn1(a4);
    double A0b = o.A[0], A1b = o.A[1], A2b = o.A[2], A3b = o.A[3], A4b = o.A[4];
    double d1b = 0, d5b = 0, srcb = 0, Mab = 0;
    // A4 = dU0 - A0 - A1
    dUb[0] += A4b; A0b -= A4b; A1b -= A4b;
    // A0 = src X / 2
    srcb += A0b * 0.5 * X;
    const double Xb = A0b * 0.5 * src;
    dUb[0] += Xb * (r1v + rc); r1vb += Xb * dU[0]; rcb += Xb * (dU[0] - A[1]); d1b -= Xb; A1b -= Xb * rc;
    // A1 = kappaM1 src^2 Y
    srcb += A1b * B.kappaM1 * 2.0 * src * Y;
    const double Yb = A1b * B.kappaM1 * src * src;
    dUb[0] += Yb * (rH - r1v * r1v); rHb += Yb * dU[0]; r1vb += Yb * (d1 - 2.0 * r1v * dU[0]); d5b -= Yb; d1b += Yb * r1v;
    rcb -= srcb * src * src;
    // A2 = Ma dU2 - r2v dU0, A3 = Ma dU3 - r3v dU0, d1 = Ma dU1
    Mab += A2b * dU[2] + A3b * dU[3] + d1b * dU[1];
    dUb[2] += A2b * Ma; r2vb -= A2b * dU[0]; dUb[0] -= A2b * r2v;
    dUb[3] += A3b * Ma; r3vb -= A3b * dU[0]; dUb[0] -= A3b * r3v;
    dUb[1] += d1b * Ma;
    // d5 = dU4 - P2 r2v - P3 r3v, P2 = dU2 - r2v dU0, P3 = dU3 - r3v dU0
    dUb[4] += d5b;
    const double P2b = -d5b * r2v, P3b = -d5b * r3v;
    r2vb -= d5b * P2; r3vb -= d5b * P3;
    dUb[2] += P2b; r2vb -= P2b * dU[0]; dUb[0] -= P2b * r2v;
    dUb[3] += P3b; r3vb -= P3b * dU[0]; dUb[0] -= P3b * r3v;
    // Ma = sqrt(absVel) / (rc sqrt(kappa))
    if (sa > 0.0) absb += Mab / (rc * sk) / (2.0 * sa);
    rcb -= Mab * Ma / rc;
    jump_adj(L, R, dUb, Lb, Rb);
    r1vb += a0b + a1b + a4b;
    rcb += a4b - a0b;
  } else {  // RoeEntropyGShockFix
    const double sg = r1v < 0.0 ? -1.0 : 1.0;
    const double lim = rc / B.riemannPhi, ar1 = fabs(r1v);
    const bool limTaken = !(lim < ar1);  // fmax(lim, |r1v|): the first argument on a tie
    const double am = sg * fmax(lim, ar1);
    const double a0 = am - rc, a1 = am, a4 = am + rc;
    const double RoeDens = sqL * sqR;
    const double dr = R.rho - L.rho, du = R.v1 - L.v1, dv = R.v2 - L.v2, dw = R.v3 - L.v3, dp = R.p - L.p;
    const double tmp = 0.5 / (rc * rc);
    const double rdc = RoeDens * rc * du;
    double A[5];
    A[0] = tmp * (dp - rdc);
    A[1] = dr - dp * (2.0 * tmp);
    A[2] = RoeDens * dv;
    A[3] = RoeDens * dw;
    A[4] = tmp * (dp + rdc);
    auto fix = [](double a, double al, double ar) {
      const double da = fmax(0.0, fmax(a - al, ar - a));
      return fabs(a) < da ? 0.5 * (a * a / da + da) : fabs(a);
    };
    const double e0 = fix(a0, L.v1 - cL, R.v1 - cR), e1 = fix(a1, L.v1, R.v1), e4 = fix(a4, L.v1 + cL, R.v1 + cR);
    roe_dissipation_adj(Db, A, e0, e1, e4, a0, a4, r1v, r2v, r3v, rH, rc, absVel, o, r1vb, r2vb, r3vb, rHb, rcb, absb);
    double a0b = o.a0, a1b = 0.0, a4b = o.a4, alb = 0, arb = 0;
    entropy_fix_adj(a0, L.v1 - cL, R.v1 - cR, o.e0, a0b, alb, arb);
    Lb.v1 += alb; cLb -= alb; Rb.v1 += arb; cRb -= arb;
    alb = arb = 0;
    entropy_fix_adj(a1, L.v1, R.v1, o.e1, a1b, alb, arb);
    Lb.v1 += alb; Rb.v1 += arb;
    alb = arb = 0;
    entropy_fix_adj(a4, L.v1 + cL, R.v1 + cR, o.e4, a4b, alb, arb);
    Lb.v1 += alb; cLb += alb; Rb.v1 += arb; cRb += arb;
    // strengths
    const double A0b = o.A[0], A1b = o.A[1], A2b = o.A[2], A3b = o.A[3], A4b = o.A[4];
    const double tmpb = A0b * (dp - rdc) - 2.0 * A1b * dp + A4b * (dp + rdc);
    const double dpb = (A0b - 2.0 * A1b + A4b) * tmp;
    const double rdcb = (A4b - A0b) * tmp;
    const double RoeDensb = A2b * dv + A3b * dw + rdcb * rc * du;
    rcb += rdcb * RoeDens * du - tmpb / (rc * rc * rc);
    const double dub = rdcb * RoeDens * rc;
    Rb.rho += A1b; Lb.rho -= A1b;
    Rb.v1 += dub; Lb.v1 -= dub;
    Rb.v2 += A2b * RoeDens; Lb.v2 -= A2b * RoeDens;
    Rb.v3 += A3b * RoeDens; Lb.v3 -= A3b * RoeDens;
    Rb.p += dpb; Lb.p -= dpb;
    sqLb += RoeDensb * sqR; sqRb += RoeDensb * sqL;
    // eigenvalues a0 = am - rc, a1 = am, a4 = am + rc; am = sg max(rc / phi, |r1v|)
    const double amb = a0b + a1b + a4b;
    rcb += a4b - a0b;
    if (limTaken) rcb += amb * sg / B.riemannPhi;
    else r1vb += amb;  // sg |r1v| = r1v
  }
  sound_speed_adj(B, L, cL, cLb, Lb);
  sound_speed_adj(B, R, cR, cRb, Rb);
  roe_average_adj(B, L, R, HL, HR, sqL, sqR, ssq, r1v, r2v, r3v, rc, r1vb, r2vb, r3vb, rHb, rcb, absb, sqLb, sqRb, Lb, Rb, HLb, HRb);
  enthalpy_adj(L, HLb, Lb);
  enthalpy_adj(R, HRb, Rb);
}

// eos.f90:PRESSURE_RIEMANN: adds the bars of rho, vn, p for the bar of the boundary pressure
FG_HD void pressure_riemann_adj(const Basis& B, double rho, double vn, double p, double pbb, double& rhob, double& vnb, double& pb) {
  if (vn <= 0.0) {
    const double c = sqrt(B.kappa * p / rho);
    const double raw = 1.0 + 0.5 * B.kappaM1 * vn / c;
    const double base = fmax(0.0001, raw);
    pb += pbb * pow(base, B.kappaFac);
    const double baseb = pbb * p * B.kappaFac * pow(base, B.kappaFac - 1.0);
    if (raw >= 0.0001) {
      vnb += baseb * 0.5 * B.kappaM1 / c;
      const double cb = -baseb * 0.5 * B.kappaM1 * vn / (c * c);
      pb += cb * B.kappa / (2.0 * c * rho);
      rhob -= cb * B.kappa * p / (2.0 * c * rho * rho);
    }
    return;
  }
  const double ar = 2.0 * B.sKappaP1 / rho;
  const double br = B.kappaM1 * B.sKappaP1 * p;
  const double Z = vn * vn + 4.0 * ar * (p + br);
  const double Q = sqrt(Z);
  // pb = p + vn / ar * 0.5 * (vn + Q)
  const double K = vn / ar * 0.5;
  pb += pbb;
  const double Kb = pbb * (vn + Q);
  vnb += pbb * K;
  const double Qb = pbb * K;
  vnb += Kb * 0.5 / ar;
  double arb = -Kb * 0.5 * vn / (ar * ar);
  const double Zb = Qb / (2.0 * Q);
  vnb += 2.0 * vn * Zb;
  arb += 4.0 * (p + br) * Zb;
  pb += 4.0 * ar * Zb;
  const double brb = 4.0 * ar * Zb;
  pb += brb * B.kappaM1 * B.sKappaP1;
  rhob -= arb * 2.0 * B.sKappaP1 / (rho * rho);
}

// Two-point volume flux of the split form (split_pair_flux, PI or SD) between the per-node inputs qa, qb
// (q0, u, v, w, q4, q5) with metric sum ms: given Gb[5], adds the bars of both nodes' inputs. PI depends on
// the sums of the inputs only, so both nodes get the same bars.
FG_HD void split_pair_flux_adj(bool pi, const double* qa, const double* qb, const double* ms, const double* Gb, double* qab, double* qbb) {
  if (pi) {
    const double rs = qa[0] + qb[0], us = qa[1] + qb[1], vs = qa[2] + qb[2], ws = qa[3] + qb[3], hs = qa[5] + qb[5];
    const double qs = us * ms[0] + vs * ms[1] + ws * ms[2];
    const double A = rs * qs;
    const double Ab = Gb[0] + Gb[1] * us + Gb[2] * vs + Gb[3] * ws + Gb[4] * hs;
    const double qsb = Ab * rs;
    const double bar[6] = {Ab * qs, Gb[1] * A + qsb * ms[0], Gb[2] * A + qsb * ms[1], Gb[3] * A + qsb * ms[2],
                           Gb[1] * ms[0] + Gb[2] * ms[1] + Gb[3] * ms[2], Gb[4] * A};
#pragma unroll
    for (int c = 0; c < 6; ++c) { qab[c] += bar[c]; qbb[c] += bar[c]; }
    return;
  }
  const double pb = Gb[1] * ms[0] + Gb[2] * ms[1] + Gb[3] * ms[2];
  const double* q[2] = {qa, qb};
  double* o[2] = {qab, qbb};
#pragma unroll
  for (int side = 0; side < 2; ++side) {
    const double* s = q[side];
    // G0 = sum m q, G1..3 = sum m q u_c + p_s ms_c, G4 = sum h q (q = u . ms, m = rho)
    const double qn = s[1] * ms[0] + s[2] * ms[1] + s[3] * ms[2];
    const double mq = s[0] * qn;
    const double mqb = Gb[0] + Gb[1] * s[1] + Gb[2] * s[2] + Gb[3] * s[3];
    const double qnb = mqb * s[0] + Gb[4] * s[5];
    o[side][0] += mqb * qn;
    o[side][1] += qnb * ms[0] + Gb[1] * mq;
    o[side][2] += qnb * ms[1] + Gb[2] * mq;
    o[side][3] += qnb * ms[2] + Gb[3] * mq;
    o[side][4] += pb;
    o[side][5] += Gb[4] * qn;
  }
}

// split_node_inputs (PI or SD) transposed to the bars of the face-state fields rho, u, v, w, p, E, 1/rho
// (PI: q4 = 4p, q5 = (E+p)/rho; SD: q4 = p, q5 = E+p); adds into fb[FS_NF]
FG_HD void split_inputs_to_face_adj(bool pi, double E, double p, double srho, const double* qb, double* fb) {
  fb[FS_RHO] += qb[0];
  fb[FS_U] += qb[1]; fb[FS_V] += qb[2]; fb[FS_W] += qb[3];
  if (pi) {
    fb[FS_P] += 4.0 * qb[4] + qb[5] * srho;
    fb[FS_E] += qb[5] * srho;
    fb[FS_SRHO] += qb[5] * (E + p);
  } else {
    fb[FS_P] += qb[4] + qb[5];
    fb[FS_E] += qb[5];
  }
}

// split_node_inputs transposed (every split form): given the bars qb[6] of (q0, u, v, w, q4, q5), adds the bars of the
// point's rho, u, v, w, p, E and 1/rho, each an independent input
FG_HD void split_node_inputs_adj(int sd, double rho, double u, double v, double w, double p, double E, double srho, const double* qb,
                                 double& rhob, double& ub, double& vb, double& wb, double& pb, double& Eb, double& srhob) {
  ub += qb[1]; vb += qb[2]; wb += qb[3];
  if (sd == SPLIT_IR) {  // q0 = sqrt(rho / p), q4 = sqrt(rho p)
    const double z1 = sqrt(rho / p), z5 = sqrt(rho * p);
    rhob += qb[0] * z1 / (2.0 * rho) + qb[4] * z5 / (2.0 * rho);
    pb += -qb[0] * z1 / (2.0 * p) + qb[4] * z5 / (2.0 * p);
    return;
  }
  rhob += qb[0];
  switch (sd) {
    case SPLIT_CH: rhob += qb[4] * 0.5 / p; pb -= qb[4] * 0.5 * rho / (p * p); break;  // q4 = rho / (2p)
    case SPLIT_PI: pb += 4.0 * qb[4] + qb[5] * srho; Eb += qb[5] * srho; srhob += qb[5] * (E + p); break;
    case SPLIT_DU: pb += 2.0 * qb[4] + qb[5]; Eb += qb[5]; break;
    case SPLIT_KG: pb += 4.0 * qb[4]; Eb += qb[5] * srho; srhob += qb[5] * E; break;
    case SPLIT_MO:  // q4 = 2p, q5 = 2 (E - rho |v|^2 / 2 + p)
      pb += 2.0 * qb[4] + 2.0 * qb[5]; Eb += 2.0 * qb[5];
      rhob -= qb[5] * (u * u + v * v + w * w);
      ub -= 2.0 * qb[5] * rho * u; vb -= 2.0 * qb[5] * rho * v; wb -= 2.0 * qb[5] * rho * w;
      break;
    default: pb += qb[4] + qb[5]; Eb += qb[5]; break;  // SD
  }
}

// split_pair_flux_gen transposed: given Gb[5], adds the bars of both nodes' inputs (q0, u, v, w, q4, q5); the metric sum ms
// is not an input. LM: CH and IR too (their logarithmic means); without it SD, PI, MO, DU, KG only, which keeps the
// volume adjoint's registers for those forms where they were
template <bool LM = true>
FG_HD void split_pair_flux_gen_adj(int sd, const Basis& B, const double* qa, const double* qb, const double* ms, const double* Gb, double* qab,
                                   double* qbb) {
  if (sd == SPLIT_PI || sd == SPLIT_SD) {
    split_pair_flux_adj(sd == SPLIT_PI, qa, qb, ms, Gb, qab, qbb);
    return;
  }
  const double us = qa[1] + qb[1], vs = qa[2] + qb[2], ws = qa[3] + qb[3];
  const double qs = us * ms[0] + vs * ms[1] + ws * ms[2];
  const double psb0 = Gb[1] * ms[0] + Gb[2] * ms[1] + Gb[3] * ms[2];
  double usb = 0.0, vsb = 0.0, wsb = 0.0;
  if (LM && sd == SPLIT_CH) {
    // q4 = beta = rho / (2p); rhoLog, betaLog the logarithmic means, pHat = (ra + rb) / (2 (beta_a + beta_b)),
    // H = sKappaM1 / (2 betaLog) + pHat / rhoLog + (u_a . u_b) / 2, A = rhoLog qs; G0 = A, G1..3 = A/2 (u_a + u_b)_c + 2 pHat ms_c,
    // G4 = A H
    const double rhoLog = log_mean(qa[0], qb[0]), betaLog = log_mean(qa[4], qb[4]);
    const double Rs = qa[0] + qb[0], Bs = qa[4] + qb[4];
    const double pHat = 0.5 * Rs / Bs;
    const double H = 0.5 * B.sKappaM1 / betaLog + pHat / rhoLog + 0.5 * (qa[1] * qb[1] + qa[2] * qb[2] + qa[3] * qb[3]);
    const double A = rhoLog * qs;
    const double Ab = Gb[0] + Gb[4] * H + 0.5 * (Gb[1] * us + Gb[2] * vs + Gb[3] * ws);
    usb = 0.5 * Gb[1] * A; vsb = 0.5 * Gb[2] * A; wsb = 0.5 * Gb[3] * A;
    const double Hb = Gb[4] * A;
    double pHatb = 2.0 * psb0 + Hb / rhoLog;
    const double rhoLogb = Ab * qs - Hb * pHat / (rhoLog * rhoLog);
    const double betaLogb = -Hb * 0.5 * B.sKappaM1 / (betaLog * betaLog);
#pragma unroll
    for (int c = 0; c < 3; ++c) { qab[1 + c] += 0.5 * Hb * qb[1 + c]; qbb[1 + c] += 0.5 * Hb * qa[1 + c]; }
    const double qsb = Ab * rhoLog;
    usb += qsb * ms[0]; vsb += qsb * ms[1]; wsb += qsb * ms[2];
    qab[0] += pHatb * 0.5 / Bs; qbb[0] += pHatb * 0.5 / Bs;
    qab[4] -= pHatb * pHat / Bs; qbb[4] -= pHatb * pHat / Bs;
    log_mean_adj(qa[0], qb[0], rhoLogb, qab[0], qbb[0]);
    log_mean_adj(qa[4], qb[4], betaLogb, qab[4], qbb[4]);
  } else if (LM && sd == SPLIT_IR) {
    // q0 = z1 = sqrt(rho / p), q4 = z5 = sqrt(rho p); rhoHat = (z1a + z1b) z5Log / 2, pHat = (z5a + z5b) / (z1a + z1b),
    // p2Hat = ((kappa + 1) z5Log / z1Log + kappaM1 pHat) / (2 kappa), uH = (z1a u_a + z1b u_b) / (z1a + z1b),
    // hH = kappa p2Hat / (rhoHat kappaM1) + |uH|^2 / 2, A = rhoHat uH . ms; G0 = A, G1..3 = A uH_c + pHat ms_c, G4 = A hH
    const double z1Log = log_mean(qa[0], qb[0]), z5Log = log_mean(qa[4], qb[4]);
    const double z1s = qa[0] + qb[0];
    const double rhoHat = 0.5 * z1s * z5Log;
    const double pHat = (qa[4] + qb[4]) / z1s;
    const double p2Hat = 0.5 / B.kappa * ((B.kappa + 1.0) * z5Log / z1Log + B.kappaM1 * pHat);
    double uH[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) uH[c] = (qa[0] * qa[1 + c] + qb[0] * qb[1 + c]) / z1s;
    const double hH = B.kappa * p2Hat / (rhoHat * B.kappaM1) + 0.5 * (uH[0] * uH[0] + uH[1] * uH[1] + uH[2] * uH[2]);
    const double qH = uH[0] * ms[0] + uH[1] * ms[1] + uH[2] * ms[2];
    const double A = rhoHat * qH;
    const double Ab = Gb[0] + Gb[1] * uH[0] + Gb[2] * uH[1] + Gb[3] * uH[2] + Gb[4] * hH;
    double uHb[3] = {Gb[1] * A, Gb[2] * A, Gb[3] * A};
    double pHatb = psb0;
    const double hHb = Gb[4] * A;
    double p2Hatb = hHb * B.kappa / (rhoHat * B.kappaM1);
    double rhoHatb = -hHb * B.kappa * p2Hat / (rhoHat * rhoHat * B.kappaM1) + Ab * qH;
    const double qHb = Ab * rhoHat;
#pragma unroll
    for (int c = 0; c < 3; ++c) uHb[c] += hHb * uH[c] + qHb * ms[c];
    double z5Logb = p2Hatb * 0.5 / B.kappa * (B.kappa + 1.0) / z1Log;
    double z1Logb = -p2Hatb * 0.5 / B.kappa * (B.kappa + 1.0) * z5Log / (z1Log * z1Log);
    pHatb += p2Hatb * 0.5 * B.kappaM1 / B.kappa;
    double z1sb = -pHatb * pHat / z1s;
    qab[4] += pHatb / z1s; qbb[4] += pHatb / z1s;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      qab[0] += uHb[c] * qa[1 + c] / z1s; qbb[0] += uHb[c] * qb[1 + c] / z1s;
      qab[1 + c] += uHb[c] * qa[0] / z1s; qbb[1 + c] += uHb[c] * qb[0] / z1s;
      z1sb -= uHb[c] * uH[c] / z1s;
    }
    z1sb += rhoHatb * 0.5 * z5Log;
    z5Logb += rhoHatb * 0.5 * z1s;
    qab[0] += z1sb; qbb[0] += z1sb;
    log_mean_adj(qa[0], qb[0], z1Logb, qab[0], qbb[0]);
    log_mean_adj(qa[4], qb[4], z5Logb, qab[4], qbb[4]);
    return;
  } else if (sd == SPLIT_DU) {
    // G0 = (ra + rb) qs, G1..3 = (ra u_a + rb u_b)_c qs + ps ms_c, G4 = (ha + hb) qs
    const double Rs = qa[0] + qb[0], Hs = qa[5] + qb[5];
    const double M[3] = {qa[0] * qa[1] + qb[0] * qb[1], qa[0] * qa[2] + qb[0] * qb[2], qa[0] * qa[3] + qb[0] * qb[3]};
    const double qsb = Gb[0] * Rs + Gb[1] * M[0] + Gb[2] * M[1] + Gb[3] * M[2] + Gb[4] * Hs;
    const double Rb = Gb[0] * qs, Hsb = Gb[4] * qs;
    qab[0] += Rb; qbb[0] += Rb;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const double Mb = Gb[1 + c] * qs;
      qab[0] += Mb * qa[1 + c]; qbb[0] += Mb * qb[1 + c];
      qab[1 + c] += Mb * qa[0]; qbb[1 + c] += Mb * qb[0];
    }
    qab[4] += psb0; qbb[4] += psb0;
    qab[5] += Hsb; qbb[5] += Hsb;
    usb = qsb * ms[0]; vsb = qsb * ms[1]; wsb = qsb * ms[2];
  } else if (sd == SPLIT_KG) {
    // A = (ra + rb) qs; G0 = A, G1..3 = A (u_a + u_b)_c + ps ms_c, G4 = A (ha + hb) + ps qs / 2
    const double Rs = qa[0] + qb[0], A = Rs * qs, Hs = qa[5] + qb[5], ps = qa[4] + qb[4];
    const double Ab = Gb[0] + Gb[1] * us + Gb[2] * vs + Gb[3] * ws + Gb[4] * Hs;
    usb = Gb[1] * A; vsb = Gb[2] * A; wsb = Gb[3] * A;
    const double Hsb = Gb[4] * A;
    const double psb = psb0 + Gb[4] * 0.5 * qs;
    const double qsb = Ab * Rs + Gb[4] * 0.5 * ps;
    const double Rb = Ab * qs;
    usb += qsb * ms[0]; vsb += qsb * ms[1]; wsb += qsb * ms[2];
    qab[0] += Rb; qbb[0] += Rb;
    qab[4] += psb; qbb[4] += psb;
    qab[5] += Hsb; qbb[5] += Hsb;
  } else {  // MO: qn = u . ms per node, mq = ra qn_a + rb qn_b; G0 = mq, G1..3 = mq (u_a + u_b)_c + ps ms_c,
            // G4 = ha qn_a + hb qn_b + mq (u_a . u_b)
    const double qna = qa[1] * ms[0] + qa[2] * ms[1] + qa[3] * ms[2], qnb = qb[1] * ms[0] + qb[2] * ms[1] + qb[3] * ms[2];
    const double mq = qa[0] * qna + qb[0] * qnb;
    const double vv = qa[1] * qb[1] + qa[2] * qb[2] + qa[3] * qb[3];
    const double mqb = Gb[0] + Gb[1] * us + Gb[2] * vs + Gb[3] * ws + Gb[4] * vv;
    usb = Gb[1] * mq; vsb = Gb[2] * mq; wsb = Gb[3] * mq;
    const double vvb = Gb[4] * mq;
    qab[5] += Gb[4] * qna; qbb[5] += Gb[4] * qnb;
    const double qnab = Gb[4] * qa[5] + mqb * qa[0], qnbb = Gb[4] * qb[5] + mqb * qb[0];
    qab[0] += mqb * qna; qbb[0] += mqb * qnb;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      qab[1 + c] += vvb * qb[1 + c] + qnab * ms[c];
      qbb[1 + c] += vvb * qa[1 + c] + qnbb * ms[c];
    }
    qab[4] += psb0; qbb[4] += psb0;
  }
  qab[1] += usb; qbb[1] += usb;
  qab[2] += vsb; qbb[2] += vsb;
  qab[3] += wsb; qbb[3] += wsb;
}

// the entropy-variable transforms of k_prep, in place on one point (the adjoint's linearisation point)
FG_HD void cons_to_entropy(const Basis& B, double* u) {
  const double srho = 1.0 / u[0];
  const double vx = u[1] * srho, vy = u[2] * srho, vz = u[3] * srho;
  const double p = B.kappaM1 * (u[4] - 0.5 * (u[1] * vx + u[2] * vy + u[3] * vz));
  const double sEnt = log(p) - B.kappa * log(u[0]);
  const double rho_p = u[0] / p;
  u[0] = (B.kappa - sEnt) * B.sKappaM1 - rho_p * 0.5 * (vx * vx + vy * vy + vz * vz);
  u[1] = rho_p * vx; u[2] = rho_p * vy; u[3] = rho_p * vz;
  u[4] = -rho_p;
}
FG_HD void entropy_to_cons(const Basis& B, double* c) {
  const double w0 = c[0] * B.kappaM1, w1 = c[1] * B.kappaM1, w2 = c[2] * B.kappaM1, w3 = c[3] * B.kappaM1, w4 = c[4] * B.kappaM1;
  const double ekin = 0.5 * (w1 * w1 + w2 * w2 + w3 * w3) / w4;
  const double sEnt = B.kappa - w0 + ekin;
  const double rhoe = exp(B.logEntC - B.kappa_kappaM1 * log(-w4) - sEnt * B.sKappaM1);
  c[0] = -rhoe * w4;
  c[1] = rhoe * w1; c[2] = rhoe * w2; c[3] = rhoe * w3;
  c[4] = rhoe * (1.0 - ekin);
}

// eos.f90:ConsToEntropy (the form of k_prep): W =((kappa - s)/(kappa-1) - rho/p |v|^2/2, rho/p v, -rho/p) with
// s = ln p - kappa ln rho. Given Wb[5], adds the conservative bars into Ub[5].
FG_HD void cons_to_entropy_adj(const Basis& B, const double* U, const double* Wb, double* Ub) {
  const double srho = 1.0 / U[0];
  const double vx = U[1] * srho, vy = U[2] * srho, vz = U[3] * srho;
  const double p = B.kappaM1 * (U[4] - 0.5 * (U[1] * vx + U[2] * vy + U[3] * vz));
  const double rho_p = U[0] / p;
  const double v2 = vx * vx + vy * vy + vz * vz;
  const double rpb = -Wb[0] * 0.5 * v2 + Wb[1] * vx + Wb[2] * vy + Wb[3] * vz - Wb[4];
  const double sb = -Wb[0] * B.sKappaM1;
  const double vxb = (Wb[1] - Wb[0] * vx) * rho_p, vyb = (Wb[2] - Wb[0] * vy) * rho_p, vzb = (Wb[3] - Wb[0] * vz) * rho_p;
  // s = ln p - kappa ln rho, rho_p = rho / p
  const double pb = sb / p - rpb * rho_p / p;
  const double rhob = -B.kappa * sb * srho + rpb / p;
  cons_to_prim_adj(B, U, 0.0, vxb, vyb, vzb, pb, 0.0, rhob, 0.0, Ub);
}

// eos.f90:EntropyToCons (the form of k_prep, one exponential): given the entropy variables W[5] of a face point
// and the bars cb[5] of the conservative result, adds the bars of W into Wb[5]
FG_HD void entropy_to_cons_adj(const Basis& B, const double* W, const double* cb, double* Wb) {
  const double w0 = W[0] * B.kappaM1, w1 = W[1] * B.kappaM1, w2 = W[2] * B.kappaM1, w3 = W[3] * B.kappaM1, w4 = W[4] * B.kappaM1;
  const double ekin = 0.5 * (w1 * w1 + w2 * w2 + w3 * w3) / w4;
  const double sEnt = B.kappa - w0 + ekin;
  const double rhoe = exp(B.logEntC - B.kappa_kappaM1 * log(-w4) - sEnt * B.sKappaM1);
  // c = rhoe (-w4, w1, w2, w3, 1 - ekin)
  const double rhoeb = -cb[0] * w4 + cb[1] * w1 + cb[2] * w2 + cb[3] * w3 + cb[4] * (1.0 - ekin);
  const double Xb = rhoeb * rhoe;  // rhoe = exp(X)
  const double sEntb = -Xb * B.sKappaM1;
  const double ekinb = -cb[4] * rhoe + sEntb;
  double w1b = cb[1] * rhoe + ekinb * w1 / w4;
  double w2b = cb[2] * rhoe + ekinb * w2 / w4;
  double w3b = cb[3] * rhoe + ekinb * w3 / w4;
  double w4b = -cb[0] * rhoe - Xb * B.kappa_kappaM1 / w4 - ekinb * ekin / w4;
  const double w0b = -sEntb;
  Wb[0] += w0b * B.kappaM1; Wb[1] += w1b * B.kappaM1; Wb[2] += w2b * B.kappaM1; Wb[3] += w3b * B.kappaM1; Wb[4] += w4b * B.kappaM1;
}

}  // namespace fg
