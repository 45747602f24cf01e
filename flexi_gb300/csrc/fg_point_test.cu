// flexi_gb300 -- host-side harness for the point-wise physics and its adjoints (built as libfgpoint.so).
//
// Exposes the __host__ __device__ functions of fg_common.cuh and fg_adjoint_point.cuh through plain C
// entry points so that the CPU test suite can check every transposed Jacobian against central finite
// differences of the very same forward code. Not part of the solver library.
#include <cmath>

#include "fg_adjoint_point.cuh"

using namespace fg;

namespace {
Basis gas(double kappa, double R) {
  Basis B{};
  B.kappa = kappa; B.kappaM1 = kappa - 1.0; B.sKappaM1 = 1.0 / (kappa - 1.0);
  B.Rgas = R; B.sR = 1.0 / R;
  B.kappaFac = 2.0 * kappa / (kappa - 1.0);
  B.sKappaP1 = 1.0 / (kappa + 1.0);
  B.logEntC = std::log(kappa - 1.0) / (kappa - 1.0);
  B.kappa_kappaM1 = kappa / (kappa - 1.0);
  return B;
}
RotState rs(const double* a) { RotState S; S.rho = a[0]; S.srho = a[1]; S.E = a[2]; S.p = a[3]; S.v1 = a[4]; S.v2 = a[5]; S.v3 = a[6]; return S; }
void rs_out(const RotState& S, double* a) { a[0] = S.rho; a[1] = S.srho; a[2] = S.E; a[3] = S.p; a[4] = S.v1; a[5] = S.v2; a[6] = S.v3; }
}  // namespace

extern "C" {

// U[5] -> (srho, u, v, w, p, T)
void fgpt_cons_to_prim(double kappa, double R, const double* U, double* out) {
  const Basis B = gas(kappa, R);
  const double srho = 1.0 / U[0];
  const double vx = U[1] * srho, vy = U[2] * srho, vz = U[3] * srho;
  const double p = B.kappaM1 * (U[4] - 0.5 * (U[1] * vx + U[2] * vy + U[3] * vz));
  out[0] = srho; out[1] = vx; out[2] = vy; out[3] = vz; out[4] = p; out[5] = p * srho * B.sR;
}
// bar[8] = bars of (srho, u, v, w, p, T, rho_direct, E_direct) -> Ub[5]
void fgpt_cons_to_prim_adj(double kappa, double R, const double* U, const double* bar, double* Ub) {
  const Basis B = gas(kappa, R);
  for (int v = 0; v < 5; ++v) Ub[v] = 0.0;
  cons_to_prim_adj(B, U, bar[0], bar[1], bar[2], bar[3], bar[4], bar[5], bar[6], bar[7], Ub);
}

// x = (u, v, w, g[12], mu), m[3]: F[1..4] -> out[4]
void fgpt_visc(double lamFac, const double* x, const double* m, double* out) {
  double F[5];
  visc_flux_dir(x[15], x[15] * lamFac, x[0], x[1], x[2], x + 3, m[0], m[1], m[2], F);
  for (int v = 0; v < 4; ++v) out[v] = F[1 + v];
}
void fgpt_visc_adj(double lamFac, const double* x, const double* m, const double* Fb4, double* xb) {
  double Fb[5] = {0.0, Fb4[0], Fb4[1], Fb4[2], Fb4[3]};
  for (int c = 0; c < 16; ++c) xb[c] = 0.0;
  visc_flux_dir_adj(x[15], lamFac, x[0], x[1], x[2], x + 3, m[0], m[1], m[2], Fb, xb[0], xb[1], xb[2], xb + 3, xb[15]);
}

// x = (u, v, w, g[12], mu): physical viscous fluxes f, g, h components 1..4 -> out[12]
void fgpt_visc_phys(double lamFac, const double* x, double* out) {
  const double e[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
  for (int d = 0; d < 3; ++d) {
    double F[5];
    visc_flux_dir(x[15], x[15] * lamFac, x[0], x[1], x[2], x + 3, e[d][0], e[d][1], e[d][2], F);
    for (int v = 0; v < 4; ++v) out[4 * d + v] = F[1 + v];
  }
}
void fgpt_visc_phys_adj(double lamFac, const double* x, const double* yb, double* xb) {
  double fb[5] = {0, yb[0], yb[1], yb[2], yb[3]}, gyb[5] = {0, yb[4], yb[5], yb[6], yb[7]}, hb[5] = {0, yb[8], yb[9], yb[10], yb[11]};
  for (int c = 0; c < 16; ++c) xb[c] = 0.0;
  visc_flux_phys_adj(x[15], lamFac, x[0], x[1], x[2], x + 3, fb, gyb, hb, xb[0], xb[1], xb[2], xb + 3, xb[15]);
}

// L[7], R[7] = (rho, srho, E, p, v1, v2, v3) -> F[5]
void fgpt_riemann(int solver, int splitDG, double kappa, double R, const double* L, const double* Rr, double* F) {
  const Basis B = gas(kappa, R);
  riemann_rotated(solver, splitDG, B, rs(L), rs(Rr), F);
}
void fgpt_riemann_adj(int solver, int splitDG, double kappa, double R, const double* L, const double* Rr, const double* Fb, double* Lb, double* Rb) {
  const Basis B = gas(kappa, R);
  RotState lb, rb;
  rot_zero(lb); rot_zero(rb);
  riemann_rotated_adj(solver, splitDG, B, rs(L), rs(Rr), Fb, lb, rb);
  rs_out(lb, Lb); rs_out(rb, Rb);
}

// every Riemann solver with any SplitDG (-1: weak form): riemann_rotated_more
void fgpt_riemann_more(int solver, int splitDG, double kappa, double R, double riemannPhi, const double* L, const double* Rr, double* F) {
  Basis B = gas(kappa, R);
  B.riemannPhi = riemannPhi;
  riemann_rotated_more(solver, splitDG, B, rs(L), rs(Rr), F);
}
void fgpt_riemann_more_adj(int solver, int splitDG, double kappa, double R, double riemannPhi, const double* L, const double* Rr, const double* Fb,
                           double* Lb, double* Rb) {
  Basis B = gas(kappa, R);
  B.riemannPhi = riemannPhi;
  RotState lb, rb;
  rot_zero(lb); rot_zero(rb);
  riemann_rotated_more_adj(solver, splitDG, B, rs(L), rs(Rr), Fb, lb, rb);
  rs_out(lb, Lb); rs_out(rb, Rb);
}
// two-point volume flux of the split form as the split kernels form it: per-node inputs, pair flux with the metric sum,
// constant factors; uR/u conservative (5), pR/p primitive (rho, u, v, w, p, T), mR/m metric vectors (3)
void fgpt_split_volume(int splitDG, double kappa, const double* uR, const double* pR, const double* u, const double* p, const double* mR,
                       const double* m, double* F) {
  Basis B = gas(kappa, 1.0);
  double qa[6], qb[6];
  qa[1] = pR[1]; qa[2] = pR[2]; qa[3] = pR[3];
  qb[1] = p[1]; qb[2] = p[2]; qb[3] = p[3];
  split_node_inputs(splitDG, uR[0], pR[1], pR[2], pR[3], pR[4], uR[4], 1.0 / uR[0], qa[0], qa[4], qa[5]);
  split_node_inputs(splitDG, u[0], p[1], p[2], p[3], p[4], u[4], 1.0 / u[0], qb[0], qb[4], qb[5]);
  double G[5], f0, f1;
  split_pair_flux_gen(splitDG, B, qa[0], qa[1], qa[2], qa[3], qa[4], qa[5], qb[0], qb[1], qb[2], qb[3], qb[4], qb[5], mR[0] + m[0],
                      mR[1] + m[1], mR[2] + m[2], G);
  split_factors(splitDG, f0, f1);
  F[0] = f0 * G[0];
  for (int v = 1; v < 5; ++v) F[v] = f1 * G[v];
}

// x = (rho, vn, p) -> boundary pressure
double fgpt_pressure_riemann(double kappa, double R, const double* x) {
  const Basis B = gas(kappa, R);
  return pressure_riemann(B, x[0], x[1], x[2]);
}
void fgpt_pressure_riemann_adj(double kappa, double R, const double* x, double pbb, double* xb) {
  const Basis B = gas(kappa, R);
  xb[0] = xb[1] = xb[2] = 0.0;
  pressure_riemann_adj(B, x[0], x[1], x[2], pbb, xb[0], xb[1], xb[2]);
}

// split_pair_flux (PI: pi = 1, SD: pi = 0) on the per-node inputs x = (qa[6], qb[6]) with the metric sum ms[3]: G[5]
void fgpt_split_pair(int pi, const double* x, const double* ms, double* G) {
  split_pair_flux(pi != 0, x[0], x[1], x[2], x[3], x[4], x[5], x[6], x[7], x[8], x[9], x[10], x[11], ms[0], ms[1], ms[2], G);
}
void fgpt_split_pair_adj(int pi, const double* x, const double* ms, const double* Gb, double* xb) {
  for (int c = 0; c < 12; ++c) xb[c] = 0.0;
  split_pair_flux_adj(pi != 0, x, x + 6, ms, Gb, xb, xb + 6);
}
// face-state fields x = (rho, E, u, v, w, p, srho) -> split inputs (q0, u, v, w, q4, q5) as the kernels form them
void fgpt_split_inputs(int pi, const double* x, double* q) {
  q[0] = x[0]; q[1] = x[2]; q[2] = x[3]; q[3] = x[4];
  q[4] = pi ? 4.0 * x[5] : x[5];
  q[5] = pi ? (x[1] + x[5]) * x[6] : x[1] + x[5];
}
void fgpt_split_inputs_adj(int pi, const double* x, const double* qb, double* xb) {
  double fb[FS_NF] = {0., 0., 0., 0., 0., 0., 0., 0.};
  split_inputs_to_face_adj(pi != 0, x[1], x[5], x[6], qb, fb);
  xb[0] = fb[FS_RHO]; xb[1] = fb[FS_E]; xb[2] = fb[FS_U]; xb[3] = fb[FS_V]; xb[4] = fb[FS_W]; xb[5] = fb[FS_P]; xb[6] = fb[FS_SRHO];
}
// the general split fluxes (SD, PI, MO, DU, KG) as the GEN kernels form them: pair flux of two nodes' inputs
// x = (q0, u, v, w, q4, q5) x 2 with metric sum ms; node inputs from x = (rho, E, u, v, w, p, srho); surface flux
void fgpt_split_pair_gen(int sd, const double* x, const double* ms, double* G) {
  const Basis B = gas(1.4, 1.0);
  split_pair_flux_gen(sd, B, x[0], x[1], x[2], x[3], x[4], x[5], x[6], x[7], x[8], x[9], x[10], x[11], ms[0], ms[1], ms[2], G);
}
void fgpt_split_pair_gen_adj(int sd, const double* x, const double* ms, const double* Gb, double* xb) {
  for (int c = 0; c < 12; ++c) xb[c] = 0.0;
  const Basis B = gas(1.4, 1.0);
  split_pair_flux_gen_adj(sd, B, x, x + 6, ms, Gb, xb, xb + 6);
}
void fgpt_split_node_inputs(int sd, const double* x, double* q) {
  q[1] = x[2]; q[2] = x[3]; q[3] = x[4];
  split_node_inputs(sd, x[0], x[2], x[3], x[4], x[5], x[1], x[6], q[0], q[4], q[5]);
}
void fgpt_split_node_inputs_adj(int sd, const double* x, const double* qb, double* xb) {
  for (int c = 0; c < 7; ++c) xb[c] = 0.0;
  split_node_inputs_adj(sd, x[0], x[2], x[3], x[4], x[5], x[1], x[6], qb, xb[0], xb[2], xb[3], xb[4], xb[5], xb[1], xb[6]);
}
void fgpt_split_surface_more(int sd, const double* L, const double* Rr, double* F) {
  const Basis B = gas(1.4, 1.0);
  split_surface_flux_more(sd, B, rs(L), rs(Rr), F);
}
void fgpt_split_surface_more_adj(int sd, const double* L, const double* Rr, const double* Fb, double* Lb, double* Rb) {
  RotState lb, rb;
  rot_zero(lb); rot_zero(rb);
  const Basis B = gas(1.4, 1.0);
  split_surface_flux_more_adj(sd, B, rs(L), rs(Rr), Fb, lb, rb);
  rs_out(lb, Lb); rs_out(rb, Rb);
}
// ConsToEntropy / EntropyToCons of k_prep and their adjoints
void fgpt_cons_to_entropy(double kappa, const double* U, double* W) {
  const Basis B = gas(kappa, 1.0);
  for (int v = 0; v < 5; ++v) W[v] = U[v];
  cons_to_entropy(B, W);
}
void fgpt_cons_to_entropy_adj(double kappa, const double* U, const double* Wb, double* Ub) {
  const Basis B = gas(kappa, 1.0);
  for (int v = 0; v < 5; ++v) Ub[v] = 0.0;
  cons_to_entropy_adj(B, U, Wb, Ub);
}
void fgpt_entropy_to_cons(double kappa, const double* W, double* U) {
  const Basis B = gas(kappa, 1.0);
  for (int v = 0; v < 5; ++v) U[v] = W[v];
  entropy_to_cons(B, U);
}
void fgpt_entropy_to_cons_adj(double kappa, const double* W, const double* Ub, double* Wb) {
  const Basis B = gas(kappa, 1.0);
  for (int v = 0; v < 5; ++v) Wb[v] = 0.0;
  entropy_to_cons_adj(B, W, Ub, Wb);
}

}  // extern "C"
