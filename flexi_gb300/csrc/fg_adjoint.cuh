// flexi_gb300 -- adjoint (vector-Jacobian product) of DGTimeDerivative_weakForm.
//
// Given the cotangent W of Ut, computes V = (dUt/dU)^T W at the state whose forward intermediates
// (primitive variables, lifted gradients, face states, face gradients) the forward kernels k_prep and
// k_lift have just written, plus the cotangent of the per-element viscosity multipliers. The forward
// kernels run prep -> lift -> flux -> volume; the adjoint runs the transposed steps in reverse:
//
//   k_vol_*_adj : Ut = -sJ (VolInt + SurfInt) -> cotangents of U (volume fluxes), of the lifted
//                 gradients, of the numerical flux of each side (one slot per neighbour) and of mu
//   k_flux_adj  : per side point, transposed Riemann-flux and viscous-flux Jacobians -> cotangents of
//                 the master and slave face states and face gradients
//   k_lift_adj  : transposed lifting (volume D sweeps, metrics, surface part, prolongation, BR2 term)
//                 -> cotangents of U (lifting variables) and of the lifting surface flux of each side
//   k_prep_adj  : face ConsToPrim and transposed prolongation of every face cotangent -> V
//
// Every array an adjoint kernel writes has exactly one writer per entry (per-side slots for the two
// neighbours, direction-by-direction passes where face points share volume nodes), so the result is
// deterministic. Supported: weak form (Gauss, Gauss-Lobatto), split form PI and SD (Gauss, Gauss-Lobatto;
// on Gauss nodes with the entropy-variable prolongation and the split-Gauss surface term), BR1/BR2 (strong,
// non-conservative), LF/HLLC/Roe/RoeEntropyFix, no-slip walls (BC 3/4).
#pragma once
#include "fg_adjoint_point.cuh"
#include "fg_kernels.cuh"

namespace fg {

struct AdjDev {
  const double* W;  // [e][5][n3] cotangent of Ut
  double* Ub;       // [e][5][n3] cotangent of U (the result V)
  double* gb;       // [e][12][n3] cotangent of the lifted gradients
  double* fluxb;    // [s][2][5][n2] cotangent of the numerical flux x SurfElem, from the master (0) / slave (1) element
  double* faceMb;   // [s][FS_NF][n2] cotangent of the master face state
  double* faceSb;   // [s][FS_NF][n2] cotangent of the slave face state
  double* gradMb;   // [s][12][n2] cotangent of the master face gradients
  double* gradSb;   // [s][12][n2] cotangent of the slave face gradients
  double* liftb;    // [s][2][4][n2] cotangent of the lifting surface flux, from the master (0) / slave (1) element
  double* muSideb;  // [s][2][n2] cotangent of the master / slave viscosity multiplier per side point
  double* muElemb;  // [e] cotangent of the element's viscosity multiplier
  double* liftMortarb;  // mortar meshes: [m][12][n2] cotangent of the projected lifting products of big mortar side m
  double* faceVolb; // split form on Gauss nodes: [s][2][FS_NF][n2] cotangent of the master (0) / slave (1) face
                    // state from the split-Gauss surface term of that element's volume integral (else null)
  int accumulate;   // 1: add V to Ub and the multiplier cotangent to muElemb instead of overwriting them
};

// -----------------------------------------------------------------------------------------------------
// helpers
// -----------------------------------------------------------------------------------------------------
// ubar = -sJ W into shared memory, and the cotangent of the six sides' numerical flux (transposed
// SurfInt, with the slave sign) into a.fluxb
template <int n, bool GL>
__device__ __forceinline__ void adj_load_ubar_and_surface(const Dev& d, const AdjDev& a, const SBasis<n>& Bs, double* sUb, int e0) {
  constexpr int n2 = n * n, n3 = n2 * n, EPB = Shape<n>::EPB, N = n - 1;
  for (int t = threadIdx.x; t < EPB * n3; t += blockDim.x) {
    const int es = t / n3, x = t - es * n3, e = e0 + es;
    if (e >= d.nElems) continue;
    const double msj = -d.sJ[(size_t)e * n3 + x];
#pragma unroll
    for (int v = 0; v < 5; ++v) sUb[(es * 5 + v) * n3 + x] = msj * a.W[((size_t)e * 5 + v) * n3 + x];
  }
  __syncthreads();
  for (int t = threadIdx.x; t < EPB * 6 * n2; t += blockDim.x) {
    const int es = t / (6 * n2), r = t - es * 6 * n2, lsi = r / n2, pq = r - lsi * n2;
    const int e = e0 + es;
    if (e >= d.nElems) continue;
    const int ls = lsi + 1, p = pq % n, q = pq / n;
    const int code = d.elemSide[e * 6 + lsi], s = code >> 3, flip = code & 7;
    int aa, bb;
    side_to_vol2(N, p, q, flip, ls, aa, bb);
    const bool minus = side_is_minus(ls);
    double fb[5] = {0., 0., 0., 0., 0.};
    if (GL) {
      const int x = face_node(ls, aa, bb, minus ? 0 : N, n);
      const double w = minus ? Bs.LhM(0) : Bs.LhP(N);
#pragma unroll
      for (int v = 0; v < 5; ++v) fb[v] = w * sUb[(es * 5 + v) * n3 + x];
    } else {
#pragma unroll
      for (int l = 0; l < n; ++l) {
        const int x = face_node(ls, aa, bb, l, n);
        const double w = minus ? Bs.LhM(l) : Bs.LhP(l);
#pragma unroll
        for (int v = 0; v < 5; ++v) fb[v] = fma(w, sUb[(es * 5 + v) * n3 + x], fb[v]);
      }
    }
    const double sg = flip == 0 ? 1.0 : -1.0;
    double* dst = a.fluxb + ((size_t)s * 2 + (flip == 0 ? 0 : 1)) * 5 * n2 + pq;
#pragma unroll
    for (int v = 0; v < 5; ++v) dst[v * n2] = sg * fb[v];
  }
}

// transposed prolongation gathered by the volume node that owns the result: node (i,j,k) collects, per
// direction, the cotangents (NC components, element face order) of the two face points on its normal
// line, weighted by L_minus(l) and L_plus(l) (Gauss) or taken at l = 0 / N (Gauss-Lobatto)
template <int n, bool GL, int NC>
__device__ __forceinline__ void prolong_gather_node(const SBasis<n>& Bs, const double* sFace, int es, int x, double* acc) {
  constexpr int n2 = n * n, N = n - 1;
  const int i = x % n, j = (x / n) % n, k = x / n2;
  const int idx3[3] = {i, j, k};
#pragma unroll
  for (int dir = 0; dir < 3; ++dir) {
    const int lsM = dir == 0 ? XI_MINUS : (dir == 1 ? ETA_MINUS : ZETA_MINUS);
    const int lsP = dir == 0 ? XI_PLUS : (dir == 1 ? ETA_PLUS : ZETA_PLUS);
    const int ab = (dir == 0 ? j : i) + n * (dir == 2 ? j : k);
    const int l = idx3[dir];
    const double* fM = sFace + ((es * 6 + lsM - 1) * n2 + ab) * NC;
    const double* fP = sFace + ((es * 6 + lsP - 1) * n2 + ab) * NC;
    if (GL) {
      if (l == 0) {
#pragma unroll
        for (int c = 0; c < NC; ++c) acc[c] += fM[c];
      }
      if (l == N) {
#pragma unroll
        for (int c = 0; c < NC; ++c) acc[c] += fP[c];
      }
    } else {
      const double LM = Bs.Lm(l), LP = Bs.Lp(l);
#pragma unroll
      for (int c = 0; c < NC; ++c) acc[c] = fma(LM, fM[c], fma(LP, fP[c], acc[c]));
    }
  }
}

// per-element sum of one value per node of the CTA (blockDim.x threads, EPB elements): sRed has THREADS slots
template <int n>
__device__ __forceinline__ void adj_element_sum(double val, double* sRed, double* out, int e0, int nElems, int accumulate) {
  constexpr int n3 = n * n * n, EPB = Shape<n>::EPB;
  sRed[threadIdx.x] = val;
  __syncthreads();
  if (threadIdx.x < EPB) {
    const int e = e0 + threadIdx.x;
    if (e < nElems) {
      double s = 0.;
      for (int x = 0; x < n3; ++x) s += sRed[threadIdx.x * n3 + x];
      out[e] = accumulate ? out[e] + s : s;
    }
  }
}

// -----------------------------------------------------------------------------------------------------
// k_vol_weak_adj: transposed VolInt_weakForm + SurfInt + Jacobian
// -----------------------------------------------------------------------------------------------------
template <int n, bool GL>
__global__ void __launch_bounds__(Shape<n>::THREADS) k_vol_weak_adj(Dev d, AdjDev a, Basis B) {
  using S = Shape<n>;
  constexpr int n2 = S::n2, n3 = S::n3, EPB = S::EPB;
  static_assert(EPB * n3 <= S::THREADS, "one node per thread");
  extern __shared__ double smem[];
  double* sD = smem;
  double* sUb = sD + SBasis<n>::SIZE;  // [EPB][5][n3]
  double* sRed = sUb + EPB * 5 * n3;   // [THREADS]
  load_basis_smem<n>(B, sD);
  SBasis<n> Bs{sD};
  const int e0 = blockIdx.x * EPB;
  adj_load_ubar_and_surface<n, GL>(d, a, Bs, sUb, e0);
  __syncthreads();
  const int t = threadIdx.x;
  const int es = t / n3, x = t - es * n3, e = e0 + es;
  double mub = 0.;
  if (es < EPB && e < d.nElems) {
    const int i = x % n, j = (x / n) % n, k = x / n2;
    const double* Ub = sUb + es * 5 * n3;
    // transposed D_hat sweeps: Ftilde_d bar at this node
    double Fb[3][5];
#pragma unroll
    for (int dd = 0; dd < 3; ++dd)
#pragma unroll
      for (int v = 0; v < 5; ++v) Fb[dd][v] = 0.;
#pragma unroll
    for (int l = 0; l < n; ++l) {
      const double ci = Bs.DhT(i, l), cj = Bs.DhT(j, l), ck = Bs.DhT(k, l);
      const int xi = l + n * (j + n * k), xj = i + n * (l + n * k), xk = i + n * (j + n * l);
#pragma unroll
      for (int v = 0; v < 5; ++v) {
        Fb[0][v] = fma(ci, Ub[v * n3 + xi], Fb[0][v]);
        Fb[1][v] = fma(cj, Ub[v * n3 + xj], Fb[1][v]);
        Fb[2][v] = fma(ck, Ub[v * n3 + xk], Fb[2][v]);
      }
    }
    // VolInt_Metrics transposed: physical flux bars
    double fb[5], gyb[5], hb[5];
    double m[9];
#pragma unroll
    for (int c = 0; c < 9; ++c) m[c] = d.metr[((size_t)e * 9 + c) * n3 + x];
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      fb[v] = Fb[0][v] * m[0] + Fb[1][v] * m[3] + Fb[2][v] * m[6];
      gyb[v] = Fb[0][v] * m[1] + Fb[1][v] * m[4] + Fb[2][v] * m[7];
      hb[v] = Fb[0][v] * m[2] + Fb[1][v] * m[5] + Fb[2][v] * m[8];
    }
    double u[5];
#pragma unroll
    for (int v = 0; v < 5; ++v) u[v] = d.U[((size_t)e * 5 + v) * n3 + x];
    const double vx = d.prim[((size_t)e * VP_NF + VP_U) * n3 + x];
    const double vy = d.prim[((size_t)e * VP_NF + VP_V) * n3 + x];
    const double vz = d.prim[((size_t)e * VP_NF + VP_W) * n3 + x];
    const double p = d.prim[((size_t)e * VP_NF + VP_P) * n3 + x];
    // advective flux (flux.f90:EvalFlux3D_Point) transposed
    const double Ep = u[4] + p;
    double ub[5] = {0., 0., 0., 0., 0.};
    ub[1] = fb[0] + fb[1] * vx + fb[2] * vy + fb[3] * vz;
    ub[2] = gyb[0] + gyb[1] * vx + gyb[2] * vy + gyb[3] * vz;
    ub[3] = hb[0] + hb[1] * vx + hb[2] * vy + hb[3] * vz;
    double vxb = fb[1] * u[1] + gyb[1] * u[2] + hb[1] * u[3] + fb[4] * Ep;
    double vyb = fb[2] * u[1] + gyb[2] * u[2] + hb[2] * u[3] + gyb[4] * Ep;
    double vzb = fb[3] * u[1] + gyb[3] * u[2] + hb[3] * u[3] + hb[4] * Ep;
    const double Epb = fb[4] * vx + gyb[4] * vy + hb[4] * vz;
    ub[4] = Epb;
    const double pb = fb[1] + gyb[2] + hb[3] + Epb;
    // viscous fluxes transposed
    double g[12], gb[12];
#pragma unroll
    for (int c = 0; c < 12; ++c) { g[c] = d.grad[((size_t)e * 12 + c) * n3 + x]; gb[c] = 0.; }
    const double mu = elem_mu(d, e);
    visc_flux_phys_adj(mu, B.lambdaFac, vx, vy, vz, g, fb, gyb, hb, vxb, vyb, vzb, gb, mub);
    mub *= d.mu0[d.elemInst[e]];
    cons_to_prim_adj(B, u, 0., vxb, vyb, vzb, pb, 0., 0., 0., ub);
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      double* o = a.Ub + ((size_t)e * 5 + v) * n3 + x;
      *o = a.accumulate ? *o + ub[v] : ub[v];
    }
#pragma unroll
    for (int c = 0; c < 12; ++c) a.gb[((size_t)e * 12 + c) * n3 + x] = gb[c];
  }
  adj_element_sum<n>(mub, sRed, a.muElemb, e0, d.nElems, a.accumulate);
}

// -----------------------------------------------------------------------------------------------------
// k_vol_split_adj: transposed VolInt_splitForm (PI, Gauss-Lobatto) + weak viscous part + SurfInt + Jacobian.
// Each pair (a, b) of a line adds the same 6-vector of cotangents of (rho, u, v, w, 4p, H) to both nodes;
// lane a evaluates the pair (a, a+dd) and hands that vector to lane a+dd by warp shuffle.
// -----------------------------------------------------------------------------------------------------
template <int n>
__global__ void __launch_bounds__(Shape<n>::THREADS) k_vol_split_adj(Dev d, AdjDev a, Basis B) {
  using S = Shape<n>;
  constexpr int n2 = S::n2, n3 = S::n3, EPB = S::EPB;
  static_assert(n == 8 || n == 4 || n == 2, "split kernel expects 2, 4 or 8 nodes per line");
  static_assert(EPB * n3 == S::THREADS, "one node per thread");
  extern __shared__ double smem[];
  double* sD = smem;
  double* sC = sD + SBasis<n>::SIZE;  // [2][n2] DVolSurf x 1/4, x 1/8
  double* sUb = sC + 2 * n2;          // [EPB][5][n3] -sJ W
  double* sR = sUb + EPB * 5 * n3;    // [EPB][15][n3] rho, u, v, w, 4p, H, metrics(9)
  double* sQb = sR + EPB * 15 * n3;   // [EPB][6][n3] cotangents of rho, u, v, w, 4p, H
  double* sRed = sQb + EPB * 6 * n3;  // [THREADS]
  load_basis_smem<n>(B, sD);
  SBasis<n> Bs{sD};
  for (int t = threadIdx.x; t < n2; t += blockDim.x) { sC[t] = B.DVS[t] * 0.25; sC[n2 + t] = B.DVS[t] * 0.125; }
  const int e0 = blockIdx.x * EPB;
  adj_load_ubar_and_surface<n, true>(d, a, Bs, sUb, e0);
  const int t = threadIdx.x;
  const int es0 = t / n3, x0 = t - es0 * n3, eT = e0 + es0;
  const bool validT = eT < d.nElems;
  if (validT) {
    double* Q = sR + es0 * 15 * n3;
    const double u0 = d.U[((size_t)eT * 5 + 0) * n3 + x0], u4 = d.U[((size_t)eT * 5 + 4) * n3 + x0];
    const double srho = d.prim[((size_t)eT * VP_NF + VP_SRHO) * n3 + x0];
    const double p = d.prim[((size_t)eT * VP_NF + VP_P) * n3 + x0];
    Q[x0] = u0;
    Q[n3 + x0] = d.prim[((size_t)eT * VP_NF + VP_U) * n3 + x0];
    Q[2 * n3 + x0] = d.prim[((size_t)eT * VP_NF + VP_V) * n3 + x0];
    Q[3 * n3 + x0] = d.prim[((size_t)eT * VP_NF + VP_W) * n3 + x0];
    Q[4 * n3 + x0] = 4.0 * p;
    Q[5 * n3 + x0] = (u4 + p) * srho;
#pragma unroll
    for (int c = 0; c < 9; ++c) Q[(6 + c) * n3 + x0] = d.metr[((size_t)eT * 9 + c) * n3 + x0];
  }
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int segBase = lane & ~(n - 1);
#pragma unroll 1
  for (int dir = 0; dir < 3; ++dir) {
    const int es = es0, r = x0;
    const int aI = r % n, c1 = (r / n) % n, c2 = r / n2;
    int xa;
    if (dir == 0) xa = aI + n * (c1 + n * c2);
    else if (dir == 1) xa = c1 + n * (aI + n * c2);
    else xa = c1 + n * (c2 + n * aI);
    const int stride = dir == 0 ? 1 : (dir == 1 ? n : n2);
    const int xline = xa - aI * stride;
    const double* Q = sR + es * 15 * n3;
    const double* Mm = Q + (6 + 3 * dir) * n3;
    const double* Ub = sUb + es * 5 * n3;
    const double ra = Q[xa], ua = Q[n3 + xa], va = Q[2 * n3 + xa], wa = Q[3 * n3 + xa], ha = Q[5 * n3 + xa];
    const double ma0 = Mm[xa], ma1 = Mm[n3 + xa], ma2 = Mm[2 * n3 + xa];
    double uba[5];
#pragma unroll
    for (int v = 0; v < 5; ++v) uba[v] = Ub[v * n3 + xa];
    double acc[6];
#pragma unroll
    for (int v = 0; v < 6; ++v) acc[v] = (dir == 0) ? 0. : sQb[(es * 6 + v) * n3 + xa];
#pragma unroll
    for (int dd = 1; dd <= n / 2; ++dd) {
      const int bI = (aI + dd) & (n - 1);
      const int xb = xline + bI * stride;
      const double rb = Q[xb], ub = Q[n3 + xb], vb = Q[2 * n3 + xb], wb = Q[3 * n3 + xb], hb = Q[5 * n3 + xb];
      const double ms0 = ma0 + Mm[xb], ms1 = ma1 + Mm[n3 + xb], ms2 = ma2 + Mm[2 * n3 + xb];
      const double rs = ra + rb, us = ua + ub, vs = va + vb, ws = wa + wb, hs = ha + hb;
      const double qs = us * ms0 + vs * ms1 + ws * ms2;
      const double A = rs * qs;
      // G bar = own coefficient x ubar(a) + partner coefficient x ubar(b)
      const double oA0 = sC[bI * n + aI], oA1 = sC[n2 + bI * n + aI];
      const double oB0 = sC[aI * n + bI], oB1 = sC[n2 + aI * n + bI];
      double Gb[5];
      Gb[0] = oA0 * uba[0] + oB0 * Ub[xb];
#pragma unroll
      for (int v = 1; v < 5; ++v) Gb[v] = oA1 * uba[v] + oB1 * Ub[v * n3 + xb];
      // G0 = A, G1..3 = A u_s + ps4 m_s, G4 = A H_s
      const double Ab = Gb[0] + Gb[1] * us + Gb[2] * vs + Gb[3] * ws + Gb[4] * hs;
      double Bv[6];
      Bv[0] = Ab * qs;                        // rho
      Bv[1] = Gb[1] * A + Ab * rs * ms0;      // u
      Bv[2] = Gb[2] * A + Ab * rs * ms1;      // v
      Bv[3] = Gb[3] * A + Ab * rs * ms2;      // w
      Bv[4] = Gb[1] * ms0 + Gb[2] * ms1 + Gb[3] * ms2;  // 4p
      Bv[5] = Gb[4] * A;                      // H
#pragma unroll
      for (int v = 0; v < 6; ++v) acc[v] += Bv[v];
      if (dd < n / 2) {
        const int src = segBase | ((aI - dd) & (n - 1));
#pragma unroll
        for (int v = 0; v < 6; ++v) acc[v] += __shfl_sync(0xffffffffu, Bv[v], src);
      }
    }
    if (validT) {
#pragma unroll
      for (int v = 0; v < 6; ++v) sQb[(es * 6 + v) * n3 + xa] = acc[v];
    }
    __syncthreads();
  }
  // per node (natural order): split-flux cotangents + weak viscous part -> U bar
  double mub = 0.;
  if (validT) {
    const int es = es0, x = x0, e = eT;
    const int i = x % n, j = (x / n) % n, k = x / n2;
    const double* Ub = sUb + es * 5 * n3;
    double Fb[3][5];
#pragma unroll
    for (int dd = 0; dd < 3; ++dd)
#pragma unroll
      for (int v = 1; v < 5; ++v) Fb[dd][v] = 0.;
#pragma unroll
    for (int l = 0; l < n; ++l) {
      const double ci = Bs.DhT(i, l), cj = Bs.DhT(j, l), ck = Bs.DhT(k, l);
      const int xi = l + n * (j + n * k), xj = i + n * (l + n * k), xk = i + n * (j + n * l);
#pragma unroll
      for (int v = 1; v < 5; ++v) {
        Fb[0][v] = fma(ci, Ub[v * n3 + xi], Fb[0][v]);
        Fb[1][v] = fma(cj, Ub[v * n3 + xj], Fb[1][v]);
        Fb[2][v] = fma(ck, Ub[v * n3 + xk], Fb[2][v]);
      }
    }
    const double* Q = sR + es * 15 * n3;
    double m[9];
#pragma unroll
    for (int c = 0; c < 9; ++c) m[c] = Q[(6 + c) * n3 + x];
    double fb[5] = {0., 0., 0., 0., 0.}, gyb[5] = {0., 0., 0., 0., 0.}, hb[5] = {0., 0., 0., 0., 0.};
#pragma unroll
    for (int v = 1; v < 5; ++v) {
      fb[v] = Fb[0][v] * m[0] + Fb[1][v] * m[3] + Fb[2][v] * m[6];
      gyb[v] = Fb[0][v] * m[1] + Fb[1][v] * m[4] + Fb[2][v] * m[7];
      hb[v] = Fb[0][v] * m[2] + Fb[1][v] * m[5] + Fb[2][v] * m[8];
    }
    double u[5];
#pragma unroll
    for (int v = 0; v < 5; ++v) u[v] = d.U[((size_t)e * 5 + v) * n3 + x];
    const double vx = Q[n3 + x], vy = Q[2 * n3 + x], vz = Q[3 * n3 + x];
    const double srho = 1.0 / u[0];
    const double p = Q[4 * n3 + x] * 0.25;
    double vxb = sQb[(es * 6 + 1) * n3 + x], vyb = sQb[(es * 6 + 2) * n3 + x], vzb = sQb[(es * 6 + 3) * n3 + x];
    const double Hb = sQb[(es * 6 + 5) * n3 + x];
    // 4p and H = (E + p) srho
    double pb = 4.0 * sQb[(es * 6 + 4) * n3 + x] + Hb * srho;
    const double Eb = Hb * srho;
    const double sb = Hb * (u[4] + p);
    double g[12], gb[12];
#pragma unroll
    for (int c = 0; c < 12; ++c) { g[c] = d.grad[((size_t)e * 12 + c) * n3 + x]; gb[c] = 0.; }
    const double mu = elem_mu(d, e);
    visc_flux_phys_adj(mu, B.lambdaFac, vx, vy, vz, g, fb, gyb, hb, vxb, vyb, vzb, gb, mub);
    mub *= d.mu0[d.elemInst[e]];
    double ubar[5] = {0., 0., 0., 0., 0.};
    cons_to_prim_adj(B, u, sb, vxb, vyb, vzb, pb, 0., sQb[(es * 6 + 0) * n3 + x], Eb, ubar);
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      double* o = a.Ub + ((size_t)e * 5 + v) * n3 + x;
      *o = a.accumulate ? *o + ubar[v] : ubar[v];
    }
#pragma unroll
    for (int c = 0; c < 12; ++c) a.gb[((size_t)e * 12 + c) * n3 + x] = gb[c];
  }
  adj_element_sum<n>(mub, sRed, a.muElemb, e0, d.nElems, a.accumulate);
}

// -----------------------------------------------------------------------------------------------------
// k_vol_split_gen_adj: transposed k_vol_split_gen (split form PI or SD, any line length, Gauss or
// Gauss-Lobatto) + weak viscous part + SurfInt + Jacobian. One thread per node: for every pair (a, b) of
// its three lines the node forms the pair's flux cotangent Gb = C(b,a) ubar(a) + C(a,b) ubar(b) and takes
// its own share of the transposed two-point flux (the partner node takes the other share from the same
// Gb), so every entry has one writer and no exchange is needed.
// Gauss nodes: the split-Gauss surface term adds, per line end, C_v(a) (sum_k Leg(k) G_k - G_a) with
// C_v(a) = -1/2 NormalSign LegHat(a) f_v; its flux cotangent is Gb_k = Leg(k) T_v - C_v(k) ubar_v(k) with the
// line sum T_v = sum_a C_v(a) ubar_v(a). The node takes the node share of each G_k; one thread per face point
// sums the face-state share over its line into a.faceVolb (k_prep_adj adds it to the face cotangent).
// -----------------------------------------------------------------------------------------------------
// LM: the split forms CH and IR (logarithmic means), in a variant of their own
template <int n, bool GL, bool LM = false>
__global__ void __launch_bounds__(Shape<n>::THREADS) k_vol_split_gen_adj(Dev d, AdjDev a, Basis B) {
  using S = Shape<n>;
  constexpr int n2 = S::n2, n3 = S::n3, EPB = S::EPB, N = n - 1;
  static_assert(EPB * n3 <= S::THREADS, "one node per thread");
  extern __shared__ double smem[];
  double* sD = smem;
  double* sC = sD + SBasis<n>::SIZE;   // [2][n2] DVolSurf x density factor, x factor of the others
  double* sUb = sC + 2 * n2;           // [EPB][5][n3] -sJ W
  double* sR = sUb + EPB * 5 * n3;     // [EPB][15][n3] split inputs (6), metrics (9)
  double* sRed = sR + EPB * 15 * n3;   // [THREADS]
  double* sFS = sRed + S::THREADS;     // Gauss: [EPB][6][9][n2] own face inputs (6) and face metric rows (3), element face order
  double* sT = sFS + (GL ? 0 : EPB * 6 * 9 * n2);  // Gauss: [EPB][6][n2][5] line sums T_v
  load_basis_smem<n>(B, sD);
  SBasis<n> Bs{sD};
  const int sd = B.splitDG;  // SD, PI, MO, DU or KG
  double f0, f1;
  split_factors(sd, f0, f1);
  for (int t = threadIdx.x; t < n2; t += blockDim.x) { sC[t] = B.DVS[t] * f0; sC[n2 + t] = B.DVS[t] * f1; }
  const int e0 = blockIdx.x * EPB;
  adj_load_ubar_and_surface<n, GL>(d, a, Bs, sUb, e0);
  for (int t = threadIdx.x; t < EPB * n3; t += blockDim.x) {
    const int es = t / n3, x = t - es * n3, e = e0 + es;
    if (e >= d.nElems) continue;
    double* Q = sR + es * 15 * n3;
    const double u0 = d.U[((size_t)e * 5 + 0) * n3 + x], u4 = d.U[((size_t)e * 5 + 4) * n3 + x];
    const double srho = d.prim[((size_t)e * VP_NF + VP_SRHO) * n3 + x];
    const double p = d.prim[((size_t)e * VP_NF + VP_P) * n3 + x];
    const double vx = d.prim[((size_t)e * VP_NF + VP_U) * n3 + x], vy = d.prim[((size_t)e * VP_NF + VP_V) * n3 + x],
                 vz = d.prim[((size_t)e * VP_NF + VP_W) * n3 + x];
    double q0, q4, q5;
    split_node_inputs(sd, u0, vx, vy, vz, p, u4, srho, q0, q4, q5);
    Q[x] = q0;
    Q[n3 + x] = vx;
    Q[2 * n3 + x] = vy;
    Q[3 * n3 + x] = vz;
    Q[4 * n3 + x] = q4;
    Q[5 * n3 + x] = q5;
#pragma unroll
    for (int c = 0; c < 9; ++c) Q[(6 + c) * n3 + x] = d.metr[((size_t)e * 9 + c) * n3 + x];
  }
  if (!GL) {
    for (int t = threadIdx.x; t < EPB * 6 * n2; t += blockDim.x) {
      const int es = t / (6 * n2), r = t - es * 6 * n2, lsi = r / n2, pq = r - lsi * n2;
      const int e = e0 + es;
      if (e >= d.nElems) continue;
      const int ls = lsi + 1, p = pq % n, q = pq / n;
      const int code = d.elemSide[e * 6 + lsi], s = code >> 3, flip = code & 7;
      int aa, bb;
      side_to_vol2(N, p, q, flip, ls, aa, bb);
      const double* src = (flip == 0 ? d.faceM : d.faceS) + (size_t)s * FS_NF * n2 + pq;
      const double pr = src[FS_P * n2];
      double* dst = sFS + (es * 6 + lsi) * 9 * n2;
      const int o = aa + n * bb;
      double q0, q4, q5;
      split_node_inputs(sd, src[FS_RHO * n2], src[FS_U * n2], src[FS_V * n2], src[FS_W * n2], pr, src[FS_E * n2], src[FS_SRHO * n2], q0, q4,
                        q5);
      dst[o] = q0;
      dst[n2 + o] = src[FS_U * n2];
      dst[2 * n2 + o] = src[FS_V * n2];
      dst[3 * n2 + o] = src[FS_W * n2];
      dst[4 * n2 + o] = q4;
      dst[5 * n2 + o] = q5;
#pragma unroll
      for (int c = 0; c < 3; ++c) dst[(6 + c) * n2 + o] = d.faceJa[(((size_t)e * 6 + lsi) * 3 + c) * n2 + o];
    }
  }
  __syncthreads();
  if (!GL) {
    // line sums T_v of the surface term, one thread per face point (element face order)
    for (int t = threadIdx.x; t < EPB * 6 * n2; t += blockDim.x) {
      const int es = t / (6 * n2), r = t - es * 6 * n2, lsi = r / n2, ab = r - lsi * n2;
      if (e0 + es >= d.nElems) continue;
      const int ls = lsi + 1, aa = ab % n, bb = ab / n;
      const bool minus = side_is_minus(ls);
      const double* Ub = sUb + es * 5 * n3;
      double T[5] = {0., 0., 0., 0., 0.};
      for (int l = 0; l < n; ++l) {
        const int x = face_node(ls, aa, bb, l, n);
        const double cs = minus ? 0.5 * Bs.LhM(l) : -0.5 * Bs.LhP(l);
#pragma unroll
        for (int v = 0; v < 5; ++v) T[v] = fma(cs * (v == 0 ? f0 : f1), Ub[v * n3 + x], T[v]);
      }
#pragma unroll
      for (int v = 0; v < 5; ++v) sT[((es * 6 + lsi) * n2 + ab) * 5 + v] = T[v];
    }
    __syncthreads();
  }
  const int t = threadIdx.x;
  const int es = t / n3, x = t - es * n3, e = e0 + es;
  const bool live = es < EPB && e < d.nElems;
  double mub = 0.;
  if (live) {
    const int i = x % n, j = (x / n) % n, k = x / n2;
    const int idx3[3] = {i, j, k};
    const double* Q = sR + es * 15 * n3;
    const double* Ub = sUb + es * 5 * n3;
    double qa[6], qbar[6] = {0., 0., 0., 0., 0., 0.};
#pragma unroll
    for (int c = 0; c < 6; ++c) qa[c] = Q[c * n3 + x];
    double uba[5];
#pragma unroll
    for (int v = 0; v < 5; ++v) uba[v] = Ub[v * n3 + x];
#pragma unroll 1
    for (int dir = 0; dir < 3; ++dir) {
      const int aI = idx3[dir];
      const int stride = dir == 0 ? 1 : (dir == 1 ? n : n2);
      const int xline = x - aI * stride;
      const double* Mm = Q + (6 + 3 * dir) * n3;
      const double ma[3] = {Mm[x], Mm[n3 + x], Mm[2 * n3 + x]};
      for (int bI = 0; bI < n; ++bI) {
        if (bI == aI) continue;
        const int xb = xline + bI * stride;
        double qb[6], dummy[6] = {0., 0., 0., 0., 0., 0.};
#pragma unroll
        for (int c = 0; c < 6; ++c) qb[c] = Q[c * n3 + xb];
        const double ms[3] = {ma[0] + Mm[xb], ma[1] + Mm[n3 + xb], ma[2] + Mm[2 * n3 + xb]};
        double Gb[5];
        Gb[0] = sC[bI * n + aI] * uba[0] + sC[aI * n + bI] * Ub[xb];
#pragma unroll
        for (int v = 1; v < 5; ++v) Gb[v] = sC[n2 + bI * n + aI] * uba[v] + sC[n2 + aI * n + bI] * Ub[v * n3 + xb];
        split_pair_flux_gen_adj<LM>(sd, B, qa, qb, ms, Gb, qbar, dummy);
      }
      if (!GL) {
        const int fo = dir == 0 ? j + n * k : (dir == 1 ? i + n * k : i + n * j);
#pragma unroll
        for (int side = 0; side < 2; ++side) {
          const int ls = side == 0 ? (dir == 0 ? XI_MINUS : (dir == 1 ? ETA_MINUS : ZETA_MINUS))
                                   : (dir == 0 ? XI_PLUS : (dir == 1 ? ETA_PLUS : ZETA_PLUS));
          const double* F = sFS + (es * 6 + ls - 1) * 9 * n2 + fo;
          const double* T = sT + ((es * 6 + ls - 1) * n2 + fo) * 5;
          const double leg = side == 0 ? Bs.Lm(aI) : Bs.Lp(aI);
          const double cs = side == 0 ? 0.5 * Bs.LhM(aI) : -0.5 * Bs.LhP(aI);
          double qf[6], dummy[6] = {0., 0., 0., 0., 0., 0.};
#pragma unroll
          for (int c = 0; c < 6; ++c) qf[c] = F[c * n2];
          const double ms[3] = {ma[0] + F[6 * n2], ma[1] + F[7 * n2], ma[2] + F[8 * n2]};
          double Gb[5];
#pragma unroll
          for (int v = 0; v < 5; ++v) Gb[v] = leg * T[v] - cs * (v == 0 ? f0 : f1) * uba[v];
          split_pair_flux_gen_adj<LM>(sd, B, qa, qf, ms, Gb, qbar, dummy);
        }
      }
    }
    // weak viscous part (transposed D_hat sweeps of the viscous fluxes) -> velocity and gradient bars
    double Fb[3][5];
#pragma unroll
    for (int dd = 0; dd < 3; ++dd)
#pragma unroll
      for (int v = 0; v < 5; ++v) Fb[dd][v] = 0.;
#pragma unroll
    for (int l = 0; l < n; ++l) {
      const double ci = Bs.DhT(i, l), cj = Bs.DhT(j, l), ck = Bs.DhT(k, l);
      const int xi = l + n * (j + n * k), xj = i + n * (l + n * k), xk = i + n * (j + n * l);
#pragma unroll
      for (int v = 1; v < 5; ++v) {
        Fb[0][v] = fma(ci, Ub[v * n3 + xi], Fb[0][v]);
        Fb[1][v] = fma(cj, Ub[v * n3 + xj], Fb[1][v]);
        Fb[2][v] = fma(ck, Ub[v * n3 + xk], Fb[2][v]);
      }
    }
    double m[9];
#pragma unroll
    for (int c = 0; c < 9; ++c) m[c] = Q[(6 + c) * n3 + x];
    double fb[5] = {0., 0., 0., 0., 0.}, gyb[5] = {0., 0., 0., 0., 0.}, hb[5] = {0., 0., 0., 0., 0.};
#pragma unroll
    for (int v = 1; v < 5; ++v) {
      fb[v] = Fb[0][v] * m[0] + Fb[1][v] * m[3] + Fb[2][v] * m[6];
      gyb[v] = Fb[0][v] * m[1] + Fb[1][v] * m[4] + Fb[2][v] * m[7];
      hb[v] = Fb[0][v] * m[2] + Fb[1][v] * m[5] + Fb[2][v] * m[8];
    }
    double u[5];
#pragma unroll
    for (int v = 0; v < 5; ++v) u[v] = d.U[((size_t)e * 5 + v) * n3 + x];
    const double vx = qa[1], vy = qa[2], vz = qa[3];
    const double srho = 1.0 / u[0];
    const double p = d.prim[((size_t)e * VP_NF + VP_P) * n3 + x];
    // the split inputs (split_node_inputs) transposed to the bars of rho, v, p, E and 1/rho
    double rhob = 0., vxb = 0., vyb = 0., vzb = 0., pb = 0., Eb = 0., sb = 0.;
    split_node_inputs_adj(sd, u[0], vx, vy, vz, p, u[4], srho, qbar, rhob, vxb, vyb, vzb, pb, Eb, sb);
    double g[12], gb[12];
#pragma unroll
    for (int c = 0; c < 12; ++c) { g[c] = d.grad[((size_t)e * 12 + c) * n3 + x]; gb[c] = 0.; }
    const double mu = elem_mu(d, e);
    visc_flux_phys_adj(mu, B.lambdaFac, vx, vy, vz, g, fb, gyb, hb, vxb, vyb, vzb, gb, mub);
    mub *= d.mu0[d.elemInst[e]];
    double ubar[5] = {0., 0., 0., 0., 0.};
    cons_to_prim_adj(B, u, sb, vxb, vyb, vzb, pb, 0., rhob, Eb, ubar);
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      double* o = a.Ub + ((size_t)e * 5 + v) * n3 + x;
      *o = a.accumulate ? *o + ubar[v] : ubar[v];
    }
#pragma unroll
    for (int c = 0; c < 12; ++c) a.gb[((size_t)e * 12 + c) * n3 + x] = gb[c];
  }
  if (!GL) {
    // face-state share of the surface term, summed over the line of each face point (side orientation)
    for (int tt = threadIdx.x; tt < EPB * 6 * n2; tt += blockDim.x) {
      const int fes = tt / (6 * n2), r = tt - fes * 6 * n2, lsi = r / n2, pq = r - lsi * n2;
      const int fe = e0 + fes;
      if (fe >= d.nElems) continue;
      const int ls = lsi + 1, p = pq % n, q = pq / n;
      const int code = d.elemSide[fe * 6 + lsi], s = code >> 3, flip = code & 7;
      int aa, bb;
      side_to_vol2(N, p, q, flip, ls, aa, bb);
      const bool minus = side_is_minus(ls);
      const int dir = (ls == XI_MINUS || ls == XI_PLUS) ? 0 : ((ls == ETA_MINUS || ls == ETA_PLUS) ? 1 : 2);
      const int ab = aa + n * bb;
      const double* F = sFS + (fes * 6 + lsi) * 9 * n2 + ab;
      const double* T = sT + ((fes * 6 + lsi) * n2 + ab) * 5;
      const double* Q = sR + fes * 15 * n3;
      const double* Ub = sUb + fes * 5 * n3;
      double qf[6], qfb[6] = {0., 0., 0., 0., 0., 0.};
#pragma unroll
      for (int c = 0; c < 6; ++c) qf[c] = F[c * n2];
      for (int l = 0; l < n; ++l) {
        const int xn = face_node(ls, aa, bb, l, n);
        double qn[6], dummy[6] = {0., 0., 0., 0., 0., 0.};
#pragma unroll
        for (int c = 0; c < 6; ++c) qn[c] = Q[c * n3 + xn];
        const double* Mm = Q + (6 + 3 * dir) * n3;
        const double ms[3] = {Mm[xn] + F[6 * n2], Mm[n3 + xn] + F[7 * n2], Mm[2 * n3 + xn] + F[8 * n2]};
        const double leg = minus ? Bs.Lm(l) : Bs.Lp(l);
        const double cs = minus ? 0.5 * Bs.LhM(l) : -0.5 * Bs.LhP(l);
        double Gb[5];
#pragma unroll
        for (int v = 0; v < 5; ++v) Gb[v] = leg * T[v] - cs * (v == 0 ? f0 : f1) * Ub[v * n3 + xn];
        split_pair_flux_gen_adj<LM>(sd, B, qn, qf, ms, Gb, dummy, qfb);
      }
      const double* src = (flip == 0 ? d.faceM : d.faceS) + (size_t)s * FS_NF * n2 + pq;
      double fb[FS_NF];
#pragma unroll
      for (int f = 0; f < FS_NF; ++f) fb[f] = 0.;
      split_node_inputs_adj(sd, src[FS_RHO * n2], src[FS_U * n2], src[FS_V * n2], src[FS_W * n2], src[FS_P * n2], src[FS_E * n2],
                            src[FS_SRHO * n2], qfb, fb[FS_RHO], fb[FS_U], fb[FS_V], fb[FS_W], fb[FS_P], fb[FS_E], fb[FS_SRHO]);
      double* dst = a.faceVolb + ((size_t)s * 2 + (flip == 0 ? 0 : 1)) * FS_NF * n2 + pq;
#pragma unroll
      for (int f = 0; f < FS_NF; ++f) dst[f * n2] = fb[f];
    }
  }
  adj_element_sum<n>(mub, sRed, a.muElemb, e0, d.nElems, a.accumulate);
}

// -----------------------------------------------------------------------------------------------------
// k_flux_adj: transposed FillFlux per side point (BC and conforming inner sides; the mortar sides are
// k_mortar_face_adj's)
// -----------------------------------------------------------------------------------------------------
// transposed numerical flux of inner side point (s, pq): Fb[5] is the cotangent of the flux before the
// SurfElem factor; gL[12] the master's face gradients (on a small mortar side: the big side's, interpolated).
// Writes the slave face-state, slave face-gradient and slave multiplier cotangents of the point, and adds the
// master face-state, master face-gradient and master multiplier (times mu0) cotangents into fbM, gLb, muLb.
// MORE: the Riemann solvers beyond LF/HLLC/Roe/RoeEntropyFix (riemann_rotated_more_adj)
template <int n, bool MORE = false>
__device__ __forceinline__ void inner_flux_adj(const Dev& d, const AdjDev& a, const Basis& B, int s, int pq, const double* Fb,
                                               const double* gL, double* gLb, double* fbM, double& muLb) {
  constexpr int n2 = n * n;
  const double* gm = d.geo + (size_t)s * FG_NF * n2 + pq;
  double nv[3], t1[3], t2[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) { nv[c] = gm[(FG_NX + c) * n2]; t1[c] = gm[(FG_T1X + c) * n2]; t2[c] = gm[(FG_T2X + c) * n2]; }
  const double mu0s = d.mu0[d.sideInst[s]];
  const double muL = d.muScale ? mu0s * d.muScale[d.sideElem[s * 4 + 0]] : mu0s;
  const double* fm = d.faceM + (size_t)s * FS_NF * n2 + pq;
  const double* fs = d.faceS + (size_t)s * FS_NF * n2 + pq;
  const double uL = fm[FS_U * n2], vL = fm[FS_V * n2], wL = fm[FS_W * n2];
  const double uR = fs[FS_U * n2], vR = fs[FS_V * n2], wR = fs[FS_W * n2];
  RotState L, R;
  L.rho = fm[FS_RHO * n2]; L.srho = fm[FS_SRHO * n2]; L.E = fm[FS_E * n2]; L.p = fm[FS_P * n2];
  R.rho = fs[FS_RHO * n2]; R.srho = fs[FS_SRHO * n2]; R.E = fs[FS_E * n2]; R.p = fs[FS_P * n2];
  L.v1 = uL * nv[0] + vL * nv[1] + wL * nv[2];
  L.v2 = uL * t1[0] + vL * t1[1] + wL * t1[2];
  L.v3 = uL * t2[0] + vL * t2[1] + wL * t2[2];
  R.v1 = uR * nv[0] + vR * nv[1] + wR * nv[2];
  R.v2 = uR * t1[0] + vR * t1[1] + wR * t1[2];
  R.v3 = uR * t2[0] + vR * t2[1] + wR * t2[2];
  double Frb[5];
  Frb[0] = Fb[0];
  Frb[1] = nv[0] * Fb[1] + nv[1] * Fb[2] + nv[2] * Fb[3];
  Frb[2] = t1[0] * Fb[1] + t1[1] * Fb[2] + t1[2] * Fb[3];
  Frb[3] = t2[0] * Fb[1] + t2[1] * Fb[2] + t2[2] * Fb[3];
  Frb[4] = Fb[4];
  RotState Lb, Rb;
  rot_zero(Lb); rot_zero(Rb);
  if constexpr (MORE) riemann_rotated_more_adj(B.riemann, B.splitDG, B, L, R, Frb, Lb, Rb);
  else riemann_rotated_adj(B.riemann, B.splitDG, B, L, R, Frb, Lb, Rb);
  double uLb = Lb.v1 * nv[0] + Lb.v2 * t1[0] + Lb.v3 * t2[0];
  double vLb = Lb.v1 * nv[1] + Lb.v2 * t1[1] + Lb.v3 * t2[1];
  double wLb = Lb.v1 * nv[2] + Lb.v2 * t1[2] + Lb.v3 * t2[2];
  double uRb = Rb.v1 * nv[0] + Rb.v2 * t1[0] + Rb.v3 * t2[0];
  double vRb = Rb.v1 * nv[1] + Rb.v2 * t1[1] + Rb.v3 * t2[1];
  double wRb = Rb.v1 * nv[2] + Rb.v2 * t1[2] + Rb.v3 * t2[2];
  // viscous side flux: 1/2 (Fv(L) + Fv(R))
  const double Fh[5] = {0., 0.5 * Fb[1], 0.5 * Fb[2], 0.5 * Fb[3], 0.5 * Fb[4]};
  const double muR = d.muScale ? mu0s * d.muScale[d.sideElem[s * 4 + 2]] : mu0s;
  double gR[12], gRb[12];
#pragma unroll
  for (int c = 0; c < 12; ++c) { gR[c] = d.gradS[((size_t)s * 12 + c) * n2 + pq]; gRb[c] = 0.; }
  double muLb0 = 0., muRb = 0.;
  visc_flux_dir_adj(muL, B.lambdaFac, uL, vL, wL, gL, nv[0], nv[1], nv[2], Fh, uLb, vLb, wLb, gLb, muLb0);
  visc_flux_dir_adj(muR, B.lambdaFac, uR, vR, wR, gR, nv[0], nv[1], nv[2], Fh, uRb, vRb, wRb, gRb, muRb);
  muLb += muLb0 * mu0s;
  fbM[FS_RHO] += Lb.rho; fbM[FS_SRHO] += Lb.srho; fbM[FS_E] += Lb.E; fbM[FS_P] += Lb.p;
  fbM[FS_U] += uLb; fbM[FS_V] += vLb; fbM[FS_W] += wLb;
  double* dS = a.faceSb + (size_t)s * FS_NF * n2 + pq;
  dS[FS_RHO * n2] = Rb.rho; dS[FS_SRHO * n2] = Rb.srho; dS[FS_E * n2] = Rb.E; dS[FS_P * n2] = Rb.p;
  dS[FS_U * n2] = uRb; dS[FS_V * n2] = vRb; dS[FS_W * n2] = wRb; dS[FS_T * n2] = 0.;
#pragma unroll
  for (int c = 0; c < 12; ++c) a.gradSb[((size_t)s * 12 + c) * n2 + pq] = gRb[c];
  a.muSideb[((size_t)s * 2 + 1) * n2 + pq] = muRb * mu0s;
}

template <int n, bool MORE = false>
__global__ void __launch_bounds__(128) k_flux_adj(Dev d, AdjDev a, Basis B) {
  constexpr int n2 = n * n;
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int s = (int)(idx / n2), pq = (int)(idx - (long long)s * n2);
  if (s >= d.nFluxSides) return;
  const double* gm = d.geo + (size_t)s * FG_NF * n2 + pq;
  const double se = gm[FG_SURF * n2];
  const double mu0s = d.mu0[d.sideInst[s]];
  double Fb[5];
#pragma unroll
  for (int v = 0; v < 5; ++v)
    Fb[v] = se * (a.fluxb[((size_t)s * 2 + 0) * 5 * n2 + v * n2 + pq] + a.fluxb[((size_t)s * 2 + 1) * 5 * n2 + v * n2 + pq]);
  double gL[12], gLb[12];
#pragma unroll
  for (int c = 0; c < 12; ++c) { gL[c] = d.gradM[((size_t)s * 12 + c) * n2 + pq]; gLb[c] = 0.; }
  double fbM[FS_NF];
#pragma unroll
  for (int f = 0; f < FS_NF; ++f) fbM[f] = 0.;
  double muLb = 0.;
  if (s < d.nBCSides) {
    const double muL = d.muScale ? mu0s * d.muScale[d.sideElem[s * 4 + 0]] : mu0s;
    const double* fm = d.faceM + (size_t)s * FS_NF * n2 + pq;
    double nv[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) nv[c] = gm[(FG_NX + c) * n2];
    const int bt = d.bcType[s];
    const double rho = fm[FS_RHO * n2], p = fm[FS_P * n2];
    const double vn = fm[FS_U * n2] * nv[0] + fm[FS_V * n2] * nv[1] + fm[FS_W * n2] * nv[2];
    const double pbb = Fb[1] * nv[0] + Fb[2] * nv[1] + Fb[3] * nv[2];
    double rhob = 0., vnb = 0., pb = 0.;
    pressure_riemann_adj(B, rho, vn, p, pbb, rhob, vnb, pb);
    fbM[FS_RHO] += rhob; fbM[FS_P] += pb;
    fbM[FS_U] += vnb * nv[0]; fbM[FS_V] += vnb * nv[1]; fbM[FS_W] += vnb * nv[2];
    double Fv[5] = {0., Fb[1], Fb[2], Fb[3], bt != 3 ? Fb[4] : 0.};
    double zu = 0., zv = 0., zw = 0., mub = 0.;
    visc_flux_dir_adj(muL, B.lambdaFac, 0., 0., 0., gL, nv[0], nv[1], nv[2], Fv, zu, zv, zw, gLb, mub);
    muLb = mub * mu0s;
  } else {
    inner_flux_adj<n, MORE>(d, a, B, s, pq, Fb, gL, gLb, fbM, muLb);
  }
  double* dM = a.faceMb + (size_t)s * FS_NF * n2 + pq;
#pragma unroll
  for (int f = 0; f < FS_NF; ++f) dM[f * n2] = fbM[f];
#pragma unroll
  for (int c = 0; c < 12; ++c) a.gradMb[((size_t)s * 12 + c) * n2 + pq] = gLb[c];
  a.muSideb[((size_t)s * 2 + 0) * n2 + pq] = muLb;
}

// -----------------------------------------------------------------------------------------------------
// mortar interfaces transposed (fillmortar.t90: U_Mortar and Flux_Mortar; mortar.f90 operators M_0_1,
// M_0_2 (interpolation) and M_1_0, M_2_0 (L2 projection)); big side in its master orientation
// -----------------------------------------------------------------------------------------------------
// transpose of mortar_interp: outb[im][v][n2] (cotangents of the small sides' interpolated fields) -> inb[v][n2]
// (of the big side's fields); tmp holds [2][nv][n2]. Ends with a barrier.
template <int n>
__device__ void mortar_interp_T(const MortarDev& M, int type, int nv, const double* outb, double* tmp, double* inb) {
  constexpr int n2 = n * n;
  if (type == 1) {
    for (int t = threadIdx.x; t < 2 * nv * n2; t += blockDim.x) {  // xi transposed: tmp[k][v][l + n q]
      const int k = t / (nv * n2), r = t - k * nv * n2, v = r / n2, lq = r - v * n2, l = lq % n, q = lq / n;
      const double* O0 = outb + ((2 * k) * nv + v) * n2;
      const double* O1 = outb + ((2 * k + 1) * nv + v) * n2;
      double acc = 0.;
#pragma unroll
      for (int p = 0; p < n; ++p) acc = fma(M.M01[l * n + p], O0[p + n * q], fma(M.M02[l * n + p], O1[p + n * q], acc));
      tmp[t] = acc;
    }
    __syncthreads();
    for (int t = threadIdx.x; t < nv * n2; t += blockDim.x) {  // eta transposed: inb[v][p + n l]
      const int v = t / n2, pl = t - v * n2, p = pl % n, l = pl / n;
      const double* T0 = tmp + v * n2;
      const double* T1 = tmp + (nv + v) * n2;
      double acc = 0.;
#pragma unroll
      for (int q = 0; q < n; ++q) acc = fma(M.M01[l * n + q], T0[p + n * q], fma(M.M02[l * n + q], T1[p + n * q], acc));
      inb[t] = acc;
    }
  } else {
    for (int t = threadIdx.x; t < nv * n2; t += blockDim.x) {
      const int v = t / n2, r = t - v * n2, i0 = r % n, i1 = r / n;
      const double* O0 = outb + v * n2;
      const double* O1 = outb + (nv + v) * n2;
      double acc = 0.;
      if (type == 2) {  // inb[v][p + n l] = sum_im sum_q M_im(l, q) outb[im][v][p + n q]
#pragma unroll
        for (int q = 0; q < n; ++q) acc = fma(M.M01[i1 * n + q], O0[i0 + n * q], fma(M.M02[i1 * n + q], O1[i0 + n * q], acc));
      } else {  // inb[v][l + n q] = sum_im sum_p M_im(l, p) outb[im][v][p + n q]
#pragma unroll
        for (int p = 0; p < n; ++p) acc = fma(M.M01[i0 * n + p], O0[p + n * i1], fma(M.M02[i0 * n + p], O1[p + n * i1], acc));
      }
      inb[t] = acc;
    }
  }
  __syncthreads();
}

// transpose of mortar_project: outb[v][n2] (cotangents of the big side's projected fields) -> inb[im][v][n2] (of the
// small sides' fields); tmp holds [2][nv][n2]. Ends with a barrier.
template <int n>
__device__ void mortar_project_T(const MortarDev& M, int type, int nv, const double* outb, double* tmp, double* inb) {
  constexpr int n2 = n * n;
  if (type == 1) {
    for (int t = threadIdx.x; t < 2 * nv * n2; t += blockDim.x) {  // eta transposed: tmp[k][v][p + n l]
      const int k = t / (nv * n2), r = t - k * nv * n2, v = r / n2, pl = r - v * n2, p = pl % n, l = pl / n;
      const double* Mk = k ? M.M20 : M.M10;
      const double* O = outb + v * n2;
      double acc = 0.;
#pragma unroll
      for (int q = 0; q < n; ++q) acc = fma(Mk[l * n + q], O[p + n * q], acc);
      tmp[t] = acc;
    }
    __syncthreads();
    for (int t = threadIdx.x; t < 4 * nv * n2; t += blockDim.x) {  // xi transposed: inb[im][v][l + n q]
      const int im = t / (nv * n2), r = t - im * nv * n2, v = r / n2, lq = r - v * n2, l = lq % n, q = lq / n;
      const double* Mi = (im & 1) ? M.M20 : M.M10;
      const double* T = tmp + ((im >> 1) * nv + v) * n2;
      double acc = 0.;
#pragma unroll
      for (int p = 0; p < n; ++p) acc = fma(Mi[l * n + p], T[p + n * q], acc);
      inb[t] = acc;
    }
  } else {
    for (int t = threadIdx.x; t < 2 * nv * n2; t += blockDim.x) {
      const int im = t / (nv * n2), r = t - im * nv * n2, v = r / n2, rr = r - v * n2, i0 = rr % n, i1 = rr / n;
      const double* Mx = im ? M.M20 : M.M10;
      const double* O = outb + v * n2;
      double acc = 0.;
      if (type == 2) {  // inb[im][v][p + n l] = sum_q M(l, q) outb[v][p + n q]
#pragma unroll
        for (int q = 0; q < n; ++q) acc = fma(Mx[i1 * n + q], O[i0 + n * q], acc);
      } else {  // inb[im][v][l + n q] = sum_p M(l, p) outb[v][p + n q]
#pragma unroll
        for (int p = 0; p < n; ++p) acc = fma(Mx[i0 * n + p], O[p + n * i1], acc);
      }
      inb[t] = acc;
    }
  }
  __syncthreads();
}

// transposed k_mortar_face, after k_flux_adj: the small sides' flux cotangent (their slave element's slot plus
// the transposed projection of the big side's), the transposed numerical fluxes of the small sides (master
// state: the interpolated big-side state, master gradients: the interpolated big-side gradients, master
// viscosity: the big element's), and the transposed gradient interpolation -> the big side's face-gradient
// cotangent. Writes every side-point cotangent of the small and big sides (zeros where a side has no such input).
template <int n>
__global__ void __launch_bounds__(256) k_mortar_face_adj(Dev d, AdjDev a, Basis B, MortarDev M) {
  constexpr int n2 = n * n;
  extern __shared__ double smem[];
  double* sG = smem;             // [12][n2] big side gradients, later their cotangent
  double* sT = sG + 12 * n2;     // [2][12][n2]
  double* sGs = sT + 24 * n2;    // [4][12][n2] interpolated gradients, later their cotangents
  double* sFb = sGs + 48 * n2;   // [5][n2] big side flux cotangent
  double* sFs = sFb + 5 * n2;    // [4][5][n2] small sides' flux cotangent (transposed projection)
  double* sMu = sFs + 20 * n2;   // [4][n2] master multiplier cotangent of each small-side point
  const int m = blockIdx.x;
  const int* info = M.info + 6 * m;
  const int type = info[0], sb = info[1], nm = type == 1 ? 4 : 2;
  for (int t = threadIdx.x; t < 12 * n2; t += blockDim.x) sG[t] = d.gradM[(size_t)sb * 12 * n2 + t];
  for (int t = threadIdx.x; t < 5 * n2; t += blockDim.x) sFb[t] = a.fluxb[(size_t)sb * 2 * 5 * n2 + t];
  __syncthreads();
  mortar_interp<n>(M, type, 12, sG, sT, sGs);
  mortar_project_T<n>(M, type, 5, sFb, sT, sFs);
  for (int t = threadIdx.x; t < nm * n2; t += blockDim.x) {
    const int im = t / n2, pq = t - im * n2, ss = info[2 + im];
    const double se = d.geo[((size_t)ss * FG_NF + FG_SURF) * n2 + pq];
    double Fb[5], gL[12], gLb[12], fbM[FS_NF];
#pragma unroll
    for (int v = 0; v < 5; ++v)
      Fb[v] = se * (sFs[(im * 5 + v) * n2 + pq] + a.fluxb[((size_t)ss * 2 + 0) * 5 * n2 + v * n2 + pq] +
                    a.fluxb[((size_t)ss * 2 + 1) * 5 * n2 + v * n2 + pq]);
#pragma unroll
    for (int c = 0; c < 12; ++c) { gL[c] = sGs[(im * 12 + c) * n2 + pq]; gLb[c] = 0.; }
#pragma unroll
    for (int f = 0; f < FS_NF; ++f) fbM[f] = 0.;
    double muLb = 0.;
    inner_flux_adj<n>(d, a, B, ss, pq, Fb, gL, gLb, fbM, muLb);
    double* dM = a.faceMb + (size_t)ss * FS_NF * n2 + pq;
#pragma unroll
    for (int f = 0; f < FS_NF; ++f) dM[f * n2] = fbM[f];
#pragma unroll
    for (int c = 0; c < 12; ++c) a.gradMb[((size_t)ss * 12 + c) * n2 + pq] = 0.;
    a.muSideb[((size_t)ss * 2 + 0) * n2 + pq] = 0.;
    sMu[t] = muLb;
    // every thread has read its interpolated gradients before any overwrites them (one thread per point)
#pragma unroll
    for (int c = 0; c < 12; ++c) sGs[(im * 12 + c) * n2 + pq] = gLb[c];
  }
  __syncthreads();
  mortar_interp_T<n>(M, type, 12, sGs, sT, sG);
  for (int t = threadIdx.x; t < 12 * n2; t += blockDim.x) {
    a.gradMb[(size_t)sb * 12 * n2 + t] = sG[t];
    a.gradSb[(size_t)sb * 12 * n2 + t] = 0.;
  }
  for (int pq = threadIdx.x; pq < n2; pq += blockDim.x) {
    double mu = 0.;
    for (int im = 0; im < nm; ++im) mu += sMu[im * n2 + pq];
    a.muSideb[((size_t)sb * 2 + 0) * n2 + pq] = mu;
    a.muSideb[((size_t)sb * 2 + 1) * n2 + pq] = 0.;
#pragma unroll
    for (int f = 0; f < FS_NF; ++f) a.faceSb[((size_t)sb * FS_NF + f) * n2 + pq] = 0.;
  }
}

// transposed k_mortar_pre, after k_lift_adj: the big side's lifting-product cotangent (a.liftMortarb) projected
// back to the small sides (transposed Flux_Mortar of the lifting fluxes), the small sides' master lifting-flux
// share of their slave element's lifting, ConsToPrim of the interpolated state transposed, and the transposed
// U_Mortar -> the big side's face-state cotangent a.faceMb (the big element's k_prep_adj takes it); the slave
// share of the projected lifting fluxes is added to the small sides' a.faceSb.
template <int n>
__global__ void __launch_bounds__(256) k_mortar_pre_adj(Dev d, AdjDev a, Basis B, MortarDev M) {
  constexpr int n2 = n * n;
  extern __shared__ double smem[];
  double* sU = smem;             // [5][n2] big side conservative state, later its cotangent
  double* sT = sU + 5 * n2;      // [2][12][n2]
  double* sUs = sT + 24 * n2;    // [4][5][n2] small sides' interpolated state, later its cotangent
  double* sP = sUs + 20 * n2;    // [12][n2] big side lifting-product cotangent
  double* sPs = sP + 12 * n2;    // [4][12][n2] small sides' lifting-product cotangent
  const int m = blockIdx.x;
  const int* info = M.info + 6 * m;
  const int type = info[0], sb = info[1], nm = type == 1 ? 4 : 2;
  for (int pq = threadIdx.x; pq < n2; pq += blockDim.x) {
    const double* fm = d.faceM + (size_t)sb * FS_NF * n2 + pq;
    const double rho = fm[FS_RHO * n2];
    sU[pq] = rho;
    sU[n2 + pq] = rho * fm[FS_U * n2];
    sU[2 * n2 + pq] = rho * fm[FS_V * n2];
    sU[3 * n2 + pq] = rho * fm[FS_W * n2];
    sU[4 * n2 + pq] = fm[FS_E * n2];
  }
  for (int t = threadIdx.x; t < 12 * n2; t += blockDim.x) sP[t] = a.liftMortarb[(size_t)m * 12 * n2 + t];
  __syncthreads();
  mortar_interp<n>(M, type, 5, sU, sT, sUs);
  mortar_project_T<n>(M, type, 12, sP, sT, sPs);
  const double sig = B.weakLifting ? 1.0 : -1.0;
  for (int t = threadIdx.x; t < nm * n2; t += blockDim.x) {
    const int im = t / n2, pq = t - im * n2, ss = info[2 + im];
    double c[5];
#pragma unroll
    for (int v = 0; v < 5; ++v) c[v] = sUs[(im * 5 + v) * n2 + pq];
    const double* gm = d.geo + (size_t)ss * FG_NF * n2 + pq;
    const double hs = 0.5 * gm[FG_SURF * n2];
    const double* fbp = a.faceMb + (size_t)ss * FS_NF * n2 + pq;
    double fb[FS_NF];
#pragma unroll
    for (int f = 0; f < FS_NF; ++f) fb[f] = fbp[f * n2];
    double* dS = a.faceSb + (size_t)ss * FS_NF * n2 + pq;
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      // lifting flux F_v = (sig um_v + us_v) SurfElem / 2, in the slave element's lifting and, times the normal,
      // in the big element's (projected products)
      double Fb = a.liftb[((size_t)ss * 2 + 0) * 4 * n2 + v * n2 + pq] + a.liftb[((size_t)ss * 2 + 1) * 4 * n2 + v * n2 + pq];
      double Fp = 0.;
#pragma unroll
      for (int cc = 0; cc < 3; ++cc) Fp = fma(sPs[(im * 12 + 4 * cc + v) * n2 + pq], gm[(FG_NX + cc) * n2], Fp);
      const int f = v < 3 ? FS_U + v : FS_T;
      fb[f] += sig * hs * (Fb + Fp);
      dS[f * n2] += hs * Fp;
    }
    double cb[5] = {0., 0., 0., 0., 0.};
    cons_to_prim_adj(B, c, fb[FS_SRHO], fb[FS_U], fb[FS_V], fb[FS_W], fb[FS_P], fb[FS_T], fb[FS_RHO], fb[FS_E], cb);
#pragma unroll
    for (int v = 0; v < 5; ++v) sUs[(im * 5 + v) * n2 + pq] = cb[v];
  }
  __syncthreads();
  mortar_interp_T<n>(M, type, 5, sUs, sT, sU);
  for (int pq = threadIdx.x; pq < n2; pq += blockDim.x) {
    const double* fm = d.faceM + (size_t)sb * FS_NF * n2 + pq;
    const double rho = fm[FS_RHO * n2];
    double* dM = a.faceMb + (size_t)sb * FS_NF * n2 + pq;
    // (rho, rho u, rho v, rho w, E) of the big side's face fields
    dM[FS_RHO * n2] = sU[pq] + sU[n2 + pq] * fm[FS_U * n2] + sU[2 * n2 + pq] * fm[FS_V * n2] + sU[3 * n2 + pq] * fm[FS_W * n2];
    dM[FS_U * n2] = sU[n2 + pq] * rho;
    dM[FS_V * n2] = sU[2 * n2 + pq] * rho;
    dM[FS_W * n2] = sU[3 * n2 + pq] * rho;
    dM[FS_E * n2] = sU[4 * n2 + pq];
    dM[FS_SRHO * n2] = 0.; dM[FS_P * n2] = 0.; dM[FS_T * n2] = 0.;
  }
}

// -----------------------------------------------------------------------------------------------------
// k_lift_adj: transposed lifting of one element per CTA tile. MORTAR (meshes with mortar interfaces): the
// cotangent of the surface lifting flux is kept as that of the 12 products F_v n_c per face point (the
// forward's layout); a big mortar side's goes to a.liftMortarb (k_mortar_pre_adj projects it back to the
// small sides), the other sides' is contracted with the normal into a.liftb.
// -----------------------------------------------------------------------------------------------------
template <int n, bool GL, bool MORTAR = false>
__global__ void __launch_bounds__(Shape<n>::THREADS) k_lift_adj(Dev d, AdjDev a, Basis B) {
  using S = Shape<n>;
  constexpr int n2 = S::n2, n3 = S::n3, EPB = S::EPB, N = S::N;
  constexpr int NFB = MORTAR ? 12 : 4;   // cotangent values per face point in sFb
  extern __shared__ double smem[];
  double* sD = smem;
  double* sGb = sD + SBasis<n>::SIZE;    // [EPB][12][n3] gradient cotangents (later: d/dxi, d/deta, d/dzeta cotangents)
  double* sFb = sGb + EPB * 12 * n3;     // [EPB][6][n2][NFB] cotangent of the lifting surface flux (MORTAR: of the products), element face order
  double* sN = sFb + EPB * 6 * n2 * NFB; // [EPB][6][n2][3] face normals, element face order
  double* sGf = sN + EPB * 6 * n2 * 3;   // [EPB][6][n2][12] face gradient cotangents, element face order
  double* sJs = sGf + EPB * 6 * n2 * 12; // [EPB][n3]
  load_basis_smem<n>(B, sD);
  SBasis<n> Bs{sD};
  const int e0 = blockIdx.x * EPB;
  const bool br2 = B.lifting == 2;
  for (int t = threadIdx.x; t < EPB * n3; t += blockDim.x) {
    const int es = t / n3, x = t - es * n3, e = e0 + es;
    if (e >= d.nElems) continue;
#pragma unroll
    for (int c = 0; c < 12; ++c) sGb[(es * 12 + c) * n3 + x] = a.gb[((size_t)e * 12 + c) * n3 + x];
    sJs[es * n3 + x] = d.sJ[(size_t)e * n3 + x];
  }
  for (int t = threadIdx.x; t < EPB * 6 * n2; t += blockDim.x) {
    const int es = t / (6 * n2), r = t - es * 6 * n2, lsi = r / n2, pq = r - lsi * n2;
    const int e = e0 + es;
    if (e >= d.nElems) continue;
    const int ls = lsi + 1, p = pq % n, q = pq / n;
    const int code = d.elemSide[e * 6 + lsi], s = code >> 3, flip = code & 7;
    int aa, bb;
    side_to_vol2(N, p, q, flip, ls, aa, bb);
    const int o = (es * 6 + lsi) * n2 + aa + n * bb;
    const double* gm = d.geo + (size_t)s * FG_NF * n2 + pq;
#pragma unroll
    for (int c = 0; c < 3; ++c) sN[o * 3 + c] = gm[(FG_NX + c) * n2];
    const double* gfb = (flip == 0 ? a.gradMb : a.gradSb) + (size_t)s * 12 * n2 + pq;
#pragma unroll
    for (int c = 0; c < 12; ++c) sGf[o * 12 + c] = gfb[c * n2];
#pragma unroll
    for (int v = 0; v < NFB; ++v) sFb[o * NFB + v] = 0.;
  }
  __syncthreads();
  // BR2 eta term of the face gradients: gf += eta wsum sF n
  if (br2) {
    for (int t = threadIdx.x; t < EPB * 6 * n2; t += blockDim.x) {
      const int es = t / (6 * n2), r = t - es * 6 * n2, lsi = r / n2, ab = r - lsi * n2;
      const int e = e0 + es;
      if (e >= d.nElems) continue;
      const int ls = lsi + 1, aa = ab % n, bb = ab / n;
      const bool minus = side_is_minus(ls);
      const int s = d.elemSide[e * 6 + lsi] >> 3;
      double eta = B.etaBR2;
      if (s < d.nBCSides && (d.bcType[s] == 3 || d.bcType[s] == 4)) eta = B.etaBR2_wall;
      double wsum = 0.;
      if (GL) {
        wsum = Bs.Lm(0) * Bs.LhM(0) * sJs[es * n3 + face_node(ls, aa, bb, minus ? 0 : N, n)];
      } else {
#pragma unroll
        for (int l = 0; l < n; ++l) wsum = fma(Bs.Lm(l) * Bs.LhM(l), sJs[es * n3 + face_node(ls, aa, bb, minus ? l : N - l, n)], wsum);
      }
      const int o = (es * 6 + lsi) * n2 + ab;
      const double ew = eta * wsum;
      if constexpr (MORTAR) {
#pragma unroll
        for (int c = 0; c < 12; ++c) sFb[o * 12 + c] += ew * sGf[o * 12 + c];
      } else {
#pragma unroll
        for (int v = 0; v < 4; ++v) {
          double acc = 0.;
#pragma unroll
          for (int c = 0; c < 3; ++c) acc = fma(sGf[o * 12 + 4 * c + v], sN[o * 3 + c], acc);
          sFb[o * 4 + v] += ew * acc;
        }
      }
    }
  }
  // transposed prolongation of the face gradients into sGb, one direction (two opposite faces) at a time.
  // BR1 prolongs the full gradient (added before the surface part is transposed), BR2 the volume part (after).
  auto prolong_adj = [&]() {
    for (int t = threadIdx.x; t < EPB * n3; t += blockDim.x) {
      const int es = t / n3, x = t - es * n3, e = e0 + es;
      if (e >= d.nElems) continue;
      double acc[12];
#pragma unroll
      for (int c = 0; c < 12; ++c) acc[c] = 0.;
      prolong_gather_node<n, GL, 12>(Bs, sGf, es, x, acc);
      double* G = sGb + es * 12 * n3;
#pragma unroll
      for (int c = 0; c < 12; ++c) G[c * n3 + x] += acc[c];
    }
    __syncthreads();
  };
  __syncthreads();
  if (!br2) prolong_adj();
  // transposed surface part: sF bar += w sJ n . gbar over the nodes of the normal line
  for (int t = threadIdx.x; t < EPB * 6 * n2; t += blockDim.x) {
    const int es = t / (6 * n2), r = t - es * 6 * n2, lsi = r / n2, ab = r - lsi * n2;
    const int e = e0 + es;
    if (e >= d.nElems) continue;
    const int ls = lsi + 1, aa = ab % n, bb = ab / n;
    const bool minus = side_is_minus(ls);
    const int o = (es * 6 + lsi) * n2 + ab;
    const double* G = sGb + es * 12 * n3;
    double acc[NFB];
#pragma unroll
    for (int v = 0; v < NFB; ++v) acc[v] = 0.;
    const int lmax = GL ? 1 : n;
    for (int li = 0; li < lmax; ++li) {
      const int l = GL ? (minus ? 0 : N) : li;
      const int x = face_node(ls, aa, bb, l, n);
      const double w = (minus ? Bs.LhM(l) : Bs.LhP(l)) * sJs[es * n3 + x];
      if constexpr (MORTAR) {
#pragma unroll
        for (int c = 0; c < 12; ++c) acc[c] = fma(w, G[c * n3 + x], acc[c]);
      } else {
#pragma unroll
        for (int v = 0; v < 4; ++v) {
          double dot = 0.;
#pragma unroll
          for (int c = 0; c < 3; ++c) dot = fma(sN[o * 3 + c], G[(4 * c + v) * n3 + x], dot);
          acc[v] = fma(w, dot, acc[v]);
        }
      }
    }
#pragma unroll
    for (int v = 0; v < NFB; ++v) sFb[o * NFB + v] += acc[v];
  }
  __syncthreads();
  if (br2) prolong_adj();
  // metrics x sJ transposed (in place: each node reads and writes only its own 12 entries)
  for (int t = threadIdx.x; t < EPB * n3; t += blockDim.x) {
    const int es = t / n3, x = t - es * n3, e = e0 + es;
    if (e >= d.nElems) continue;
    double mJ[9];
    if (d.metrJ) {
#pragma unroll
      for (int c = 0; c < 9; ++c) mJ[c] = d.metrJ[((size_t)e * 9 + c) * n3 + x];
    } else {
      const double sj = sJs[es * n3 + x];
#pragma unroll
      for (int c = 0; c < 9; ++c) mJ[c] = d.metr[((size_t)e * 9 + c) * n3 + x] * sj;
    }
    double* G = sGb + es * 12 * n3;
    double gb[12];
#pragma unroll
    for (int c = 0; c < 12; ++c) gb[c] = G[c * n3 + x];
    // g[4dd+v] = mJ[dd] gx[v] + mJ[3+dd] ge[v] + mJ[6+dd] gz[v]
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      double gx = 0., ge = 0., gz = 0.;
#pragma unroll
      for (int dd = 0; dd < 3; ++dd) {
        gx = fma(mJ[dd], gb[4 * dd + v], gx);
        ge = fma(mJ[3 + dd], gb[4 * dd + v], ge);
        gz = fma(mJ[6 + dd], gb[4 * dd + v], gz);
      }
      G[v * n3 + x] = gx; G[(4 + v) * n3 + x] = ge; G[(8 + v) * n3 + x] = gz;
    }
  }
  __syncthreads();
  // transposed D sweeps -> cotangents of (u, v, w, T) -> U bar
  for (int t = threadIdx.x; t < EPB * n3; t += blockDim.x) {
    const int es = t / n3, x = t - es * n3, e = e0 + es;
    if (e >= d.nElems) continue;
    const int i = x % n, j = (x / n) % n, k = x / n2;
    const double* G = sGb + es * 12 * n3;
    double Lb[4] = {0., 0., 0., 0.};
#pragma unroll
    for (int l = 0; l < n; ++l) {
      // gx(l,j,k) = sum_i' DT(i',l) L(i',j,k): L(i,j,k) gets DT(i,l) gxbar(l,j,k)
      const double ci = Bs.DT(i, l), cj = Bs.DT(j, l), ck = Bs.DT(k, l);
      const int xi = l + n * (j + n * k), xj = i + n * (l + n * k), xk = i + n * (j + n * l);
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        Lb[v] = fma(ci, G[v * n3 + xi], Lb[v]);
        Lb[v] = fma(cj, G[(4 + v) * n3 + xj], Lb[v]);
        Lb[v] = fma(ck, G[(8 + v) * n3 + xk], Lb[v]);
      }
    }
    double u[5], ub[5] = {0., 0., 0., 0., 0.};
#pragma unroll
    for (int v = 0; v < 5; ++v) u[v] = d.U[((size_t)e * 5 + v) * n3 + x];
    cons_to_prim_adj(B, u, 0., Lb[0], Lb[1], Lb[2], 0., Lb[3], 0., 0., ub);
#pragma unroll
    for (int v = 0; v < 5; ++v) a.Ub[((size_t)e * 5 + v) * n3 + x] += ub[v];
  }
  // lifting surface flux cotangents to the side slots (side orientation)
  for (int t = threadIdx.x; t < EPB * 6 * n2; t += blockDim.x) {
    const int es = t / (6 * n2), r = t - es * 6 * n2, lsi = r / n2, pq = r - lsi * n2;
    const int e = e0 + es;
    if (e >= d.nElems) continue;
    const int ls = lsi + 1, p = pq % n, q = pq / n;
    const int code = d.elemSide[e * 6 + lsi], s = code >> 3, flip = code & 7;
    int aa, bb;
    side_to_vol2(N, p, q, flip, ls, aa, bb);
    const int o = (es * 6 + lsi) * n2 + aa + n * bb;
    if constexpr (MORTAR) {
      const int mb = s - (d.nSides - d.nMortars);
      if (mb >= 0) {  // big mortar side: the products' cotangent, side orientation
        double* ml = a.liftMortarb + (size_t)mb * 12 * n2 + pq;
#pragma unroll
        for (int c = 0; c < 12; ++c) ml[c * n2] = sFb[o * 12 + c];
        continue;
      }
      double* dst = a.liftb + ((size_t)s * 2 + (flip == 0 ? 0 : 1)) * 4 * n2 + pq;
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        double acc = 0.;
#pragma unroll
        for (int c = 0; c < 3; ++c) acc = fma(sFb[o * 12 + 4 * c + v], sN[o * 3 + c], acc);
        dst[v * n2] = acc;
      }
    } else {
      double* dst = a.liftb + ((size_t)s * 2 + (flip == 0 ? 0 : 1)) * 4 * n2 + pq;
#pragma unroll
      for (int v = 0; v < 4; ++v) dst[v * n2] = sFb[o * 4 + v];
    }
  }
}

// -----------------------------------------------------------------------------------------------------
// k_prep_adj: face ConsToPrim and prolongation transposed; adds the face parts to U bar, sums mu bar
// -----------------------------------------------------------------------------------------------------
template <int n, bool GL>
__global__ void __launch_bounds__(Shape<n>::THREADS) k_prep_adj(Dev d, AdjDev a, Basis B) {
  using S = Shape<n>;
  constexpr int n2 = S::n2, n3 = S::n3, EPB = S::EPB, N = S::N;
  extern __shared__ double smem[];
  double* sD = smem;
  double* sU = sD + SBasis<n>::SIZE;   // [EPB][5][n3] state
  double* sCb = sU + EPB * 5 * n3;     // [EPB][6][n2][5] cotangents of the prolonged face states, element face order
  double* sMub = sCb + EPB * 6 * n2 * 5;  // [EPB][6][n2] viscosity-multiplier cotangent of each face point
  load_basis_smem<n>(B, sD);
  SBasis<n> Bs{sD};
  const int e0 = blockIdx.x * EPB;
  // split form on Gauss nodes: the faces carry EntropyToCons of the prolonged entropy variables (k_prep)
  const bool entropy = !GL && B.splitDG >= 0;
  for (int t = threadIdx.x; t < EPB * n3; t += blockDim.x) {
    const int es = t / n3, x = t - es * n3, e = e0 + es;
    if (e >= d.nElems) continue;
    double u[5];
#pragma unroll
    for (int v = 0; v < 5; ++v) u[v] = d.U[((size_t)e * 5 + v) * n3 + x];
    if (entropy) cons_to_entropy(B, u);
#pragma unroll
    for (int v = 0; v < 5; ++v) sU[(es * 5 + v) * n3 + x] = u[v];
  }
  __syncthreads();
  const double sig = B.weakLifting ? 1.0 : -1.0;
  for (int t = threadIdx.x; t < EPB * 6 * n2; t += blockDim.x) {
    const int es = t / (6 * n2), r = t - es * 6 * n2, lsi = r / n2, pq = r - lsi * n2;
    const int e = e0 + es;
    if (e >= d.nElems) continue;
    const int ls = lsi + 1, p = pq % n, q = pq / n;
    const int code = d.elemSide[e * 6 + lsi], s = code >> 3, flip = code & 7;
    int aa, bb;
    side_to_vol2(N, p, q, flip, ls, aa, bb);
    const bool master = flip == 0;
    const double* fbp = (master ? a.faceMb : a.faceSb) + (size_t)s * FS_NF * n2 + pq;
    double fb[FS_NF];
#pragma unroll
    for (int f = 0; f < FS_NF; ++f) fb[f] = fbp[f * n2];
    const double se = d.geo[((size_t)s * FG_NF + FG_SURF) * n2 + pq];
    double Lf[4];
#pragma unroll
    for (int v = 0; v < 4; ++v) Lf[v] = a.liftb[((size_t)s * 2 + 0) * 4 * n2 + v * n2 + pq];
    if (s < d.nBCSides) {
      // F = (bval - fm) se: walls (velocity 0; T = Twall for BC 4, T = fm for BC 3 -> no dependence)
      fb[FS_U] -= se * Lf[0]; fb[FS_V] -= se * Lf[1]; fb[FS_W] -= se * Lf[2];
      if (d.bcType[s] == 4) fb[FS_T] -= se * Lf[3];
    } else {
      // F = (sig fm + fs) se / 2, the same F in both neighbours' lifting
#pragma unroll
      for (int v = 0; v < 4; ++v) Lf[v] += a.liftb[((size_t)s * 2 + 1) * 4 * n2 + v * n2 + pq];
      const double fac = (master ? sig : 1.0) * 0.5 * se;
      fb[FS_U] += fac * Lf[0]; fb[FS_V] += fac * Lf[1]; fb[FS_W] += fac * Lf[2]; fb[FS_T] += fac * Lf[3];
    }
    sMub[t] = a.muSideb[((size_t)s * 2 + (master ? 0 : 1)) * n2 + pq];
    if (entropy) {
      const double* vb = a.faceVolb + ((size_t)s * 2 + (master ? 0 : 1)) * FS_NF * n2 + pq;
#pragma unroll
      for (int f = 0; f < FS_NF; ++f) fb[f] += vb[f * n2];
    }
    // conservative face state (prolongation of U, or EntropyToCons of the prolonged entropy variables) and
    // its ConsToPrim transposed
    const bool minus = side_is_minus(ls);
    double c[5];
    if (GL) {
      const int x = face_node(ls, aa, bb, minus ? 0 : N, n);
#pragma unroll
      for (int v = 0; v < 5; ++v) c[v] = sU[(es * 5 + v) * n3 + x];
    } else {
#pragma unroll
      for (int v = 0; v < 5; ++v) c[v] = 0.;
#pragma unroll
      for (int l = 0; l < n; ++l) {
        const int x = face_node(ls, aa, bb, l, n);
        const double L = minus ? Bs.Lm(l) : Bs.Lp(l);
#pragma unroll
        for (int v = 0; v < 5; ++v) c[v] = fma(sU[(es * 5 + v) * n3 + x], L, c[v]);
      }
    }
    double cb[5] = {0., 0., 0., 0., 0.};
    if (entropy) {
      double cc[5] = {c[0], c[1], c[2], c[3], c[4]};
      entropy_to_cons(B, cc);
      double ccb[5] = {0., 0., 0., 0., 0.};
      cons_to_prim_adj(B, cc, fb[FS_SRHO], fb[FS_U], fb[FS_V], fb[FS_W], fb[FS_P], fb[FS_T], fb[FS_RHO], fb[FS_E], ccb);
      entropy_to_cons_adj(B, c, ccb, cb);
    } else {
      cons_to_prim_adj(B, c, fb[FS_SRHO], fb[FS_U], fb[FS_V], fb[FS_W], fb[FS_P], fb[FS_T], fb[FS_RHO], fb[FS_E], cb);
    }
    const int o = (es * 6 + lsi) * n2 + aa + n * bb;
#pragma unroll
    for (int v = 0; v < 5; ++v) sCb[o * 5 + v] = cb[v];
  }
  __syncthreads();
  // transposed prolongation, gathered per volume node
  for (int t = threadIdx.x; t < EPB * n3; t += blockDim.x) {
    const int es = t / n3, x = t - es * n3, e = e0 + es;
    if (e >= d.nElems) continue;
    double acc[5] = {0., 0., 0., 0., 0.};
    prolong_gather_node<n, GL, 5>(Bs, sCb, es, x, acc);
    if (entropy) {
      // acc holds the cotangent of the node's entropy variables
      double u[5], ub[5] = {0., 0., 0., 0., 0.};
#pragma unroll
      for (int v = 0; v < 5; ++v) u[v] = d.U[((size_t)e * 5 + v) * n3 + x];
      cons_to_entropy_adj(B, u, acc, ub);
#pragma unroll
      for (int v = 0; v < 5; ++v) acc[v] = ub[v];
    }
#pragma unroll
    for (int v = 0; v < 5; ++v) a.Ub[((size_t)e * 5 + v) * n3 + x] += acc[v];
  }
  // mu bar of the element: volume part (k_vol_*_adj) + its sides' viscous fluxes
  if (threadIdx.x < EPB) {
    const int e = e0 + threadIdx.x;
    if (e < d.nElems) {
      double s = a.muElemb[e];
      for (int f = 0; f < 6 * n2; ++f) s += sMub[threadIdx.x * 6 * n2 + f];
      a.muElemb[e] = s;
    }
  }
}

}  // namespace fg
