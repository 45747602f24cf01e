// flexi_gb300 -- element and side kernels of one DGSEM right-hand-side evaluation (FLEXI's
// DGTimeDerivative_weakForm, src/dg/dg.f90:221-678) and the fused low-storage RK stage update
// (src/timedisc/timestep.f90:82-152).
//
// Per RK stage four launches:
//   k_prep  (element)  ConsToPrim of the volume, ProlongToFace of U, ConsToPrim of the face values
//   k_lift  (element)  BR1/BR2 lifting: volume gradient (D sweeps + metrics), surface lifting terms,
//                      Jacobian, ProlongToFaceLifting (+ the BR2 face penalty)
//   k_flux  (side)     Riemann solver + viscous flux (+ wall BCs), times SurfElem
//   k_vol   (element)  volume integral (weak or split form), surface integral, -Ut*sJ, source,
//                      and the LSERK register update -- or plain Ut output for fg_time_derivative
// One CTA processes EPB elements with one thread per volume node; all face work is done by the
// element that owns the data, reading its neighbour's face values from global memory.
#pragma once
#include "fg_common.cuh"

namespace fg {

// E = elements per CTA; E = 0 selects the default, which fills at least ~128 threads for small n (the
// autotuner may pick another E for the element kernels that have variants). One thread per volume node
// up to 512 threads; larger elements (lines of 9..12 nodes) give each thread several nodes.
template <int n, int E = 0> struct Shape {
  static constexpr int N = n - 1, n2 = n * n, n3 = n * n * n;
  static constexpr int EPB = E > 0 ? E : ((n3 >= 128) ? 1 : (128 + n3 - 1) / n3);
  static constexpr int THREADS = ((EPB * n3 + 31) / 32) * 32 > 512 ? 512 : ((EPB * n3 + 31) / 32) * 32;
};

// Shared-memory plan of an element kernel: the basis matrices always live in shared memory, the kernel's
// per-element arrays ("big", in doubles per CTA) too unless basis + big exceed FG_SMEM_LIMIT; then they
// live in the CTA's slice of the global array Dev::scratch (L1/L2-cached; lines of 10..12 nodes).
constexpr long long FG_SMEM_LIMIT = 220 * 1024;
template <int n> struct SBasisSize { static constexpr int value = 3 * n * n + 4 * n; };
template <int n>
__host__ __device__ constexpr bool big_in_global(long long big) { return (SBasisSize<n>::value + big) * 8 > FG_SMEM_LIMIT; }
template <int n>
constexpr size_t dyn_smem_bytes(long long big) { return 8 * (size_t)(SBasisSize<n>::value + (big_in_global<n>(big) ? 0 : big)); }
template <int n>
__device__ __forceinline__ double* big_base(const Dev& d, double* smem, long long big) {
  return big_in_global<n>(big) ? d.scratch + (size_t)blockIdx.x * d.scratchStride : smem + SBasisSize<n>::value;
}
// per-element arrays of the element kernels (doubles per CTA)
template <int n, int E = 0> struct Big {
  using S = Shape<n, E>;
  static constexpr long long prep = (long long)S::EPB * (5 + VP_NF) * S::n3;
  static constexpr long long lift = (long long)S::EPB * (17 * S::n3 + 42 * S::n2);
  static constexpr long long liftMortar = (long long)S::EPB * (17 * S::n3 + 72 * S::n2);
  // k_lift variants: MORTAR keeps 12 products per face point, CONS stages the 9 metric terms
  __host__ __device__ static constexpr long long liftVariant(bool mortar, bool cons) { return (mortar ? liftMortar : lift) + (cons ? (long long)S::EPB * 9 * S::n3 : 0); }
  static constexpr long long weak = (long long)S::EPB * (15 * S::n3 + 30 * S::n2);
};

// copies the basis matrices a kernel indexes with thread-dependent indices into shared memory
template <int n>
__device__ __forceinline__ void load_basis_smem(const Basis& B, double* sD) {
  for (int t = threadIdx.x; t < n * n; t += blockDim.x) {
    sD[t] = B.D_T[t];
    sD[n * n + t] = B.Dhat_T[t];
    sD[2 * n * n + t] = B.DVS[t];
  }
  for (int t = threadIdx.x; t < n; t += blockDim.x) {
    sD[3 * n * n + t] = B.Lm[t];
    sD[3 * n * n + n + t] = B.Lp[t];
    sD[3 * n * n + 2 * n + t] = B.LhM[t];
    sD[3 * n * n + 3 * n + t] = B.LhP[t];
  }
}
template <int n> struct SBasis {
  static constexpr int SIZE = 3 * n * n + 4 * n;
  const double* s;
  __device__ double DT(int l, int i) const { return s[l * n + i]; }
  __device__ double DhT(int l, int i) const { return s[n * n + l * n + i]; }
  __device__ double DVS(int l, int i) const { return s[2 * n * n + l * n + i]; }
  __device__ double Lm(int l) const { return s[3 * n * n + l]; }
  __device__ double Lp(int l) const { return s[3 * n * n + n + l]; }
  __device__ double LhM(int l) const { return s[3 * n * n + 2 * n + l]; }
  __device__ double LhP(int l) const { return s[3 * n * n + 3 * n + l]; }
};

// Line sweeps in the even-odd form: lines of n nodes are held one node per lane, SEG = 32/n lines to a warp
// (lane a of segment seg = node a); for lines of 6 nodes and more this takes fewer FP64 instructions than
// n FMAs per node
template <int n> struct EOShape {
  static constexpr bool ON = n >= 6;    // lifting: three direction sweeps per variable, no sum across directions
  static constexpr bool VOL = n >= 8;   // volume kernels: the three directions' results are summed per node
                                        // afterwards (one FP64 add each), which offsets the gain below n = 8
  static constexpr int SEG = 32 / n;
};
// this lane's row of an even-odd table (Basis::eoD, or eoDh when DHAT) into registers
template <int n, bool DHAT>
__device__ __forceinline__ void eo_row(const Basis& B, double* eo) {
  const int lane = threadIdx.x & 31, a = lane - n * (lane / n);
#pragma unroll
  for (int c = 0; c < 8; ++c) eo[c] = DHAT ? B.eoDh[a * 8 + c] : B.eoD[a * 8 + c];
}

// derivative along a line held one node per lane (lane a = node a of the segment starting at lane segBase) with a
// centro-antisymmetric matrix M (M(N-i,N-l) = -M(i,l): D and D_Hat on symmetric nodes), by its even-odd form: with
// s_l = u_l + u_{N-l}, d_l = u_l - u_{N-l} (l < n/2) and the middle node m of odd n,
//   du_i + du_{N-i} = sum_l (M(i,l) - M(i,N-l)) d_l,   du_i - du_{N-i} = sum_l (M(i,l) + M(i,N-l)) s_l + 2 M(i,m) u_m,
// du_m = sum_l M(m,l) d_l: n/2 + 2 FP64 operations per output (+1 for odd n) instead of n. eo: this lane's row of the
// basis table (Basis::eoD / eoDh); every lane of the warp takes part (lanes outside a segment pass their own values).
template <int n, int NV>
__device__ __forceinline__ void eo_line_derivative(const double* eo, int a, int segBase, const double* u, double* du) {
  constexpr int N = n - 1, h = n / 2, m = N / 2;
  const int lane = threadIdx.x & 31;
  const bool inSeg = a < n && segBase + n <= 32;
  const int mirror = inSeg ? segBase + N - a : lane;
  const double sgnA = a < h ? 1.0 : -1.0;
  double sd[NV], acc[NV];
#pragma unroll
  for (int v = 0; v < NV; ++v) sd[v] = fma(sgnA, u[v], __shfl_sync(0xffffffffu, u[v], mirror));  // s_a or d_{N-a}
#pragma unroll
  for (int c = 0; c < h; ++c) {
    const int src = inSeg ? segBase + (a < h ? c : N - c) : lane;
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      const double x = __shfl_sync(0xffffffffu, sd[v], src);
      acc[v] = c == 0 ? eo[0] * x : fma(eo[c], x, acc[v]);
    }
  }
  if constexpr (n % 2 == 1) {
    const int srcM = inSeg ? segBase + m : lane;
#pragma unroll
    for (int v = 0; v < NV; ++v) acc[v] = fma(eo[h], __shfl_sync(0xffffffffu, u[v], srcM), acc[v]);
  }
#pragma unroll
  for (int v = 0; v < NV; ++v) du[v] = fma(eo[h + 1], __shfl_sync(0xffffffffu, acc[v], mirror), acc[v]);
}


// even-odd sweeps of NV components of a [EPB][*][n3] shared array along each direction: input component
// inC0 + inDirStep*dir + v (v < NV) differentiated along direction dir with a row of Basis::eoD or eoDh into
// output component outC0 + outDirStep*dir + v (in place when both name the same entries: each line and component belongs to
// one work item, and a warp reads its lines before it writes them). The lines of all three directions run in one
// flat loop of whole warps. Ends with a barrier.
// (eo: the row of the table for this lane's node a = (lane % 32) - n * ((lane % 32) / n), loaded by the caller)
template <int n, int NV, int E = 0>
__device__ __forceinline__ void eo_sweep_all(const double* eo, const double* in, int inStride, int inC0, int inDirStep, double* out,
                                             int outStride, int outC0, int outDirStep, int e0, int nElems) {
  constexpr int n2 = n * n, n3 = n2 * n, EPB = Shape<n, E>::EPB, SEG = EOShape<n>::SEG;
  constexpr int LINES = EPB * n2, L3 = 3 * LINES, W = (L3 + SEG - 1) / SEG;
  const int lane = threadIdx.x & 31, seg = lane / n, a = lane - seg * n, segBase = seg * n;
  for (int base = 0; base < W * 32; base += blockDim.x) {
    const int tt = base + threadIdx.x;
    if (tt < W * 32) {  // whole warps
      const int k = (tt >> 5) * SEG + seg;
      const bool valid = seg < SEG && k < L3;
      const int kc = valid ? k : 0;
      const int dir = kc / LINES, line = kc - dir * LINES;
      const int es = line / n2, lr = line - es * n2, c1 = lr % n, c2 = lr / n;
      const int stride = dir == 0 ? 1 : (dir == 1 ? n : n2);
      const int xline = dir == 0 ? n * (c1 + n * c2) : (dir == 1 ? c1 + n2 * c2 : c1 + n * c2);
      const int x = xline + a * stride;
      const double* I = in + ((size_t)es * inStride + inC0 + inDirStep * dir) * n3 + x;
      double u[NV], du[NV];
#pragma unroll
      for (int v = 0; v < NV; ++v) u[v] = I[v * n3];
      eo_line_derivative<n, NV>(eo, a, segBase, u, du);
      if (valid && e0 + es < nElems) {
        double* O = out + ((size_t)es * outStride + outC0 + outDirStep * dir) * n3 + x;
#pragma unroll
        for (int v = 0; v < NV; ++v) O[v * n3] = du[v];
      }
    }
  }
  __syncthreads();
}

// =====================================================================================================
// k_prep: eos.f90:ConsToPrim (volume), prolongtoface.t90:ProlongToFace, equation.f90:GetPrimitiveStateSurface.
// Split form on Gauss nodes (PP_EntropyVars): the entropy variables are prolonged instead of U and turned
// back into conservative face states (eos.f90:ConsToPrimToEntropy, prolongtoface.t90:ProlongToFaceEntropy,
// eos.f90:EntropyToCons).
// =====================================================================================================
template <int n, bool GL, int E = 0>
__global__ void __launch_bounds__(Shape<n, E>::THREADS) k_prep(Dev d, Basis B) {
  using S = Shape<n, E>;
  constexpr int n2 = S::n2, n3 = S::n3, EPB = S::EPB, N = S::N;
  extern __shared__ double smem[];
  double* sD = smem;
  double* sU = big_base<n>(d, smem, Big<n, E>::prep);  // [EPB][5][n3] U, or the entropy variables
  double* sP = sU + EPB * 5 * n3;              // [EPB][VP_NF][n3]
  load_basis_smem<n>(B, sD);
  SBasis<n> Bs{sD};
  const bool entropy = !GL && B.splitDG >= 0;
  const int e0 = blockIdx.x * EPB;
  for (int t = threadIdx.x; t < EPB * n3; t += blockDim.x) {
    const int es = t / n3, x = t - es * n3, e = e0 + es;
    if (e >= d.nElems) continue;
    double u[5];
#pragma unroll
    for (int v = 0; v < 5; ++v) u[v] = d.U[((size_t)e * 5 + v) * n3 + x];
    const double srho = 1.0 / u[0];
    const double vx = u[1] * srho, vy = u[2] * srho, vz = u[3] * srho;
    const double p = B.kappaM1 * (u[4] - 0.5 * (u[1] * vx + u[2] * vy + u[3] * vz));
    const double T = p * srho * B.sR;
    const double pr[VP_NF] = {srho, vx, vy, vz, p, T};
#pragma unroll
    for (int f = 0; f < VP_NF; ++f) {
      d.prim[((size_t)e * VP_NF + f) * n3 + x] = pr[f];
      sP[(es * VP_NF + f) * n3 + x] = pr[f];
    }
    if (entropy) {
      // PrimToEntropy: s = ln p - kappa ln rho; W = ((kappa - s)/(kappa-1) - rho/p |v|^2/2, rho/p v, -rho/p)
      const double sEnt = log(p) - B.kappa * log(u[0]);
      const double rho_p = u[0] / p;
      u[0] = (B.kappa - sEnt) * B.sKappaM1 - rho_p * 0.5 * (vx * vx + vy * vy + vz * vz);
      u[1] = rho_p * vx; u[2] = rho_p * vy; u[3] = rho_p * vz;
      u[4] = -rho_p;
    }
#pragma unroll
    for (int v = 0; v < 5; ++v) sU[(es * 5 + v) * n3 + x] = u[v];
  }
  __syncthreads();
  for (int t = threadIdx.x; t < EPB * 6 * n2; t += blockDim.x) {
    const int es = t / (6 * n2), r = t - es * 6 * n2, lsi = r / n2, pq = r - lsi * n2;
    const int e = e0 + es;
    if (e >= d.nElems) continue;
    const int ls = lsi + 1, p = pq % n, q = pq / n;
    const int code = d.elemSide[e * 6 + lsi], s = code >> 3, flip = code & 7;
    int a, b;
    side_to_vol2(N, p, q, flip, ls, a, b);
    double fs[FS_NF];
    if (GL) {
      const int x = face_node(ls, a, b, side_is_minus(ls) ? 0 : N, n);
      fs[FS_RHO] = sU[(es * 5 + 0) * n3 + x];
      fs[FS_E] = sU[(es * 5 + 4) * n3 + x];
      fs[FS_SRHO] = sP[(es * VP_NF + VP_SRHO) * n3 + x];
      fs[FS_U] = sP[(es * VP_NF + VP_U) * n3 + x];
      fs[FS_V] = sP[(es * VP_NF + VP_V) * n3 + x];
      fs[FS_W] = sP[(es * VP_NF + VP_W) * n3 + x];
      fs[FS_P] = sP[(es * VP_NF + VP_P) * n3 + x];
      fs[FS_T] = sP[(es * VP_NF + VP_T) * n3 + x];
    } else {
      const bool minus = side_is_minus(ls);
      double c[5] = {0., 0., 0., 0., 0.};
#pragma unroll
      for (int l = 0; l < n; ++l) {
        const int x = face_node(ls, a, b, l, n);
        const double L = minus ? Bs.Lm(l) : Bs.Lp(l);
#pragma unroll
        for (int v = 0; v < 5; ++v) c[v] = fma(sU[(es * 5 + v) * n3 + x], L, c[v]);
      }
      if (entropy) {
        // EntropyToCons: rho e = (kappa-1)^(1/(kappa-1)) (-W5')^(-kappa/(kappa-1)) exp(-s/(kappa-1)), W' = (kappa-1) W;
        const double w0 = c[0] * B.kappaM1, w1 = c[1] * B.kappaM1, w2 = c[2] * B.kappaM1, w3 = c[3] * B.kappaM1, w4 = c[4] * B.kappaM1;
        const double ekin = 0.5 * (w1 * w1 + w2 * w2 + w3 * w3) / w4;
        const double sEnt = B.kappa - w0 + ekin;
        // (kappa-1)^(1/(kappa-1)) (-W5')^(-kappa/(kappa-1)) exp(-s/(kappa-1)) as one exponential
        const double rhoe = exp(B.logEntC - B.kappa_kappaM1 * log(-w4) - sEnt * B.sKappaM1);
        c[0] = -rhoe * w4;
        c[1] = rhoe * w1; c[2] = rhoe * w2; c[3] = rhoe * w3;
        c[4] = rhoe * (1.0 - ekin);
      }
      const double srho = 1.0 / c[0];
      const double vx = c[1] * srho, vy = c[2] * srho, vz = c[3] * srho;
      const double pp = B.kappaM1 * (c[4] - 0.5 * (c[1] * vx + c[2] * vy + c[3] * vz));
      fs[FS_RHO] = c[0]; fs[FS_E] = c[4]; fs[FS_SRHO] = srho;
      fs[FS_U] = vx; fs[FS_V] = vy; fs[FS_W] = vz; fs[FS_P] = pp; fs[FS_T] = pp * srho * B.sR;
    }
    double* dst = (flip == 0 ? d.faceM : d.faceS) + (size_t)s * FS_NF * n2 + pq;
#pragma unroll
    for (int f = 0; f < FS_NF; ++f) dst[f * n2] = fs[f];
  }
}

// ProlongToFaceLifting of the gradients in sG (+ BR2: eta * lifting contribution of this face,
// lifting_br2.t90:Lifting_SurfInt_BR2) for the six faces of the CTA's elements; MORTAR: sF holds the 12
// products F_v n_c per face point (sN unused)
template <int n, bool GL, int E = 0, bool MORTAR = false>
__device__ __forceinline__ void lift_prolong_faces(const Dev& d, const Basis& B, const SBasis<n>& Bs, const double* sG, const double* sF,
                                                   const double* sN, const double* sJs, int e0, bool br2) {
  constexpr int n2 = n * n, n3 = n2 * n, EPB = Shape<n, E>::EPB, N = n - 1;
  for (int t = threadIdx.x; t < EPB * 6 * n2; t += blockDim.x) {
    const int es = t / (6 * n2), r = t - es * 6 * n2, lsi = r / n2, pq = r - lsi * n2;
    const int e = e0 + es;
    if (e >= d.nElems) continue;
    const int ls = lsi + 1, p = pq % n, q = pq / n;
    const int code = d.elemSide[e * 6 + lsi], s = code >> 3, flip = code & 7;
    int a, b;
    side_to_vol2(N, p, q, flip, ls, a, b);
    const bool minus = side_is_minus(ls);
    double gf[12];
    if (GL) {
      const int x = face_node(ls, a, b, minus ? 0 : N, n);
#pragma unroll
      for (int c = 0; c < 12; ++c) gf[c] = sG[(es * 12 + c) * n3 + x];
    } else {
#pragma unroll
      for (int c = 0; c < 12; ++c) gf[c] = 0.;
#pragma unroll
      for (int l = 0; l < n; ++l) {
        const int x = face_node(ls, a, b, l, n);
        const double L = minus ? Bs.Lm(l) : Bs.Lp(l);
#pragma unroll
        for (int c = 0; c < 12; ++c) gf[c] = fma(sG[(es * 12 + c) * n3 + x], L, gf[c]);
      }
    }
    if (br2) {
      double eta = B.etaBR2;
      if (s < d.nBCSides && (d.bcType[s] == 3 || d.bcType[s] == 4)) eta = B.etaBR2_wall;
      // sum_l L_Minus(l) * L_HatMinus(l) * sJ(node at distance l from this face)
      double wsum = 0.;
      if (GL) {
        wsum = Bs.Lm(0) * Bs.LhM(0) * sJs[es * n3 + face_node(ls, a, b, minus ? 0 : N, n)];
      } else {
#pragma unroll
        for (int l = 0; l < n; ++l) wsum = fma(Bs.Lm(l) * Bs.LhM(l), sJs[es * n3 + face_node(ls, a, b, minus ? l : N - l, n)], wsum);
      }
      const int o = (es * 6 + lsi) * n2 + a + n * b;
      const double ew = eta * wsum;
      if constexpr (MORTAR) {
#pragma unroll
        for (int c = 0; c < 12; ++c) gf[c] = fma(sF[o * 12 + c], ew, gf[c]);
      } else {
#pragma unroll
        for (int v = 0; v < 4; ++v) {
          const double f = sF[o * 4 + v] * ew;
#pragma unroll
          for (int c = 0; c < 3; ++c) gf[4 * c + v] = fma(f, sN[o * 3 + c], gf[4 * c + v]);
        }
      }
    }
    double* dst = (flip == 0 ? d.gradM : d.gradS) + (size_t)s * 12 * n2 + pq;
#pragma unroll
    for (int c = 0; c < 12; ++c) dst[c * n2] = gf[c];
  }
}

// =====================================================================================================
// k_lift: lifting_br1.t90 / lifting_br2.t90 (strong or weak BR1, BR2), non-conservative volume part
// (lifting_volint.t90:Lifting_VolInt_Nonconservative), surface part, ApplyJacobianLifting,
// ProlongToFaceLifting. The volume part uses the metrics pre-multiplied by sJ when the mesh provides
// them (Dev::metrJ), else forms the products itself. On Gauss-Lobatto nodes the surface part reaches
// only the face nodes: it is added face-parallel, one direction (two opposite faces, disjoint node
// sets) at a time, so that no warp runs it for interior nodes.
// MORTAR (meshes with mortar interfaces): the surface flux is kept as the 12 products F_v n_c per face
// point, so that a big mortar side can take the projection of its small sides' products
// (lifting_br1.t90:106-109, lifting_br2.t90:103-106: Flux_Mortar of the lifting fluxes), which k_mortar_pre
// leaves in Dev::mortarLift; with BR2 the face penalty uses the same products.
// =====================================================================================================
template <int n, bool GL, int E = 0, bool MORTAR = false, bool CONS = false>
__global__ void __launch_bounds__(Shape<n, E>::THREADS, (n == 8 && GL ? 2 : 1)) k_lift(Dev d, Basis B) {
  using S = Shape<n, E>;
  constexpr int n2 = S::n2, n3 = S::n3, EPB = S::EPB, N = S::N;
  constexpr int NFN = MORTAR ? 12 : 4;  // values per face point in sF
  extern __shared__ double smem[];
  double* sD = smem;
  double* sL = big_base<n>(d, smem, Big<n, E>::liftVariant(MORTAR, CONS));  // [EPB][4][n3] lifting variables u,v,w,T
  double* sF = sL + EPB * 4 * n3;        // [EPB][6][n2][NFN] surface lifting flux (times SurfElem), local face order
  double* sN = sF + EPB * 6 * n2 * NFN;  // [EPB][6][n2][3] face normal of the side point mapped to local face order (not MORTAR)
  double* sG = sN + (MORTAR ? 0 : EPB * 6 * n2 * 3);  // [EPB][12][n3] gradients
  double* sJs = sG + EPB * 12 * n3;      // [EPB][n3]
  double* sMc = sJs + EPB * n3;          // CONS: [EPB][9][n3] metrics (not times sJ) of the conservative volume part
  load_basis_smem<n>(B, sD);
  SBasis<n> Bs{sD};
  const int e0 = blockIdx.x * EPB;
  const bool br2 = B.lifting == 2;
  for (int t = threadIdx.x; t < EPB * n3; t += blockDim.x) {
    const int es = t / n3, x = t - es * n3, e = e0 + es;
    if (e >= d.nElems) continue;
#pragma unroll
    for (int v = 0; v < 4; ++v) sL[(es * 4 + v) * n3 + x] = d.prim[((size_t)e * VP_NF + (v < 3 ? VP_U + v : VP_T)) * n3 + x];
    sJs[es * n3 + x] = d.sJ[(size_t)e * n3 + x];
    if constexpr (CONS) {
#pragma unroll
      for (int c = 0; c < 9; ++c) sMc[(es * 9 + c) * n3 + x] = d.metr[((size_t)e * 9 + c) * n3 + x];
    }
  }
  // surface lifting fluxes of the six sides (lifting_fillflux.t90), stored in this element's face order
  const double sig = B.weakLifting ? 1.0 : -1.0;
  for (int t = threadIdx.x; t < EPB * 6 * n2; t += blockDim.x) {
    const int es = t / (6 * n2), r = t - es * 6 * n2, lsi = r / n2, pq = r - lsi * n2;
    const int e = e0 + es;
    if (e >= d.nElems) continue;
    const int ls = lsi + 1, p = pq % n, q = pq / n;
    const int code = d.elemSide[e * 6 + lsi], s = code >> 3, flip = code & 7;
    int a, b;
    side_to_vol2(N, p, q, flip, ls, a, b);
    const int o = ((es * 6 + lsi) * n2 + a + n * b);
    if constexpr (MORTAR) {
      const int mb = s - (d.nSides - d.nMortars);
      if (mb >= 0) {  // big mortar side (this element is its master): the projected products
        const double* ml = d.mortarLift + (size_t)mb * 12 * n2 + pq;
#pragma unroll
        for (int c = 0; c < 12; ++c) sF[o * 12 + c] = ml[c * n2];
        continue;
      }
    }
    const double* gm = d.geo + (size_t)s * FG_NF * n2 + pq;
    const double se = gm[FG_SURF * n2];
    const double* fm = d.faceM + (size_t)s * FS_NF * n2 + pq;
    double F[4];
    if (s < d.nBCSides) {
      // getboundaryflux.f90:Lifting_GetBoundaryFlux, no-slip walls (BC 3/4)
      const int bt = d.bcType[s];
      const double Tb = (bt == 4) ? d.bcTwall[s] : fm[FS_T * n2];
      const double bval[4] = {0., 0., 0., Tb};
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        const double um = fm[(v < 3 ? FS_U + v : FS_T) * n2];
        const double f = B.weakLifting ? bval[v] : bval[v] - um;
        F[v] = f * se;
      }
    } else {
      const double* fsl = d.faceS + (size_t)s * FS_NF * n2 + pq;
      const double hs = 0.5 * se;
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        const int f = v < 3 ? FS_U + v : FS_T;
        F[v] = (sig * fm[f * n2] + fsl[f * n2]) * hs;
      }
      // slave side of a weak lifting integrates -Flux
      if (flip != 0 && B.weakLifting) for (int v = 0; v < 4; ++v) F[v] = -F[v];
    }
    if constexpr (MORTAR) {
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const double nc = gm[(FG_NX + c) * n2];
#pragma unroll
        for (int v = 0; v < 4; ++v) sF[o * 12 + 4 * c + v] = F[v] * nc;
      }
    } else {
#pragma unroll
      for (int v = 0; v < 4; ++v) sF[o * 4 + v] = F[v];
#pragma unroll
      for (int c = 0; c < 3; ++c) sN[o * 3 + c] = gm[(FG_NX + c) * n2];
    }
  }
  __syncthreads();
  constexpr bool EO = EOShape<n>::ON && !CONS;
  if constexpr (EO) {
    // reference derivatives of the four lifting variables along each direction, line by line in the even-odd
    // form, into sG[es][4 dir + v]
    double eo[8];
    eo_row<n, false>(B, eo);
    eo_sweep_all<n, 4, E>(eo, sL, 4, 0, 0, sG, 12, 0, 4, e0, d.nElems);
  }
  // volume gradient: d/dxi via D_T sweeps, contravariant -> Cartesian with the metrics times sJ
  for (int t = threadIdx.x; t < EPB * n3; t += blockDim.x) {
    const int es = t / n3, x = t - es * n3, e = e0 + es;
    if (e >= d.nElems) continue;
    const int i = x % n, j = (x / n) % n, k = x / n2;
    const double* L = sL + es * 4 * n3;
    double g[12];
    if constexpr (CONS) {
      // lifting_volint.t90:Lifting_VolInt_Conservative: d/dx_c (v) = sJ sum_d sum_l DMat(l, i_d) Ja_d,c(l) v(l), DMat = D_T
      // (doConservativeLifting) or D_Hat_T (doWeakLifting)
      const double* Mc = sMc + es * 9 * n3;
#pragma unroll
      for (int c = 0; c < 12; ++c) g[c] = 0.;
      const int idx3[3] = {i, j, k};
#pragma unroll
      for (int dir = 0; dir < 3; ++dir) {
#pragma unroll
        for (int l = 0; l < n; ++l) {
          const double cf = B.weakLifting ? Bs.DhT(l, idx3[dir]) : Bs.DT(l, idx3[dir]);
          const int xl = dir == 0 ? l + n * (j + n * k) : (dir == 1 ? i + n * (l + n * k) : i + n * (j + n * l));
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            const double f = cf * Mc[(3 * dir + c) * n3 + xl];
#pragma unroll
            for (int v = 0; v < 4; ++v) g[4 * c + v] = fma(f, L[v * n3 + xl], g[4 * c + v]);
          }
        }
      }
      const double sj = sJs[es * n3 + x];
#pragma unroll
      for (int c = 0; c < 12; ++c) g[c] *= sj;
    } else {
      double gx[4], ge[4], gz[4];
      if constexpr (EO) {
#pragma unroll
        for (int v = 0; v < 4; ++v) {
          gx[v] = sG[(es * 12 + v) * n3 + x];
          ge[v] = sG[(es * 12 + 4 + v) * n3 + x];
          gz[v] = sG[(es * 12 + 8 + v) * n3 + x];
        }
      } else {
#pragma unroll
        for (int v = 0; v < 4; ++v) { gx[v] = 0.; ge[v] = 0.; gz[v] = 0.; }
#pragma unroll
        for (int l = 0; l < n; ++l) {
          const double dxi = Bs.DT(l, i), deta = Bs.DT(l, j), dzeta = Bs.DT(l, k);
#pragma unroll
          for (int v = 0; v < 4; ++v) {
            gx[v] = fma(dxi, L[v * n3 + l + n * (j + n * k)], gx[v]);
            ge[v] = fma(deta, L[v * n3 + i + n * (l + n * k)], ge[v]);
            gz[v] = fma(dzeta, L[v * n3 + i + n * (j + n * l)], gz[v]);
          }
        }
      }
      double mJ[9];
      if (d.metrJ) {
#pragma unroll
        for (int c = 0; c < 9; ++c) mJ[c] = d.metrJ[((size_t)e * 9 + c) * n3 + x];
      } else {
        const double sj = sJs[es * n3 + x];
#pragma unroll
        for (int c = 0; c < 9; ++c) mJ[c] = d.metr[((size_t)e * 9 + c) * n3 + x] * sj;
      }
#pragma unroll
      for (int dd = 0; dd < 3; ++dd)
#pragma unroll
        for (int v = 0; v < 4; ++v) g[4 * dd + v] = mJ[dd] * gx[v] + mJ[3 + dd] * ge[v] + mJ[6 + dd] * gz[v];
    }
    if constexpr (GL) {
#pragma unroll
      for (int c = 0; c < 12; ++c) sG[(es * 12 + c) * n3 + x] = g[c];
    } else {
      // Gauss nodes: the surface part reaches every node of the normal lines (DoSurfIntLifting)
      const double sj = sJs[es * n3 + x];
      double sg[12];
#pragma unroll
      for (int c = 0; c < 12; ++c) sg[c] = 0.;
      const int idx3[3] = {i, j, k};
#pragma unroll
      for (int dir = 0; dir < 3; ++dir) {
        const int lsM = dir == 0 ? XI_MINUS : (dir == 1 ? ETA_MINUS : ZETA_MINUS);
        const int lsP = dir == 0 ? XI_PLUS : (dir == 1 ? ETA_PLUS : ZETA_PLUS);
        const int a = dir == 0 ? j : i, b = dir == 2 ? j : k;
        const int l = idx3[dir];
        const double wM = Bs.LhM(l), wP = Bs.LhP(l);
        const int oM = (es * 6 + lsM - 1) * n2 + a + n * b, oP = (es * 6 + lsP - 1) * n2 + a + n * b;
        if constexpr (MORTAR) {
#pragma unroll
          for (int c = 0; c < 12; ++c) sg[c] = fma(sF[oP * 12 + c], wP, fma(sF[oM * 12 + c], wM, sg[c]));
        } else {
#pragma unroll
          for (int v = 0; v < 4; ++v) {
            const double fM = sF[oM * 4 + v] * wM, fP = sF[oP * 4 + v] * wP;
#pragma unroll
            for (int c = 0; c < 3; ++c) sg[4 * c + v] = fma(fP, sN[oP * 3 + c], fma(fM, sN[oM * 3 + c], sg[4 * c + v]));
          }
        }
      }
      // BR1: face gradients are prolonged from the full gradient; BR2: from the volume part only
#pragma unroll
      for (int c = 0; c < 12; ++c) {
        const double full = fma(sg[c], sj, g[c]);
        d.grad[((size_t)e * 12 + c) * n3 + x] = full;
        sG[(es * 12 + c) * n3 + x] = br2 ? g[c] : full;
      }
    }
  }
  __syncthreads();
  if constexpr (GL) {
    // BR2 prolongs the volume part, before the surface part is added
    if (br2) {
      lift_prolong_faces<n, GL, E, MORTAR>(d, B, Bs, sG, sF, sN, sJs, e0, true);
      __syncthreads();
    }
    // surface part (DoSurfIntLifting) on the face nodes l = 0 and l = N of one direction at a time
#pragma unroll 1
    for (int dir = 0; dir < 3; ++dir) {
      for (int t = threadIdx.x; t < EPB * 2 * n2; t += blockDim.x) {
        const int es = t / (2 * n2), r = t - es * 2 * n2, plus = r / n2, ab = r - plus * n2;
        const int e = e0 + es;
        if (e >= d.nElems) continue;
        const int a = ab % n, b = ab / n, l = plus ? N : 0;
        const int ls = plus ? (dir == 0 ? XI_PLUS : (dir == 1 ? ETA_PLUS : ZETA_PLUS))
                            : (dir == 0 ? XI_MINUS : (dir == 1 ? ETA_MINUS : ZETA_MINUS));
        const int x = dir == 0 ? l + n * (a + n * b) : (dir == 1 ? a + n * (l + n * b) : a + n * (b + n * l));
        const double w = (plus ? Bs.LhP(N) : Bs.LhM(0)) * sJs[es * n3 + x];
        const int o = (es * 6 + ls - 1) * n2 + a + n * b;
        double* G = sG + es * 12 * n3 + x;
        if constexpr (MORTAR) {
#pragma unroll
          for (int c = 0; c < 12; ++c) G[c * n3] = fma(sF[o * 12 + c], w, G[c * n3]);
        } else {
#pragma unroll
          for (int v = 0; v < 4; ++v) {
            const double f = sF[o * 4 + v] * w;
#pragma unroll
            for (int c = 0; c < 3; ++c) G[(4 * c + v) * n3] = fma(f, sN[o * 3 + c], G[(4 * c + v) * n3]);
          }
        }
      }
      __syncthreads();
    }
    // BR1 prolongs the full gradient
    if (!br2) lift_prolong_faces<n, GL, E, MORTAR>(d, B, Bs, sG, sF, sN, sJs, e0, false);
    for (int t = threadIdx.x; t < EPB * n3; t += blockDim.x) {
      const int es = t / n3, x = t - es * n3, e = e0 + es;
      if (e >= d.nElems) continue;
#pragma unroll
      for (int c = 0; c < 12; ++c) d.grad[((size_t)e * 12 + c) * n3 + x] = sG[(es * 12 + c) * n3 + x];
    }
  } else {
    lift_prolong_faces<n, GL, E, MORTAR>(d, B, Bs, sG, sF, sN, sJs, e0, br2);
  }
}

// =====================================================================================================
// k_flux: fillflux.f90:FillFlux -- riemann.f90:Riemann_Side + ViscousFlux_Side on inner sides,
// getboundaryflux.f90:GetBoundaryFlux (no-slip walls) on BC sides, times SurfElem; conforming sides only
// (the mortar sides are k_mortar_face's).
// =====================================================================================================
// numerical flux times SurfElem of point pq of side s, with the master's face gradients gL (12 values)
// MORE: the Riemann solvers and split central fluxes beyond LF/HLLC/Roe/RoeEntropyFix with SD/PI (riemann_rotated_more)
template <int n, bool MORE = false>
__device__ __forceinline__ void side_flux(const Dev& d, const Basis& B, int s, int pq, const double* gL, double* Fout) {
  constexpr int n2 = n * n;
  const double* gm = d.geo + (size_t)s * FG_NF * n2 + pq;
  double nv[3], t1[3], t2[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) { nv[c] = gm[(FG_NX + c) * n2]; t1[c] = gm[(FG_T1X + c) * n2]; t2[c] = gm[(FG_T2X + c) * n2]; }
  const double se = gm[FG_SURF * n2];
  // viscosity of each neighbour (its own instance viscosity times its element multiplier)
  const double mu0s = d.mu0[d.sideInst[s]];
  const double mu = d.muScale ? mu0s * d.muScale[d.sideElem[s * 4 + 0]] : mu0s;
  const double lam = mu * B.lambdaFac;
  const double* fm = d.faceM + (size_t)s * FS_NF * n2 + pq;
  double F[5];
  if (s < d.nBCSides) {
    const int bt = d.bcType[s];
    const double rho = fm[FS_RHO * n2], p = fm[FS_P * n2];
    const double vn = fm[FS_U * n2] * nv[0] + fm[FS_V * n2] * nv[1] + fm[FS_W * n2] * nv[2];
    const double pb = pressure_riemann(B, rho, vn, p);
    F[0] = 0.;
    F[1] = pb * nv[0]; F[2] = pb * nv[1]; F[3] = pb * nv[2];
    F[4] = 0.;
    double Fv[5];
    visc_flux_dir(mu, lam, 0., 0., 0., gL, nv[0], nv[1], nv[2], Fv);
    F[1] += Fv[1]; F[2] += Fv[2]; F[3] += Fv[3];
    if (bt != 3) F[4] += Fv[4];
  } else {
    const double* fs = d.faceS + (size_t)s * FS_NF * n2 + pq;
    RotState L, R;
    const double uL = fm[FS_U * n2], vL = fm[FS_V * n2], wL = fm[FS_W * n2];
    const double uR = fs[FS_U * n2], vR = fs[FS_V * n2], wR = fs[FS_W * n2];
    L.rho = fm[FS_RHO * n2]; L.srho = fm[FS_SRHO * n2]; L.E = fm[FS_E * n2]; L.p = fm[FS_P * n2];
    R.rho = fs[FS_RHO * n2]; R.srho = fs[FS_SRHO * n2]; R.E = fs[FS_E * n2]; R.p = fs[FS_P * n2];
    L.v1 = uL * nv[0] + vL * nv[1] + wL * nv[2];
    L.v2 = uL * t1[0] + vL * t1[1] + wL * t1[2];
    L.v3 = uL * t2[0] + vL * t2[1] + wL * t2[2];
    R.v1 = uR * nv[0] + vR * nv[1] + wR * nv[2];
    R.v2 = uR * t1[0] + vR * t1[1] + wR * t1[2];
    R.v3 = uR * t2[0] + vR * t2[1] + wR * t2[2];
    double Fr[5];
    if constexpr (MORE) riemann_rotated_more(B.riemann, B.splitDG, B, L, R, Fr);
    else riemann_rotated(B.riemann, B.splitDG, B, L, R, Fr);
    F[0] = Fr[0];
#pragma unroll
    for (int c = 0; c < 3; ++c) F[1 + c] = nv[c] * Fr[1] + t1[c] * Fr[2] + t2[c] * Fr[3];
    F[4] = Fr[4];
    double gR[12];
#pragma unroll
    for (int c = 0; c < 12; ++c) gR[c] = d.gradS[((size_t)s * 12 + c) * n2 + pq];
    double FvL[5], FvR[5];
    const double muR = d.muScale ? mu0s * d.muScale[d.sideElem[s * 4 + 2]] : mu0s;
    visc_flux_dir(mu, lam, uL, vL, wL, gL, nv[0], nv[1], nv[2], FvL);
    visc_flux_dir(muR, muR * B.lambdaFac, uR, vR, wR, gR, nv[0], nv[1], nv[2], FvR);
#pragma unroll
    for (int v = 1; v < 5; ++v) F[v] += 0.5 * (FvL[v] + FvR[v]);
  }
#pragma unroll
  for (int v = 0; v < 5; ++v) Fout[v] = F[v] * se;
}

template <int n, bool MORE = false>
__global__ void __launch_bounds__(256) k_flux(Dev d, Basis B) {
  constexpr int n2 = n * n;
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  const int s = idx / n2, pq = idx - s * n2;
  if (s >= d.nFluxSides) return;
  double gL[12], F[5];
#pragma unroll
  for (int c = 0; c < 12; ++c) gL[c] = d.gradM[((size_t)s * 12 + c) * n2 + pq];
  side_flux<n, MORE>(d, B, s, pq, gL, F);
#pragma unroll
  for (int v = 0; v < 5; ++v) d.flux[((size_t)s * 5 + v) * n2 + pq] = F[v];
}

// =====================================================================================================
// Mortar interfaces (mortar.f90, fillmortar.t90), one CTA per big mortar side m. Small side im covers the
// quadrant iNb = im % 2, jNb = im / 2 of the big side (type 1), the half jNb = im (type 2, split in eta)
// or iNb = im (type 3, split in xi), in the big side's master orientation.
// =====================================================================================================
// fillmortar.t90:U_Mortar: nv fields in[v][p + n*q] of the big side interpolated to out[im][v][n2];
// tmp holds [2][nv][n2]. Ends with a barrier.
template <int n>
__device__ void mortar_interp(const MortarDev& M, int type, int nv, const double* in, double* tmp, double* out) {
  constexpr int n2 = n * n;
  if (type == 1) {
    for (int t = threadIdx.x; t < 2 * nv * n2; t += blockDim.x) {  // eta: tmp[jNb]
      const int k = t / (nv * n2), r = t - k * nv * n2, v = r / n2, pq = r - v * n2, p = pq % n, q = pq / n;
      const double* Mq = k ? M.M02 : M.M01;
      double acc = 0.;
#pragma unroll
      for (int l = 0; l < n; ++l) acc = fma(Mq[l * n + q], in[v * n2 + p + n * l], acc);
      tmp[t] = acc;
    }
    __syncthreads();
    for (int t = threadIdx.x; t < 4 * nv * n2; t += blockDim.x) {  // xi
      const int im = t / (nv * n2), r = t - im * nv * n2, v = r / n2, pq = r - v * n2, p = pq % n, q = pq / n;
      const double* Mp = (im & 1) ? M.M02 : M.M01;
      const double* T = tmp + ((im >> 1) * nv + v) * n2;
      double acc = 0.;
#pragma unroll
      for (int l = 0; l < n; ++l) acc = fma(Mp[l * n + p], T[l + n * q], acc);
      out[t] = acc;
    }
  } else {
    for (int t = threadIdx.x; t < 2 * nv * n2; t += blockDim.x) {
      const int im = t / (nv * n2), r = t - im * nv * n2, v = r / n2, pq = r - v * n2, p = pq % n, q = pq / n;
      const double* Mx = im ? M.M02 : M.M01;
      double acc = 0.;
      if (type == 2) {
#pragma unroll
        for (int l = 0; l < n; ++l) acc = fma(Mx[l * n + q], in[v * n2 + p + n * l], acc);
      } else {
#pragma unroll
        for (int l = 0; l < n; ++l) acc = fma(Mx[l * n + p], in[v * n2 + l + n * q], acc);
      }
      out[t] = acc;
    }
  }
  __syncthreads();
}

// fillmortar.t90:Flux_Mortar: nv fields in[im][v][n2] of the small sides projected onto the big side,
// out[v][p + n*q]; tmp holds [2][nv][n2]
template <int n>
__device__ void mortar_project(const MortarDev& M, int type, int nv, const double* in, double* tmp, double* out) {
  constexpr int n2 = n * n;
  if (type == 1) {
    for (int t = threadIdx.x; t < 2 * nv * n2; t += blockDim.x) {  // xi: tmp[jNb]
      const int k = t / (nv * n2), r = t - k * nv * n2, v = r / n2, pq = r - v * n2, p = pq % n, q = pq / n;
      const double* F1 = in + ((2 * k) * nv + v) * n2;
      const double* F2 = in + ((2 * k + 1) * nv + v) * n2;
      double acc = 0.;
#pragma unroll
      for (int l = 0; l < n; ++l) acc = fma(M.M10[l * n + p], F1[l + n * q], fma(M.M20[l * n + p], F2[l + n * q], acc));
      tmp[t] = acc;
    }
    __syncthreads();
    for (int t = threadIdx.x; t < nv * n2; t += blockDim.x) {  // eta
      const int v = t / n2, pq = t - v * n2, p = pq % n, q = pq / n;
      const double* T1 = tmp + v * n2;
      const double* T2 = tmp + (nv + v) * n2;
      double acc = 0.;
#pragma unroll
      for (int l = 0; l < n; ++l) acc = fma(M.M10[l * n + q], T1[p + n * l], fma(M.M20[l * n + q], T2[p + n * l], acc));
      out[t] = acc;
    }
  } else {
    for (int t = threadIdx.x; t < nv * n2; t += blockDim.x) {
      const int v = t / n2, pq = t - v * n2, p = pq % n, q = pq / n;
      const double* F1 = in + v * n2;
      const double* F2 = in + (nv + v) * n2;
      double acc = 0.;
      if (type == 2) {
#pragma unroll
        for (int l = 0; l < n; ++l) acc = fma(M.M10[l * n + q], F1[p + n * l], fma(M.M20[l * n + q], F2[p + n * l], acc));
      } else {
#pragma unroll
        for (int l = 0; l < n; ++l) acc = fma(M.M10[l * n + p], F1[l + n * q], fma(M.M20[l * n + p], F2[l + n * q], acc));
      }
      out[t] = acc;
    }
  }
}

// between k_prep and k_lift: the big side's conservative face state interpolated to its small sides' master
// slots, turned into face primitives (dg.f90:372-416, U_Mortar before GetPrimitiveStateSurface), and the
// small sides' lifting fluxes times normal (lifting_fillflux.t90) projected onto the big side
// (lifting_br1.t90:106-109, lifting_br2.t90:103-106) for k_lift<MORTAR>.
template <int n>
__global__ void __launch_bounds__(256, 2) k_mortar_pre(Dev d, Basis B, MortarDev M) {
  constexpr int n2 = n * n;
  extern __shared__ double smem[];
  double* sUb = smem;          // [5][n2] big side U
  double* sT = sUb + 5 * n2;   // [2][12][n2]
  double* sUs = sT + 24 * n2;  // [4][5][n2] small sides' U
  double* sFN = sUs + 20 * n2; // [4][12][n2] small sides' lifting flux times normal
  const int m = blockIdx.x;
  const int* info = M.info + 6 * m;
  const int type = info[0], sb = info[1], nm = type == 1 ? 4 : 2;
  for (int pq = threadIdx.x; pq < n2; pq += blockDim.x) {
    const double* fm = d.faceM + (size_t)sb * FS_NF * n2 + pq;
    const double rho = fm[FS_RHO * n2];
    sUb[pq] = rho;
    sUb[n2 + pq] = rho * fm[FS_U * n2];
    sUb[2 * n2 + pq] = rho * fm[FS_V * n2];
    sUb[3 * n2 + pq] = rho * fm[FS_W * n2];
    sUb[4 * n2 + pq] = fm[FS_E * n2];
  }
  __syncthreads();
  mortar_interp<n>(M, type, 5, sUb, sT, sUs);
  const double sig = B.weakLifting ? 1.0 : -1.0;
  for (int t = threadIdx.x; t < nm * n2; t += blockDim.x) {
    const int im = t / n2, pq = t - im * n2, ss = info[2 + im];
    double c[5];
#pragma unroll
    for (int v = 0; v < 5; ++v) c[v] = sUs[(im * 5 + v) * n2 + pq];
    const double srho = 1.0 / c[0];
    const double vx = c[1] * srho, vy = c[2] * srho, vz = c[3] * srho;
    const double pp = B.kappaM1 * (c[4] - 0.5 * (c[1] * vx + c[2] * vy + c[3] * vz));
    const double T = pp * srho * B.sR;
    double* dst = d.faceM + (size_t)ss * FS_NF * n2 + pq;
    dst[FS_RHO * n2] = c[0]; dst[FS_E * n2] = c[4]; dst[FS_SRHO * n2] = srho;
    dst[FS_U * n2] = vx; dst[FS_V * n2] = vy; dst[FS_W * n2] = vz; dst[FS_P * n2] = pp; dst[FS_T * n2] = T;
    const double* fsl = d.faceS + (size_t)ss * FS_NF * n2 + pq;
    const double* gm = d.geo + (size_t)ss * FG_NF * n2 + pq;
    const double hs = 0.5 * gm[FG_SURF * n2];
    const double um[4] = {vx, vy, vz, T};
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const double F = (sig * um[v] + fsl[(v < 3 ? FS_U + v : FS_T) * n2]) * hs;
#pragma unroll
      for (int cc = 0; cc < 3; ++cc) sFN[(im * 12 + 4 * cc + v) * n2 + pq] = F * gm[(FG_NX + cc) * n2];
    }
  }
  __syncthreads();
  mortar_project<n>(M, type, 12, sFN, sT, d.mortarLift + (size_t)m * 12 * n2);
}

// between k_flux and the volume kernel: the big side's face gradients interpolated to its small sides
// (lifting_br1.t90:175-178, lifting_br2.t90:176-181), the small sides' numerical fluxes (fillflux.f90, master viscosity of the big
// element), and their projection onto the big side (dg.f90:625, Flux_Mortar)
template <int n>
__global__ void __launch_bounds__(256, 2) k_mortar_face(Dev d, Basis B, MortarDev M) {
  constexpr int n2 = n * n;
  extern __shared__ double smem[];
  double* sGb = smem;           // [12][n2] big side gradients
  double* sT = sGb + 12 * n2;   // [2][12][n2]
  double* sGs = sT + 24 * n2;   // [4][12][n2]
  double* sF = sGs + 48 * n2;   // [4][5][n2]
  const int m = blockIdx.x;
  const int* info = M.info + 6 * m;
  const int type = info[0], sb = info[1], nm = type == 1 ? 4 : 2;
  for (int t = threadIdx.x; t < 12 * n2; t += blockDim.x) sGb[t] = d.gradM[(size_t)sb * 12 * n2 + t];
  __syncthreads();
  mortar_interp<n>(M, type, 12, sGb, sT, sGs);
  for (int t = threadIdx.x; t < nm * n2; t += blockDim.x) {
    const int im = t / n2, pq = t - im * n2, ss = info[2 + im];
    double gL[12], F[5];
#pragma unroll
    for (int c = 0; c < 12; ++c) gL[c] = sGs[(im * 12 + c) * n2 + pq];
    side_flux<n>(d, B, ss, pq, gL, F);
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      d.flux[((size_t)ss * 5 + v) * n2 + pq] = F[v];
      sF[(im * 5 + v) * n2 + pq] = F[v];
    }
  }
  __syncthreads();
  mortar_project<n>(M, type, 5, sF, sT, d.flux + (size_t)sb * 5 * n2);
}

// stage parameters of the fused LSERK update
struct Stage {
  int mode;        // 0: write Ut only (fg_time_derivative); 1: first RK stage; 2: later RK stage;
                   // 3: write J u_t (before ApplyJacobianCons) for the overintegration kernel
  double rkA;      // RKA(stage) (stage >= 2)
  double rkB;      // RKb(stage)
};

// surface integral + Jacobian + source + RK update for the node owned by this thread
// SURF = false: the surface integral was added face-parallel before (gl_surface_faces)
template <int n, bool GL, bool SURF = true>
__device__ __forceinline__ void finish_node(const Dev& d, const SBasis<n>& Bs, const Stage& st, const double* sFl, int es, int e, int x,
                                            double* ut) {
  constexpr int n2 = n * n, n3 = n * n * n, N = n - 1;
  const int i = x % n, j = (x / n) % n, k = x / n2;
  const int idx3[3] = {i, j, k};
#pragma unroll
  for (int dir = 0; dir < (SURF ? 3 : 0); ++dir) {
    const int lsM = dir == 0 ? XI_MINUS : (dir == 1 ? ETA_MINUS : ZETA_MINUS);
    const int lsP = dir == 0 ? XI_PLUS : (dir == 1 ? ETA_PLUS : ZETA_PLUS);
    const int a = dir == 0 ? j : i, b = dir == 2 ? j : k;
    const int l = idx3[dir];
    double wM, wP;
    if (GL) { wM = (l == 0) ? Bs.LhM(0) : 0.; wP = (l == N) ? Bs.LhP(N) : 0.; }
    else { wM = Bs.LhM(l); wP = Bs.LhP(l); }
    if (wM != 0.) {
      const int o = (es * 6 + lsM - 1) * n2 + a + n * b;
#pragma unroll
      for (int v = 0; v < 5; ++v) ut[v] = fma(sFl[o * 5 + v], wM, ut[v]);
    }
    if (wP != 0.) {
      const int o = (es * 6 + lsP - 1) * n2 + a + n * b;
#pragma unroll
      for (int v = 0; v < 5; ++v) ut[v] = fma(sFl[o * 5 + v], wP, ut[v]);
    }
  }
  const double sj = d.sJ[(size_t)e * n3 + x];
  const int inst = d.elemInst[e];
  const double dpdx = d.dpdx[inst];
  double src[5] = {0., 0., 0., 0., 0.};
  const bool haveSrc = d.srcPar != nullptr;
  if (haveSrc) {
    // exactfunc.f90:CalcSource CASE(4): rho = m_i = 2 + A sin(omega sum(x) - a t), E = rho^2
    const double* P = d.srcPar;
    const double* X = d.elemX + (size_t)e * 3 * n3 + x;
    const double ph = P[0] * (X[0] + X[n3] + X[2 * n3]) - P[1] * d.tStage[inst];
    double sn, cs;
    sincos(ph, &sn, &cs);
    const double s2 = 2. * sn * cs;
    src[0] = P[2] * cs;
    src[1] = src[2] = src[3] = fma(P[3], cs, P[4] * s2);
    src[4] = fma(P[5], cs, fma(P[6], s2, P[7] * sn));
  }
  if (st.mode == 3) {
    // dg.f90:656-662: Ut = -Ut, sources in reference space (divided by sJ); the Jacobian follows the filter
#pragma unroll
    for (int v = 0; v < 5; ++v) ut[v] = -ut[v];
    if (dpdx != 0.) { ut[1] -= dpdx / sj; ut[4] -= dpdx / sj * d.bulkVel[inst]; }
    if (haveSrc) {
#pragma unroll
      for (int v = 0; v < 5; ++v) ut[v] += src[v] / sj;
    }
    if (d.forceField) {
      const double F = d.forceField[(size_t)e * n3 + x];
      ut[1] += F / sj;
      ut[4] += F / sj * d.bulkVel[inst];
    }
#pragma unroll
    for (int v = 0; v < 5; ++v) d.Ut[((size_t)e * 5 + v) * n3 + x] = ut[v];
    return;
  }
  const double msj = -sj;
#pragma unroll
  for (int v = 0; v < 5; ++v) ut[v] *= msj;
  if (dpdx != 0.) {  // channel testcase.f90:TestcaseSource, applied before ApplyJacobian
    ut[1] -= dpdx;
    ut[4] -= dpdx * d.bulkVel[inst];
  }
  if (haveSrc) {
#pragma unroll
    for (int v = 0; v < 5; ++v) ut[v] += src[v];
  }
  if (d.forceField) {  // additional per-node body force of the same form
    const double F = d.forceField[(size_t)e * n3 + x];
    ut[1] += F;
    ut[4] += F * d.bulkVel[inst];
  }
  if (st.mode == 0) {
#pragma unroll
    for (int v = 0; v < 5; ++v) d.Ut[((size_t)e * 5 + v) * n3 + x] = ut[v];
    return;
  }
  const double bdt = st.rkB * d.dt[inst];
#pragma unroll
  for (int v = 0; v < 5; ++v) {
    const size_t o = ((size_t)e * 5 + v) * n3 + x;
    double r = ut[v];
    if (st.mode == 2) r = fma(-st.rkA, d.Ut_tmp[o], r);
    d.Ut_tmp[o] = r;
    d.U[o] = fma(bdt, r, d.U[o]);
  }
}

// loads the six sides' numerical fluxes into shared memory in this element's face order,
// with the sign of the slave side (surfint.t90: -Flux_slave)
template <int n, int E = 0>
__device__ __forceinline__ void load_face_fluxes(const Dev& d, double* sFl, int e0) {
  constexpr int n2 = n * n, EPB = Shape<n, E>::EPB, N = n - 1;
  for (int t = threadIdx.x; t < EPB * 6 * n2; t += blockDim.x) {
    const int es = t / (6 * n2), r = t - es * 6 * n2, lsi = r / n2, pq = r - lsi * n2;
    const int e = e0 + es;
    if (e >= d.nElems) continue;
    const int ls = lsi + 1, p = pq % n, q = pq / n;
    const int code = d.elemSide[e * 6 + lsi], s = code >> 3, flip = code & 7;
    int a, b;
    side_to_vol2(N, p, q, flip, ls, a, b);
    const int o = (es * 6 + lsi) * n2 + a + n * b;
    const double sg = flip == 0 ? 1.0 : -1.0;
#pragma unroll
    for (int v = 0; v < 5; ++v) sFl[o * 5 + v] = sg * d.flux[((size_t)s * 5 + v) * n2 + pq];
  }
}

// surfint.t90:SurfInt on Gauss-Lobatto nodes, face-parallel: the flux of each face point times L_HatMinus(0) /
// L_HatPlus(N) added to its face node's entry of sA ([EPB][5][n3]), one direction (two opposite faces, disjoint node
// sets) at a time, so that no lane of a warp idles on interior nodes (the FP64 pipe pays for idle lanes). Ends with
// a barrier.
template <int n, int E = 0>
__device__ __forceinline__ void gl_surface_faces(const SBasis<n>& Bs, const double* sFl, double* sA, int e0, int nElems) {
  constexpr int n2 = n * n, n3 = n2 * n, EPB = Shape<n, E>::EPB, N = n - 1;
#pragma unroll 1
  for (int dir = 0; dir < 3; ++dir) {
    for (int t = threadIdx.x; t < EPB * 2 * n2; t += blockDim.x) {
      const int es = t / (2 * n2), r = t - es * 2 * n2, side = r / n2, ab = r - side * n2;
      if (e0 + es >= nElems) continue;
      const int ls = side == 0 ? (dir == 0 ? XI_MINUS : (dir == 1 ? ETA_MINUS : ZETA_MINUS))
                               : (dir == 0 ? XI_PLUS : (dir == 1 ? ETA_PLUS : ZETA_PLUS));
      const int x = face_node(ls, ab % n, ab / n, side == 0 ? 0 : N, n);
      const double w = side == 0 ? Bs.LhM(0) : Bs.LhP(N);
      const double* F = sFl + ((es * 6 + ls - 1) * n2 + ab) * 5;
      double* A = sA + es * 5 * n3 + x;
#pragma unroll
      for (int v = 0; v < 5; ++v) A[v * n3] = fma(F[v], w, A[v * n3]);
    }
    __syncthreads();
  }
}

// =====================================================================================================
// k_vol_weak: volint.f90:VolInt_weakForm (advective + viscous fluxes, VolInt_Metrics, D_Hat^T sweeps),
// surfint.t90:SurfInt, Ut=-Ut, ApplyJacobian, and the LSERK stage update.
// =====================================================================================================
template <int n, bool GL, int E = 0>
__global__ void __launch_bounds__(Shape<n, E>::THREADS) k_vol_weak(Dev d, Basis B, Stage st) {
  using S = Shape<n, E>;
  constexpr int n2 = S::n2, n3 = S::n3, EPB = S::EPB;
  extern __shared__ double smem[];
  double* sD = smem;
  double* sT = big_base<n>(d, smem, Big<n, E>::weak);  // [EPB][15][n3] transformed fluxes f~(5) g~(5) h~(5)
  double* sFl = sT + EPB * 15 * n3;      // [EPB][6][n2][5]
  load_basis_smem<n>(B, sD);
  SBasis<n> Bs{sD};
  const int e0 = d.volBegin + blockIdx.x * EPB;
  load_face_fluxes<n, E>(d, sFl, e0);
  for (int t = threadIdx.x; t < EPB * n3; t += blockDim.x) {
    const int es = t / n3, x = t - es * n3, e = e0 + es;
    if (e >= d.nElems) continue;
    double u[5];
#pragma unroll
    for (int v = 0; v < 5; ++v) u[v] = d.U[((size_t)e * 5 + v) * n3 + x];
    const double vx = d.prim[((size_t)e * VP_NF + VP_U) * n3 + x];
    const double vy = d.prim[((size_t)e * VP_NF + VP_V) * n3 + x];
    const double vz = d.prim[((size_t)e * VP_NF + VP_W) * n3 + x];
    const double p = d.prim[((size_t)e * VP_NF + VP_P) * n3 + x];
    double g[12];
#pragma unroll
    for (int c = 0; c < 12; ++c) g[c] = d.grad[((size_t)e * 12 + c) * n3 + x];
    const double mu = elem_mu(d, e);
    const double lam = mu * B.lambdaFac;
    // physical flux (advective + viscous, flux.f90:EvalFlux3D_Point + EvalDiffFlux3D_Point)
    const double div = g[0] + g[5] + g[10];
    const double mdiv = (2.0 / 3.0) * div;
    const double txx = mu * (2.0 * g[0] - mdiv), tyy = mu * (2.0 * g[5] - mdiv), tzz = mu * (2.0 * g[10] - mdiv);
    const double txy = mu * (g[4] + g[1]), txz = mu * (g[8] + g[2]), tyz = mu * (g[9] + g[6]);
    const double Ep = u[4] + p;
    double f[5], gg[5], h[5];
    f[0] = u[1];
    f[1] = fma(u[1], vx, p) - txx;
    f[2] = u[1] * vy - txy;
    f[3] = u[1] * vz - txz;
    f[4] = Ep * vx - (txx * vx + txy * vy + txz * vz) - lam * g[3];
    gg[0] = u[2];
    gg[1] = u[2] * vx - txy;
    gg[2] = fma(u[2], vy, p) - tyy;
    gg[3] = u[2] * vz - tyz;
    gg[4] = Ep * vy - (txy * vx + tyy * vy + tyz * vz) - lam * g[7];
    h[0] = u[3];
    h[1] = u[3] * vx - txz;
    h[2] = u[3] * vy - tyz;
    h[3] = fma(u[3], vz, p) - tzz;
    h[4] = Ep * vz - (txz * vx + tyz * vy + tzz * vz) - lam * g[11];
    // VolInt_Metrics
#pragma unroll
    for (int dd = 0; dd < 3; ++dd) {
      const double m1 = d.metr[((size_t)e * 9 + 3 * dd + 0) * n3 + x];
      const double m2 = d.metr[((size_t)e * 9 + 3 * dd + 1) * n3 + x];
      const double m3 = d.metr[((size_t)e * 9 + 3 * dd + 2) * n3 + x];
#pragma unroll
      for (int v = 0; v < 5; ++v) sT[(es * 15 + 5 * dd + v) * n3 + x] = f[v] * m1 + gg[v] * m2 + h[v] * m3;
    }
  }
  __syncthreads();
  for (int t = threadIdx.x; t < EPB * n3; t += blockDim.x) {
    const int es = t / n3, x = t - es * n3, e = e0 + es;
    if (e >= d.nElems) continue;
    const int i = x % n, j = (x / n) % n, k = x / n2;
    const double* T = sT + es * 15 * n3;
    double ut[5] = {0., 0., 0., 0., 0.};
#pragma unroll
    for (int l = 0; l < n; ++l) {
      const double ci = Bs.DhT(l, i), cj = Bs.DhT(l, j), ck = Bs.DhT(l, k);
      const int xi = l + n * (j + n * k), xj = i + n * (l + n * k), xk = i + n * (j + n * l);
#pragma unroll
      for (int v = 0; v < 5; ++v) {
        ut[v] = fma(ci, T[v * n3 + xi], ut[v]);
        ut[v] = fma(cj, T[(5 + v) * n3 + xj], ut[v]);
        ut[v] = fma(ck, T[(10 + v) * n3 + xk], ut[v]);
      }
    }
    finish_node<n, GL>(d, Bs, st, sFl, es, e, x, ut);
  }
}

// two-point volume flux of a node pair in contravariant form, without its constant factor (in the scaled
// DVolSurf): PI or SD (split_pair_flux) in the PI/SD kernels, any SplitDG (split_pair_flux_gen) in the GEN ones.
template <bool GEN>
__device__ __forceinline__ void split_pair(int sd, bool pi, const Basis& B, double ra, double ua, double va, double wa, double pa, double ha,
                                           double rb, double ub, double vb, double wb, double pb, double hb, double ms0, double ms1, double ms2,
                                           double* G) {
  if constexpr (GEN) split_pair_flux_gen(sd, B, ra, ua, va, wa, pa, ha, rb, ub, vb, wb, pb, hb, ms0, ms1, ms2, G);
  else split_pair_flux(pi, ra, ua, va, wa, pa, ha, rb, ub, vb, wb, pb, hb, ms0, ms1, ms2, G);
}

// =====================================================================================================
// k_vol_split: volint.f90:VolInt_splitForm with SplitVolumeFluxPI / SD (Gauss-Lobatto nodes, n nodes
// per line handled by an n-lane segment of a warp), viscous part in weak form, surface integral,
// Jacobian, LSERK update. Each two-point flux of a line is evaluated once: lane a evaluates the pair
// (a, a+dd mod n) for dd = 1..n/2-1, applies its own coefficient, and hands the unscaled flux to lane
// a+dd with a warp shuffle, which applies its coefficient with one FMA per component; the pairs at
// distance n/2 follow in a pass of their own, one thread per pair (half the warps). The coefficients DVolSurf(l,i) are pre-scaled in shared
// memory by the split flux's constant factors (exact: powers of two).
// Shared memory: one region holds the split-flux inputs (rho, u, v, w, p-term, H-term and the metrics)
// and afterwards the transformed viscous fluxes, so that two CTAs of 8^3 nodes fit on one SM.
// =====================================================================================================
// GEN: any SplitDG (MO, DU, KG, CH, IR as well as SD, PI), with the kind chosen at run time; the PI/SD kernel
// stays free of the other kinds' code.
template <int n, bool GEN = false>
__global__ void __launch_bounds__(Shape<n>::THREADS, (n == 8 ? 2 : 1)) k_vol_split(Dev d, Basis B, Stage st) {
  using S = Shape<n>;
  constexpr int n2 = S::n2, n3 = S::n3, EPB = S::EPB;
  static_assert(n == 8 || n == 4 || n == 2, "split kernel expects 2, 4 or 8 nodes per line");
  extern __shared__ double smem[];
  double* sD = smem;
  double* sC = sD + SBasis<n>::SIZE;   // [2][n2]: DVolSurf(l,i) x density factor, x factor of the other components
  double* sR = sC + 2 * n2;            // [EPB][15][n3]: rho, u, v, w, p-term, H-term, metrics(9); later viscous fluxes(12)
  double* sA = sR + EPB * 15 * n3;     // [EPB][5][n3] split-flux divergence
  double* sFl = sA + EPB * 5 * n3;     // [EPB][6][n2][5]
  load_basis_smem<n>(B, sD);
  SBasis<n> Bs{sD};
  const bool pi = B.splitDG == 4;
  const int skind = B.splitDG;
  {
    // SplitVolumeFluxPI: 1/4 (density), 1/8 (others) of the contravariant sums below; SD: 1/2
    double f0 = pi ? 0.25 : 0.5, f1 = pi ? 0.125 : 0.5;
    if constexpr (GEN) split_factors(skind, f0, f1);
    for (int t = threadIdx.x; t < n2; t += blockDim.x) { sC[t] = B.DVS[t] * f0; sC[n2 + t] = B.DVS[t] * f1; }
  }
  const int e0 = d.volBegin + blockIdx.x * EPB;
  load_face_fluxes<n>(d, sFl, e0);
  for (int t = threadIdx.x; t < EPB * n3; t += blockDim.x) {
    const int es = t / n3, x = t - es * n3, e = e0 + es;
    if (e >= d.nElems) continue;
    double* Q = sR + es * 15 * n3;
    const double u0 = d.U[((size_t)e * 5 + 0) * n3 + x], u4 = d.U[((size_t)e * 5 + 4) * n3 + x];
    const double srho = d.prim[((size_t)e * VP_NF + VP_SRHO) * n3 + x];
    const double p = d.prim[((size_t)e * VP_NF + VP_P) * n3 + x];
    Q[x] = u0;
    Q[n3 + x] = d.prim[((size_t)e * VP_NF + VP_U) * n3 + x];
    Q[2 * n3 + x] = d.prim[((size_t)e * VP_NF + VP_V) * n3 + x];
    Q[3 * n3 + x] = d.prim[((size_t)e * VP_NF + VP_W) * n3 + x];
    if constexpr (GEN) {
      split_node_inputs(skind, u0, Q[n3 + x], Q[2 * n3 + x], Q[3 * n3 + x], p, u4, srho, Q[x], Q[4 * n3 + x], Q[5 * n3 + x]);
    } else if (pi) {
      Q[4 * n3 + x] = 4.0 * p;
      Q[5 * n3 + x] = (u4 + p) * srho;
    } else {
      Q[4 * n3 + x] = p;
      Q[5 * n3 + x] = u4 + p;
    }
#pragma unroll
    for (int c = 0; c < 9; ++c) Q[(6 + c) * n3 + x] = d.metr[((size_t)e * 9 + c) * n3 + x];
  }
  __syncthreads();
  // split-flux divergence, one direction at a time; the sum carries over from the previous direction
  const int lane = threadIdx.x & 31;
  const int segBase = lane & ~(n - 1);
#pragma unroll 1
  for (int dir = 0; dir < 3; ++dir) {
    for (int t = threadIdx.x; t < EPB * n3; t += blockDim.x) {
      const int es = t / n3, r = t - es * n3;
      const int e = e0 + es;
      const bool valid = e < d.nElems;
      const int a = r % n, c1 = (r / n) % n, c2 = r / n2;  // a = index along the line
      int xa;
      if (dir == 0) xa = a + n * (c1 + n * c2);
      else if (dir == 1) xa = c1 + n * (a + n * c2);
      else xa = c1 + n * (c2 + n * a);
      const int stride = dir == 0 ? 1 : (dir == 1 ? n : n2);
      const int xline = xa - a * stride;
      const double* Q = sR + es * 15 * n3;
      const double* Mm = Q + (6 + 3 * dir) * n3;
      const double ra = Q[xa], ua = Q[n3 + xa], va = Q[2 * n3 + xa], wa = Q[3 * n3 + xa], pa = Q[4 * n3 + xa], ha = Q[5 * n3 + xa];
      const double ma0 = Mm[xa], ma1 = Mm[n3 + xa], ma2 = Mm[2 * n3 + xa];
      double acc[5];
#pragma unroll
      for (int v = 0; v < 5; ++v) acc[v] = (dir == 0) ? 0. : sA[(es * 5 + v) * n3 + xa];
#pragma unroll
      for (int dd = 1; dd < n / 2; ++dd) {
        const int bI = (a + dd) & (n - 1);
        const int xb = xline + bI * stride;
        const double rb = Q[xb], ub = Q[n3 + xb], vb = Q[2 * n3 + xb], wb = Q[3 * n3 + xb], pb = Q[4 * n3 + xb], hb = Q[5 * n3 + xb];
        const double ms0 = ma0 + Mm[xb], ms1 = ma1 + Mm[n3 + xb], ms2 = ma2 + Mm[2 * n3 + xb];
        double G[5];
        split_pair<GEN>(skind, pi, B, ra, ua, va, wa, pa, ha, rb, ub, vb, wb, pb, hb, ms0, ms1, ms2, G);
        // contribution to node i from its partner l: DVolSurf(l, i)
        const double o0 = sC[bI * n + a], o1 = sC[n2 + bI * n + a];
        acc[0] = fma(o0, G[0], acc[0]);
#pragma unroll
        for (int v = 1; v < 5; ++v) acc[v] = fma(o1, G[v], acc[v]);
        {
          // receive the flux of the pair (a-dd, a) from lane a-dd
          const int aS = (a - dd) & (n - 1);
          const int src = segBase | aS;
          const double r0 = sC[aS * n + a], r1 = sC[n2 + aS * n + a];
          const double g0 = __shfl_sync(0xffffffffu, G[0], src);
          acc[0] = fma(r0, g0, acc[0]);
#pragma unroll
          for (int v = 1; v < 5; ++v) {
            const double gv = __shfl_sync(0xffffffffu, G[v], src);
            acc[v] = fma(r1, gv, acc[v]);
          }
        }
      }
      if (valid) {
#pragma unroll
        for (int v = 0; v < 5; ++v) sA[(es * 5 + v) * n3 + xa] = acc[v];
      }
    }
    __syncthreads();
  }
  // the pairs at distance n/2, (a, a+n/2) with a < n/2: each evaluated once, by one thread that adds it to
  // both nodes; one direction at a time (every node is in exactly one such pair per direction)
  {
    constexpr int HP = n / 2, NPAIR = n2 * HP;
#pragma unroll 1
    for (int dir = 0; dir < 3; ++dir) {
      for (int t = threadIdx.x; t < EPB * NPAIR; t += blockDim.x) {
        const int es = t / NPAIR, r = t - es * NPAIR;
        if (e0 + es >= d.nElems) continue;
        const int a = r % HP, c1 = (r / HP) % n, c2 = r / (HP * n);
        const int stride = dir == 0 ? 1 : (dir == 1 ? n : n2);
        const int xline = dir == 0 ? n * (c1 + n * c2) : (dir == 1 ? c1 + n2 * c2 : c1 + n * c2);
        const int xa = xline + a * stride, xb = xa + HP * stride, b = a + HP;
        const double* Q = sR + es * 15 * n3;
        const double* Mm = Q + (6 + 3 * dir) * n3;
        double G[5];
        split_pair<GEN>(skind, pi, B, Q[xa], Q[n3 + xa], Q[2 * n3 + xa], Q[3 * n3 + xa], Q[4 * n3 + xa], Q[5 * n3 + xa], Q[xb], Q[n3 + xb],
                        Q[2 * n3 + xb], Q[3 * n3 + xb], Q[4 * n3 + xb], Q[5 * n3 + xb], Mm[xa] + Mm[xb], Mm[n3 + xa] + Mm[n3 + xb],
                        Mm[2 * n3 + xa] + Mm[2 * n3 + xb], G);
        double* A = sA + es * 5 * n3;
        // node a from partner b: DVolSurf(b, a); node b from partner a: DVolSurf(a, b)
        A[xa] = fma(sC[b * n + a], G[0], A[xa]);
        A[xb] = fma(sC[a * n + b], G[0], A[xb]);
#pragma unroll
        for (int v = 1; v < 5; ++v) {
          A[v * n3 + xa] = fma(sC[n2 + b * n + a], G[v], A[v * n3 + xa]);
          A[v * n3 + xb] = fma(sC[n2 + a * n + b], G[v], A[v * n3 + xb]);
        }
      }
      __syncthreads();
    }
  }
  gl_surface_faces<n>(Bs, sFl, sA, e0, d.nElems);
  // viscous fluxes (weak form): transformed fluxes of this node from the metrics still in sR, written
  // over sR once every thread has finished reading it (one node per thread: EPB * n3 == THREADS)
  static_assert(EPB * n3 == S::THREADS, "one node per thread");
  {
    const int t = threadIdx.x;
    const int es = t / n3, x = t - es * n3, e = e0 + es;
    double Fv[12];
    if (e < d.nElems) {
      const double* Q = sR + es * 15 * n3;
      const double vx = Q[n3 + x], vy = Q[2 * n3 + x], vz = Q[3 * n3 + x];
      double m[9], g[12];
#pragma unroll
      for (int c = 0; c < 9; ++c) m[c] = Q[(6 + c) * n3 + x];
#pragma unroll
      for (int c = 0; c < 12; ++c) g[c] = d.grad[((size_t)e * 12 + c) * n3 + x];
      const double mu = elem_mu(d, e);
      const double lam = mu * B.lambdaFac;
      double tau[6];
      visc_tau(mu, g, tau);
#pragma unroll
      for (int dd = 0; dd < 3; ++dd) {
        double F[5];
        visc_flux_tau(tau, lam, vx, vy, vz, g, m[3 * dd], m[3 * dd + 1], m[3 * dd + 2], F);
#pragma unroll
        for (int v = 0; v < 4; ++v) Fv[4 * dd + v] = F[1 + v];
      }
    }
    __syncthreads();
    if (e < d.nElems) {
#pragma unroll
      for (int c = 0; c < 12; ++c) sR[(es * 15 + c) * n3 + x] = Fv[c];
    }
  }
  __syncthreads();
  constexpr bool EO = EOShape<n>::VOL;
  if constexpr (EO) {
    // D_Hat sweeps of the viscous fluxes in the even-odd form, in place: component 4 dir + v becomes its
    // contribution to Ut
    double eo[8];
    eo_row<n, true>(B, eo);
    eo_sweep_all<n, 4>(eo, sR, 15, 0, 4, sR, 15, 0, 4, e0, d.nElems);
  }
  for (int t = threadIdx.x; t < EPB * n3; t += blockDim.x) {
    const int es = t / n3, x = t - es * n3, e = e0 + es;
    if (e >= d.nElems) continue;
    const int i = x % n, j = (x / n) % n, k = x / n2;
    double ut[5];
#pragma unroll
    for (int v = 0; v < 5; ++v) ut[v] = sA[(es * 5 + v) * n3 + x];
    const double* V = sR + es * 15 * n3;
    if constexpr (EO) {
#pragma unroll
      for (int v = 0; v < 4; ++v) ut[1 + v] += (V[v * n3 + x] + V[(4 + v) * n3 + x]) + V[(8 + v) * n3 + x];
    } else {
#pragma unroll
      for (int l = 0; l < n; ++l) {
        const double ci = Bs.DhT(l, i), cj = Bs.DhT(l, j), ck = Bs.DhT(l, k);
        const int xi = l + n * (j + n * k), xj = i + n * (l + n * k), xk = i + n * (j + n * l);
#pragma unroll
        for (int v = 0; v < 4; ++v) {
          ut[1 + v] = fma(ci, V[v * n3 + xi], ut[1 + v]);
          ut[1 + v] = fma(cj, V[(4 + v) * n3 + xj], ut[1 + v]);
          ut[1 + v] = fma(ck, V[(8 + v) * n3 + xk], ut[1 + v]);
        }
      }
    }
    finish_node<n, true, false>(d, Bs, st, sFl, es, e, x, ut);
  }
}

// =====================================================================================================
// k_vol_split_gen: volint.f90:VolInt_splitForm for any number of nodes per line, Gauss or Gauss-Lobatto.
// The lines of one direction are packed SEG = 32/n to a warp (n lanes each, the last 32 - SEG*n lanes of a
// warp idle); a lane evaluates the pairs (a, a+dd mod n) for dd = 1..(n-1)/2 and hands the unscaled flux to
// its partner by shuffle as in k_vol_split; for even n the pairs at distance n/2 follow in a pass of their
// own, one thread per pair.
// Gauss nodes (surfint.t90:90-140, 177-215, split-Gauss surface integral): in the same pass each lane
// evaluates the two-point flux FluxB between its node and the element's own face state at both ends of the
// line (metric: its node's metric vector plus the face metric row Ja_Face / Ja_slave), the segment forms
// FluxB_sum = sum_k Leg(k) FluxB(k) once per face point (shared-memory slot of the warp), and the lane adds
// -1/2 NormalSign LegHat(a) (FluxB_sum - FluxB(a)); the numerical-flux part is the Gauss surface integral
// of finish_node. Up to 512 threads: larger elements loop over groups of lines and over nodes.
// =====================================================================================================
template <int n> struct SplitShape {
  static constexpr int EPB = Shape<n>::EPB, n2 = n * n, n3 = n * n * n;
  static constexpr int SEG = 32 / n;                       // lines per warp
  static constexpr int LINES = EPB * n2;                   // lines per direction per CTA
  // each direction's pass runs whole warps of SEG lines; the LO lines of each direction left over go to one joint
  // pass over the three directions (a warp with a single line would issue its FP64 work for 32 lanes)
  static constexpr int MAIN_WARPS = LINES / SEG;
  static constexpr int LO = LINES - MAIN_WARPS * SEG;
  static constexpr int LO_WARPS = (3 * LO + SEG - 1) / SEG;
  static constexpr int LINE_THREADS = (MAIN_WARPS > LO_WARPS ? MAIN_WARPS : LO_WARPS) * 32;
  static constexpr int NODE_THREADS = ((EPB * n3 + 31) / 32) * 32;
  static constexpr int WANT = LINE_THREADS > NODE_THREADS ? LINE_THREADS : NODE_THREADS;
  static constexpr int THREADS = WANT > 512 ? 512 : WANT;
  static constexpr int NPT = (EPB * n3 + THREADS - 1) / THREADS;  // volume nodes per thread
  static constexpr int FACE_NF = 9;  // rho, u, v, w, p-term, H-term, face metric row (3)
  static constexpr int SCRATCH = (THREADS / 32) * 32 * 5;  // Gauss: per-lane Leg*FluxB of the segment sums
  // per-CTA arrays: coefficients, split-flux inputs, divergence, face fluxes (+ Gauss: face states,
  // segment-sum slots) (+ several nodes per thread: a separate viscous-flux array)
  template <bool GL>
  __host__ __device__ static constexpr long long big() {
    return 2LL * n2 + (long long)EPB * (20 * n3 + 30 * n2) + (GL ? 0LL : (long long)EPB * 6 * FACE_NF * n2 + SCRATCH) +
           (NPT > 1 ? (long long)EPB * 12 * n3 : 0LL) + 3LL * LO * n * 5;
  }
};

template <int n, bool GL, bool GEN = false>
__global__ void __launch_bounds__(SplitShape<n>::THREADS) k_vol_split_gen(Dev d, Basis B, Stage st) {
  using SS = SplitShape<n>;
  constexpr int n2 = SS::n2, n3 = SS::n3, EPB = SS::EPB, N = n - 1, SEG = SS::SEG, FNF = SS::FACE_NF;
  extern __shared__ double smem[];
  double* sD = smem;
  double* sC = big_base<n>(d, smem, SS::template big<GL>());  // [2][n2]: DVolSurf(l,i) x density factor, x factor of the others
  double* sR = sC + 2 * n2;            // [EPB][15][n3]: rho, u, v, w, p-term, H-term, metrics(9); later viscous fluxes(12)
  double* sA = sR + EPB * 15 * n3;     // [EPB][5][n3] split-flux divergence
  double* sFl = sA + EPB * 5 * n3;     // [EPB][6][n2][5]
  double* sFS = sFl + EPB * 6 * n2 * 5;  // Gauss: [EPB][6][FNF][n2] own face states and face metric rows
  double* sScr = sFS + (GL ? 0 : EPB * 6 * FNF * n2);  // Gauss: [warp][lane][5]
  double* sV = SS::NPT > 1 ? sScr + (GL ? 0 : SS::SCRATCH) : sR;  // viscous fluxes [EPB][12][n3]
  double* sX = sScr + (GL ? 0 : SS::SCRATCH) + (SS::NPT > 1 ? EPB * 12 * n3 : 0);  // [3][LO][n][5] joint-pass line sums
  load_basis_smem<n>(B, sD);
  SBasis<n> Bs{sD};
  const bool pi = B.splitDG == 4;
  const int skind = B.splitDG;
  double f0 = pi ? 0.25 : 0.5, f1 = pi ? 0.125 : 0.5;
  if constexpr (GEN) split_factors(skind, f0, f1);
  for (int t = threadIdx.x; t < n2; t += blockDim.x) { sC[t] = B.DVS[t] * f0; sC[n2 + t] = B.DVS[t] * f1; }
  const int e0 = d.volBegin + blockIdx.x * EPB;
  load_face_fluxes<n>(d, sFl, e0);
  for (int t = threadIdx.x; t < EPB * n3; t += blockDim.x) {
    const int es = t / n3, x = t - es * n3, e = e0 + es;
    if (e >= d.nElems) continue;
    double* Q = sR + es * 15 * n3;
    const double u0 = d.U[((size_t)e * 5 + 0) * n3 + x], u4 = d.U[((size_t)e * 5 + 4) * n3 + x];
    const double srho = d.prim[((size_t)e * VP_NF + VP_SRHO) * n3 + x];
    const double p = d.prim[((size_t)e * VP_NF + VP_P) * n3 + x];
    Q[x] = u0;
    Q[n3 + x] = d.prim[((size_t)e * VP_NF + VP_U) * n3 + x];
    Q[2 * n3 + x] = d.prim[((size_t)e * VP_NF + VP_V) * n3 + x];
    Q[3 * n3 + x] = d.prim[((size_t)e * VP_NF + VP_W) * n3 + x];
    if constexpr (GEN) {
      split_node_inputs(skind, u0, Q[n3 + x], Q[2 * n3 + x], Q[3 * n3 + x], p, u4, srho, Q[x], Q[4 * n3 + x], Q[5 * n3 + x]);
    } else {
      Q[4 * n3 + x] = pi ? 4.0 * p : p;
      Q[5 * n3 + x] = pi ? (u4 + p) * srho : u4 + p;
    }
#pragma unroll
    for (int c = 0; c < 9; ++c) Q[(6 + c) * n3 + x] = d.metr[((size_t)e * 9 + c) * n3 + x];
    if constexpr (SS::LO > 0) {
      // nodes of lines left over in the first direction get that direction's sum only at the end
#pragma unroll
      for (int v = 0; v < 5; ++v) sA[(es * 5 + v) * n3 + x] = 0.;
    }
  }
  if (!GL) {
    // this element's face states (U_master/U_slave of its own sides) and face metric rows, in face order
    for (int t = threadIdx.x; t < EPB * 6 * n2; t += blockDim.x) {
      const int es = t / (6 * n2), r = t - es * 6 * n2, lsi = r / n2, pq = r - lsi * n2;
      const int e = e0 + es;
      if (e >= d.nElems) continue;
      const int ls = lsi + 1, p = pq % n, q = pq / n;
      const int code = d.elemSide[e * 6 + lsi], sd = code >> 3, flip = code & 7;
      int a, b;
      side_to_vol2(N, p, q, flip, ls, a, b);
      const double* src = (flip == 0 ? d.faceM : d.faceS) + (size_t)sd * FS_NF * n2 + pq;
      const double rho = src[FS_RHO * n2], E = src[FS_E * n2], pr = src[FS_P * n2], sr = src[FS_SRHO * n2];
      double* dst = sFS + (es * 6 + lsi) * FNF * n2;
      const int o = a + n * b;
      dst[o] = rho;
      dst[n2 + o] = src[FS_U * n2];
      dst[2 * n2 + o] = src[FS_V * n2];
      dst[3 * n2 + o] = src[FS_W * n2];
      if constexpr (GEN) {
        split_node_inputs(skind, rho, dst[n2 + o], dst[2 * n2 + o], dst[3 * n2 + o], pr, E, sr, dst[o], dst[4 * n2 + o], dst[5 * n2 + o]);
      } else {
        dst[4 * n2 + o] = pi ? 4.0 * pr : pr;
        dst[5 * n2 + o] = pi ? (E + pr) * sr : E + pr;
      }
#pragma unroll
      for (int c = 0; c < 3; ++c) dst[(6 + c) * n2 + o] = d.faceJa[(((size_t)e * 6 + lsi) * 3 + c) * n2 + o];
    }
  }
  __syncthreads();
  // two-point flux G (unscaled; density factor f0, others f1) between state a and state b with metric sum ms
  auto two_point = [pi, skind, &B](double ra, double ua, double va, double wa, double pa, double ha, double rb, double ub, double vb, double wb,
                                double pb, double hb, double ms0, double ms1, double ms2, double* G) {
    split_pair<GEN>(skind, pi, B, ra, ua, va, wa, pa, ha, rb, ub, vb, wb, pb, hb, ms0, ms1, ms2, G);
  };
  const int lane = threadIdx.x & 31;
  const int seg = lane / n, a = lane - seg * n, segBase = seg * n;
  // node a of line `line` of direction dir for this lane: its pairs and, on Gauss nodes, the split-Gauss surface
  // term. carry: added to the previous directions' sums in sA and stored there; else the line's own contribution
  // is stored into out[a][5]. Lanes of invalid segments compute on line 0 and store nothing.
  // Gauss: this lane's weights of the split-Gauss surface term, -1/2 NormalSign LegHat(a) times the density factor
  // and the others' (minus side, plus side), formed once
  double csW[4] = {0., 0., 0., 0.};
  if (!GL) {
    const double hM = 0.5 * Bs.LhM(a), hP = -0.5 * Bs.LhP(a);
    csW[0] = hM * f0; csW[1] = hM * f1; csW[2] = hP * f0; csW[3] = hP * f1;
  }
  auto line_pass = [&](int dir, int line, bool valid, bool carry, double* out) {
    const int lineC = valid ? line : 0;  // idle lanes compute on line 0 and store nothing
    const int es = lineC / n2, lr = lineC - es * n2, c1 = lr % n, c2 = lr / n;
    const bool store = valid && e0 + es < d.nElems;
    const int stride = dir == 0 ? 1 : (dir == 1 ? n : n2);
    const int xline = dir == 0 ? n * (c1 + n * c2) : (dir == 1 ? c1 + n2 * c2 : c1 + n * c2);
    const int xa = xline + a * stride;
    const double* Q = sR + es * 15 * n3;
    const double* Mm = Q + (6 + 3 * dir) * n3;
    const double ra = Q[xa], ua = Q[n3 + xa], va = Q[2 * n3 + xa], wa = Q[3 * n3 + xa], pa = Q[4 * n3 + xa], ha = Q[5 * n3 + xa];
    const double ma0 = Mm[xa], ma1 = Mm[n3 + xa], ma2 = Mm[2 * n3 + xa];
    double acc[5];
#pragma unroll
    for (int v = 0; v < 5; ++v) acc[v] = (carry && dir > 0) ? sA[(es * 5 + v) * n3 + xa] : 0.;
#pragma unroll
    for (int dd = 1; dd <= (n - 1) / 2; ++dd) {
      const int bI = a + dd < n ? a + dd : a + dd - n;
      const int xb = xline + bI * stride;
      double G[5];
      two_point(ra, ua, va, wa, pa, ha, Q[xb], Q[n3 + xb], Q[2 * n3 + xb], Q[3 * n3 + xb], Q[4 * n3 + xb], Q[5 * n3 + xb],
                ma0 + Mm[xb], ma1 + Mm[n3 + xb], ma2 + Mm[2 * n3 + xb], G);
      const double o0 = sC[bI * n + a], o1 = sC[n2 + bI * n + a];
      acc[0] = fma(o0, G[0], acc[0]);
#pragma unroll
      for (int v = 1; v < 5; ++v) acc[v] = fma(o1, G[v], acc[v]);
      {
        // receive the flux of the pair (a-dd, a) from lane a-dd of this segment
        const int aS = a - dd >= 0 ? a - dd : a - dd + n;
        const int src = valid ? segBase + aS : lane;
        const double r0 = sC[aS * n + a], r1 = sC[n2 + aS * n + a];
        acc[0] = fma(r0, __shfl_sync(0xffffffffu, G[0], src), acc[0]);
#pragma unroll
        for (int v = 1; v < 5; ++v) acc[v] = fma(r1, __shfl_sync(0xffffffffu, G[v], src), acc[v]);
      }
    }
    if (!GL) {
      const int fo = c1 + n * c2;  // face coordinate of this line on both end faces
      double* scr = sScr + (threadIdx.x >> 5) * 160;
      constexpr int ROUNDS = (5 + n - 1) / n;  // components summed per lane
#pragma unroll
      for (int side = 0; side < 2; ++side) {
        const int ls = side == 0 ? (dir == 0 ? XI_MINUS : (dir == 1 ? ETA_MINUS : ZETA_MINUS))
                                 : (dir == 0 ? XI_PLUS : (dir == 1 ? ETA_PLUS : ZETA_PLUS));
        const double* F = sFS + (es * 6 + ls - 1) * FNF * n2 + fo;
        double G[5];
        two_point(ra, ua, va, wa, pa, ha, F[0], F[n2], F[2 * n2], F[3 * n2], F[4 * n2], F[5 * n2], ma0 + F[6 * n2], ma1 + F[7 * n2],
                  ma2 + F[8 * n2], G);
        const double leg = side == 0 ? Bs.Lm(a) : Bs.Lp(a);
        // -1/2 NormalSign LegHat(a): NormalSign = -1 on the minus, +1 on the plus side
        const double cw0 = csW[2 * side], cw1 = csW[2 * side + 1];
        // FluxB_sum of the segment: every lane stores Leg(a) G(a); lane a sums components a, a+n, ... over
        // the segment's n lanes (in lane order); the sums are broadcast back by shuffles
        __syncwarp();
#pragma unroll
        for (int v = 0; v < 5; ++v) scr[lane * 5 + v] = G[v] * leg;
        __syncwarp();
        double S[ROUNDS];
#pragma unroll
        for (int r = 0; r < ROUNDS; ++r) {
          const int c = a + r * n;
          S[r] = 0.;
          if (seg < SEG && c < 5) {
            S[r] = scr[segBase * 5 + c];
#pragma unroll
            for (int m = 1; m < n; ++m) S[r] += scr[(segBase + m) * 5 + c];
          }
        }
#pragma unroll
        for (int v = 0; v < 5; ++v) {
          const double sum = __shfl_sync(0xffffffffu, S[v / n], valid ? segBase + v % n : lane);
          acc[v] = fma(v == 0 ? cw0 : cw1, sum - G[v], acc[v]);
        }
      }
    }
    if (store) {
#pragma unroll
      for (int v = 0; v < 5; ++v) {
        if (carry) sA[(es * 5 + v) * n3 + xa] = acc[v];
        else out[a * 5 + v] = acc[v];
      }
    }
  };
#pragma unroll 1
  for (int dir = 0; dir < 3; ++dir) {
#pragma unroll 1
    for (int base = 0; base < SS::MAIN_WARPS * 32; base += SS::THREADS) {
      const int tt = base + threadIdx.x;
      if (tt < SS::MAIN_WARPS * 32) line_pass(dir, (tt >> 5) * SEG + seg, seg < SEG, true, nullptr);  // whole warps
    }
    __syncthreads();
  }
  if constexpr (SS::LO > 0) {
    // the LO lines left over in each direction, the three directions in one pass; their sums are added per node
    // at the end (sX)
#pragma unroll 1
    for (int base = 0; base < SS::LO_WARPS * 32; base += SS::THREADS) {
      const int tt = base + threadIdx.x;
      if (tt < SS::LO_WARPS * 32) {
        const int kk = (tt >> 5) * SEG + seg;
        const bool valid = seg < SEG && kk < 3 * SS::LO;
        const int kc = valid ? kk : 0;
        const int dir = kc / SS::LO;
        line_pass(dir, SS::MAIN_WARPS * SEG + kc - dir * SS::LO, valid, false, sX + kc * n * 5);
      }
    }
    __syncthreads();
  }
  if constexpr (n % 2 == 0) {
    // even n: the pairs at distance n/2, (a, a+n/2) with a < n/2, each evaluated once by one thread that adds
    // it to both nodes; one direction at a time (every node is in exactly one such pair per direction)
    constexpr int HP = n / 2, NPAIR = n2 * HP;
#pragma unroll 1
    for (int dir = 0; dir < 3; ++dir) {
      for (int t = threadIdx.x; t < EPB * NPAIR; t += blockDim.x) {
        const int es = t / NPAIR, r = t - es * NPAIR;
        if (e0 + es >= d.nElems) continue;
        const int a = r % HP, c1 = (r / HP) % n, c2 = r / (HP * n);
        const int stride = dir == 0 ? 1 : (dir == 1 ? n : n2);
        const int xline = dir == 0 ? n * (c1 + n * c2) : (dir == 1 ? c1 + n2 * c2 : c1 + n * c2);
        const int xa = xline + a * stride, xb = xa + HP * stride, b = a + HP;
        const double* Q = sR + es * 15 * n3;
        const double* Mm = Q + (6 + 3 * dir) * n3;
        double G[5];
        split_pair<GEN>(skind, pi, B, Q[xa], Q[n3 + xa], Q[2 * n3 + xa], Q[3 * n3 + xa], Q[4 * n3 + xa], Q[5 * n3 + xa], Q[xb], Q[n3 + xb],
                        Q[2 * n3 + xb], Q[3 * n3 + xb], Q[4 * n3 + xb], Q[5 * n3 + xb], Mm[xa] + Mm[xb], Mm[n3 + xa] + Mm[n3 + xb],
                        Mm[2 * n3 + xa] + Mm[2 * n3 + xb], G);
        double* A = sA + es * 5 * n3;
        A[xa] = fma(sC[b * n + a], G[0], A[xa]);
        A[xb] = fma(sC[a * n + b], G[0], A[xb]);
#pragma unroll
        for (int v = 1; v < 5; ++v) {
          A[v * n3 + xa] = fma(sC[n2 + b * n + a], G[v], A[v * n3 + xa]);
          A[v * n3 + xb] = fma(sC[n2 + a * n + b], G[v], A[v * n3 + xb]);
        }
      }
      __syncthreads();
    }
  }
  if constexpr (GL) gl_surface_faces<n>(Bs, sFl, sA, e0, d.nElems);
  // viscous fluxes (weak form): transformed fluxes of each node from the metrics still in sR; with one node
  // per thread they are written over sR once every thread has finished reading it, else into sV
  constexpr int VS = SS::NPT > 1 ? 12 : 15;  // field stride of the viscous-flux array
  for (int t = threadIdx.x; t < SS::NPT * SS::THREADS; t += blockDim.x) {
    const int es = t < EPB * n3 ? t / n3 : 0, x = t - es * n3, e = e0 + es;
    const bool live = t < EPB * n3 && e < d.nElems;
    double Fv[12];
    if (live) {
      const double* Q = sR + es * 15 * n3;
      const double vx = Q[n3 + x], vy = Q[2 * n3 + x], vz = Q[3 * n3 + x];
      double m[9], g[12];
#pragma unroll
      for (int c = 0; c < 9; ++c) m[c] = Q[(6 + c) * n3 + x];
#pragma unroll
      for (int c = 0; c < 12; ++c) g[c] = d.grad[((size_t)e * 12 + c) * n3 + x];
      const double mu = elem_mu(d, e);
      const double lam = mu * B.lambdaFac;
      double tau[6];
      visc_tau(mu, g, tau);
#pragma unroll
      for (int dd = 0; dd < 3; ++dd) {
        double F[5];
        visc_flux_tau(tau, lam, vx, vy, vz, g, m[3 * dd], m[3 * dd + 1], m[3 * dd + 2], F);
#pragma unroll
        for (int v = 0; v < 4; ++v) Fv[4 * dd + v] = F[1 + v];
      }
    }
    if (SS::NPT == 1) __syncthreads();  // one pass: every thread reaches it
    if (live) {
#pragma unroll
      for (int c = 0; c < 12; ++c) sV[(es * VS + c) * n3 + x] = Fv[c];
    }
  }
  __syncthreads();
  constexpr bool EO = EOShape<n>::VOL;
  if constexpr (EO) {
    // D_Hat sweeps of the viscous fluxes in the even-odd form, in place (component 4 dir + v becomes its
    // contribution to Ut)
    double eo[8];
    eo_row<n, true>(B, eo);
    eo_sweep_all<n, 4>(eo, sV, VS, 0, 4, sV, VS, 0, 4, e0, d.nElems);
  }
  for (int t = threadIdx.x; t < EPB * n3; t += blockDim.x) {
    const int es = t / n3, x = t - es * n3, e = e0 + es;
    if (e >= d.nElems) continue;
    const int i = x % n, j = (x / n) % n, k = x / n2;
    double ut[5];
#pragma unroll
    for (int v = 0; v < 5; ++v) ut[v] = sA[(es * 5 + v) * n3 + x];
    if constexpr (SS::LO > 0) {
      // contributions of the joint pass: the node's line in each direction, if that line was left over
      const int lines[3] = {es * n2 + j + n * k, es * n2 + i + n * k, es * n2 + i + n * j};
      const int pos[3] = {i, j, k};
#pragma unroll
      for (int dir = 0; dir < 3; ++dir) {
        const int l = lines[dir] - SS::MAIN_WARPS * SEG;
        if (l >= 0) {
          const double* X = sX + ((dir * SS::LO + l) * n + pos[dir]) * 5;
#pragma unroll
          for (int v = 0; v < 5; ++v) ut[v] += X[v];
        }
      }
    }
    const double* V = sV + es * VS * n3;
    if constexpr (EO) {
#pragma unroll
      for (int v = 0; v < 4; ++v) ut[1 + v] += (V[v * n3 + x] + V[(4 + v) * n3 + x]) + V[(8 + v) * n3 + x];
    } else {
#pragma unroll
      for (int l = 0; l < n; ++l) {
        const double ci = Bs.DhT(l, i), cj = Bs.DhT(l, j), ck = Bs.DhT(l, k);
        const int xi = l + n * (j + n * k), xj = i + n * (l + n * k), xk = i + n * (j + n * l);
#pragma unroll
        for (int v = 0; v < 4; ++v) {
          ut[1 + v] = fma(ci, V[v * n3 + xi], ut[1 + v]);
          ut[1 + v] = fma(cj, V[(4 + v) * n3 + xj], ut[1 + v]);
          ut[1 + v] = fma(ck, V[(8 + v) * n3 + xk], ut[1 + v]);
        }
      }
    }
    finish_node<n, GL, !GL>(d, Bs, st, sFl, es, e, x, ut);
  }
}

// =====================================================================================================
// k_overint: overintegration.f90 -- dg.f90:663-675 after the volume kernel has written J u_t to Ut (stage
// mode 3): type 1 filters it with OverintegrationMat in xi, eta, zeta and applies ApplyJacobianCons; type 2
// applies FilterConservative, whose result is u_t; then the LSERK register update of the stage.
// With state = 1 it is the overintegration of U before the first time step (timedisc.f90:115-123: type 1
// filters U, type 2 applies FilterConservative to J U). One CTA per element, both buffers in shared memory.
// =====================================================================================================
template <int n> struct OverintShape {
  static constexpr int n3 = n * n * n;
  static constexpr int T = ((n3 + 31) / 32) * 32;
  static constexpr int THREADS = T < 64 ? 64 : (T > 512 ? 512 : T);
};

// one ChangeBasis sweep along axis ax of X(5, d0, d1, d2) -> Y with extent nout along ax; M row a holds the
// weights of output index a (leading dimension ldm)
__device__ __forceinline__ void overint_sweep(const double* X, double* Y, const double* M, int ldm, int ax, int d0, int d1, int d2,
                                              int nout) {
  const int o0 = ax == 0 ? nout : d0, o1 = ax == 1 ? nout : d1, o2 = ax == 2 ? nout : d2;
  const int On = o0 * o1 * o2, In = d0 * d1 * d2;
  const int nin = ax == 0 ? d0 : (ax == 1 ? d1 : d2);
  const int sIn = ax == 0 ? 1 : (ax == 1 ? d0 : d0 * d1);
  for (int t = threadIdx.x; t < 5 * On; t += blockDim.x) {
    const int v = t / On, r = t - v * On;
    const int i = r % o0, j = (r / o0) % o1, k = r / (o0 * o1);
    const int a = ax == 0 ? i : (ax == 1 ? j : k);
    const int base = v * In + (ax == 0 ? 0 : i) + d0 * ((ax == 1 ? 0 : j) + d1 * (ax == 2 ? 0 : k));
    const double* m = M + a * ldm;
    double acc = m[0] * X[base];
    for (int l = 1; l < nin; ++l) acc = fma(m[l], X[base + l * sIn], acc);
    Y[v * On + r] = acc;
  }
  __syncthreads();
}

template <int n>
__global__ void __launch_bounds__(OverintShape<n>::THREADS) k_overint(Dev d, OverintDev o, Stage st, int state) {
  constexpr int n3 = n * n * n;
  extern __shared__ double smem[];
  double* A = smem;           // [5][n3]
  double* Bf = A + 5 * n3;    // [5][n3]
  double* sM = Bf + 5 * n3;   // type 1: F [n][n]; type 2: VNU [nu][n], VUN [n][nu]
  const int e = d.volBegin + blockIdx.x;
  const int nu = o.nu;
  if (o.type == 1) {
    for (int t = threadIdx.x; t < n * n; t += blockDim.x) sM[t] = o.F[t];
  } else {
    for (int t = threadIdx.x; t < nu * n; t += blockDim.x) { sM[t] = o.VNU[t]; sM[nu * n + t] = o.VUN[t]; }
  }
  const double* src = state ? d.U : d.Ut;
  const bool toRef = state && o.type == 2;  // the state's conservative cut-off acts on J U = U / sJ
  for (int t = threadIdx.x; t < 5 * n3; t += blockDim.x) {
    const int v = t / n3, x = t - v * n3;
    const double val = src[((size_t)e * 5 + v) * n3 + x];
    A[t] = toRef ? val / d.sJ[(size_t)e * n3 + x] : val;
  }
  __syncthreads();
  const double* R;
  if (o.type == 1) {
    overint_sweep(A, Bf, sM, n, 0, n, n, n, n);
    overint_sweep(Bf, A, sM, n, 1, n, n, n, n);
    overint_sweep(A, Bf, sM, n, 2, n, n, n, n);
    R = Bf;
  } else {
    const double* V = sM;
    const double* W = sM + nu * n;
    overint_sweep(A, Bf, V, n, 0, n, n, n, nu);
    overint_sweep(Bf, A, V, n, 1, nu, n, n, nu);
    overint_sweep(A, Bf, V, n, 2, nu, nu, n, nu);
    const int nu3 = nu * nu * nu;
    for (int t = threadIdx.x; t < 5 * nu3; t += blockDim.x) {
      const int r = t % nu3;
      Bf[t] *= o.sJNU[(size_t)e * nu3 + r];
    }
    __syncthreads();
    overint_sweep(Bf, A, W, nu, 0, nu, nu, nu, n);
    overint_sweep(A, Bf, W, nu, 1, n, nu, nu, n);
    overint_sweep(Bf, A, W, nu, 2, n, n, nu, n);
    R = A;
  }
  const int inst = d.elemInst[e];
  const double bdt = st.rkB * d.dt[inst];
  for (int t = threadIdx.x; t < 5 * n3; t += blockDim.x) {
    const int x = t % n3;
    const size_t g = (size_t)e * 5 * n3 + t;
    double r = R[t];
    if (o.type == 1 && !state) r *= d.sJ[(size_t)e * n3 + x];  // ApplyJacobianCons
    if (state) { d.U[g] = r; continue; }
    if (st.mode == 0) { d.Ut[g] = r; continue; }
    if (st.mode == 2) r = fma(-st.rkA, d.Ut_tmp[g], r);
    d.Ut_tmp[g] = r;
    d.U[g] = fma(bdt, r, d.U[g]);
  }
}

// =====================================================================================================
// k_dt: calctimestep.f90:CALCTIMESTEP per element (convective and viscous eigenvalue bounds with the
// precomputed MetricsAdv / MetricsVisc), reduced per instance with an atomic minimum on the bit pattern
// of the (positive) time step; plus the channel bulk velocity partial sums (testcase.f90:CalcForcing).
// =====================================================================================================
__device__ __forceinline__ void atomic_min_pos_double(double* addr, double v) {
  // positive doubles order like their bit patterns
  atomicMin((unsigned long long*)addr, (unsigned long long)__double_as_longlong(v));
}
template <int n>
__global__ void __launch_bounds__(Shape<n>::THREADS) k_dt(Dev d, Basis B, const double* metAdv, const double* metVisc, double cfl, double dfl,
                                                          double* bulkPart /* [nElems] or null */, const double* wVol) {
  using S = Shape<n>;
  constexpr int n3 = S::n3, EPB = S::EPB;
  // nodes handled by one thread: one, or (elements larger than the block) n3 / THREADS rounded up
  constexpr int NPT = (EPB * n3 + S::THREADS - 1) / S::THREADS;
  constexpr int NR = NPT > 1 ? S::THREADS : n3;  // entries reduced per element
  // per-thread values: convective bound per direction (3), viscous bound per direction (3), bulk-velocity part
  __shared__ double sred[7][S::THREADS];
  const int e0 = blockIdx.x * EPB;
  const int t = threadIdx.x;
  const int es = NPT > 1 ? 0 : t / n3, x = NPT > 1 ? t : t - es * n3, e = e0 + es;
  // elements of instances that reuse their time step (nCalcTimeStep >= 1, held or finished) are skipped
  // unless the bulk velocity needs their nodes
  const bool active = es < EPB && e < d.nElems && (bulkPart || !d.dtSkip || !d.dtSkip[d.elemInst[e]]);
  double v7[7] = {0., 0., 0., 0., 0., 0., 0.};
  if (active) {
#pragma unroll 1
    for (int xn = x; xn < n3; xn += (NPT > 1 ? S::THREADS : n3)) {
      double u[5];
#pragma unroll
      for (int v = 0; v < 5; ++v) u[v] = d.U[((size_t)e * 5 + v) * n3 + xn];
      if (u[0] != u[0]) set_error(d.err, 1);
      const double srho = 1.0 / u[0];
      const double vx = u[1] * srho, vy = u[2] * srho, vz = u[3] * srho;
      const double p = B.kappaM1 * (u[4] - 0.5 * (vx * u[1] + vy * u[2] + vz * u[3]));
      const double c = sqrt(B.kappa * p * srho);
      const double sj = d.sJ[(size_t)e * n3 + xn];
      const double lv = elem_mu(d, e) * srho;
#pragma unroll
      for (int dd = 0; dd < 3; ++dd) {
        const double* mm = d.metr + ((size_t)e * 9 + 3 * dd) * n3 + xn;
        const double q = (mm[0] * vx + mm[n3] * vy + mm[2 * n3] * vz) * sj;
        const double lc = fabs(q) + c * metAdv[((size_t)e * 3 + dd) * n3 + xn];
        const double lvd = lv * metVisc[((size_t)e * 3 + dd) * n3 + xn];
        v7[dd] = NPT > 1 ? fmax(v7[dd], lc) : lc;
        v7[3 + dd] = NPT > 1 ? fmax(v7[3 + dd], lvd) : lvd;
      }
      if (bulkPart) v7[6] += vx * wVol[xn] / sj;
    }
  }
#pragma unroll
  for (int c = 0; c < 7; ++c) sred[c][t] = v7[c];
  __syncthreads();
  // tree reduction inside each element's thread range [es*NR, es*NR+NR): max for the bounds, sum for the bulk part
  constexpr int P2 = (NR <= 1) ? 1 : (1 << (32 - __builtin_clz(NR - 1)));
#pragma unroll 1
  for (int st = P2 / 2; st > 0; st >>= 1) {
    if (es < EPB && x < st && x + st < NR) {
#pragma unroll
      for (int c = 0; c < 6; ++c) sred[c][t] = fmax(sred[c][t], sred[c][t + st]);
      sred[6][t] += sred[6][t + st];
    }
    __syncthreads();
  }
  if (active && x == 0) {
    const double dtC = cfl * 2.0 / (sred[0][t] + sred[1][t] + sred[2][t]);
    const double sv = sred[3][t] + sred[4][t] + sred[5][t];
    const double dtV = sv > 0. ? dfl * 4.0 / sv : INFINITY;
    d.dtElem[e] = dtC;
    d.dtElem[d.nElems + e] = dtV;
    const double dtE = fmin(dtC, dtV);
    if (!(dtE == dtE) || !(dtE > 0.)) set_error(d.err, 2);
    else atomic_min_pos_double(&d.dt[d.elemInst[e]], dtE);
    if (bulkPart) bulkPart[e] = sred[6][t];
  }
}

}  // namespace fg
