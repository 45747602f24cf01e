// flexi_gb300 -- launch wrappers for one (n, node type) instantiation; included by fg_inst_n*.cu
#pragma once
#include "fg_adjoint.cuh"
#include "fg_kernels.cuh"
#include "fg_launch.cuh"

namespace fg {

template <int n, bool GL>
struct Inst {
  using S = Shape<n>;
  static int blocks(const Dev& d) { return (d.nElems + S::EPB - 1) / S::EPB; }
  // CTAs of a volume-kernel launch over Dev::volCount elements from Dev::volBegin (all elements when volCount is 0)
  static int vol_blocks(const Dev& d, int epb) { return ((d.volCount > 0 ? d.volCount : d.nElems) + epb - 1) / epb; }
  static size_t smem_prep() { return dyn_smem_bytes<n>(Big<n>::prep); }
  // Gauss nodes (lines of up to 8): the lifting keeps the 12 products F_v n_c per face point (the mortar layout, inert
  // without mortar sides): the surface part then costs 2 FMA per gradient component and direction at every node of
  // the normal lines, instead of forming F_v w and three normal products there
  static constexpr bool LIFT12 = !GL && n <= 8;
  static size_t smem_lift() { return dyn_smem_bytes<n>(LIFT12 ? Big<n>::liftMortar : Big<n>::lift); }
  static size_t smem_weak() { return dyn_smem_bytes<n>(Big<n>::weak); }
  static size_t smem_split() { return sizeof(double) * (SBasis<n>::SIZE + 2 * S::n2 + S::EPB * (20 * S::n3 + 6 * S::n2 * 5)); }
  // the tuned shuffle-pair kernel for Gauss-Lobatto lines of 2, 4 or 8 nodes; k_vol_split_gen otherwise
  static constexpr bool SPLIT_POW2 = GL && (n == 2 || n == 4 || n == 8);
  static size_t smem_split_gen() { return dyn_smem_bytes<n>(SplitShape<n>::template big<GL>()); }
  // doubles per CTA of the global scratch array: the largest per-element array set that does not fit in
  // shared memory (0: every kernel of this instantiation stages in shared memory)
  static constexpr long long gs(long long big) { return big_in_global<n>(big) ? big : 0; }
  static constexpr long long mx(long long a, long long b) { return a > b ? a : b; }
  static constexpr long long SCRATCH_PER_BLOCK =
      mx(mx(mx(gs(Big<n>::prep), gs(Big<n>::lift)), mx(gs(Big<n>::weak), gs(SplitShape<n>::template big<GL>()))), gs(Big<n>::liftVariant(true, true)));
  static size_t smem_weak_adj() { return sizeof(double) * (SBasis<n>::SIZE + S::EPB * 5 * S::n3 + S::THREADS); }
  static size_t smem_split_adj() { return sizeof(double) * (SBasis<n>::SIZE + 2 * S::n2 + S::EPB * 26 * S::n3 + S::THREADS); }
  static size_t smem_split_gen_adj() {
    return sizeof(double) * (SBasis<n>::SIZE + 2 * S::n2 + S::EPB * 20 * S::n3 + S::THREADS + (GL ? 0 : S::EPB * 6 * S::n2 * 14));
  }
  static size_t smem_lift_adj() { return sizeof(double) * (SBasis<n>::SIZE + S::EPB * (13 * S::n3 + 6 * S::n2 * 19)); }
  static size_t smem_prep_adj() { return sizeof(double) * (SBasis<n>::SIZE + S::EPB * (5 * S::n3 + 6 * S::n2 * 6)); }
  static size_t smem_lift_mortar_adj() { return sizeof(double) * (SBasis<n>::SIZE + S::EPB * (13 * S::n3 + 6 * S::n2 * 27)); }
  static size_t smem_mortar_face_adj() { return sizeof(double) * 113 * S::n2; }
  static size_t smem_mortar_pre_adj() { return sizeof(double) * 109 * S::n2; }
  // elements per CTA of the autotuner's alternative element kernels (N=5: 2, N=3: 4; 0: none)
  static constexpr int ALT_E = (n == 6) ? 2 : ((n == 4) ? 4 : 0);
  template <int E>
  static size_t smem_prep_E() { return dyn_smem_bytes<n>(Big<n, E>::prep); }
  template <int E>
  static size_t smem_lift_E() { return dyn_smem_bytes<n>(LIFT12 ? Big<n, E>::liftMortar : Big<n, E>::lift); }
  template <int E>
  static size_t smem_weak_E() { return dyn_smem_bytes<n>(Big<n, E>::weak); }
  template <int E>
  static void prep_E(const Dev& d, const Basis& B, cudaStream_t st) {
    using SE = Shape<n, E>;
    k_prep<n, GL, E><<<(d.nElems + SE::EPB - 1) / SE::EPB, SE::THREADS, smem_prep_E<E>(), st>>>(d, B);
  }
  template <int E>
  static void lift_E(const Dev& d, const Basis& B, cudaStream_t st) {
    using SE = Shape<n, E>;
    k_lift<n, GL, E, LIFT12><<<(d.nElems + SE::EPB - 1) / SE::EPB, SE::THREADS, smem_lift_E<E>(), st>>>(d, B);
  }
  template <int E>
  static void vol_weak_E(const Dev& d, const Basis& B, int mode, double rkA, double rkB, cudaStream_t st) {
    using SE = Shape<n, E>;
    k_vol_weak<n, GL, E><<<vol_blocks(d, SE::EPB), SE::THREADS, smem_weak_E<E>(), st>>>(d, B, Stage{mode, rkA, rkB});
  }
  // the Riemann solvers and split fluxes beyond LF/HLLC/Roe/RoeEntropyFix with the weak form, SD or PI
  static bool flux_more(const Basis& B) {
    const bool base = B.riemann == RIEMANN_LF || B.riemann == RIEMANN_HLLC || B.riemann == RIEMANN_ROE || B.riemann == RIEMANN_ROEENTROPYFIX;
    return !base || (B.splitDG >= 0 && B.splitDG != SPLIT_SD && B.splitDG != SPLIT_PI);
  }
  static bool split_more(const Basis& B) { return B.splitDG != SPLIT_SD && B.splitDG != SPLIT_PI; }
  static void flux_block(const Dev& d, const Basis& B, int block, cudaStream_t st) {
    const long long pts = (long long)d.nFluxSides * S::n2;
    if (flux_more(B)) k_flux<n, true><<<(unsigned)((pts + block - 1) / block), block, 0, st>>>(d, B);
    else k_flux<n><<<(unsigned)((pts + block - 1) / block), block, 0, st>>>(d, B);
  }
  template <class K>
  static void set_smem(K kern, size_t bytes) {
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  }
  static void prepare() {
    set_smem(k_prep<n, GL>, smem_prep());
    set_smem(k_lift<n, GL, 0, LIFT12>, smem_lift());
    set_smem(k_vol_weak<n, GL>, smem_weak());
    if constexpr (SPLIT_POW2) {
      set_smem(k_vol_split<n>, smem_split());
      set_smem(k_vol_split<n, true>, smem_split());
    } else {
      set_smem(k_vol_split_gen<n, GL>, smem_split_gen());
      set_smem(k_vol_split_gen<n, GL, true>, smem_split_gen());
    }
    set_smem(k_overint<n>, smem_overint());
    set_smem(k_lift<n, GL, 0, true>, smem_lift_mortar());
    set_smem(k_lift<n, GL, 0, false, true>, smem_lift_v(false, true));
    set_smem(k_lift<n, GL, 0, true, true>, smem_lift_v(true, true));
    set_smem(k_mortar_pre<n>, smem_mortar_pre());
    set_smem(k_mortar_face<n>, smem_mortar_face());
    if constexpr (ADJ) {
      set_smem(k_vol_weak_adj<n, GL>, smem_weak_adj());
      set_smem(k_lift_adj<n, GL>, smem_lift_adj());
      set_smem(k_prep_adj<n, GL>, smem_prep_adj());
      set_smem(k_vol_split_gen_adj<n, GL>, smem_split_gen_adj());
      set_smem(k_vol_split_gen_adj<n, GL, true>, smem_split_gen_adj());
      set_smem(k_lift_adj<n, GL, true>, smem_lift_mortar_adj());
      set_smem(k_mortar_face_adj<n>, smem_mortar_face_adj());
      set_smem(k_mortar_pre_adj<n>, smem_mortar_pre_adj());
    }
    if constexpr (GL && (n == 2 || n == 4 || n == 8)) set_smem(k_vol_split_adj<n>, smem_split_adj());
    if constexpr (ALT_E > 0) {
      set_smem(k_prep<n, GL, ALT_E>, smem_prep_E<ALT_E>());
      set_smem(k_lift<n, GL, ALT_E, LIFT12>, smem_lift_E<ALT_E>());
      set_smem(k_vol_weak<n, GL, ALT_E>, smem_weak_E<ALT_E>());
    }
  }
  // adjoint kernels: lines of up to 8 nodes (one thread per node, shared-memory staging)
  static constexpr bool ADJ = n <= 8;
  // split form: the shuffle-pair kernel for PI on Gauss-Lobatto lines of 2, 4 or 8 nodes, the per-node kernel
  // otherwise (SD, other line lengths, Gauss nodes)
  static void vol_adj(const Dev& d, const AdjDev& a, const Basis& B, cudaStream_t st) {
    if constexpr (GL && (n == 2 || n == 4 || n == 8)) {
      if (B.splitDG == SPLIT_PI) {
        k_vol_split_adj<n><<<blocks(d), S::THREADS, smem_split_adj(), st>>>(d, a, B);
        return;
      }
    }
    if constexpr (ADJ) {
      if (B.splitDG == SPLIT_CH || B.splitDG == SPLIT_IR) k_vol_split_gen_adj<n, GL, true><<<blocks(d), S::THREADS, smem_split_gen_adj(), st>>>(d, a, B);
      else if (B.splitDG >= 0) k_vol_split_gen_adj<n, GL><<<blocks(d), S::THREADS, smem_split_gen_adj(), st>>>(d, a, B);
      else k_vol_weak_adj<n, GL><<<blocks(d), S::THREADS, smem_weak_adj(), st>>>(d, a, B);
    }
  }
  static void flux_adj(const Dev& d, const AdjDev& a, const Basis& B, cudaStream_t st) {
    const long long pts = (long long)d.nFluxSides * S::n2;
    if constexpr (ADJ) {
      if (pts > 0) {
        if (flux_more(B)) k_flux_adj<n, true><<<(unsigned)((pts + 127) / 128), 128, 0, st>>>(d, a, B);
        else k_flux_adj<n><<<(unsigned)((pts + 127) / 128), 128, 0, st>>>(d, a, B);
      }
    }
  }
  static void lift_adj(const Dev& d, const AdjDev& a, const Basis& B, cudaStream_t st) {
    if constexpr (ADJ) k_lift_adj<n, GL><<<blocks(d), S::THREADS, smem_lift_adj(), st>>>(d, a, B);
  }
  static void prep_adj(const Dev& d, const AdjDev& a, const Basis& B, cudaStream_t st) {
    if constexpr (ADJ) k_prep_adj<n, GL><<<blocks(d), S::THREADS, smem_prep_adj(), st>>>(d, a, B);
  }
  static void mortar_face_adj(const Dev& d, const AdjDev& a, const Basis& B, const MortarDev& M, cudaStream_t st) {
    // mortar meshes take LF, HLLC, Roe and RoeEntropyFix only (fg_build_mesh)
    if constexpr (ADJ) k_mortar_face_adj<n><<<d.nMortars, 256, smem_mortar_face_adj(), st>>>(d, a, B, M);
  }
  static void lift_mortar_adj(const Dev& d, const AdjDev& a, const Basis& B, cudaStream_t st) {
    if constexpr (ADJ) k_lift_adj<n, GL, true><<<blocks(d), S::THREADS, smem_lift_mortar_adj(), st>>>(d, a, B);
  }
  static void mortar_pre_adj(const Dev& d, const AdjDev& a, const Basis& B, const MortarDev& M, cudaStream_t st) {
    if constexpr (ADJ) k_mortar_pre_adj<n><<<d.nMortars, 256, smem_mortar_pre_adj(), st>>>(d, a, B, M);
  }
  static void prep(const Dev& d, const Basis& B, cudaStream_t st) {
    k_prep<n, GL><<<blocks(d), S::THREADS, smem_prep(), st>>>(d, B);
  }
  static void lift(const Dev& d, const Basis& B, cudaStream_t st) {
    k_lift<n, GL, 0, LIFT12><<<blocks(d), S::THREADS, smem_lift(), st>>>(d, B);
  }
  static void flux(const Dev& d, const Basis& B, cudaStream_t st) {
    const long long pts = (long long)d.nFluxSides * S::n2;
    if (flux_more(B)) k_flux<n, true><<<(unsigned)((pts + 127) / 128), 128, 0, st>>>(d, B);
    else k_flux<n><<<(unsigned)((pts + 127) / 128), 128, 0, st>>>(d, B);
  }
  static void vol_weak(const Dev& d, const Basis& B, int mode, double rkA, double rkB, cudaStream_t st) {
    k_vol_weak<n, GL><<<vol_blocks(d, S::EPB), S::THREADS, smem_weak(), st>>>(d, B, Stage{mode, rkA, rkB});
  }
  static void vol_split(const Dev& d, const Basis& B, int mode, double rkA, double rkB, cudaStream_t st) {
    const Stage sg{mode, rkA, rkB};
    if (split_more(B)) {
      if constexpr (SPLIT_POW2) k_vol_split<n, true><<<vol_blocks(d, S::EPB), S::THREADS, smem_split(), st>>>(d, B, sg);
      else k_vol_split_gen<n, GL, true><<<vol_blocks(d, S::EPB), SplitShape<n>::THREADS, smem_split_gen(), st>>>(d, B, sg);
      return;
    }
    if constexpr (SPLIT_POW2) k_vol_split<n><<<vol_blocks(d, S::EPB), S::THREADS, smem_split(), st>>>(d, B, sg);
    else k_vol_split_gen<n, GL><<<vol_blocks(d, S::EPB), SplitShape<n>::THREADS, smem_split_gen(), st>>>(d, B, sg);
  }
  // mortar interfaces (one CTA of 256 threads per big mortar side)
  static size_t smem_lift_mortar() { return dyn_smem_bytes<n>(Big<n>::liftMortar); }
  static size_t smem_lift_v(bool mortar, bool cons) { return dyn_smem_bytes<n>(Big<n>::liftVariant(mortar, cons)); }
  // conservative / weak volume part of the lifting (doConservativeLifting, doWeakLifting), without and with mortars
  static void lift_cons(const Dev& d, const Basis& B, cudaStream_t st) {
    k_lift<n, GL, 0, false, true><<<blocks(d), S::THREADS, smem_lift_v(false, true), st>>>(d, B);
  }
  static void lift_mortar_cons(const Dev& d, const Basis& B, cudaStream_t st) {
    k_lift<n, GL, 0, true, true><<<blocks(d), S::THREADS, smem_lift_v(true, true), st>>>(d, B);
  }
  static size_t smem_mortar_pre() { return sizeof(double) * 97 * S::n2; }
  static size_t smem_mortar_face() { return sizeof(double) * 104 * S::n2; }
  static void mortar_pre(const Dev& d, const Basis& B, const MortarDev& M, cudaStream_t st) {
    k_mortar_pre<n><<<d.nMortars, 256, smem_mortar_pre(), st>>>(d, B, M);
  }
  static void lift_mortar(const Dev& d, const Basis& B, cudaStream_t st) {
    k_lift<n, GL, 0, true><<<blocks(d), S::THREADS, smem_lift_mortar(), st>>>(d, B);
  }
  static void mortar_face(const Dev& d, const Basis& B, const MortarDev& M, cudaStream_t st) {
    k_mortar_face<n><<<d.nMortars, 256, smem_mortar_face(), st>>>(d, B, M);
  }
  static size_t smem_overint() { return sizeof(double) * (10 * S::n3 + 2 * S::n2); }
  static void overint(const Dev& d, const OverintDev& o, int mode, double rkA, double rkB, int state, cudaStream_t st) {
    k_overint<n><<<d.volCount > 0 ? d.volCount : d.nElems, OverintShape<n>::THREADS, smem_overint(), st>>>(d, o, Stage{mode, rkA, rkB}, state);
  }
  static void dt(const Dev& d, const Basis& B, const double* ma, const double* mv, double cfl, double dfl, double* bulk, const double* wv,
                 cudaStream_t st) {
    k_dt<n><<<blocks(d), S::THREADS, 0, st>>>(d, B, ma, mv, cfl, dfl, bulk, wv);
  }
  static KernelSet make() {
    KernelSet k;
    k.n = n; k.gl = GL;
    k.prepare = &prepare;
    k.prep = &prep; k.lift = &lift; k.flux = &flux; k.vol_weak = &vol_weak; k.dt = &dt;
    k.vol_split = &vol_split;
    k.overint = &overint;
    k.mortar_pre = &mortar_pre; k.lift_mortar = &lift_mortar; k.mortar_face = &mortar_face;
    k.lift_cons = &lift_cons; k.lift_mortar_cons = &lift_mortar_cons;
    if constexpr (ADJ) {
      k.vol_adj = &vol_adj; k.flux_adj = &flux_adj; k.lift_adj = &lift_adj; k.prep_adj = &prep_adj;
      k.mortar_face_adj = &mortar_face_adj; k.lift_mortar_adj = &lift_mortar_adj; k.mortar_pre_adj = &mortar_pre_adj;
    }
    k.defEPB = S::EPB;
    k.scratchPerBlock = SCRATCH_PER_BLOCK;
    k.flux_block = &flux_block;
    if constexpr (ALT_E > 0) {
      k.altEPB = ALT_E;
      k.prep_alt = &prep_E<ALT_E>;
      k.lift_alt = &lift_E<ALT_E>;
      k.vol_weak_alt = &vol_weak_E<ALT_E>;
    }
    return k;
  }
};

}  // namespace fg
