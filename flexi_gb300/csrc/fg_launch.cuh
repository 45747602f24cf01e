// flexi_gb300 -- kernel sets per (nodes per direction, node type); instantiated in fg_inst_*.cu
#pragma once
#include "fg_common.cuh"

namespace fg {

struct AdjDev;

struct KernelSet {
  int n = 0;
  bool gl = false;
  void (*prep)(const Dev&, const Basis&, cudaStream_t) = nullptr;
  void (*lift)(const Dev&, const Basis&, cudaStream_t) = nullptr;
  void (*flux)(const Dev&, const Basis&, cudaStream_t) = nullptr;
  void (*vol_weak)(const Dev&, const Basis&, int, double, double, cudaStream_t) = nullptr;
  void (*vol_split)(const Dev&, const Basis&, int, double, double, cudaStream_t) = nullptr;
  void (*dt)(const Dev&, const Basis&, const double*, const double*, double, double, double*, const double*, cudaStream_t) = nullptr;
  // overintegration of Ut (state = 0, after a volume kernel in mode 0, with the stage's register update) or of U
  void (*overint)(const Dev&, const OverintDev&, int, double, double, int, cudaStream_t) = nullptr;
  // mortar interfaces: k_mortar_pre, k_lift<MORTAR> (BR1) and k_mortar_face
  void (*mortar_pre)(const Dev&, const Basis&, const MortarDev&, cudaStream_t) = nullptr;
  void (*lift_mortar)(const Dev&, const Basis&, cudaStream_t) = nullptr;
  void (*mortar_face)(const Dev&, const Basis&, const MortarDev&, cudaStream_t) = nullptr;
  // lifting with the conservative (doConservativeLifting) or weak (doWeakLifting) volume part
  void (*lift_cons)(const Dev&, const Basis&, cudaStream_t) = nullptr;
  void (*lift_mortar_cons)(const Dev&, const Basis&, cudaStream_t) = nullptr;
  // adjoint (vector-Jacobian product) of the right-hand side; vol_adj is null where unsupported
  void (*vol_adj)(const Dev&, const AdjDev&, const Basis&, cudaStream_t) = nullptr;
  void (*flux_adj)(const Dev&, const AdjDev&, const Basis&, cudaStream_t) = nullptr;
  void (*lift_adj)(const Dev&, const AdjDev&, const Basis&, cudaStream_t) = nullptr;
  void (*prep_adj)(const Dev&, const AdjDev&, const Basis&, cudaStream_t) = nullptr;
  // adjoint on mortar meshes: k_mortar_face_adj (after flux_adj), k_lift_adj<MORTAR>, k_mortar_pre_adj (before prep_adj)
  void (*mortar_face_adj)(const Dev&, const AdjDev&, const Basis&, const MortarDev&, cudaStream_t) = nullptr;
  void (*lift_mortar_adj)(const Dev&, const AdjDev&, const Basis&, cudaStream_t) = nullptr;
  void (*mortar_pre_adj)(const Dev&, const AdjDev&, const Basis&, const MortarDev&, cudaStream_t) = nullptr;
  // autotuner candidates: element kernels with another number of elements per CTA (altEPB = 0: none) and
  // the side kernel with a given block size (64, 128 or 256 threads); fluxBlock is the block size in use
  int defEPB = 0, altEPB = 0;
  void (*prep_alt)(const Dev&, const Basis&, cudaStream_t) = nullptr;
  void (*lift_alt)(const Dev&, const Basis&, cudaStream_t) = nullptr;
  void (*vol_weak_alt)(const Dev&, const Basis&, int, double, double, cudaStream_t) = nullptr;
  void (*flux_block)(const Dev&, const Basis&, int, cudaStream_t) = nullptr;
  int fluxBlock = 128;
  // doubles per CTA of Dev::scratch needed by element kernels whose arrays exceed shared memory (0: none)
  long long scratchPerBlock = 0;
  // sets the dynamic shared-memory limits of all kernels; must run before any stream capture
  void (*prepare)() = nullptr;
};

// returns the kernel set for n nodes per direction (2..8) and the node type; n == 0 if unsupported
KernelSet get_kernel_set(int n, bool gl);

}  // namespace fg
