// flexi_gb300 -- host runtime and C ABI (include/flexi_gpu.h).
//
// One fg_handle owns all device memory of one solver (one or many ensemble instances), one CUDA stream
// and, after the first fg_run, one captured CUDA graph of a whole time step. The per-stage sequence is
//   k_prep -> k_lift -> k_flux -> k_vol (fused LSERK update)
// and a step is  k_reset -> k_dt (CALCTIMESTEP + bulk velocity partial sums) -> k_finish_dt -> 5 stages.
#include <cuda_runtime.h>

#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/flexi_gpu.h"
#include "fg_adjoint.cuh"
#include "fg_common.cuh"
#include "fg_launch.cuh"
#include "fg_lserk.hpp"
#include "fg_mesh.hpp"

namespace fg {
KernelSet kernel_set_n2(bool);
KernelSet kernel_set_n3(bool);
KernelSet kernel_set_n4(bool);
KernelSet kernel_set_n5(bool);
KernelSet kernel_set_n6(bool);
KernelSet kernel_set_n7(bool);
KernelSet kernel_set_n8(bool);
KernelSet kernel_set_n9(bool);
KernelSet kernel_set_n10(bool);
KernelSet kernel_set_n11(bool);
KernelSet kernel_set_n12(bool);
KernelSet get_kernel_set(int n, bool gl) {
  switch (n) {
    case 2: return kernel_set_n2(gl);
    case 3: return kernel_set_n3(gl);
    case 4: return kernel_set_n4(gl);
    case 5: return kernel_set_n5(gl);
    case 6: return kernel_set_n6(gl);
    case 7: return kernel_set_n7(gl);
    case 8: return kernel_set_n8(gl);
    case 9: return kernel_set_n9(gl);
    case 10: return kernel_set_n10(gl);
    case 11: return kernel_set_n11(gl);
    case 12: return kernel_set_n12(gl);
    default: return KernelSet{};
  }
}

// ---- small helper kernels ----
__global__ void k_fill(double* a, double v, int cnt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < cnt) a[i] = v;
}
// per-instance reductions of the step set-up: bulk velocity = sum(bulkPart of the instance)/Vol,
// and the per-instance time counter. One thread per instance, elements of an instance are contiguous
// in [instStart[i], instStart[i+1]).
__global__ void k_finish_step(Dev d, const double* bulkPart, const int* instStart, const double* instVol, double* tInst, int doBulk,
                              int checkDt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.nInst) return;
  if (doBulk) {
    double s = 0.;
    for (int e = instStart[i]; e < instStart[i + 1]; ++e) s += bulkPart[e];
    d.bulkVel[i] = s / instVol[i];
  }
  if (!checkDt) return;
  const double dt = d.dt[i];
  if (!(dt > 0.) || dt > 1e300) set_error(d.err, 2);
  if (tInst) {
    if (d.tStep) d.tStep[i] = tInst[i];
    tInst[i] += dt;
  }
}
// Time-loop bookkeeping of fg_run per instance (timedisc_vars.f90: tAnalyze, dt_minOld, dt, dt_Min(DT_MIN),
// nCalcTimeStep, doAnalyze/doFinalize, iter, nDtLimited) and the parameters of InitTimeDisc.
enum { TD_HOLD = 1, TD_DONE = 2 };  // flags: the last step ended on an analysis time / at TEnd or maxIter
struct TimeDiscDev {
  double* tAnalyze;
  double* dtMinOld;
  double* dtPrev;  // the time step of the last step (reused while nCalc >= 1)
  double* dtMin;   // dt_Min(DT_MIN) of the last CALCTIMESTEP
  int* nCalc;
  int* flags;
  int* skip;       // Dev::dtSkip of the next step
  int* nDtLimited;
  long long* iter;
  double tEnd, analyzeDt, dtmin, dtkill;
  int nCalcMax;
  long long maxIter;
};
// InitTimeStep state at the instance times t (timedisc.f90:105-112, timedisc_func.f90:194-195)
__global__ void k_timedisc_reset(TimeDiscDev td, const double* t, int nInst) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nInst) return;
  td.tAnalyze[i] = fmin(t[i] + td.analyzeDt, td.tEnd);
  td.dtMinOld[i] = -999.;
  td.dtPrev[i] = 0.;
  td.dtMin[i] = 0.;
  td.nCalc[i] = 0;
  td.flags[i] = 0;
  td.skip[i] = 0;
  td.nDtLimited[i] = 0;
  td.iter[i] = 0;
}
// start of an fg_run call: instances held at an analysis time continue (AnalyzeTimeStep has run on the host)
__global__ void k_timedisc_release(TimeDiscDev td, int nInst) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nInst) return;
  const int f = td.flags[i] & ~TD_HOLD;
  td.flags[i] = f;
  td.skip[i] = (f != 0) || td.nCalc[i] >= 1;
}
// UpdateTimeStep (timedisc_func.f90:215-268) with EvalTimeStep (:433-454) and the step counting of TimeDisc /
// AnalyzeTimeStep (timedisc.f90:190-212, timedisc_func.f90:316-380), one thread per instance, after k_dt has
// written CALCTIMESTEP's dt (unless the instance skips it). Also the bulk velocity of CalcForcing.
__global__ void k_update_timestep(Dev d, TimeDiscDev td, const double* bulkPart, const int* instStart, const double* instVol, double* tInst,
                                  int doBulk) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.nInst) return;
  if (doBulk) {
    double s = 0.;
    for (int e = instStart[i]; e < instStart[i + 1]; ++e) s += bulkPart[e];
    d.bulkVel[i] = s / instVol[i];
  }
  const double t = tInst[i];
  if (d.tStep) d.tStep[i] = t;
  const int fl = td.flags[i];
  // held, finished, or the run stopped on an error: the stages run with dt = 0 and leave the state as it is
  if ((fl & (TD_HOLD | TD_DONE)) || *(volatile int*)d.err != 0) {
    d.dt[i] = 0.;
    td.skip[i] = 1;
    return;
  }
  double dt;
  bool ana = false, fin = false;
  if (td.nCalc[i] >= 1) {  // no time-step update in this step
    td.nCalc[i] -= 1;
    dt = td.dtPrev[i];
  } else {
    double dtm = d.dt[i];  // CALCTIMESTEP
    if (!(dtm > 0.) || dtm > 1e300) {
      set_error(d.err, 2);
      d.dt[i] = 0.;
      td.skip[i] = 1;
      return;
    }
    if (dtm < td.dtmin) {
      dtm = td.dtmin;
      td.nDtLimited[i] += 1;
    }
    td.dtMin[i] = dtm;
    if (dtm < td.dtkill) {  // "Critical Kill timestep reached": keep the state of time t
      set_error(d.err, 4);
      d.dt[i] = 0.;
      td.skip[i] = 1;
      return;
    }
    const double dA = td.tAnalyze[i] - t, dE = td.tEnd - t;
    const double m = fmin(dtm, fmin(dA, dE));
    if (m == dA) ana = true;
    if (m == dE) ana = fin = true;
    dt = dtm;  // MINVAL(dt_min, MASK=dt_min > 0); dtm > 0 here
    if (dA > 0.) dt = fmin(dt, dA);
    if (dE > 0.) dt = fmin(dt, dE);
    // steps until the next update: fewer the more dt changed since the last update
    const double q = td.dtMinOld[i] / dt - 1.;
    const double lg = fabs(log10(q * q * 100. + 2.220446049250313e-16));
    td.nCalc[i] = (lg >= (double)td.nCalcMax ? td.nCalcMax : (int)floor(lg)) - 1;
    td.dtMinOld[i] = dt;
    // stretch the step if the next analysis / the end would otherwise follow after less than dt/100
    if (dA - dt < dt / 100. && dA > 0.) { dt = dA; ana = true; }
    if (dE - dt < dt / 100. && dE > 0.) { dt = dE; ana = fin = true; }
    td.dtPrev[i] = dt;
  }
  d.dt[i] = dt;
  tInst[i] = t + dt;
  const long long it = td.iter[i] + 1;
  td.iter[i] = it;
  if (it == td.maxIter) ana = fin = true;
  int nf = fl;
  if (ana) {
    td.tAnalyze[i] = fmin(td.tAnalyze[i] + td.analyzeDt, td.tEnd);
    nf |= TD_HOLD;
  }
  if (fin) nf |= TD_DONE;
  td.flags[i] = nf;
  td.skip[i] = (nf != 0) || td.nCalc[i] >= 1;
}
// out = in * sJ (mul = 1) or in / sJ (mul = 0), per node of [e][5][n3] arrays
__global__ void k_scale_by_sj(const double* __restrict__ in, const double* __restrict__ sJ, double* out, int n3, long long cnt, int mul) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= cnt) return;
  const long long e = i / (5LL * n3);
  const double s = sJ[e * n3 + i % n3];
  out[i] = mul ? in[i] * s : in[i] / s;
}
// start time of step k of an adjoint solve, t0 + k dt (recomputed steps of the reverse sweep)
__global__ void k_step_time(Dev d, const double* t0, double off) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < d.nInst) d.tStep[i] = t0[i] + off;
}
// time of RK stage c of the current step, t_n + c dt, for the time-dependent source
__global__ void k_stage_time(Dev d, double c) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < d.nInst) d.tStage[i] = fma(c, d.dt[i], d.tStep[i]);
}
// LSERK adjoint stage update: G = alpha G + beta U (cotangents of the RK register and of the state);
// alpha = 0 starts G afresh without reading it
__global__ void k_adj_axpby(double* __restrict__ G, const double* __restrict__ U, double alpha, double beta, long long count) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < count) G[i] = alpha == 0.0 ? beta * U[i] : fma(alpha, G[i], beta * U[i]);
}
// body-force adjoint of one RK stage, one CTA per element: Fbar += G_mom1 + bulkVel G_ener (cotangent of the
// additional body force at each node) and partial[e] += sum_x G_ener (body force at x) (the stage's share of
// the bulk-velocity cotangent; uniform body force -dpdx plus the field)
__global__ void k_adj_source(const Dev d, const double* __restrict__ G, double* __restrict__ Fbar, double* __restrict__ partial,
                             const double* __restrict__ bulkVel, int n3) {
  __shared__ double red[128];
  const int e = blockIdx.x;
  const int inst = d.elemInst[e];
  const double bv = bulkVel[inst], mdp = -d.dpdx[inst];
  double s = 0.;
  for (int x = threadIdx.x; x < n3; x += blockDim.x) {
    const double g1 = G[((size_t)e * 5 + 1) * n3 + x], g4 = G[((size_t)e * 5 + 4) * n3 + x];
    if (Fbar) Fbar[(size_t)e * n3 + x] += fma(bv, g4, g1);
    s = fma(g4, mdp + (d.forceField ? d.forceField[(size_t)e * n3 + x] : 0.), s);
  }
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[e] += red[0];
}
// per-instance bulk-velocity cotangent from the element partials (elements of an instance are contiguous)
__global__ void k_adj_bulk_reduce(int nInst, const int* instStart, double* partial, double* bulkBar) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nInst) return;
  double s = 0.;
  for (int e = instStart[i]; e < instStart[i + 1]; ++e) { s += partial[e]; partial[e] = 0.; }
  bulkBar[i] = s;
}
// Ubar += bulkBar dBulkVel/dU at the step-start state U (testcase.f90:CalcForcing: sum of m1/rho w J / Vol)
__global__ void k_adj_bulk_apply(const Dev d, double* __restrict__ Ubar, const double* __restrict__ U, const double* __restrict__ bulkBar,
                                 const double* __restrict__ wVol, const double* __restrict__ instVol, int n3) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)d.nElems * n3) return;
  const int e = (int)(t / n3), x = (int)(t - (long long)e * n3);
  const int inst = d.elemInst[e];
  const double c = bulkBar[inst] * wVol[x] / (d.sJ[(size_t)e * n3 + x] * instVol[inst]);
  const double rho = U[((size_t)e * 5 + 0) * n3 + x], m1 = U[((size_t)e * 5 + 1) * n3 + x];
  const double srho = 1.0 / rho;
  Ubar[((size_t)e * 5 + 0) * n3 + x] -= c * m1 * srho * srho;
  Ubar[((size_t)e * 5 + 1) * n3 + x] += c * srho;
}
// mean wall shear: per wall side point the x-momentum viscous flux through the wall x SurfElem (the shear the
// fluid exerts on the wall) and SurfElem; with seed != 0 also the cotangent of the master face gradients
// for the seed's weight (cotangent of the mean)
__global__ void k_wall_shear(const Dev d, const Basis B, int n2, double* terms, double* areas, double seed, double* gradMb) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= d.nBCSides * n2) return;
  const int s = t / n2, pq = t - s * n2;
  const double* gm = d.geo + (size_t)s * FG_NF * n2 + pq;
  const double nv[3] = {gm[FG_NX * n2], gm[FG_NY * n2], gm[FG_NZ * n2]};
  const double se = gm[FG_SURF * n2];
  const double mu = elem_mu(d, d.sideElem[s * 4 + 0]);
  double g[12];
  for (int c = 0; c < 12; ++c) g[c] = d.gradM[((size_t)s * 12 + c) * n2 + pq];
  double F[5];
  visc_flux_dir(mu, mu * B.lambdaFac, 0., 0., 0., g, nv[0], nv[1], nv[2], F);
  terms[t] = F[1] * se;
  areas[t] = se;
  if (gradMb) {
    const double Fb[5] = {0., seed * se, 0., 0., 0.};
    double gb[12] = {0., 0., 0., 0., 0., 0., 0., 0., 0., 0., 0., 0.};
    double zu = 0., zv = 0., zw = 0., mub = 0.;
    visc_flux_dir_adj(mu, B.lambdaFac, 0., 0., 0., g, nv[0], nv[1], nv[2], Fb, zu, zv, zw, gb, mub);
    for (int c = 0; c < 12; ++c) gradMb[((size_t)s * 12 + c) * n2 + pq] = gb[c];
  }
}
// finite-difference JVP helpers: out = x + alpha y; out = (a - b) s; per-block partial sums of x.x
__global__ void k_axpy_out(double* __restrict__ out, const double* __restrict__ x, double alpha, const double* __restrict__ y, long long count) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < count) out[i] = fma(alpha, y[i], x[i]);
}
__global__ void k_fd_diff(double* out, const double* a, const double* b, double s, long long count) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < count) out[i] = (a[i] - b[i]) * s;
}
__global__ void k_sumsq_partial(const double* __restrict__ x, long long count, double* __restrict__ partial) {
  __shared__ double red[256];
  double s = 0.;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (long long)gridDim.x * blockDim.x) s = fma(x[i], x[i], s);
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}
// layout conversion between FLEXI's U(v,i,j,k,e) and [e][v][ijk]
__global__ void k_fortran_to_dev(const double* __restrict__ f, double* __restrict__ d, int nv, int n3, long long total) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= total) return;
  const int v = (int)(t % nv);
  const long long r = t / nv;
  const int x = (int)(r % n3);
  const long long e = r / n3;
  d[(e * nv + v) * n3 + x] = f[t];
}
__global__ void k_dev_to_fortran(const double* __restrict__ d, double* __restrict__ f, int nvDev, int v0, int nv, int n3, long long total) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= total) return;
  const int v = (int)(t % nv);
  const long long r = t / nv;
  const int x = (int)(r % n3);
  const long long e = r / n3;
  f[t] = d[(e * nvDev + v0 + v) * n3 + x];
}
// One CTA per element: the element's nv x n3 block between the Fortran layout (variable fastest) and the device layout
// (variable-major), staged through shared memory so that the global reads and writes are both contiguous and the
// index arithmetic is 32-bit (the element-wise kernels above serve blocks larger than the tile limit)
__global__ void k_fortran_to_dev_tiled(const double* __restrict__ f, double* __restrict__ d, int nv, int n3) {
  extern __shared__ double s[];
  const int m = nv * n3;
  const size_t base = (size_t)blockIdx.x * m;
  for (int t = threadIdx.x; t < m; t += blockDim.x) s[t] = f[base + t];
  __syncthreads();
  for (int t = threadIdx.x; t < m; t += blockDim.x) {
    const int v = t / n3, x = t - v * n3;
    d[base + t] = s[x * nv + v];
  }
}
__global__ void k_dev_to_fortran_tiled(const double* __restrict__ d, double* __restrict__ f, int nvDev, int v0, int nv, int n3) {
  extern __shared__ double s[];
  const int m = nv * n3;
  const double* src = d + ((size_t)blockIdx.x * nvDev + v0) * n3;
  for (int t = threadIdx.x; t < m; t += blockDim.x) s[t] = src[t];
  __syncthreads();
  double* dst = f + (size_t)blockIdx.x * m;
  for (int t = threadIdx.x; t < m; t += blockDim.x) {
    const int x = t / nv, v = t - x * nv;
    dst[t] = s[v * n3 + x];
  }
}
constexpr size_t FG_TILE_SMEM_MAX = 96 * 1024;

// FP64 pipe throughput probe: 8 independent chains per thread of one FP64 operation (OP 0 DFMA, 1 DADD, 2 DMUL) or of
// the three mixed (OP 3: chain c uses operation c mod 3); every grid shape from 4 to 32 chains and 128 to 512 threads,
// and every mix, gives the same rate on GB300
template <int OP>
__global__ void k_probe_fp64(double* out, double a, double b, int iters) {
  double x[8];
#pragma unroll
  for (int c = 0; c < 8; ++c) x[c] = threadIdx.x * 1e-3 + c;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      const int op = OP < 3 ? OP : c % 3;
      x[c] = op == 0 ? fma(x[c], a, b) : op == 1 ? x[c] + b : x[c] * a;
    }
  }
  double s = 0.;
#pragma unroll
  for (int c = 0; c < 8; ++c) s += x[c];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// FP64 tensor-core MMA (mma.sync m8n8k4, 8x8x4 per warp instruction = 512 flops) in NM independent accumulator
// chains per warp; WITH_FMA adds eight independent DFMA chains per thread to every iteration, to see whether the two
// share the FP64 units (register operands only; one store per thread at the end)
template <int NM, bool WITH_FMA>
__global__ void k_probe_dmma(double* out, double a, double b, int iters) {
  double c[NM][2], x[8];
#pragma unroll
  for (int m = 0; m < NM; ++m) { c[m][0] = threadIdx.x * 1e-4 + m; c[m][1] = 0.5 * m; }
#pragma unroll
  for (int i = 0; i < 8; ++i) x[i] = threadIdx.x * 1e-3 + i;
  const double av = 1e-3 * (threadIdx.x & 7), bv = 2e-3 * (threadIdx.x & 3);
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int m = 0; m < NM; ++m)
      asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};\n"
                   : "+d"(c[m][0]), "+d"(c[m][1]) : "d"(av), "d"(bv));
    if (WITH_FMA) {
#pragma unroll
      for (int i = 0; i < 8; ++i) x[i] = fma(x[i], a, b);
    }
  }
  double s = 0.;
#pragma unroll
  for (int m = 0; m < NM; ++m) s += c[m][0] + c[m][1];
#pragma unroll
  for (int i = 0; i < 8; ++i) s += x[i];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// the DFMA chains of k_probe_fp64<0> run by the first K lanes of every warp only: whether the FP64 pipe's issue
// time for a warp instruction depends on its active lanes
template <int K>
__global__ void k_probe_fp64_lanes(double* out, double a, double b, int iters) {
  double x[8];
#pragma unroll
  for (int c = 0; c < 8; ++c) x[c] = threadIdx.x * 1e-3 + c;
  if ((threadIdx.x & 31) < K) {
    for (int i = 0; i < iters; ++i) {
#pragma unroll
      for (int c = 0; c < 8; ++c) x[c] = fma(x[c], a, b);
    }
  }
  double s = 0.;
#pragma unroll
  for (int c = 0; c < 8; ++c) s += x[c];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}
}  // namespace fg

using namespace fg;

struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
};

// element chunks of the last stage's volume kernel in fg_run_to_host
constexpr int FG_OUT_CHUNKS = 6;

struct fg_handle {
  fg_config cfg{};
  Basis B{};
  KernelSet K{};      // kernels in use (after autotuning)
  KernelSet Kdef{};   // the default kernel set of this (N, node type)
  fgh::HostMesh M;
  Dev d{};
  bool haveMesh = false;      // device arrays ready
  bool haveHostMesh = false;  // host-side mesh ready (set-up can be inspected without a GPU)
  cudaStream_t st = nullptr;
  std::vector<DevBuf> bufs;
  double* dMetAdv = nullptr;
  double* dMetVisc = nullptr;
  double* dWVol = nullptr;
  double* dBulkPart = nullptr;
  int* dInstStart = nullptr;
  double* dInstVol = nullptr;
  double* dTime = nullptr;
  TimeDiscDev td{};  // time-loop bookkeeping of fg_run
  double* dStage = nullptr;  // staging for layout conversion (size nElems*5*n3)
  double RKA[21]{}, RKb[21]{}, RKc[21]{};
  int nStages = 5;
  double cflEff = 0., dflEff = 0.;
  // overintegration in use (type 2 is off when NUnder >= N, overintegration.f90:139-141) and its matrices
  OverintDev ov{};
  OverintDev ovT{};  // the transposed filter (adjoint of overintegration): F^T, or VUN^T / VNU^T in the roles of VNU / VUN
  double* adjWov = nullptr;  // [e][5][n3] cotangent of Ut carried through the transposed filter
  double* adjT0 = nullptr;   // [nInst] time at the start of the last fg_adjoint_forward (time-dependent source)
  int NU = 0;
  // mortar interfaces: operators and the device copy of the mortar table (Dev::nMortars > 0)
  MortarDev mort{};
  cudaGraphExec_t graph = nullptr;
  long long launchesPerStep = 0;  // kernel launches of one captured TimeDisc step
  // fg_run_to_host: the stream of the state download that overlaps the last stage, and its events
  cudaStream_t stOut = nullptr;
  cudaEvent_t evOut[FG_OUT_CHUNKS] = {};
  cudaEvent_t evOutDone = nullptr;
  long long launches = 0;
  std::string err;
  std::vector<double> instMu0;
  // adjoint buffers (allocated on the first fg_vjp_time_derivative)
  AdjDev a{};
  bool haveAdj = false;
  // LSERK adjoint: U checkpoints of the last fg_adjoint_forward, stage states of one segment, the
  // running cotangents, and the final forward state (restored after the reverse sweep)
  std::vector<void*> adjStore;
  std::vector<double*> adjCkpt, adjStage;
  // with enough device memory, the forward intermediates of every stage of the segment being reversed
  // (primitive variables, lifted gradients, face states and face gradients), so that the adjoint right-hand
  // sides need not recompute them
  bool adjKeepInter = false;
  std::vector<Dev> adjInter;
  double* adjGbar = nullptr;
  double* adjUbar = nullptr;
  double* adjUfinal = nullptr;
  double* adjBulkHist = nullptr;  // [ckptEvery][nInst] bulk velocity of each step of the segment being reversed
  double* adjPartial = nullptr;   // [nElems] element shares of the bulk-velocity cotangent of the current step
  double* adjBulkBar = nullptr;   // [nInst]
  double* adjFbar = nullptr;      // [e][n3] cotangent of the body-force field
  // finite-difference JVP (fg_jvp_time_derivative): saved state, perturbation, result, reduction partials
  double* jvpXk = nullptr;
  double* jvpV = nullptr;
  double* jvpR = nullptr;
  double* jvpPartial = nullptr;
  int adjSteps = 0, adjEvery = 0;
  double adjDt = 0.;
  // binomial schedule: snapshot slots (slot 0 = U at t_0) and the steps whose states the forward pass
  // already stored (the schedule's first right spine) with their slots
  bool adjBinomial = false;
  std::vector<double*> adjSlots;
  std::vector<std::pair<int, int>> adjSpine;
  long long adjRecomputed = 0;  // forward steps the last reverse sweep re-ran
  // per-kernel event timing (fg_profile_enable)
  bool profiling = false;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> evPool;
  std::vector<int> evClass;
  size_t evUsed = 0;
};

namespace {

thread_local std::string g_err;  // errors without a handle (fg_create, fg_probe_fp64)

int fail(fg_handle* h, int code, const std::string& msg) {
  if (h) h->err = msg;
  else g_err = msg;
  return code;
}
#define CUDA_TRY(x)                                                                                   \
  do {                                                                                                \
    cudaError_t e_ = (x);                                                                             \
    if (e_ != cudaSuccess) return fail(h, FG_ERR_CUDA, std::string(#x) + ": " + cudaGetErrorString(e_)); \
  } while (0)

template <class T>
int dalloc(fg_handle* h, T*& ptr, size_t count) {
  void* p = nullptr;
  if (count == 0) count = 1;
  cudaError_t e = cudaMalloc(&p, count * sizeof(T));
  if (e != cudaSuccess) return fail(h, FG_ERR_CUDA, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  h->bufs.push_back({p, count * sizeof(T)});
  ptr = (T*)p;
  return 0;
}
template <class T>
int upload(fg_handle* h, T*& ptr, const std::vector<T>& v) {
  if (int r = dalloc(h, ptr, v.size())) return r;
  if (!v.empty()) {
    cudaError_t e = cudaMemcpy(ptr, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return fail(h, FG_ERR_CUDA, std::string("cudaMemcpy: ") + cudaGetErrorString(e));
  }
  return 0;
}
void free_adjoint_store(fg_handle* h) {
  for (void* p : h->adjStore) cudaFree(p);
  h->adjStore.clear();
  h->adjCkpt.clear();
  h->adjStage.clear();
  h->adjInter.clear();
  h->adjKeepInter = false;
  h->adjGbar = h->adjUbar = h->adjUfinal = nullptr;
  h->adjBulkHist = h->adjPartial = h->adjBulkBar = h->adjFbar = nullptr;
  h->adjSteps = h->adjEvery = 0;
  h->adjBinomial = false;
  h->adjSlots.clear();
  h->adjSpine.clear();
}
void free_device(fg_handle* h) {
  free_adjoint_store(h);
  if (h->graph) { cudaGraphExecDestroy(h->graph); h->graph = nullptr; }
  for (auto& e : h->evPool) { cudaEventDestroy(e.first); cudaEventDestroy(e.second); }
  h->evPool.clear(); h->evClass.clear(); h->evUsed = 0;
  for (auto& b : h->bufs) cudaFree(b.p);
  h->bufs.clear();
  h->haveMesh = false;
  h->haveAdj = false;
  h->a = AdjDev{};
  h->jvpXk = h->jvpV = h->jvpR = h->jvpPartial = nullptr;
}

void init_basis(fg_handle* h) {
  const fg_config& c = h->cfg;
  Basis& B = h->B;
  std::memset(&B, 0, sizeof(B));
  const int N = c.N, n = N + 1;
  B.N = N; B.n = n; B.nodeType = c.NodeType; B.splitDG = c.SplitDG;
  B.riemann = c.Riemann; B.riemannBC = c.RiemannBC < 0 ? c.Riemann : c.RiemannBC;
  B.lifting = c.Lifting; B.weakLifting = c.doWeakLifting;
  fgh::Vec x, w;
  fgh::nodes(N, c.NodeType == FG_NODE_GAUSS_LOBATTO ? fgh::LOBATTO : fgh::GAUSS, x, w);
  const fgh::Mat D = fgh::diff_matrix(x);
  const fgh::Vec wb = fgh::bary_weights(x);
  const fgh::Vec Lm = fgh::lagrange_at(-1., x, wb), Lp = fgh::lagrange_at(1., x, wb);
  for (int i = 0; i < n; ++i)
    for (int l = 0; l < n; ++l) {
      B.D_T[l * n + i] = D(i, l);                        // D_T(l,i) = D(i,l)
      B.Dhat_T[l * n + i] = -(1. / w[i]) * D(l, i) * w[l];  // D_Hat_T(l,i) = D_Hat(i,l) = -w_i^-1 D(l,i) w_l
    }
  // DVolSurf (dg.f90:180-203): GL: D^T with the corner corrections; Gauss: transpose of D - 1/2 M^-1 Vf^T B Vf
  for (int l = 0; l < n; ++l)
    for (int i = 0; i < n; ++i) {
      double v;
      if (c.NodeType == FG_NODE_GAUSS_LOBATTO) {
        v = D(i, l);  // DVolSurf(l,i) = D_T(l,i) = D(i,l)
        if (l == 0 && i == 0) v += 1.0 / (2.0 * w[0]);
        if (l == N && i == N) v -= 1.0 / (2.0 * w[N]);
      } else {
        v = D(i, l) - 0.5 * (1. / w[i]) * (-Lm[i] * Lm[l] + Lp[i] * Lp[l]);  // DVolSurf(l,i) = S(i,l)
      }
      B.DVS[l * n + i] = v;
    }
  for (int i = 0; i < n; ++i) { B.Lm[i] = Lm[i]; B.Lp[i] = Lp[i]; B.LhM[i] = Lm[i] / w[i]; B.LhP[i] = Lp[i] / w[i]; }
  // even-odd tables of D and D_Hat; both are centro-antisymmetric on symmetric nodes, M(N-i,N-l) = -M(i,l)
  fill_even_odd(B);
  B.kappa = c.kappa; B.kappaM1 = c.kappa - 1.; B.sKappaM1 = 1. / (c.kappa - 1.);
  B.Rgas = c.R; B.sR = 1. / c.R;
  const double cp = c.R * c.kappa / (c.kappa - 1.);
  B.lambdaFac = cp / c.Pr;
  B.etaBR2 = c.etaBR2; B.etaBR2_wall = (c.etaBR2_wall == -1.) ? c.etaBR2 : c.etaBR2_wall;
  B.kappaFac = 2. * c.kappa / (c.kappa - 1.);
  B.sKappaP1 = 1. / (c.kappa + 1.);
  B.logEntC = std::log(c.kappa - 1.) / (c.kappa - 1.);
  B.kappa_kappaM1 = c.kappa / (c.kappa - 1.);
  B.riemannPhi = c.RiemannPhiFactor;
  // the low-storage scheme of TimeDiscMethod (timedisc_vars.f90:137-457)
  const fgh::LSERKScheme* sch = fgh::lserk_scheme(c.TimeDiscMethod);
  h->nStages = sch->stages;
  for (int s = 0; s <= sch->stages; ++s) { h->RKA[s] = sch->A[s]; h->RKb[s] = sch->b[s]; h->RKc[s] = sch->c[s]; }
  // FillCFL_DFL (timedisc_func.f90:463-527)
  const double* cflG = sch->cflGauss;
  const double* cflGL = sch->cflGL;
  static const double dflG[10] = {1.12, 0.76, 0.55, 0.41, 0.32, 0.25, 0.20, 0.17, 0.14, 0.12};
  static const double dflGL[10] = {4.50, 1.95, 1.18, 0.79, 0.56, 0.42, 0.32, 0.25, 0.20, 0.17};
  const bool gl = c.NodeType == FG_NODE_GAUSS_LOBATTO;
  // table lookups through plain pointers: indexing a conditional expression of two arrays with a
  // non-literal subscript mis-compiles with the host compiler in use here (g++ 13 returns 0)
  const double* cflTab = gl ? cflGL : cflG;
  const double* dflTab = gl ? dflGL : dflG;
  // overintegration (overintegration.f90:99-141): NUnder defaults to N; the conservative cut-off is off
  // for NUnder >= N; the CFL uses NEff = MIN(N, NUnder) (timedisc_func.f90:142-144), and Gauss-Lobatto
  // nodes take the Gauss table (timedisc_vars.f90:183-190)
  h->NU = c.NUnder < 0 ? N : c.NUnder;
  h->ov = OverintDev{};
  h->ov.type = c.OverintegrationType;
  if (h->ov.type == 2 && !(h->NU < N)) h->ov.type = 0;
  h->ov.nu = (h->NU < N ? h->NU : N) + 1;
  if (h->ov.type > 0) cflTab = cflG;
  const int NEff = h->NU < N ? h->NU : N;
  const int iC = (NEff < 15 ? NEff : 15) - 1, iD = (N < 10 ? N : 10) - 1;
  h->cflEff = c.CFLScale * cflTab[iC] / (2. * NEff + 1.);
  h->dflEff = c.DFLScale * dflTab[iD] * sch->relativeDFL / ((2. * N + 1.) * (2. * N + 1.));
}

int upload_mesh(fg_handle* h) {
  fgh::HostMesh& M = h->M;
  fgh::finish_mesh(M, h->cfg.kappa, h->cfg.Pr);
  if (h->cfg.IniExactFunc == 4 && M.elemX.empty())
    return fail(h, FG_ERR_CONFIG, "the source of exact function 4 needs the solution coordinates (fg_build_mesh)");
  h->haveHostMesh = true;
  free_device(h);
  if (!h->st) CUDA_TRY(cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking));
  h->K.prepare();
  CUDA_TRY(cudaGetLastError());
  const int n = M.n, n2 = n * n, n3 = n2 * n, nE = M.nElems, nS = M.nSides;
  Dev& d = h->d;
  d = Dev{};
  d.nElems = nE; d.nSides = nS; d.nBCSides = M.nBCSides; d.nInst = M.nInst;
  d.nFluxSides = M.nFluxSides; d.nMortars = M.nMortars;
  int r = 0;
  if (M.nMortars > 0) {
    const fg_config& c = h->cfg;
    const bool baseRiemann = c.Riemann == FG_RIEMANN_LF || c.Riemann == FG_RIEMANN_HLLC || c.Riemann == FG_RIEMANN_ROE ||
                             c.Riemann == FG_RIEMANN_ROEENTROPYFIX;
    if (!baseRiemann || (c.SplitDG != FG_SPLIT_NONE && c.SplitDG != FG_SPLIT_SD && c.SplitDG != FG_SPLIT_PI))
      return fail(h, FG_ERR_CONFIG, "mortar interfaces support the Riemann solvers LF, HLLC, Roe, RoeEntropyFix and SplitDG SD or PI");
    // mortar.f90:InitMortar: M_0_1/M_0_2 interpolate to the halves [-1,0]/[0,1]; M_1_0/M_2_0 = (Vdm_Leg
    // Vphi^T W VGP)^T project back, with Vphi the orthonormal Legendre polynomials at the Gauss points mapped
    // to each half, W the Gauss weights and VGP the interpolation from the solution nodes to the Gauss points
    const int N = M.N;
    fgh::Vec x, w, xg, wg, x1, x2;
    fgh::nodes(N, M.nodeType, x, w);
    fgh::nodes(N, fgh::GAUSS, xg, wg);
    for (double v : x) { x1.push_back(0.5 * (v - 1.)); x2.push_back(0.5 * (v + 1.)); }
    const fgh::Mat I1 = fgh::interp_matrix(x, x1), I2 = fgh::interp_matrix(x, x2), VGP = fgh::interp_matrix(x, xg);
    MortarDev& mo = h->mort;
    mo = MortarDev{};
    double dL;
    for (int l = 0; l < n; ++l)
      for (int p = 0; p < n; ++p) { mo.M01[l * n + p] = I1(p, l); mo.M02[l * n + p] = I2(p, l); }
    for (int p = 0; p < n; ++p)
      for (int l = 0; l < n; ++l) {
        double a1 = 0., a2 = 0.;
        for (int j = 0; j < n; ++j) {
          double vl, b1 = 0., b2 = 0.;
          fgh::legendre(j, x[p], vl, dL);
          for (int i = 0; i < n; ++i) {
            double v1, v2;
            fgh::legendre(j, 0.5 * (xg[i] - 1.), v1, dL);
            fgh::legendre(j, 0.5 * (xg[i] + 1.), v2, dL);
            b1 += v1 * wg[i] * VGP(i, l);
            b2 += v2 * wg[i] * VGP(i, l);
          }
          a1 += vl * b1;
          a2 += vl * b2;
        }
        mo.M10[l * n + p] = a1;
        mo.M20[l * n + p] = a2;
      }
  }
  if ((r = dalloc(h, d.U, (size_t)nE * 5 * n3))) return r;
  if ((r = dalloc(h, d.Ut, (size_t)nE * 5 * n3))) return r;
  if ((r = dalloc(h, d.Ut_tmp, (size_t)nE * 5 * n3))) return r;
  if ((r = dalloc(h, d.prim, (size_t)nE * VP_NF * n3))) return r;
  if ((r = dalloc(h, d.grad, (size_t)nE * 12 * n3))) return r;
  if ((r = upload(h, d.metr, M.metr))) return r;
  if ((r = upload(h, d.sJ, M.sJ))) return r;
  {
    std::vector<double> mJ(M.metr.size());
    for (size_t e = 0; e < (size_t)nE; ++e)
      for (int c = 0; c < 9; ++c)
        for (int x = 0; x < n3; ++x) mJ[(e * 9 + c) * n3 + x] = M.metr[(e * 9 + c) * n3 + x] * M.sJ[e * n3 + x];
    if ((r = upload(h, d.metrJ, mJ))) return r;
  }
  if ((r = upload(h, d.elemSide, M.elemSide))) return r;
  if ((r = upload(h, d.elemInst, M.elemInst))) return r;
  if ((r = dalloc(h, d.faceM, (size_t)nS * FS_NF * n2))) return r;
  if ((r = dalloc(h, d.faceS, (size_t)nS * FS_NF * n2))) return r;
  if ((r = dalloc(h, d.gradM, (size_t)nS * 12 * n2))) return r;
  if ((r = dalloc(h, d.gradS, (size_t)nS * 12 * n2))) return r;
  if ((r = upload(h, d.geo, M.geo))) return r;
  if (h->cfg.SplitDG >= 0 && h->cfg.NodeType == FG_NODE_GAUSS)
    if ((r = upload(h, d.faceJa, M.faceJa))) return r;
  if ((r = dalloc(h, d.flux, (size_t)nS * 5 * n2))) return r;
  if ((r = upload(h, d.sideElem, M.sideElem))) return r;
  if ((r = upload(h, d.sideInst, M.sideInst))) return r;
  if ((r = upload(h, d.bcType, M.bcType))) return r;
  if ((r = upload(h, d.bcTwall, M.bcTwall))) return r;
  if (M.nMortars > 0) {
    int* info = nullptr;
    if ((r = upload(h, info, M.mortarInfo))) return r;
    h->mort.info = info;
    if ((r = dalloc(h, d.mortarLift, (size_t)M.nMortars * 12 * n2))) return r;
  }
  std::vector<double> mu(M.nInst, h->cfg.mu0), zero(M.nInst, 0.), dp(M.nInst, h->cfg.doTCSource ? h->cfg.dpdx : 0.);
  if (h->instMu0.size() == (size_t)M.nInst) mu = h->instMu0;
  if ((r = upload(h, d.mu0, mu))) return r;
  if ((r = upload(h, d.dt, zero))) return r;
  if ((r = upload(h, d.bulkVel, zero))) return r;
  if ((r = upload(h, d.dpdx, dp))) return r;
  if ((r = upload(h, d.err, std::vector<int>(1, 0)))) return r;
  if ((r = upload(h, d.muScale, std::vector<double>(nE, 1.0)))) return r;
  if ((r = dalloc(h, d.dtElem, (size_t)2 * nE))) return r;
  if (h->K.scratchPerBlock > 0) {
    // per-CTA slices of the element kernels whose arrays exceed shared memory (one element per CTA here)
    d.scratchStride = h->K.scratchPerBlock;
    if ((r = dalloc(h, d.scratch, (size_t)nE * (size_t)d.scratchStride))) return r;
  }
  if (h->cfg.IniExactFunc == 4) {
    // exactfunc.f90:CalcSource CASE(4) (3D) coefficients
    const fg_config& c = h->cfg;
    const double om = M_PI * c.IniFrequency, A = c.IniAmplitude, a = c.AdvVel[0] * 2. * M_PI, k = c.kappa, km1 = c.kappa - 1.;
    std::vector<double> P = {om, a, A * (-a + 3. * om), A * (-a + 0.5 * om * (1. + k * 5.)), A * (A * om * km1),
                             A * (0.5 * ((9. + k * 15.) * om - 8. * a)), A * (A * (3. * om * k - a)), A * (3. * c.mu0 * k * om * om / c.Pr)};
    double* dP = nullptr;
    if ((r = upload(h, dP, P))) return r;
    d.srcPar = dP;
    double* dX = nullptr;
    if ((r = upload(h, dX, M.elemX))) return r;
    d.elemX = dX;
    if ((r = upload(h, d.tStage, std::vector<double>(M.nInst, 0.)))) return r;
    if ((r = upload(h, d.tStep, std::vector<double>(M.nInst, 0.)))) return r;
  }
  if ((r = upload(h, h->dMetAdv, M.metAdv))) return r;
  if ((r = upload(h, h->dMetVisc, M.metVisc))) return r;
  if ((r = upload(h, h->dWVol, M.wVol))) return r;
  if (h->ov.type > 0) {
    // overintegration.f90:InitOverintegration
    const int N = M.N, nu = h->ov.nu, NU = nu - 1;
    const int type = M.nodeType;
    fgh::Vec x, w;
    fgh::nodes(N, type, x, w);
    if (h->ov.type == 1) {
      fgh::Mat V(n, n);
      double dL;
      for (int i = 0; i < n; ++i) for (int m = 0; m < n; ++m) fgh::legendre(m, x[i], V(i, m), dL);
      const fgh::Mat sV = fgh::inverse(V);
      std::vector<double> F((size_t)n * n, 0.);
      for (int i = 0; i < n; ++i)
        for (int l = 0; l < n; ++l) {
          double acc = 0.;
          for (int m = 0; m < nu; ++m) acc += V(i, m) * sV(m, l);
          F[(size_t)i * n + l] = acc;
        }
      double* dF = nullptr;
      if ((r = upload(h, dF, F))) return r;
      h->ov.F = dF;
      std::vector<double> FT((size_t)n * n);
      for (int i = 0; i < n; ++i) for (int l = 0; l < n; ++l) FT[(size_t)l * n + i] = F[(size_t)i * n + l];
      double* dFT = nullptr;
      if ((r = upload(h, dFT, FT))) return r;
      h->ovT = h->ov;
      h->ovT.F = dFT;
    } else {
      const fgh::Mat Vd = fgh::vandermonde(N, type, NU, type, true), Vu = fgh::vandermonde(NU, type, N, type, true);
      std::vector<double> VNU((size_t)nu * n), VUN((size_t)n * nu);
      for (int a = 0; a < nu; ++a) for (int i = 0; i < n; ++i) VNU[(size_t)a * n + i] = Vd(a, i);
      for (int i = 0; i < n; ++i) for (int a = 0; a < nu; ++a) VUN[(size_t)i * nu + a] = Vu(i, a);
      // 1/J on NUnder: the modal projection of J = 1/sJ (equal to the projection of DetJac_Ref that
      // overintegration.f90:129-137 forms, up to round-off: both keep the Legendre modes up to NUnder)
      const int nu3 = nu * nu * nu;
      std::vector<double> sJNU((size_t)nE * nu3), t1((size_t)nu * n2), t2((size_t)nu * nu * n);
      for (int e = 0; e < nE; ++e) {
        const double* sj = &M.sJ[(size_t)e * n3];
        for (int k = 0; k < n; ++k) for (int j = 0; j < n; ++j) for (int a = 0; a < nu; ++a) {
          double acc = 0.;
          for (int i = 0; i < n; ++i) acc += VNU[(size_t)a * n + i] / sj[i + n * (j + n * k)];
          t1[a + nu * (j + n * k)] = acc;
        }
        for (int k = 0; k < n; ++k) for (int b = 0; b < nu; ++b) for (int a = 0; a < nu; ++a) {
          double acc = 0.;
          for (int j = 0; j < n; ++j) acc += VNU[(size_t)b * n + j] * t1[a + nu * (j + n * k)];
          t2[a + nu * (b + nu * k)] = acc;
        }
        for (int c = 0; c < nu; ++c) for (int b = 0; b < nu; ++b) for (int a = 0; a < nu; ++a) {
          double acc = 0.;
          for (int k = 0; k < n; ++k) acc += VNU[(size_t)c * n + k] * t2[a + nu * (b + nu * k)];
          sJNU[(size_t)e * nu3 + a + nu * (b + nu * c)] = 1. / acc;
        }
      }
      double *dV = nullptr, *dW = nullptr, *dS = nullptr;
      if ((r = upload(h, dV, VNU))) return r;
      if ((r = upload(h, dW, VUN))) return r;
      if ((r = upload(h, dS, sJNU))) return r;
      h->ov.VNU = dV; h->ov.VUN = dW; h->ov.sJNU = dS;
      // transposes: VUN^T [nu][n] takes the role of VNU, VNU^T [n][nu] that of VUN
      std::vector<double> VUNT((size_t)nu * n), VNUT((size_t)n * nu);
      for (int i = 0; i < n; ++i) for (int a = 0; a < nu; ++a) { VUNT[(size_t)a * n + i] = VUN[(size_t)i * nu + a]; VNUT[(size_t)i * nu + a] = VNU[(size_t)a * n + i]; }
      double *dVT = nullptr, *dWT = nullptr;
      if ((r = upload(h, dVT, VUNT))) return r;
      if ((r = upload(h, dWT, VNUT))) return r;
      h->ovT = h->ov;
      h->ovT.VNU = dVT; h->ovT.VUN = dWT;
    }
  }
  if ((r = dalloc(h, h->dBulkPart, (size_t)nE))) return r;
  // instances must be contiguous element ranges
  std::vector<int> start(M.nInst + 1, 0);
  for (int e = 0; e < nE; ++e) {
    if (e > 0 && M.elemInst[e] < M.elemInst[e - 1]) return fail(h, FG_ERR_MESH, "ensemble instances must be contiguous element ranges");
    start[M.elemInst[e] + 1] = e + 1;
  }
  for (int i = 1; i <= M.nInst; ++i) start[i] = std::max(start[i], start[i - 1]);
  if ((r = upload(h, h->dInstStart, start))) return r;
  if ((r = upload(h, h->dInstVol, M.instVol))) return r;
  if ((r = upload(h, h->dTime, zero))) return r;
  {
    TimeDiscDev& td = h->td;
    const int nI = M.nInst;
    if ((r = dalloc(h, td.tAnalyze, nI)) || (r = dalloc(h, td.dtMinOld, nI)) || (r = dalloc(h, td.dtPrev, nI)) || (r = dalloc(h, td.dtMin, nI)) ||
        (r = dalloc(h, td.nCalc, nI)) || (r = dalloc(h, td.flags, nI)) || (r = dalloc(h, td.skip, nI)) || (r = dalloc(h, td.nDtLimited, nI)) ||
        (r = dalloc(h, td.iter, nI)))
      return r;
    const fg_config& c = h->cfg;
    td.tEnd = c.TEnd;
    td.analyzeDt = c.Analyze_dt > 0. ? c.Analyze_dt : c.TEnd;  // analyze.f90:127-130
    td.dtmin = c.dtmin;
    td.dtkill = c.dtkill;
    td.nCalcMax = c.nCalcTimeStepMax;
    td.maxIter = c.maxIter;
    CUDA_TRY(cudaDeviceSynchronize());
    k_timedisc_reset<<<(nI + 127) / 128, 128>>>(td, h->dTime, nI);
    CUDA_TRY(cudaGetLastError());
  }
  if ((r = dalloc(h, h->dStage, (size_t)nE * 12 * n3))) return r;
  // the uploads above run on the legacy default stream, which the solver's non-blocking stream does not
  // order against: finish them before any kernel can read the arrays
  CUDA_TRY(cudaDeviceSynchronize());
  h->haveMesh = true;
  return 0;
}

// event pair around one launch of kernel class cls (profiling mode only)
struct ProfScope {
  fg_handle* h;
  size_t slot = (size_t)-1;
  ProfScope(fg_handle* h_, int cls) : h(h_) {
    if (!h->profiling) return;
    if (h->evUsed == h->evPool.size()) {
      cudaEvent_t a, b;
      cudaEventCreate(&a); cudaEventCreate(&b);
      h->evPool.push_back({a, b});
      h->evClass.push_back(0);
    }
    slot = h->evUsed++;
    h->evClass[slot] = cls;
    cudaEventRecord(h->evPool[slot].first, h->st);
  }
  ~ProfScope() {
    if (slot != (size_t)-1) cudaEventRecord(h->evPool[slot].second, h->st);
  }
};

// state sequence of one right-hand side evaluation up to the volume kernel
void launch_rhs_front(fg_handle* h, const Dev& d) {
  const bool mortars = d.nMortars > 0;
  { ProfScope p(h, 0); h->K.prep(d, h->B, h->st); }
  if (mortars) { ProfScope p(h, 5); h->K.mortar_pre(d, h->B, h->mort, h->st); h->launches += 1; }
  {
    ProfScope p(h, 1);
    const bool cons = h->cfg.doConservativeLifting || h->cfg.doWeakLifting;
    (mortars ? (cons ? h->K.lift_mortar_cons : h->K.lift_mortar) : (cons ? h->K.lift_cons : h->K.lift))(d, h->B, h->st);
  }
  if (d.nFluxSides > 0) { ProfScope p(h, 2); h->K.flux_block(d, h->B, h->K.fluxBlock, h->st); }
  if (mortars) { ProfScope p(h, 5); h->K.mortar_face(d, h->B, h->mort, h->st); h->launches += 1; }
}
// state sequence of one right-hand side evaluation plus the RK register update
void launch_rhs_dev(fg_handle* h, const Dev& d, int mode, double rkA, double rkB) {
  launch_rhs_front(h, d);
  {
    ProfScope p(h, 3);
    // with overintegration the volume kernel writes J u_t and k_overint filters it and updates the registers
    const bool oi = h->ov.type > 0;
    if (h->cfg.SplitDG >= 0) h->K.vol_split(d, h->B, oi ? 3 : mode, rkA, rkB, h->st);
    else h->K.vol_weak(d, h->B, oi ? 3 : mode, rkA, rkB, h->st);
    if (oi) { h->K.overint(d, h->ov, mode, rkA, rkB, 0, h->st); h->launches += 1; }
  }
  h->launches += 4;
}
void launch_rhs(fg_handle* h, int mode, double rkA, double rkB) { launch_rhs_dev(h, h->d, mode, rkA, rkB); }
// step set-up: mode 0 = CALCTIMESTEP, 1 = fixed dt, 2 = bulk velocity only (plain right-hand side)
void launch_step_setup(fg_handle* h, int mode, double fixedDt, bool advanceTime) {
  const Dev& d = h->d;
  const int nI = d.nInst;
  const bool doBulk = h->cfg.doTCSource != 0;
  const bool computeDt = mode == 0;
  if (mode == 2) {
    if (!doBulk) return;
    h->K.dt(d, h->B, h->dMetAdv, h->dMetVisc, h->cflEff, h->dflEff, h->dBulkPart, h->dWVol, h->st);
    k_finish_step<<<(nI + 127) / 128, 128, 0, h->st>>>(d, h->dBulkPart, h->dInstStart, h->dInstVol, nullptr, 1, 0);
    h->launches += 2;
    return;
  }
  if (computeDt) {
    k_fill<<<(nI + 127) / 128, 128, 0, h->st>>>(d.dt, INFINITY, nI);
    if (advanceTime) {  // the TimeDisc loop: CALCTIMESTEP only for instances that update dt, then UpdateTimeStep
      Dev dd = d;
      dd.dtSkip = h->td.skip;
      { ProfScope p(h, 4); h->K.dt(dd, h->B, h->dMetAdv, h->dMetVisc, h->cflEff, h->dflEff, doBulk ? h->dBulkPart : nullptr, h->dWVol, h->st); }
      k_update_timestep<<<(nI + 127) / 128, 128, 0, h->st>>>(d, h->td, h->dBulkPart, h->dInstStart, h->dInstVol, h->dTime, doBulk);
      h->launches += 3;
      return;
    }
    { ProfScope p(h, 4); h->K.dt(d, h->B, h->dMetAdv, h->dMetVisc, h->cflEff, h->dflEff, h->dBulkPart, h->dWVol, h->st); }
    h->launches += 2;
  } else {
    k_fill<<<(nI + 127) / 128, 128, 0, h->st>>>(d.dt, fixedDt, nI);
    h->launches += 1;
    if (doBulk) {
      h->K.dt(d, h->B, h->dMetAdv, h->dMetVisc, h->cflEff, h->dflEff, h->dBulkPart, h->dWVol, h->st);
      k_fill<<<(nI + 127) / 128, 128, 0, h->st>>>(d.dt, fixedDt, nI);
      h->launches += 2;
    }
  }
  k_finish_step<<<(nI + 127) / 128, 128, 0, h->st>>>(d, h->dBulkPart, h->dInstStart, h->dInstVol, advanceTime ? h->dTime : nullptr, doBulk, 1);
  h->launches += 1;
}
void launch_lserk(fg_handle* h) {
  for (int s = 1; s <= h->nStages; ++s) {
    if (h->d.srcPar) {
      k_stage_time<<<(h->d.nInst + 127) / 128, 128, 0, h->st>>>(h->d, h->RKc[s]);
      h->launches += 1;
    }
    launch_rhs(h, s == 1 ? 1 : 2, s == 1 ? 0. : h->RKA[s], h->RKb[s]);
  }
}
int check_err(fg_handle* h) {
  int e = 0;
  CUDA_TRY(cudaMemcpyAsync(&e, h->d.err, sizeof(int), cudaMemcpyDeviceToHost, h->st));
  CUDA_TRY(cudaStreamSynchronize(h->st));
  if (e == 1) return fail(h, FG_ERR_NAN, "NaN density found");
  if (e == 4) return fail(h, FG_ERR_DTKILL, "time step below dtkill (critical kill time step reached)");
  if (e) return fail(h, FG_ERR_DT, "non-finite or non-positive time step");
  return 0;
}

bool riemann_known(int r) {
  switch (r) {
    case FG_RIEMANN_LF: case FG_RIEMANN_HLLC: case FG_RIEMANN_ROE: case FG_RIEMANN_ROEENTROPYFIX: case FG_RIEMANN_ROEL2:
    case FG_RIEMANN_ROEENTROPYGSHOCKFIX: case FG_RIEMANN_HLL: case FG_RIEMANN_HLLE: case FG_RIEMANN_HLLEM: case FG_RIEMANN_CH:
    case FG_RIEMANN_IR: case FG_RIEMANN_AVERAGE: return true;
    default: return false;
  }
}

std::string lower(std::string s) {
  for (char& c : s) c = (char)std::tolower((unsigned char)c);
  return s;
}
std::string trim(const std::string& s) {
  size_t a = s.find_first_not_of(" \t\r\n"), b = s.find_last_not_of(" \t\r\n");
  return a == std::string::npos ? "" : s.substr(a, b - a + 1);
}

}  // namespace

namespace fg {
void set_error_without_handle(const char* msg) { g_err = msg; }
}  // namespace fg

namespace {

// the adjoint kernels cover: the weak form and every split form (Gauss, Gauss-Lobatto), every Riemann solver, strong
// non-conservative BR1/BR2 lifting, N <= 7
const char* adjoint_unsupported(const fg_config& c) {
  if (c.N > 7) return "the adjoint supports N = 1..7";
  if (c.doWeakLifting || c.doConservativeLifting) return "the adjoint supports the strong, non-conservative lifting";
  return nullptr;
}

int ensure_adjoint(fg_handle* h) {
  if (h->haveAdj) return 0;
  const int n = h->M.n, n2 = n * n, n3 = n2 * n, nE = h->M.nElems, nS = h->M.nSides;
  AdjDev& a = h->a;
  double* W = nullptr;
  int r = 0;
  if ((r = dalloc(h, W, (size_t)nE * 5 * n3))) return r;
  a.W = W;
  if ((r = dalloc(h, a.Ub, (size_t)nE * 5 * n3))) return r;
  if (h->ov.type > 0 && (r = dalloc(h, h->adjWov, (size_t)nE * 5 * n3))) return r;
  if ((r = dalloc(h, a.gb, (size_t)nE * 12 * n3))) return r;
  if ((r = dalloc(h, a.fluxb, (size_t)nS * 2 * 5 * n2))) return r;
  if ((r = dalloc(h, a.faceMb, (size_t)nS * FS_NF * n2))) return r;
  if ((r = dalloc(h, a.faceSb, (size_t)nS * FS_NF * n2))) return r;
  if ((r = dalloc(h, a.gradMb, (size_t)nS * 12 * n2))) return r;
  if ((r = dalloc(h, a.gradSb, (size_t)nS * 12 * n2))) return r;
  if ((r = dalloc(h, a.liftb, (size_t)nS * 2 * 4 * n2))) return r;
  if ((r = dalloc(h, a.muSideb, (size_t)nS * 2 * n2))) return r;
  if ((r = dalloc(h, a.muElemb, (size_t)nE))) return r;
  a.liftMortarb = nullptr;
  if (h->d.nMortars > 0) {
    if ((r = dalloc(h, a.liftMortarb, (size_t)h->d.nMortars * 12 * n2))) return r;
    CUDA_TRY(cudaMemset(a.liftMortarb, 0, sizeof(double) * h->d.nMortars * 12 * n2));
  }
  a.faceVolb = nullptr;
  if (h->cfg.SplitDG != FG_SPLIT_NONE && h->cfg.NodeType == FG_NODE_GAUSS) {
    if ((r = dalloc(h, a.faceVolb, (size_t)nS * 2 * FS_NF * n2))) return r;
    CUDA_TRY(cudaMemset(a.faceVolb, 0, sizeof(double) * nS * 2 * FS_NF * n2));
  }
  // entries no kernel writes (slave slots of boundary sides) stay zero
  CUDA_TRY(cudaMemset(a.faceSb, 0, sizeof(double) * nS * FS_NF * n2));
  CUDA_TRY(cudaMemset(a.gradSb, 0, sizeof(double) * nS * 12 * n2));
  CUDA_TRY(cudaMemset(a.liftb, 0, sizeof(double) * nS * 2 * 4 * n2));
  CUDA_TRY(cudaMemset(a.fluxb, 0, sizeof(double) * nS * 2 * 5 * n2));
  CUDA_TRY(cudaMemset(a.muSideb, 0, sizeof(double) * nS * 2 * n2));
  h->haveAdj = true;
  return 0;
}

// V = (dUt/dU)^T W at the state d.U, W in a.W; leaves V in a.Ub and the viscosity-multiplier
// cotangent in a.muElemb (added to them when a.accumulate)
// overintegration.f90 transposed: the cotangent W of Ut = G(J u_t) becomes W' = G^T(W) / sJ, which the
// adjoint volume kernel (that multiplies by -sJ, the transposed Jacobian) then carries into J u_t; G^T is the
// state-mode filter kernel run with the transposed matrices on sJ W (type 1: G = sJ F3, G^T W = F3^T (sJ W);
// type 2: G = VUN sJNU VNU, G^T W = VNU^T sJNU VUN^T W, the state mode dividing its input by sJ first)
AdjDev overint_adj_cotangent(fg_handle* h, const Dev& d, const AdjDev& a) {
  if (h->ov.type == 0) return a;
  const int n3 = h->M.n * h->M.n * h->M.n;
  const long long cnt = (long long)d.nElems * 5 * n3;
  k_scale_by_sj<<<(unsigned)((cnt + 255) / 256), 256, 0, h->st>>>(a.W, d.sJ, h->adjWov, n3, cnt, 1);
  Dev dv = d;
  dv.U = h->adjWov;
  h->K.overint(dv, h->ovT, 0, 0., 0., 1, h->st);
  k_scale_by_sj<<<(unsigned)((cnt + 255) / 256), 256, 0, h->st>>>(h->adjWov, d.sJ, h->adjWov, n3, cnt, 0);
  h->launches += 3;
  AdjDev b = a;
  b.W = h->adjWov;
  return b;
}

// the transposed kernels in reverse order of the forward's (prep, mortar_pre, lift, flux, mortar_face, volume)
static void launch_vjp_sweep(fg_handle* h, const Dev& d, const AdjDev& a) {
  const bool mortars = d.nMortars > 0;
  h->K.vol_adj(d, a, h->B, h->st);
  h->K.flux_adj(d, a, h->B, h->st);
  if (mortars) h->K.mortar_face_adj(d, a, h->B, h->mort, h->st);
  (mortars ? h->K.lift_mortar_adj : h->K.lift_adj)(d, a, h->B, h->st);
  if (mortars) h->K.mortar_pre_adj(d, a, h->B, h->mort, h->st);
  h->K.prep_adj(d, a, h->B, h->st);
  h->launches += mortars ? 6 : 4;
}

void launch_vjp(fg_handle* h, const Dev& d, const AdjDev& a0) {
  const AdjDev a = overint_adj_cotangent(h, d, a0);
  h->K.prep(d, h->B, h->st);
  if (d.nMortars > 0) {
    h->K.mortar_pre(d, h->B, h->mort, h->st);
    h->K.lift_mortar(d, h->B, h->st);
    h->launches += 1;
  } else {
    h->K.lift(d, h->B, h->st);
  }
  h->launches += 2;
  launch_vjp_sweep(h, d, a);
}

// adjoint right-hand side on forward intermediates the caller kept (no prep/lift recomputation)
void launch_vjp_kept(fg_handle* h, const Dev& d, const AdjDev& a0) {
  launch_vjp_sweep(h, d, overint_adj_cotangent(h, d, a0));
}

int adj_alloc(fg_handle* h, double*& p, size_t count) {
  void* q = nullptr;
  cudaError_t e = cudaMalloc(&q, count * sizeof(double));
  if (e != cudaSuccess) return fail(h, FG_ERR_CUDA, std::string("cudaMalloc (adjoint checkpoints): ") + cudaGetErrorString(e));
  h->adjStore.push_back(q);
  p = (double*)q;
  return 0;
}

}  // namespace

extern "C" {

int fg_config_default(fg_config* c) {
  if (!c) return FG_ERR_CONFIG;
  std::memset(c, 0, sizeof(*c));
  c->N = 3; c->NodeType = FG_NODE_GAUSS; c->Riemann = FG_RIEMANN_ROEENTROPYFIX; c->RiemannBC = FG_RIEMANN_SAME;
  c->Lifting = 1; c->doWeakLifting = 0; c->doConservativeLifting = 0; c->SplitDG = FG_SPLIT_PI;
  c->etaBR2 = 2.; c->etaBR2_wall = -1.; c->kappa = 1.4; c->R = 287.058; c->Pr = 0.72; c->mu0 = 0.;
  c->CFLScale = 0.9; c->DFLScale = 0.9; c->doTCSource = 0; c->dpdx = -1.; c->TimeDiscMethod = 0;
  c->OverintegrationType = 0; c->NUnder = -1;
  c->IniExactFunc = 0; c->AdvVel[0] = c->AdvVel[1] = c->AdvVel[2] = 0.; c->IniFrequency = 1.; c->IniAmplitude = 0.1;
  c->TEnd = INFINITY; c->Analyze_dt = 0.; c->dtmin = -1.; c->dtkill = -1.; c->nCalcTimeStepMax = 1; c->maxIter = -1;
  c->RiemannPhiFactor = 5.;
  return FG_OK;
}

int fg_config_from_ini(const char* text, fg_config* c) {
  if (!text || !c) return FG_ERR_CONFIG;
  std::istringstream in(text);
  std::string line;
  while (std::getline(in, line)) {
    const size_t bang = line.find('!');
    if (bang != std::string::npos) line = line.substr(0, bang);
    const size_t eq = line.find('=');
    if (eq == std::string::npos) continue;
    const std::string key = lower(trim(line.substr(0, eq))), val = trim(line.substr(eq + 1)), lv = lower(val);
    try {
      if (key == "n") c->N = std::stoi(val);
      else if (key == "nodetype") c->NodeType = (lv == "gauss-lobatto" || lv == "2") ? FG_NODE_GAUSS_LOBATTO : FG_NODE_GAUSS;
      else if (key == "riemann" || key == "riemannbc") {
        int id;
        if (lv == "lf") id = FG_RIEMANN_LF;
        else if (lv == "hllc") id = FG_RIEMANN_HLLC;
        else if (lv == "roe") id = FG_RIEMANN_ROE;
        else if (lv == "roeentropyfix") id = FG_RIEMANN_ROEENTROPYFIX;
        else if (lv == "roel2") id = FG_RIEMANN_ROEL2;
        else if (lv == "roeentropygshockfix") id = FG_RIEMANN_ROEENTROPYGSHOCKFIX;
        else if (lv == "hll") id = FG_RIEMANN_HLL;
        else if (lv == "hlle") id = FG_RIEMANN_HLLE;
        else if (lv == "hllem") id = FG_RIEMANN_HLLEM;
        else if (lv == "ch") id = FG_RIEMANN_CH;
        else if (lv == "ir") id = FG_RIEMANN_IR;
        else if (lv == "avg") id = FG_RIEMANN_AVERAGE;
        else if (lv == "same") id = FG_RIEMANN_SAME;
        else id = std::stoi(val);
        (key == "riemann" ? c->Riemann : c->RiemannBC) = id;
      } else if (key == "splitdg") {
        if (lv == "sd") c->SplitDG = FG_SPLIT_SD;
        else if (lv == "mo") c->SplitDG = FG_SPLIT_MO;
        else if (lv == "du") c->SplitDG = FG_SPLIT_DU;
        else if (lv == "kg") c->SplitDG = FG_SPLIT_KG;
        else if (lv == "pi") c->SplitDG = FG_SPLIT_PI;
        else if (lv == "ch") c->SplitDG = FG_SPLIT_CH;
        else if (lv == "ir") c->SplitDG = FG_SPLIT_IR;
        else if (lv == "none" || lv == "off") c->SplitDG = FG_SPLIT_NONE;
        else c->SplitDG = std::stoi(val);
      } else if (key == "lifting") c->Lifting = (lv == "br2" || lv == "2") ? 2 : 1;
      else if (key == "doweaklifting") c->doWeakLifting = (lv == "t" || lv == ".true." || lv == "true" || lv == "1");
      else if (key == "doconservativelifting") c->doConservativeLifting = (lv == "t" || lv == ".true." || lv == "true" || lv == "1");
      else if (key == "etabr2") c->etaBR2 = std::stod(val);
      else if (key == "etabr2_wall") c->etaBR2_wall = std::stod(val);
      else if (key == "kappa") c->kappa = std::stod(val);
      else if (key == "r") c->R = std::stod(val);
      else if (key == "pr") c->Pr = std::stod(val);
      else if (key == "mu0") c->mu0 = std::stod(val);
      else if (key == "cflscale") c->CFLScale = std::stod(val);
      else if (key == "dflscale") c->DFLScale = std::stod(val);
      else if (key == "timediscmethod") c->TimeDiscMethod = fgh::lserk_method(lv.c_str());
      else if (key == "overintegrationtype") {
        if (lv == "none") c->OverintegrationType = 0;
        else if (lv == "cutoff") c->OverintegrationType = 1;
        else if (lv == "conscutoff") c->OverintegrationType = 2;
        else c->OverintegrationType = std::stoi(val);
      } else if (key == "nunder") c->NUnder = std::stoi(val);
      else if (key == "iniexactfunc") c->IniExactFunc = std::stoi(val);
      else if (key == "inifrequency") c->IniFrequency = std::stod(val);
      else if (key == "iniamplitude") c->IniAmplitude = std::stod(val);
      else if (key == "tend") c->TEnd = std::stod(val);
      else if (key == "analyze_dt") c->Analyze_dt = std::stod(val);
      else if (key == "dtmin") c->dtmin = std::stod(val);
      else if (key == "dtkill") c->dtkill = std::stod(val);
      else if (key == "ncalctimestepmax") c->nCalcTimeStepMax = std::stoi(val);
      else if (key == "maxiter") c->maxIter = std::stoi(val);
      else if (key == "riemannphifactor") c->RiemannPhiFactor = std::stod(val);
      else if (key == "advvel") {  // (/a,b,c/)
        std::string v = val;
        for (char& ch : v) if (ch == '(' || ch == ')' || ch == '/' || ch == ',') ch = ' ';
        std::istringstream vs(v);
        for (int d = 0; d < 3; ++d)
          if (!(vs >> c->AdvVel[d])) return FG_ERR_CONFIG;
      }
    } catch (...) {
      return FG_ERR_CONFIG;
    }
  }
  return FG_OK;
}

int fg_create(const fg_config* cfg, fg_handle** out) {
  if (!cfg || !out) return FG_ERR_CONFIG;
  *out = nullptr;
  fg_handle* h = new fg_handle();
  h->cfg = *cfg;
  if (h->cfg.Lifting == 2) h->cfg.doWeakLifting = 0;  // lifting.f90:137-139: BR2 lifts in strong form
  const fg_config& c = h->cfg;
  std::string why;
  if (c.N < 1 || c.N > 11) why = "N must be in 1..11";
  else if (c.NodeType != FG_NODE_GAUSS && c.NodeType != FG_NODE_GAUSS_LOBATTO) why = "NodeType must be 1 (Gauss) or 2 (Gauss-Lobatto)";
  else if (!riemann_known(c.Riemann))
    why = "Riemann must be one of LF, HLLC, Roe, RoeEntropyFix, RoeL2, RoeEntropyGShockFix, HLL, HLLE, HLLEM (and with the split form CH, IR, avg)";
  else if (c.SplitDG == FG_SPLIT_NONE && (c.Riemann == FG_RIEMANN_CH || c.Riemann == FG_RIEMANN_IR || c.Riemann == FG_RIEMANN_AVERAGE))
    why = "the Riemann solvers CH, IR and avg need the split form (riemann.f90:204-223)";
  else if (c.RiemannBC != FG_RIEMANN_SAME && !riemann_known(c.RiemannBC)) why = "RiemannBC must be Same or one of the Riemann solvers";
  else if (c.Lifting != 1 && c.Lifting != 2) why = "Lifting must be 1 (BR1) or 2 (BR2)";
  else if (c.SplitDG < FG_SPLIT_NONE || c.SplitDG > FG_SPLIT_IR) why = "SplitDG must be -1 (weak), 0 SD, 1 MO, 2 DU, 3 KG, 4 PI, 5 CH or 6 IR";
  else if (c.Riemann == FG_RIEMANN_ROEENTROPYGSHOCKFIX && !(c.RiemannPhiFactor > 0.)) why = "RiemannPhiFactor must be > 0";
  else if (!fgh::lserk_scheme(c.TimeDiscMethod))
    why = "TimeDiscMethod must be one of the low-storage schemes 0..5 (carpenterrk4-5, standardrk3-3, niegemannrk4-14, "
          "toulorgerk4-8c, toulorgerk3-7c, toulorgerk4-8f)";
  else if (c.OverintegrationType < 0 || c.OverintegrationType > 2) why = "OverintegrationType must be 0 (none), 1 (cutoff) or 2 (conscutoff)";
  else if (c.OverintegrationType > 0 && c.NUnder < -1) why = "NUnder must be >= 0";
  else if (c.nCalcTimeStepMax < 1) why = "nCalcTimeStepMax must be >= 1";
  else if (!(c.TEnd > 0.)) why = "TEnd must be > 0";
  if (!why.empty()) { delete h; return fail(nullptr, FG_ERR_CONFIG, why); }
  h->K = get_kernel_set(c.N + 1, c.NodeType == FG_NODE_GAUSS_LOBATTO);
  h->Kdef = h->K;
  if (h->K.n == 0) { delete h; return fail(nullptr, FG_ERR_CONFIG, "no kernels for this N"); }
  init_basis(h);
  *out = h;
  return FG_OK;
}

int fg_destroy(fg_handle* h) {
  if (!h) return FG_OK;
  free_device(h);
  for (auto& e : h->evOut)
    if (e) cudaEventDestroy(e);
  if (h->evOutDone) cudaEventDestroy(h->evOutDone);
  if (h->stOut) cudaStreamDestroy(h->stOut);
  if (h->st) cudaStreamDestroy(h->st);
  delete h;
  return FG_OK;
}

const char* fg_last_error(const fg_handle* h) { return h ? h->err.c_str() : g_err.c_str(); }

int fg_build_mesh(fg_handle* h, int nElems, int NGeo, const double* NodeCoords, const int* ElemNb, int nBCs, const int* BoundaryType,
                  int nRefStates, const double* RefStatePrim, const int* ElemInst) {
  return fg_build_mesh_mortar(h, nElems, NGeo, NodeCoords, ElemNb, nBCs, BoundaryType, nRefStates, RefStatePrim, ElemInst, 0, nullptr);
}

int fg_build_mesh_mortar(fg_handle* h, int nElems, int NGeo, const double* NodeCoords, const int* ElemNb, int nBCs, const int* BoundaryType,
                         int nRefStates, const double* RefStatePrim, const int* ElemInst, int nMortars, const int* Mortars) {
  if (!h) return FG_ERR_STATE;
  if (nElems <= 0 || NGeo < 1 || !NodeCoords || !ElemNb) return fail(h, FG_ERR_MESH, "invalid mesh arguments");
  if (nMortars < 0 || (nMortars > 0 && !Mortars)) return fail(h, FG_ERR_MESH, "invalid mortar table");
  try {
    fgh::RawMesh R;
    R.nElems = nElems; R.NGeo = NGeo; R.nodeCoords = NodeCoords; R.elemNb = ElemNb; R.nBCs = nBCs; R.boundaryType = BoundaryType;
    R.nRefStates = nRefStates; R.refStatePrim = RefStatePrim; R.elemInst = ElemInst;
    R.nMortars = nMortars; R.mortars = Mortars;
    fgh::build_from_raw(R, h->cfg.N, h->cfg.NodeType == FG_NODE_GAUSS_LOBATTO ? fgh::LOBATTO : fgh::GAUSS, h->M);
  } catch (std::exception& e) {
    return fail(h, FG_ERR_MESH, e.what());
  }
  return upload_mesh(h);
}

int fg_set_mesh(fg_handle* h, int nElems, int nSides, int nBCSides, const int* SideToElem, const int* ElemToSide, const int* BC, int nBCs,
                const int* BoundaryType, int nRefStates, const double* RefStatePrim, const double* Mf, const double* Mg, const double* Mh,
                const double* sJ, const double* NormVec, const double* TangVec1, const double* TangVec2, const double* SurfElem) {
  return fg_set_mesh_mortar(h, nElems, nSides, nBCSides, SideToElem, ElemToSide, BC, nBCs, BoundaryType, nRefStates, RefStatePrim, Mf, Mg,
                            Mh, sJ, NormVec, TangVec1, TangVec2, SurfElem, 0, nullptr, nullptr);
}

int fg_set_mesh_mortar(fg_handle* h, int nElems, int nSides, int nBCSides, const int* SideToElem, const int* ElemToSide, const int* BC,
                       int nBCs, const int* BoundaryType, int nRefStates, const double* RefStatePrim, const double* Mf, const double* Mg,
                       const double* Mh, const double* sJ, const double* NormVec, const double* TangVec1, const double* TangVec2,
                       const double* SurfElem, int nMortars, const int* MortarType, const int* MortarInfo) {
  if (!h) return FG_ERR_STATE;
  try {
    fgh::build_from_flexi(h->cfg.N, h->cfg.NodeType == FG_NODE_GAUSS_LOBATTO ? fgh::LOBATTO : fgh::GAUSS, nElems, nSides, nBCSides,
                          SideToElem, ElemToSide, BC, nBCs, BoundaryType, nRefStates, RefStatePrim, Mf, Mg, Mh, sJ, NormVec, TangVec1,
                          TangVec2, SurfElem, nMortars, MortarType, MortarInfo, h->M);
  } catch (std::exception& e) {
    return fail(h, FG_ERR_MESH, e.what());
  }
  return upload_mesh(h);
}

int fg_set_face_metrics(fg_handle* h, const double* Ja_Face, const double* Ja_slave) {
  if (!h || !h->haveHostMesh) return fail(h, FG_ERR_STATE, "fg_set_face_metrics needs a mesh");
  if (!Ja_Face || !Ja_slave) return fail(h, FG_ERR_CONFIG, "Ja_Face and Ja_slave are required");
  fgh::HostMesh& M = h->M;
  const int n = M.n, n2 = n * n, N = M.N;
  static const int normalDir[7] = {0, 2, 1, 0, 1, 0, 2};  // 0-based row, mesh_vars.f90:105-111
  for (int e = 0; e < M.nElems; ++e)
    for (int ls = 1; ls <= 6; ++ls) {
      const int code = M.elemSide[e * 6 + ls - 1], flip = code & 7;
      const int s = M.flexiSide.empty() ? code >> 3 : M.flexiSide[code >> 3];  // FLEXI's side numbering
      const double* J = flip == 0 ? Ja_Face : Ja_slave;
      for (int q = 0; q < n; ++q)
        for (int p = 0; p < n; ++p) {
          int a, b;
          side_to_vol2(N, p, q, flip, ls, a, b);
          for (int c = 0; c < 3; ++c)
            M.faceJa[(((size_t)e * 6 + ls - 1) * 3 + c) * n2 + a + n * b] = J[((((size_t)s * n + q) * n + p) * 3 + c) * 3 + normalDir[ls]];
        }
    }
  if (h->haveMesh && h->d.faceJa)
    CUDA_TRY(cudaMemcpy(h->d.faceJa, M.faceJa.data(), sizeof(double) * M.faceJa.size(), cudaMemcpyHostToDevice));
  return FG_OK;
}

int fg_overintegrate_state(fg_handle* h) {
  if (!h || !h->haveMesh) return fail(h, FG_ERR_STATE, "fg_overintegrate_state needs a mesh");
  if (h->ov.type == 0) return FG_OK;
  h->K.overint(h->d, h->ov, 0, 0., 0., 1, h->st);
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaStreamSynchronize(h->st));
  return FG_OK;
}

int fg_set_instance_mu0(fg_handle* h, int nInst, const double* mu0) {
  if (!h || !mu0 || nInst <= 0) return FG_ERR_CONFIG;
  h->instMu0.assign(mu0, mu0 + nInst);
  if (h->haveMesh) {
    if (nInst != h->d.nInst) return fail(h, FG_ERR_CONFIG, "instance count mismatch");
    CUDA_TRY(cudaMemcpy(h->d.mu0, mu0, sizeof(double) * nInst, cudaMemcpyHostToDevice));
  }
  return FG_OK;
}

int fg_lserk_table(int method, int* stages, double* A, double* b, double* c, double* cflAlpha, double* relativeDFL) {
  const fgh::LSERKScheme* s = fgh::lserk_scheme(method);
  if (!s || !stages) return FG_ERR_CONFIG;
  *stages = s->stages;
  for (int i = 0; i < 21; ++i) {
    if (A) A[i] = s->A[i];
    if (b) b[i] = s->b[i];
    if (c) c[i] = s->c[i];
  }
  if (cflAlpha)
    for (int i = 0; i < 15; ++i) { cflAlpha[i] = s->cflGauss[i]; cflAlpha[15 + i] = s->cflGL[i]; }
  if (relativeDFL) *relativeDFL = s->relativeDFL;
  return FG_OK;
}

int fg_get_config(const fg_handle* h, fg_config* out) {
  if (!h || !out) return FG_ERR_STATE;
  *out = h->cfg;
  return FG_OK;
}

int fg_get_sizes(const fg_handle* h, int* out) {
  if (!h || !out) return FG_ERR_STATE;
  out[0] = h->M.nElems; out[1] = h->M.nSides; out[2] = h->M.nBCSides; out[3] = h->cfg.N; out[4] = h->M.nInst;
  return FG_OK;
}

int fg_get_elem_xgp(fg_handle* h, double* X) {
  if (!h || !h->haveHostMesh || h->M.elemX.empty()) return fail(h, FG_ERR_STATE, "no solution coordinates (mesh not built from nodes)");
  const int n3 = h->M.n * h->M.n * h->M.n;
  for (int e = 0; e < h->M.nElems; ++e)
    for (int x = 0; x < n3; ++x)
      for (int c = 0; c < 3; ++c) X[((size_t)e * n3 + x) * 3 + c] = h->M.elemX[((size_t)e * 3 + c) * n3 + x];
  return FG_OK;
}

int fg_get_mesh_array(fg_handle* h, int which, double* out) {
  if (!h || !h->haveHostMesh) return fail(h, FG_ERR_STATE, "no mesh");
  const fgh::HostMesh& M = h->M;
  const int n = M.n, n2 = n * n, n3 = n2 * n;
  if (which >= 0 && which <= 2) {
    for (int e = 0; e < M.nElems; ++e) for (int x = 0; x < n3; ++x) for (int c = 0; c < 3; ++c)
      out[((size_t)e * n3 + x) * 3 + c] = M.metr[((size_t)e * 9 + 3 * which + c) * n3 + x];
  } else if (which == 3) {
    std::copy(M.sJ.begin(), M.sJ.end(), out);
  } else if (which >= 4 && which <= 6) {
    for (int s = 0; s < M.nSides; ++s) for (int pq = 0; pq < n2; ++pq) for (int c = 0; c < 3; ++c)
      out[((size_t)s * n2 + pq) * 3 + c] = M.geo[((size_t)s * 10 + 3 * (which - 4) + c) * n2 + pq];
  } else if (which == 7) {
    for (int s = 0; s < M.nSides; ++s) for (int pq = 0; pq < n2; ++pq) out[(size_t)s * n2 + pq] = M.geo[((size_t)s * 10 + 9) * n2 + pq];
  } else return fail(h, FG_ERR_CONFIG, "unknown mesh array");
  return FG_OK;
}

int fg_get_side_to_elem(fg_handle* h, int* out) {
  if (!h || !h->haveHostMesh) return fail(h, FG_ERR_STATE, "no mesh");
  for (int s = 0; s < h->M.nSides; ++s) {
    const int* r = &h->M.sideElem[s * 4];
    out[s * 5 + 0] = r[0] + 1; out[s * 5 + 2] = r[1];
    out[s * 5 + 1] = r[2] >= 0 ? r[2] + 1 : -1;
    out[s * 5 + 3] = r[2] >= 0 ? r[3] >> 3 : -1;
    out[s * 5 + 4] = r[2] >= 0 ? r[3] & 7 : 0;
  }
  return FG_OK;
}

// Fortran layout (nv, n, n, n, nElems) in device memory -> device layout [e][nv][n3], on the handle's stream
static void fortran_to_dev(fg_handle* h, const double* f, double* d, int nv) {
  const int n3 = h->M.n * h->M.n * h->M.n;
  const size_t bytes = sizeof(double) * nv * n3;
  if (bytes <= FG_TILE_SMEM_MAX) {
    cudaFuncSetAttribute(k_fortran_to_dev_tiled, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    k_fortran_to_dev_tiled<<<(unsigned)h->M.nElems, 256, bytes, h->st>>>(f, d, nv, n3);
  } else {
    const long long total = (long long)h->M.nElems * nv * n3;
    k_fortran_to_dev<<<(unsigned)((total + 255) / 256), 256, 0, h->st>>>(f, d, nv, n3, total);
  }
}
// device layout [e][nvDev][n3], variables v0 .. v0+nv-1 -> Fortran layout (nv, n, n, n, nElems) in device memory
// nElems elements (all: -1) from the device layout at d to the Fortran layout at f, on stream st (null: the handle's)
static void dev_to_fortran(fg_handle* h, const double* d, double* f, int nvDev, int v0, int nv, int nElems = -1, cudaStream_t st = nullptr) {
  const int n3 = h->M.n * h->M.n * h->M.n;
  const size_t bytes = sizeof(double) * nv * n3;
  if (nElems < 0) nElems = h->M.nElems;
  if (!st) st = h->st;
  if (nElems == 0) return;
  if (bytes <= FG_TILE_SMEM_MAX) {
    cudaFuncSetAttribute(k_dev_to_fortran_tiled, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    k_dev_to_fortran_tiled<<<(unsigned)nElems, 256, bytes, st>>>(d, f, nvDev, v0, nv, n3);
  } else {
    const long long total = (long long)nElems * nv * n3;
    k_dev_to_fortran<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(d, f, nvDev, v0, nv, n3, total);
  }
}

int fg_set_state(fg_handle* h, const double* U) {
  if (!h || !h->haveMesh) return fail(h, FG_ERR_STATE, "no mesh");
  const int n3 = h->M.n * h->M.n * h->M.n;
  const long long total = (long long)h->M.nElems * 5 * n3;
  CUDA_TRY(cudaMemcpyAsync(h->dStage, U, total * sizeof(double), cudaMemcpyHostToDevice, h->st));
  fortran_to_dev(h, h->dStage, h->d.U, 5);
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaStreamSynchronize(h->st));
  return FG_OK;
}

static int export_field(fg_handle* h, const double* dsrc, int nvDev, int v0, int nv, double* out) {
  const int n3 = h->M.n * h->M.n * h->M.n;
  const long long total = (long long)h->M.nElems * nv * n3;
  dev_to_fortran(h, dsrc, h->dStage, nvDev, v0, nv);
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaMemcpyAsync(out, h->dStage, total * sizeof(double), cudaMemcpyDeviceToHost, h->st));
  CUDA_TRY(cudaStreamSynchronize(h->st));
  return FG_OK;
}

int fg_get_state(fg_handle* h, double* U) {
  if (!h || !h->haveMesh) return fail(h, FG_ERR_STATE, "no mesh");
  return export_field(h, h->d.U, 5, 0, 5, U);
}

int fg_state_device_ptr(fg_handle* h, double** p) {
  if (!h || !h->haveMesh || !p) return fail(h, FG_ERR_STATE, "no mesh");
  *p = h->d.U;
  return FG_OK;
}

int fg_time_derivative(fg_handle* h, double t, double* Ut) {
  if (!h || !h->haveMesh) return fail(h, FG_ERR_STATE, "no mesh");
  h->launches = 0;
  if (h->d.srcPar) {  // the source is evaluated at t
    k_fill<<<(h->d.nInst + 127) / 128, 128, 0, h->st>>>(h->d.tStage, t, h->d.nInst);
    h->launches += 1;
  }
  launch_step_setup(h, 2, 0., false);
  launch_rhs(h, 0, 0., 0.);
  CUDA_TRY(cudaGetLastError());
  if (Ut) return export_field(h, h->d.Ut, 5, 0, 5, Ut);
  CUDA_TRY(cudaStreamSynchronize(h->st));
  return FG_OK;
}

int fg_set_elem_mu_scale(fg_handle* h, const double* scale) {
  if (!h || !h->haveMesh) return fail(h, FG_ERR_STATE, "no mesh");
  const int nE = h->M.nElems;
  if (scale) {
    CUDA_TRY(cudaMemcpy(h->d.muScale, scale, sizeof(double) * nE, cudaMemcpyHostToDevice));
  } else {
    k_fill<<<(nE + 127) / 128, 128, 0, h->st>>>(h->d.muScale, 1.0, nE);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaStreamSynchronize(h->st));
  }
  return FG_OK;
}

int fg_jvp_time_derivative(fg_handle* h, double t, const double* V, double* JV, int fdOrder, int epsMethod, double scaleps) {
  (void)t;  // no time-dependent source on this path
  if (!h || !h->haveMesh) return fail(h, FG_ERR_STATE, "no mesh");
  if (!V || !JV) return fail(h, FG_ERR_CONFIG, "null vector");
  if ((fdOrder != 1 && fdOrder != 2) || (epsMethod != 1 && epsMethod != 2) || !(scaleps > 0.))
    return fail(h, FG_ERR_CONFIG, "fdOrder 1/2, epsMethod 1/2 and scaleps > 0 required");
  const int n3 = h->M.n * h->M.n * h->M.n;
  const long long cnt = (long long)h->M.nElems * 5 * n3;
  const size_t bytes = (size_t)cnt * sizeof(double);
  const unsigned grid = (unsigned)((cnt + 255) / 256);
  const int nPart = 1024;
  if (!h->jvpXk) {
    int r = 0;
    if ((r = dalloc(h, h->jvpXk, (size_t)cnt)) || (r = dalloc(h, h->jvpV, (size_t)cnt)) || (r = dalloc(h, h->jvpR, (size_t)cnt)) ||
        (r = dalloc(h, h->jvpPartial, (size_t)nPart))) return r;
  }
  h->launches = 0;
  // step size of InitImplicit / MatrixVector: |V| from the host vector, |Xk| from the device state
  double Vabs = 0.;
  for (long long i = 0; i < cnt; ++i) Vabs += V[i] * V[i];
  if (!(Vabs > 0.)) return fail(h, FG_ERR_CONFIG, "zero direction");
  double normXk = 0.;
  if (epsMethod == 2) {
    k_sumsq_partial<<<nPart, 256, 0, h->st>>>(h->d.U, cnt, h->jvpPartial);
    std::vector<double> part(nPart);
    CUDA_TRY(cudaMemcpyAsync(part.data(), h->jvpPartial, sizeof(double) * nPart, cudaMemcpyDeviceToHost, h->st));
    CUDA_TRY(cudaStreamSynchronize(h->st));
    for (double p : part) normXk += p;
    normXk = std::sqrt(normXk);
  }
  const double mach = 2.220446049250313e-16;
  const double rEps0 = fdOrder == 1 ? scaleps * std::sqrt(mach) : std::cbrt(scaleps * scaleps * 0.5 * mach);
  double eps = rEps0 / std::sqrt(Vabs);
  if (epsMethod == 2) eps *= std::sqrt(1. + normXk);
  CUDA_TRY(cudaMemcpyAsync(h->dStage, V, bytes, cudaMemcpyHostToDevice, h->st));
  fortran_to_dev(h, h->dStage, h->jvpV, 5);
  CUDA_TRY(cudaMemcpyAsync(h->jvpXk, h->d.U, bytes, cudaMemcpyDeviceToDevice, h->st));
  launch_step_setup(h, 2, 0., false);  // bulk velocity of Xk, held for every evaluation
  if (fdOrder == 1) {
    launch_rhs(h, 0, 0., 0.);
    CUDA_TRY(cudaMemcpyAsync(h->jvpR, h->d.Ut, bytes, cudaMemcpyDeviceToDevice, h->st));
  }
  k_axpy_out<<<grid, 256, 0, h->st>>>(h->d.U, h->jvpXk, eps, h->jvpV, cnt);
  launch_rhs(h, 0, 0., 0.);
  if (fdOrder == 1) {
    k_fd_diff<<<grid, 256, 0, h->st>>>(h->jvpR, h->d.Ut, h->jvpR, 1. / eps, cnt);
  } else {
    CUDA_TRY(cudaMemcpyAsync(h->jvpR, h->d.Ut, bytes, cudaMemcpyDeviceToDevice, h->st));
    k_axpy_out<<<grid, 256, 0, h->st>>>(h->d.U, h->jvpXk, -eps, h->jvpV, cnt);
    launch_rhs(h, 0, 0., 0.);
    k_fd_diff<<<grid, 256, 0, h->st>>>(h->jvpR, h->jvpR, h->d.Ut, 1. / (2. * eps), cnt);
  }
  CUDA_TRY(cudaMemcpyAsync(h->d.U, h->jvpXk, bytes, cudaMemcpyDeviceToDevice, h->st));
  CUDA_TRY(cudaGetLastError());
  return export_field(h, h->jvpR, 5, 0, 5, JV);
}

int fg_vjp_time_derivative(fg_handle* h, double t, const double* W, double* V, double* muScaleBar) {
  (void)t;  // no time-dependent source on this path
  if (!h || !h->haveMesh) return fail(h, FG_ERR_STATE, "no mesh");
  if (!W) return fail(h, FG_ERR_CONFIG, "null cotangent");
  if (const char* why = adjoint_unsupported(h->cfg)) return fail(h, FG_ERR_CONFIG, why);
  if (int r = ensure_adjoint(h)) return r;
  const int n3 = h->M.n * h->M.n * h->M.n;
  const long long total = (long long)h->M.nElems * 5 * n3;
  h->launches = 0;
  CUDA_TRY(cudaMemcpyAsync(h->dStage, W, total * sizeof(double), cudaMemcpyHostToDevice, h->st));
  fortran_to_dev(h, h->dStage, const_cast<double*>(h->a.W), 5);
  AdjDev a = h->a;
  a.accumulate = 0;
  launch_vjp(h, h->d, a);
  CUDA_TRY(cudaGetLastError());
  if (V) { if (int r = export_field(h, h->a.Ub, 5, 0, 5, V)) return r; }
  if (muScaleBar) CUDA_TRY(cudaMemcpyAsync(muScaleBar, h->a.muElemb, sizeof(double) * h->M.nElems, cudaMemcpyDeviceToHost, h->st));
  CUDA_TRY(cudaStreamSynchronize(h->st));
  return FG_OK;
}

// buffers of the reverse sweep for segments of up to segSteps steps: stage states (and, when they fit
// in half of the free device memory, the stage intermediates), running cotangents, final state
static int adjoint_alloc_common(fg_handle* h, int segSteps) {
  const int n3 = h->M.n * h->M.n * h->M.n, n2 = h->M.n * h->M.n;
  const size_t cnt = (size_t)h->M.nElems * 5 * n3;
  h->adjStage.assign((size_t)segSteps * h->nStages, nullptr);
  for (auto& p : h->adjStage) if (int r = adj_alloc(h, p, cnt)) return r;
  const size_t perStage = (size_t)h->M.nElems * (VP_NF + 12) * n3 + (size_t)h->M.nSides * (2 * FS_NF + 24) * n2;
  size_t freeB = 0, totalB = 0;
  cudaMemGetInfo(&freeB, &totalB);
  const char* env = std::getenv("FLEXI_GB300_ADJOINT_RECOMPUTE");
  const bool forceRecompute = env && env[0] == '1';
  if (!forceRecompute && perStage * sizeof(double) * h->adjStage.size() < freeB / 2) {
    h->adjKeepInter = true;
    h->adjInter.assign(h->adjStage.size(), h->d);
    for (size_t i = 0; i < h->adjStage.size(); ++i) {
      Dev& v = h->adjInter[i];
      v.U = h->adjStage[i];
      int r = 0;
      if ((r = adj_alloc(h, v.prim, (size_t)h->M.nElems * VP_NF * n3)) || (r = adj_alloc(h, v.grad, (size_t)h->M.nElems * 12 * n3)) ||
          (r = adj_alloc(h, v.faceM, (size_t)h->M.nSides * FS_NF * n2)) || (r = adj_alloc(h, v.faceS, (size_t)h->M.nSides * FS_NF * n2)) ||
          (r = adj_alloc(h, v.gradM, (size_t)h->M.nSides * 12 * n2)) || (r = adj_alloc(h, v.gradS, (size_t)h->M.nSides * 12 * n2)))
        return r;
    }
  }
  int r = 0;
  if ((r = adj_alloc(h, h->adjGbar, cnt)) || (r = adj_alloc(h, h->adjUbar, cnt)) || (r = adj_alloc(h, h->adjUfinal, cnt)) ||
      (r = adj_alloc(h, h->adjBulkHist, (size_t)segSteps * h->d.nInst)) || (r = adj_alloc(h, h->adjPartial, (size_t)h->M.nElems)) ||
      (r = adj_alloc(h, h->adjBulkBar, (size_t)h->d.nInst)) || (r = adj_alloc(h, h->adjFbar, (size_t)h->M.nElems * n3)))
    return r;
  return 0;
}

// ns fixed-dt steps forward from the state in d.U (nothing recorded)
// stage times of step k of the adjoint solve for the source (no-op without one)
static void adjoint_step_time(fg_handle* h, int k) {
  if (!h->d.srcPar) return;
  k_step_time<<<(h->d.nInst + 127) / 128, 128, 0, h->st>>>(h->d, h->adjT0, k * h->adjDt);
  h->launches += 1;
}

// ns forward steps from step firstStep of the adjoint solve
static void adjoint_advance(fg_handle* h, int ns, int firstStep) {
  for (int s = 0; s < ns; ++s) {
    adjoint_step_time(h, firstStep + s);
    launch_step_setup(h, 1, h->adjDt, false);
    launch_lserk(h);
  }
}

// reverse ns steps that start from the state Ustart (device; may be d.U itself): recompute their stage
// states (and intermediates), then run the transposed stages in reverse, accumulating into a.Ub (the
// running state cotangent), a.muElemb, adjFbar
static int adjoint_reverse_segment(fg_handle* h, const double* Ustart, int ns, const AdjDev& a, bool bulkAdj, int firstStep) {
  const int n3 = h->M.n * h->M.n * h->M.n;
  const long long cnt = (long long)h->M.nElems * 5 * n3;
  const size_t bytes = (size_t)cnt * sizeof(double);
  const unsigned gridAx = (unsigned)((cnt + 255) / 256);
  const double dt = h->adjDt;
  const int nI = h->d.nInst;
  if (Ustart != h->d.U) CUDA_TRY(cudaMemcpyAsync(h->d.U, Ustart, bytes, cudaMemcpyDeviceToDevice, h->st));
  for (int s = 0; s < ns; ++s) {
    adjoint_step_time(h, firstStep + s);
    launch_step_setup(h, 1, dt, false);
    CUDA_TRY(cudaMemcpyAsync(h->adjBulkHist + (size_t)s * nI, h->d.bulkVel, sizeof(double) * nI, cudaMemcpyDeviceToDevice, h->st));
    for (int k = 1; k <= h->nStages; ++k) {
      const size_t slot = (size_t)s * h->nStages + k - 1;
      if (h->d.srcPar) { k_stage_time<<<(nI + 127) / 128, 128, 0, h->st>>>(h->d, h->RKc[k]); h->launches += 1; }
      CUDA_TRY(cudaMemcpyAsync(h->adjStage[slot], h->d.U, bytes, cudaMemcpyDeviceToDevice, h->st));
      if (h->adjKeepInter) {
        // the stage writes its intermediates into the slot; the state is updated in place as usual
        Dev dv = h->adjInter[slot];
        dv.U = h->d.U;
        launch_rhs_dev(h, dv, k == 1 ? 1 : 2, k == 1 ? 0. : h->RKA[k], h->RKb[k]);
      } else {
        launch_rhs(h, k == 1 ? 1 : 2, k == 1 ? 0. : h->RKA[k], h->RKb[k]);
      }
    }
  }
  // Gbar_k = -A_{k+1} Gbar_{k+1} + b_k dt Ubar; Ubar += J(U_{k-1})^T Gbar_k
  for (int s = ns - 1; s >= 0; --s) {
    for (int k = h->nStages; k >= 1; --k) {
      k_adj_axpby<<<gridAx, 256, 0, h->st>>>(h->adjGbar, h->adjUbar, k == h->nStages ? 0. : -h->RKA[k + 1], h->RKb[k] * dt, cnt);
      k_adj_source<<<h->M.nElems, 128, 0, h->st>>>(h->d, h->adjGbar, h->adjFbar, h->adjPartial, h->adjBulkHist + (size_t)s * nI, n3);
      h->launches += 2;
      const size_t slot = (size_t)s * h->nStages + k - 1;
      if (h->adjKeepInter) {
        launch_vjp_kept(h, h->adjInter[slot], a);
      } else {
        Dev dv = h->d;
        dv.U = h->adjStage[slot];
        launch_vjp(h, dv, a);
      }
    }
    if (bulkAdj) {
      // the step's bulk velocity depends on its start state (stage 1 input)
      k_adj_bulk_reduce<<<(nI + 127) / 128, 128, 0, h->st>>>(nI, h->dInstStart, h->adjPartial, h->adjBulkBar);
      k_adj_bulk_apply<<<gridAx, 256, 0, h->st>>>(h->d, h->adjUbar, h->adjStage[(size_t)s * h->nStages], h->adjBulkBar, h->dWVol, h->dInstVol, n3);
      h->launches += 2;
    }
  }
  CUDA_TRY(cudaGetLastError());
  return 0;
}

// binomial checkpointing (Griewank): beta(s, r) = C(s + r, s) steps are reversible with s free snapshot
// slots and r forward repetitions. For t steps and s >= 1 free slots, the next snapshot is placed so that
// the part after it is the longest reversible with s - 1 slots at the smallest sufficient r.
static double binom_d(int n, int k) {
  double b = 1.;
  for (int i = 1; i <= k; ++i) b = b * (n - k + i) / i;
  return b;
}
static int revolve_split(int t, int s) {
  int r = 0;
  while (binom_d(s + r, s) < t) ++r;
  const double right = std::min((double)(t - 1), binom_d(s - 1 + r, s - 1));
  return t - (int)right;
}

struct RevolveRun {
  fg_handle* h;
  AdjDev a;
  bool bulkAdj;
  std::vector<int> freeSlots;
  size_t bytes;
};

// reverse steps [l, r) with U_l in slot slotL and s free slots
static int revolve_reverse(RevolveRun& R, int l, int r, int slotL, int s) {
  fg_handle* h = R.h;
  if (r - l == 1) {
    h->adjRecomputed += 1;
    return adjoint_reverse_segment(h, h->adjSlots[slotL], 1, R.a, R.bulkAdj, l);
  }
  if (s == 0) {  // no free slot: restart from U_l for every step
    for (int i = r - 1; i >= l; --i) {
      CUDA_TRY(cudaMemcpyAsync(h->d.U, h->adjSlots[slotL], R.bytes, cudaMemcpyDeviceToDevice, h->st));
      adjoint_advance(h, i - l, l);
      h->adjRecomputed += i - l + 1;
      if (int e = adjoint_reverse_segment(h, h->d.U, 1, R.a, R.bulkAdj, i)) return e;
    }
    return 0;
  }
  const int m = l + revolve_split(r - l, s);
  int slotM = -1;
  for (auto it = h->adjSpine.begin(); it != h->adjSpine.end(); ++it)
    if (it->first == m) { slotM = it->second; h->adjSpine.erase(it); break; }
  if (slotM < 0) {
    slotM = R.freeSlots.back();
    R.freeSlots.pop_back();
    CUDA_TRY(cudaMemcpyAsync(h->d.U, h->adjSlots[slotL], R.bytes, cudaMemcpyDeviceToDevice, h->st));
    adjoint_advance(h, m - l, l);
    h->adjRecomputed += m - l;
    CUDA_TRY(cudaMemcpyAsync(h->adjSlots[slotM], h->d.U, R.bytes, cudaMemcpyDeviceToDevice, h->st));
  }
  if (int e = revolve_reverse(R, m, r, slotM, s - 1)) return e;
  R.freeSlots.push_back(slotM);
  return revolve_reverse(R, l, m, slotL, s);
}

int fg_adjoint_forward(fg_handle* h, int nSteps, double dt, int ckptEvery) {
  if (!h || !h->haveMesh) return fail(h, FG_ERR_STATE, "no mesh");
  if (const char* why = adjoint_unsupported(h->cfg)) return fail(h, FG_ERR_CONFIG, why);
  if (nSteps < 1 || ckptEvery == 0 || !(dt > 0.) || !std::isfinite(dt))
    return fail(h, FG_ERR_CONFIG, "nSteps >= 1, ckptEvery != 0 and dt > 0 required");
  if (int r = ensure_adjoint(h)) return r;
  free_adjoint_store(h);
  const int n3 = h->M.n * h->M.n * h->M.n;
  const size_t cnt = (size_t)h->M.nElems * 5 * n3, bytes = cnt * sizeof(double);
  const bool binomial = ckptEvery < 0;
  h->adjDt = dt;
  if (binomial) {
    const int nSnap = -ckptEvery;
    h->adjSlots.assign(nSnap, nullptr);
    for (auto& p : h->adjSlots) if (int r = adj_alloc(h, p, cnt)) { free_adjoint_store(h); return r; }
    if (int r = adjoint_alloc_common(h, 1)) { free_adjoint_store(h); return r; }
    // the schedule's first right spine: where the reverse sweep's first snapshots go
    int l = 0, sFree = nSnap - 1;
    while (nSteps - l > 1 && sFree > 0) {
      l += revolve_split(nSteps - l, sFree);
      h->adjSpine.push_back({l, nSnap - sFree});
      --sFree;
    }
  } else {
    const int nCk = (nSteps + ckptEvery - 1) / ckptEvery;
    h->adjCkpt.assign(nCk, nullptr);
    for (auto& p : h->adjCkpt) if (int r = adj_alloc(h, p, cnt)) { free_adjoint_store(h); return r; }
    if (int r = adjoint_alloc_common(h, ckptEvery)) { free_adjoint_store(h); return r; }
  }
  h->launches = 0;
  if (h->d.srcPar) {  // the source's stage times in the reverse sweep start from the solve's start time
    if (!h->adjT0)
      if (int r = dalloc(h, h->adjT0, (size_t)h->d.nInst)) return r;
    CUDA_TRY(cudaMemcpyAsync(h->adjT0, h->dTime, sizeof(double) * h->d.nInst, cudaMemcpyDeviceToDevice, h->st));
  }
  size_t spineIdx = 0;
  for (int step = 0; step < nSteps; ++step) {
    if (binomial) {
      if (step == 0) CUDA_TRY(cudaMemcpyAsync(h->adjSlots[0], h->d.U, bytes, cudaMemcpyDeviceToDevice, h->st));
      if (spineIdx < h->adjSpine.size() && h->adjSpine[spineIdx].first == step) {
        CUDA_TRY(cudaMemcpyAsync(h->adjSlots[h->adjSpine[spineIdx].second], h->d.U, bytes, cudaMemcpyDeviceToDevice, h->st));
        ++spineIdx;
      }
    } else if (step % ckptEvery == 0) {
      CUDA_TRY(cudaMemcpyAsync(h->adjCkpt[step / ckptEvery], h->d.U, bytes, cudaMemcpyDeviceToDevice, h->st));
    }
    launch_step_setup(h, 1, dt, true);
    launch_lserk(h);
  }
  CUDA_TRY(cudaMemcpyAsync(h->adjUfinal, h->d.U, bytes, cudaMemcpyDeviceToDevice, h->st));
  CUDA_TRY(cudaGetLastError());
  if (int r = check_err(h)) { free_adjoint_store(h); return r; }
  h->adjSteps = nSteps;
  h->adjEvery = binomial ? 0 : ckptEvery;
  h->adjBinomial = binomial;
  return FG_OK;
}

int fg_adjoint_reverse(fg_handle* h, const double* UbarT, double* Ubar0, double* muScaleBar, double* forceBar) {
  if (!h || !h->haveMesh) return fail(h, FG_ERR_STATE, "no mesh");
  if (h->adjSteps < 1) return fail(h, FG_ERR_STATE, "no fg_adjoint_forward run to reverse");
  if (!UbarT) return fail(h, FG_ERR_CONFIG, "null cotangent");
  const int n3 = h->M.n * h->M.n * h->M.n;
  const long long cnt = (long long)h->M.nElems * 5 * n3;
  const size_t bytes = (size_t)cnt * sizeof(double);
  h->launches = 0;
  h->adjRecomputed = 0;
  CUDA_TRY(cudaMemcpyAsync(h->dStage, UbarT, bytes, cudaMemcpyHostToDevice, h->st));
  fortran_to_dev(h, h->dStage, h->adjUbar, 5);
  CUDA_TRY(cudaMemsetAsync(h->a.muElemb, 0, sizeof(double) * h->M.nElems, h->st));
  CUDA_TRY(cudaMemsetAsync(h->adjPartial, 0, sizeof(double) * h->M.nElems, h->st));
  CUDA_TRY(cudaMemsetAsync(h->adjFbar, 0, sizeof(double) * h->M.nElems * n3, h->st));
  // with the channel forcing, each step's bulk velocity is a function of its start state, and the energy
  // source of the body force (uniform and/or field) couples to it
  const bool bulkAdj = h->cfg.doTCSource != 0;
  AdjDev a = h->a;
  a.accumulate = 1;
  a.Ub = h->adjUbar;
  a.W = h->adjGbar;
  if (h->adjBinomial) {
    RevolveRun R{h, a, bulkAdj, {}, bytes};
    const int nSnap = (int)h->adjSlots.size();
    std::vector<bool> used(nSnap, false);
    used[0] = true;
    for (auto& sp : h->adjSpine) used[sp.second] = true;
    for (int i = nSnap - 1; i >= 1; --i) if (!used[i]) R.freeSlots.push_back(i);
    const auto spineCopy = h->adjSpine;
    const int e = revolve_reverse(R, 0, h->adjSteps, 0, nSnap - 1);
    h->adjSpine = spineCopy;  // the forward's snapshots stay valid for another reverse sweep only if untouched
    if (e) return e;
  } else {
    const int nCk = (int)h->adjCkpt.size();
    for (int seg = nCk - 1; seg >= 0; --seg) {
      const int s0 = seg * h->adjEvery, ns = std::min(h->adjEvery, h->adjSteps - s0);
      h->adjRecomputed += ns;
      if (int e = adjoint_reverse_segment(h, h->adjCkpt[seg], ns, a, bulkAdj, s0)) return e;
    }
  }
  CUDA_TRY(cudaGetLastError());
  // leave the handle at the final forward state
  CUDA_TRY(cudaMemcpyAsync(h->d.U, h->adjUfinal, bytes, cudaMemcpyDeviceToDevice, h->st));
  if (Ubar0) { if (int r = export_field(h, h->adjUbar, 5, 0, 5, Ubar0)) return r; }
  if (muScaleBar) CUDA_TRY(cudaMemcpyAsync(muScaleBar, h->a.muElemb, sizeof(double) * h->M.nElems, cudaMemcpyDeviceToHost, h->st));
  if (forceBar) { if (int r = export_field(h, h->adjFbar, 1, 0, 1, forceBar)) return r; }
  CUDA_TRY(cudaStreamSynchronize(h->st));
  // a binomial sweep overwrites snapshot slots it reused: another sweep needs a new forward
  if (h->adjBinomial) h->adjSteps = 0;
  return FG_OK;
}

long long fg_adjoint_recomputed_steps(const fg_handle* h) { return h ? h->adjRecomputed : -1; }

int fg_set_body_force_field(fg_handle* h, const double* F) {
  if (!h || !h->haveMesh) return fail(h, FG_ERR_STATE, "no mesh");
  const int n3 = h->M.n * h->M.n * h->M.n;
  const long long total = (long long)h->M.nElems * n3;
  if (!h->d.forceField) {
    if (!F) return FG_OK;
    if (int r = dalloc(h, h->d.forceField, (size_t)total)) return r;
    // the captured time loop holds the device pointers by value: capture it again with the field
    if (h->graph) { cudaGraphExecDestroy(h->graph); h->graph = nullptr; }
  }
  if (F) {
    CUDA_TRY(cudaMemcpyAsync(h->dStage, F, total * sizeof(double), cudaMemcpyHostToDevice, h->st));
    fortran_to_dev(h, h->dStage, h->d.forceField, 1);
  } else {
    k_fill<<<(unsigned)((total + 255) / 256), 256, 0, h->st>>>(h->d.forceField, 0., (int)total);
  }
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaStreamSynchronize(h->st));
  return FG_OK;
}

int fg_wall_shear(fg_handle* h, double* J, double* dJdU) {
  if (!h || !h->haveMesh) return fail(h, FG_ERR_STATE, "no mesh");
  if (h->M.nBCSides == 0) return fail(h, FG_ERR_MESH, "the mesh has no wall sides");
  if (dJdU) {
    if (const char* why = adjoint_unsupported(h->cfg)) return fail(h, FG_ERR_CONFIG, why);
    if (int r = ensure_adjoint(h)) return r;
  }
  const int n = h->M.n, n2 = n * n, n3 = n2 * n, nE = h->M.nElems, nS = h->M.nSides, nBC = h->M.nBCSides;
  h->launches = 0;
  const Dev& d = h->d;
  h->K.prep(d, h->B, h->st);
  h->K.lift(d, h->B, h->st);
  // per-point terms in the (otherwise unused) staging buffer: [0, nBC n2) terms, [nBC n2, 2 nBC n2) areas
  double* terms = h->dStage;
  double* areas = h->dStage + (size_t)nBC * n2;
  const int pts = nBC * n2;
  k_wall_shear<<<(pts + 127) / 128, 128, 0, h->st>>>(d, h->B, n2, terms, areas, 0., nullptr);
  std::vector<double> tv(pts), av(pts);
  CUDA_TRY(cudaMemcpyAsync(tv.data(), terms, sizeof(double) * pts, cudaMemcpyDeviceToHost, h->st));
  CUDA_TRY(cudaMemcpyAsync(av.data(), areas, sizeof(double) * pts, cudaMemcpyDeviceToHost, h->st));
  CUDA_TRY(cudaStreamSynchronize(h->st));
  double T = 0., A = 0.;
  for (int i = 0; i < pts; ++i) { T += tv[i]; A += av[i]; }
  if (J) *J = T / A;
  if (!dJdU) return FG_OK;
  AdjDev a = h->a;
  a.accumulate = 0;
  CUDA_TRY(cudaMemsetAsync(a.Ub, 0, sizeof(double) * nE * 5 * n3, h->st));
  CUDA_TRY(cudaMemsetAsync(a.gb, 0, sizeof(double) * nE * 12 * n3, h->st));
  CUDA_TRY(cudaMemsetAsync(a.gradMb, 0, sizeof(double) * nS * 12 * n2, h->st));
  CUDA_TRY(cudaMemsetAsync(a.gradSb, 0, sizeof(double) * nS * 12 * n2, h->st));
  CUDA_TRY(cudaMemsetAsync(a.faceMb, 0, sizeof(double) * nS * FS_NF * n2, h->st));
  CUDA_TRY(cudaMemsetAsync(a.faceSb, 0, sizeof(double) * nS * FS_NF * n2, h->st));
  CUDA_TRY(cudaMemsetAsync(a.muSideb, 0, sizeof(double) * nS * 2 * n2, h->st));
  CUDA_TRY(cudaMemsetAsync(a.muElemb, 0, sizeof(double) * nE, h->st));
  k_wall_shear<<<(pts + 127) / 128, 128, 0, h->st>>>(d, h->B, n2, terms, areas, 1.0 / A, a.gradMb);
  h->K.lift_adj(d, a, h->B, h->st);
  h->K.prep_adj(d, a, h->B, h->st);
  h->launches += 6;
  CUDA_TRY(cudaGetLastError());
  return export_field(h, a.Ub, 5, 0, 5, dJdU);
}

// mean time per launch of fn over reps launches on the handle's stream (ms), after one untimed launch
extern "C++" {
template <class F>
static double time_launches(fg_handle* h, int reps, F fn) {
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  fn();
  cudaEventRecord(a, h->st);
  for (int i = 0; i < reps; ++i) fn();
  cudaEventRecord(b, h->st);
  cudaEventSynchronize(b);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return ms / reps;
}
}  // extern "C++"

int fg_autotune(fg_handle* h, int reps, double* report) {
  if (!h || !h->haveMesh) return fail(h, FG_ERR_STATE, "no mesh");
  if (reps < 1) return fail(h, FG_ERR_CONFIG, "reps >= 1 required");
  double rep[9];
  for (double& v : rep) v = NAN;
  const Dev& d = h->d;
  KernelSet& K = h->K;
  const KernelSet& D = h->Kdef;
  // valid intermediates for every candidate (prep, lift and the side kernel only write intermediates, the
  // volume kernel in mode 0 only Ut: the state is not changed)
  D.prep(d, h->B, h->st);
  D.lift(d, h->B, h->st);
  D.flux_block(d, h->B, 128, h->st);
  CUDA_TRY(cudaGetLastError());
  K.prep = D.prep; K.lift = D.lift; K.vol_weak = D.vol_weak;
  if (D.altEPB > 0) {
    rep[0] = time_launches(h, reps, [&] { D.prep(d, h->B, h->st); });
    rep[1] = time_launches(h, reps, [&] { D.prep_alt(d, h->B, h->st); });
    rep[2] = time_launches(h, reps, [&] { D.lift(d, h->B, h->st); });
    rep[3] = time_launches(h, reps, [&] { D.lift_alt(d, h->B, h->st); });
    if (rep[1] < rep[0]) K.prep = D.prep_alt;
    if (rep[3] < rep[2]) K.lift = D.lift_alt;
    if (h->cfg.SplitDG < 0) {
      rep[4] = time_launches(h, reps, [&] { D.vol_weak(d, h->B, 0, 0., 0., h->st); });
      rep[5] = time_launches(h, reps, [&] { D.vol_weak_alt(d, h->B, 0, 0., 0., h->st); });
      if (rep[5] < rep[4]) K.vol_weak = D.vol_weak_alt;
    }
  }
  const int blocks[3] = {64, 128, 256};
  int best = 1;
  for (int i = 0; i < 3; ++i) {
    rep[6 + i] = time_launches(h, reps, [&] { D.flux_block(d, h->B, blocks[i], h->st); });
    if (rep[6 + i] < rep[6 + best]) best = i;
  }
  K.fluxBlock = blocks[best];
  CUDA_TRY(cudaGetLastError());
  // the captured time loop holds the kernels it was captured with
  if (h->graph) { cudaGraphExecDestroy(h->graph); h->graph = nullptr; }
  if (report) std::copy(rep, rep + 9, report);
  return FG_OK;
}

int fg_set_launch_shapes(fg_handle* h, int epbPrep, int epbLift, int epbVol, int fluxBlock) {
  if (!h) return FG_ERR_STATE;
  const KernelSet& D = h->Kdef;
  auto ok = [&](int e) { return e == D.defEPB || (D.altEPB > 0 && e == D.altEPB); };
  if (!ok(epbPrep) || !ok(epbLift) || !ok(epbVol) || (fluxBlock != 64 && fluxBlock != 128 && fluxBlock != 256))
    return fail(h, FG_ERR_CONFIG, "elements per CTA must be the default or the alternative of this N, the side block 64/128/256");
  h->K.prep = epbPrep == D.defEPB ? D.prep : D.prep_alt;
  h->K.lift = epbLift == D.defEPB ? D.lift : D.lift_alt;
  h->K.vol_weak = epbVol == D.defEPB ? D.vol_weak : D.vol_weak_alt;
  h->K.fluxBlock = fluxBlock;
  if (h->graph) { cudaGraphExecDestroy(h->graph); h->graph = nullptr; }
  return FG_OK;
}

int fg_autotune_choice(const fg_handle* h, int* out) {
  if (!h || !out) return FG_ERR_STATE;
  out[0] = h->K.prep == h->Kdef.prep ? h->Kdef.defEPB : h->Kdef.altEPB;
  out[1] = h->K.lift == h->Kdef.lift ? h->Kdef.defEPB : h->Kdef.altEPB;
  out[2] = h->K.vol_weak == h->Kdef.vol_weak ? h->Kdef.defEPB : h->Kdef.altEPB;
  out[3] = h->K.fluxBlock;
  return FG_OK;
}

int fg_calc_timestep(fg_handle* h, double* dt, int* errType) {
  if (!h || !h->haveMesh) return fail(h, FG_ERR_STATE, "no mesh");
  CUDA_TRY(cudaMemsetAsync(h->d.err, 0, sizeof(int), h->st));
  const int nI = h->d.nInst;
  k_fill<<<(nI + 127) / 128, 128, 0, h->st>>>(h->d.dt, INFINITY, nI);
  h->K.dt(h->d, h->B, h->dMetAdv, h->dMetVisc, h->cflEff, h->dflEff, nullptr, h->dWVol, h->st);
  CUDA_TRY(cudaGetLastError());
  std::vector<double> v(nI);
  int e = 0;
  CUDA_TRY(cudaMemcpyAsync(v.data(), h->d.dt, sizeof(double) * nI, cudaMemcpyDeviceToHost, h->st));
  CUDA_TRY(cudaMemcpyAsync(&e, h->d.err, sizeof(int), cudaMemcpyDeviceToHost, h->st));
  CUDA_TRY(cudaStreamSynchronize(h->st));
  if (dt) std::copy(v.begin(), v.end(), dt);
  if (errType) *errType = e;
  return FG_OK;
}

int fg_get_dt_elem(fg_handle* h, double* dtConv, double* dtVisc) {
  if (!h || !h->haveMesh) return fail(h, FG_ERR_STATE, "no mesh");
  const int nE = h->d.nElems;
  if (dtConv) CUDA_TRY(cudaMemcpyAsync(dtConv, h->d.dtElem, sizeof(double) * nE, cudaMemcpyDeviceToHost, h->st));
  if (dtVisc) CUDA_TRY(cudaMemcpyAsync(dtVisc, h->d.dtElem + nE, sizeof(double) * nE, cudaMemcpyDeviceToHost, h->st));
  CUDA_TRY(cudaStreamSynchronize(h->st));
  return FG_OK;
}

int fg_timestep_lserkw2(fg_handle* h, double* t, double dt) {
  if (!h || !h->haveMesh) return fail(h, FG_ERR_STATE, "no mesh");
  h->launches = 0;
  CUDA_TRY(cudaMemsetAsync(h->d.err, 0, sizeof(int), h->st));
  if (h->d.srcPar) {  // stage times from the caller's t
    k_fill<<<(h->d.nInst + 127) / 128, 128, 0, h->st>>>(h->d.tStep, t ? *t : 0., h->d.nInst);
    h->launches += 1;
  }
  launch_step_setup(h, 1, dt, false);
  launch_lserk(h);
  CUDA_TRY(cudaGetLastError());
  if (int r = check_err(h)) return r;
  if (t) *t += dt;
  return FG_OK;
}

// nSteps replays of the captured TimeDisc step (captured on first use) on the handle's stream; h->launches = launches
// per step
static int launch_steps_graph(fg_handle* h, int nSteps) {
  if (!h->graph) {
    cudaGraph_t g;
    const long long before = h->launches;
    CUDA_TRY(cudaStreamBeginCapture(h->st, cudaStreamCaptureModeThreadLocal));
    launch_step_setup(h, 0, 0., true);
    launch_lserk(h);
    CUDA_TRY(cudaStreamEndCapture(h->st, &g));
    CUDA_TRY(cudaGraphInstantiate(&h->graph, g, 0));
    cudaGraphDestroy(g);
    h->launchesPerStep = h->launches - before;
  }
  for (int s = 0; s < nSteps; ++s) CUDA_TRY(cudaGraphLaunch(h->graph, h->st));
  h->launches = h->launchesPerStep;
  return 0;
}

// elements per CTA of the volume kernel in use (chunks of its grid start at multiples of it)
static int vol_epb(const fg_handle* h) {
  if (h->cfg.SplitDG >= 0) return h->Kdef.defEPB;
  return h->K.vol_weak == h->Kdef.vol_weak ? h->Kdef.defEPB : h->Kdef.altEPB;
}

// The last LSERK stage of fg_run_to_host. Its volume kernel writes each element's final state, so it runs over
// element chunks: four of a fifth of the elements, then 15 % and the last 5 %. Once a chunk is done, the second
// stream converts its elements to the Fortran layout and copies them to Uhost while the later chunks run. The copy of
// a fifth of the state takes less time than the kernel's work on the next fifth down to about 45 GB/s of link rate
// (the link runs at 190 GB/s device-to-host when nothing else loads it, but far slower at times), so the copies keep
// pace and only the last chunk's is left when the kernel ends. With overintegration each chunk is followed by its
// elements' filter kernel (which writes their final state).
static int launch_last_stage_to_host(fg_handle* h, int mode, double rkA, double rkB, double* Uhost) {
  static const double ends[FG_OUT_CHUNKS] = {0.2, 0.4, 0.6, 0.8, 0.95, 1.0};
  const Dev& d = h->d;
  launch_rhs_front(h, d);
  h->launches += d.nFluxSides > 0 ? 3 : 2;  // prep, lifting, side kernel
  const int nE = d.nElems, epb = vol_epb(h);
  const long long per = 5LL * h->M.n * h->M.n * h->M.n;  // doubles per element
  int begin = 0;
  for (int c = 0; c < FG_OUT_CHUNKS && begin < nE; ++c) {
    // chunk ends at multiples of the elements per CTA (the last at nElems)
    const long long want = (long long)std::ceil(ends[c] * nE);
    const int end = c == FG_OUT_CHUNKS - 1 ? nE : (int)std::min<long long>(nE, (want + epb - 1) / epb * epb);
    if (end <= begin) continue;
    const int cnt = end - begin;
    Dev dc = d;
    dc.volBegin = begin;
    dc.volCount = cnt;
    // with overintegration the volume kernel writes J u_t and k_overint filters it and updates the registers
    const bool oi = h->ov.type > 0;
    if (h->cfg.SplitDG >= 0) h->K.vol_split(dc, h->B, oi ? 3 : mode, rkA, rkB, h->st);
    else h->K.vol_weak(dc, h->B, oi ? 3 : mode, rkA, rkB, h->st);
    if (oi) { h->K.overint(dc, h->ov, mode, rkA, rkB, 0, h->st); h->launches += 1; }
    CUDA_TRY(cudaEventRecord(h->evOut[c], h->st));
    CUDA_TRY(cudaStreamWaitEvent(h->stOut, h->evOut[c], 0));
    dev_to_fortran(h, d.U + begin * per, h->dStage + begin * per, 5, 0, 5, cnt, h->stOut);
    CUDA_TRY(cudaMemcpyAsync(Uhost + begin * per, h->dStage + begin * per, sizeof(double) * cnt * per, cudaMemcpyDeviceToHost, h->stOut));
    h->launches += 2;
    begin = end;
  }
  CUDA_TRY(cudaEventRecord(h->evOutDone, h->stOut));
  CUDA_TRY(cudaStreamWaitEvent(h->st, h->evOutDone, 0));
  return 0;
}

int fg_run(fg_handle* h, int nSteps, double* t) {
  if (!h || !h->haveMesh) return fail(h, FG_ERR_STATE, "no mesh");
  if (nSteps < 0) return fail(h, FG_ERR_CONFIG, "nSteps < 0");
  CUDA_TRY(cudaMemsetAsync(h->d.err, 0, sizeof(int), h->st));
  k_timedisc_release<<<(h->d.nInst + 127) / 128, 128, 0, h->st>>>(h->td, h->d.nInst);
  if (h->profiling) {  // direct launches with per-kernel events
    h->launches = 0;
    for (int s = 0; s < nSteps; ++s) {
      launch_step_setup(h, 0, 0., true);
      launch_lserk(h);
    }
    CUDA_TRY(cudaGetLastError());
    if (int r = check_err(h)) return r;
    if (t) CUDA_TRY(cudaMemcpy(t, h->dTime, sizeof(double) * h->d.nInst, cudaMemcpyDeviceToHost));
    if (nSteps > 0) h->launches /= nSteps;
    return FG_OK;
  }
  if (int r = launch_steps_graph(h, nSteps)) return r;
  const long long perStep = h->launches;
  CUDA_TRY(cudaGetLastError());
  if (int r = check_err(h)) return r;
  if (t) CUDA_TRY(cudaMemcpy(t, h->dTime, sizeof(double) * h->d.nInst, cudaMemcpyDeviceToHost));
  h->launches = perStep;
  return FG_OK;
}

int fg_run_to_host(fg_handle* h, int nSteps, double* t, double* U) {
  if (!h || !h->haveMesh) return fail(h, FG_ERR_STATE, "no mesh");
  if (!U) return fail(h, FG_ERR_CONFIG, "fg_run_to_host: null state pointer");
  if (nSteps < 0) return fail(h, FG_ERR_CONFIG, "nSteps < 0");
  // per-kernel profiling takes the plain sequence
  if (nSteps == 0 || h->profiling) {
    if (int r = fg_run(h, nSteps, t)) return r;
    return fg_get_state(h, U);
  }
  if (!h->stOut) {
    // the highest priority: at each chunk boundary the conversion of the finished chunk gets the SMs before the next
    // volume chunk (whose CTAs fill the register files while they run)
    int least = 0, greatest = 0;
    CUDA_TRY(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    CUDA_TRY(cudaStreamCreateWithPriority(&h->stOut, cudaStreamNonBlocking, greatest));
    for (auto& e : h->evOut) CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    CUDA_TRY(cudaEventCreateWithFlags(&h->evOutDone, cudaEventDisableTiming));
  }
  CUDA_TRY(cudaMemsetAsync(h->d.err, 0, sizeof(int), h->st));
  k_timedisc_release<<<(h->d.nInst + 127) / 128, 128, 0, h->st>>>(h->td, h->d.nInst);
  if (int r = launch_steps_graph(h, nSteps - 1)) return r;
  // the last step as direct launches: the sequence of the graph with the last stage's volume kernel in chunks
  h->launches = 0;
  launch_step_setup(h, 0, 0., true);
  for (int s = 1; s <= h->nStages; ++s) {
    if (h->d.srcPar) {
      k_stage_time<<<(h->d.nInst + 127) / 128, 128, 0, h->st>>>(h->d, h->RKc[s]);
      h->launches += 1;
    }
    const int mode = s == 1 ? 1 : 2;
    const double rkA = s == 1 ? 0. : h->RKA[s];
    if (s < h->nStages) launch_rhs(h, mode, rkA, h->RKb[s]);
    else if (int r = launch_last_stage_to_host(h, mode, rkA, h->RKb[s], U)) return r;
  }
  CUDA_TRY(cudaGetLastError());
  if (int r = check_err(h)) return r;
  if (t) CUDA_TRY(cudaMemcpy(t, h->dTime, sizeof(double) * h->d.nInst, cudaMemcpyDeviceToHost));
  return FG_OK;
}

int fg_set_time(fg_handle* h, const double* t) {
  if (!h || !h->haveMesh || !t) return fail(h, FG_ERR_STATE, "fg_set_time needs a mesh and times");
  CUDA_TRY(cudaMemcpyAsync(h->dTime, t, sizeof(double) * h->d.nInst, cudaMemcpyHostToDevice, h->st));
  k_timedisc_reset<<<(h->d.nInst + 127) / 128, 128, 0, h->st>>>(h->td, h->dTime, h->d.nInst);
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaStreamSynchronize(h->st));
  return FG_OK;
}

int fg_get_timedisc_state(fg_handle* h, int nInst, fg_timedisc_state* out) {
  if (!h || !h->haveMesh) return fail(h, FG_ERR_STATE, "no mesh");
  if (!out || nInst < 1 || nInst > h->d.nInst) return fail(h, FG_ERR_CONFIG, "fg_get_timedisc_state: nInst must be in 1..number of instances");
  const int n = nInst;
  std::vector<double> t(n), dt(n), dtMin(n);
  std::vector<long long> it(n);
  std::vector<int> fl(n), lim(n);
  CUDA_TRY(cudaStreamSynchronize(h->st));
  CUDA_TRY(cudaMemcpy(t.data(), h->dTime, sizeof(double) * n, cudaMemcpyDeviceToHost));
  CUDA_TRY(cudaMemcpy(dt.data(), h->td.dtPrev, sizeof(double) * n, cudaMemcpyDeviceToHost));
  CUDA_TRY(cudaMemcpy(dtMin.data(), h->td.dtMin, sizeof(double) * n, cudaMemcpyDeviceToHost));
  CUDA_TRY(cudaMemcpy(it.data(), h->td.iter, sizeof(long long) * n, cudaMemcpyDeviceToHost));
  CUDA_TRY(cudaMemcpy(fl.data(), h->td.flags, sizeof(int) * n, cudaMemcpyDeviceToHost));
  CUDA_TRY(cudaMemcpy(lim.data(), h->td.nDtLimited, sizeof(int) * n, cudaMemcpyDeviceToHost));
  for (int i = 0; i < n; ++i) {
    out[i].t = t[i];
    out[i].dt = dt[i];
    out[i].dtMin = dtMin[i];
    out[i].iter = it[i];
    out[i].atAnalyze = (fl[i] & TD_HOLD) ? 1 : 0;
    out[i].finished = (fl[i] & TD_DONE) ? 1 : 0;
    out[i].nDtLimited = lim[i];
  }
  return FG_OK;
}

int fg_get_gradients(fg_handle* h, double* gx, double* gy, double* gz) {
  if (!h || !h->haveMesh) return fail(h, FG_ERR_STATE, "no mesh");
  double* outs[3] = {gx, gy, gz};
  for (int dd = 0; dd < 3; ++dd)
    if (outs[dd])
      if (int r = export_field(h, h->d.grad, 12, 4 * dd, 4, outs[dd])) return r;
  return FG_OK;
}

int fg_get_stream(fg_handle* h, void** s) {
  if (!h || !s) return FG_ERR_STATE;
  *s = (void*)h->st;
  return FG_OK;
}

long long fg_launch_count(const fg_handle* h) { return h ? h->launches : 0; }

int fg_debug_array(fg_handle* h, const char* name, void* out, long long* count) {
  if (!h || !h->haveMesh || !name || !count) return fail(h, FG_ERR_STATE, "no mesh");
  const long long n3 = (long long)h->M.n * h->M.n * h->M.n, nE = h->d.nElems, nS = h->d.nSides;
  const std::string k = name;
  const void* src = nullptr;
  long long cnt = 0;
  size_t esz = sizeof(double);
  if (k == "U") { src = h->d.U; cnt = nE * 5 * n3; }
  else if (k == "Ut") { src = h->d.Ut; cnt = nE * 5 * n3; }
  else if (k == "prim") { src = h->d.prim; cnt = nE * VP_NF * n3; }
  else if (k == "grad") { src = h->d.grad; cnt = nE * 12 * n3; }
  else if (k == "metr") { src = h->d.metr; cnt = nE * 9 * n3; }
  else if (k == "sJ") { src = h->d.sJ; cnt = nE * n3; }
  else if (k == "metAdv") { src = h->dMetAdv; cnt = nE * 3 * n3; }
  else if (k == "metVisc") { src = h->dMetVisc; cnt = nE * 3 * n3; }
  else if (k == "mu0") { src = h->d.mu0; cnt = h->d.nInst; }
  else if (k == "dt") { src = h->d.dt; cnt = h->d.nInst; }
  else if (k == "dtElem") { src = h->d.dtElem; cnt = 2 * nE; }
  else if (k == "elemInst") { src = h->d.elemInst; cnt = nE; esz = sizeof(int); }
  else if (k == "elemSide") { src = h->d.elemSide; cnt = nE * 6; esz = sizeof(int); }
  else if (k == "sideElem") { src = h->d.sideElem; cnt = nS * 4; esz = sizeof(int); }
  else if (k == "geo") { src = h->d.geo; cnt = nS * FG_NF * (long long)h->M.n * h->M.n; }
  else if (k == "bcType") { src = h->d.bcType; cnt = h->d.nBCSides; esz = sizeof(int); }
  else if (k == "bcTwall") { src = h->d.bcTwall; cnt = h->d.nBCSides; }
  else return fail(h, FG_ERR_CONFIG, "unknown array " + k);
  if (cnt == 0) { *count = 0; return FG_OK; }
  *count = cnt;
  if (out) {
    CUDA_TRY(cudaStreamSynchronize(h->st));
    CUDA_TRY(cudaMemcpy(out, src, cnt * esz, cudaMemcpyDeviceToHost));
  }
  return FG_OK;
}

int fg_profile_enable(fg_handle* h, int on) {
  if (!h) return FG_ERR_STATE;
  h->profiling = on != 0;
  h->evUsed = 0;
  return FG_OK;
}

int fg_profile_read(fg_handle* h, double* ms, long long* counts) {
  if (!h) return FG_ERR_STATE;
  for (int c = 0; c < 6; ++c) { if (ms) ms[c] = 0.; if (counts) counts[c] = 0; }
  if (h->st) CUDA_TRY(cudaStreamSynchronize(h->st));
  for (size_t i = 0; i < h->evUsed; ++i) {
    float t = 0.f;
    CUDA_TRY(cudaEventElapsedTime(&t, h->evPool[i].first, h->evPool[i].second));
    const int c = h->evClass[i];
    if (ms) ms[c] += t;
    if (counts) counts[c] += 1;
  }
  h->evUsed = 0;
  return FG_OK;
}

int fg_probe_fp64_pipe(double* rates) {
  fg_handle* h = nullptr;
  if (!rates) return fail(h, FG_ERR_CONFIG, "fg_probe_fp64_pipe: rates is NULL");
  int dev = 0;
  cudaDeviceProp p;
  CUDA_TRY(cudaGetDevice(&dev));
  CUDA_TRY(cudaGetDeviceProperties(&p, dev));
  const int blocks = p.multiProcessorCount * 8, threads = 256, iters = 4096;
  double* out = nullptr;
  CUDA_TRY(cudaMalloc(&out, sizeof(double) * blocks * threads));
  cudaEvent_t a, b;
  cudaEventCreate(&a); cudaEventCreate(&b);
  void (*kern[4])(double*, double, double, int) = {k_probe_fp64<0>, k_probe_fp64<1>, k_probe_fp64<2>, k_probe_fp64<3>};
  for (int op = 0; op < 4; ++op) {
    kern[op]<<<blocks, threads>>>(out, 0.999, 1e-3, 256);
    float best = 1e30f;
    for (int r = 0; r < 3; ++r) {
      cudaEventRecord(a);
      kern[op]<<<blocks, threads>>>(out, 0.999, 1e-3, iters);
      cudaEventRecord(b);
      cudaEventSynchronize(b);
      float ms = 0.f;
      cudaEventElapsedTime(&ms, a, b);
      best = std::min(best, ms);
    }
    rates[op] = (double)blocks * threads * iters * 8 / (best * 1e-3) / 1e12;
  }
  cudaEventDestroy(a); cudaEventDestroy(b);
  cudaFree(out);
  CUDA_TRY(cudaGetLastError());
  return FG_OK;
}

int fg_probe_fp64_tensor(double* rates) {
  fg_handle* h = nullptr;
  if (!rates) return fail(h, FG_ERR_CONFIG, "fg_probe_fp64_tensor: rates is NULL");
  int dev = 0;
  cudaDeviceProp p;
  CUDA_TRY(cudaGetDevice(&dev));
  CUDA_TRY(cudaGetDeviceProperties(&p, dev));
  const int blocks = p.multiProcessorCount * 4, threads = 256, iters = 4096;
  double* out = nullptr;
  CUDA_TRY(cudaMalloc(&out, sizeof(double) * blocks * threads));
  cudaEvent_t a, b;
  cudaEventCreate(&a); cudaEventCreate(&b);
  auto best_ms = [&](void (*k)(double*, double, double, int)) {
    k<<<blocks, threads>>>(out, 0.999, 1e-3, 64);
    float best = 1e30f;
    for (int r = 0; r < 3; ++r) {
      cudaEventRecord(a);
      k<<<blocks, threads>>>(out, 0.999, 1e-3, iters);
      cudaEventRecord(b);
      cudaEventSynchronize(b);
      float ms = 0.f;
      cudaEventElapsedTime(&ms, a, b);
      best = std::min(best, ms);
    }
    return (double)best * 1e-3;
  };
  const double warps = (double)blocks * threads / 32.;
  const double t0 = best_ms(k_probe_dmma<2, false>);
  rates[0] = warps * iters * 2 * 512. / t0 / 1e12;
  const double t1 = best_ms(k_probe_dmma<2, true>);
  rates[1] = (warps * iters * 2 * 512. + (double)blocks * threads * iters * 8 * 2.) / t1 / 1e12;
  cudaEventDestroy(a); cudaEventDestroy(b);
  cudaFree(out);
  CUDA_TRY(cudaGetLastError());
  return FG_OK;
}

int fg_probe_fp64_lanes(double* ms) {
  fg_handle* h = nullptr;
  if (!ms) return fail(h, FG_ERR_CONFIG, "fg_probe_fp64_lanes: ms is NULL");
  int dev = 0;
  cudaDeviceProp p;
  CUDA_TRY(cudaGetDevice(&dev));
  CUDA_TRY(cudaGetDeviceProperties(&p, dev));
  const int blocks = p.multiProcessorCount * 8, threads = 256, iters = 4096;
  double* out = nullptr;
  CUDA_TRY(cudaMalloc(&out, sizeof(double) * blocks * threads));
  cudaEvent_t a, b;
  cudaEventCreate(&a); cudaEventCreate(&b);
  void (*kern[5])(double*, double, double, int) = {k_probe_fp64_lanes<32>, k_probe_fp64_lanes<16>, k_probe_fp64_lanes<8>,
                                                   k_probe_fp64_lanes<4>, k_probe_fp64_lanes<1>};
  for (int v = 0; v < 5; ++v) {
    kern[v]<<<blocks, threads>>>(out, 0.999, 1e-3, 64);
    float best = 1e30f;
    for (int r = 0; r < 3; ++r) {
      cudaEventRecord(a);
      kern[v]<<<blocks, threads>>>(out, 0.999, 1e-3, iters);
      cudaEventRecord(b);
      cudaEventSynchronize(b);
      float t = 0.f;
      cudaEventElapsedTime(&t, a, b);
      best = std::min(best, t);
    }
    ms[v] = best;
  }
  cudaEventDestroy(a); cudaEventDestroy(b);
  cudaFree(out);
  CUDA_TRY(cudaGetLastError());
  return FG_OK;
}

int fg_probe_fp64(double* tflops) {
  double r[4];
  if (int e = fg_probe_fp64_pipe(r)) return e;
  *tflops = 2. * r[0];
  return FG_OK;
}

}  // extern "C"
