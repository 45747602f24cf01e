// flexi_gb300 -- allocation-free evaluation of the DG time derivative.
//
// Some callers cannot allocate device memory: a host code whose device memory all comes from its own
// pool or caching allocator (and that forbids other allocations in its context), a time loop that must
// not allocate once it is running (real-time or memory-accounted runs, where an allocation can fail or
// fragment memory at the wrong moment), or a code that issues this call between the set-up and the
// capture of its own CUDA graphs. They pass the state, the output and the mesh in their own device
// memory; every intermediate array of the right-hand side (primitive variables, lifted gradients, face
// states, face gradients, numerical fluxes, per-instance constants) lives in one file-scope
// __device__ array of FG_NOALLOC_SCRATCH_BYTES, which every GPU that loads the library holds until exit.
//
// Rules of use:
//  * The first call on a device resolves the device address of the scratch array with
//    cudaGetSymbolAddress (host code may only use that address, never the array's name) and sets the
//    kernels' shared-memory limits; make that first call on each device before any stream capture. The
//    set-up is kept per device and per CUDA context: a call in a context created after it (e.g. after
//    cudaDeviceReset) does it again. Host threads making their first calls together are serialised on it.
//  * All calls share the array, which keeps the last call's contents; calls that overlap on the GPU
//    (on different streams, or from different host threads without ordering) race on it.
//  * Meshes whose intermediates need more than FG_NOALLOC_SCRATCH_BYTES are rejected with
//    FG_ERR_CONFIG before anything is launched.
//  * The call is asynchronous on the caller's stream and calls no cudaMalloc, cudaFree or other
//    allocating routine, on the device or on the host.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <mutex>

#include "../../include/flexi_gpu.h"
#include "fg_common.cuh"
#include "fg_launch.cuh"

namespace fg {

// records the reason of a failed call that has no handle, for fg_last_error(NULL)
void set_error_without_handle(const char* msg);

namespace {

int reject(int code, const char* msg) {
  set_error_without_handle(msg);
  return code;
}

static __device__ __align__(256) double g_noalloc_scratch[FG_NOALLOC_SCRATCH_BYTES / sizeof(double)];

constexpr int kMaxDevices = 64;
// per-device set-up: the scratch array's device address in the context it was resolved in
struct DeviceSetup {
  std::mutex m;
  unsigned long long ctxId = 0;
  double* scratch = nullptr;
};
DeviceSetup g_setup[kMaxDevices];

// unique id of the calling thread's current CUDA context (driver cuCtxGetCurrent / cuCtxGetId through the runtime's
// entry-point query, no link to the driver library); 0 when there is none or the query is unavailable
unsigned long long current_context_id() {
  using PfnGetCurrent = CUresult (*)(CUcontext*);
  using PfnGetId = CUresult (*)(CUcontext, unsigned long long*);
  static PfnGetCurrent getCurrent = nullptr;
  static PfnGetId getId = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      getCurrent = (PfnGetCurrent)p;
    p = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) == cudaSuccess && q == cudaDriverEntryPointSuccess)
      getId = (PfnGetId)p;
  });
  if (!getCurrent || !getId) return 0;
  CUcontext c = nullptr;
  unsigned long long id = 0;
  if (getCurrent(&c) != CUDA_SUCCESS || !c || getId(c, &id) != CUDA_SUCCESS) return 0;
  return id;
}

// per-call constants of the scratch: one instance, no body force
__global__ void k_noalloc_init(double* perInst, int* err, int* elemInst, int nE, int* sideInst, int nS, double mu0) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0) {
    perInst[0] = mu0;  // mu0
    perInst[1] = 0.;   // dt (unused: plain time derivative)
    perInst[2] = 0.;   // bulk velocity
    perInst[3] = 0.;   // dpdx
    *err = 0;
  }
  if (i < nE) elemInst[i] = 0;
  if (i < nS) sideInst[i] = 0;
}

// The operator's 1D basis, built in fixed-size stack arrays (no host heap): the same node iterations,
// barycentric weights and loop orders as the set-up code of the solver handle, so that both entry
// points launch the kernels with bit-identical constants.
void stack_legendre(int m, double x, double& L, double& dL) {  // scaled by sqrt(m+1/2)
  double l0 = 1., l1 = x, d1 = 1.;
  if (m == 0) { L = 1.; dL = 0.; }
  else if (m == 1) { L = x; dL = 1.; }
  else {
    for (int k = 2; k <= m; ++k) {
      const double lk = ((2. * k - 1.) * x * l1 - (k - 1.) * l0) / k;
      const double dk = k * l1 + x * d1;
      l0 = l1; l1 = lk; d1 = dk;
    }
    L = l1; dL = d1;
  }
  const double s = std::sqrt(m + 0.5);
  L *= s; dL *= s;
}
void stack_nodes(int N, bool gl, double* x, double* w) {
  for (int i = 0; i <= N; ++i) x[i] = w[i] = 0.;
  if (!gl) {
    if (N == 1) { x[0] = -std::sqrt(1. / 3.); x[1] = -x[0]; w[0] = w[1] = 1.; return; }
    const double h = 2. * std::atan(1.) / (N + 1);
    for (int i = 0; i <= (N + 1) / 2 - 1; ++i) {
      double xi = -std::cos(h * (2 * i + 1)), L, dL;
      for (int it = 0; it <= 10; ++it) {
        stack_legendre(N + 1, xi, L, dL);
        const double dx = -L / dL;
        xi += dx;
        if (std::fabs(dx) < 1e-15 * std::fabs(xi)) break;
      }
      stack_legendre(N + 1, xi, L, dL);
      x[i] = xi; x[N - i] = -xi;
      w[i] = w[N - i] = (2. * N + 3.) / ((1. - xi * xi) * dL * dL);
    }
    if (N % 2 == 0) { double L, dL; stack_legendre(N + 1, 0., L, dL); x[N / 2] = 0.; w[N / 2] = (2. * N + 3.) / (dL * dL); }
    return;
  }
  x[0] = -1.; x[N] = 1.; w[0] = w[N] = 2. / (N * (N + 1.));
  // inner Gauss-Lobatto nodes: roots of q = L_{N+1} - L_{N-1} (unscaled Legendre polynomials)
  auto qeval = [N](double xx, double& q, double& dq, double& LN) {
    double l0 = 1., l1 = xx;
    for (int k = 2; k <= N; ++k) { const double lk = ((2. * k - 1.) * xx * l1 - (k - 1.) * l0) / k; l0 = l1; l1 = lk; }
    LN = l1;
    q = (2. * N + 1.) / (N + 1.) * (xx * l1 - l0);
    dq = (2. * N + 1.) * l1;
  };
  for (int i = 1; i <= (N + 1) / 2 - 1; ++i) {
    double xi = -std::cos(M_PI / N * (i + 0.25) - 3. / (8. * N * M_PI) / (i + 0.25)), q, dq, LN;
    for (int it = 0; it <= 10; ++it) {
      qeval(xi, q, dq, LN);
      const double dx = -q / dq;
      xi += dx;
      if (std::fabs(dx) < 1e-15 * std::fabs(xi)) break;
    }
    qeval(xi, q, dq, LN);
    x[i] = xi; x[N - i] = -xi;
    w[i] = w[N - i] = w[0] / (LN * LN);
  }
  if (N % 2 == 0) { double q, dq, LN; qeval(0., q, dq, LN); x[N / 2] = 0.; w[N / 2] = w[0] / (LN * LN); }
}
void stack_lagrange_at(double xp, int n, const double* x, const double* wb, double* L) {
  const double eps = 2.220446049250313e-16;
  bool hit = false;
  for (int i = 0; i < n; ++i) {
    L[i] = 0.;
    const double a = xp, b = x[i];
    const bool eq = (a == 0. || b == 0.) ? std::fabs(a - b) <= 2. * eps
                                         : (std::fabs(a - b) <= eps * std::fabs(a) && std::fabs(a - b) <= eps * std::fabs(b));
    if (eq) { L[i] = 1.; hit = true; }
  }
  if (hit) return;
  double s = 0.;
  for (int i = 0; i < n; ++i) { L[i] = wb[i] / (xp - x[i]); s += L[i]; }
  for (int i = 0; i < n; ++i) L[i] /= s;
}
void stack_basis(const fg_config& c, Basis& B) {
  const int N = c.N, n = N + 1;
  const bool gl = c.NodeType == FG_NODE_GAUSS_LOBATTO;
  double x[FG_MAXN], w[FG_MAXN], wb[FG_MAXN], D[FG_MAXN][FG_MAXN], Lm[FG_MAXN], Lp[FG_MAXN];
  stack_nodes(N, gl, x, w);
  for (int i = 0; i < n; ++i) wb[i] = 1.;
  for (int i = 1; i < n; ++i)
    for (int j = 0; j < i; ++j) { wb[j] *= (x[j] - x[i]); wb[i] *= (x[i] - x[j]); }
  for (int i = 0; i < n; ++i) wb[i] = 1. / wb[i];
  for (int i = 0; i < n; ++i)
    for (int l = 0; l < n; ++l) D[i][l] = 0.;
  for (int l = 0; l < n; ++l)
    for (int i = 0; i < n; ++i)
      if (l != i) { D[i][l] = wb[l] / (wb[i] * (x[i] - x[l])); D[i][i] -= D[i][l]; }
  stack_lagrange_at(-1., n, x, wb, Lm);
  stack_lagrange_at(1., n, x, wb, Lp);
  B.N = N; B.n = n; B.nodeType = c.NodeType; B.splitDG = c.SplitDG;
  B.riemann = c.Riemann; B.riemannBC = c.RiemannBC < 0 ? c.Riemann : c.RiemannBC;
  B.lifting = c.Lifting; B.weakLifting = 0;
  for (int i = 0; i < n; ++i)
    for (int l = 0; l < n; ++l) {
      B.D_T[l * n + i] = D[i][l];
      B.Dhat_T[l * n + i] = -(1. / w[i]) * D[l][i] * w[l];
    }
  for (int l = 0; l < n; ++l)
    for (int i = 0; i < n; ++i) {
      double v;
      if (gl) {
        v = D[i][l];
        if (l == 0 && i == 0) v += 1.0 / (2.0 * w[0]);
        if (l == N && i == N) v -= 1.0 / (2.0 * w[N]);
      } else {
        v = D[i][l] - 0.5 * (1. / w[i]) * (-Lm[i] * Lm[l] + Lp[i] * Lp[l]);
      }
      B.DVS[l * n + i] = v;
    }
  for (int i = 0; i < n; ++i) { B.Lm[i] = Lm[i]; B.Lp[i] = Lp[i]; B.LhM[i] = Lm[i] / w[i]; B.LhP[i] = Lp[i] / w[i]; }
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
}

// kernel shared-memory limits of every kernel set, once per device (they are per-device settings)
void prepare_all_sets() {
  for (int n = 2; n <= 8; ++n)
    for (int gl = 0; gl < 2; ++gl) {
      KernelSet K = get_kernel_set(n, gl != 0);
      if (K.n != 0 && K.prepare) K.prepare();
    }
}

bool config_ok(const fg_config& c) {
  if (c.N < 1 || c.N > 7) return false;
  if (c.OverintegrationType != 0) return false;
  if (c.NodeType != FG_NODE_GAUSS && c.NodeType != FG_NODE_GAUSS_LOBATTO) return false;
  if (c.Riemann != FG_RIEMANN_LF && c.Riemann != FG_RIEMANN_HLLC && c.Riemann != FG_RIEMANN_ROE && c.Riemann != FG_RIEMANN_ROEENTROPYFIX) return false;
  if (c.Lifting != 1 && c.Lifting != 2) return false;
  if (c.doWeakLifting || c.doConservativeLifting || c.doTCSource) return false;
  if (c.SplitDG != FG_SPLIT_NONE && c.SplitDG != FG_SPLIT_SD && c.SplitDG != FG_SPLIT_PI) return false;
  if (c.SplitDG != FG_SPLIT_NONE && (c.NodeType != FG_NODE_GAUSS_LOBATTO || (c.N != 1 && c.N != 3 && c.N != 7))) return false;
  return true;
}

}  // namespace
}  // namespace fg

extern "C" int fg_time_derivative_noalloc(const fg_config* cfg, const fg_device_mesh* mesh, const double* U, double* Ut, void* stream) {
  using namespace fg;
  char msg[192];
  if (!cfg || !mesh) return reject(FG_ERR_CONFIG, "fg_time_derivative_noalloc: null config or mesh");
  if (!config_ok(*cfg))
    return reject(FG_ERR_CONFIG, "fg_time_derivative_noalloc: unsupported configuration (N 1..7, strong non-conservative "
                                 "lifting, no body force, no overintegration; split form only on Gauss-Lobatto nodes with N in {1,3,7})");
  const long long n = cfg->N + 1, n2 = n * n, n3 = n2 * n;
  const long long nE = mesh->nElems, nS = mesh->nSides;
  if (nE <= 0 || nS <= 0 || mesh->nBCSides < 0 || mesh->nBCSides > nS)
    return reject(FG_ERR_MESH, "fg_time_derivative_noalloc: invalid nElems/nSides/nBCSides");
  // scratch layout, in doubles, each block 32-double (256 B) aligned
  auto up = [](long long v) { return (v + 31) / 32 * 32; };
  const long long oPrim = 0;
  const long long oGrad = oPrim + up(nE * VP_NF * n3);
  const long long oFaceM = oGrad + up(nE * 12 * n3);
  const long long oFaceS = oFaceM + up(nS * FS_NF * n2);
  const long long oGradM = oFaceS + up(nS * FS_NF * n2);
  const long long oGradS = oGradM + up(nS * 12 * n2);
  const long long oFlux = oGradS + up(nS * 12 * n2);
  const long long oInst = oFlux + up(nS * 5 * n2);  // mu0, dt, bulk velocity, dpdx of the one instance
  const long long oErr = oInst + 32;                 // sticky error word (int)
  const long long oElemInst = oErr + 32;             // [nElems] ints
  const long long oSideInst = oElemInst + up((nE + 1) / 2);
  const long long need = oSideInst + up((nS + 1) / 2);
  if ((unsigned long long)need * sizeof(double) > FG_NOALLOC_SCRATCH_BYTES) {
    std::snprintf(msg, sizeof msg, "fg_time_derivative_noalloc: mesh needs %lld bytes of scratch, the maximum is %llu (nElems=%lld, nSides=%lld, N=%d)",
                  need * (long long)sizeof(double), (unsigned long long)FG_NOALLOC_SCRATCH_BYTES, nE, nS, cfg->N);
    return reject(FG_ERR_CONFIG, msg);
  }
  if (!mesh->elemSide || !mesh->sideElem || !mesh->metr || !mesh->sJ || !mesh->geo || !U || !Ut ||
      (mesh->nBCSides > 0 && (!mesh->bcType || !mesh->bcTwall)))
    return reject(FG_ERR_MESH, "fg_time_derivative_noalloc: null device pointer");

  // an error left by earlier work of the caller stays where it is, for the caller's own check
  const cudaError_t pending = cudaPeekAtLastError();
  if (pending != cudaSuccess) {
    std::snprintf(msg, sizeof msg, "fg_time_derivative_noalloc: a CUDA error from earlier work is pending (%s); nothing launched",
                  cudaGetErrorString(pending));
    return reject(FG_ERR_CUDA, msg);
  }
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    return reject(FG_ERR_CUDA, "fg_time_derivative_noalloc: no usable current device");
  KernelSet K = get_kernel_set((int)n, cfg->NodeType == FG_NODE_GAUSS_LOBATTO);
  if (K.n == 0 || (cfg->SplitDG >= 0 && !K.vol_split))
    return reject(FG_ERR_CONFIG, "fg_time_derivative_noalloc: no kernels for this N and node type");
  double* S = nullptr;
  {
    DeviceSetup& su = g_setup[dev];
    std::lock_guard<std::mutex> lock(su.m);
    const unsigned long long ctx = current_context_id();
    if (!su.scratch || ctx == 0 || ctx != su.ctxId) {
      // first call on this device in this context (the current one): device address of the scratch array, kernel limits
      void* p = nullptr;
      const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess || !p) {
        std::snprintf(msg, sizeof msg, "fg_time_derivative_noalloc: cudaGetSymbolAddress: %s", cudaGetErrorString(e));
        return reject(FG_ERR_CUDA, msg);
      }
      prepare_all_sets();
      const cudaError_t e2 = cudaGetLastError();
      if (e2 != cudaSuccess) {
        std::snprintf(msg, sizeof msg, "fg_time_derivative_noalloc: kernel set-up: %s", cudaGetErrorString(e2));
        return reject(FG_ERR_CUDA, msg);
      }
      su.scratch = (double*)p;
      su.ctxId = current_context_id();  // the look-up has made the primary context current if none was
    }
    S = su.scratch;
  }
  Basis B{};
  stack_basis(*cfg, B);
  Dev d{};
  d.nElems = (int)nE; d.nSides = (int)nS; d.nBCSides = mesh->nBCSides; d.nInst = 1;
  d.nFluxSides = (int)nS; d.nMortars = 0;
  d.U = const_cast<double*>(U);
  d.Ut = Ut;
  d.Ut_tmp = nullptr;
  d.prim = S + oPrim;
  d.grad = S + oGrad;
  d.metr = const_cast<double*>(mesh->metr);
  d.sJ = const_cast<double*>(mesh->sJ);
  d.elemSide = const_cast<int*>(mesh->elemSide);
  d.elemInst = (int*)(S + oElemInst);
  d.faceM = S + oFaceM;
  d.faceS = S + oFaceS;
  d.gradM = S + oGradM;
  d.gradS = S + oGradS;
  d.geo = const_cast<double*>(mesh->geo);
  d.flux = S + oFlux;
  d.sideElem = const_cast<int*>(mesh->sideElem);
  d.sideInst = (int*)(S + oSideInst);
  d.bcType = const_cast<int*>(mesh->bcType);
  d.bcTwall = const_cast<double*>(mesh->bcTwall);
  d.mu0 = S + oInst;
  d.dt = S + oInst + 1;
  d.bulkVel = S + oInst + 2;
  d.dpdx = S + oInst + 3;
  d.err = (int*)(S + oErr);
  d.dtElem = nullptr;
  cudaStream_t st = (cudaStream_t)stream;
  const long long nInit = nE > nS ? nE : nS;
  k_noalloc_init<<<(unsigned)((nInit + 255) / 256), 256, 0, st>>>(d.mu0, d.err, d.elemInst, (int)nE, d.sideInst, (int)nS, cfg->mu0);
  K.prep(d, B, st);
  K.lift(d, B, st);
  K.flux(d, B, st);
  if (cfg->SplitDG >= 0) K.vol_split(d, B, 0, 0., 0., st);
  else K.vol_weak(d, B, 0, 0., 0., st);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    std::snprintf(msg, sizeof msg, "fg_time_derivative_noalloc: launch: %s", cudaGetErrorString(e));
    return reject(FG_ERR_CUDA, msg);
  }
  return FG_OK;
}
