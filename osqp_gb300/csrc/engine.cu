// engine.cu -- OSQP public C API on the GB300 device engine.
//
// Implements include/osqp_gb300.h (the OSQP 1.0 public API,
// include/public/osqp_api_functions.h) for one QP per solver object:
//   osqp_setup           osqp_api.c:332-631
//   osqp_solve           osqp_api.c:636-1038
//   osqp_update_*        osqp_api.c:1184-1530
//   osqp_warm_start      osqp_api.c:1260-1304
// The ADMM loop itself runs on the device (gb_solver.cuh) in one launch:
// a single CTA for small problems, one thread-block cluster (16 CTAs, else
// 8, else one CTA) for medium ones, a cooperative persistent grid for large
// ones (OSQP_GB300_MODE = block | grid | clusterN overrides the choice).
// Every CUDA failure is returned as an OSQP error code; nothing calls exit().
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include <signal.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <mutex>
#include <thread>
#include <vector>

#include "osqp_gb300.h"
#include "osqp_gb300_ext.h"
#include "gb_solver.cuh"
#include "gb_structure.cuh"
#include "gb_launch.cuh"
#include "gb_engine.h"
#include "gb_kkt_plan.h"

using T = OSQPFloat;
using namespace gb;

#define GB_TRY(call)                                                              \
  do {                                                                            \
    cudaError_t _e = (call);                                                      \
    if (_e != cudaSuccess) {                                                      \
      fprintf(stderr, "osqp_gb300: %s failed: %s (%s:%d)\n", #call,               \
              cudaGetErrorString(_e), __FILE__, __LINE__);                        \
      return OSQP_ALGEBRA_LOAD_ERROR;                                             \
    }                                                                             \
  } while (0)

static double wall_s() {
  struct timespec t;
  clock_gettime(CLOCK_MONOTONIC, &t);
  return (double)t.tv_sec + 1e-9 * (double)t.tv_nsec;
}

// ---------------------------------------------------------------------------
// Kernels: setup / solve in block (one CTA) and grid (cooperative) form
// ---------------------------------------------------------------------------
constexpr int kBlockThreads = 1024;
constexpr int kGridThreads = 1024;

// Dynamic shared memory of the CTA form: the direct solver's workspace
// (gb_direct.cuh; empty for the indirect solver).
extern __shared__ __align__(16) unsigned char g_engine_dsm[];

template <typename TT>
__device__ __forceinline__ void attach_direct_ws(DevProblem<TT>& pr, KktPipe* kpipe = nullptr) {
  if (pr.kkt.nb > 0) {
    pr.kws = (TT*)g_engine_dsm;
    pr.kpipe = kpipe;
    if (!kpipe) pr.kkt.ring = 0;
    kkt_plan_on_chip(pr.kkt, (int*)(g_engine_dsm + kkt_ws_elems(pr.n, pr.m, pr.kkt.bmax, pr.kkt.segmax, pr.kkt.ring) * sizeof(TT)),
                     pr.n);
    __syncthreads();
  }
}

template <typename TT>
__global__ void __launch_bounds__(kBlockThreads, 1)
k_setup_block(DevProblem<TT> pr, DevSettings s, int kktL, int keep_state) {
  __shared__ GroupShared gsh;
  __shared__ SolverScalars ssc;
  if (threadIdx.x == 0) { gsh.parity = 0; gsh.flag = 0; if (keep_state) ssc = *pr.st; }
  attach_direct_ws(pr);
  __syncthreads();
  BlockGroup g{&gsh};
  Solver<TT> S{pr, s, &ssc, kktL};
  if (keep_state) S.prepare_data(g, true); else S.setup(g);
  __syncthreads();
  if (threadIdx.x == 0) *pr.st = ssc;
}

template <typename TT>
__global__ void __launch_bounds__(kBlockThreads, 1)
k_solve_block(DevProblem<TT> pr, DevSettings s, int kktL) {
  __shared__ GroupShared gsh;
  __shared__ SolverScalars ssc;
  __shared__ KktPipe kpipe;
  if (threadIdx.x == 0) { gsh.parity = 0; gsh.flag = 0; ssc = *pr.st; }
  kkt_pipe_init(&kpipe);
  attach_direct_ws(pr, &kpipe);
  __syncthreads();
  BlockGroup g{&gsh};
  Solver<TT> S{pr, s, &ssc, kktL};
  S.solve(g);
  __syncthreads();
  if (threadIdx.x == 0) *pr.st = ssc;
}

// Direct solver: refactor K for the rho (vector) in device memory after a
// host-driven change of rho or of the constraint types; records a
// non-positive pivot in the scalar state's kkt_fail.
template <typename TT>
__global__ void __launch_bounds__(kBlockThreads, 1)
k_refactor_block(DevProblem<TT> pr, DevSettings s, int kktL) {
  __shared__ GroupShared gsh;
  __shared__ SolverScalars ssc;
  if (threadIdx.x == 0) { gsh.parity = 0; gsh.flag = 0; ssc = *pr.st; }
  attach_direct_ws(pr);
  __syncthreads();
  BlockGroup g{&gsh};
  Solver<TT> S{pr, s, &ssc, kktL};
  S.update_precond(g);
  __syncthreads();
  if (threadIdx.x == 0) pr.st->kkt_fail = ssc.kkt_fail;
}

template <typename TT>
__global__ void __launch_bounds__(kGridThreads, 1)
k_setup_grid(DevProblem<TT> pr, DevSettings s, int kktL, int keep_state, GridSync gs) {
  __shared__ GroupShared gsh;
  __shared__ SolverScalars ssc;
  if (threadIdx.x == 0) { gsh.parity = 0; gsh.flag = 0; if (keep_state) ssc = *pr.st; }
  __syncthreads();
  GridGroup g{&gsh, gs};
  Solver<TT> S{pr, s, &ssc, kktL};
  bool ok = keep_state ? S.prepare_data(g, true) : S.setup(g);
  __syncthreads();
  if (ok && blockIdx.x == 0 && threadIdx.x == 0) *pr.st = ssc;
}

template <typename TT>
__global__ void __launch_bounds__(kGridThreads, 1)
k_solve_grid(DevProblem<TT> pr, DevSettings s, int kktL, GridSync gs) {
  __shared__ GroupShared gsh;
  __shared__ SolverScalars ssc;
  if (threadIdx.x == 0) { gsh.parity = 0; gsh.flag = 0; ssc = *pr.st; }
  __syncthreads();
  GridGroup g{&gsh, gs};
  Solver<TT> S{pr, s, &ssc, kktL};
  bool ok = S.solve(g);
  __syncthreads();
  if (ok && blockIdx.x == 0 && threadIdx.x == 0) *pr.st = ssc;
}

// One thread-block cluster solves the problem (medium sizes).
constexpr int kClusterThreads = 1024;
template <typename TT>
__global__ void __launch_bounds__(kClusterThreads, 1)
k_setup_cluster(DevProblem<TT> pr, DevSettings s, int kktL, int keep_state) {
  namespace cgr = cooperative_groups;
  __shared__ GroupShared gsh;
  __shared__ SolverScalars ssc;
  cgr::cluster_group cl = cgr::this_cluster();
  if (threadIdx.x == 0) { gsh.parity = 0; gsh.flag = 0; if (keep_state) ssc = *pr.st; }
  __syncthreads();
  ClusterGroup g{&gsh, cl.block_rank(), cl.num_blocks()};
  Solver<TT> S{pr, s, &ssc, kktL};
  if (keep_state) S.prepare_data(g, true); else S.setup(g);
  __syncthreads();
  if (g.rank == 0 && threadIdx.x == 0) *pr.st = ssc;
  cl.sync();
}
template <typename TT>
__global__ void __launch_bounds__(kClusterThreads, 1)
k_solve_cluster(DevProblem<TT> pr, DevSettings s, int kktL) {
  namespace cgr = cooperative_groups;
  __shared__ GroupShared gsh;
  __shared__ SolverScalars ssc;
  cgr::cluster_group cl = cgr::this_cluster();
  if (threadIdx.x == 0) { gsh.parity = 0; gsh.flag = 0; ssc = *pr.st; }
  __syncthreads();
  ClusterGroup g{&gsh, cl.block_rank(), cl.num_blocks()};
  Solver<TT> S{pr, s, &ssc, kktL};
  S.solve(g);
  __syncthreads();
  if (g.rank == 0 && threadIdx.x == 0) *pr.st = ssc;
  cl.sync();
}

// Small element-wise kernels used by the update / warm-start entry points.
template <typename TT>
__global__ void k_update_vec(DevProblem<TT> pr, int has_q, int has_l, int has_u, int scaling, double c,
                             int* bad) {
  const int n = pr.n, m = pr.m;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < (n > m ? n : m); i += gridDim.x * blockDim.x) {
    if (has_q && i < n) pr.q[i] = scaling ? (TT)((pr.q_in[i] * pr.D[i]) * (TT)c) : pr.q_in[i];
    if (i < m) {
      const TT l = has_l ? (scaling ? pr.l_in[i] * pr.E[i] : pr.l_in[i]) : pr.l[i];
      const TT u = has_u ? (scaling ? pr.u_in[i] * pr.E[i] : pr.u_in[i]) : pr.u[i];
      if (l > u) atomicExch(bad, 1);
      pr.t[i] = l;     // staged; committed by k_commit_bounds when valid
      pr.Et[i] = u;
    }
  }
}
template <typename TT>
__global__ void k_commit_bounds(DevProblem<TT> pr) {
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < pr.m; j += gridDim.x * blockDim.x) {
    pr.l[j] = pr.t[j];
    pr.u[j] = pr.Et[j];
  }
}
// rho vector (optional) and Jacobi preconditioner after a rho / bounds change
template <typename TT>
__global__ void k_rho_vec(DevProblem<TT> pr, double rho, double infty, int recompute_types, int* changed) {
  const double infval = infty * kMinScaling;
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < pr.m; j += gridDim.x * blockDim.x) {
    int t = pr.ctype[j];
    if (recompute_types) {
      const double l = pr.l[j], u = pr.u[j];
      int nt;
      if (l < -infval && u > infval) nt = -1;
      else if (u - l < kRhoTol) nt = 1;
      else nt = 0;
      if (nt != t) atomicExch(changed, 1);
      t = nt;
      pr.ctype[j] = t;
    }
    const double rv = t < 0 ? kRhoMin : (t == 0 ? rho : kRhoEqOverIneq * rho);
    pr.rho_vec[j] = (TT)rv;
    pr.rho_inv_vec[j] = TT(1) / (TT)rv;
  }
}
template <typename TT>
__global__ void k_precond(DevProblem<TT> pr, double sigma, double rho, int rho_is_vec, int precond) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < pr.n; i += gridDim.x * blockDim.x) {
    if (precond == 0) { pr.Minv[i] = TT(1); continue; }
    TT d = TT(0);
    for (int k = pr.At.rowptr[i]; k < pr.At.rowptr[i + 1]; k++) {
      const TT a = pr.At.val[k];
      d += rho_is_vec ? a * a * pr.rho_vec[pr.At.col[k]] : a * a;
    }
    if (!rho_is_vec) d *= (TT)rho;
    pr.Minv[i] = TT(1) / ((TT)sigma + pr.P.val[pr.Pdiag[i]] + d);
  }
}
template <typename TT>
__global__ void k_warm_start(DevProblem<TT> pr, const TT* xin, const TT* yin, int scaling, double c) {
  const int n = pr.n, m = pr.m;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < (n > m ? n : m); i += gridDim.x * blockDim.x) {
    if (xin && i < n) pr.x[i] = scaling ? xin[i] * pr.Dinv[i] : xin[i];
    if (yin && i < m) pr.y[i] = scaling ? (TT)((yin[i] * pr.Einv[i]) * (TT)c) : yin[i];
  }
}
template <typename TT>
__global__ void k_z_from_x(DevProblem<TT> pr) {
  // z = A x and the PCG iterate follows x (osqp_api.c:1284-1290)
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < pr.m; j += gridDim.x * blockDim.x) {
    TT a = TT(0);
    for (int k = pr.A.rowptr[j]; k < pr.A.rowptr[j + 1]; k++) a += pr.A.val[k] * pr.x[pr.A.col[k]];
    pr.z[j] = a;
  }
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < pr.n; i += gridDim.x * blockDim.x) pr.xp[i] = pr.x[i];
}
template <typename TT>
__global__ void k_cold_start(DevProblem<TT> pr) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < pr.n; i += gridDim.x * blockDim.x) { pr.x[i] = TT(0); pr.xp[i] = TT(0); }
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < pr.m; j += gridDim.x * blockDim.x) { pr.z[j] = TT(0); pr.y[j] = TT(0); }
}
template <typename TT>
__global__ void k_scatter_vals(TT* dst, const TT* src, const int* idx, int cnt) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < cnt; k += gridDim.x * blockDim.x)
    dst[idx ? idx[k] : k] = src[k];
}

// ---------------------------------------------------------------------------
// Workspace
// ---------------------------------------------------------------------------
struct OSQPWorkspace_ {
  int n, m, nnzT, nnzA, nnzPf;
  int device;
  cudaStream_t stream;
  char* arena;            // one device allocation for the whole problem
  size_t arena_bytes;
  DevProblem<T> pr;
  DevSettings ds;
  int kktL;
  int use_grid;
  int grid_blocks;
  int cluster;            // >1: one thread-block cluster of this many CTAs
  unsigned int* bar;      // [count, gen]
  int* err;
  int* flag;              // scratch flag for update checks
  double* partials;
  T* h_x;                 // pinned staging for solution transfers
  SolverScalars* h_st;    // pinned copy of the device scalars
  int first_run, clear_update_time;
  cudaEvent_t ev0, ev1;
  float last_kernel_ms;
  void* polish;           // polish workspace (gb_polish.cu)
  size_t kdsm;                 // direct solver: dynamic shared memory of the CTA-form kernels
  cudaStream_t cancel_stream;  // interrupt requests: a write of pr.st->cancel beside the running solve
  int* h_one;                  // pinned staging of the generation that write copies
  std::atomic<int> gen{0};     // interrupt generation: one per osqp_solve
};

// Interrupt of a running solve (osqp_api.c:728-737, interrupt_unix.c): the
// solve kernel reads pr.st->cancel once per ADMM iteration (it rides on the
// iteration's first reduction, so every CTA stops at the same iteration) and
// ends with status OSQP_SIGINT.  The request is a copy into that word on a
// stream of its own, which runs while the solve kernel does.
static int request_cancel(OSQPWorkspace* w) {
  if (cudaSetDevice(w->device) != cudaSuccess) return OSQP_ALGEBRA_LOAD_ERROR;
  // the request names the generation of the solve running (or starting) now;
  // a later solve has a newer generation, so a stale request never stops it
  *w->h_one = w->gen.load();
  if (cudaMemcpyAsync(&w->pr.st->cancel, w->h_one, sizeof(int), cudaMemcpyHostToDevice, w->cancel_stream) != cudaSuccess ||
      cudaStreamSynchronize(w->cancel_stream) != cudaSuccess)
    return OSQP_ALGEBRA_LOAD_ERROR;
  return 0;
}

// Ctrl-C during osqp_solve, as the reference's listener: a SIGINT handler is
// installed while solves run and the previous one restored after.  Solves
// running at the same time (other threads) share one installation, counted,
// so the caller's handler comes back when the last of them returns.  The
// handler only bumps a counter; each thread waiting for a solve turns a
// change of it into an interrupt request for its own solve.
static volatile sig_atomic_t g_sigint = 0;
static void on_sigint(int) { g_sigint = g_sigint + 1; }
static std::mutex g_listener_mu;
static int g_listeners = 0;
static struct sigaction g_saved_act;
static bool g_installed = false;
struct InterruptListener {
  sig_atomic_t seen;
  InterruptListener() {
    std::lock_guard<std::mutex> lk(g_listener_mu);
    if (g_listeners++ == 0) {
      struct sigaction act;
      memset(&act, 0, sizeof(act));
      act.sa_handler = on_sigint;
      sigemptyset(&act.sa_mask);
      g_installed = sigaction(SIGINT, &act, &g_saved_act) == 0;
    }
    seen = g_sigint;
  }
  bool fired() const { return g_sigint != seen; }
  ~InterruptListener() {
    std::lock_guard<std::mutex> lk(g_listener_mu);
    if (--g_listeners == 0 && g_installed) {
      sigaction(SIGINT, &g_saved_act, nullptr);
      g_installed = false;
    }
  }
};

// Block-Jacobi storage, allocated when cg_precond = 2 is first asked for
// (set-up or a settings update) and kept until cleanup.
static int ensure_block_precond(OSQPWorkspace* w) {
  if (w->pr.Binv || w->ds.cg_precond != kPrecondBlockDiagonal) return 0;
  T* p = nullptr;
  if (cudaMalloc((void**)&p, sizeof(T) * block_precond_elems(w->n)) != cudaSuccess) return OSQP_MEM_ALLOC_ERROR;
  w->pr.Binv = p;
  return 0;
}

// FP64 polish stage (polish.cu); returns >0 on a hard failure.
int gb_polish_run(OSQPSolver* solver);
void gb_polish_free(void* p);

static int g_sm_count[64];

static int device_sms(int dev) {
  if (dev < 0 || dev >= 64) return 148;
  if (!g_sm_count[dev]) {
    int v = 0;
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    g_sm_count[dev] = v > 0 ? v : 148;
  }
  return g_sm_count[dev];
}

static DevSettings make_dev_settings(const OSQPSettings* st) {
  DevSettings d;
  d.rho = st->rho; d.sigma = st->sigma; d.alpha = st->alpha;
  d.eps_abs = st->eps_abs; d.eps_rel = st->eps_rel;
  d.eps_prim_inf = st->eps_prim_inf; d.eps_dual_inf = st->eps_dual_inf;
  d.cg_tol_fraction = st->cg_tol_fraction;
  d.adaptive_rho_tolerance = st->adaptive_rho_tolerance;
  d.adaptive_rho_fraction = st->adaptive_rho_fraction;
  d.time_limit = st->time_limit;
  d.infty = (double)OSQP_INFTY;
  d.zero_deadzone = OSQP_ZERO_DEADZONE;
  d.scaling = st->scaling; d.rho_is_vec = st->rho_is_vec; d.max_iter = st->max_iter;
  d.check_termination = st->check_termination;
  d.adaptive_rho = st->adaptive_rho; d.adaptive_rho_interval = st->adaptive_rho_interval;
  d.cg_max_iter = st->cg_max_iter; d.cg_tol_reduction = st->cg_tol_reduction;
  d.cg_precond = (int)st->cg_precond;
  d.scaled_termination = st->scaled_termination; d.check_dualgap = st->check_dualgap;
  d.warm_starting = st->warm_starting;
  d.cancel_gen = 0;
  d.profile = 0;
  return d;
}

// ---------------------------------------------------------------------------
// Status strings (src/auxil.c:785-799) and error strings (src/error.c)
// ---------------------------------------------------------------------------
const char* OSQP_STATUS_MESSAGE[] = {
  "", "solved", "solved inaccurate", "primal infeasible", "primal infeasible inaccurate",
  "dual infeasible", "dual infeasible inaccurate", "maximum iterations reached",
  "run time limit reached", "problem non convex", "interrupted", "unsolved"};
const char* OSQP_ERROR_MESSAGE[] = {
  "", "Problem data validation.", "Solver settings validation.",
  "Linear system solver initialization.", "KKT matrix factorization.", "Memory allocation.",
  "Solver workspace not initialized.", "Algebra library loading.", "File open.",
  "Invalid defines for codegen.", "Vector/matrix not initialized.", "Function not implemented."};

static void set_status(OSQPInfo* info, int s) {
  info->status_val = s;
  strncpy(info->status, OSQP_STATUS_MESSAGE[s], 31);
  info->status[31] = 0;
}

extern "C" {

OSQPInt osqp_capabilities(void) {
  return OSQP_CAPABILITY_DIRECT_SOLVER | OSQP_CAPABILITY_INDIRECT_SOLVER | OSQP_CAPABILITY_UPDATE_MATRICES;
}
const char* osqp_version(void) { return "1.0.0-gb300"; }
const char* osqp_error_message(OSQPInt e) {
  if (e < 0 || e >= OSQP_LAST_ERROR_PLACE) return "Unrecognised error code.";
  return OSQP_ERROR_MESSAGE[e];
}
void osqp_get_dimensions(OSQPSolver* s, OSQPInt* m, OSQPInt* n) {
  if (!s || !s->work) { *m = -1; *n = -1; return; }
  *m = s->work->m; *n = s->work->n;
}

void osqp_set_default_settings(OSQPSettings* st) {
  if (!st) return;
  st->device = 0;
  st->linsys_solver = OSQP_INDIRECT_SOLVER;
  st->allocate_solution = 1;
  st->verbose = OSQP_VERBOSE;
  st->profiler_level = 0;
  st->warm_starting = OSQP_WARM_STARTING;
  st->scaling = OSQP_SCALING;
  st->polishing = OSQP_POLISHING;
  st->rho = (OSQPFloat)OSQP_RHO;
  st->rho_is_vec = OSQP_RHO_IS_VEC;
  st->sigma = (OSQPFloat)OSQP_SIGMA;
  st->alpha = (OSQPFloat)OSQP_ALPHA;
  st->cg_max_iter = OSQP_CG_MAX_ITER;
  st->cg_tol_reduction = OSQP_CG_TOL_REDUCTION;
  st->cg_tol_fraction = (OSQPFloat)OSQP_CG_TOL_FRACTION;
  st->cg_precond = OSQP_DIAGONAL_PRECONDITIONER;
  st->adaptive_rho = OSQP_ADAPTIVE_RHO_UPDATE_DEFAULT;
  st->adaptive_rho_interval = OSQP_ADAPTIVE_RHO_INTERVAL;
  st->adaptive_rho_fraction = (OSQPFloat)OSQP_ADAPTIVE_RHO_FRACTION;
  st->adaptive_rho_tolerance = (OSQPFloat)OSQP_ADAPTIVE_RHO_TOLERANCE;
  st->max_iter = OSQP_MAX_ITER;
  st->eps_abs = (OSQPFloat)OSQP_EPS_ABS;
  st->eps_rel = (OSQPFloat)OSQP_EPS_REL;
  st->eps_prim_inf = (OSQPFloat)OSQP_EPS_PRIM_INF;
  st->eps_dual_inf = (OSQPFloat)OSQP_EPS_DUAL_INF;
  st->scaled_termination = OSQP_SCALED_TERMINATION;
  st->check_termination = OSQP_CHECK_TERMINATION;
  st->check_dualgap = OSQP_CHECK_DUALGAP;
  st->time_limit = (OSQPFloat)OSQP_TIME_LIMIT;
  st->delta = (OSQPFloat)OSQP_DELTA;
  st->polish_refine_iter = OSQP_POLISH_REFINE_ITER;
}

OSQPSettings* OSQPSettings_new(void) {
  OSQPSettings* s = (OSQPSettings*)calloc(1, sizeof(OSQPSettings));
  if (s) osqp_set_default_settings(s);
  return s;
}
void OSQPSettings_free(OSQPSettings* s) { free(s); }
OSQPCodegenDefines* OSQPCodegenDefines_new(void) {
  OSQPCodegenDefines* d = (OSQPCodegenDefines*)calloc(1, sizeof(OSQPCodegenDefines));
  if (d) osqp_set_default_codegen_defines(d);
  return d;
}
void OSQPCodegenDefines_free(OSQPCodegenDefines* d) { free(d); }
void osqp_set_default_codegen_defines(OSQPCodegenDefines* d) {
  if (!d) return;
  d->embedded_mode = 1; d->float_type = 0; d->printing_enable = 0;
  d->profiling_enable = 0; d->interrupt_enable = 0; d->derivatives_enable = 0;
}
OSQPInt osqp_codegen(OSQPSolver*, const char*, const char*, OSQPCodegenDefines*) { return OSQP_FUNC_NOT_IMPLEMENTED; }
OSQPInt osqp_adjoint_derivative_compute(OSQPSolver*, OSQPFloat*, OSQPFloat*) { return OSQP_FUNC_NOT_IMPLEMENTED; }
OSQPInt osqp_adjoint_derivative_get_mat(OSQPSolver*, OSQPCscMatrix*, OSQPCscMatrix*) { return OSQP_FUNC_NOT_IMPLEMENTED; }
OSQPInt osqp_adjoint_derivative_get_vec(OSQPSolver*, OSQPFloat*, OSQPFloat*, OSQPFloat*) { return OSQP_FUNC_NOT_IMPLEMENTED; }

// CSC helpers (osqp_api_functions.h:36-120): host-side containers.
OSQPCscMatrix* OSQPCscMatrix_new(OSQPInt m, OSQPInt n, OSQPInt nzmax, OSQPFloat* x, OSQPInt* i, OSQPInt* p) {
  OSQPCscMatrix* M = (OSQPCscMatrix*)calloc(1, sizeof(OSQPCscMatrix));
  if (!M) return NULL;
  OSQPCscMatrix_set_data(M, m, n, nzmax, x, i, p);
  return M;
}
void OSQPCscMatrix_set_data(OSQPCscMatrix* M, OSQPInt m, OSQPInt n, OSQPInt nzmax, OSQPFloat* x, OSQPInt* i, OSQPInt* p) {
  M->m = m; M->n = n; M->nzmax = nzmax; M->nz = -1; M->x = x; M->i = i; M->p = p; M->owned = 0;
}
// An owned m x n matrix with room for nnz entries; a matrix without entries
// has NULL i and x (src/osqp_api.c:122-145).
static OSQPCscMatrix* csc_owned(OSQPInt m, OSQPInt n, OSQPInt nnz) {
  OSQPCscMatrix* M = (OSQPCscMatrix*)calloc(1, sizeof(OSQPCscMatrix));
  if (!M) return NULL;
  M->m = m; M->n = n; M->nzmax = nnz; M->nz = -1; M->owned = 1;
  M->p = (OSQPInt*)calloc((size_t)n + 1, sizeof(OSQPInt));
  if (nnz > 0) {
    M->i = (OSQPInt*)calloc((size_t)nnz, sizeof(OSQPInt));
    M->x = (OSQPFloat*)calloc((size_t)nnz, sizeof(OSQPFloat));
  }
  if (!M->p || (nnz > 0 && (!M->i || !M->x))) { OSQPCscMatrix_free(M); return NULL; }
  return M;
}
void OSQPCscMatrix_free(OSQPCscMatrix* M) {
  if (!M) return;
  if (M->owned) { free(M->p); free(M->i); free(M->x); }
  free(M);
}
OSQPCscMatrix* OSQPCscMatrix_zeros(OSQPInt m, OSQPInt n) { return csc_owned(m, n, 0); }
OSQPCscMatrix* OSQPCscMatrix_diag_vec(OSQPInt m, OSQPInt n, OSQPFloat* vals) {
  OSQPInt d = m < n ? m : n;
  OSQPCscMatrix* M = csc_owned(m, n, d);
  if (!M) return NULL;
  for (OSQPInt j = 0; j < n; j++) M->p[j + 1] = M->p[j] + (j < d ? 1 : 0);
  for (OSQPInt j = 0; j < d; j++) { M->i[j] = j; M->x[j] = vals[j]; }
  return M;
}
OSQPCscMatrix* OSQPCscMatrix_diag_scalar(OSQPInt m, OSQPInt n, OSQPFloat sc) {
  OSQPInt d = m < n ? m : n;
  std::vector<OSQPFloat> v((size_t)(d > 0 ? d : 1), sc);
  return OSQPCscMatrix_diag_vec(m, n, v.data());
}
OSQPCscMatrix* OSQPCscMatrix_identity(OSQPInt m) { return OSQPCscMatrix_diag_scalar(m, m, (OSQPFloat)1.0); }

// --- validation (src/auxil.c:950-1223) -------------------------------------
static int validate_settings(const OSQPSettings* s, int from_setup) {
  if (!s) return 1;
  if (from_setup && s->linsys_solver != OSQP_INDIRECT_SOLVER && s->linsys_solver != OSQP_DIRECT_SOLVER) return 1;
  if (from_setup && s->allocate_solution != 0 && s->allocate_solution != 1) return 1;
  if (s->verbose != 0 && s->verbose != 1) return 1;
  if (s->profiler_level < 0 || s->profiler_level > 2) return 1;
  if (s->warm_starting != 0 && s->warm_starting != 1) return 1;
  if (from_setup && s->scaling < 0) return 1;
  if (s->polishing != 0 && s->polishing != 1) return 1;
  if (from_setup && s->rho <= 0.0) return 1;
  if (from_setup && s->rho_is_vec != 0 && s->rho_is_vec != 1) return 1;
  if (from_setup && s->sigma <= 0.0) return 1;
  if (s->alpha <= 0.0 || s->alpha >= 2.0) return 1;
  if (s->cg_max_iter <= 0 || s->cg_tol_reduction <= 0) return 1;
  if (s->cg_tol_fraction <= 0.0 || s->cg_tol_fraction >= 1.0) return 1;
  if ((from_setup && s->adaptive_rho < 0) || s->adaptive_rho >= _OSQP_ADAPTIVE_RHO_UPDATE_LAST_VALUE) return 1;
  if (from_setup && s->adaptive_rho == OSQP_ADAPTIVE_RHO_UPDATE_TIME) return 1;  // needs host timers per iteration
  if (from_setup && s->adaptive_rho_interval < 0) return 1;
  if (from_setup && s->adaptive_rho_fraction <= 0) return 1;
  if (from_setup && s->adaptive_rho_tolerance < 1.0) return 1;
  if (s->max_iter <= 0 || s->eps_abs < 0.0 || s->eps_rel < 0.0) return 1;
  if (s->eps_rel == 0.0 && s->eps_abs == 0.0) return 1;
  if (s->eps_prim_inf <= 0.0 || s->eps_dual_inf <= 0.0) return 1;
  if (s->scaled_termination != 0 && s->scaled_termination != 1) return 1;
  if (s->check_termination < 0) return 1;
  if (s->check_dualgap != 0 && s->check_dualgap != 1) return 1;
  if (s->time_limit <= 0.0 || s->delta <= 0.0 || s->polish_refine_iter < 0) return 1;
  return 0;
}

}  // extern "C"

// Copies p (n+1) and i (nnz) of a CSC matrix that may live on host or device.
static int fetch_pattern(const OSQPCscMatrix* M, std::vector<OSQPInt>& p, std::vector<OSQPInt>& i) {
  p.resize((size_t)M->n + 1);
  if (cudaMemcpy(p.data(), M->p, sizeof(OSQPInt) * ((size_t)M->n + 1), cudaMemcpyDefault) != cudaSuccess) return 1;
  const OSQPInt nnz = p[M->n];
  i.resize((size_t)(nnz > 0 ? nnz : 1));
  if (nnz && cudaMemcpy(i.data(), M->i, sizeof(OSQPInt) * nnz, cudaMemcpyDefault) != cudaSuccess) return 1;
  return 0;
}

static int validate_data(const OSQPCscMatrix* P, const OSQPFloat* q, const OSQPCscMatrix* A,
                         const OSQPFloat* l, const OSQPFloat* u, OSQPInt m, OSQPInt n,
                         const std::vector<OSQPInt>& Pp, const std::vector<OSQPInt>& Pi) {
  if (!P || !A || !q) return 1;
  if (n <= 0 || m < 0) return 1;
  if (P->m != n || P->m != P->n) return 1;
  for (OSQPInt j = 0; j < n; j++)
    for (OSQPInt k = Pp[j]; k < Pp[j + 1]; k++)
      if (Pi[k] > j) return 1;
  if (A->m != m || A->n != n) return 1;
  if (m) {
    std::vector<OSQPFloat> hl(m), hu(m);
    if (cudaMemcpy(hl.data(), l, sizeof(OSQPFloat) * m, cudaMemcpyDefault) != cudaSuccess) return 1;
    if (cudaMemcpy(hu.data(), u, sizeof(OSQPFloat) * m, cudaMemcpyDefault) != cudaSuccess) return 1;
    for (OSQPInt j = 0; j < m; j++) if (hl[j] > hu[j]) return 1;
  }
  return 0;
}

// ---------------------------------------------------------------------------
// Device arena layout
// ---------------------------------------------------------------------------
struct ArenaPlan {
  size_t off = 0;
  template <typename U>
  size_t take(size_t count) {
    off = (off + 255) & ~size_t(255);
    size_t o = off;
    off += sizeof(U) * (count > 0 ? count : 1);
    return o;
  }
};

static int launch_setup(OSQPWorkspace* w, int keep_state);

static void free_workspace(OSQPWorkspace* w) {
  if (!w) return;
  if (w->polish) { gb_polish_free(w->polish); w->polish = NULL; }
  if (w->arena) cudaFree(w->arena);
  if (w->pr.Binv) cudaFree(w->pr.Binv);
  if (w->cancel_stream) cudaStreamDestroy(w->cancel_stream);
  if (w->h_one) cudaFreeHost(w->h_one);
  if (w->h_x) cudaFreeHost(w->h_x);
  if (w->h_st) cudaFreeHost(w->h_st);
  if (w->ev0) cudaEventDestroy(w->ev0);
  if (w->ev1) cudaEventDestroy(w->ev1);
  if (w->stream) cudaStreamDestroy(w->stream);
  free(w);
}

extern "C" OSQPInt osqp_setup(OSQPSolver** solverp, const OSQPCscMatrix* P, const OSQPFloat* q,
                              const OSQPCscMatrix* A, const OSQPFloat* l, const OSQPFloat* u,
                              OSQPInt m, OSQPInt n, const OSQPSettings* settings) {
  double t0 = wall_s();
  if (!solverp) return OSQP_DATA_VALIDATION_ERROR;
  *solverp = NULL;
  if (!P || !A || !q || (m > 0 && (!l || !u))) return OSQP_DATA_VALIDATION_ERROR;
  if (validate_settings(settings, 1)) return OSQP_SETTINGS_VALIDATION_ERROR;
  if (cudaSetDevice(settings->device) != cudaSuccess) return OSQP_ALGEBRA_LOAD_ERROR;

  std::vector<OSQPInt> Pp, Pi, Ap, Ai;
  if (n <= 0 || fetch_pattern(P, Pp, Pi) || fetch_pattern(A, Ap, Ai)) return OSQP_DATA_VALIDATION_ERROR;
  if (validate_data(P, q, A, l, u, m, n, Pp, Pi)) return OSQP_DATA_VALIDATION_ERROR;

  OSQPSolver* solver = (OSQPSolver*)calloc(1, sizeof(OSQPSolver));
  OSQPWorkspace* w = (OSQPWorkspace*)calloc(1, sizeof(OSQPWorkspace));
  if (!solver || !w) { free(solver); free(w); return OSQP_MEM_ALLOC_ERROR; }
  solver->work = w;
  solver->info = (OSQPInfo*)calloc(1, sizeof(OSQPInfo));
  solver->settings = (OSQPSettings*)malloc(sizeof(OSQPSettings));
  if (!solver->info || !solver->settings) { osqp_cleanup(solver); *solverp = NULL; return OSQP_MEM_ALLOC_ERROR; }
  memcpy(solver->settings, settings, sizeof(OSQPSettings));
  *solverp = solver;

  w->n = n; w->m = m; w->device = settings->device;
  w->nnzT = Pp[n]; w->nnzA = Ap[n];
  int ndiag = 0;
  for (OSQPInt j = 0; j < n; j++)
    for (OSQPInt k = Pp[j]; k < Pp[j + 1]; k++) if (Pi[k] == j) { ndiag++; break; }
  w->nnzPf = 2 * w->nnzT - ndiag + (n - ndiag);
  const int nnzT = w->nnzT, nnzA = w->nnzA, nnzPf = w->nnzPf;

  if (cudaStreamCreateWithFlags(&w->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&w->cancel_stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaMallocHost((void**)&w->h_one, sizeof(int)) != cudaSuccess) {
    osqp_cleanup(solver); *solverp = NULL; return OSQP_ALGEBRA_LOAD_ERROR;
  }
  *w->h_one = 1;
  if (cudaEventCreate(&w->ev0) != cudaSuccess || cudaEventCreate(&w->ev1) != cudaSuccess) { osqp_cleanup(solver); *solverp = NULL; return OSQP_ALGEBRA_LOAD_ERROR; }

  // Execution form: one CTA for small problems, cooperative grid otherwise.
  // Execution form by problem size: one CTA, one thread-block cluster, or
  // the cooperative grid.
  const long long work_nnz = (long long)nnzPf + 2LL * nnzA + n + m;
  const char* mode = getenv("OSQP_GB300_MODE");
  w->use_grid = work_nnz > 2000000;
  w->cluster = (!w->use_grid && work_nnz > 30000) ? 16 : 1;
  if (mode && !strcmp(mode, "block")) { w->use_grid = 0; w->cluster = 1; }
  if (mode && !strcmp(mode, "grid")) { w->use_grid = 1; w->cluster = 1; }
  if (mode && !strncmp(mode, "cluster", 7)) { w->use_grid = 0; w->cluster = mode[7] ? atoi(mode + 7) : 16; }
  if (w->cluster > 1) {
    const int c1 = max_active_clusters(k_solve_cluster<T>, w->cluster, kClusterThreads);
    const int c2 = max_active_clusters(k_setup_cluster<T>, w->cluster, kClusterThreads);
    if (c1 < 1 || c2 < 1) w->cluster = (w->cluster > 8 && max_active_clusters(k_solve_cluster<T>, 8, kClusterThreads) > 0 &&
                                        max_active_clusters(k_setup_cluster<T>, 8, kClusterThreads) > 0) ? 8 : 1;
  }
  // Direct solver: the plan on the host, then the CTA form with the
  // factorisation and block solve in shared memory
  KktPlan kplan;
  int kring = 0;
  const bool direct = settings->linsys_solver == OSQP_DIRECT_SOLVER;
  if (direct) {
    cudaFuncAttributes fa;
    int optin = 0;
    if (cudaFuncGetAttributes(&fa, k_solve_block<T>) != cudaSuccess ||
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, w->device) != cudaSuccess) {
      osqp_cleanup(solver); *solverp = NULL; return OSQP_ALGEBRA_LOAD_ERROR;
    }
    const long long room = (long long)optin - (long long)fa.sharedSizeBytes - 1024;
    const int blim = kkt_bmax_limit(kBlockThreads, room, (int)sizeof(T));
    const int prc = kkt_plan_build(n, m, Pp.data(), Pi.data(), Ap.data(), Ai.data(), blim, kplan);
    int R = kKktRingMax;
    while (!prc && R >= 2 && kkt_ws_bytes(n, m, kplan.bmax, kplan.nb, kplan.segmax, R, (int)sizeof(T)) > room) R--;
    if (R < 2) R = 0;
    const long long need = prc ? 0 : kkt_ws_bytes(n, m, kplan.bmax, kplan.nb, kplan.segmax, R, (int)sizeof(T));
    kring = R;
    if (prc || need > room) {
      fprintf(stderr, "osqp_gb300: the direct KKT solver does not apply to this problem (n=%d, m=%d): %s\n", n, m,
              prc == 1 ? "a block of its block-tridiagonal ordering exceeds the on-chip limit"
              : prc ? "inconsistent structure" : "its solve vectors exceed the on-chip workspace");
      osqp_cleanup(solver); *solverp = NULL; return OSQP_LINSYS_SOLVER_INIT_ERROR;
    }
    w->kdsm = (size_t)((need + 1023) & ~1023LL);
    if (cudaFuncSetAttribute(k_solve_block<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)w->kdsm) != cudaSuccess ||
        cudaFuncSetAttribute(k_setup_block<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)w->kdsm) != cudaSuccess ||
        cudaFuncSetAttribute(k_refactor_block<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)w->kdsm) != cudaSuccess) {
      osqp_cleanup(solver); *solverp = NULL; return OSQP_ALGEBRA_LOAD_ERROR;
    }
    w->use_grid = 0;
    w->cluster = 1;
  }
  if (w->use_grid) {
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_solve_grid<T>, kGridThreads, 0);
    int per_sm2 = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm2, k_setup_grid<T>, kGridThreads, 0);
    per_sm = std::min(per_sm, per_sm2);
    if (per_sm < 1) w->use_grid = 0;
    else w->grid_blocks = device_sms(w->device);
  }

  // ---- arena ----
  ArenaPlan ap;
  size_t o_Prow = ap.take<int>(n + 1), o_Pcol = ap.take<int>(nnzPf), o_Pval = ap.take<T>(nnzPf);
  size_t o_Pdiag = ap.take<int>(n), o_Psrc = ap.take<int>(nnzPf), o_Praw = ap.take<T>(nnzT);
  size_t o_Arow = ap.take<int>(m + 1), o_Acol = ap.take<int>(nnzA), o_Aval = ap.take<T>(nnzA);
  size_t o_Asrc = ap.take<int>(nnzA), o_Araw = ap.take<T>(nnzA);
  size_t o_Atrow = ap.take<int>(n + 1), o_Atcol = ap.take<int>(nnzA), o_Atval = ap.take<T>(nnzA);
  size_t o_vn[16], o_vm[16];
  for (int k = 0; k < 16; k++) o_vn[k] = ap.take<T>(n);
  for (int k = 0; k < 16; k++) o_vm[k] = ap.take<T>(m);
  size_t o_ctype = ap.take<int>(m);
  size_t o_st = ap.take<SolverScalars>(1);
  size_t o_bar = ap.take<unsigned int>(4);
  size_t o_err = ap.take<int>(4);
  const int gb = w->use_grid ? w->grid_blocks : 1;
  size_t o_part = ap.take<double>((size_t)(4 * kMaxSum + 2 * kMaxMax) * gb);
  const size_t knb1 = direct ? (size_t)kplan.nb + 1 : 0;
  size_t o_kperm = ap.take<int>(direct ? n : 0), o_kiperm = ap.take<int>(direct ? n : 0);
  size_t o_kbs = ap.take<int>(knb1), o_kfo = ap.take<int>(knb1), o_kco = ap.take<int>(knb1), o_kbo = ap.take<int>(knb1);
  size_t o_kcr = ap.take<int>(direct ? kplan.cr.size() : 0), o_kF = ap.take<T>(direct ? (size_t)kplan.fsize : 0);
  w->arena_bytes = ap.off;
  if (cudaMalloc(&w->arena, w->arena_bytes) != cudaSuccess) { osqp_cleanup(solver); *solverp = NULL; return OSQP_MEM_ALLOC_ERROR; }
  cudaMemsetAsync(w->arena, 0, w->arena_bytes, w->stream);
  char* b = w->arena;
  DevProblem<T>& pr = w->pr;
  pr.n = n; pr.m = m;
  pr.P = CSR<T>{(int*)(b + o_Prow), (int*)(b + o_Pcol), (T*)(b + o_Pval), n, n, 1};
  pr.A = CSR<T>{(int*)(b + o_Arow), (int*)(b + o_Acol), (T*)(b + o_Aval), m, n, 1};
  pr.At = CSR<T>{(int*)(b + o_Atrow), (int*)(b + o_Atcol), (T*)(b + o_Atval), n, m, 1};
  pr.Pdiag = (int*)(b + o_Pdiag); pr.Psrc = (int*)(b + o_Psrc); pr.Praw = (T*)(b + o_Praw);
  pr.Asrc = (int*)(b + o_Asrc); pr.Araw = (T*)(b + o_Araw);
  T* vn[16]; T* vm[16];
  for (int k = 0; k < 16; k++) { vn[k] = (T*)(b + o_vn[k]); vm[k] = (T*)(b + o_vm[k]); }
  pr.q = vn[0]; pr.q_in = vn[1]; pr.D = vn[2]; pr.Dinv = vn[3]; pr.x = vn[4]; pr.dx = vn[5];
  pr.xp = vn[6]; pr.r = vn[7]; pr.p0 = vn[8]; pr.p1 = vn[9]; pr.Kp = vn[10]; pr.yv = vn[11];
  pr.rhs = vn[12]; pr.Minv = vn[13]; pr.xo = vn[14]; pr.dcert = vn[15];
  pr.Dt = (T*)pr.Kp;  // scaling scratch aliases PCG vectors (setup only)
  pr.l = vm[0]; pr.u = vm[1]; pr.l_in = vm[2]; pr.u_in = vm[3]; pr.E = vm[4]; pr.Einv = vm[5];
  pr.rho_vec = vm[6]; pr.rho_inv_vec = vm[7]; pr.z = vm[8]; pr.y = vm[9]; pr.dy = vm[10];
  pr.t = vm[11]; pr.yo = vm[12]; pr.pcert = vm[13]; pr.Et = vm[14];
  pr.ctype = (int*)(b + o_ctype);
  pr.st = (SolverScalars*)(b + o_st);
  pr.Arow_g = pr.A.rowptr; pr.Acol_g = pr.A.col; pr.Aval_g = pr.A.val;
  pr.Binv = nullptr;
  w->bar = (unsigned int*)(b + o_bar);
  w->err = (int*)(b + o_err);
  w->flag = w->err + 1;
  w->partials = (double*)(b + o_part);
  if (direct) {
    pr.kkt.nb = kplan.nb; pr.kkt.bmax = kplan.bmax;
    pr.kkt.ring = kring; pr.kkt.segmax = kplan.segmax;
    pr.kkt.bo = (int*)(b + o_kbo);
    pr.kkt.perm = (int*)(b + o_kperm); pr.kkt.iperm = (int*)(b + o_kiperm);
    pr.kkt.bs = (int*)(b + o_kbs); pr.kkt.fo = (int*)(b + o_kfo); pr.kkt.co = (int*)(b + o_kco);
    pr.kkt.cr = (int*)(b + o_kcr); pr.kkt.F = (T*)(b + o_kF);
    cudaStream_t s0 = w->stream;
    GB_TRY(cudaMemcpyAsync((void*)pr.kkt.perm, kplan.perm.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s0));
    GB_TRY(cudaMemcpyAsync((void*)pr.kkt.iperm, kplan.iperm.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s0));
    GB_TRY(cudaMemcpyAsync((void*)pr.kkt.bs, kplan.bs.data(), sizeof(int) * knb1, cudaMemcpyHostToDevice, s0));
    GB_TRY(cudaMemcpyAsync((void*)pr.kkt.fo, kplan.fo.data(), sizeof(int) * knb1, cudaMemcpyHostToDevice, s0));
    GB_TRY(cudaMemcpyAsync((void*)pr.kkt.bo, kplan.bo.data(), sizeof(int) * knb1, cudaMemcpyHostToDevice, s0));
    GB_TRY(cudaMemcpyAsync((void*)pr.kkt.co, kplan.co.data(), sizeof(int) * knb1, cudaMemcpyHostToDevice, s0));
    if (!kplan.cr.empty())
      GB_TRY(cudaMemcpyAsync((void*)pr.kkt.cr, kplan.cr.data(), sizeof(int) * kplan.cr.size(), cudaMemcpyHostToDevice, s0));
    GB_TRY(cudaStreamSynchronize(s0));   // the plan's host vectors end with this call
  }

  // ---- raw data in (host or device pointers) ----
  cudaStream_t s = w->stream;
  if (nnzT) GB_TRY(cudaMemcpyAsync((void*)pr.Praw, P->x, sizeof(T) * nnzT, cudaMemcpyDefault, s));
  if (nnzA) GB_TRY(cudaMemcpyAsync((void*)pr.Araw, A->x, sizeof(T) * nnzA, cudaMemcpyDefault, s));
  GB_TRY(cudaMemcpyAsync((void*)pr.q_in, q, sizeof(T) * n, cudaMemcpyDefault, s));
  if (m) {
    GB_TRY(cudaMemcpyAsync((void*)pr.l_in, l, sizeof(T) * m, cudaMemcpyDefault, s));
    GB_TRY(cudaMemcpyAsync((void*)pr.u_in, u, sizeof(T) * m, cudaMemcpyDefault, s));
  }
  GB_TRY(cudaMemcpyAsync((void*)pr.At.rowptr, Ap.data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice, s));
  if (nnzA) GB_TRY(cudaMemcpyAsync((void*)pr.At.col, Ai.data(), sizeof(int) * nnzA, cudaMemcpyHostToDevice, s));

  // ---- structures: CSR(A) by stable sort of CSC row keys ----
  {
    int *keys_in = nullptr, *keys_out = nullptr, *idx_in = nullptr, *cols = nullptr;
    void* tmp = nullptr; size_t tmp_bytes = 0;
    const int na = nnzA > 0 ? nnzA : 1;
    GB_TRY(cudaMallocAsync((void**)&keys_in, sizeof(int) * na, s));
    GB_TRY(cudaMallocAsync((void**)&keys_out, sizeof(int) * na, s));
    GB_TRY(cudaMallocAsync((void**)&idx_in, sizeof(int) * na, s));
    GB_TRY(cudaMallocAsync((void**)&cols, sizeof(int) * na, s));
    if (nnzA) {
      GB_TRY(cudaMemcpyAsync(keys_in, Ai.data(), sizeof(int) * nnzA, cudaMemcpyHostToDevice, s));
      k_iota<<<256, 256, 0, s>>>(idx_in, nnzA);
      k_csc_entry_cols<<<(n + 255) / 256, 256, 0, s>>>(pr.At.rowptr, n, cols);
      const int bits = bits_for((unsigned long long)(m > 0 ? m : 1));
      cub::DeviceRadixSort::SortPairs(tmp, tmp_bytes, keys_in, keys_out, idx_in, (int*)pr.Asrc, nnzA, 0, bits, s);
      GB_TRY(cudaMallocAsync(&tmp, tmp_bytes ? tmp_bytes : 1, s));
      GB_TRY(cub::DeviceRadixSort::SortPairs(tmp, tmp_bytes, keys_in, keys_out, idx_in, (int*)pr.Asrc, nnzA, 0, bits, s));
      k_gather_int<<<256, 256, 0, s>>>(cols, pr.Asrc, nnzA, (int*)pr.A.col);
      cudaFreeAsync(tmp, s);
    }
    k_rowptr_from_sorted<<<std::max(1, (nnzA + 256) / 256), 256, 0, s>>>(keys_out, nnzA, m, (int*)pr.A.rowptr);
    cudaFreeAsync(keys_in, s); cudaFreeAsync(keys_out, s); cudaFreeAsync(idx_in, s); cudaFreeAsync(cols, s);
  }
  // ---- structures: full symmetric CSR(P) from its upper triangle ----
  {
    const int slots = 2 * nnzT + n;
    unsigned long long *k_in = nullptr, *k_out = nullptr;
    int *s_in = nullptr, *s_out = nullptr, *dPp = nullptr, *dPi = nullptr;
    void* tmp = nullptr; size_t tmp_bytes = 0;
    GB_TRY(cudaMallocAsync((void**)&k_in, sizeof(unsigned long long) * slots, s));
    GB_TRY(cudaMallocAsync((void**)&k_out, sizeof(unsigned long long) * slots, s));
    GB_TRY(cudaMallocAsync((void**)&s_in, sizeof(int) * slots, s));
    GB_TRY(cudaMallocAsync((void**)&s_out, sizeof(int) * slots, s));
    GB_TRY(cudaMallocAsync((void**)&dPp, sizeof(int) * (n + 1), s));
    GB_TRY(cudaMallocAsync((void**)&dPi, sizeof(int) * (nnzT > 0 ? nnzT : 1), s));
    GB_TRY(cudaMemcpyAsync(dPp, Pp.data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice, s));
    if (nnzT) GB_TRY(cudaMemcpyAsync(dPi, Pi.data(), sizeof(int) * nnzT, cudaMemcpyHostToDevice, s));
    k_triu_expand<<<(n + 255) / 256, 256, 0, s>>>(dPp, dPi, n, nnzT, k_in, s_in);
    cub::DeviceRadixSort::SortPairs(tmp, tmp_bytes, k_in, k_out, s_in, s_out, slots, 0, 64, s);
    GB_TRY(cudaMallocAsync(&tmp, tmp_bytes ? tmp_bytes : 1, s));
    GB_TRY(cub::DeviceRadixSort::SortPairs(tmp, tmp_bytes, k_in, k_out, s_in, s_out, slots, 0, 64, s));
    k_full_from_sorted<<<(nnzPf + 256) / 256, 256, 0, s>>>(k_out, nnzPf, n, (int*)pr.P.col, (int*)pr.P.rowptr, (int*)pr.Pdiag);
    GB_TRY(cudaMemcpyAsync((void*)pr.Psrc, s_out, sizeof(int) * nnzPf, cudaMemcpyDeviceToDevice, s));
    cudaFreeAsync(tmp, s); cudaFreeAsync(k_in, s); cudaFreeAsync(k_out, s);
    cudaFreeAsync(s_in, s); cudaFreeAsync(s_out, s); cudaFreeAsync(dPp, s); cudaFreeAsync(dPi, s);
  }
  pr.P.lanes = pick_lanes(nnzPf, n);
  pr.A.lanes = pick_lanes(nnzA, m);
  pr.At.lanes = pick_lanes(nnzA, n);
  w->kktL = pick_lanes((long long)nnzPf + nnzA, n);

  // ---- settings (adaptive interval rule of osqp_api.c:569-603) ----
  OSQPSettings* st = solver->settings;
  st->rho = (OSQPFloat)fmin(fmax((double)st->rho, 1e-6), 1e6);
  if (st->adaptive_rho == OSQP_ADAPTIVE_RHO_UPDATE_ITERATIONS && st->adaptive_rho_interval == 0)
    st->adaptive_rho_interval = st->check_termination ? OSQP_ADAPTIVE_RHO_MULTIPLE_TERMINATION * st->check_termination
                                                      : OSQP_ADAPTIVE_RHO_FIXED;
  if (st->adaptive_rho == OSQP_ADAPTIVE_RHO_UPDATE_KKT_ERROR && st->adaptive_rho_interval == 0)
    st->adaptive_rho_interval = 1;
  w->ds = make_dev_settings(st);
  if (ensure_block_precond(w)) { osqp_cleanup(solver); *solverp = NULL; return OSQP_MEM_ALLOC_ERROR; }

  if (cudaMallocHost((void**)&w->h_st, sizeof(SolverScalars)) != cudaSuccess) { osqp_cleanup(solver); *solverp = NULL; return OSQP_MEM_ALLOC_ERROR; }
  int rc = launch_setup(w, 0);
  if (rc) { osqp_cleanup(solver); *solverp = NULL; return rc; }
  if (direct) {
    // the builtin's set-up reports a KKT matrix that is not quasi-definite
    // (P not positive semidefinite) as OSQP_NONCVX_ERROR (osqp_api.c:500-505)
    int fail = 0;
    if (cudaMemcpy(&fail, &w->pr.st->kkt_fail, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) fail = -1;
    if (fail) { osqp_cleanup(solver); *solverp = NULL; return fail > 0 ? OSQP_NONCVX_ERROR : OSQP_ALGEBRA_LOAD_ERROR; }
  }

  if (settings->allocate_solution) {
    solver->solution = (OSQPSolution*)calloc(1, sizeof(OSQPSolution));
    if (!solver->solution) { osqp_cleanup(solver); *solverp = NULL; return OSQP_MEM_ALLOC_ERROR; }
    solver->solution->x = (OSQPFloat*)calloc((size_t)n, sizeof(OSQPFloat));
    solver->solution->y = (OSQPFloat*)calloc((size_t)(m ? m : 1), sizeof(OSQPFloat));
    solver->solution->prim_inf_cert = (OSQPFloat*)calloc((size_t)(m ? m : 1), sizeof(OSQPFloat));
    solver->solution->dual_inf_cert = (OSQPFloat*)calloc((size_t)n, sizeof(OSQPFloat));
  }
  OSQPInfo* info = solver->info;
  info->status_polish = OSQP_POLISH_NOT_PERFORMED;
  set_status(info, OSQP_UNSOLVED);
  info->rho_updates = 0;
  info->rho_estimate = st->rho;
  info->obj_val = OSQP_INFTY; info->prim_res = OSQP_INFTY; info->dual_res = OSQP_INFTY;
  info->rel_kkt_error = OSQP_INFTY;
  w->first_run = 1;
  info->setup_time = (OSQPFloat)(wall_s() - t0);
  return 0;
}

static void grid_sync_args(OSQPWorkspace* w, GridSync& gs) {
  gs.count = w->bar; gs.gen = w->bar + 1; gs.err = w->err;
  gs.partial_sum = w->partials;
  gs.partial_max = w->partials + (size_t)4 * kMaxSum * w->grid_blocks;
}

static int check_device_error(OSQPWorkspace* w) {
  cudaError_t e = cudaStreamSynchronize(w->stream);
  if (e != cudaSuccess) {
    fprintf(stderr, "osqp_gb300: device error: %s\n", cudaGetErrorString(e));
    return OSQP_ALGEBRA_LOAD_ERROR;
  }
  int err = 0;
  if (cudaMemcpy(&err, w->err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return OSQP_ALGEBRA_LOAD_ERROR;
  if (err) {
    fprintf(stderr, "osqp_gb300: device barrier timed out (error %d)\n", err);
    return OSQP_ALGEBRA_LOAD_ERROR;
  }
  return 0;
}

static int launch_setup(OSQPWorkspace* w, int keep_state) {
  cudaStream_t s = w->stream;
  cudaMemsetAsync(w->bar, 0, sizeof(unsigned int) * 4 + sizeof(int) * 4, s);
  if (w->use_grid) {
    GridSync gs; grid_sync_args(w, gs);
    void* args[] = {(void*)&w->pr, (void*)&w->ds, (void*)&w->kktL, (void*)&keep_state, (void*)&gs};
    GB_TRY(cudaLaunchCooperativeKernel((void*)k_setup_grid<T>, dim3(w->grid_blocks), dim3(kGridThreads), args, 0, s));
  } else if (w->cluster > 1) {
    GB_TRY(launch_clusters(k_setup_cluster<T>, 1, w->cluster, kClusterThreads, s, w->pr, w->ds, w->kktL, keep_state));
  } else {
    k_setup_block<T><<<1, kBlockThreads, w->kdsm, s>>>(w->pr, w->ds, w->kktL, keep_state);
    GB_TRY(cudaGetLastError());
  }
  return check_device_error(w);
}

static int launch_solve(OSQPWorkspace* w) {
  cudaStream_t s = w->stream;
  cudaMemsetAsync(w->bar, 0, sizeof(unsigned int) * 4 + sizeof(int) * 4, s);
  // an interrupt counts for the solve it arrives in (the reference's
  // listener also starts clear on every solve): this solve's generation is
  // new, so the cancel word matches it only after a request made from now on
  w->ds.cancel_gen = ++w->gen;
  cudaEventRecord(w->ev0, s);
  if (w->use_grid) {
    GridSync gs; grid_sync_args(w, gs);
    void* args[] = {(void*)&w->pr, (void*)&w->ds, (void*)&w->kktL, (void*)&gs};
    GB_TRY(cudaLaunchCooperativeKernel((void*)k_solve_grid<T>, dim3(w->grid_blocks), dim3(kGridThreads), args, 0, s));
  } else if (w->cluster > 1) {
    GB_TRY(launch_clusters(k_solve_cluster<T>, 1, w->cluster, kClusterThreads, s, w->pr, w->ds, w->kktL));
  } else {
    k_solve_block<T><<<1, kBlockThreads, w->kdsm, s>>>(w->pr, w->ds, w->kktL);
    GB_TRY(cudaGetLastError());
  }
  cudaEventRecord(w->ev1, s);
  return 0;
}

// store the device solution into user buffers (host or device pointers)
static int copy_solution(OSQPWorkspace* w, OSQPSolution* sol) {
  if (!sol) return 0;
  cudaStream_t s = w->stream;
  const int n = w->n, m = w->m;
  if (sol->x) GB_TRY(cudaMemcpyAsync(sol->x, w->pr.xo, sizeof(T) * n, cudaMemcpyDefault, s));
  if (sol->dual_inf_cert) GB_TRY(cudaMemcpyAsync(sol->dual_inf_cert, w->pr.dcert, sizeof(T) * n, cudaMemcpyDefault, s));
  if (m && sol->y) GB_TRY(cudaMemcpyAsync(sol->y, w->pr.yo, sizeof(T) * m, cudaMemcpyDefault, s));
  if (m && sol->prim_inf_cert) GB_TRY(cudaMemcpyAsync(sol->prim_inf_cert, w->pr.pcert, sizeof(T) * m, cudaMemcpyDefault, s));
  return 0;
}

static void fill_info(OSQPSolver* solver) {
  const SolverScalars* c = solver->work->h_st;
  OSQPInfo* info = solver->info;
  set_status(info, c->status);
  info->obj_val = (OSQPFloat)c->obj_val;
  info->dual_obj_val = (OSQPFloat)c->dual_obj_val;
  info->prim_res = (OSQPFloat)c->prim_res;
  info->dual_res = (OSQPFloat)c->dual_res;
  info->duality_gap = (OSQPFloat)c->duality_gap;
  info->iter = c->iter;
  info->rho_updates = c->rho_updates;
  info->rho_estimate = (OSQPFloat)c->rho_estimate;
  info->primdual_int = (OSQPFloat)c->primdual_int;
  info->rel_kkt_error = (OSQPFloat)c->rel_kkt_error;
  if (!Solver<T>::has_solution(c->status)) {
    if (c->status == OSQP_PRIMAL_INFEASIBLE || c->status == OSQP_PRIMAL_INFEASIBLE_INACCURATE) info->obj_val = OSQP_INFTY;
    if (c->status == OSQP_DUAL_INFEASIBLE || c->status == OSQP_DUAL_INFEASIBLE_INACCURATE) info->obj_val = -OSQP_INFTY;
  }
}

extern "C" OSQPInt osqp_solve(OSQPSolver* solver) {
  if (!solver || !solver->work) return OSQP_WORKSPACE_NOT_INIT_ERROR;
  OSQPWorkspace* w = solver->work;
  OSQPInfo* info = solver->info;
  if (w->clear_update_time) info->update_time = 0.0;
  double t0 = wall_s();
  cudaSetDevice(w->device);
  int rc;
  {
    InterruptListener listener;
    rc = launch_solve(w);
    if (rc) return rc;
    cudaMemcpyAsync(w->h_st, w->pr.st, sizeof(SolverScalars), cudaMemcpyDeviceToHost, w->stream);
    // wait for the solve; a Ctrl-C meanwhile becomes an interrupt request
    bool sent = false;
    while (cudaStreamQuery(w->stream) == cudaErrorNotReady) {
      if (!sent && listener.fired()) { request_cancel(w); sent = true; }
      std::this_thread::sleep_for(std::chrono::microseconds(50));   // a core is not pinned per solve
    }
  }
  rc = check_device_error(w);
  if (rc) return rc;
  cudaEventElapsedTime(&w->last_kernel_ms, w->ev0, w->ev1);
  fill_info(solver);
  info->solve_time = (OSQPFloat)(wall_s() - t0);
  info->polish_time = 0.0;
  info->status_polish = OSQP_POLISH_NOT_PERFORMED;
  if (solver->settings->polishing && info->status_val == OSQP_SOLVED) {
    double tp = wall_s();
    rc = gb_polish_run(solver);
    info->polish_time = (OSQPFloat)(wall_s() - tp);
    if (rc > 0) return rc;
  }
  info->run_time = (w->first_run ? info->setup_time : info->update_time) + info->solve_time + info->polish_time;
  w->first_run = 0;
  w->clear_update_time = 1;
  // an interrupted solve stores no solution and returns 1 (osqp_api.c:730-736)
  if (info->status_val == OSQP_SIGINT) return 1;
  rc = copy_solution(w, solver->solution);
  if (rc) return rc;
  if (cudaStreamSynchronize(w->stream) != cudaSuccess) return OSQP_ALGEBRA_LOAD_ERROR;
  return 0;
}

extern "C" OSQPInt osqp_gb300_interrupt(OSQPSolver* solver) {
  if (!solver || !solver->work) return OSQP_WORKSPACE_NOT_INIT_ERROR;
  return request_cancel(solver->work);
}

extern "C" OSQPInt osqp_get_solution(OSQPSolver* solver, OSQPSolution* solution) {
  if (!solver || !solver->work || !solution) return OSQP_WORKSPACE_NOT_INIT_ERROR;
  int rc = copy_solution(solver->work, solution);
  if (rc) return rc;
  return cudaStreamSynchronize(solver->work->stream) == cudaSuccess ? 0 : OSQP_ALGEBRA_LOAD_ERROR;
}

extern "C" OSQPInt osqp_cleanup(OSQPSolver* solver) {
  if (!solver) return 0;
  if (solver->work) free_workspace(solver->work);
  if (solver->solution) {
    free(solver->solution->x); free(solver->solution->y);
    free(solver->solution->prim_inf_cert); free(solver->solution->dual_inf_cert);
    free(solver->solution);
  }
  free(solver->settings);
  free(solver->info);
  free(solver);
  return 0;
}

static void reset_info(OSQPInfo* info) {
  info->solve_time = 0.0;
  info->polish_time = 0.0;
  set_status(info, OSQP_UNSOLVED);
  info->rho_updates = 0;
}

static const int kEwBlocks = 296, kEwThreads = 256;

// Preconditioner refresh driven by the host: the Jacobi diagonal and, with
// cg_precond = 2, the blocks of the block-Jacobi one.
static void refresh_precond(OSQPWorkspace* w, cudaStream_t s, double rho, int rho_is_vec) {
  if (w->pr.kkt.nb > 0) {
    // direct solver: refactor for the rho in the device scalar state (and
    // the rho vector, already refreshed on this stream)
    k_refactor_block<T><<<1, kBlockThreads, w->kdsm, s>>>(w->pr, w->ds, w->kktL);
    return;
  }
  k_precond<T><<<kEwBlocks, kEwThreads, 0, s>>>(w->pr, w->ds.sigma, rho, rho_is_vec, w->ds.cg_precond);
  if (w->ds.cg_precond == kPrecondBlockDiagonal && w->pr.Binv)
    k_block_precond<T><<<block_precond_grid(w->n), kBlockPrecondThreads, 0, s>>>(w->pr, w->ds.sigma, rho, rho_is_vec);
}

extern "C" OSQPInt osqp_update_data_vec(OSQPSolver* solver, const OSQPFloat* q_new, const OSQPFloat* l_new,
                                        const OSQPFloat* u_new) {
  if (!solver || !solver->work) return OSQP_WORKSPACE_NOT_INIT_ERROR;
  OSQPWorkspace* w = solver->work;
  double t0 = wall_s();
  if (w->clear_update_time) { w->clear_update_time = 0; solver->info->update_time = 0.0; }
  cudaSetDevice(w->device);
  cudaStream_t s = w->stream;
  const int n = w->n, m = w->m;
  // the staged copies keep the previous inputs until the bounds check passes
  std::vector<T> keep_l, keep_u;
  if (q_new) GB_TRY(cudaMemcpyAsync((void*)w->pr.q_in, q_new, sizeof(T) * n, cudaMemcpyDefault, s));
  int bad = 0;
  if (m && (l_new || u_new)) {
    // stage into l_in / u_in after saving them (restored on a failed check)
    keep_l.resize(m); keep_u.resize(m);
    GB_TRY(cudaMemcpyAsync(keep_l.data(), w->pr.l_in, sizeof(T) * m, cudaMemcpyDeviceToHost, s));
    GB_TRY(cudaMemcpyAsync(keep_u.data(), w->pr.u_in, sizeof(T) * m, cudaMemcpyDeviceToHost, s));
    if (l_new) GB_TRY(cudaMemcpyAsync((void*)w->pr.l_in, l_new, sizeof(T) * m, cudaMemcpyDefault, s));
    if (u_new) GB_TRY(cudaMemcpyAsync((void*)w->pr.u_in, u_new, sizeof(T) * m, cudaMemcpyDefault, s));
  }
  GB_TRY(cudaMemcpyAsync(w->h_st, w->pr.st, sizeof(SolverScalars), cudaMemcpyDeviceToHost, s));
  GB_TRY(cudaStreamSynchronize(s));
  const double c = w->h_st->c;
  GB_TRY(cudaMemsetAsync(w->flag, 0, sizeof(int), s));
  k_update_vec<T><<<kEwBlocks, kEwThreads, 0, s>>>(w->pr, q_new != NULL, l_new != NULL, u_new != NULL,
                                                   solver->settings->scaling, c, w->flag);
  GB_TRY(cudaMemcpyAsync(&bad, w->flag, sizeof(int), cudaMemcpyDeviceToHost, s));
  GB_TRY(cudaStreamSynchronize(s));
  if (bad) {
    if (m && (l_new || u_new)) {
      GB_TRY(cudaMemcpyAsync((void*)w->pr.l_in, keep_l.data(), sizeof(T) * m, cudaMemcpyHostToDevice, s));
      GB_TRY(cudaMemcpyAsync((void*)w->pr.u_in, keep_u.data(), sizeof(T) * m, cudaMemcpyHostToDevice, s));
      GB_TRY(cudaStreamSynchronize(s));
    }
    return OSQP_DATA_VALIDATION_ERROR;
  }
  int rc = 0;
  if (m && (l_new || u_new)) {
    k_commit_bounds<T><<<kEwBlocks, kEwThreads, 0, s>>>(w->pr);
    if (solver->settings->rho_is_vec) {
      int changed = 0;
      GB_TRY(cudaMemsetAsync(w->flag, 0, sizeof(int), s));
      k_rho_vec<T><<<kEwBlocks, kEwThreads, 0, s>>>(w->pr, w->h_st->rho, (double)OSQP_INFTY, 1, w->flag);
      GB_TRY(cudaMemcpyAsync(&changed, w->flag, sizeof(int), cudaMemcpyDeviceToHost, s));
      GB_TRY(cudaStreamSynchronize(s));
      if (changed) refresh_precond(w, s, w->h_st->rho, 1);
    }
  }
  GB_TRY(cudaStreamSynchronize(s));
  reset_info(solver->info);
  solver->info->update_time += (OSQPFloat)(wall_s() - t0);
  return rc;
}

extern "C" OSQPInt osqp_warm_start(OSQPSolver* solver, const OSQPFloat* x, const OSQPFloat* y) {
  if (!solver || !solver->work) return OSQP_WORKSPACE_NOT_INIT_ERROR;
  OSQPWorkspace* w = solver->work;
  cudaSetDevice(w->device);
  cudaStream_t s = w->stream;
  if (!solver->settings->warm_starting) { solver->settings->warm_starting = 1; w->ds.warm_starting = 1; }
  T *dx = NULL, *dy = NULL;
  if (x) { GB_TRY(cudaMallocAsync((void**)&dx, sizeof(T) * w->n, s)); GB_TRY(cudaMemcpyAsync(dx, x, sizeof(T) * w->n, cudaMemcpyDefault, s)); }
  if (y && w->m) { GB_TRY(cudaMallocAsync((void**)&dy, sizeof(T) * w->m, s)); GB_TRY(cudaMemcpyAsync(dy, y, sizeof(T) * w->m, cudaMemcpyDefault, s)); }
  GB_TRY(cudaMemcpyAsync(w->h_st, w->pr.st, sizeof(SolverScalars), cudaMemcpyDeviceToHost, s));
  GB_TRY(cudaStreamSynchronize(s));
  k_warm_start<T><<<kEwBlocks, kEwThreads, 0, s>>>(w->pr, dx, dy, solver->settings->scaling, w->h_st->c);
  if (x) k_z_from_x<T><<<kEwBlocks, kEwThreads, 0, s>>>(w->pr);
  if (dx) cudaFreeAsync(dx, s);
  if (dy) cudaFreeAsync(dy, s);
  GB_TRY(cudaStreamSynchronize(s));
  return 0;
}

extern "C" void osqp_cold_start(OSQPSolver* solver) {
  if (!solver || !solver->work) return;
  OSQPWorkspace* w = solver->work;
  cudaSetDevice(w->device);
  k_cold_start<T><<<kEwBlocks, kEwThreads, 0, w->stream>>>(w->pr);
  cudaStreamSynchronize(w->stream);
}

extern "C" OSQPInt osqp_update_rho(OSQPSolver* solver, OSQPFloat rho_new) {
  if (!solver || !solver->work) return OSQP_WORKSPACE_NOT_INIT_ERROR;
  if (rho_new <= 0) return 1;
  OSQPWorkspace* w = solver->work;
  cudaSetDevice(w->device);
  cudaStream_t s = w->stream;
  const double rho = fmin(fmax((double)rho_new, 1e-6), 1e6);
  solver->settings->rho = (OSQPFloat)rho;
  GB_TRY(cudaMemcpyAsync(w->h_st, w->pr.st, sizeof(SolverScalars), cudaMemcpyDeviceToHost, s));
  GB_TRY(cudaStreamSynchronize(s));
  w->h_st->rho = rho;
  w->h_st->rho_inv = 1.0 / rho;
  GB_TRY(cudaMemcpyAsync(w->pr.st, w->h_st, sizeof(SolverScalars), cudaMemcpyHostToDevice, s));
  if (solver->settings->rho_is_vec) k_rho_vec<T><<<kEwBlocks, kEwThreads, 0, s>>>(w->pr, rho, (double)OSQP_INFTY, 0, w->flag);
  refresh_precond(w, s, rho, solver->settings->rho_is_vec);
  GB_TRY(cudaStreamSynchronize(s));
  return 0;
}

extern "C" OSQPInt osqp_update_data_mat(OSQPSolver* solver, const OSQPFloat* Px_new, const OSQPInt* Px_new_idx,
                                        OSQPInt P_new_n, const OSQPFloat* Ax_new, const OSQPInt* Ax_new_idx,
                                        OSQPInt A_new_n) {
  if (!solver || !solver->work) return OSQP_WORKSPACE_NOT_INIT_ERROR;
  OSQPWorkspace* w = solver->work;
  double t0 = wall_s();
  if (w->clear_update_time) { w->clear_update_time = 0; solver->info->update_time = 0.0; }
  const int nnzP = w->nnzT, nnzA = w->nnzA;
  if (P_new_n > nnzP || P_new_n < 0) return 1;
  if (!Px_new_idx && P_new_n != 0 && P_new_n != nnzP) return 1;
  if (P_new_n == 0) P_new_n = nnzP;
  if (A_new_n > nnzA || A_new_n < 0) return 2;
  if (!Ax_new_idx && A_new_n != 0 && A_new_n != nnzA) return 2;
  if (A_new_n == 0) A_new_n = nnzA;
  cudaSetDevice(w->device);
  cudaStream_t s = w->stream;
  T* tmpv = NULL; int* tmpi = NULL;
  const int mx = std::max(P_new_n, A_new_n);
  GB_TRY(cudaMallocAsync((void**)&tmpv, sizeof(T) * (mx > 0 ? mx : 1), s));
  GB_TRY(cudaMallocAsync((void**)&tmpi, sizeof(int) * (mx > 0 ? mx : 1), s));
  if (Px_new && P_new_n) {
    GB_TRY(cudaMemcpyAsync(tmpv, Px_new, sizeof(T) * P_new_n, cudaMemcpyDefault, s));
    if (Px_new_idx) GB_TRY(cudaMemcpyAsync(tmpi, Px_new_idx, sizeof(int) * P_new_n, cudaMemcpyDefault, s));
    k_scatter_vals<T><<<kEwBlocks, kEwThreads, 0, s>>>((T*)w->pr.Praw, tmpv, Px_new_idx ? tmpi : NULL, P_new_n);
  }
  if (Ax_new && A_new_n) {
    GB_TRY(cudaMemcpyAsync(tmpv, Ax_new, sizeof(T) * A_new_n, cudaMemcpyDefault, s));
    if (Ax_new_idx) GB_TRY(cudaMemcpyAsync(tmpi, Ax_new_idx, sizeof(int) * A_new_n, cudaMemcpyDefault, s));
    k_scatter_vals<T><<<kEwBlocks, kEwThreads, 0, s>>>((T*)w->pr.Araw, tmpv, Ax_new_idx ? tmpi : NULL, A_new_n);
  }
  cudaFreeAsync(tmpv, s); cudaFreeAsync(tmpi, s);
  int rc = launch_setup(w, 1);
  if (rc) return rc;
  reset_info(solver->info);
  solver->info->update_time += (OSQPFloat)(wall_s() - t0);
  return 0;
}

extern "C" OSQPInt osqp_update_settings(OSQPSolver* solver, const OSQPSettings* ns) {
  if (!solver || !solver->work) return OSQP_WORKSPACE_NOT_INIT_ERROR;
  if (validate_settings(ns, 0)) return OSQP_SETTINGS_VALIDATION_ERROR;
  OSQPSettings* s = solver->settings;
  OSQPWorkspace* w = solver->work;
  const int precond_changed = s->cg_precond != ns->cg_precond;
  const osqp_precond_type precond_before = s->cg_precond;
  s->profiler_level = ns->profiler_level; s->verbose = ns->verbose; s->warm_starting = ns->warm_starting;
  s->polishing = ns->polishing; s->alpha = ns->alpha;
  s->cg_max_iter = ns->cg_max_iter; s->cg_tol_reduction = ns->cg_tol_reduction;
  s->cg_tol_fraction = ns->cg_tol_fraction; s->cg_precond = ns->cg_precond;
  s->max_iter = ns->max_iter; s->eps_abs = ns->eps_abs; s->eps_rel = ns->eps_rel;
  s->eps_prim_inf = ns->eps_prim_inf; s->eps_dual_inf = ns->eps_dual_inf;
  s->scaled_termination = ns->scaled_termination; s->check_termination = ns->check_termination;
  s->check_dualgap = ns->check_dualgap; s->time_limit = ns->time_limit;
  s->delta = ns->delta; s->polish_refine_iter = ns->polish_refine_iter;
  w->ds = make_dev_settings(s);
  if (precond_changed) {
    cudaSetDevice(w->device);
    if (ensure_block_precond(w)) {
      // no room for the blocks: keep the previous preconditioner
      s->cg_precond = precond_before;
      w->ds = make_dev_settings(s);
      return OSQP_MEM_ALLOC_ERROR;
    }
    GB_TRY(cudaMemcpyAsync(w->h_st, w->pr.st, sizeof(SolverScalars), cudaMemcpyDeviceToHost, w->stream));
    GB_TRY(cudaStreamSynchronize(w->stream));
    refresh_precond(w, w->stream, w->h_st->rho, s->rho_is_vec);
    GB_TRY(cudaStreamSynchronize(w->stream));
  }
  return 0;
}

extern "C" OSQPInt osqp_gb300_solve_stats(OSQPSolver* solver, OSQPInt* admm_iter, long long* pcg_iter,
                                          double* kernel_ms, OSQPInt* grid_form) {
  if (!solver || !solver->work) return OSQP_WORKSPACE_NOT_INIT_ERROR;
  OSQPWorkspace* w = solver->work;
  if (admm_iter) *admm_iter = w->h_st->iter;
  if (pcg_iter) *pcg_iter = w->h_st->pcg_iters_total;
  if (kernel_ms) *kernel_ms = w->last_kernel_ms;
  if (grid_form) *grid_form = w->use_grid ? 1 : (w->cluster > 1 ? w->cluster : 0);
  return 0;
}

extern "C" OSQPInt osqp_gb300_structure(OSQPSolver* solver, OSQPInt which, OSQPInt* rowptr, OSQPInt* col,
                                        OSQPInt* src, OSQPInt* diag) {
  if (!solver || !solver->work || which < 0 || which > 1) return -1;
  OSQPWorkspace* w = solver->work;
  if (cudaSetDevice(w->device) != cudaSuccess || cudaStreamSynchronize(w->stream) != cudaSuccess) return -1;
  const CSR<T>& M = which == 0 ? w->pr.P : w->pr.A;
  const int rows = which == 0 ? w->n : w->m, nz = which == 0 ? w->nnzPf : w->nnzA;
  const int* sp = which == 0 ? w->pr.Psrc : w->pr.Asrc;
  if (rowptr && cudaMemcpy(rowptr, M.rowptr, sizeof(int) * (rows + 1), cudaMemcpyDeviceToHost) != cudaSuccess) return -1;
  if (col && nz && cudaMemcpy(col, M.col, sizeof(int) * nz, cudaMemcpyDeviceToHost) != cudaSuccess) return -1;
  if (src && nz && cudaMemcpy(src, sp, sizeof(int) * nz, cudaMemcpyDeviceToHost) != cudaSuccess) return -1;
  if (diag && which == 0 && cudaMemcpy(diag, w->pr.Pdiag, sizeof(int) * w->n, cudaMemcpyDeviceToHost) != cudaSuccess) return -1;
  return nz;
}

extern "C" OSQPInt osqp_gb300_precond_blocks(OSQPSolver* solver, OSQPFloat* out) {
  if (!solver || !solver->work) return 0;
  OSQPWorkspace* w = solver->work;
  if (w->ds.cg_precond != kPrecondBlockDiagonal || !w->pr.Binv) return 0;
  const size_t cnt = block_precond_elems(w->n);
  if (out) {
    cudaSetDevice(w->device);
    if (cudaMemcpyAsync(out, w->pr.Binv, sizeof(T) * cnt, cudaMemcpyDefault, w->stream) != cudaSuccess ||
        cudaStreamSynchronize(w->stream) != cudaSuccess)
      return 0;
  }
  return (OSQPInt)cnt;
}

// The workspace as the polish stage sees it.
GbEngineView gb_engine_view(OSQPSolver* solver) {
  OSQPWorkspace* w = solver->work;
  GbEngineView v;
  v.pr = w->pr; v.ds = w->ds;
  v.n = w->n; v.m = w->m; v.nnzA = w->nnzA; v.nnzPf = w->nnzPf;
  v.use_grid = w->use_grid; v.grid_blocks = w->grid_blocks;
  grid_sync_args(w, v.gs);
  v.stream = w->stream;
  v.h_st = w->h_st;
  return v;
}

