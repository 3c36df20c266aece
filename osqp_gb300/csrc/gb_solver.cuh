// gb_solver.cuh -- the OSQP algorithm as group-generic device code.
//
// One OSQP problem is solved by a "group" (gb_common.cuh): a CTA for batched
// or small problems, a cooperative persistent grid for a large one.  All
// phases -- Ruiz scaling, rho vector, Jacobi preconditioner, ADMM iterations
// with the reduced-KKT PCG, residual/termination evaluation, adaptive rho and
// the solution store -- run inside one kernel launch; the only host traffic is
// the launch and the final copy of the results.
//
// Reference behaviour restated here (file:line in the OSQP 1.0 sources):
//   scaling          src/scaling.c:48-164
//   rho vector       src/auxil.c:76-122, osqp_api.c:1412-1464
//   ADMM steps       src/auxil.c:136-229
//   reduced KKT PCG  algebra/cuda/lin_sys/indirect/cuda_pcg.cu:50-208,
//                    cuda_pcg_interface.cu:32-92,229-273
//   Jacobi           algebra/cuda/lin_sys/indirect/cuda_pcg.cu:211-285
//   update_info      src/auxil.c:231-458,676-762
//   termination      src/auxil.c:460-588,808-945
//   adaptive rho     src/auxil.c:14-74; osqp_api.c:776-889
//   solve loop       src/osqp_api.c:636-1038
//   store_solution   src/auxil.c:598-674
#pragma once

#include <type_traits>

#include "gb_common.cuh"
#include "gb_direct.cuh"

namespace gb {

// Status values (include/public/osqp_api_constants.h:28-40)
enum : int {
  ST_SOLVED = 1, ST_SOLVED_INACCURATE, ST_PRIMAL_INFEASIBLE, ST_PRIMAL_INFEASIBLE_INACCURATE,
  ST_DUAL_INFEASIBLE, ST_DUAL_INFEASIBLE_INACCURATE, ST_MAX_ITER_REACHED, ST_TIME_LIMIT_REACHED,
  ST_NON_CVX, ST_SIGINT, ST_UNSOLVED
};

constexpr double kRhoMin = 1e-06, kRhoMax = 1e06, kRhoTol = 1e-04, kRhoEqOverIneq = 1e03;
constexpr double kMinScaling = 1e-04, kMaxScaling = 1e+04;
constexpr double kCgTolMin = 1e-7;

// Solver settings as kernel-side plain values (OSQPSettings fields).
struct DevSettings {
  double rho, sigma, alpha;
  double eps_abs, eps_rel, eps_prim_inf, eps_dual_inf;
  double cg_tol_fraction, adaptive_rho_tolerance, adaptive_rho_fraction;
  double time_limit;      // seconds
  double infty;           // OSQP_INFTY of the build
  double zero_deadzone;   // OSQP_ZERO_DEADZONE of the build
  int scaling, rho_is_vec, max_iter, check_termination;
  int adaptive_rho, adaptive_rho_interval;
  int cg_max_iter, cg_tol_reduction, cg_precond;
  int scaled_termination, check_dualgap, warm_starting;
  // interrupt generation of this solve (> 0): the solve stops when its
  // cancel word holds this value; 0: no interrupts
  int cancel_gen;
  int profile;   // accumulate per-phase clock cycles of each solve (SolverScalars::prof)
};

// Per-problem scalar state.  Lives in global memory between launches; during
// a launch every CTA of the group keeps an identical copy in shared memory.
struct SolverScalars {
  double rho, rho_inv, c, cinv;
  double scaled_prim_res, scaled_dual_res;
  double eps_prev, reduction_factor;
  double obj_val, dual_obj_val, prim_res, dual_res, duality_gap;
  double rho_estimate, rel_kkt_error, primdual_int, last_rel_kkt;
  double xtPx, qtx, SC, scaled_dual_gap;
  // norms kept from the last update_info (termination and rho estimate)
  double nz_s, nAx_s, nz_u, nAx_u;          // ||z||, ||Ax|| (scaled / unscaled)
  double nq_s, nAty_s, nPx_s, nq_u, nAty_u, nPx_u;
  double dy_norm, dy_lhs, atdy_norm;        // primal infeasibility
  double dx_norm, dx_q, pdx_norm, recc_max; // dual infeasibility
  double elapsed;                           // seconds since solve start
  double rhs_norm;
  double pcg_rTy, pcg_rnorm, pcg_eps, pcg_alpha, pcg_beta;
  unsigned long long t_start;
  long long pcg_iters_total;
  int zero_pcg_iters;
  int status, iter, rho_updates, rho_updated;
  int err;
  int cancel;
  int p_parity;
  int kkt_fail;   // direct solver: the last factorisation met a non-positive pivot
  // DevSettings::profile: SM clock cycles of the last solve, thread 0's view,
  // per phase: 0 right-hand side, 1 linear solve, 2 x / z / y updates,
  // 3 residuals and termination, 4 refactorisation / preconditioner refresh;
  // of the direct solve: 5 waits for factor segments, 6 block-step barriers,
  // 7 forward sweep, 8 backward sweep; 9 the sparse product of the
  // right-hand side, 10 the sparse product of the updates; 11 issuing the
  // direct solve's bulk copies (the issuing thread's view); counts of direct
  // solves: 12 all, 13 through the bulk-copy ring, 14 that read the factor
  // from global memory after a failed wait
  unsigned long long prof[kProfSlots];
};

template <typename T>
struct DevProblem {
  int n, m;
  CSR<T> P;    // full symmetric P (n x n), explicit diagonal
  CSR<T> A;    // A (m x n)
  CSR<T> At;   // A' (n x m) = CSC arrays of A
  const int* Pdiag;       // position of P(i,i) in P.val
  const int* Psrc;        // P.val[k] = Praw[Psrc[k]] (or 0 if Psrc[k] < 0)
  const int* Asrc;        // A.val[k] = Araw[Asrc[k]]
  const T* Praw;          // upper-triangular CSC values as given
  const T* Araw;          // CSC values of A as given
  T *q, *l, *u;           // scaled problem vectors
  const T *q_in, *l_in, *u_in;  // unscaled inputs (setup only)
  T *D, *Dinv, *E, *Einv;
  T *rho_vec, *rho_inv_vec;
  int* ctype;
  T *x, *z, *y, *dx, *dy;
  T *xp, *r, *p0, *p1, *Kp, *yv, *rhs, *t, *Minv;
  T *xo, *yo, *pcert, *dcert;   // stored solution (unscaled)
  T *Dt, *Et;                   // scaling scratch
  SolverScalars* st;            // persistent scalars
  // Block-Jacobi preconditioner (cg_precond = 2): the inverted 32 x 32
  // diagonal blocks of K (nullptr when not allocated), and A's CSR arrays in
  // global memory, which shared-memory staging never redirects
  T* Binv;
  const int *Arow_g, *Acol_g;
  const T* Aval_g;
  // Direct KKT solve (linsys_solver = direct; kkt.nb == 0 otherwise): the
  // block-tridiagonal factor and its plan (gb_direct.cuh), and the CTA's
  // on-chip workspace for it (set by the kernel)
  KktView<T> kkt;
  T* kws = nullptr;
  KktPipe* kpipe = nullptr;   // bulk-copy pipeline state of the CTA (static shared memory)
};

// ---------------------------------------------------------------------------
// Block-Jacobi preconditioner (cg_precond = 2).  The reference's PCG has the
// diagonal one only (cuda_pcg.cu:211-266); this is the block form of it.  M
// is the block diagonal of K = P + sigma I + A' R A with 32-variable blocks
// [32 b, 32 b + 32) (the last one shorter when 32 does not divide n).  Block
// b of M^-1 is stored at Binv + 1024 b, entry (j, i) at 32 j + i: the inverse
// is symmetric, so the lanes of a warp applying it read one row with one
// coalesced load per column.
// ---------------------------------------------------------------------------
constexpr int kPrecondBlock = 32;
enum : int { kPrecondNone = 0, kPrecondDiagonal = 1, kPrecondBlockDiagonal = 2 };

// Elements of M^-1 storage for n variables.
__host__ __device__ inline size_t block_precond_elems(long long n) {
  return (size_t)((n + kPrecondBlock - 1) / kPrecondBlock) * kPrecondBlock * kPrecondBlock;
}

// Block b of M^-1, computed by one whole warp (b warp-uniform).  Lane i forms
// row i of the block of K in FP64 (P entries, then the A' R A terms in
// ascending constraint order, then sigma on the diagonal), then the warp
// inverts the block in place by symmetric Gauss-Jordan sweeps (the sweep
// operator; sweeping every pivot leaves -K^-1):
//   d = 1 / a_kk;  a_ij -= (a_ik a_kj) d  (i, j != k);  a_ik = a_ik d;  a_kk = -d
// with row k broadcast by shuffles.  Each product is formed alike for (i, j)
// and (j, i), so the block stays symmetric.  A pivot that is not positive and
// finite (a block that is not numerically positive definite) leaves the
// whole block diagonal, 1 / K_ii, as the Jacobi preconditioner would.
// P and A' rows of the block are read through their (possibly staged) CSR;
// rows of A through the global arrays, any of which a block may touch.
template <typename T>
__device__ __noinline__ void kkt_block_inverse(CSR<T> P, CSR<T> At, const int* Arow, const int* Acol, const T* Aval,
                                               const T* rho_vec, T* Binv, int n, int b, double sig, double rho) {
  const int lane = threadIdx.x & 31;
  const int i0 = b * kPrecondBlock, nb = min(kPrecondBlock, n - i0);
  const int i = i0 + lane;
  double a[kPrecondBlock];
#pragma unroll
  for (int j = 0; j < kPrecondBlock; j++) a[j] = (j == lane) ? 1.0 : 0.0;   // padding rows: identity
  if (lane < nb) {
#pragma unroll
    for (int j = 0; j < kPrecondBlock; j++) a[j] = 0.0;
    const int* col; const T* val; int kb, ke;
    row_ptrs(P, i, true, col, val, kb, ke);
    for (int k = kb; k < ke; k++) {
      const int c = col[k] - i0;
      const double v = (double)val[k];
#pragma unroll
      for (int j = 0; j < kPrecondBlock; j++) if (j == c) a[j] += v;
    }
    row_ptrs(At, i, true, col, val, kb, ke);
    for (int e = kb; e < ke; e++) {
      const int k = col[e];
      const double aki = (double)val[e];
      const double rk = rho_vec ? (double)rho_vec[k] : rho;
      // entries of row k of A in columns [i0, i0 + nb): first one by bisection
      int lo = Arow[k], hi = Arow[k + 1];
      const int end = hi;
      while (lo < hi) { const int mid = (lo + hi) >> 1; if (Acol[mid] < i0) lo = mid + 1; else hi = mid; }
      for (int f = lo; f < end; f++) {
        const int c = Acol[f] - i0;
        if (c >= nb) break;
        const double w = rk * (aki * (double)Aval[f]);
#pragma unroll
        for (int j = 0; j < kPrecondBlock; j++) if (j == c) a[j] += w;
      }
    }
#pragma unroll
    for (int j = 0; j < kPrecondBlock; j++) if (j == lane) a[j] += sig;
  }
  double d0 = 1.0;   // K_ii
#pragma unroll
  for (int j = 0; j < kPrecondBlock; j++) if (j == lane) d0 = a[j];
  bool ok = true;
  for (int k = 0; k < nb; k++) {
    double aik = 0.0;
#pragma unroll
    for (int j = 0; j < kPrecondBlock; j++) if (j == k) aik = a[j];
    const double piv = __shfl_sync(0xffffffffu, aik, k);
    if (!(piv > 0.0) || !isfinite(piv)) { ok = false; break; }   // warp-uniform
    const double d = 1.0 / piv;
#pragma unroll
    for (int j = 0; j < kPrecondBlock; j++) {
      const double akj = __shfl_sync(0xffffffffu, a[j], k);
      if (j == k) a[j] = (lane == k) ? -d : aik * d;
      else a[j] = (lane == k) ? akj * d : a[j] - (aik * akj) * d;
    }
  }
  // padding rows and columns (past n) are stored as zeros
  T* Bb = Binv + (size_t)b * kPrecondBlock * kPrecondBlock;
#pragma unroll
  for (int j = 0; j < kPrecondBlock; j++)
    Bb[j * kPrecondBlock + lane] = (lane >= nb || j >= nb) ? T(0)
                                   : ok ? (T)(-a[j]) : (j == lane ? (T)(1.0 / d0) : T(0));
}

// (M^-1 r)_i for the block holding i; r must hold the whole block.  Fixed
// summation order (ascending j), whatever thread computes it.
template <typename T>
__device__ __forceinline__ T block_apply(const T* __restrict__ Binv, const T* r, int n, int i) {
  const int b0 = i & ~(kPrecondBlock - 1), li = i & (kPrecondBlock - 1);
  const T* Bb = Binv + (size_t)b0 * kPrecondBlock;
  const int nb = min(kPrecondBlock, n - b0);
  T acc = T(0);
#pragma unroll 8
  for (int j = 0; j < nb; j++) acc = fma(Bb[j * kPrecondBlock + li], r[b0 + j], acc);
  return acc;
}

// The block build as its own launch (preconditioner refreshes the host
// drives: rho and settings updates): one warp per block.
constexpr int kBlockPrecondThreads = 256;
template <typename T>
__global__ void __launch_bounds__(kBlockPrecondThreads) k_block_precond(DevProblem<T> pr, double sigma, double rho,
                                                                        int rho_is_vec) {
  const int nblk = (pr.n + kPrecondBlock - 1) / kPrecondBlock;
  const int w = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5), nw = (int)((gridDim.x * blockDim.x) >> 5);
  for (int b = w; b < nblk; b += nw)
    kkt_block_inverse<T>(pr.P, pr.At, pr.Arow_g, pr.Acol_g, pr.Aval_g, rho_is_vec ? pr.rho_vec : nullptr, pr.Binv,
                         pr.n, b, sigma, rho);
}
inline int block_precond_grid(int n) {
  const long long warps = (n + kPrecondBlock - 1) / kPrecondBlock;
  const long long blocks = (warps * 32 + kBlockPrecondThreads - 1) / kBlockPrecondThreads;
  return (int)(blocks < 1 ? 1 : (blocks > 4096 ? 4096 : blocks));
}

template <typename T> __device__ __forceinline__ T tmin(T a, T b) { return a < b ? a : b; }
template <typename T> __device__ __forceinline__ T tmax(T a, T b) { return a > b ? a : b; }
__device__ __forceinline__ double dlimit_scaling(double v) {
  v = v < kMinScaling ? 1.0 : v;
  return v > kMaxScaling ? kMaxScaling : v;
}
template <typename T> __device__ __forceinline__ T tnan() { return T(NAN); }

// P and A' share the row index space 0..n-1; one sub-warp handles row i of
// both so the reduced-KKT product needs a single pass.
template <int L, typename T, typename G, typename XP, typename XA, typename FN>
__device__ __forceinline__ void kkt_rows_L(G& g, const CSR<T>& P, const CSR<T>& At, XP xp, XA xa, FN fn) {
  const int lane = threadIdx.x & 31;
  const int sub = lane / L, sl = lane % L;
  constexpr int RPW = 32 / L;
  const Rng rg = span_n(g, P.rows);
  const int n = rg.hi;
  const int step = g.ws() * RPW;
  constexpr int NR = kRowsInFlight;
  // several rows per lane group at a time (gb_common.cuh lane_rows_dot);
  // each row's P and A' sums keep their lane and order
  for (int base = rg.lo + g.w0() * RPW; base < n; base += NR * step) {
    const int* pc[NR]; const T* pv[NR]; int pb[NR], pe[NR];
    const int* ac[NR]; const T* av[NR]; int ab[NR], ae[NR];
    T ps[NR], as[NR];
#pragma unroll
    for (int r = 0; r < NR; r++) {
      const int i = base + r * step + sub;
      row_ptrs(P, i, i < n, pc[r], pv[r], pb[r], pe[r]);
      row_ptrs(At, i, i < n, ac[r], av[r], ab[r], ae[r]);
      ps[r] = T(0); as[r] = T(0);
    }
    if (P.diag) {
      // diagonal P: the row's one entry times x_i on the row's first lane
      // (the sub-warp sum below adds zeros, so the value is the same)
#pragma unroll
      for (int r = 0; r < NR; r++)
        if (sl == 0 && pb[r] < pe[r]) ps[r] = pv[r][pb[r]] * xp(base + r * step + sub);
    } else {
      lane_rows_dot<L, NR>(pc, pv, pb, pe, sl, xp, ps);
    }
    lane_rows_dot<L, NR>(ac, av, ab, ae, sl, xa, as);
#pragma unroll
    for (int r = 0; r < NR; r++) {
      const T p1 = subwarp_sum<L>(ps[r]), a1 = subwarp_sum<L>(as[r]);
      const int i = base + r * step + sub;
      if (i < n && sl == 0) fn(i, p1, a1);
    }
  }
}
template <typename T, typename G, typename XP, typename XA, typename FN>
__device__ __forceinline__ void kkt_rows(G& g, int L, const CSR<T>& P, const CSR<T>& At, XP xp, XA xa, FN fn) {
  switch (L) {
    case 1:  kkt_rows_L<1>(g, P, At, xp, xa, fn); break;
    case 2:  kkt_rows_L<2>(g, P, At, xp, xa, fn); break;
    case 4:  kkt_rows_L<4>(g, P, At, xp, xa, fn); break;
    case 8:  kkt_rows_L<8>(g, P, At, xp, xa, fn); break;
    case 16: kkt_rows_L<16>(g, P, At, xp, xa, fn); break;
    default: kkt_rows_L<32>(g, P, At, xp, xa, fn); break;
  }
}

template <typename T>
struct Solver {
  DevProblem<T> pr;
  DevSettings s;
  SolverScalars* sc;  // shared-memory copy
  int kktL;           // lanes per row for the P / A' pair

  __device__ bool unscaled_term() const { return s.scaling && !s.scaled_termination; }
  __device__ double rho_of(int j) const { return s.rho_is_vec ? (double)pr.rho_vec[j] : sc->rho; }

  // ---------------------------------------------------------------------
  // Setup: data from the raw inputs, Ruiz scaling, rho, preconditioner.
  // ---------------------------------------------------------------------
  template <typename G>
  __device__ bool load_values(G& g) {
    // row pointers hold absolute positions (a QP of a batch is a slice)
    for_range(g, pr.P.rowptr[0], pr.P.rowptr[pr.n], [&](int k) { int s0 = pr.Psrc[k]; pr.P.val[k] = s0 >= 0 ? pr.Praw[s0] : T(0); });
    if (pr.m) for_range(g, pr.A.rowptr[0], pr.A.rowptr[pr.m], [&](int k) { pr.A.val[k] = pr.Araw[pr.Asrc[k]]; });
    for_range(g, pr.At.rowptr[0], pr.At.rowptr[pr.n], [&](int k) { pr.At.val[k] = pr.Araw[k]; });
    for_each(g, pr.n, [&](int i) { pr.q[i] = pr.q_in[i]; pr.D[i] = T(1); pr.Dinv[i] = T(1); });
    for_each(g, pr.m, [&](int j) { pr.l[j] = pr.l_in[j]; pr.u[j] = pr.u_in[j]; pr.E[j] = T(1); pr.Einv[j] = T(1); });
    return g.sync();
  }

  template <typename G>
  __device__ bool scale_data(G& g) {
    const int n = pr.n, m = pr.m;
    if (threadIdx.x == 0) sc->c = 1.0;
    for (int pass = 0; pass < s.scaling; pass++) {
      // column inf-norms of [P; A] (rows of symmetric P and of A') and row
      // inf-norms of A, limited, square-rooted and inverted (scaling.c:84-101)
      rows_norm_pair(g);
      for_each(g, m, [&](int j) {
        T a = T(0);
        for (int k = pr.A.rowptr[j]; k < pr.A.rowptr[j + 1]; k++) a = tmax(a, (T)fabs((double)pr.A.val[k]));
        pr.Et[j] = T(1) / (T)sqrt((double)(T)dlimit_scaling((double)a));
      });
      if (!g.sync()) return false;
      // P <- D P D ; A <- E A D ; A' likewise ; q <- D q (scaling.c:103-117)
      for_each_row_entries(g);
      for_each(g, n, [&](int i) { pr.q[i] *= pr.Dt[i]; pr.D[i] *= pr.Dt[i]; });
      for_each(g, m, [&](int j) { pr.E[j] *= pr.Et[j]; });
      if (!g.sync()) return false;
      // cost scaling (scaling.c:119-146)
      Acc<T> sm[1];
      T mx[1] = {T(0)};
      for_each(g, n, [&](int i) {
        T a = T(0);
        for (int k = pr.P.rowptr[i]; k < pr.P.rowptr[i + 1]; k++) a = tmax(a, (T)fabs(pr.P.val[k]));
        sm[0].add(a);
        mx[0] = tmax(mx[0], (T)fabs(pr.q[i]));
      });
      double rs[1], rm[1];
      g.reduce(sm, mx, rs, rm);
      if (!g.ok()) return false;
      double ct = rs[0] / n;
      double nq = dlimit_scaling(rm[0]);
      ct = dlimit_scaling(fmax(ct, nq));
      ct = 1.0 / ct;
      const T ctt = (T)ct;
      for_range(g, pr.P.rowptr[0], pr.P.rowptr[n], [&](int k) { pr.P.val[k] *= ctt; });
      for_each(g, n, [&](int i) { pr.q[i] *= ctt; });
      if (threadIdx.x == 0) sc->c *= ct;
      if (!g.sync()) return false;
    }
    if (threadIdx.x == 0) sc->cinv = 1.0 / sc->c;
    for_each(g, n, [&](int i) { pr.Dinv[i] = T(1) / pr.D[i]; });
    for_each(g, m, [&](int j) {
      pr.Einv[j] = T(1) / pr.E[j];
      pr.l[j] *= pr.E[j];
      pr.u[j] *= pr.E[j];
    });
    return g.sync();
  }

  // Column norms of [P; A] for rows i (P symmetric, A' rows): Dt[i]
  template <typename G>
  __device__ void rows_norm_pair(G& g) {
    for_each(g, pr.n, [&](int i) {
      T a = T(0);
      for (int k = pr.P.rowptr[i]; k < pr.P.rowptr[i + 1]; k++) a = tmax(a, (T)fabs((double)pr.P.val[k]));
      T b = T(0);
      for (int k = pr.At.rowptr[i]; k < pr.At.rowptr[i + 1]; k++) b = tmax(b, (T)fabs((double)pr.At.val[k]));
      a = tmax(a, b);
      pr.Dt[i] = T(1) / (T)sqrt((double)(T)dlimit_scaling((double)a));
    });
  }

  template <typename G>
  __device__ void for_each_row_entries(G& g) {
    for_each(g, pr.n, [&](int i) {
      const T di = pr.Dt[i];
      // D_i * D_j is commutative, so the stored full P stays exactly symmetric
      for (int k = pr.P.rowptr[i]; k < pr.P.rowptr[i + 1]; k++) pr.P.val[k] = pr.P.val[k] * (di * pr.Dt[pr.P.col[k]]);
      for (int k = pr.At.rowptr[i]; k < pr.At.rowptr[i + 1]; k++) pr.At.val[k] = (pr.At.val[k] * pr.Et[pr.At.col[k]]) * di;
    });
    for_each(g, pr.m, [&](int j) {
      const T ej = pr.Et[j];
      for (int k = pr.A.rowptr[j]; k < pr.A.rowptr[j + 1]; k++) pr.A.val[k] = (pr.A.val[k] * ej) * pr.Dt[pr.A.col[k]];
    });
  }

  // rho vector from constraint types (auxil.c:76-104)
  // changed (optional): set when a constraint type differs from the stored one
  template <typename G>
  __device__ void set_rho_vec(G& g, int* changed = nullptr) {
    const double infval = s.infty * kMinScaling;
    const double rho = sc->rho;
    for_m(g, pr.m, [&](int j) {
      const double l = pr.l[j], u = pr.u[j];
      int t;
      if (l < -infval && u > infval) t = -1;
      else if (u - l < kRhoTol) t = 1;
      else t = 0;
      if (changed && pr.ctype[j] != t) *changed = 1;
      pr.ctype[j] = t;
      const double rv = t < 0 ? kRhoMin : (t == 0 ? rho : kRhoEqOverIneq * rho);
      g.put(pr.rho_vec, j, (T)rv);
      pr.rho_inv_vec[j] = T(1) / (T)rv;
    });
  }
  template <typename G>
  __device__ void refresh_rho_vec(G& g) {
    const DevProblem<T> pr = this->pr;
    SolverScalars* const sc = this->sc;
    const double rho = sc->rho;
    for_m(g, pr.m, [&](int j) {
      const int t = pr.ctype[j];
      const double rv = t < 0 ? kRhoMin : (t == 0 ? rho : kRhoEqOverIneq * rho);
      g.put(pr.rho_vec, j, (T)rv);
      pr.rho_inv_vec[j] = T(1) / (T)rv;
    });
  }

  // Jacobi preconditioner M = sigma + diag(P) + diag(A' R A) (cuda_pcg.cu:211-266),
  // and with cg_precond = 2 the inverted blocks of the block-Jacobi one
  template <typename G>
  __device__ void update_precond(G& g) {
    if (kkt_direct(pr.kkt)) { direct_factor(g); return; }
    // local copies: hot loops keep the pointers in registers instead of
    // re-reading them through `this` after every store
    const DevProblem<T> pr = this->pr;
    const DevSettings s = this->s;
    SolverScalars* const sc = this->sc;
    const T sig = (T)s.sigma;
    const bool vec = s.rho_is_vec;
    const T rho = (T)sc->rho;
    for_n(g, pr.n, [&](int i) {
      if (s.cg_precond == 0) { pr.Minv[i] = T(1); return; }
      T d = T(0);
      for (int k = pr.At.rowptr[i]; k < pr.At.rowptr[i + 1]; k++) {
        const T a = pr.At.val[k];
        d += vec ? a * a * pr.rho_vec[pr.At.col[k]] : a * a;
      }
      if (!vec) d *= rho;
      pr.Minv[i] = T(1) / (sig + pr.P.val[pr.Pdiag[i]] + d);
    });
    if (s.cg_precond == kPrecondBlockDiagonal && pr.Binv) {
      // one warp per block, over the blocks of this CTA's part of the n-space
      // (a sliced cluster's spans start on block boundaries)
      const Rng rg = span_n(g, pr.n);
      const int b_lo = rg.lo / kPrecondBlock, b_hi = (rg.hi + kPrecondBlock - 1) / kPrecondBlock;
      for (int b = b_lo + g.w0(); b < b_hi; b += g.ws())
        kkt_block_inverse<T>(pr.P, pr.At, pr.Arow_g, pr.Acol_g, pr.Aval_g, vec ? pr.rho_vec : nullptr, pr.Binv,
                             pr.n, b, s.sigma, sc->rho);
    }
  }

  // Direct solver: factor K = P + sigma I + A' R A for the current rho
  // (gb_direct.cuh).  Only the CTA form holds a plan; sc->kkt_fail records a
  // non-positive pivot.
  template <typename G>
  __device__ void direct_factor(G& g) {
    if constexpr (std::is_same<G, BlockGroup>::value) {
      const T* rv = s.rho_is_vec ? pr.rho_vec : nullptr;
      const bool ok = pr.kkt.dr > 0
                          ? dr_factor<T>(pr.kkt, pr.n, pr.P, pr.A, pr.At, rv, (T)sc->rho, (T)s.sigma, pr.kws)
                          : kkt_factor<T>(pr.kkt, pr.P, pr.A, pr.At, rv, (T)sc->rho, (T)s.sigma, pr.kws);
      if (threadIdx.x == 0) sc->kkt_fail = ok ? 0 : 1;
      __syncthreads();
    }
  }

  // Diagonal-plus-dense-rows solve (gb_kkt_plan.h), in the saddle-point form
  // of the builtin's KKT system restricted to the dense rows: with b_s the
  // right-hand side without the dense rows' terms (kc on entry),
  //   nu = C^-1 (A_d Dg^-1 b_s - (z_d - R_d^-1 y_d)),   x~ = Dg^-1 (b_s - A_d' nu),
  // which equals K^-1 (b_s + A_d'(R_d z_d - y_d)) without forming that
  // right-hand side: its rho-weighted dense-row terms would cancel in x~ and
  // cost FP32 most of its digits.  The three products accumulate in
  // double-float (FP32 build) and carry t and nu as (hi, lo) pairs, since a
  // dense row sums many entries whose total nearly cancels.  kc becomes
  // Dg^-1 b_s; x~ goes to kxs; tv: 4 r elements of on-chip scratch.  One warp
  // per dense row for A_d u and C^-1 t, one warp per variable for A_d' nu
  // (fixed lane order).
  template <typename G>
  __device__ void dr_solve(G& g, int n, T* kc, T* kxs, T* tv) {
    const KktView<T>& kv = pr.kkt;
    const bool vec = s.rho_is_vec;
    const double rinv_s = sc->rho_inv;
    const int r = kv.dr;
    T* th = tv;
    T* tl = tv + r;
    T* nh = tv + 2 * r;
    T* nl = tv + 3 * r;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for_n(g, n, [&](int i) { kc[i] = kc[i] * kv.Dginv[i]; });
    __syncthreads();
    for (int a = warp; a < r; a += nw) {
      const int ra = kv.drows[a];
      Acc<T> acc;
      for (int e = pr.A.rowptr[ra] + lane; e < pr.A.rowptr[ra + 1]; e += 32) acc.add_prod(pr.A.val[e], kc[pr.A.col[e]]);
      warp_accT(acc);
      if (lane == 0) {
        const double ri = vec ? (double)pr.rho_inv_vec[ra] : rinv_s;
        const double t = acc.value() - ((double)pr.z[ra] - ri * (double)pr.y[ra]);
        th[a] = (T)t;
        tl[a] = (T)(t - (double)th[a]);
      }
    }
    __syncthreads();
    for (int a = warp; a < r; a += nw) {
      const T* row = kv.Cinv + (size_t)a * r;
      Acc<T> acc;
      for (int b = lane; b < r; b += 32) { acc.add_prod(row[b], th[b]); acc.add_prod(row[b], tl[b]); }
      warp_accT(acc);
      if (lane == 0) {
        const double v = acc.value();
        nh[a] = (T)v;
        nl[a] = (T)(v - (double)nh[a]);
      }
    }
    __syncthreads();
    const Rng rg = span_n(g, n);
    for (int i = rg.lo + warp; i < rg.hi; i += nw) {
      Acc<T> acc;
      for (int e = pr.At.rowptr[i] + lane; e < pr.At.rowptr[i + 1]; e += 32) {
        const int d = kv.didx[pr.At.col[e]];
        if (d >= 0) { acc.add_prod(pr.At.val[e], nh[d]); acc.add_prod(pr.At.val[e], nl[d]); }
      }
      warp_accT(acc);
      if (lane == 0) kxs[i] = (T)((double)kc[i] - (double)kv.Dginv[i] * acc.value());
    }
    __syncthreads();
  }

  template <typename G>
  __device__ void cold_start(G& g) {
    for_n(g, pr.n, [&](int i) { pr.x[i] = T(0); g.put(pr.xp, i, T(0)); });
    for_m(g, pr.m, [&](int j) { pr.z[j] = T(0); pr.y[j] = T(0); });
  }

  // Values, scaling, rho vector and preconditioner.  keep = true is the matrix
  // update path (osqp_api.c:1309-1409): rho and the iterates are kept.
  template <typename G>
  __device__ bool prepare_data(G& g, bool keep) {
    if (!load_values(g)) return false;
    if (s.scaling) { if (!scale_data(g)) return false; }
    else if (threadIdx.x == 0) { sc->c = 1.0; sc->cinv = 1.0; }
    if (!keep && s.rho_is_vec) set_rho_vec(g);
    if (!g.sync()) return false;
    update_precond(g);
    return g.sync();
  }

  // Whole setup: values, scaling, rho, preconditioner, cold start.
  template <typename G>
  __device__ bool setup(G& g) {
    if (threadIdx.x == 0) {
      sc->c = 1.0; sc->cinv = 1.0;
      sc->rho = fmin(fmax(s.rho, kRhoMin), kRhoMax);
      sc->rho_inv = 1.0 / sc->rho;
      sc->rho_updates = 0; sc->status = ST_UNSOLVED; sc->iter = 0;
      sc->scaled_prim_res = 0.0; sc->scaled_dual_res = 0.0;
      sc->obj_val = s.infty; sc->prim_res = s.infty; sc->dual_res = s.infty;
      sc->rel_kkt_error = s.infty; sc->last_rel_kkt = s.infty;
      sc->rho_estimate = sc->rho; sc->primdual_int = 0.0;
      sc->zero_pcg_iters = 0; sc->reduction_factor = s.cg_tol_fraction; sc->eps_prev = 1.0;
      sc->err = 0; sc->p_parity = 0; sc->pcg_iters_total = 0; sc->cancel = 0; sc->kkt_fail = 0;
    }
    __syncthreads();
    if (!prepare_data(g, false)) return false;
    if (threadIdx.x == 0 && kkt_direct(pr.kkt) && sc->kkt_fail) sc->status = ST_NON_CVX;
    cold_start(g);
    return g.sync();
  }

  // ---------------------------------------------------------------------
  // One ADMM iteration (auxil.c:136-229) with the PCG solve in between.
  // ---------------------------------------------------------------------
  template <typename G>
  __device__ bool admm_iteration(G& g, int iter) {
    // local copies: hot loops keep the pointers in registers instead of
    // re-reading them through `this` after every store
    const DevProblem<T> pr = this->pr;
    const DevSettings s = this->s;
    SolverScalars* const sc = this->sc;
    const int n = pr.n, m = pr.m;
    const bool vec = s.rho_is_vec;
    const T sig = (T)s.sigma;
    const T rho_s = (T)sc->rho, rinv_s = (T)sc->rho_inv;
    T* __restrict__ x = pr.x; T* __restrict__ z = pr.z; T* __restrict__ y = pr.y;
    T* __restrict__ xp = pr.xp;
    const bool direct = kkt_direct(pr.kkt);
    T* const kc = pr.kws;            // direct: permuted right-hand side
    const bool prof = s.profile && threadIdx.x == 0;
    long long pt = prof ? clock64() : 0;
    const int* const kip = pr.kkt.iperm;
    // direct: on-chip copies of the vectors the sparse products gather,
    // x~ and w = rho z - y (after the block solve's vectors and ring)
    T* const kxs = direct ? kc + kkt_pad4(2LL * n) + (long long)pr.kkt.ring * pr.kkt.segmax : nullptr;
    T* const kw = direct ? kxs + kkt_pad4(n) : nullptr;

    // Phase R: rhs = (sigma x - q) + A'(rho .* (z - rho^-1 y)) and, for the
    // PCG, t = rho .* (A xp)
    Acc<T> sm0[1];
    T mx0[3] = {T(0), T(-INFINITY), T(-INFINITY)};
    if (direct) {
      // w = rho .* z - y (one rounding) on chip, so the product gathers from shared memory
      for_m(g, m, [&](int j) { kw[j] = fma(vec ? pr.rho_vec[j] : rho_s, z[j], -y[j]); });
      __syncthreads();
    }
    if (prof) { const long long t = clock64(); sc->prof[0] += (unsigned long long)(t - pt); pt = t; }
    // the dense-row form leaves its dense rows out of the right-hand side (they
    // enter its solve through z - rho^-1 y, dr_solve)
    const int* const ddx = pr.kkt.dr > 0 ? pr.kkt.didx : nullptr;
    // the vectors as locals (not reloaded from the problem struct per row)
    const T* const qv = pr.q;
    const T* const rv = pr.rho_vec;
    const T* const riv = pr.rho_inv_vec;
    T* const rhsv = pr.rhs;
    rows_auto(g, span_n(g, n), pr.At,
      [&](int j) {
        if (direct) return (ddx && ddx[j] >= 0) ? T(0) : kw[j];
        const T rj = vec ? rv[j] : rho_s;
        const T ij = vec ? riv[j] : rinv_s;
        return rj * (z[j] - ij * y[j]);
      },
      [&](int i, T v) {
        const T b1 = sig * x[i] - qv[i];
        const T rr = b1 + v;
        if (direct) {
          // the block form's solve vector (double-float in the FP64 build);
          // the dense-row form reads plain values
          if (ddx) kc[kip ? kip[i] : i] = rr;
          else kkt_vput(kc, n, kip ? kip[i] : i, rr);
        } else {
          rhsv[i] = rr;
          mx0[0] = tmax(mx0[0], (T)fabs(rr));   // the PCG's tolerance only
        }
      });
    if (m > 0 && !direct) {
      rows_rng(g, span_m(g, m), pr.A, [&](int c) { return xp[c]; },
        [&](int j, T v) { g.put(pr.t, j, (vec ? pr.rho_vec[j] : rho_s) * v); });
    }
    if (prof) { const long long t = clock64(); sc->prof[9] += (unsigned long long)(t - pt); pt = t; }
    double rhs_norm = 0.0, elapsed = 0.0;
    int cancel = 0;
    if (direct && std::is_same<G, BlockGroup>::value) {
      // one CTA: thread 0, the only reader of the time and the cancel word,
      // reads them itself; the barrier completes the right-hand side
      if (threadIdx.x == 0) {
        elapsed = (double)(T)((double)(global_ns() - sc->t_start) * 1e-9);
        const int cw = *((volatile int*)&pr.st->cancel);
        cancel = s.cancel_gen > 0 && cw == s.cancel_gen;
      }
      __syncthreads();
    } else {
      // time / cancellation ride on this reduction so every CTA sees the same values
      if (g.tid() == 0) {
        mx0[1] = (T)((double)(global_ns() - sc->t_start) * 1e-9);
        const int cw = *((volatile int*)&pr.st->cancel);
        mx0[2] = (s.cancel_gen > 0 && cw == s.cancel_gen) ? T(1) : T(0);
      }
      double rs0[1], rm0[3];
      g.reduce(sm0, mx0, rs0, rm0);
      if (!g.ok()) return false;
      rhs_norm = rm0[0];
      elapsed = rm0[1];
      cancel = rm0[2] > 0.0;
    }
    if (prof) { const long long t = clock64(); sc->prof[0] += (unsigned long long)(t - pt); pt = t; }

    // PCG tolerance (cuda_pcg_interface.cu:32-64), computed once per CTA
    if (threadIdx.x == 0 && !direct) {
      double e;
      if (iter == 1) {
        sc->reduction_factor = s.cg_tol_fraction;
        sc->eps_prev = rhs_norm < kCgTolMin ? 1.0 : rhs_norm * sc->reduction_factor;
        e = sc->eps_prev;
      } else {
        if (sc->zero_pcg_iters >= s.cg_tol_reduction) {
          sc->reduction_factor /= 2;
          sc->zero_pcg_iters = 0;
        }
        e = sc->reduction_factor * sqrt(sc->scaled_prim_res * sc->scaled_dual_res);
        e = fmax(fmin(e, sc->eps_prev), kCgTolMin);
        sc->eps_prev = e;
      }
      sc->pcg_eps = e;
      sc->rhs_norm = rhs_norm;
    }
    __syncthreads();
    const double eps = sc->pcg_eps;

    if (direct) {
      // x~ = K^-1 rhs (gb_direct.cuh), kept on chip (kxs)
      if constexpr (std::is_same<G, BlockGroup>::value) {
       if (pr.kkt.dr > 0) {
        dr_solve(g, n, kc, kxs, kw + kkt_pad4(m));
       } else {
        const bool piped = pr.kkt.ring >= 2 && pr.kpipe;
        if (piped)
          kkt_solve_pipe<T>(pr.kkt, pr.kpipe, kc, kc + n, kc + kkt_pad4(2LL * n),
                            [kxs](int i, T v) { kxs[i] = v; }, prof ? sc->prof + 5 : nullptr,
                            s.profile ? sc->prof + 11 : nullptr, prof ? sc->prof + 15 : nullptr);
        else
          kkt_solve<T>(pr.kkt, kc, kc + n, [kxs](int i, T v) { kxs[i] = v; });
        if (prof) {
          sc->prof[12] += 1;
          if (piped) { sc->prof[13] += 1; if (pr.kpipe->err) sc->prof[14] += 1; }
        }
       }
      }
    } else {
      const int pcg_it = pcg_core(g, eps, sig, rho_s);
      if (pcg_it < 0) return false;
    }
    if (threadIdx.x == 0) {
      sc->elapsed = elapsed;
      sc->cancel = cancel;
    }
    if (prof) { const long long t = clock64(); sc->prof[1] += (unsigned long long)(t - pt); pt = t; }

    // Phase U: x~ = xp, z~ = A xp, then the x / z / y updates (auxil.c:172-229)
    const T al = (T)s.alpha, oma = (T)(1.0 - s.alpha);
    for_n(g, n, [&](int i) {
      const T xo = x[i];
      const T xn = al * (direct ? kxs[i] : xp[i]) + oma * xo;
      x[i] = xn;
      pr.dx[i] = xn - xo;
    });
    if (prof) { const long long t = clock64(); sc->prof[2] += (unsigned long long)(t - pt); pt = t; }
    if (m > 0) {
      // the vectors as locals (not reloaded from the problem struct per row)
      const T* const lv = pr.l;
      const T* const uv = pr.u;
      T* const dyv = pr.dy;
      rows_auto(g, span_m(g, m), pr.A, [&](int c) { return direct ? kxs[c] : xp[c]; }, [&](int j, T zt) {
        const T ri = vec ? riv[j] : rinv_s;
        const T rr = vec ? rv[j] : rho_s;
        const T zo = z[j];
        const T zr = al * zt + oma * zo;
        const T zz = zr + ri * y[j];
        const T zn = tmin(tmax(zz, lv[j]), uv[j]);
        const T d = rr * (zr - zn);
        z[j] = zn;
        dyv[j] = d;
        y[j] = y[j] + d;
      });
    }
    if (prof) { const long long t = clock64(); sc->prof[10] += (unsigned long long)(t - pt); pt = t; }
    __syncthreads();
    const bool ok = g.sync();
    if (prof) sc->prof[2] += (unsigned long long)(clock64() - pt);
    return ok;
  }


  // ---------------------------------------------------------------------
  // The PCG of pcg_core for the FP32 build on one CTA with one barrier per
  // reduction: every thread finishes each reduction (BlockGroup::reduce1) and
  // keeps rTy as a double-float pair; alpha = rTy / pKp and beta =
  // rTy_new / rTy are double-float quotients rounded to float (df_div), all on
  // the FP32 pipe.  The stopping test ||r|| > eps is exact: ||r|| is a float
  // and thr is the smallest float above eps.  Same recurrence and phases as
  // pcg_core; barriers per iteration: 4 instead of 6.
  // ---------------------------------------------------------------------
  template <bool BLK>
  __device__ int pcg_core_block32(BlockGroup& g, double eps, float sig, float rho_s) {
    const DevProblem<float> pr = this->pr;
    const DevSettings s = this->s;
    SolverScalars* const sc = this->sc;
    const int n = pr.n, m = pr.m;
    const bool vec = s.rho_is_vec && pr.rho_vec;
    const int cg_max = s.cg_max_iter;
    float* __restrict__ xp = pr.xp;
    float thr = (float)eps;                        // smallest float > eps
    if ((double)thr <= eps) thr = nextafterf(thr, INFINITY);
    int par = 0;
    // Phase I: r = K xp - rhs, yv = M^-1 r, p = -yv, rTy, ||r||
    float* p = sc->p_parity ? pr.p1 : pr.p0;
    // BLK (block-Jacobi): M^-1 r needs the whole block of r, so it is a
    // second pass after a barrier (one more barrier per iteration).  A
    // separate instantiation keeps the Jacobi loop's registers as they were.
    constexpr bool blk = BLK;
    Acc<float> rty;
    float rn = 0.f;
    kkt_rows(g, kktL, pr.P, pr.At, [&](int c) { return xp[c]; }, [&](int c) { return m ? pr.t[c] : 0.f; },
      [&](int i, float pv, float av) {
        const float kx = sig * xp[i] + pv + av;
        const float r = kx - pr.rhs[i];
        pr.r[i] = r;
        rn = tmax(rn, fabsf(r));
        if constexpr (!blk) {
          const float yv = pr.Minv[i] * r;
          pr.yv[i] = yv; p[i] = -yv;
          rty.add_prod(yv, r);
        }
      });
    if constexpr (blk) {
      __syncthreads();
      for_n(g, n, [&](int i) {
        const float yv = block_apply(pr.Binv, pr.r, n, i);
        pr.yv[i] = yv; p[i] = -yv;
        rty.add_prod(yv, pr.r[i]);
      });
    }
    g.reduce1(rty, rn, par);
    int it = 0;
    bool cont = rn >= thr && 0 < cg_max;
    while (cont) {
      // Phase A: t = rho .* (A p)
      if (m > 0) {
        rows_rng(g, span_m(g, m), pr.A, [&](int c) { return p[c]; },
                 [&](int j, float v) { pr.t[j] = (vec ? pr.rho_vec[j] : rho_s) * v; });
        __syncthreads();
      }
      // Phase B: Kp = sigma p + P p + A' t ; pKp
      Acc<float> pkp;
      float dummy = 0.f;
      kkt_rows(g, kktL, pr.P, pr.At, [&](int c) { return p[c]; }, [&](int c) { return m ? pr.t[c] : 0.f; },
        [&](int i, float pv, float av) {
          const float pi = p[i];
          const float kp = sig * pi + pv + av;
          pr.Kp[i] = kp;
          pkp.add_prod(pi, kp);
        });
      g.reduce1(pkp, dummy, par);
      const float at = df_div(rty.hi, rty.lo, pkp.hi, pkp.lo);
      // Phase C: x += alpha p ; r += alpha Kp ; yv = M^-1 r ; rTy ; ||r||
      Acc<float> rty_new;
      float rn2 = 0.f;
      for_n(g, n, [&](int i) {
        xp[i] = xp[i] + at * p[i];
        const float r = pr.r[i] + at * pr.Kp[i];
        pr.r[i] = r;
        rn2 = tmax(rn2, fabsf(r));
        if constexpr (!blk) {
          const float yv = pr.Minv[i] * r;
          pr.yv[i] = yv;
          rty_new.add_prod(yv, r);
        }
      });
      if constexpr (blk) {
        __syncthreads();
        for_n(g, n, [&](int i) {
          const float yv = block_apply(pr.Binv, pr.r, n, i);
          pr.yv[i] = yv;
          rty_new.add_prod(yv, pr.r[i]);
        });
      }
      g.reduce1(rty_new, rn2, par);
      const float bt = df_div(rty_new.hi, rty_new.lo, rty.hi, rty.lo);
      rty = rty_new;
      it++;
      cont = rn2 >= thr && it < cg_max;
      // Phase D: p = beta p - yv (skipped when the loop is about to end)
      if (cont) {
        for_n(g, n, [&](int i) { p[i] = bt * p[i] - pr.yv[i]; });
        __syncthreads();
      }
    }
    if (threadIdx.x == 0) {
      sc->pcg_iters_total += it;
      if (it == 0) sc->zero_pcg_iters++; else sc->zero_pcg_iters = 0;
    }
    __syncthreads();
    return it;
  }

  // ---------------------------------------------------------------------
  // PCG on the reduced KKT system K = P + sigma I + A' R A from the current
  // iterate xp and right-hand side rhs (cuda_pcg.cu:113-208): start-up
  // product r = K xp - rhs, then four phases per iteration.  t holds
  // R A p between phases.  Returns the iteration count, -1 on a barrier error.
  // ---------------------------------------------------------------------
  template <typename G>
  __device__ int pcg_core(G& g, double eps, T sig, T rho_s) {
    const bool blk = s.cg_precond == kPrecondBlockDiagonal && pr.Binv;
    if constexpr (std::is_same<T, float>::value && std::is_same<G, BlockGroup>::value)
      return blk ? pcg_core_block32<true>(g, eps, sig, rho_s) : pcg_core_block32<false>(g, eps, sig, rho_s);
    else
      return pcg_core_any(g, eps, sig, rho_s, blk);
  }
  template <typename G>
  __device__ int pcg_core_any(G& g, double eps, T sig, T rho_s, const bool blk) {
    // local copies: hot loops keep the pointers in registers instead of
    // re-reading them through `this` after every store
    const DevProblem<T> pr = this->pr;
    const DevSettings s = this->s;
    SolverScalars* const sc = this->sc;
    const int n = pr.n, m = pr.m;
    const bool vec = s.rho_is_vec && pr.rho_vec;
    const int cg_max = s.cg_max_iter;
    T* __restrict__ xp = pr.xp;
    // Scalar recurrences (rTy, alpha, beta, the stopping test) run in FP64 on
    // one thread inside each reduction; the other threads read the results
    // from shared memory: GB300's FP64 rate makes per-thread FP64 scalar
    // math cost more than a whole vector phase.
    GroupShared* gs = g.sh;
    T* bT = bcast_slots<T>(gs);   // [0] alpha  [1] beta
    // Phase I: r = K xp - rhs, yv = M^-1 r, p = -yv, rTy, ||r||
    T* pA = sc->p_parity ? pr.p1 : pr.p0;
    // blk (block-Jacobi): M^-1 r needs the whole block of r, so it is a
    // second pass after a group barrier (one more barrier per iteration)
    Acc<T> sm1[1];
    T mx1[1] = {T(0)};
    kkt_rows(g, kktL, pr.P, pr.At, [&](int c) { return xp[c]; }, [&](int c) { return m ? pr.t[c] : T(0); },
      [&](int i, T pv, T av) {
        const T kx = sig * xp[i] + pv + av;
        const T r = kx - pr.rhs[i];
        pr.r[i] = r;
        mx1[0] = tmax(mx1[0], (T)fabs(r));
        if (!blk) {
          const T yv = pr.Minv[i] * r;
          pr.yv[i] = yv; g.put(pA, i, -yv);
          sm1[0].add_prod(yv, r);
        }
      });
    if (blk) {
      if (!g.sync()) return -1;
      for_n(g, n, [&](int i) {
        const T yv = block_apply(pr.Binv, pr.r, n, i);
        pr.yv[i] = yv; g.put(pA, i, -yv);
        sm1[0].add_prod(yv, pr.r[i]);
      });
    }
    double rs1[1], rm1[1];
    // bd[0] = rTy, bi[0] = continue, bi[1] = iterations
    g.reduce(sm1, mx1, rs1, rm1, [&](const double* rsum, const double* rmax) {
      gs->bd[0] = rsum[0];
      gs->bi[1] = 0;
      gs->bi[0] = (rmax[0] > eps && 0 < cg_max) ? 1 : 0;
    });
    if (!g.ok()) return -1;

    // PCG loop (cuda_pcg.cu:155-200).  Four phases per iteration; each ends
    // at a group barrier (the two reductions carry theirs).
    T* p = pA;
    while (gs->bi[0]) {
      // Phase A: t = rho .* (A p)
      if (m > 0) {
        rows_rng(g, span_m(g, m), pr.A, [&](int c) { return p[c]; },
                 [&](int j, T v) { g.put(pr.t, j, (vec ? pr.rho_vec[j] : rho_s) * v); });
        if (!g.sync()) return -1;
      }
      // Phase B: Kp = sigma p + P p + A' t ; pKp
      Acc<T> sm2[1];
      T mx2[1] = {T(0)};
      kkt_rows(g, kktL, pr.P, pr.At, [&](int c) { return p[c]; }, [&](int c) { return m ? pr.t[c] : T(0); },
        [&](int i, T pv, T av) {
          const T pi = p[i];
          const T kp = sig * pi + pv + av;
          pr.Kp[i] = kp;
          sm2[0].add_prod(pi, kp);
        });
      double rs2[1], rm2[1];
      g.reduce(sm2, mx2, rs2, rm2, [&](const double* rsum, const double*) {
        bT[0] = (T)(gs->bd[0] / rsum[0]);
      });
      if (!g.ok()) return -1;
      const T at = bT[0];
      // Phase C: x += alpha p ; r += alpha Kp ; yv = M^-1 r ; rTy ; ||r||
      Acc<T> sm3[1];
      T mx3[1] = {T(0)};
      for_n(g, n, [&](int i) {
        g.put(xp, i, xp[i] + at * p[i]);
        const T r = pr.r[i] + at * pr.Kp[i];
        pr.r[i] = r;
        mx3[0] = tmax(mx3[0], (T)fabs(r));
        if (!blk) {
          const T yv = pr.Minv[i] * r;
          pr.yv[i] = yv;
          sm3[0].add_prod(yv, r);
        }
      });
      if (blk) {
        if (!g.sync()) return -1;
        for_n(g, n, [&](int i) {
          const T yv = block_apply(pr.Binv, pr.r, n, i);
          pr.yv[i] = yv;
          sm3[0].add_prod(yv, pr.r[i]);
        });
      }
      double rs3[1], rm3[1];
      g.reduce(sm3, mx3, rs3, rm3, [&](const double* rsum, const double* rmax) {
        const double rTy_new = rsum[0];
        bT[1] = (T)(rTy_new / gs->bd[0]);
        gs->bd[0] = rTy_new;
        const int it = gs->bi[1] + 1;
        gs->bi[1] = it;
        gs->bi[0] = (rmax[0] > eps && it < cg_max) ? 1 : 0;
      });
      if (!g.ok()) return -1;
      // Phase D: p = beta p - yv (skipped when the loop is about to end)
      if (gs->bi[0]) {
        const T bt = bT[1];
        for_n(g, n, [&](int i) { g.put(p, i, bt * p[i] - pr.yv[i]); });
        if (!g.sync()) return -1;
      }
    }
    const int it = gs->bi[1];
    if (threadIdx.x == 0) {
      sc->pcg_iters_total += it;
      if (it == 0) sc->zero_pcg_iters++; else sc->zero_pcg_iters = 0;
    }
    __syncthreads();
    return it;
  }


  // Reduced-KKT solve behind the linear-system interface (LinSysSolver.solve,
  // cuda_pcg_interface.cu:229-273): b = [b1; b2] in, [x~; A x~] out
  // (polishing: [x; (A x - b2) / delta]).  The CG tolerance follows
  // cuda_pcg_interface.cu:32-64 with the caller's scaled residuals.
  template <typename G>
  __device__ bool linsys_solve(G& g, T* b, int admm_iter, bool polishing, double spr, double sdr) {
    // local copies: hot loops keep the pointers in registers instead of
    // re-reading them through `this` after every store
    const DevProblem<T> pr = this->pr;
    const DevSettings s = this->s;
    SolverScalars* const sc = this->sc;
    const int n = pr.n, m = pr.m;
    const bool vec = s.rho_is_vec && pr.rho_vec;
    const T sig = (T)s.sigma;
    const T rho_s = (T)sc->rho;
    T* __restrict__ xp = pr.xp;
    const T* b1 = b;
    T* b2 = b + n;
    Acc<T> sm0[1];
    T mx0[1] = {T(0)};
    rows_rng(g, span_n(g, n), pr.At, [&](int j) { return (vec ? pr.rho_vec[j] : rho_s) * b2[j]; },
               [&](int i, T v) {
                 const T rr = b1[i] + v;
                 pr.rhs[i] = rr;
                 mx0[0] = tmax(mx0[0], (T)fabs(rr));
               });
    if (m > 0)
      rows_rng(g, span_m(g, m), pr.A, [&](int c) { return xp[c]; },
               [&](int j, T v) { g.put(pr.t, j, (vec ? pr.rho_vec[j] : rho_s) * v); });
    double rs0[1], rm0[1];
    g.reduce(sm0, mx0, rs0, rm0);
    if (!g.ok()) return false;
    const double rhs_norm = rm0[0];
    if (threadIdx.x == 0) {
      double e;
      if (polishing) e = fmax(rhs_norm * 1e-5, kCgTolMin);
      else if (admm_iter == 1) {
        sc->reduction_factor = s.cg_tol_fraction;
        sc->eps_prev = rhs_norm < kCgTolMin ? 1.0 : rhs_norm * sc->reduction_factor;
        e = sc->eps_prev;
      } else {
        if (sc->zero_pcg_iters >= s.cg_tol_reduction) { sc->reduction_factor /= 2; sc->zero_pcg_iters = 0; }
        e = sc->reduction_factor * sqrt(spr * sdr);
        e = fmax(fmin(e, sc->eps_prev), kCgTolMin);
        sc->eps_prev = e;
      }
      sc->pcg_eps = e;
    }
    __syncthreads();
    const double eps = sc->pcg_eps;
    if (pcg_core(g, eps, sig, rho_s) < 0) return false;
    // outputs: b1 <- x ; b2 <- A x  (or (A x - b2) / delta when polishing)
    for_n(g, n, [&](int i) { b[i] = xp[i]; });
    if (m > 0) {
      const T rp = (T)sc->rho;
      rows_rng(g, span_m(g, m), pr.A, [&](int c) { return xp[c]; },
                 [&](int j, T v) { b2[j] = polishing ? (v - b2[j]) * rp : v; });
    }
    return g.sync();
  }

  // ---------------------------------------------------------------------
  // Residuals, objective and all termination quantities (update_info).
  // ---------------------------------------------------------------------
  template <typename G>
  __device__ bool update_info(G& g, int iter) {
    // local copies: hot loops keep the pointers in registers instead of
    // re-reading them through `this` after every store
    const DevProblem<T> pr = this->pr;
    const DevSettings s = this->s;
    SolverScalars* const sc = this->sc;
    const int n = pr.n, m = pr.m;
    const double infval = s.infty * kMinScaling;
    const bool uns = unscaled_term();
    T* x = pr.x; T* z = pr.z; T* y = pr.y;

    // Maxima are integer keys (FKey): on GB300 the FP64 max / compare
    // instructions would cost a slow FP64 warp instruction each.  The bound
    // tests compare bit patterns with the thresholds (l and u are never NaN).
    typedef FKey<T> K;
    typedef typename K::U U;
    typedef typename K::I I;
    const I inf_gt = K::thr_gt(infval), inf_lt = K::thr_lt(infval), dz_lt = K::thr_lt(s.zero_deadzone);

    // the vectors as locals (not reloaded from the problem struct per row)
    const T* const lv = pr.l;
    const T* const uv = pr.u;
    const T* const Ev = pr.E;
    const T* const Eiv = pr.Einv;
    T* const dyv = pr.dy;
    const T* const dxv = pr.dx;
    const T* const qv = pr.q;
    const T* const Dv = pr.D;
    const T* const Div = pr.Dinv;

    // Phase T1 over the rows of A: Ax, A dx and the m-length terms.
    // mx: 0 |Ax-z|  1 |Einv(Ax-z)|  2 |z|  3 |Ax|  4 |Einv z|  5 |Einv Ax|
    //     6 |dy_proj| (|E dy_proj| for unscaled termination)
    //     7 recession-cone violation of (Einv) A dx
    // sm: 0 support function  1 u'max(dy,0) + l'min(dy,0)
    Acc<T> sm[2];
    U km[8];
#pragma unroll
    for (int k = 0; k < 7; k++) km[k] = 0;
    km[7] = K::key(T(-INFINITY));
    if (m > 0) {
      rows_auto2(g, span_m(g, m), pr.A, [&](int c) { return x[c]; }, [&](int c) { return dxv[c]; },
        [&](int j, T ax, T adx) {
          const T l = lv[j], u = uv[j];
          const T ei = Eiv[j];
          const T zj = z[j];
          const T pres = ax - zj;
          km[0] = umaxk(km[0], K::absk(pres));
          km[1] = umaxk(km[1], K::absk(ei * pres));
          km[2] = umaxk(km[2], K::absk(zj));
          km[3] = umaxk(km[3], K::absk(ax));
          km[4] = umaxk(km[4], K::absk(ei * zj));
          km[5] = umaxk(km[5], K::absk(ei * ax));
          const bool u_inf = K::gt(u, inf_gt);       // u > infval
          const bool l_inf = K::neg_gt(l, inf_gt);   // l < -infval
          // support function of [l,u] at y (auxil.c:254-266)
          T yp = y[j];
          if (u_inf) yp = l_inf ? T(0) : K::neg(yp);
          else if (l_inf) yp = K::pos(yp);
          if (K::abs_lt(yp, dz_lt)) yp = T(0);
          sm[0].add_prod(u, K::pos(yp));
          sm[0].add_prod(l, K::neg(yp));
          // project dy onto the polar recession cone (in place) (auxil.c:476-480)
          T dp = dyv[j];
          if (u_inf) dp = l_inf ? T(0) : K::neg(dp);
          else if (l_inf) dp = K::pos(dp);
          dyv[j] = dp;
          km[6] = umaxk(km[6], K::absk(uns ? Ev[j] * dp : dp));
          sm[1].add_prod(u, K::pos(dp));
          sm[1].add_prod(l, K::neg(dp));
          // recession cone test of A dx (vector.c:704-727): violation if
          // (u finite and v > tol) or (l finite and v < -tol)
          const T v = uns ? adx * ei : adx;
          if (K::lt(u, inf_lt)) km[7] = umaxk(km[7], K::key(v));          // u < infval
          if (K::neg_lt(l, inf_lt)) km[7] = umaxk(km[7], K::key_neg(v));  // l > -infval
        });
    }
    T mx[8];
#pragma unroll
    for (int k = 0; k < 7; k++) mx[k] = K::from_absk(warp_umax(km[k]));
    mx[7] = K::from_key(warp_umax(km[7]));
    double smr[2], mxr[8];
    g.reduce_w(sm, mx, smr, mxr);
    if (!g.ok()) return false;

    // Phase T2 over the rows of P / A': Px, P dx, A'y, A'dy and the n-length terms.
    // mx: 0 |q+Px+A'y|  1 |Dinv(q+Px+A'y)|  2 |q|  3 |A'y|  4 |Px|  5 |Dinv q|
    //     6 |Dinv A'y|  7 |Dinv Px|  8 |dx|  9 |P dx|  10 |A'dy| (8-10 with
    //     D, Dinv, Dinv for unscaled termination)
    // sm: 0 x'Px  1 q'x  2 q'dx
    Acc<T> s2[3];
    U k2[11];
#pragma unroll
    for (int k = 0; k < 11; k++) k2[k] = 0;
    {
      auto fn = [&](int i, T px, T pdx, T aty, T atdy) {
        const T q = qv[i];
        const T di = Div[i];
        const T dr = (m > 0) ? (q + px) + aty : q + px;
        k2[0] = umaxk(k2[0], K::absk(dr));
        k2[1] = umaxk(k2[1], K::absk(di * dr));
        k2[2] = umaxk(k2[2], K::absk(q));
        k2[3] = umaxk(k2[3], K::absk(aty));
        k2[4] = umaxk(k2[4], K::absk(px));
        k2[5] = umaxk(k2[5], K::absk(di * q));
        k2[6] = umaxk(k2[6], K::absk(di * aty));
        k2[7] = umaxk(k2[7], K::absk(di * px));
        const T dxi = dxv[i];
        k2[8] = umaxk(k2[8], K::absk(uns ? Dv[i] * dxi : dxi));
        k2[9] = umaxk(k2[9], K::absk(uns ? pdx * di : pdx));
        k2[10] = umaxk(k2[10], K::absk(uns ? atdy * di : atdy));
        s2[0].add_prod(px, x[i]);
        s2[1].add_prod(q, x[i]);
        s2[2].add_prod(q, dxi);
      };
      auto xp1 = [&](int c) { return x[c]; };
      auto xp2 = [&](int c) { return dxv[c]; };
      auto xa1 = [&](int c) { return y[c]; };
      auto xa2 = [&](int c) { return dyv[c]; };
      const Rng rg = span_n(g, n);
      const int L = kktL;
      if constexpr (std::is_same<G, GridGroup>::value || !std::is_same<T, double>::value) {
        // one large QP: sub-warp rows keep every warp of the grid busy; FP32:
        // the sub-warp epilogue is cheap on the FP32 pipe
        auto body = [&](auto Lc) {
          constexpr int LL = decltype(Lc)::value;
          const int lane = threadIdx.x & 31;
          const int sub = lane / LL, sl = lane % LL;
          constexpr int RPW = 32 / LL;
          const int ws = g.ws();
          for (int base = rg.lo + g.w0() * RPW; base < rg.hi; base += ws * RPW) {
            const int i = base + sub;
            T px = T(0), pdx = T(0), aty = T(0), atdy = T(0);
            if (i < rg.hi) {
              lane_row_dot2<LL>(pr.P.col, pr.P.val, pr.P.rowptr[i], pr.P.rowptr[i + 1], sl, xp1, xp2, px, pdx);
              lane_row_dot2<LL>(pr.At.col, pr.At.val, pr.At.rowptr[i], pr.At.rowptr[i + 1], sl, xa1, xa2, aty, atdy);
            }
            px = subwarp_sum<LL>(px); pdx = subwarp_sum<LL>(pdx);
            aty = subwarp_sum<LL>(aty); atdy = subwarp_sum<LL>(atdy);
            if (i < rg.hi && sl == 0) fn(i, px, pdx, aty, atdy);
          }
        };
        switch (L) {
          case 1:  body(std::integral_constant<int, 1>{}); break;
          case 2:  body(std::integral_constant<int, 2>{}); break;
          case 4:  body(std::integral_constant<int, 4>{}); break;
          case 8:  body(std::integral_constant<int, 8>{}); break;
          case 16: body(std::integral_constant<int, 16>{}); break;
          default: body(std::integral_constant<int, 32>{}); break;
        }
      } else {
        switch (L) {
          case 1:  rows_dense_pair_L<1>(g, rg, pr.P, pr.At, xp1, xp2, xa1, xa2, fn); break;
          case 2:  rows_dense_pair_L<2>(g, rg, pr.P, pr.At, xp1, xp2, xa1, xa2, fn); break;
          case 4:  rows_dense_pair_L<4>(g, rg, pr.P, pr.At, xp1, xp2, xa1, xa2, fn); break;
          case 8:  rows_dense_pair_L<8>(g, rg, pr.P, pr.At, xp1, xp2, xa1, xa2, fn); break;
          case 16: rows_dense_pair_L<16>(g, rg, pr.P, pr.At, xp1, xp2, xa1, xa2, fn); break;
          default: rows_dense_pair_L<32>(g, rg, pr.P, pr.At, xp1, xp2, xa1, xa2, fn); break;
        }
      }
    }
    T m2[11];
#pragma unroll
    for (int k = 0; k < 11; k++) m2[k] = K::from_absk(warp_umax(k2[k]));
    double s2r[3], m2r[11];
    g.reduce_w(s2, m2, s2r, m2r);
    if (!g.ok()) return false;

    if (threadIdx.x == 0) {
      SolverScalars* c = sc;
      // primal residual (auxil.c:308-332)
      double prim = 0.0;
      if (m > 0) {
        c->scaled_prim_res = mxr[0];
        prim = uns ? mxr[1] : mxr[0];
      }
      // dual residual (auxil.c:371-407)
      c->scaled_dual_res = m2r[0];
      const double dual = uns ? c->cinv * m2r[1] : m2r[0];
      // objective and gap (auxil.c:231-285)
      const double quad = s2r[0], lin = s2r[1], sup = smr[0];
      double po = 0.5 * quad + lin, dob = -0.5 * quad - sup, gap;
      c->scaled_dual_gap = quad + lin + sup;
      if (s.scaling) { po *= c->cinv; dob *= c->cinv; gap = c->cinv * c->scaled_dual_gap; }
      else gap = c->scaled_dual_gap;
      c->xtPx = quad; c->qtx = lin; c->SC = sup;
      c->obj_val = po; c->dual_obj_val = dob; c->duality_gap = gap;
      c->prim_res = prim; c->dual_res = dual;
      c->iter = iter;
      c->primdual_int += fabs(gap);
      c->rel_kkt_error = fmax(fmax(dual, prim), gap);
      // norms for tolerances and the rho estimate
      c->nz_s = mxr[2]; c->nAx_s = mxr[3]; c->nz_u = mxr[4]; c->nAx_u = mxr[5];
      c->nq_s = m2r[2]; c->nAty_s = m2r[3]; c->nPx_s = m2r[4];
      c->nq_u = m2r[5]; c->nAty_u = m2r[6]; c->nPx_u = m2r[7];
      // infeasibility quantities
      c->dy_norm = mxr[6];
      c->dy_lhs = smr[1];
      c->atdy_norm = m2r[10];
      c->dx_norm = m2r[8];
      c->dx_q = s2r[2];
      c->pdx_norm = m2r[9];
      c->recc_max = mxr[7];
    }
    __syncthreads();
    return true;
  }

  // check_termination (auxil.c:808-945) on the quantities from update_info.
  // Scalar code executed by thread 0 of every CTA.
  __device__ int check_termination_scalar(int approximate) {
    SolverScalars* c = sc;
    const bool uns = unscaled_term();
    const double div_tol = 1.0 / s.infty;
    double ea = s.eps_abs, er = s.eps_rel, epi = s.eps_prim_inf, edi = s.eps_dual_inf;
    int prc = 0, drc = 0, pic = 0, dic = 0, gc = 0;
    if (c->prim_res > s.infty || c->dual_res > s.infty) {
      c->status = ST_NON_CVX;
      c->obj_val = NAN;
      return 1;
    }
    if (approximate) { ea *= 10; er *= 10; epi *= 10; edi *= 10; }
    if (pr.m == 0) prc = 1;
    else {
      const double base = uns ? fmax(c->nz_u, c->nAx_u) : fmax(c->nz_s, c->nAx_s);
      if (c->prim_res < ea + er * base) prc = 1;
      else if (c->dy_norm > div_tol && c->dy_lhs < 0.0)
        pic = c->atdy_norm < epi * c->dy_norm;
    }
    double dbase = uns ? c->cinv * fmax(fmax(c->nq_u, c->nAty_u), c->nPx_u)
                       : fmax(fmax(c->nq_s, c->nAty_s), c->nPx_s);
    if (c->dual_res < ea + er * dbase) drc = 1;
    else {
      const double cs = uns ? c->c : 1.0;
      if (c->dx_norm > div_tol && c->dx_q < 0.0 && c->pdx_norm < cs * edi * c->dx_norm)
        dic = c->recc_max <= edi * c->dx_norm;
    }
    if (s.check_dualgap) {
      double r = fmax(fmax(fabs(c->xtPx), fabs(c->qtx)), fabs(c->SC));
      if (uns) r *= c->cinv;
      const double g = uns ? c->duality_gap : c->scaled_dual_gap;
      gc = fabs(g) < ea + er * r;
    } else gc = 1;
    if (prc && drc && gc) { c->status = approximate ? ST_SOLVED_INACCURATE : ST_SOLVED; return 1; }
    if (pic) { c->status = approximate ? ST_PRIMAL_INFEASIBLE_INACCURATE : ST_PRIMAL_INFEASIBLE; c->obj_val = s.infty; return 1; }
    if (dic) { c->status = approximate ? ST_DUAL_INFEASIBLE_INACCURATE : ST_DUAL_INFEASIBLE; c->obj_val = -s.infty; return 1; }
    return 0;
  }

  // compute_rho_estimate (auxil.c:14-47)
  __device__ double rho_estimate_scalar() const {
    const double div_tol = 1.0 / s.infty;
    double p = sc->scaled_prim_res / (fmax(sc->nz_s, sc->nAx_s) + div_tol);
    double d = sc->scaled_dual_res / (fmax(fmax(sc->nq_s, sc->nAty_s), sc->nPx_s) + div_tol);
    double r = sc->rho * sqrt(p / d);
    return fmin(fmax(r, kRhoMin), kRhoMax);
  }

  // ---------------------------------------------------------------------
  // The solve loop (osqp_api.c:636-1038)
  // ---------------------------------------------------------------------
  //
  // Iterations it_lo..it_hi of the loop.  A solve that reaches it_hi before
  // max_iter without terminating is suspended: status stays ST_UNSOLVED,
  // sc->iter = it_hi, and every iterate stays in place, so a later call with
  // it_lo = it_hi + 1 (by any group form) continues exactly where it stopped.
  template <typename G>
  __device__ bool solve(G& g, int it_lo = 1, int it_hi = 0x7fffffff) {
    __shared__ int s_flags[4];
    if (threadIdx.x == 0) {
      s_flags[0] = 0;
      if (it_lo <= 1) {
        sc->t_start = global_ns();
        sc->status = ST_UNSOLVED;
        sc->pcg_iters_total = 0;
        for (int q = 0; q < kProfSlots; q++) sc->prof[q] = 0;
      }
    }
    if (it_lo <= 1 && !s.warm_starting) { cold_start(g); }
    if (!g.sync()) return false;
    if (kkt_direct(pr.kkt) && sc->kkt_fail) {
      // the factorisation for this rho failed: K is not positive definite
      if (threadIdx.x == 0) { sc->status = ST_NON_CVX; sc->obj_val = NAN; sc->iter = it_lo > 1 ? it_lo - 1 : 0; }
      __syncthreads();
      return store_solution(g);
    }
    if (it_lo < 1) it_lo = 1;
    const int it_end = it_hi < s.max_iter ? it_hi : s.max_iter;
    int can_check = 0;
    int iter;
    bool stopped = false;
    for (iter = it_lo; iter <= it_end; iter++) {
      if (!admm_iteration(g, iter)) return false;
      if (threadIdx.x == 0) {
        int stop = 0;
        if (sc->cancel) { sc->status = ST_SIGINT; stop = 2; }
        else if (s.time_limit > 0 && sc->elapsed >= s.time_limit) { sc->status = ST_TIME_LIMIT_REACHED; stop = 1; }
        s_flags[0] = stop;
        int cc = s.check_termination && (iter % s.check_termination == 0);
        int ca = 0;
        if (s.adaptive_rho == 1 || s.adaptive_rho == 3)
          ca = s.adaptive_rho_interval && (iter % s.adaptive_rho_interval == 0);
        s_flags[1] = cc; s_flags[2] = ca;
      }
      __syncthreads();
      if (s_flags[0]) { stopped = true; break; }
      can_check = s_flags[1];
      int can_adapt = s_flags[2];
      const long long t_info = (s.profile && threadIdx.x == 0) ? clock64() : 0;
      if (can_check || can_adapt || iter == 1) { if (!update_info(g, iter)) return false; }
      if (threadIdx.x == 0) {
        s_flags[3] = 0;
        if (can_check && check_termination_scalar(0)) s_flags[3] = 1;
        sc->rho_updated = 0;
        int ca = can_adapt;
        if (!s_flags[3]) {
          if (ca && s.adaptive_rho == 3) ca = sc->rel_kkt_error <= s.adaptive_rho_fraction * sc->last_rel_kkt;
          if (ca) {
            double rn = rho_estimate_scalar();
            sc->rho_estimate = rn;
            if (rn > sc->rho * s.adaptive_rho_tolerance || rn < sc->rho / s.adaptive_rho_tolerance) {
              sc->rho = fmin(fmax(rn, kRhoMin), kRhoMax);
              sc->rho_inv = 1.0 / sc->rho;
              sc->rho_updates += 1;
              sc->rho_updated = 1;
            }
          }
          if (sc->rho_updated) sc->last_rel_kkt = sc->rel_kkt_error;
        }
      }
      __syncthreads();
      if (s.profile && threadIdx.x == 0) sc->prof[3] += (unsigned long long)(clock64() - t_info);
      if (s_flags[3]) { stopped = true; break; }
      const long long t_fac = (s.profile && threadIdx.x == 0) ? clock64() : 0;
      if (sc->rho_updated) {
        if (s.rho_is_vec) { refresh_rho_vec(g); if (!g.sync()) return false; }
        update_precond(g);
        if (!g.sync()) return false;
        if (kkt_direct(pr.kkt) && sc->kkt_fail) {
          if (threadIdx.x == 0) { sc->status = ST_NON_CVX; sc->obj_val = NAN; s_flags[0] = 3; }
          __syncthreads();
          stopped = true;
          break;
        }
      }
      if (s.profile && threadIdx.x == 0) sc->prof[4] += (unsigned long long)(clock64() - t_fac);
    }
    if (!stopped && it_end < s.max_iter) {
      // suspended at it_hi: no post-loop, no solution store
      if (threadIdx.x == 0) sc->iter = it_end;
      __syncthreads();
      return g.sync();
    }
    // post-loop (osqp_api.c:906-960); an interrupted solve skips it, as the
    // reference jumps to its exit label on SIGINT (and so does a failed
    // refactorisation of the direct solver)
    if (s_flags[0] < 2) {
      if (!can_check) {
        if (!update_info(g, iter - 1)) return false;
        if (threadIdx.x == 0) check_termination_scalar(0);
        __syncthreads();
      }
      if (threadIdx.x == 0) {
        if (sc->status == ST_UNSOLVED) {
          if (!check_termination_scalar(1)) sc->status = ST_MAX_ITER_REACHED;
        } else if (sc->status == ST_TIME_LIMIT_REACHED) {
          check_termination_scalar(1);
        }
        sc->rho_estimate = rho_estimate_scalar();
      }
      __syncthreads();
    }
    return store_solution(g);
  }

  __host__ __device__ static bool has_solution(int st) {
    return st != ST_PRIMAL_INFEASIBLE && st != ST_PRIMAL_INFEASIBLE_INACCURATE &&
           st != ST_DUAL_INFEASIBLE && st != ST_DUAL_INFEASIBLE_INACCURATE && st != ST_NON_CVX;
  }

  // store_solution (auxil.c:598-674) into xo / yo / pcert / dcert
  template <typename G>
  __device__ bool store_solution(G& g) {
    // local copies: hot loops keep the pointers in registers instead of
    // re-reading them through `this` after every store
    const DevProblem<T> pr = this->pr;
    const DevSettings s = this->s;
    SolverScalars* const sc = this->sc;
    const int st = sc->status, n = pr.n, m = pr.m;
    const bool uns = unscaled_term();
    if (has_solution(st)) {
      const T cinv = (T)sc->cinv;
      for_n(g, n, [&](int i) {
        pr.xo[i] = s.scaling ? pr.D[i] * pr.x[i] : pr.x[i];
        pr.dcert[i] = tnan<T>(); pr.dx[i] = tnan<T>();
      });
      for_m(g, m, [&](int j) {
        pr.yo[j] = s.scaling ? (pr.E[j] * pr.y[j]) * cinv : pr.y[j];
        pr.pcert[j] = tnan<T>(); pr.dy[j] = tnan<T>();
      });
      return g.sync();
    }
    const bool pinf = st == ST_PRIMAL_INFEASIBLE || st == ST_PRIMAL_INFEASIBLE_INACCURATE;
    const bool dinf = st == ST_DUAL_INFEASIBLE || st == ST_DUAL_INFEASIBLE_INACCURATE;
    // certificates in the user's scaling (auxil.c:914-935)
    if (pinf && uns) for_m(g, m, [&](int j) { pr.dy[j] *= pr.E[j]; });
    if (dinf && uns) for_n(g, n, [&](int i) { pr.dx[i] *= pr.D[i]; });
    if (!g.sync()) return false;
    Acc<T> sm[1];
    T mx[2] = {T(0), T(0)};
    for_m(g, m, [&](int j) { mx[0] = tmax(mx[0], (T)fabs(pr.dy[j])); });
    for_n(g, n, [&](int i) { mx[1] = tmax(mx[1], (T)fabs(pr.dx[i])); });
    double smr[1], mxr[2];
    g.reduce(sm, mx, smr, mxr);
    if (!g.ok()) return false;
    const T iny = (T)(1.0 / mxr[0]), inx = (T)(1.0 / mxr[1]);
    for_n(g, n, [&](int i) {
      pr.xo[i] = tnan<T>();
      pr.dcert[i] = dinf ? pr.dx[i] * inx : tnan<T>();
      pr.x[i] = T(0); g.put(pr.xp, i, T(0));
    });
    for_m(g, m, [&](int j) {
      pr.yo[j] = tnan<T>();
      pr.pcert[j] = pinf ? pr.dy[j] * iny : tnan<T>();
      pr.z[j] = T(0); pr.y[j] = T(0);
    });
    return g.sync();
  }
};

}  // namespace gb
