// polish.cu -- solution polishing (src/polish.c:19-515) on the device, in FP64.
//
// After an OSQP_SOLVED solve with settings->polishing:
//   1. active set from the scaled ADMM iterates (polish.c:60-78): row j is
//      lower-active if z_j - l_j < -y_j or l_j == u_j, upper-active if
//      u_j - z_j < y_j; Ared = the active rows of A in order (polish.c:81-86);
//   2. reduced KKT solve [P + dI, Ared'; Ared, -dI] [x; yred] = [-q; l_low/u_upp]
//      (polish.c:106-171) by the reduced-KKT PCG in polishing mode, as the
//      CUDA backend does (cuda_pcg_interface.cu:149-156, 229-273): sigma = d,
//      rho = 1/d, output [x; (Ared x - b2) / d];
//   3. polish_refine_iter steps of iterative refinement against the
//      unregularized KKT matrix (polish.c:183-245);
//   4. x, z = A x, y from yred, then y <- y + z, z <- proj(y), y <- y - z
//      (polish.c:452-459), residuals and objective (update_info, polishing
//      mode), and the acceptance test of polish.c:464-476.
// Everything from the active set to the acceptance runs in one kernel launch
// (one CTA, or a cooperative grid for large problems).  The reduced system
// is solved in FP64 whatever the build's OSQPFloat: the data are converted
// once; the PCG iteration cap is raised to kPolishCgMaxIter because the
// 1/delta-weighted reduced system is far worse conditioned than the ADMM
// system: with the reference's 20 iterations the CUDA backend's polish fails
// on every pinned workload, and the refinement corrections of a 1745-variable
// MPC QP need up to ~4200 Jacobi-PCG iterations to reach the tolerance.
#include <cuda_runtime.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>

#include <cub/device/device_scan.cuh>

#include "osqp_gb300.h"
#include "gb_solver.cuh"
#include "gb_engine.h"

using T = OSQPFloat;
using namespace gb;

namespace gbp {

constexpr int kPolishThreads = 1024;
constexpr int kPolishCgMaxIter = 10000;

// Result of one polish launch (device -> host).
struct PolishOut {
  int accepted;
  double obj_val, dual_obj_val, duality_gap, prim_res, dual_res;
};

struct PolishArgs {
  DevProblem<T> pr;          // main problem (scaled data, iterates x z y)
  DevSettings s;             // main settings
  int kktL;                  // main lanes for P / A'
  DevProblem<double> rd;     // reduced system: P, Ared, Ared' in FP64
  DevSettings sd;            // reduced-system settings (sigma = delta, scalar rho)
  int kktLr;
  const int* flags;          // -1 / 0 / +1 per constraint
  const int* red;            // reduced index of an active constraint
  double* b;                 // [n + mred] reduced right-hand side
  double* sol;               // [n + mred] reduced solution
  double* res;               // [n + mred] refinement residual / correction
  T *px, *pz, *py;           // polished x, z, y (scaled, OSQPFloat)
  T *sdx, *sdy;              // scratch for update_info
  double delta;
  int refine;
  PolishOut* out;
};

// Active flags, Ared row lengths and reduced indices (polish.c:60-78).
__global__ void k_pol_flags(DevProblem<T> pr, int* flags, int* active, int* rowlen) {
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < pr.m; j += gridDim.x * blockDim.x) {
    const T z = pr.z[j], y = pr.y[j], l = pr.l[j], u = pr.u[j];
    int f = 0;
    if ((z - l < -y) || (l == u)) f = -1;
    else if (u - z < y) f = 1;
    flags[j] = f;
    active[j] = f != 0;
    rowlen[j] = f != 0 ? pr.A.rowptr[j + 1] - pr.A.rowptr[j] : 0;
  }
}

// Entries of A' (columns of A) that survive in Ared', per column.
__global__ void k_pol_count_at(DevProblem<T> pr, const int* flags, int* cnt) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < pr.n; i += gridDim.x * blockDim.x) {
    int c = 0;
    for (int k = pr.At.rowptr[i]; k < pr.At.rowptr[i + 1]; k++) c += flags[pr.At.col[k]] != 0;
    cnt[i] = c;
  }
}

// Ared (CSR, rows in order), Ared' (CSR of the transpose, from A'), FP64
// values of P, and rhs_red = [-q; l_low / u_upp] (polish.c:106-171).
__global__ void k_pol_build(DevProblem<T> pr, const int* flags, const int* red, const int* aoff,
                            const int* atoff, int* ar_row, int* ar_col, double* ar_val, int* at_col,
                            double* at_val, double* pval, int nnzPf, double* b, int mred) {
  const int tid = blockIdx.x * blockDim.x + threadIdx.x, nt = gridDim.x * blockDim.x;
  const int n = pr.n;
  for (int j = tid; j < pr.m; j += nt) {
    if (!flags[j]) continue;
    const int r = red[j];
    int o = aoff[j];
    ar_row[r] = o;
    for (int k = pr.A.rowptr[j]; k < pr.A.rowptr[j + 1]; k++, o++) {
      ar_col[o] = pr.A.col[k];
      ar_val[o] = (double)pr.A.val[k];
    }
    b[n + r] = flags[j] < 0 ? (double)pr.l[j] : (double)pr.u[j];
  }
  if (tid == 0) ar_row[mred] = aoff[pr.m];
  for (int i = tid; i < n; i += nt) {
    int o = atoff[i];
    for (int k = pr.At.rowptr[i]; k < pr.At.rowptr[i + 1]; k++) {
      const int j = pr.At.col[k];
      if (!flags[j]) continue;
      at_col[o] = red[j];
      at_val[o] = (double)pr.At.val[k];
      o++;
    }
    b[i] = -(double)pr.q[i];
  }
  const int p0 = pr.P.rowptr[0];
  for (int k = tid; k < nnzPf; k += nt) pval[k] = (double)pr.P.val[p0 + k];
}

// Steps 2-4 on one group.
template <typename G>
__device__ void polish_body(G& g, const PolishArgs& a, SolverScalars* ssr, SolverScalars* ssp,
                            const SolverScalars& main_sc) {
  const int n = a.pr.n, m = a.pr.m, mred = a.rd.m;
  Solver<double> R{a.rd, a.sd, ssr, a.kktLr};
  if (threadIdx.x == 0) {
    *ssr = main_sc;
    ssr->rho = 1.0 / a.delta;
    ssr->rho_inv = a.delta;
    ssr->pcg_iters_total = 0;
    ssr->zero_pcg_iters = 0;
  }
  __syncthreads();
  // Jacobi preconditioner of the reduced system; warm start from the ADMM x
  // (polish.c:431); sol = rhs_red (polish.c:406)
  R.update_precond(g);
  for_each(g, n, [&](int i) { a.rd.xp[i] = (double)a.pr.x[i]; });
  for_each(g, n + mred, [&](int k) { a.sol[k] = a.b[k]; });
  if (!g.sync()) return;
  if (!R.linsys_solve(g, a.sol, 1, true, 0.0, 0.0)) return;
  // iterative refinement (polish.c:203-236): res = b - K sol ; solve ; sol += res
  for (int it = 0; it < a.refine; it++) {
    kkt_rows(g, a.kktLr, a.rd.P, a.rd.At, [&](int c) { return a.sol[c]; },
             [&](int c) { return a.sol[n + c]; },
             [&](int i, double pv, double av) { a.res[i] = a.b[i] - pv - av; });
    if (mred > 0)
      rows_rng(g, span_m(g, mred), a.rd.A, [&](int c) { return a.sol[c]; },
               [&](int j, double v) { a.res[n + j] = a.b[n + j] - v; });
    if (!g.sync()) return;
    if (!R.linsys_solve(g, a.res, 1, true, 0.0, 0.0)) return;
    for_each(g, n + mred, [&](int k) { a.sol[k] += a.res[k]; });
    if (!g.sync()) return;
  }
  // polished x, z = A x, y from yred; y <- y + z ; z <- proj(y) ; y <- y - z
  for_each(g, n, [&](int i) { a.px[i] = (T)a.sol[i]; a.sdx[i] = T(0); });
  if (!g.sync()) return;
  if (m > 0) {
    rows_apply(g, a.pr.A, [&](int c) { return a.px[c]; }, [&](int j, T v) {
      const T yj = a.flags[j] ? (T)a.sol[n + a.red[j]] : T(0);
      const T yz = yj + v;
      const T zz = tmin(tmax(yz, a.pr.l[j]), a.pr.u[j]);
      a.pz[j] = zz;
      a.py[j] = yz - zz;
      a.sdy[j] = T(0);
    });
  }
  if (!g.sync()) return;
  // residuals and objective at the polished point (update_info, polishing mode)
  DevProblem<T> pp = a.pr;
  pp.x = a.px; pp.z = a.pz; pp.y = a.py; pp.dx = a.sdx; pp.dy = a.sdy;
  if (threadIdx.x == 0) *ssp = main_sc;
  __syncthreads();
  Solver<T> M{pp, a.s, ssp, a.kktL};
  if (!M.update_info(g, main_sc.iter)) return;
  // acceptance (polish.c:464-476)
  __shared__ int s_acc;
  if (threadIdx.x == 0) {
    const double pp_res = ssp->prim_res, pd_res = ssp->dual_res;
    const double ip = main_sc.prim_res, id = main_sc.dual_res;
    s_acc = (pp_res < ip && pd_res < id) || (pp_res < ip && id < 1e-10) || (pd_res < id && ip < 1e-10);
  }
  __syncthreads();
  const bool acc = s_acc != 0;
  if (acc) {
    // x, z, y <- polished; the stored (unscaled) solution follows (auxil.c:598-674)
    const T cinv = (T)main_sc.cinv;
    const bool sc_on = a.s.scaling != 0;
    for_each(g, n, [&](int i) {
      a.pr.x[i] = a.px[i];
      a.pr.xo[i] = sc_on ? a.pr.D[i] * a.px[i] : a.px[i];
    });
    for_each(g, m, [&](int j) {
      a.pr.z[j] = a.pz[j];
      a.pr.y[j] = a.py[j];
      a.pr.yo[j] = sc_on ? (a.pr.E[j] * a.py[j]) * cinv : a.py[j];
    });
  }
  if (!g.sync()) return;
  if (g.tid() == 0) {
    a.out->accepted = acc ? 1 : 0;
    a.out->obj_val = ssp->obj_val;
    a.out->dual_obj_val = ssp->dual_obj_val;
    a.out->duality_gap = ssp->duality_gap;
    a.out->prim_res = ssp->prim_res;
    a.out->dual_res = ssp->dual_res;
  }
}

__global__ void __launch_bounds__(kPolishThreads, 1) k_polish_block(PolishArgs a) {
  __shared__ GroupShared gsh;
  __shared__ SolverScalars ssr, ssp, smain;
  if (threadIdx.x == 0) { gsh.parity = 0; gsh.flag = 0; smain = *a.pr.st; }
  __syncthreads();
  BlockGroup g{&gsh};
  polish_body(g, a, &ssr, &ssp, smain);
}

__global__ void __launch_bounds__(kPolishThreads, 1) k_polish_grid(PolishArgs a, GridSync gs) {
  __shared__ GroupShared gsh;
  __shared__ SolverScalars ssr, ssp, smain;
  if (threadIdx.x == 0) { gsh.parity = 0; gsh.flag = 0; smain = *a.pr.st; }
  __syncthreads();
  GridGroup g{&gsh, gs};
  polish_body(g, a, &ssr, &ssp, smain);
}

}  // namespace gbp

using namespace gbp;

// Returns 0 when the polish ran (its outcome is recorded in
// info->status_polish), OSQP_ALGEBRA_LOAD_ERROR on a device failure.
int gb_polish_run(OSQPSolver* solver) {
  GbEngineView v = gb_engine_view(solver);
  OSQPInfo* info = solver->info;
  const OSQPSettings* st = solver->settings;
  const int n = v.n, m = v.m;
  cudaStream_t s = v.stream;
  if (m == 0) { info->status_polish = OSQP_POLISH_NO_ACTIVE_SET_FOUND; return 0; }

  // ---- scratch: one allocation ----
  struct Plan { size_t off = 0; size_t take(size_t b) { off = (off + 255) & ~size_t(255); size_t o = off; off += b > 0 ? b : 1; return o; } } pl;
  const int nnzA = v.nnzA, nnzPf = v.nnzPf;
  const size_t o_flags = pl.take(sizeof(int) * m), o_act = pl.take(sizeof(int) * (m + 1));
  const size_t o_red = pl.take(sizeof(int) * (m + 1)), o_rl = pl.take(sizeof(int) * (m + 1));
  const size_t o_aoff = pl.take(sizeof(int) * (m + 1)), o_atc = pl.take(sizeof(int) * (n + 1));
  const size_t o_atrow = pl.take(sizeof(int) * (n + 1));
  const size_t o_arrow = pl.take(sizeof(int) * (m + 1)), o_arcol = pl.take(sizeof(int) * nnzA);
  const size_t o_arval = pl.take(sizeof(double) * nnzA), o_atcol = pl.take(sizeof(int) * nnzA);
  const size_t o_atval = pl.take(sizeof(double) * nnzA), o_pval = pl.take(sizeof(double) * nnzPf);
  size_t o_dn[7];
  for (int k = 0; k < 7; k++) o_dn[k] = pl.take(sizeof(double) * n);
  const size_t o_t = pl.take(sizeof(double) * m);
  const size_t o_b = pl.take(sizeof(double) * (n + m)), o_sol = pl.take(sizeof(double) * (n + m));
  const size_t o_res = pl.take(sizeof(double) * (n + m));
  const size_t o_px = pl.take(sizeof(T) * n), o_sdx = pl.take(sizeof(T) * n);
  const size_t o_pz = pl.take(sizeof(T) * m), o_py = pl.take(sizeof(T) * m), o_sdy = pl.take(sizeof(T) * m);
  const size_t o_out = pl.take(sizeof(PolishOut));
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, solver->settings->device);
  const int gblocks = std::max(1, sms);
  const size_t o_bar = pl.take(sizeof(unsigned int) * 4), o_err = pl.take(sizeof(int) * 4);
  const size_t o_part = pl.take(sizeof(double) * (size_t)(4 * kMaxSum + 2 * kMaxMax) * gblocks);
  size_t tmp_bytes = 0;
  cub::DeviceScan::ExclusiveSum(nullptr, tmp_bytes, (int*)nullptr, (int*)nullptr, std::max(n, m) + 1, s);
  const size_t o_tmp = pl.take(tmp_bytes);
  char* ws = nullptr;
  if (cudaMallocAsync((void**)&ws, pl.off, s) != cudaSuccess) {
    cudaGetLastError();
    info->status_polish = OSQP_POLISH_FAILED;
    return OSQP_MEM_ALLOC_ERROR;
  }
  auto P_ = [&](size_t o) { return (void*)(ws + o); };
  int* flags = (int*)P_(o_flags); int* act = (int*)P_(o_act); int* red = (int*)P_(o_red);
  int* rl = (int*)P_(o_rl); int* aoff = (int*)P_(o_aoff); int* atc = (int*)P_(o_atc);
  int* atrow = (int*)P_(o_atrow);
  PolishOut* dout = (PolishOut*)P_(o_out);
  int rc = 0;
  int counts[3] = {0, 0, 0};   // n_active, nnz(Ared), nnz(Ared')
  {
    const int blocks = (std::max(n, m) + 255) / 256;
    k_pol_flags<<<std::min(blocks, 4096), 256, 0, s>>>(v.pr, flags, act, rl);
    k_pol_count_at<<<std::min((n + 255) / 256, 4096), 256, 0, s>>>(v.pr, flags, atc);
    cudaMemsetAsync(act + m, 0, sizeof(int), s);
    cudaMemsetAsync(rl + m, 0, sizeof(int), s);
    cudaMemsetAsync(atc + n, 0, sizeof(int), s);
    size_t tb = tmp_bytes;
    if (cub::DeviceScan::ExclusiveSum(P_(o_tmp), tb, act, red, m + 1, s) != cudaSuccess ||
        cub::DeviceScan::ExclusiveSum(P_(o_tmp), tb, rl, aoff, m + 1, s) != cudaSuccess ||
        cub::DeviceScan::ExclusiveSum(P_(o_tmp), tb, atc, atrow, n + 1, s) != cudaSuccess) rc = -1;
    if (!rc && (cudaMemcpyAsync(&counts[0], red + m, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
                cudaMemcpyAsync(&counts[1], aoff + m, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
                cudaMemcpyAsync(&counts[2], atrow + n, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
                cudaStreamSynchronize(s) != cudaSuccess)) rc = -1;
  }
  if (rc) { cudaFreeAsync(ws, s); info->status_polish = OSQP_POLISH_FAILED; return OSQP_ALGEBRA_LOAD_ERROR; }
  const int mred = counts[0];
  if (mred == 0) {
    cudaFreeAsync(ws, s);
    info->status_polish = OSQP_POLISH_NO_ACTIVE_SET_FOUND;
    return 0;
  }

  PolishArgs a;
  a.pr = v.pr; a.s = v.ds; a.kktL = pick_lanes((long long)nnzPf + nnzA, n);
  a.flags = flags; a.red = red;
  DevProblem<double> rd;
  memset(&rd, 0, sizeof(rd));
  rd.n = n; rd.m = mred;
  rd.P = CSR<double>{v.pr.P.rowptr, v.pr.P.col, (double*)P_(o_pval), n, n, v.pr.P.lanes};
  rd.A = CSR<double>{(int*)P_(o_arrow), (int*)P_(o_arcol), (double*)P_(o_arval), mred, n,
                     pick_lanes(counts[1], mred)};
  rd.At = CSR<double>{atrow, (int*)P_(o_atcol), (double*)P_(o_atval), n, mred, pick_lanes(counts[2], n)};
  rd.Pdiag = v.pr.Pdiag;
  double* dn[7];
  for (int k = 0; k < 7; k++) dn[k] = (double*)P_(o_dn[k]);
  rd.xp = dn[0]; rd.r = dn[1]; rd.p0 = dn[2]; rd.p1 = dn[2]; rd.Kp = dn[3]; rd.yv = dn[4]; rd.rhs = dn[5];
  rd.Minv = dn[6]; rd.t = (double*)P_(o_t);
  rd.rho_vec = nullptr;
  a.rd = rd;
  a.kktLr = pick_lanes((long long)nnzPf + counts[2], n);
  a.sd = v.ds;
  a.sd.sigma = st->delta;
  a.sd.rho_is_vec = 0;
  a.sd.cg_max_iter = std::max((int)st->cg_max_iter, kPolishCgMaxIter);
  a.b = (double*)P_(o_b); a.sol = (double*)P_(o_sol); a.res = (double*)P_(o_res);
  a.px = (T*)P_(o_px); a.pz = (T*)P_(o_pz); a.py = (T*)P_(o_py);
  a.sdx = (T*)P_(o_sdx); a.sdy = (T*)P_(o_sdy);
  a.delta = st->delta;
  a.refine = (int)st->polish_refine_iter;
  a.out = dout;
  // The P values are rebased: rd.P.rowptr holds the main arrays' positions,
  // which start at 0 for a single-QP workspace.
  k_pol_build<<<std::min((std::max(n, m) + 255) / 256, 4096), 256, 0, s>>>(
      v.pr, flags, red, aoff, atrow, (int*)P_(o_arrow), (int*)P_(o_arcol), (double*)P_(o_arval),
      (int*)P_(o_atcol), (double*)P_(o_atval), (double*)P_(o_pval), nnzPf, a.b, mred);
  if (cudaGetLastError() != cudaSuccess) rc = -1;
  const long long work = (long long)nnzPf + 2LL * counts[1] + n + mred;
  if (!rc) {
    if (work > 2000000LL) {
      GridSync gs;
      gs.count = (unsigned int*)P_(o_bar); gs.gen = gs.count + 1; gs.err = (int*)P_(o_err);
      gs.partial_sum = (double*)P_(o_part);
      gs.partial_max = gs.partial_sum + (size_t)4 * kMaxSum * gblocks;
      cudaMemsetAsync(P_(o_bar), 0, sizeof(unsigned int) * 4, s);
      cudaMemsetAsync(P_(o_err), 0, sizeof(int) * 4, s);
      int per_sm = 0;
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_polish_grid, kPolishThreads, 0);
      if (per_sm < 1) rc = -1;
      else {
        void* args[] = {(void*)&a, (void*)&gs};
        if (cudaLaunchCooperativeKernel((void*)k_polish_grid, dim3(gblocks), dim3(kPolishThreads), args, 0, s) !=
            cudaSuccess) rc = -1;
      }
    } else {
      k_polish_block<<<1, kPolishThreads, 0, s>>>(a);
      if (cudaGetLastError() != cudaSuccess) rc = -1;
    }
  }
  PolishOut out;
  memset(&out, 0, sizeof(out));
  int err = 0;
  if (!rc && (cudaMemcpyAsync(&out, dout, sizeof(out), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
              cudaMemcpyAsync(&err, P_(o_err), sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
              cudaStreamSynchronize(s) != cudaSuccess)) rc = -1;
  cudaFreeAsync(ws, s);
  if (rc || err) {
    info->status_polish = OSQP_POLISH_FAILED;
    return OSQP_ALGEBRA_LOAD_ERROR;
  }
  if (out.accepted) {
    info->obj_val = (OSQPFloat)out.obj_val;
    info->dual_obj_val = (OSQPFloat)out.dual_obj_val;
    info->duality_gap = (OSQPFloat)out.duality_gap;
    info->prim_res = (OSQPFloat)out.prim_res;
    info->dual_res = (OSQPFloat)out.dual_res;
    info->status_polish = OSQP_POLISH_SUCCESS;
  } else {
    info->status_polish = OSQP_POLISH_FAILED;
  }
  return 0;
}

void gb_polish_free(void*) {}
