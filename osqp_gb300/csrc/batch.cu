// batch.cu -- many independent QPs in one persistent launch.
//
// Layout: the QPs are packed block-diagonally.  Every per-QP array (CSR
// structures, values, vectors) is one slice of a batch-wide array; row
// pointers hold batch-global positions and column indices are QP-local, so
// the per-QP view used by the device solver (gb_solver.cuh) is a set of
// offset pointers.  Structures are built once at setup with the same stable
// radix-sort transposes as the single-QP path (gb_structure.cuh), for all
// QPs at once.
//
// Execution: a persistent grid pulls QPs from an atomic work queue ordered by
// decreasing nonzero count (largest first).  Two group forms run the same
// device solver (gb_solver.cuh):
//   * CTA form (k_batch): one CTA per QP, block barriers only.  For a solve the
//     CTA stages the QP's PCG vectors and row pointers (and, when they fit,
//     its matrices) in dynamic shared memory.
//   * cluster form (k_batch_cluster): a thread-block cluster per QP.  Each CTA
//     owns a contiguous slice of rows, holds its slice of the matrices in
//     shared memory and a full copy of the gathered vectors (p, A p, x~, rho),
//     written to every CTA through distributed shared memory; reductions push
//     per-CTA partials to every CTA and merge them in rank order.
// A solve runs the CTA form up to a fixed ADMM iteration (the split); the QPs
// still running then continue, from exactly where they stopped, in the
// cluster form, so the slowest QPs no longer set the launch's makespan.  The
// split is a fixed iteration count, so a QP's result does not depend on the
// rest of the batch.  No QP ever waits on another.
#include <cuda_runtime.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <thread>
#include <type_traits>
#include <unordered_map>
#include <numeric>
#include <vector>

#include "osqp_gb300.h"
#include "osqp_gb300_ext.h"
#include "gb_solver.cuh"
#include "gb_structure.cuh"
#include "gb_launch.cuh"
#include "gb_kkt_plan.h"

using T = OSQPFloat;
using namespace gb;

#define BT_TRY(call)                                                              \
  do {                                                                            \
    cudaError_t _e = (call);                                                      \
    if (_e != cudaSuccess) {                                                      \
      fprintf(stderr, "osqp_gb300 batch: %s failed: %s (%s:%d)\n", #call,         \
              cudaGetErrorString(_e), __FILE__, __LINE__);                        \
      return OSQP_ALGEBRA_LOAD_ERROR;                                             \
    }                                                                             \
  } while (0)

namespace gbb {

constexpr int kBatchThreads = 512;

struct BatchInst {
  int n, m, n_off, m_off;
  int pt_off, a_off;    // offsets of the QP's triu-P and A entries (input order)
  int kktL, PL, AL, AtL;
  int Pdiag_only;       // P holds exactly its full diagonal
  int blk_off;          // first 32 x 32 block-Jacobi block of the QP (cg_precond = 2)
  // direct KKT solve (knb == 0: the PCG): blocks, largest block, offsets of
  // the QP's block lists, constraint lists and factor
  int knb, kbmax, kb_off, kcr_off;
  int kring, ksegmax;   // bulk-copy ring slots of the solve and largest factor segment
  long long kf_off;
  // diagonal-plus-dense-rows form (kdr > 0; knb == 0): dense rows, offset of
  // the QP's dense-row list and of its inverse capacitance matrix
  int kdr, kdr_off;
  long long kc_off;
};

template <typename TT>
struct BatchArrays {
  int *Prow, *Pcol, *Pdiag, *Psrc;
  TT *Pval, *Praw;
  int *Arow, *Acol, *Asrc, *Atrow, *Atcol;
  TT *Aval, *Araw, *Atval;
  TT* vn[16];
  TT* vm[16];
  int* ctype;
  SolverScalars* st;
  const BatchInst* inst;
  TT* Binv;             // block-Jacobi blocks of every QP (nullptr unless cg_precond = 2)
  // direct KKT solve: plans and factors of every QP (gb_kkt_plan.h)
  int *kperm, *kiperm, *kbs, *kfo, *kbo, *kco, *kcr;
  TT* kF;
  int *kdrows, *kdidx;  // dense-row lists, row -> dense-row maps (msum)
  TT *kCinv, *kDginv;   // inverse capacitance matrices, Dg^-1 (nsum)

  __device__ DevProblem<TT> problem(int k) const {
    const BatchInst b = inst[k];
    DevProblem<TT> pr;
    pr.n = b.n; pr.m = b.m;
    pr.P = CSR<TT>{Prow + b.n_off, Pcol, Pval, b.n, b.n, b.PL};
    pr.P.diag = b.Pdiag_only;
    pr.A = CSR<TT>{Arow + b.m_off, Acol, Aval, b.m, b.n, b.AL};
    pr.At = CSR<TT>{Atrow + b.n_off, Atcol, Atval, b.n, b.m, b.AtL};
    pr.Pdiag = Pdiag + b.n_off; pr.Psrc = Psrc; pr.Asrc = Asrc;
    pr.Praw = Praw; pr.Araw = Araw;
    const int o = b.n_off, p = b.m_off;
    pr.q = vn[0] + o; pr.q_in = vn[1] + o; pr.D = vn[2] + o; pr.Dinv = vn[3] + o; pr.x = vn[4] + o;
    pr.dx = vn[5] + o; pr.xp = vn[6] + o; pr.r = vn[7] + o; pr.p0 = vn[8] + o; pr.p1 = vn[9] + o;
    pr.Kp = vn[10] + o; pr.yv = vn[11] + o; pr.rhs = vn[12] + o; pr.Minv = vn[13] + o;
    pr.xo = vn[14] + o; pr.dcert = vn[15] + o; pr.Dt = pr.Kp;
    pr.l = vm[0] + p; pr.u = vm[1] + p; pr.l_in = vm[2] + p; pr.u_in = vm[3] + p; pr.E = vm[4] + p;
    pr.Einv = vm[5] + p; pr.rho_vec = vm[6] + p; pr.rho_inv_vec = vm[7] + p; pr.z = vm[8] + p;
    pr.y = vm[9] + p; pr.dy = vm[10] + p; pr.t = vm[11] + p; pr.yo = vm[12] + p;
    pr.pcert = vm[13] + p; pr.Et = vm[14] + p;
    pr.ctype = ctype + p;
    pr.st = st + k;
    pr.Binv = Binv ? Binv + (size_t)b.blk_off * kPrecondBlock * kPrecondBlock : nullptr;
    pr.Arow_g = pr.A.rowptr; pr.Acol_g = Acol; pr.Aval_g = Aval;
    if (b.knb > 0) {
      pr.kkt.nb = b.knb; pr.kkt.bmax = b.kbmax;
      pr.kkt.ring = b.kring; pr.kkt.segmax = b.ksegmax;
      pr.kkt.bs = kbs + b.kb_off; pr.kkt.fo = kfo + b.kb_off; pr.kkt.bo = kbo + b.kb_off;
      pr.kkt.co = kco + b.kb_off;
      pr.kkt.cr = kcr + b.kcr_off;
      pr.kkt.perm = kperm + o; pr.kkt.iperm = kiperm + o;
      pr.kkt.F = kF + b.kf_off;
    } else if (b.kdr > 0) {
      pr.kkt.dr = b.kdr;
      pr.kkt.drows = kdrows + b.kdr_off;
      pr.kkt.didx = kdidx + p;
      pr.kkt.Cinv = kCinv + b.kc_off;
      pr.kkt.Dginv = kDginv + o;
    }
    return pr;
  }
};

enum BatchMode : int { kModeSetup = 0, kModeSolve = 1, kModeUpdateVec = 2, kModeUpdateMat = 3 };

// Shared-memory staging of one QP for a solve.
//
// Every CTA of the group keeps, at the same offsets, full copies of the
// vectors that the sparse products gather (p, t = R A p, xp and the rho
// vector): writes go to all copies (group put()).  Then, for the CTA's own
// rows only (its Spans), the CSR row pointers, the element-wise PCG vectors
// (r, M^-1 r, K p, M^-1, rhs) and, while they fit, the CSR entries of A, A'
// and P.  Span-only arrays are addressed by global index through an offset
// pointer (buffer - first index), so the solver code is unchanged.  Contents
// that persist across ADMM iterations (xp, the rho vector, M^-1) are copied
// in (dir > 0) and their own span back (dir < 0); the row pointers and
// entries are copied in; the rest is scratch written before it is read.  The
// layout is a pure function of sizes and spans, so the copy-back call
// recomputes it.  Returns false (and changes nothing) when the gathered
// vectors do not fit.
template <typename TT>
struct Stager {
  unsigned char* base;
  int cap, off, dir;
  __device__ __forceinline__ unsigned* take(long long words) {
    const long long bytes = (words * 4 + 15) & ~15LL;
    if (words <= 0 || off + bytes > cap) return nullptr;
    unsigned* q = (unsigned*)(base + off);
    off += (int)bytes;
    return q;
  }
  __device__ __forceinline__ static void copy(unsigned* dst, const unsigned* from, long long words) {
    for (long long i = threadIdx.x; i < words; i += blockDim.x) dst[i] = from[i];
  }
  static constexpr int W = (int)(sizeof(TT) / 4);
  // full-length copy; in: everything, back: [lo, hi)
  __device__ __forceinline__ TT* full(TT* v, int len, int lo, int hi, bool io, bool& ok) {
    unsigned* q = take((long long)len * W);
    if (!q) { ok = false; return v; }
    if (io && dir > 0) copy(q, (const unsigned*)v, (long long)len * W);
    if (io && dir < 0) copy((unsigned*)(v + lo), (const unsigned*)((TT*)q + lo), (long long)(hi - lo) * W);
    return (TT*)q;
  }
  // [lo, hi) only
  __device__ __forceinline__ TT* span(TT* v, int lo, int hi, bool io) {
    unsigned* q = take((long long)(hi - lo) * W);
    if (!q) return v;
    if (io && dir > 0) copy(q, (const unsigned*)(v + lo), (long long)(hi - lo) * W);
    if (io && dir < 0) copy((unsigned*)(v + lo), q, (long long)(hi - lo) * W);
    return (TT*)q - lo;
  }
  __device__ __forceinline__ const int* rows(const int* rowptr, int lo, int hi) {
    unsigned* q = take(hi - lo + 1);
    if (!q) return rowptr;
    if (dir > 0) copy(q, (const unsigned*)(rowptr + lo), hi - lo + 1);
    return (const int*)q - lo;
  }
  // entries of rows [lo, hi); rowptr holds global positions.  When they do
  // not all fit, the entries of the longest prefix of rows that fits go on
  // chip (M.scol / M.sval for rows below M.srow) and the rest stay in HBM.
  __device__ __forceinline__ void entries(CSR<TT>& M, const int* grow, int lo, int hi, int share = 1) {
    if (hi <= lo) return;
    const int k0 = grow[lo], k1 = grow[hi];
    if (k1 <= k0) return;
    const long long room = (long long)(cap - off) / 4 / share - 8;   // words, less alignment slack
    const long long fit = room > 0 ? room / (1 + W) : 0;         // entries
    int rs = hi;
    if ((long long)(k1 - k0) > fit) {                             // largest rs with grow[rs] - k0 <= fit
      int a = lo, b = hi;
      while (a < b) {
        const int mid = (a + b + 1) >> 1;
        if ((long long)(grow[mid] - k0) <= fit) a = mid; else b = mid - 1;
      }
      rs = a;
    }
    const int ke = grow[rs];
    if (rs <= lo || ke <= k0) return;
    unsigned* qc = take(ke - k0);
    unsigned* qv = qc ? take((long long)(ke - k0) * W) : nullptr;
    if (!qv) return;
    if (dir > 0) {
      copy(qc, (const unsigned*)(M.col + k0), ke - k0);
      copy(qv, (const unsigned*)(M.val + k0), (long long)(ke - k0) * W);
    }
    if (rs == hi) {
      M.col = (const int*)qc - k0;
      M.val = (TT*)qv - k0;
    } else {
      M.scol = (const int*)qc - k0;
      M.sval = (TT*)qv - k0;
      M.srow = rs;
    }
  }
};

template <typename TT>
__device__ __forceinline__ bool stage_problem(DevProblem<TT>& pr, const Spans& sp, bool rho_vec,
                                              unsigned char* base, int cap, int dir, bool matrices = true,
                                              bool matrices_first = false) {
  Stager<TT> sg{base, cap, 0, dir};
  const int n = pr.n, m = pr.m;
  const int nlo = sp.nlo, nhi = n < sp.nhi ? n : sp.nhi;
  const int mlo = sp.mlo, mhi = m < sp.mhi ? m : sp.mhi;
  bool ok = true;
  DevProblem<TT> q = pr;
  q.p0 = sg.full(pr.p0, n, nlo, nhi, false, ok);
  if (m) q.t = sg.full(pr.t, m, mlo, mhi, false, ok);
  q.xp = sg.full(pr.xp, n, nlo, nhi, true, ok);
  if (m && rho_vec) q.rho_vec = sg.full(pr.rho_vec, m, mlo, mhi, true, ok);
  if (!ok) return false;
  const int* growA = pr.A.rowptr;
  const int* growAt = pr.At.rowptr;
  const int* growP = pr.P.rowptr;
  if (m) q.A.rowptr = sg.rows(pr.A.rowptr, mlo, mhi);
  q.At.rowptr = sg.rows(pr.At.rowptr, nlo, nhi);
  q.P.rowptr = sg.rows(pr.P.rowptr, nlo, nhi);
  auto streamed = [&]() {
    q.Minv = sg.span(pr.Minv, nlo, nhi, true);
    q.r = sg.span(pr.r, nlo, nhi, false);
    q.yv = sg.span(pr.yv, nlo, nhi, false);
    q.Kp = sg.span(pr.Kp, nlo, nhi, false);
    q.rhs = sg.span(pr.rhs, nlo, nhi, false);
  };
  if (!matrices_first) streamed();
  if (matrices) {
    // matrices first: A may take half of the room, A' the rest of it
    if (m) sg.entries(q.A, growA, mlo, mhi, matrices_first ? 2 : 1);
    sg.entries(q.At, growAt, nlo, nhi);
    sg.entries(q.P, growP, nlo, nhi);
  }
  if (matrices_first) streamed();
  pr = q;
  return true;
}

// Shared-memory staging for a direct solve (one CTA), in the room after the
// direct solver's workspace: the CSR row pointers of A, A' and P (every
// sparse-product row starts with them), then the QP's vectors in the order
// an ADMM iteration touches them -- z, y, the rho vector and its inverse, l,
// u, dy (m), x, q, dx (n) -- while they fit, then CSR entries of A', A and P
// while room remains.  The vectors are copied in (dir > 0) and back (dir <
// 0); row pointers and entries are copied in.  The layout is a pure function
// of the sizes, so the copy-back call recomputes it.
template <typename TT>
__device__ __forceinline__ bool stage_direct(DevProblem<TT>& pr, bool rho_vec, unsigned char* base, int cap, int dir,
                                             bool matrices) {
  Stager<TT> sg{base, cap, 0, dir};
  const int n = pr.n, m = pr.m;
  DevProblem<TT> q = pr;
  const int* growA = pr.A.rowptr;
  const int* growAt = pr.At.rowptr;
  const int* growP = pr.P.rowptr;
  if (m) q.A.rowptr = sg.rows(pr.A.rowptr, 0, m);
  q.At.rowptr = sg.rows(pr.At.rowptr, 0, n);
  q.P.rowptr = sg.rows(pr.P.rowptr, 0, n);
  if (m) {
    q.z = sg.span(pr.z, 0, m, true);
    q.y = sg.span(pr.y, 0, m, true);
    if (rho_vec) {
      q.rho_vec = sg.span(pr.rho_vec, 0, m, true);
      q.rho_inv_vec = sg.span(pr.rho_inv_vec, 0, m, true);
    }
    q.l = sg.span(pr.l, 0, m, true);
    q.u = sg.span(pr.u, 0, m, true);
    q.dy = sg.span(pr.dy, 0, m, true);
  }
  q.x = sg.span(pr.x, 0, n, true);
  q.q = sg.span(pr.q, 0, n, true);
  q.dx = sg.span(pr.dx, 0, n, true);
  if (matrices) {
    sg.entries(q.At, growAt, 0, n);
    if (m) sg.entries(q.A, growA, 0, m);
    sg.entries(q.P, growP, 0, n);
  }
  pr = q;
  return true;
}

// Contiguous slices of a QP's rows for rank r of a c-CTA cluster, balanced by
// estimated work: a row costs its entries plus 4 x (lanes per row), the
// entries a sub-warp could have processed in the row's fixed per-row work.
// n-space rows cost their P and A' entries, m-space rows their A entries.
// n-slice boundaries are rounded down to multiples of `align`.
template <typename TT>
__device__ Spans cluster_spans(const DevProblem<TT>& pr, int kktL, int r, int c, int align) {
  Spans sp;
  auto cut = [&](const int* r1, const int* r2, int rows, long long per_row, long long target) {
    int lo = 0, hi = rows;   // first row i with cost(i) >= target
    const long long b1 = r1[0], b2 = r2 ? r2[0] : 0;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      const long long cst = (r1[mid] - b1) + (r2 ? (r2[mid] - b2) : 0) + per_row * mid;
      if (cst < target) lo = mid + 1; else hi = mid;
    }
    return lo;
  };
  const long long wn = 4LL * kktL;
  const long long Fn = (pr.P.rowptr[pr.n] - pr.P.rowptr[0]) + (pr.At.rowptr[pr.n] - pr.At.rowptr[0]) + wn * pr.n;
  sp.nlo = r == 0 ? 0 : cut(pr.P.rowptr, pr.At.rowptr, pr.n, wn, Fn * r / c) / align * align;
  sp.nhi = r == c - 1 ? pr.n : cut(pr.P.rowptr, pr.At.rowptr, pr.n, wn, Fn * (r + 1) / c) / align * align;
  if (pr.m) {
    const long long wm = 4LL * pr.A.lanes;
    const long long Fm = (pr.A.rowptr[pr.m] - pr.A.rowptr[0]) + wm * pr.m;
    sp.mlo = r == 0 ? 0 : cut(pr.A.rowptr, nullptr, pr.m, wm, Fm * r / c);
    sp.mhi = r == c - 1 ? pr.m : cut(pr.A.rowptr, nullptr, pr.m, wm, Fm * (r + 1) / c);
  } else {
    sp.mlo = 0; sp.mhi = 0;
  }
  return sp;
}

// Work on one QP by a group (a CTA, or the CTAs of a cluster).  `dsm` /
// `dsm_bytes`: the CTA's dynamic shared memory for staged vectors.  A cluster
// solving with staged vectors works on contiguous row slices per CTA.  Solves
// run iterations it_lo..it_hi (gb_solver.cuh).
template <typename TT, typename G>
__device__ void batch_item(G& g, const BatchArrays<TT>& B, const DevSettings& s, int k, int mode,
                           GroupShared& gsh, SolverScalars& ssc, unsigned char* dsm, int dsm_bytes,
                           int it_lo, int it_hi, int stage_mat, KktPipe* kpipe = nullptr) {
  DevProblem<TT> pv = B.problem(k);
  if (threadIdx.x == 0) { gsh.parity = 0; gsh.flag = 0; if (mode != kModeSetup) ssc = *pv.st; }
  __syncthreads();
  bool staged = false;
  // direct KKT solve: the dynamic shared memory is the factorisation's and the
  // block solve's workspace (the QP's data stay in HBM / L2)
  const bool direct = kkt_direct(pv.kkt);
  int dstage = 0;   // direct solve: offset of the staged QP data in dsm (0: none)
  if (direct) {
    pv.kws = (TT*)dsm;
    pv.kpipe = kpipe;
    long long wsb;
    if (pv.kkt.dr > 0) {
      dr_on_chip(pv.kkt, (int*)(dsm + dr_ws_elems(pv.n, pv.m, pv.kkt.dr) * sizeof(TT)), pv.m);
      wsb = dr_ws_bytes(pv.n, pv.m, pv.kkt.dr, (int)sizeof(TT));
    } else {
      if (!kpipe) pv.kkt.ring = 0;
      kkt_plan_on_chip(pv.kkt, (int*)(dsm + kkt_ws_elems(pv.n, pv.m, pv.kkt.bmax, pv.kkt.segmax, pv.kkt.ring) * sizeof(TT)),
                       pv.n);
      wsb = kkt_ws_bytes(pv.n, pv.m, pv.kkt.bmax, pv.kkt.nb, pv.kkt.segmax, pv.kkt.ring, (int)sizeof(TT));
    }
    const int off = (int)((wsb + 15) & ~15LL);
    if (mode == kModeSolve && stage_mat >= 0 && off + 1024 < dsm_bytes) {
      dstage = off;
      staged = stage_direct(pv, s.rho_is_vec != 0, dsm + off, dsm_bytes - off, 1, stage_mat != 0);
    }
    __syncthreads();
  }
  if (mode == kModeSolve && dsm_bytes > 0 && !direct) {
    if constexpr (std::is_same<G, ClusterGroup>::value) {
      // block-Jacobi needs each block of r in one CTA: n-slices start on block boundaries
      g.sp = cluster_spans(pv, B.inst[k].kktL, (int)g.rank, (int)g.size,
                           s.cg_precond == kPrecondBlockDiagonal ? kPrecondBlock : 1);
      g.sliced = true;
    }
    staged = stage_problem(pv, g.sp, s.rho_is_vec != 0, dsm, dsm_bytes, 1, stage_mat != 0, stage_mat == 2);
    if constexpr (std::is_same<G, ClusterGroup>::value) g.repl = staged;
    g.sync();   // staged copies complete in every CTA before any peer writes them
  }
  Solver<TT> S{pv, s, &ssc, B.inst[k].kktL};
  if (mode == kModeSetup) {
    S.setup(g);
  } else if (mode == kModeSolve) {
    S.solve(g, it_lo, it_hi);
  } else if (mode == kModeUpdateMat) {
    // new P / A values already in Praw / Araw (osqp_api.c:1309-1409): values,
    // scaling (q, l, u re-scaled from their inputs) and preconditioner or
    // factor; rho and the iterates are kept
    S.prepare_data(g, true);
    if (threadIdx.x == 0) { ssc.status = ST_UNSOLVED; ssc.rho_updates = 0; }
  } else {
    // new q / l / u from *_in with the QP's existing scaling (osqp_api.c:1184-1257)
    const TT c = (TT)ssc.c;
    const bool sc_on = s.scaling != 0;
    const DevProblem<TT>& pr = pv;
    for_each(g, pr.n, [&](int i) { pr.q[i] = sc_on ? (pr.q_in[i] * pr.D[i]) * c : pr.q_in[i]; });
    for_each(g, pr.m, [&](int j) {
      pr.l[j] = sc_on ? pr.l_in[j] * pr.E[j] : pr.l_in[j];
      pr.u[j] = sc_on ? pr.u_in[j] * pr.E[j] : pr.u_in[j];
    });
    g.sync();
    if (s.rho_is_vec) {
      // the direct factor depends on the constraint types only through the
      // rho vector: refactor when a type changed
      __shared__ int s_changed;
      if (threadIdx.x == 0) s_changed = 0;
      g.sync();
      S.set_rho_vec(g, &s_changed);
      g.sync();
      if (!direct || s_changed) S.update_precond(g);
    }
    if (threadIdx.x == 0) { ssc.status = ST_UNSOLVED; ssc.rho_updates = 0; }
  }
  g.sync();
  if (staged) {
    DevProblem<TT> pb = B.problem(k);
    if (dstage) stage_direct(pb, s.rho_is_vec != 0, dsm + dstage, dsm_bytes - dstage, -1, stage_mat != 0);
    else stage_problem(pb, g.sp, s.rho_is_vec != 0, dsm, dsm_bytes, -1, stage_mat != 0, stage_mat == 2);
    g.sync();   // peers may still read this CTA's copies until here
  }
  if constexpr (std::is_same<G, ClusterGroup>::value) {
    g.sp = Spans{};
    g.sliced = false;
    g.repl = false;
  }
}

// Batch launch parameters shared by both kernels.  The queue holds `count`
// entries of `order`, or *count_dev entries when count_dev is set (a list
// built on the device by an earlier launch of the same stream).
struct BatchLaunch {
  int count;
  const int* count_dev;
  int* queue;
  const int* order;
  int mode;
  int it_lo, it_hi;   // solve window
  int dsm_bytes;      // dynamic shared memory for staged vectors
  int stage_mat;      // also stage matrix entries (whole, or a prefix of rows)
};

extern __shared__ __align__(16) unsigned char g_batch_dsm[];

// Persistent kernel, one CTA per QP: CTAs pull QPs from the queue.  NT
// threads per CTA, MINB CTAs per SM.
template <typename TT, int NT, int MINB>
__global__ void __launch_bounds__(NT, MINB)
k_batch(BatchArrays<TT> B, DevSettings s, BatchLaunch L) {
  __shared__ GroupShared gsh;
  __shared__ SolverScalars ssc;
  __shared__ int s_idx;
  __shared__ KktPipe kpipe;
  BlockGroup g{&gsh};
  kkt_pipe_init(&kpipe);
  const int count = L.count_dev ? *L.count_dev : L.count;
  for (;;) {
    if (threadIdx.x == 0) s_idx = atomicAdd(L.queue, 1);
    __syncthreads();
    const int idx = s_idx;
    __syncthreads();
    if (idx >= count) break;
    batch_item(g, B, s, L.order[idx], L.mode, gsh, ssc, g_batch_dsm, L.dsm_bytes, L.it_lo, L.it_hi,
               L.stage_mat, &kpipe);
    if (threadIdx.x == 0) *B.problem(L.order[idx]).st = ssc;
    __syncthreads();
  }
}

// Persistent kernel, one thread-block cluster per QP: the cluster's rank-0 CTA
// pulls a QP and broadcasts it through distributed shared memory.
template <typename TT, int NT>
__global__ void __launch_bounds__(NT, 1)
k_batch_cluster(BatchArrays<TT> B, DevSettings s, BatchLaunch L) {
  namespace cgr = cooperative_groups;
  __shared__ GroupShared gsh;
  __shared__ SolverScalars ssc;
  cgr::cluster_group cl = cgr::this_cluster();
  ClusterGroup g{&gsh, cl.block_rank(), cl.num_blocks()};
  const int count = L.count_dev ? *L.count_dev : L.count;
  for (;;) {
    if (g.rank == 0 && threadIdx.x == 0) gsh.cidx = atomicAdd(L.queue, 1);
    cl.sync();
    const int idx = *cl.map_shared_rank(&gsh.cidx, 0);
    cl.sync();   // rank 0 keeps its shared memory until every CTA has read idx
    if (idx >= count) break;
    batch_item(g, B, s, L.order[idx], L.mode, gsh, ssc, g_batch_dsm, L.dsm_bytes, L.it_lo, L.it_hi,
               L.stage_mat);
    if (g.rank == 0 && threadIdx.x == 0) *B.problem(L.order[idx]).st = ssc;
    cl.sync();
  }
}

// The QPs of `order` whose solve is suspended (status still ST_UNSOLVED after
// a windowed launch), in queue order, and their count.  One CTA.
__global__ void k_batch_unfinished(const SolverScalars* st, const int* order, int count, int* order2,
                                   int* count2) {
  __shared__ int wtot[32];
  __shared__ int base;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if (threadIdx.x == 0) base = 0;
  __syncthreads();
  for (int c0 = 0; c0 < count; c0 += blockDim.x) {
    const int i = c0 + threadIdx.x;
    const int k = i < count ? order[i] : -1;
    const bool f = k >= 0 && st[k].status == ST_UNSOLVED;
    const unsigned bal = __ballot_sync(0xffffffffu, f);
    if (lane == 0) wtot[w] = __popc(bal);
    __syncthreads();
    int off = base;
    for (int q = 0; q < w; q++) off += wtot[q];
    if (f) order2[off + __popc(bal & ((1u << lane) - 1u))] = k;
    __syncthreads();
    if (threadIdx.x == 0) { int t = 0; for (int q = 0; q < nw; q++) t += wtot[q]; base += t; }
    __syncthreads();
  }
  if (threadIdx.x == 0) *count2 = base;
}

// ---- structure kernels (one CTA per QP) ----
// A entries: sort key = batch-global row, plus the entry's local column.
__global__ void k_batch_A_keys(const BatchInst* inst, int count, const int* Ap_all, const int* ap_off,
                               const int* Ai, int* keys, int* cols, int* Atrow) {
  for (int k = blockIdx.x; k < count; k += gridDim.x) {
    const BatchInst b = inst[k];
    const int* Ap = Ap_all + ap_off[k];
    for (int j = threadIdx.x; j < b.n; j += blockDim.x) {
      Atrow[b.n_off + j] = b.a_off + Ap[j];
      for (int e = Ap[j]; e < Ap[j + 1]; e++) {
        keys[b.a_off + e] = b.m_off + Ai[b.a_off + e];
        cols[b.a_off + e] = j;
      }
    }
  }
}

// Symmetric expansion of each QP's triu P with keys (global_row << 32 | local_col).
__global__ void k_batch_P_keys(const BatchInst* inst, int count, const int* Pp_all, const int* pp_off,
                               const int* Pi, int nnzT_total, unsigned long long* keys, int* src) {
  for (int k = blockIdx.x; k < count; k += gridDim.x) {
    const BatchInst b = inst[k];
    const int* Pp = Pp_all + pp_off[k];
    for (int j = threadIdx.x; j < b.n; j += blockDim.x) {
      bool has_diag = false;
      for (int e = Pp[j]; e < Pp[j + 1]; e++) {
        const int ge = b.pt_off + e;
        const int i = Pi[ge];
        keys[ge] = ((unsigned long long)(b.n_off + i) << 32) | (unsigned)j;
        src[ge] = ge;
        if (i == j) {
          has_diag = true;
          keys[nnzT_total + ge] = ~0ull;
          src[nnzT_total + ge] = -1;
        } else {
          keys[nnzT_total + ge] = ((unsigned long long)(b.n_off + j) << 32) | (unsigned)i;
          src[nnzT_total + ge] = ge;
        }
      }
      keys[2 * nnzT_total + b.n_off + j] = has_diag ? ~0ull : (((unsigned long long)(b.n_off + j) << 32) | (unsigned)j);
      src[2 * nnzT_total + b.n_off + j] = -1;
    }
  }
}

__global__ void k_batch_P_from_sorted(const unsigned long long* keys, int nnzF, int rows, int* col, int* rowptr) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k <= nnzF; k += gridDim.x * blockDim.x) {
    if (k < nnzF) col[k] = (int)(keys[k] & 0xffffffffu);   // diagonals: k_batch_P_diag
    const int prev = (k == 0) ? -1 : (int)(keys[k - 1] >> 32);
    const int cur = (k == nnzF) ? rows : (int)(keys[k] >> 32);
    for (int r = prev + 1; r <= cur; r++) rowptr[r] = k;
  }
}

// Diagonal positions: for every QP row, the entry whose local column equals the local row.
__global__ void k_batch_P_diag(const BatchInst* inst, int count, const int* rowptr, const int* col, int* diag) {
  for (int k = blockIdx.x; k < count; k += gridDim.x) {
    const BatchInst b = inst[k];
    for (int i = threadIdx.x; i < b.n; i += blockDim.x) {
      const int gr = b.n_off + i;
      for (int e = rowptr[gr]; e < rowptr[gr + 1]; e++)
        if (col[e] == i) { diag[gr] = e; break; }
    }
  }
}

template <typename TT>
__global__ void k_batch_check_bounds(const TT* l, const TT* u, long long msum, int* bad) {
  for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < msum; j += (long long)gridDim.x * blockDim.x)
    if (l[j] > u[j]) atomicExch(bad, 1);
}

template <typename TT>
__global__ void k_batch_scatter_vals(TT* dst, const TT* src, const int* idx, int cnt) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < cnt; k += gridDim.x * blockDim.x)
    dst[idx ? idx[k] : k] = src[k];
}

struct BatchInfo { int status, iter; long long pcg; double obj, prim, dual, seconds; int rho_updates, pad; };

__global__ void k_batch_info(const SolverScalars* st, int count, BatchInfo* out, long long* totals) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < count; k += gridDim.x * blockDim.x) {
    out[k].status = st[k].status;
    out[k].iter = st[k].iter;
    out[k].pcg = st[k].pcg_iters_total;
    out[k].obj = st[k].obj_val;
    out[k].prim = st[k].prim_res;
    out[k].dual = st[k].dual_res;
    out[k].seconds = st[k].elapsed;
    out[k].rho_updates = st[k].rho_updates;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    long long a = 0, p = 0;
    for (int k = 0; k < count; k++) { a += st[k].iter; p += st[k].pcg_iters_total; }
    totals[0] = a; totals[1] = p;
    for (int q = 0; q < kProfSlots; q++) {
      unsigned long long c = 0;
      for (int k = 0; k < count; k++) c += st[k].prof[q];
      totals[2 + q] = (long long)c;
    }
  }
}

// Results of the QPs listed in order[0..count) (serving launches).
__global__ void k_serve_info(const SolverScalars* st, const int* order, int count, BatchInfo* out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
    const SolverScalars& c = st[order[i]];
    out[i].status = c.status;
    out[i].iter = c.iter;
    out[i].pcg = c.pcg_iters_total;
    out[i].obj = c.obj_val;
    out[i].prim = c.prim_res;
    out[i].dual = c.dual_res;
  }
}

}  // namespace gbb

using namespace gbb;

typedef void (*BatchKernel)(BatchArrays<T>, DevSettings, BatchLaunch);

static int env_int(const char* name, int dflt);

// The CTA form's kernel: 1024 threads x 1 per SM, 512 x 2, or 512 x 1 (128
// registers per thread), from OSQP_GB300_BATCH_THREADS and
// OSQP_GB300_BATCH_CTAS_PER_SM.  Defaults measured on 4096 batched MPC QPs
// (one box, alternating): the PCG runs 1024 x 1 (512 x 2: -7 %); the direct
// solver runs 512 x 1 (against 1024 x 1: +4.7 % FP64, +6.7 % FP32; its block
// solve uses a few warps, and the sparse products of the FP64 build are bound
// by the FP64 pipe rather than by the number of warps; 768 x 1, 80 registers,
// 8 lanes per block row: -25 % FP64, -2.5 % FP32).
static void cta_form(bool direct, BatchKernel* fn, int* nt, int* minb) {
  const int threads = env_int("OSQP_GB300_BATCH_THREADS", direct ? 512 : 1024);
  const int per_sm = env_int("OSQP_GB300_BATCH_CTAS_PER_SM", direct ? 1 : 2);
  if (threads >= 1024) { *fn = k_batch<T, 1024, 1>; *nt = 1024; *minb = 1; }
  else if (per_sm == 1) { *fn = k_batch<T, kBatchThreads, 1>; *nt = kBatchThreads; *minb = 1; }
  else { *fn = k_batch<T, kBatchThreads, 2>; *nt = kBatchThreads; *minb = 2; }
}
// The cluster form's kernel for a CTA size (one CTA per SM).
static void cluster_form(int threads, BatchKernel* fn, int* nt) {
  if (threads >= 1024) { *fn = k_batch_cluster<T, 1024>; *nt = 1024; }
  else { *fn = k_batch_cluster<T, kBatchThreads>; *nt = kBatchThreads; }
}

// Largest dynamic shared memory per CTA (whole KiB, at most cap_bytes) that
// keeps minb CTAs of the kernel resident per SM; 0 if none.
static int configure_dsm(BatchKernel fn, int threads, int minb, int device, long cap_bytes) {
  cudaFuncAttributes fa;
  if (cudaFuncGetAttributes(&fa, fn) != cudaSuccess) return 0;
  int smem_sm = 0, reserved = 0, optin = 0;
  cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, device);
  cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, device);
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
  long per_cta = (long)smem_sm / minb - reserved - (long)fa.sharedSizeBytes;
  per_cta = std::min(per_cta, (long)optin - (long)fa.sharedSizeBytes);
  if (cap_bytes >= 0) per_cta = std::min(per_cta, cap_bytes);
  per_cta &= ~1023L;
  while (per_cta > 0) {
    if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)per_cta) == cudaSuccess) {
      int nb = 0;
      if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, threads, (size_t)per_cta) == cudaSuccess &&
          nb >= minb)
        break;
    }
    per_cta -= 1024;
  }
  cudaGetLastError();
  return (int)std::max(per_cta, 0L);
}

// SpMV tile of every QP: lanes per row for P, A, A' and the fused P / A'
// pass, from the mean row length and the target entries per lane.  The
// default target was measured on batched MPC (one box, alternating): 1 -> 315,
// 2 -> 401, 4 -> 521, 8 -> 546, 16 -> 430, 32 -> 260 solves/s;
// osqp_gb300_batch_autotune picks it per batch by timing.
constexpr int kDefaultPerLane = 8;

static void assign_lanes(OSQPBatch_* b, int per_lane);

static int env_int(const char* name, int dflt) {
  const char* e = getenv(name);
  return (e && *e) ? atoi(e) : dflt;
}

struct OSQPBatch_ {
  int count, device;
  int direct;             // linsys_solver = direct: every QP has a KKT plan
  long long kf_total;     // direct: factor elements of the whole batch
  long long kc_total;     // direct, dense-row form: inverse capacitance elements of the whole batch
  long long nsum, msum, nnzT, nnzA, nnzPf;
  size_t binv_elems;    // block-Jacobi storage (0 unless cg_precond = 2)
  cudaStream_t stream;
  cudaEvent_t ev0, ev1, evu;
  int upd_pending;
  char* arena;
  BatchArrays<T> B;
  BatchInst* d_inst;
  int* d_order;
  int* d_queue;
  int* d_flag;
  BatchInfo* d_info;
  long long* d_totals;
  T *stage_q, *stage_l, *stage_u;
  DevSettings ds;
  OSQPSettings settings;
  int grid;
  int cluster;   // 0: one CTA per QP (k_batch); c >= 1: clusters of c CTAs per QP
  BatchKernel kfn;        // CTA form: k_batch instantiation
  int threads;            // CTA form: threads per CTA
  int dsm;                // CTA form: dynamic shared memory per CTA for staged vectors (solves)
  BatchKernel cfn;        // cluster forms (main and tail): k_batch_cluster instantiation
  int cthreads, cdsm;     // cluster forms: threads and dynamic shared memory per CTA
  int split;              // ADMM iteration after which unfinished QPs move to the tail form (0: never)
  int tail_cluster, tail_grid;   // tail form: CTAs per QP and resident clusters
  int *d_order2, *d_count2, *d_queue2;
  int stage_mat;          // stage matrix entries on chip when they (partly) fit
  int per_lane;           // SpMV tile: target entries per lane of a row's sub-warp
  std::vector<long long> nnzT_k, nnzA_k;   // per QP: entries of triu(P) and of A
  std::vector<int> order_h;                 // host copy of the queue order
  std::vector<long long> work_h;            // per QP: entries + rows (cost of one pass)
  int reorder;            // order the queue by the last solve's measured work
  float last_ms, last_step_ms;
  long long last_admm, last_pcg;
  std::vector<BatchInst> inst;
};

static void assign_lanes(OSQPBatch_* b, int per_lane) {
  for (int k = 0; k < b->count; k++) {
    BatchInst& I = b->inst[k];
    const long long nPf_est = 2 * b->nnzT_k[k] + I.n;   // lane choice only needs the mean row length
    const long long nA = b->nnzA_k[k];
    I.PL = pick_lanes(nPf_est, I.n, per_lane);
    I.AL = pick_lanes(nA, I.m, per_lane);
    I.AtL = pick_lanes(nA, I.n, per_lane);
    I.kktL = pick_lanes(nPf_est + nA, I.n, per_lane);
  }
  b->per_lane = per_lane;
}

// settings translation shared with the single-QP engine
static DevSettings batch_dev_settings(const OSQPSettings* st) {
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
  d.profile = env_int("OSQP_GB300_PROFILE", 0) != 0;
  return d;
}

// Device work list of one launch: `count` instances in `order`, plus the
// launch's own queue counters and tail list, so launches over disjoint
// instance sets can run concurrently on different streams.
struct LaunchBufs {
  const int* order;
  int count;
  int* queue;     // [3]: main queue, tail queue, tail count
  int* order2;    // [count] tail list
};

// allow_split = false keeps every QP of the launch in the first form: a
// serving launch must not wait for a whole cluster of idle SMs while other
// launches occupy the GPU.
// it_stop > 0: stop every QP after that many ADMM iterations (suspended, as
// at a split, but without a tail launch).
static int launch_batch(OSQPBatch* b, int mode, const LaunchBufs& lb, cudaStream_t st, bool allow_split = true,
                        int it_stop = 0) {
  int* q1 = lb.queue;
  int* q2 = lb.queue + 1;
  int* c2 = lb.queue + 2;
  BT_TRY(cudaMemsetAsync(lb.queue, 0, 3 * sizeof(int), st));
  BatchLaunch L{lb.count, nullptr, q1, lb.order, mode, 1, 0x7fffffff, 0, b->stage_mat};
  const bool split = allow_split && mode == kModeSolve && b->split > 0 && b->split < b->ds.max_iter &&
                     b->cluster < b->tail_cluster;
  if (split) L.it_hi = b->split;
  if (it_stop > 0 && !split) L.it_hi = it_stop;
  const int grid = std::max(1, std::min(lb.count, b->grid));   // a small launch leaves SMs to others
  if (b->cluster >= 1) {
    L.dsm_bytes = mode == kModeSolve ? b->cdsm : 0;
    BT_TRY(launch_clusters_dsm(b->cfn, grid, b->cluster, b->cthreads, (size_t)b->cdsm, st, b->B, b->ds, L));
  } else {
    // the direct solver factors in every mode (set-up, updates, solves)
    L.dsm_bytes = (mode == kModeSolve || b->direct) ? b->dsm : 0;
    b->kfn<<<grid, b->threads, (size_t)L.dsm_bytes, st>>>(b->B, b->ds, L);
    BT_TRY(cudaGetLastError());
  }
  if (split) {
    // QPs still running after `split` iterations continue, from where they
    // stopped, with a cluster of CTAs each: the slowest QPs set the makespan
    k_batch_unfinished<<<1, 1024, 0, st>>>(b->B.st, lb.order, lb.count, lb.order2, c2);
    BT_TRY(cudaGetLastError());
    BatchLaunch T2{0, c2, q2, lb.order2, kModeSolve, b->split + 1, 0x7fffffff, 0, b->stage_mat};
    const int tgrid = std::max(1, std::min(lb.count, b->tail_grid));
    if (b->tail_cluster >= 1) {
      T2.dsm_bytes = b->cdsm;
      BT_TRY(launch_clusters_dsm(b->cfn, tgrid, b->tail_cluster, b->cthreads, (size_t)b->cdsm, st,
                                 b->B, b->ds, T2));
    } else {
      T2.dsm_bytes = b->dsm;
      b->kfn<<<grid, b->threads, (size_t)b->dsm, st>>>(b->B, b->ds, T2);
      BT_TRY(cudaGetLastError());
    }
  }
  return 0;
}

static int run_batch_kernel(OSQPBatch* b, int mode) {
  LaunchBufs lb{b->d_order, b->count, b->d_queue2, b->d_order2};
  return launch_batch(b, mode, lb, b->stream);
}

extern "C" OSQPInt osqp_gb300_batch_cleanup(OSQPBatch* b) {
  if (!b) return 0;
  if (b->arena) cudaFree(b->arena);
  if (b->ev0) cudaEventDestroy(b->ev0);
  if (b->ev1) cudaEventDestroy(b->ev1);
  if (b->evu) cudaEventDestroy(b->evu);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
  return 0;
}

extern "C" OSQPInt osqp_gb300_batch_setup(OSQPBatch** batchp, OSQPInt count, const OSQPInt* n, const OSQPInt* m,
                                          const OSQPInt* Pp, const OSQPInt* Pi, const OSQPFloat* Px,
                                          const OSQPInt* Ap, const OSQPInt* Ai, const OSQPFloat* Ax,
                                          const OSQPFloat* q, const OSQPFloat* l, const OSQPFloat* u,
                                          const OSQPSettings* settings) {
  if (!batchp || count <= 0 || !n || !m || !Pp || !Ap || !q || !settings) return OSQP_DATA_VALIDATION_ERROR;
  *batchp = NULL;
  if (settings->linsys_solver != OSQP_INDIRECT_SOLVER && settings->linsys_solver != OSQP_DIRECT_SOLVER)
    return OSQP_SETTINGS_VALIDATION_ERROR;
  if (settings->alpha <= 0 || settings->alpha >= 2 || settings->rho <= 0 || settings->sigma <= 0 ||
      settings->max_iter <= 0 || settings->adaptive_rho == OSQP_ADAPTIVE_RHO_UPDATE_TIME)
    return OSQP_SETTINGS_VALIDATION_ERROR;
  if (cudaSetDevice(settings->device) != cudaSuccess) return OSQP_ALGEBRA_LOAD_ERROR;

  OSQPBatch* b = new OSQPBatch_();
  b->count = count;
  b->device = settings->device;
  b->settings = *settings;
  OSQPSettings& st = b->settings;
  st.rho = (OSQPFloat)fmin(fmax((double)st.rho, 1e-6), 1e6);
  if (st.adaptive_rho == OSQP_ADAPTIVE_RHO_UPDATE_ITERATIONS && st.adaptive_rho_interval == 0)
    st.adaptive_rho_interval = st.check_termination ? OSQP_ADAPTIVE_RHO_MULTIPLE_TERMINATION * st.check_termination
                                                    : OSQP_ADAPTIVE_RHO_FIXED;
  if (st.adaptive_rho == OSQP_ADAPTIVE_RHO_UPDATE_KKT_ERROR && st.adaptive_rho_interval == 0)
    st.adaptive_rho_interval = 1;
  b->ds = batch_dev_settings(&st);

  // ---- host-side sizes and offsets ----
  std::vector<OSQPInt> hn(count), hm(count);
  if (cudaMemcpy(hn.data(), n, sizeof(OSQPInt) * count, cudaMemcpyDefault) != cudaSuccess ||
      cudaMemcpy(hm.data(), m, sizeof(OSQPInt) * count, cudaMemcpyDefault) != cudaSuccess) {
    delete b; return OSQP_DATA_VALIDATION_ERROR;
  }
  long long nsum = 0, msum = 0, colptr_len = 0;
  for (int k = 0; k < count; k++) {
    if (hn[k] <= 0 || hm[k] < 0) { delete b; return OSQP_DATA_VALIDATION_ERROR; }
    nsum += hn[k]; msum += hm[k]; colptr_len += hn[k] + 1;
  }
  std::vector<OSQPInt> hPp(colptr_len), hAp(colptr_len);
  if (cudaMemcpy(hPp.data(), Pp, sizeof(OSQPInt) * colptr_len, cudaMemcpyDefault) != cudaSuccess ||
      cudaMemcpy(hAp.data(), Ap, sizeof(OSQPInt) * colptr_len, cudaMemcpyDefault) != cudaSuccess) {
    delete b; return OSQP_DATA_VALIDATION_ERROR;
  }
  b->inst.resize(count);
  std::vector<int> pp_off(count), work(count);
  long long no = 0, mo = 0, pto = 0, ao = 0, co = 0, blk = 0;
  for (int k = 0; k < count; k++) {
    BatchInst& I = b->inst[k];
    I.n = hn[k]; I.m = hm[k]; I.n_off = (int)no; I.m_off = (int)mo; I.pt_off = (int)pto; I.a_off = (int)ao;
    I.blk_off = (int)blk;
    blk += (hn[k] + kPrecondBlock - 1) / kPrecondBlock;
    pp_off[k] = (int)co;
    const int nT = hPp[co + hn[k]], nA = hAp[co + hn[k]];
    no += hn[k]; mo += hm[k]; pto += nT; ao += nA; co += hn[k] + 1;
    work[k] = 2 * nT + 2 * nA + hn[k] + hm[k];
  }
  if (pto > INT32_MAX / 2 || ao > INT32_MAX || no > INT32_MAX / 2) { delete b; return OSQP_DATA_VALIDATION_ERROR; }
  b->nsum = nsum; b->msum = msum; b->nnzT = pto; b->nnzA = ao;
  b->binv_elems = b->ds.cg_precond == kPrecondBlockDiagonal ? (size_t)blk * kPrecondBlock * kPrecondBlock : 0;
  // diagonal count of P (host scan of the triu pattern) -> full-P size
  std::vector<OSQPInt> hPi(pto > 0 ? pto : 1);
  if (pto && cudaMemcpy(hPi.data(), Pi, sizeof(OSQPInt) * pto, cudaMemcpyDefault) != cudaSuccess) { delete b; return OSQP_DATA_VALIDATION_ERROR; }
  long long ndiag = 0;
  for (int k = 0; k < count; k++) {
    BatchInst& I = b->inst[k];
    const OSQPInt* P = hPp.data() + pp_off[k];
    int only_diag = 1;
    for (int j = 0; j < I.n; j++) {
      for (int e = P[j]; e < P[j + 1]; e++) {
        const OSQPInt r = hPi[I.pt_off + e];
        if (r > j) { delete b; return OSQP_DATA_VALIDATION_ERROR; }   // P must be upper triangular
        if (r != j) only_diag = 0;
      }
      for (int e = P[j]; e < P[j + 1]; e++)
        if (hPi[I.pt_off + e] == j) { ndiag++; break; }
    }
    I.Pdiag_only = only_diag;
  }
  b->nnzPf = 2 * pto - 2 * ndiag + nsum;
  b->nnzT_k.resize(count); b->nnzA_k.resize(count);
  for (int k = 0; k < count; k++) {
    const OSQPInt* P = hPp.data() + pp_off[k];
    const OSQPInt* A = hAp.data() + pp_off[k];
    b->nnzT_k[k] = P[b->inst[k].n];
    b->nnzA_k[k] = A[b->inst[k].n];
  }
  b->per_lane = std::max(1, std::min(64, env_int("OSQP_GB300_LANE_TARGET", kDefaultPerLane)));
  assign_lanes(b, b->per_lane);
  std::vector<int> order(count);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int c) { return work[a] > work[c]; });

  // ---- direct KKT solve: symbolic analysis of every QP on the host ----
  b->direct = st.linsys_solver == OSQP_DIRECT_SOLVER;
  const int cap_kib0 = env_int("OSQP_GB300_BATCH_SMEM_KIB", -1);
  std::vector<KktPlan> plans;
  std::vector<DrPlan> drplans;
  long long kb_tot = 0, kcr_tot = 0, kf_tot = 0, kdr_tot = 0, kc_tot = 0;
  if (b->direct) {
    // the factorisation and the block solve work in the CTA's shared memory
    int minb0 = 1;
    cta_form(true, &b->kfn, &b->threads, &minb0);
    b->dsm = configure_dsm(b->kfn, b->threads, minb0, b->device, cap_kib0 < 0 ? -1L : 1024L * cap_kib0);
    const int blim = kkt_bmax_limit(b->threads, b->dsm, (int)sizeof(T));
    std::vector<OSQPInt> hAi(ao > 0 ? ao : 1);
    if (ao && cudaMemcpy(hAi.data(), Ai, sizeof(OSQPInt) * ao, cudaMemcpyDefault) != cudaSuccess) { delete b; return OSQP_DATA_VALIDATION_ERROR; }
    plans.resize(count);
    drplans.resize(count);
    // ring slots of the block solve's copy pipeline: deeper rings measured no
    // faster, and the room they leave holds the QP's vectors on chip
    const int ring_max = std::max(2, std::min(kKktRingMax, env_int("OSQP_GB300_KKT_RING_SLOTS", 4)));
    std::vector<int> prc(count, 0), ring(count, 0);
    const int nthr = std::max(1, std::min((int)std::thread::hardware_concurrency(), std::min(count, 64)));
    std::vector<std::thread> pool;
    for (int t = 0; t < nthr; t++)
      pool.emplace_back([&, t]() {
        for (int k = t; k < count; k += nthr) {
          const BatchInst& I = b->inst[k];
          prc[k] = kkt_plan_build(I.n, I.m, hPp.data() + pp_off[k], hPi.data() + I.pt_off, hAp.data() + pp_off[k],
                                  hAi.data() + I.a_off, blim, plans[k]);
          if (prc[k] == 1 && sizeof(T) == 8) {
            // no block ordering within the limit: the diagonal-plus-dense-rows
            // form, with as many dense rows as its workspace allows.  FP64
            // build only: with FP32 iterates its solves left factor-model
            // portfolios at 1.5-8x the builtin's ADMM iterations (some not
            // converging), so the FP32 build keeps the PCG for such QPs
            int rmax = 0;
            while (rmax < kDrMaxRows && dr_ws_bytes(I.n, I.m, rmax + 1, (int)sizeof(T)) <= b->dsm) rmax++;
            if (!dr_plan_build(I.n, I.m, hPp.data() + pp_off[k], hPi.data() + I.pt_off, hAp.data() + pp_off[k],
                               hAi.data() + I.a_off, rmax, drplans[k])) {
              prc[k] = 0;
              plans[k] = KktPlan();
              continue;
            }
          }
          if (!prc[k]) {
            // ring slots of the solve's bulk-copy pipeline: as many as fit (at least 2), else none
            int R = ring_max;
            while (R >= 2 && kkt_ws_bytes(I.n, I.m, plans[k].bmax, plans[k].nb, plans[k].segmax, R, (int)sizeof(T)) > b->dsm) R--;
            if (R < 2) R = 0;
            if (kkt_ws_bytes(I.n, I.m, plans[k].bmax, plans[k].nb, plans[k].segmax, R, (int)sizeof(T)) > b->dsm) prc[k] = 3;
            ring[k] = R;
          }
        }
      });
    for (auto& th : pool) th.join();
    for (int k = 0; k < count; k++) {
      if (prc[k]) {
        fprintf(stderr, "osqp_gb300 batch: direct KKT solve does not apply to QP %d (n=%d, m=%d): %s "
                "(at most %d variables per block, %d bytes of shared memory per CTA)\n", k,
                b->inst[k].n, b->inst[k].m,
                prc[k] == 1 ? "a block of its block-tridiagonal ordering exceeds the on-chip limit"
                : prc[k] == 3 ? "its solve vectors exceed the on-chip workspace" : "inconsistent structure",
                blim, b->dsm);
        delete b;
        return OSQP_LINSYS_SOLVER_INIT_ERROR;
      }
      BatchInst& I = b->inst[k];
      I.kdr = drplans[k].r; I.kdr_off = (int)kdr_tot; I.kc_off = kc_tot;
      kdr_tot += drplans[k].r; kc_tot += (long long)drplans[k].r * drplans[k].r;
      I.knb = plans[k].nb; I.kbmax = plans[k].bmax;
      I.kring = env_int("OSQP_GB300_KKT_RING", 1) ? ring[k] : 0; I.ksegmax = plans[k].segmax;
      I.kb_off = (int)kb_tot; I.kcr_off = (int)kcr_tot; I.kf_off = kf_tot;
      if (I.kdr == 0) { kb_tot += plans[k].nb + 1; kcr_tot += (long long)plans[k].cr.size(); kf_tot += plans[k].fsize; }
    }
    if (kb_tot > INT32_MAX || kcr_tot > INT32_MAX) { delete b; return OSQP_DATA_VALIDATION_ERROR; }
    b->kf_total = kf_tot;
    b->kc_total = kc_tot;
  } else {
    for (int k = 0; k < count; k++) {
      BatchInst& I = b->inst[k];
      I.knb = 0; I.kbmax = 0; I.kb_off = 0; I.kcr_off = 0; I.kf_off = 0; I.kring = 0; I.ksegmax = 0;
      I.kdr = 0; I.kdr_off = 0; I.kc_off = 0;
    }
  }

  // ---- arena ----
  if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&b->ev0) != cudaSuccess || cudaEventCreate(&b->ev1) != cudaSuccess ||
      cudaEventCreate(&b->evu) != cudaSuccess) {
    osqp_gb300_batch_cleanup(b); return OSQP_ALGEBRA_LOAD_ERROR;
  }
  struct Plan { size_t off = 0; size_t take(size_t bytes) { off = (off + 255) & ~size_t(255); size_t o = off; off += bytes > 0 ? bytes : 1; return o; } } pl;
  const long long nPf = b->nnzPf;
  size_t o_Prow = pl.take(sizeof(int) * (nsum + 1)), o_Pcol = pl.take(sizeof(int) * nPf), o_Pdiag = pl.take(sizeof(int) * nsum);
  size_t o_Psrc = pl.take(sizeof(int) * nPf), o_Pval = pl.take(sizeof(T) * nPf), o_Praw = pl.take(sizeof(T) * pto);
  size_t o_Arow = pl.take(sizeof(int) * (msum + 1)), o_Acol = pl.take(sizeof(int) * ao), o_Asrc = pl.take(sizeof(int) * ao);
  size_t o_Atrow = pl.take(sizeof(int) * (nsum + 1)), o_Atcol = pl.take(sizeof(int) * ao);
  size_t o_Aval = pl.take(sizeof(T) * ao), o_Araw = pl.take(sizeof(T) * ao), o_Atval = pl.take(sizeof(T) * ao);
  size_t o_vn[16], o_vm[16];
  for (int k = 0; k < 16; k++) o_vn[k] = pl.take(sizeof(T) * nsum);
  for (int k = 0; k < 16; k++) o_vm[k] = pl.take(sizeof(T) * msum);
  size_t o_ctype = pl.take(sizeof(int) * msum), o_st = pl.take(sizeof(SolverScalars) * count);
  size_t o_inst = pl.take(sizeof(BatchInst) * count), o_order = pl.take(sizeof(int) * count);
  size_t o_order2 = pl.take(sizeof(int) * count);
  size_t o_misc = pl.take(sizeof(int) * 8), o_info = pl.take(sizeof(BatchInfo) * count), o_tot = pl.take(sizeof(long long) * (2 + kProfSlots));
  size_t o_sq = pl.take(sizeof(T) * nsum), o_sl = pl.take(sizeof(T) * msum), o_su = pl.take(sizeof(T) * msum);
  size_t o_binv = pl.take(sizeof(T) * b->binv_elems);
  size_t o_kperm = pl.take(sizeof(int) * (b->direct ? nsum : 0)), o_kiperm = pl.take(sizeof(int) * (b->direct ? nsum : 0));
  size_t o_kbs = pl.take(sizeof(int) * kb_tot), o_kfo = pl.take(sizeof(int) * kb_tot), o_kco = pl.take(sizeof(int) * kb_tot);
  size_t o_kbo = pl.take(sizeof(int) * kb_tot);
  size_t o_kcr = pl.take(sizeof(int) * kcr_tot), o_kF = pl.take(sizeof(T) * kf_tot);
  size_t o_kdrows = pl.take(sizeof(int) * kdr_tot), o_kdidx = pl.take(sizeof(int) * (kdr_tot ? msum : 0));
  size_t o_kCinv = pl.take(sizeof(T) * kc_tot), o_kDginv = pl.take(sizeof(T) * (kdr_tot ? nsum : 0));
  {
    // admission by free device memory: refuse (rather than fail part-way)
    // when the pool and the set-up scratch would not fit
    size_t fr = 0, tot = 0;
    const size_t scratch = (size_t)(2 * pto + nsum) * 24 + (size_t)ao * 16 + (64u << 20);
    if (cudaMemGetInfo(&fr, &tot) == cudaSuccess && pl.off + scratch > fr) {
      osqp_gb300_batch_cleanup(b);
      return OSQP_MEM_ALLOC_ERROR;
    }
  }
  if (cudaMalloc(&b->arena, pl.off) != cudaSuccess) { osqp_gb300_batch_cleanup(b); return OSQP_MEM_ALLOC_ERROR; }
  char* a = b->arena;
  cudaStream_t s = b->stream;
  BT_TRY(cudaMemsetAsync(a, 0, pl.off, s));
  BatchArrays<T>& B = b->B;
  B.Prow = (int*)(a + o_Prow); B.Pcol = (int*)(a + o_Pcol); B.Pdiag = (int*)(a + o_Pdiag); B.Psrc = (int*)(a + o_Psrc);
  B.Pval = (T*)(a + o_Pval); B.Praw = (T*)(a + o_Praw);
  B.Arow = (int*)(a + o_Arow); B.Acol = (int*)(a + o_Acol); B.Asrc = (int*)(a + o_Asrc);
  B.Atrow = (int*)(a + o_Atrow); B.Atcol = (int*)(a + o_Atcol);
  B.Aval = (T*)(a + o_Aval); B.Araw = (T*)(a + o_Araw); B.Atval = (T*)(a + o_Atval);
  for (int k = 0; k < 16; k++) { B.vn[k] = (T*)(a + o_vn[k]); B.vm[k] = (T*)(a + o_vm[k]); }
  B.ctype = (int*)(a + o_ctype); B.st = (SolverScalars*)(a + o_st);
  B.Binv = b->binv_elems ? (T*)(a + o_binv) : nullptr;
  B.kperm = (int*)(a + o_kperm); B.kiperm = (int*)(a + o_kiperm);
  B.kbs = (int*)(a + o_kbs); B.kfo = (int*)(a + o_kfo); B.kco = (int*)(a + o_kco); B.kcr = (int*)(a + o_kcr);
  B.kbo = (int*)(a + o_kbo);
  B.kF = (T*)(a + o_kF);
  B.kdrows = (int*)(a + o_kdrows); B.kdidx = (int*)(a + o_kdidx);
  B.kCinv = (T*)(a + o_kCinv); B.kDginv = (T*)(a + o_kDginv);
  b->d_inst = (BatchInst*)(a + o_inst); B.inst = b->d_inst;
  b->d_order = (int*)(a + o_order);
  b->d_queue = (int*)(a + o_misc); b->d_flag = b->d_queue + 1;
  b->d_queue2 = b->d_queue + 2; b->d_count2 = b->d_queue + 4; b->d_order2 = (int*)(a + o_order2);
  b->d_info = (BatchInfo*)(a + o_info); b->d_totals = (long long*)(a + o_tot);
  b->stage_q = (T*)(a + o_sq); b->stage_l = (T*)(a + o_sl); b->stage_u = (T*)(a + o_su);

  BT_TRY(cudaMemcpyAsync(b->d_inst, b->inst.data(), sizeof(BatchInst) * count, cudaMemcpyHostToDevice, s));
  BT_TRY(cudaMemcpyAsync(b->d_order, order.data(), sizeof(int) * count, cudaMemcpyHostToDevice, s));
  b->order_h = order;
  b->work_h.assign(work.begin(), work.end());
  if (pto) BT_TRY(cudaMemcpyAsync(B.Praw, Px, sizeof(T) * pto, cudaMemcpyDefault, s));
  if (ao) BT_TRY(cudaMemcpyAsync(B.Araw, Ax, sizeof(T) * ao, cudaMemcpyDefault, s));
  BT_TRY(cudaMemcpyAsync(B.vn[1], q, sizeof(T) * nsum, cudaMemcpyDefault, s));
  if (msum) {
    BT_TRY(cudaMemcpyAsync(B.vm[2], l, sizeof(T) * msum, cudaMemcpyDefault, s));
    BT_TRY(cudaMemcpyAsync(B.vm[3], u, sizeof(T) * msum, cudaMemcpyDefault, s));
  }
  BT_TRY(cudaMemcpyAsync(B.Atcol, Ai, sizeof(int) * ao, cudaMemcpyDefault, s));
  std::vector<int> kperm_h, kiperm_h, kbs_h, kfo_h, kbo_h, kco_h, kcr_h;
  if (b->direct) {
    kperm_h.reserve(nsum); kiperm_h.reserve(nsum); kbs_h.reserve(kb_tot); kfo_h.reserve(kb_tot); kco_h.reserve(kb_tot);
    kcr_h.reserve(kcr_tot);
    for (int k = 0; k < count; k++) {
      const KktPlan& q = plans[k];
      if (q.perm.empty()) {
        // a QP of the dense-row form: no permutation, its slots keep their place
        kperm_h.insert(kperm_h.end(), b->inst[k].n, 0);
        kiperm_h.insert(kiperm_h.end(), b->inst[k].n, 0);
      }
      kperm_h.insert(kperm_h.end(), q.perm.begin(), q.perm.end());
      kiperm_h.insert(kiperm_h.end(), q.iperm.begin(), q.iperm.end());
      kbs_h.insert(kbs_h.end(), q.bs.begin(), q.bs.end());
      kfo_h.insert(kfo_h.end(), q.fo.begin(), q.fo.end());
      kbo_h.insert(kbo_h.end(), q.bo.begin(), q.bo.end());
      kco_h.insert(kco_h.end(), q.co.begin(), q.co.end());
      kcr_h.insert(kcr_h.end(), q.cr.begin(), q.cr.end());
    }
    BT_TRY(cudaMemcpyAsync(B.kperm, kperm_h.data(), sizeof(int) * nsum, cudaMemcpyHostToDevice, s));
    BT_TRY(cudaMemcpyAsync(B.kiperm, kiperm_h.data(), sizeof(int) * nsum, cudaMemcpyHostToDevice, s));
    if (kb_tot) BT_TRY(cudaMemcpyAsync(B.kbs, kbs_h.data(), sizeof(int) * kb_tot, cudaMemcpyHostToDevice, s));
    if (kb_tot) BT_TRY(cudaMemcpyAsync(B.kfo, kfo_h.data(), sizeof(int) * kb_tot, cudaMemcpyHostToDevice, s));
    if (kb_tot) BT_TRY(cudaMemcpyAsync(B.kbo, kbo_h.data(), sizeof(int) * kb_tot, cudaMemcpyHostToDevice, s));
    if (kb_tot) BT_TRY(cudaMemcpyAsync(B.kco, kco_h.data(), sizeof(int) * kb_tot, cudaMemcpyHostToDevice, s));
    if (kcr_tot) BT_TRY(cudaMemcpyAsync(B.kcr, kcr_h.data(), sizeof(int) * kcr_tot, cudaMemcpyHostToDevice, s));
    plans.clear();
    if (kdr_tot) {
      std::vector<int> drows_h, didx_h(msum, -1);
      drows_h.reserve(kdr_tot);
      for (int k = 0; k < count; k++) {
        const DrPlan& q = drplans[k];
        drows_h.insert(drows_h.end(), q.rows.begin(), q.rows.end());
        for (int a2 = 0; a2 < q.r; a2++) didx_h[b->inst[k].m_off + q.rows[a2]] = a2;
      }
      BT_TRY(cudaMemcpyAsync(B.kdrows, drows_h.data(), sizeof(int) * kdr_tot, cudaMemcpyHostToDevice, s));
      BT_TRY(cudaMemcpyAsync(B.kdidx, didx_h.data(), sizeof(int) * msum, cudaMemcpyHostToDevice, s));
      BT_TRY(cudaStreamSynchronize(s));   // the host vectors go out of scope
    }
    drplans.clear();
  }

  // ---- device structure build ----
  int *dPp = nullptr, *dAp = nullptr, *dppoff = nullptr, *dPi = nullptr;
  BT_TRY(cudaMallocAsync((void**)&dPp, sizeof(int) * colptr_len, s));
  BT_TRY(cudaMallocAsync((void**)&dAp, sizeof(int) * colptr_len, s));
  BT_TRY(cudaMallocAsync((void**)&dppoff, sizeof(int) * count, s));
  BT_TRY(cudaMallocAsync((void**)&dPi, sizeof(int) * (pto > 0 ? pto : 1), s));
  BT_TRY(cudaMemcpyAsync(dPp, hPp.data(), sizeof(int) * colptr_len, cudaMemcpyHostToDevice, s));
  BT_TRY(cudaMemcpyAsync(dAp, hAp.data(), sizeof(int) * colptr_len, cudaMemcpyHostToDevice, s));
  BT_TRY(cudaMemcpyAsync(dppoff, pp_off.data(), sizeof(int) * count, cudaMemcpyHostToDevice, s));
  if (pto) BT_TRY(cudaMemcpyAsync(dPi, hPi.data(), sizeof(int) * pto, cudaMemcpyHostToDevice, s));
  const int sblocks = std::min(count, 4096);
  {  // A: stable sort of CSC entries by global row
    int *keys = nullptr, *keys_out = nullptr, *idx = nullptr, *cols = nullptr;
    void* tmp = nullptr; size_t tmp_bytes = 0;
    const long long na = ao > 0 ? ao : 1;
    BT_TRY(cudaMallocAsync((void**)&keys, sizeof(int) * na, s));
    BT_TRY(cudaMallocAsync((void**)&keys_out, sizeof(int) * na, s));
    BT_TRY(cudaMallocAsync((void**)&idx, sizeof(int) * na, s));
    BT_TRY(cudaMallocAsync((void**)&cols, sizeof(int) * na, s));
    k_batch_A_keys<<<sblocks, 256, 0, s>>>(b->d_inst, count, dAp, dppoff, B.Atcol, keys, cols, B.Atrow);
    BT_TRY(cudaMemcpyAsync(B.Atrow + nsum, &ao, sizeof(int), cudaMemcpyHostToDevice, s));
    if (ao) {
      k_iota<<<1024, 256, 0, s>>>(idx, (int)ao);
      const int bits = bits_for((unsigned long long)(msum > 0 ? msum : 1));
      cub::DeviceRadixSort::SortPairs(tmp, tmp_bytes, keys, keys_out, idx, B.Asrc, (int)ao, 0, bits, s);
      BT_TRY(cudaMallocAsync(&tmp, tmp_bytes ? tmp_bytes : 1, s));
      BT_TRY(cub::DeviceRadixSort::SortPairs(tmp, tmp_bytes, keys, keys_out, idx, B.Asrc, (int)ao, 0, bits, s));
      k_gather_int<<<1024, 256, 0, s>>>(cols, B.Asrc, (int)ao, B.Acol);
      cudaFreeAsync(tmp, s);
    }
    k_rowptr_from_sorted<<<(int)std::max(1LL, (ao + 256) / 256), 256, 0, s>>>(keys_out, (int)ao, (int)msum, B.Arow);
    cudaFreeAsync(keys, s); cudaFreeAsync(keys_out, s); cudaFreeAsync(idx, s); cudaFreeAsync(cols, s);
  }
  {  // P: symmetric expansion + 64-bit key sort
    const long long slots = 2 * pto + nsum;
    unsigned long long *k_in = nullptr, *k_out = nullptr;
    int *s_in = nullptr;
    void* tmp = nullptr; size_t tmp_bytes = 0;
    BT_TRY(cudaMallocAsync((void**)&k_in, sizeof(unsigned long long) * slots, s));
    BT_TRY(cudaMallocAsync((void**)&k_out, sizeof(unsigned long long) * slots, s));
    BT_TRY(cudaMallocAsync((void**)&s_in, sizeof(int) * slots, s));
    int* s_out = nullptr;
    BT_TRY(cudaMallocAsync((void**)&s_out, sizeof(int) * slots, s));
    k_batch_P_keys<<<sblocks, 256, 0, s>>>(b->d_inst, count, dPp, dppoff, dPi, (int)pto, k_in, s_in);
    cub::DeviceRadixSort::SortPairs(tmp, tmp_bytes, k_in, k_out, s_in, s_out, (int)slots, 0, 64, s);
    BT_TRY(cudaMallocAsync(&tmp, tmp_bytes ? tmp_bytes : 1, s));
    BT_TRY(cub::DeviceRadixSort::SortPairs(tmp, tmp_bytes, k_in, k_out, s_in, s_out, (int)slots, 0, 64, s));
    k_batch_P_from_sorted<<<(int)((nPf + 256) / 256), 256, 0, s>>>(k_out, (int)nPf, (int)nsum, B.Pcol, B.Prow);
    BT_TRY(cudaMemcpyAsync(B.Psrc, s_out, sizeof(int) * nPf, cudaMemcpyDeviceToDevice, s));
    k_batch_P_diag<<<sblocks, 256, 0, s>>>(b->d_inst, count, B.Prow, B.Pcol, B.Pdiag);
    cudaFreeAsync(tmp, s); cudaFreeAsync(k_in, s); cudaFreeAsync(k_out, s); cudaFreeAsync(s_in, s); cudaFreeAsync(s_out, s);
  }
  cudaFreeAsync(dPp, s); cudaFreeAsync(dAp, s); cudaFreeAsync(dppoff, s); cudaFreeAsync(dPi, s);

  // ---- persistent grid: SMs x resident CTAs, or resident clusters ----
  int per_sm = 0, sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->device);
  const int cap_kib = env_int("OSQP_GB300_BATCH_SMEM_KIB", -1);
  const long cap = cap_kib < 0 ? -1L : 1024L * cap_kib;
  cluster_form(env_int("OSQP_GB300_BATCH_CLUSTER_THREADS", 1024), &b->cfn, &b->cthreads);
  b->cdsm = configure_dsm(b->cfn, b->cthreads, 1, b->device, cap);
  // OSQP_GB300_BATCH_CLUSTER: 0 = one CTA per QP (k_batch), c >= 1 = clusters
  // of c CTAs per QP (k_batch_cluster, sliced rows, replicated vectors)
  b->cluster = b->direct ? 0 : std::max(0, std::min(16, env_int("OSQP_GB300_BATCH_CLUSTER", 0)));
  if (b->cluster >= 1) {
    int nclusters = max_active_clusters(b->cfn, b->cluster, b->cthreads, (size_t)b->cdsm);
    if (nclusters < 1) b->cluster = 0;
    else b->grid = std::max(1, std::min(count, nclusters));   // grid counted in clusters
  }
  int minb = 2;
  cta_form(b->direct != 0, &b->kfn, &b->threads, &minb);
  b->dsm = configure_dsm(b->kfn, b->threads, minb, b->device, cap);
  if (b->cluster == 0) {
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, b->kfn, b->threads, (size_t)b->dsm);
    b->grid = std::max(1, std::min(count, sms * std::max(per_sm, 1)));
  }
  // Defaults measured on 4096 batched MPC QPs (GB300, one box, alternating
  // configurations): one 1024-thread CTA per QP with staged vectors (512 x 2
  // per SM: -7 %), and QPs still running after 2000 ADMM iterations continue
  // on 8-CTA clusters with the QP in shared memory (split 600: -10 %, 1000:
  // -4 %; tail clusters of 16: -12 %, of 4: -1 %).
  // (the direct solver runs in the CTA form only: no split)
  b->split = b->direct ? 0 : std::max(0, env_int("OSQP_GB300_BATCH_SPLIT", 2000));
  // 0: vectors only; 1: vectors, then matrix rows; 2: matrix rows before the
  // element-wise PCG vectors
  b->stage_mat = std::max(0, std::min(2, env_int("OSQP_GB300_BATCH_STAGE_MATRIX", 1)));
  b->reorder = env_int("OSQP_GB300_BATCH_REORDER", 1) != 0;
  b->tail_cluster = std::max(0, std::min(16, env_int("OSQP_GB300_BATCH_TAIL", 8)));
  b->tail_grid = 0;
  while (b->split > 0 && b->tail_cluster >= 1) {
    b->tail_grid = max_active_clusters(b->cfn, b->tail_cluster, b->cthreads, (size_t)b->cdsm);
    if (b->tail_grid >= 1) break;
    b->tail_cluster /= 2;
  }
  cudaGetLastError();

  int rc = run_batch_kernel(b, kModeSetup);
  if (rc) { osqp_gb300_batch_cleanup(b); return rc; }
  if (cudaStreamSynchronize(s) != cudaSuccess) { osqp_gb300_batch_cleanup(b); return OSQP_ALGEBRA_LOAD_ERROR; }
  *batchp = b;
  return 0;
}

extern "C" OSQPInt osqp_gb300_kkt_plan(OSQPInt n, OSQPInt m, const OSQPInt* Pp, const OSQPInt* Pi, const OSQPInt* Ap,
                                       const OSQPInt* Ai, OSQPInt bmax_limit, OSQPInt* nblocks, OSQPInt* block_start,
                                       OSQPInt* perm) {
  if (n <= 0 || m < 0 || !Pp || !Ap || !nblocks || !block_start || !perm) return 2;
  KktPlan pl;
  const int rc = kkt_plan_build(n, m, Pp, Pi, Ap, Ai, bmax_limit, pl);
  if (rc) return rc;
  *nblocks = pl.nb;
  for (int k = 0; k <= pl.nb; k++) block_start[k] = pl.bs[k];
  for (int p = 0; p < n; p++) perm[p] = pl.perm[p];
  return 0;
}

extern "C" OSQPInt osqp_gb300_batch_update_data_vec(OSQPBatch* b, const OSQPFloat* q, const OSQPFloat* l,
                                                    const OSQPFloat* u) {
  if (!b) return OSQP_WORKSPACE_NOT_INIT_ERROR;
  cudaSetDevice(b->device);
  cudaStream_t s = b->stream;
  BatchArrays<T>& B = b->B;
  cudaEventRecord(b->evu, s);
  b->upd_pending = 1;
  if (l || u) {
    BT_TRY(cudaMemcpyAsync(b->stage_l, l ? (const void*)l : (const void*)B.vm[2], sizeof(T) * b->msum,
                           l ? cudaMemcpyDefault : cudaMemcpyDeviceToDevice, s));
    BT_TRY(cudaMemcpyAsync(b->stage_u, u ? (const void*)u : (const void*)B.vm[3], sizeof(T) * b->msum,
                           u ? cudaMemcpyDefault : cudaMemcpyDeviceToDevice, s));
    BT_TRY(cudaMemsetAsync(b->d_flag, 0, sizeof(int), s));
    k_batch_check_bounds<T><<<1024, 256, 0, s>>>(b->stage_l, b->stage_u, b->msum, b->d_flag);
    int bad = 0;
    BT_TRY(cudaMemcpyAsync(&bad, b->d_flag, sizeof(int), cudaMemcpyDeviceToHost, s));
    BT_TRY(cudaStreamSynchronize(s));
    if (bad) return OSQP_DATA_VALIDATION_ERROR;
    BT_TRY(cudaMemcpyAsync(B.vm[2], b->stage_l, sizeof(T) * b->msum, cudaMemcpyDeviceToDevice, s));
    BT_TRY(cudaMemcpyAsync(B.vm[3], b->stage_u, sizeof(T) * b->msum, cudaMemcpyDeviceToDevice, s));
  }
  if (q) BT_TRY(cudaMemcpyAsync(B.vn[1], q, sizeof(T) * b->nsum, cudaMemcpyDefault, s));
  int rc = run_batch_kernel(b, kModeUpdateVec);
  if (rc) return rc;
  return cudaStreamSynchronize(s) == cudaSuccess ? 0 : OSQP_ALGEBRA_LOAD_ERROR;
}

// New values of QP k's P (upper triangle, input order) and A entries
// (osqp_update_data_mat, osqp_api.c:1309-1409).  Return codes as the
// reference's: 1 / 2 for a bad P / A count.  Indices are checked on the host
// (an index outside the QP's entries is OSQP_DATA_VALIDATION_ERROR, nothing
// changed), then one launch re-scales QP k and refactors (direct solver) or
// rebuilds its preconditioner, keeping rho and the iterates.
extern "C" OSQPInt osqp_gb300_batch_update_data_mat(OSQPBatch* b, OSQPInt k, const OSQPFloat* Px_new,
                                                    const OSQPInt* Px_new_idx, OSQPInt P_new_n,
                                                    const OSQPFloat* Ax_new, const OSQPInt* Ax_new_idx,
                                                    OSQPInt A_new_n) {
  if (!b) return OSQP_WORKSPACE_NOT_INIT_ERROR;
  if (k < 0 || k >= b->count) return OSQP_DATA_VALIDATION_ERROR;
  const long long nnzP = b->nnzT_k[k], nnzA = b->nnzA_k[k];
  if (P_new_n > nnzP || P_new_n < 0) return 1;
  if (!Px_new_idx && P_new_n != 0 && P_new_n != nnzP) return 1;
  if (P_new_n == 0) P_new_n = (OSQPInt)nnzP;
  if (A_new_n > nnzA || A_new_n < 0) return 2;
  if (!Ax_new_idx && A_new_n != 0 && A_new_n != nnzA) return 2;
  if (A_new_n == 0) A_new_n = (OSQPInt)nnzA;
  const bool doP = Px_new && P_new_n > 0, doA = Ax_new && A_new_n > 0;
  if (!doP && !doA) return 0;
  cudaSetDevice(b->device);
  cudaStream_t s = b->stream;
  // indices on the host first: nothing reaches the device unless all are in range
  std::vector<int> pi, ai;
  auto fetch_idx = [&](const OSQPInt* idx, OSQPInt cnt, long long lim, std::vector<int>& out) -> bool {
    if (!idx) return true;
    std::vector<OSQPInt> h(cnt);
    if (cudaMemcpy(h.data(), idx, sizeof(OSQPInt) * cnt, cudaMemcpyDefault) != cudaSuccess) return false;
    out.resize(cnt);
    for (OSQPInt i = 0; i < cnt; i++) {
      if (h[i] < 0 || h[i] >= lim) return false;
      out[i] = (int)h[i];
    }
    return true;
  };
  if ((doP && !fetch_idx(Px_new_idx, P_new_n, nnzP, pi)) || (doA && !fetch_idx(Ax_new_idx, A_new_n, nnzA, ai)))
    return OSQP_DATA_VALIDATION_ERROR;
  const int mx = std::max(doP ? P_new_n : 0, doA ? A_new_n : 0);
  T* tmpv = nullptr;
  int* tmpi = nullptr;
  int* d_k = nullptr;
  BT_TRY(cudaMallocAsync((void**)&tmpv, sizeof(T) * mx, s));
  BT_TRY(cudaMallocAsync((void**)&tmpi, sizeof(int) * mx, s));
  BT_TRY(cudaMallocAsync((void**)&d_k, sizeof(int), s));
  const BatchInst& I = b->inst[k];
  const int qk = (int)k;
  BT_TRY(cudaMemcpyAsync(d_k, &qk, sizeof(int), cudaMemcpyHostToDevice, s));
  if (doP) {
    BT_TRY(cudaMemcpyAsync(tmpv, Px_new, sizeof(T) * P_new_n, cudaMemcpyDefault, s));
    if (Px_new_idx) BT_TRY(cudaMemcpyAsync(tmpi, pi.data(), sizeof(int) * P_new_n, cudaMemcpyHostToDevice, s));
    k_batch_scatter_vals<T><<<64, 256, 0, s>>>(b->B.Praw + I.pt_off, tmpv, Px_new_idx ? tmpi : nullptr, P_new_n);
    BT_TRY(cudaGetLastError());
  }
  if (doA) {
    BT_TRY(cudaMemcpyAsync(tmpv, Ax_new, sizeof(T) * A_new_n, cudaMemcpyDefault, s));
    if (Ax_new_idx) BT_TRY(cudaMemcpyAsync(tmpi, ai.data(), sizeof(int) * A_new_n, cudaMemcpyHostToDevice, s));
    k_batch_scatter_vals<T><<<64, 256, 0, s>>>(b->B.Araw + I.a_off, tmpv, Ax_new_idx ? tmpi : nullptr, A_new_n);
    BT_TRY(cudaGetLastError());
  }
  LaunchBufs lb{d_k, 1, b->d_queue2, b->d_order2};
  const int rc = launch_batch(b, kModeUpdateMat, lb, s, false);
  cudaFreeAsync(tmpv, s);
  cudaFreeAsync(tmpi, s);
  cudaFreeAsync(d_k, s);
  if (rc) return rc;
  return cudaStreamSynchronize(s) == cudaSuccess ? 0 : OSQP_ALGEBRA_LOAD_ERROR;
}

extern "C" OSQPInt osqp_gb300_batch_solve(OSQPBatch* b) {
  if (!b) return OSQP_WORKSPACE_NOT_INIT_ERROR;
  cudaSetDevice(b->device);
  cudaEventRecord(b->ev0, b->stream);
  int rc = run_batch_kernel(b, kModeSolve);
  if (rc) return rc;
  cudaEventRecord(b->ev1, b->stream);
  k_batch_info<<<(b->count + 255) / 256, 256, 0, b->stream>>>(b->B.st, b->count, b->d_info, b->d_totals);
  long long tot[2] = {0, 0};
  BT_TRY(cudaMemcpyAsync(tot, b->d_totals, sizeof(tot), cudaMemcpyDeviceToHost, b->stream));
  if (cudaStreamSynchronize(b->stream) != cudaSuccess) return OSQP_ALGEBRA_LOAD_ERROR;
  cudaEventElapsedTime(&b->last_ms, b->ev0, b->ev1);
  if (b->upd_pending) cudaEventElapsedTime(&b->last_step_ms, b->evu, b->ev1);
  else b->last_step_ms = b->last_ms;
  b->upd_pending = 0;
  b->last_admm = tot[0]; b->last_pcg = tot[1];
  if (b->reorder && b->count > 1) {
    // history-based queue order: the QPs that just took longest (PCG
    // iterations x cost of one pass) go first next time, so the launch does
    // not end with a few long QPs running on an otherwise idle GPU.  The
    // order never changes a QP's result.
    std::vector<BatchInfo> info(b->count);
    BT_TRY(cudaMemcpy(info.data(), b->d_info, sizeof(BatchInfo) * b->count, cudaMemcpyDeviceToHost));
    std::vector<int> order(b->count);
    std::iota(order.begin(), order.end(), 0);
    std::vector<double> key(b->count);
    for (int k = 0; k < b->count; k++) key[k] = (double)(info[k].pcg + info[k].iter + 1) * (double)b->work_h[k];
    std::stable_sort(order.begin(), order.end(), [&](int a, int c) { return key[a] > key[c]; });
    BT_TRY(cudaMemcpyAsync(b->d_order, order.data(), sizeof(int) * b->count, cudaMemcpyHostToDevice, b->stream));
    BT_TRY(cudaStreamSynchronize(b->stream));
    b->order_h = order;
  }
  return 0;
}

// SpMV tile autotuner: time a short windowed solve (probe_iter ADMM iterations,
// one QP per resident CTA, sampled evenly along the queue) for each candidate
// target of entries per lane, keep the fastest, and put every iterate and
// scalar back as it was.
extern "C" OSQPInt osqp_gb300_batch_autotune(OSQPBatch* b, OSQPInt probe_iter, OSQPInt* per_lane) {
  if (!b) return OSQP_WORKSPACE_NOT_INIT_ERROR;
  cudaSetDevice(b->device);
  cudaStream_t s = b->stream;
  const int probe = std::max(1, std::min((int)(probe_iter > 0 ? probe_iter : 60), b->ds.max_iter));
  const int ns = std::max(1, std::min(b->count, b->grid));   // one QP per resident CTA / cluster
  std::vector<int> sample(ns);
  for (int i = 0; i < ns; i++) sample[i] = b->order_h[(long long)i * b->count / ns];
  BatchArrays<T>& B = b->B;
  const size_t vbytes = sizeof(T) * 16 * (size_t)(b->nsum + b->msum);
  const size_t sbytes = sizeof(SolverScalars) * (size_t)b->count;
  const size_t bbytes = sizeof(T) * b->binv_elems;   // block-Jacobi blocks follow rho
  char* snap = nullptr;
  int* dbuf = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int rc = 0;
  int best = b->per_lane;
  if (cudaMallocAsync((void**)&snap, vbytes + sbytes + bbytes, s) != cudaSuccess ||
      cudaMallocAsync((void**)&dbuf, sizeof(int) * (2 * (size_t)ns + 4), s) != cudaSuccess ||
      cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) rc = OSQP_MEM_ALLOC_ERROR;
  size_t off = 0;
  for (int k = 0; !rc && k < 16; k++) {
    cudaMemcpyAsync(snap + off, B.vn[k], sizeof(T) * b->nsum, cudaMemcpyDeviceToDevice, s); off += sizeof(T) * b->nsum;
    cudaMemcpyAsync(snap + off, B.vm[k], sizeof(T) * b->msum, cudaMemcpyDeviceToDevice, s); off += sizeof(T) * b->msum;
  }
  if (!rc) cudaMemcpyAsync(snap + off, B.st, sbytes, cudaMemcpyDeviceToDevice, s);
  if (!rc && bbytes) cudaMemcpyAsync(snap + off + sbytes, B.Binv, bbytes, cudaMemcpyDeviceToDevice, s);
  if (!rc) cudaMemcpyAsync(dbuf, sample.data(), sizeof(int) * ns, cudaMemcpyHostToDevice, s);
  // the direct solver refactors when a probe changes rho: keep the sampled
  // QPs' factors too
  T* fsnap = nullptr;
  std::vector<std::pair<long long, long long>> fsl;   // (offset, elements) of each sampled factor
  if (!rc && b->direct) {
    long long tot = 0;
    for (int k : sample) {
      const long long o = b->inst[k].kf_off, e = (k + 1 < b->count ? b->inst[k + 1].kf_off : b->kf_total) - o;
      fsl.push_back({o, e});
      tot += e;
    }
    if (cudaMallocAsync((void**)&fsnap, sizeof(T) * (size_t)std::max(1LL, tot), s) != cudaSuccess) rc = OSQP_MEM_ALLOC_ERROR;
    long long fo = 0;
    for (size_t i = 0; !rc && i < fsl.size(); i++) {
      cudaMemcpyAsync(fsnap + fo, B.kF + fsl[i].first, sizeof(T) * fsl[i].second, cudaMemcpyDeviceToDevice, s);
      fo += fsl[i].second;
    }
  }
  // and the dense-row form's inverse capacitance matrices and Dg^-1
  T* csnap = nullptr;
  if (!rc && b->kc_total > 0) {
    if (cudaMallocAsync((void**)&csnap, sizeof(T) * (size_t)(b->kc_total + b->nsum), s) != cudaSuccess) rc = OSQP_MEM_ALLOC_ERROR;
    else {
      cudaMemcpyAsync(csnap, B.kCinv, sizeof(T) * b->kc_total, cudaMemcpyDeviceToDevice, s);
      cudaMemcpyAsync(csnap + b->kc_total, B.kDginv, sizeof(T) * b->nsum, cudaMemcpyDeviceToDevice, s);
    }
  }
  LaunchBufs lb{dbuf, ns, dbuf + 2 * (size_t)ns, dbuf + ns};
  float best_ms = 1e30f, default_ms = 1e30f;
  for (int cand : {kDefaultPerLane, 4, 16}) {
    if (rc) break;
    assign_lanes(b, cand);
    cudaMemcpyAsync(b->d_inst, b->inst.data(), sizeof(BatchInst) * b->count, cudaMemcpyHostToDevice, s);
    float ms = 1e30f;
    for (int rep = 0; rep < 2 && !rc; rep++) {
      // back to the saved state, then a solve of the sample stopped after `probe` iterations
      cudaMemcpyAsync(B.st, snap + off, sbytes, cudaMemcpyDeviceToDevice, s);
      cudaEventRecord(e0, s);
      if (launch_batch(b, kModeSolve, lb, s, false, probe)) rc = OSQP_ALGEBRA_LOAD_ERROR;
      cudaEventRecord(e1, s);
      if (cudaEventSynchronize(e1) != cudaSuccess) rc = OSQP_ALGEBRA_LOAD_ERROR;
      float t = 0.f;
      cudaEventElapsedTime(&t, e0, e1);
      ms = std::min(ms, t);
    }
    if (cand == kDefaultPerLane) default_ms = ms;
    if (ms < best_ms) { best_ms = ms; best = cand; }
  }
  // keep the default tile unless another one is clearly faster on the probe
  if (best != kDefaultPerLane && best_ms > 0.97f * default_ms) best = kDefaultPerLane;
  // the chosen tile, and every vector and scalar as before the probes
  assign_lanes(b, best);
  cudaMemcpyAsync(b->d_inst, b->inst.data(), sizeof(BatchInst) * b->count, cudaMemcpyHostToDevice, s);
  if (snap) {
    off = 0;
    for (int k = 0; k < 16; k++) {
      cudaMemcpyAsync(B.vn[k], snap + off, sizeof(T) * b->nsum, cudaMemcpyDeviceToDevice, s); off += sizeof(T) * b->nsum;
      cudaMemcpyAsync(B.vm[k], snap + off, sizeof(T) * b->msum, cudaMemcpyDeviceToDevice, s); off += sizeof(T) * b->msum;
    }
    cudaMemcpyAsync(B.st, snap + off, sbytes, cudaMemcpyDeviceToDevice, s);
    if (bbytes) cudaMemcpyAsync(B.Binv, snap + off + sbytes, bbytes, cudaMemcpyDeviceToDevice, s);
    cudaFreeAsync(snap, s);
  }
  if (fsnap) {
    long long fo = 0;
    for (size_t i = 0; i < fsl.size(); i++) {
      cudaMemcpyAsync(B.kF + fsl[i].first, fsnap + fo, sizeof(T) * fsl[i].second, cudaMemcpyDeviceToDevice, s);
      fo += fsl[i].second;
    }
    cudaFreeAsync(fsnap, s);
  }
  if (csnap) {
    cudaMemcpyAsync(B.kCinv, csnap, sizeof(T) * b->kc_total, cudaMemcpyDeviceToDevice, s);
    cudaMemcpyAsync(B.kDginv, csnap + b->kc_total, sizeof(T) * b->nsum, cudaMemcpyDeviceToDevice, s);
    cudaFreeAsync(csnap, s);
  }
  if (dbuf) cudaFreeAsync(dbuf, s);
  if (cudaStreamSynchronize(s) != cudaSuccess) rc = OSQP_ALGEBRA_LOAD_ERROR;
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (per_lane) *per_lane = best;
  return rc;
}

extern "C" OSQPInt osqp_gb300_batch_get_solution(OSQPBatch* b, OSQPFloat* x, OSQPFloat* y, OSQPInt* status,
                                                 OSQPInt* iter, OSQPFloat* obj_val, OSQPFloat* prim_res,
                                                 OSQPFloat* dual_res) {
  if (!b) return OSQP_WORKSPACE_NOT_INIT_ERROR;
  cudaStream_t s = b->stream;
  if (x) BT_TRY(cudaMemcpyAsync(x, b->B.vn[14], sizeof(T) * b->nsum, cudaMemcpyDefault, s));
  if (y && b->msum) BT_TRY(cudaMemcpyAsync(y, b->B.vm[12], sizeof(T) * b->msum, cudaMemcpyDefault, s));
  if (status || iter || obj_val || prim_res || dual_res) {
    std::vector<BatchInfo> info(b->count);
    BT_TRY(cudaMemcpyAsync(info.data(), b->d_info, sizeof(BatchInfo) * b->count, cudaMemcpyDeviceToHost, s));
    BT_TRY(cudaStreamSynchronize(s));
    for (int k = 0; k < b->count; k++) {
      if (status) status[k] = info[k].status;
      if (iter) iter[k] = info[k].iter;
      if (obj_val) obj_val[k] = (OSQPFloat)info[k].obj;
      if (prim_res) prim_res[k] = (OSQPFloat)info[k].prim;
      if (dual_res) dual_res[k] = (OSQPFloat)info[k].dual;
    }
  }
  return cudaStreamSynchronize(s) == cudaSuccess ? 0 : OSQP_ALGEBRA_LOAD_ERROR;
}

extern "C" OSQPInt osqp_gb300_batch_step_ms(OSQPBatch* b, double* step_ms) {
  if (!b || !step_ms) return OSQP_WORKSPACE_NOT_INIT_ERROR;
  *step_ms = b->last_step_ms;
  return 0;
}

extern "C" OSQPInt osqp_gb300_batch_qp_seconds(OSQPBatch* b, double* seconds) {
  if (!b || !seconds) return OSQP_WORKSPACE_NOT_INIT_ERROR;
  std::vector<BatchInfo> info(b->count);
  BT_TRY(cudaMemcpy(info.data(), b->d_info, sizeof(BatchInfo) * b->count, cudaMemcpyDeviceToHost));
  for (int k = 0; k < b->count; k++) seconds[k] = info[k].seconds;
  return 0;
}

extern "C" OSQPInt osqp_gb300_batch_pcg_iters(OSQPBatch* b, long long* pcg) {
  if (!b || !pcg) return OSQP_WORKSPACE_NOT_INIT_ERROR;
  std::vector<BatchInfo> info(b->count);
  BT_TRY(cudaMemcpy(info.data(), b->d_info, sizeof(BatchInfo) * b->count, cudaMemcpyDeviceToHost));
  for (int k = 0; k < b->count; k++) pcg[k] = info[k].pcg;
  return 0;
}

extern "C" OSQPInt osqp_gb300_batch_structure(OSQPBatch* b, OSQPInt k, OSQPInt which, OSQPInt* rowptr, OSQPInt* col,
                                              OSQPInt* src, OSQPInt* diag) {
  if (!b || k < 0 || k >= b->count || which < 0 || which > 1) return -1;
  if (cudaSetDevice(b->device) != cudaSuccess || cudaStreamSynchronize(b->stream) != cudaSuccess) return -1;
  const BatchInst& I = b->inst[k];
  const int rows = which == 0 ? I.n : I.m;
  std::vector<int> rp(rows + 1);
  const int* grp = which == 0 ? b->B.Prow + I.n_off : b->B.Arow + I.m_off;
  BT_TRY(cudaMemcpy(rp.data(), grp, sizeof(int) * (rows + 1), cudaMemcpyDeviceToHost));
  const int base = rp[0], nz = rp[rows] - rp[0];
  if (rowptr) for (int r = 0; r <= rows; r++) rowptr[r] = rp[r] - base;
  const int* gcol = which == 0 ? b->B.Pcol : b->B.Acol;
  const int* gsrc = which == 0 ? b->B.Psrc : b->B.Asrc;
  if (col && nz) BT_TRY(cudaMemcpy(col, gcol + base, sizeof(int) * nz, cudaMemcpyDeviceToHost));
  if (src && nz) {
    BT_TRY(cudaMemcpy(src, gsrc + base, sizeof(int) * nz, cudaMemcpyDeviceToHost));
    const int off = which == 0 ? I.pt_off : I.a_off;   // positions within the QP's own input arrays
    for (int e = 0; e < nz; e++) if (src[e] >= 0) src[e] -= off;
  }
  if (diag && which == 0) {
    BT_TRY(cudaMemcpy(diag, b->B.Pdiag + I.n_off, sizeof(int) * I.n, cudaMemcpyDeviceToHost));
    for (int i = 0; i < I.n; i++) diag[i] -= base;
  }
  return nz;
}

extern "C" OSQPInt osqp_gb300_batch_phase_cycles(OSQPBatch* b, double* cycles) {
  if (!b || !cycles) return OSQP_WORKSPACE_NOT_INIT_ERROR;
  long long tot[2 + kProfSlots];
  BT_TRY(cudaMemcpy(tot, b->d_totals, sizeof(tot), cudaMemcpyDeviceToHost));
  for (int q = 0; q < kProfSlots; q++) cycles[q] = (double)tot[2 + q];
  return 0;
}

extern "C" OSQPInt osqp_gb300_batch_rho_updates(OSQPBatch* b, OSQPInt* rho_updates) {
  if (!b || !rho_updates) return OSQP_WORKSPACE_NOT_INIT_ERROR;
  std::vector<BatchInfo> info(b->count);
  BT_TRY(cudaMemcpy(info.data(), b->d_info, sizeof(BatchInfo) * b->count, cudaMemcpyDeviceToHost));
  for (int k = 0; k < b->count; k++) rho_updates[k] = info[k].rho_updates;
  return 0;
}

extern "C" OSQPInt osqp_gb300_batch_factor_elems(OSQPBatch* b, long long* elems) {
  if (!b || !elems) return OSQP_WORKSPACE_NOT_INIT_ERROR;
  for (int k = 0; k < b->count; k++)
    elems[k] = b->direct ? ((k + 1 < b->count ? b->inst[k + 1].kf_off : b->kf_total) - b->inst[k].kf_off) : 0;
  return 0;
}

extern "C" OSQPInt osqp_gb300_batch_dense_rows(OSQPBatch* b, OSQPInt k, OSQPInt* r, OSQPInt* rows, OSQPFloat* cinv,
                                               OSQPFloat* dginv) {
  if (!b || k < 0 || k >= b->count || !r) return OSQP_WORKSPACE_NOT_INIT_ERROR;
  const BatchInst& I = b->inst[k];
  *r = b->direct ? I.kdr : 0;
  if (!*r) return 0;
  cudaStream_t s = b->stream;
  if (rows) {
    std::vector<int> h(I.kdr);
    BT_TRY(cudaMemcpyAsync(h.data(), b->B.kdrows + I.kdr_off, sizeof(int) * I.kdr, cudaMemcpyDeviceToHost, s));
    BT_TRY(cudaStreamSynchronize(s));
    for (int a = 0; a < I.kdr; a++) rows[a] = h[a];
  }
  if (cinv) BT_TRY(cudaMemcpyAsync(cinv, b->B.kCinv + I.kc_off, sizeof(T) * (size_t)I.kdr * I.kdr, cudaMemcpyDefault, s));
  if (dginv) BT_TRY(cudaMemcpyAsync(dginv, b->B.kDginv + I.n_off, sizeof(T) * I.n, cudaMemcpyDefault, s));
  BT_TRY(cudaStreamSynchronize(s));
  return 0;
}

extern "C" OSQPInt osqp_gb300_batch_stats(OSQPBatch* b, double* kernel_ms, long long* admm_iter, long long* pcg_iter) {
  if (!b) return OSQP_WORKSPACE_NOT_INIT_ERROR;
  if (kernel_ms) *kernel_ms = b->last_ms;
  if (admm_iter) *admm_iter = b->last_admm;
  if (pcg_iter) *pcg_iter = b->last_pcg;
  return 0;
}

// ---------------------------------------------------------------------------
// Request serving: continuous batching over resident pools
// ---------------------------------------------------------------------------
namespace gbs {

static double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

struct ServeReq {
  long long ticket = 0;
  int pool = 0, qp = 0;
  std::vector<T> q, l, u;
  double t0 = 0.0, t1 = 0.0;
  std::vector<T> x;
  int status = 0, iter = 0;
  double obj = 0.0;
  bool done = false;
};

// One CUDA stream and the buffers of the launch in flight on it.
struct Slot {
  cudaStream_t stream = nullptr;
  cudaEvent_t ev = nullptr;
  int cap = 0;                 // requests per launch the buffers hold
  int* d_buf = nullptr;        // order[cap], order2[cap], queue[3]
  BatchInfo* d_info = nullptr;
  int* h_order = nullptr;      // pinned
  BatchInfo* h_info = nullptr; // pinned
  T* h_vec = nullptr;          // pinned staging: vectors in, x out
  size_t vec_cap = 0;
  std::vector<ServeReq*> reqs;
  int pool = -1;
  bool busy = false;
};

}  // namespace gbs

using namespace gbs;

struct OSQPServer_ {
  int device = 0;
  std::vector<OSQPBatch*> pools;
  std::vector<std::vector<char>> busy;   // per pool, per QP: a request is in flight
  std::vector<Slot> slots;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<ServeReq*> pending;
  std::unordered_map<long long, ServeReq*> reqs;
  long long next_ticket = 1;
  bool stop = false;
  int err = 0;
  std::thread worker;
};

static int slot_reserve(Slot& sl, int cap, size_t vec) {
  if (cap > sl.cap) {
    if (sl.d_buf) cudaFree(sl.d_buf);
    if (sl.d_info) cudaFree(sl.d_info);
    if (sl.h_order) cudaFreeHost(sl.h_order);
    if (sl.h_info) cudaFreeHost(sl.h_info);
    sl.d_buf = nullptr; sl.d_info = nullptr; sl.h_order = nullptr; sl.h_info = nullptr; sl.cap = 0;
    if (cudaMalloc((void**)&sl.d_buf, sizeof(int) * (2 * (size_t)cap + 4)) != cudaSuccess ||
        cudaMalloc((void**)&sl.d_info, sizeof(BatchInfo) * cap) != cudaSuccess ||
        cudaHostAlloc((void**)&sl.h_order, sizeof(int) * cap, cudaHostAllocDefault) != cudaSuccess ||
        cudaHostAlloc((void**)&sl.h_info, sizeof(BatchInfo) * cap, cudaHostAllocDefault) != cudaSuccess)
      return OSQP_MEM_ALLOC_ERROR;
    sl.cap = cap;
  }
  if (vec > sl.vec_cap) {
    if (sl.h_vec) cudaFreeHost(sl.h_vec);
    sl.h_vec = nullptr; sl.vec_cap = 0;
    const size_t want = std::max(vec, (size_t)1 << 16);
    if (cudaHostAlloc((void**)&sl.h_vec, sizeof(T) * want, cudaHostAllocDefault) != cudaSuccess)
      return OSQP_MEM_ALLOC_ERROR;
    sl.vec_cap = want;
  }
  return 0;
}

// Issue one launch for the requests of one pool (all asynchronous on the slot's stream).
static int slot_start(OSQPServer* S, Slot& sl, int pool, std::vector<ServeReq*>& rq) {
  OSQPBatch* b = S->pools[pool];
  const int k = (int)rq.size();
  size_t vec = 0;
  for (ServeReq* r : rq) {
    const BatchInst& I = b->inst[r->qp];
    vec += (size_t)I.n * 2 + (size_t)I.m * 2;
  }
  int rc = slot_reserve(sl, k, vec);
  if (rc) return rc;
  cudaStream_t st = sl.stream;
  BatchArrays<T>& B = b->B;
  size_t off = 0;
  for (int i = 0; i < k; i++) {
    ServeReq* r = rq[i];
    const BatchInst& I = b->inst[r->qp];
    sl.h_order[i] = r->qp;
    auto put = [&](const std::vector<T>& v, T* dst, int len) -> int {
      if (v.empty() || len == 0) return 0;
      memcpy(sl.h_vec + off, v.data(), sizeof(T) * len);
      BT_TRY(cudaMemcpyAsync(dst, sl.h_vec + off, sizeof(T) * len, cudaMemcpyHostToDevice, st));
      off += len;
      return 0;
    };
    if ((rc = put(r->q, B.vn[1] + I.n_off, I.n))) return rc;
    if ((rc = put(r->l, B.vm[2] + I.m_off, I.m))) return rc;
    if ((rc = put(r->u, B.vm[3] + I.m_off, I.m))) return rc;
  }
  int* d_order = sl.d_buf;
  LaunchBufs lb{d_order, k, sl.d_buf + 2 * (size_t)sl.cap, sl.d_buf + sl.cap};
  BT_TRY(cudaMemcpyAsync(d_order, sl.h_order, sizeof(int) * k, cudaMemcpyHostToDevice, st));
  if ((rc = launch_batch(b, kModeUpdateVec, lb, st, false))) return rc;
  if ((rc = launch_batch(b, kModeSolve, lb, st, false))) return rc;
  k_serve_info<<<(k + 255) / 256, 256, 0, st>>>(B.st, d_order, k, sl.d_info);
  BT_TRY(cudaGetLastError());
  BT_TRY(cudaMemcpyAsync(sl.h_info, sl.d_info, sizeof(BatchInfo) * k, cudaMemcpyDeviceToHost, st));
  for (int i = 0; i < k; i++) {
    const BatchInst& I = b->inst[rq[i]->qp];
    BT_TRY(cudaMemcpyAsync(sl.h_vec + off, B.vn[14] + I.n_off, sizeof(T) * I.n, cudaMemcpyDeviceToHost, st));
    off += I.n;
  }
  BT_TRY(cudaEventRecord(sl.ev, st));
  sl.reqs = rq;
  sl.pool = pool;
  sl.busy = true;
  for (ServeReq* r : rq) S->busy[pool][r->qp] = 1;
  return 0;
}

static void slot_finish(OSQPServer* S, Slot& sl) {
  OSQPBatch* b = S->pools[sl.pool];
  // x of request i follows all input vectors of the launch in the staging buffer
  size_t off = 0;
  for (ServeReq* r : sl.reqs) off += r->q.size() + r->l.size() + r->u.size();
  const double t = now_s();
  for (size_t i = 0; i < sl.reqs.size(); i++) {
    ServeReq* r = sl.reqs[i];
    const BatchInst& I = b->inst[r->qp];
    r->x.assign(sl.h_vec + off, sl.h_vec + off + I.n);
    off += I.n;
    r->status = sl.h_info[i].status;
    r->iter = sl.h_info[i].iter;
    r->obj = sl.h_info[i].obj;
    r->t1 = t;
    r->done = true;
    S->busy[sl.pool][r->qp] = 0;
  }
  sl.reqs.clear();
  sl.busy = false;
}

static void serve_worker(OSQPServer* S) {
  cudaSetDevice(S->device);
  std::unique_lock<std::mutex> lk(S->mu);
  for (;;) {
    bool in_flight = false;
    for (Slot& sl : S->slots) {
      if (!sl.busy) continue;
      const cudaError_t q = cudaEventQuery(sl.ev);
      if (q == cudaErrorNotReady) { in_flight = true; continue; }
      if (q != cudaSuccess) S->err = OSQP_ALGEBRA_LOAD_ERROR;
      slot_finish(S, sl);
      S->cv_done.notify_all();
    }
    if (S->err && !S->pending.empty()) {
      // after a failed launch no new launch is issued: every waiting request
      // completes unsolved (its wait returns the error) instead of waiting forever
      const double t = now_s();
      for (ServeReq* r : S->pending) { r->done = true; r->status = OSQP_UNSOLVED; r->t1 = t; }
      S->pending.clear();
      S->cv_done.notify_all();
    }
    // every free stream takes the waiting requests of the pool of the oldest
    // one (one request per QP in flight; later ones for a busy QP wait)
    for (Slot& sl : S->slots) {
      if (sl.busy || S->pending.empty() || S->err) continue;
      int pool = -1;
      size_t cap = 0;
      std::vector<ServeReq*> take;
      std::vector<char> used;
      for (auto it = S->pending.begin(); it != S->pending.end() && (pool < 0 || take.size() < cap);) {
        ServeReq* r = *it;
        if (pool < 0 && !S->busy[r->pool][r->qp]) {
          pool = r->pool;
          used.assign(S->pools[pool]->count, 0);
          // launches hold at most the pool's resident CTA slots / streams
          // requests, so a slow request holds back few others and new
          // arrivals find a free stream soon
          const int slots = S->pools[pool]->grid;   // resident QP slots (CTAs or clusters)
          cap = (size_t)std::max(1, (slots + (int)S->slots.size() - 1) / (int)S->slots.size());
        }
        if (pool >= 0 && r->pool == pool && !S->busy[pool][r->qp] && !used[r->qp]) {
          used[r->qp] = 1;
          take.push_back(r);
          it = S->pending.erase(it);
        } else {
          ++it;
        }
      }
      if (take.empty()) break;
      if (slot_start(S, sl, pool, take)) {
        S->err = OSQP_ALGEBRA_LOAD_ERROR;
        for (ServeReq* r : take) { r->done = true; r->status = OSQP_UNSOLVED; r->t1 = now_s(); }
        S->cv_done.notify_all();
        continue;
      }
      in_flight = true;
    }
    if (S->stop && S->pending.empty() && !in_flight) break;
    if (in_flight) {
      lk.unlock();
      std::this_thread::sleep_for(std::chrono::microseconds(20));
      lk.lock();
    } else {
      S->cv_work.wait(lk, [&] { return S->stop || !S->pending.empty(); });
    }
  }
}

extern "C" OSQPInt osqp_gb300_server_create(OSQPServer** server, OSQPInt concurrency) {
  if (!server || concurrency < 1 || concurrency > 64) return OSQP_DATA_VALIDATION_ERROR;
  *server = nullptr;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return OSQP_ALGEBRA_LOAD_ERROR;
  OSQPServer* S = new OSQPServer_();
  S->device = dev;
  S->slots.resize(concurrency);
  for (Slot& sl : S->slots) {
    if (cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&sl.ev, cudaEventDisableTiming) != cudaSuccess) {
      osqp_gb300_server_destroy(S);
      return OSQP_ALGEBRA_LOAD_ERROR;
    }
  }
  S->worker = std::thread(serve_worker, S);
  *server = S;
  return 0;
}

extern "C" OSQPInt osqp_gb300_server_add_pool(OSQPServer* S, OSQPBatch* pool, OSQPInt* pool_id) {
  if (!S || !pool || !pool_id) return OSQP_DATA_VALIDATION_ERROR;
  if (pool->device != S->device) return OSQP_DATA_VALIDATION_ERROR;
  std::lock_guard<std::mutex> g(S->mu);
  S->pools.push_back(pool);
  S->busy.emplace_back(pool->count, 0);
  *pool_id = (OSQPInt)S->pools.size() - 1;
  return 0;
}

extern "C" OSQPInt osqp_gb300_server_submit(OSQPServer* S, OSQPInt pool_id, OSQPInt qp, const OSQPFloat* q,
                                            const OSQPFloat* l, const OSQPFloat* u, long long* ticket) {
  if (!S || !ticket) return OSQP_DATA_VALIDATION_ERROR;
  ServeReq* r = new ServeReq();
  {
    std::lock_guard<std::mutex> g(S->mu);
    if (pool_id < 0 || pool_id >= (OSQPInt)S->pools.size() || qp < 0 || qp >= S->pools[pool_id]->count) {
      delete r;
      return OSQP_DATA_VALIDATION_ERROR;
    }
    const BatchInst& I = S->pools[pool_id]->inst[qp];
    if (q) r->q.assign(q, q + I.n);
    if (l) r->l.assign(l, l + I.m);
    if (u) r->u.assign(u, u + I.m);
  }
  if (!r->l.empty() && !r->u.empty())
    for (size_t j = 0; j < r->l.size(); j++)
      if (!(r->l[j] <= r->u[j])) { delete r; return OSQP_DATA_VALIDATION_ERROR; }
  r->pool = pool_id;
  r->qp = qp;
  r->t0 = now_s();
  {
    std::lock_guard<std::mutex> g(S->mu);
    if (S->stop) { delete r; return OSQP_WORKSPACE_NOT_INIT_ERROR; }
    r->ticket = S->next_ticket++;
    S->reqs[r->ticket] = r;
    S->pending.push_back(r);
    *ticket = r->ticket;
  }
  S->cv_work.notify_one();
  return 0;
}

extern "C" OSQPInt osqp_gb300_server_wait(OSQPServer* S, long long ticket, OSQPFloat* x, OSQPInt* status,
                                          OSQPInt* iter, OSQPFloat* obj_val, double* latency_ms) {
  if (!S) return OSQP_DATA_VALIDATION_ERROR;
  std::unique_lock<std::mutex> lk(S->mu);
  auto it = S->reqs.find(ticket);
  if (it == S->reqs.end()) return OSQP_DATA_VALIDATION_ERROR;
  ServeReq* r = it->second;
  S->cv_done.wait(lk, [&] { return r->done; });
  S->reqs.erase(it);
  const int err = S->err;
  lk.unlock();
  if (x && !r->x.empty()) memcpy(x, r->x.data(), sizeof(T) * r->x.size());
  if (status) *status = r->status;
  if (iter) *iter = r->iter;
  if (obj_val) *obj_val = (OSQPFloat)r->obj;
  if (latency_ms) *latency_ms = (r->t1 - r->t0) * 1e3;
  delete r;
  return err;
}

extern "C" OSQPInt osqp_gb300_server_destroy(OSQPServer* S) {
  if (!S) return 0;
  {
    std::lock_guard<std::mutex> g(S->mu);
    S->stop = true;
  }
  S->cv_work.notify_all();
  if (S->worker.joinable()) S->worker.join();
  cudaSetDevice(S->device);
  for (Slot& sl : S->slots) {
    if (sl.stream) cudaStreamSynchronize(sl.stream);
    if (sl.d_buf) cudaFree(sl.d_buf);
    if (sl.d_info) cudaFree(sl.d_info);
    if (sl.h_order) cudaFreeHost(sl.h_order);
    if (sl.h_info) cudaFreeHost(sl.h_info);
    if (sl.h_vec) cudaFreeHost(sl.h_vec);
    if (sl.ev) cudaEventDestroy(sl.ev);
    if (sl.stream) cudaStreamDestroy(sl.stream);
  }
  for (auto& kv : S->reqs) delete kv.second;
  delete S;
  return 0;
}
