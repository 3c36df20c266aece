// gb_direct.cuh -- direct solve of the reduced KKT system on one CTA.
//
// linsys_solver = OSQP_DIRECT_SOLVER.  The builtin backend solves
// [P + sigma I, A'; A, -R^-1] [x~; nu] = [sigma x - q; z - R^-1 y] by an
// LDL' factorisation refreshed on every rho change
// (algebra/_common/lin_sys/qdldl/qdldl_interface.c:216-530).  Here the
// constraint block is eliminated first, K = P + sigma I + A' R A, and K is
// factored as a block-tridiagonal LDL' (block Thomas algorithm) in the
// ordering of gb_kkt_plan.h:
//   S_0 = K_00,  G_k = K_{k,k-1} S_{k-1}^-1,  S_k = K_kk - G_k K_{k,k-1}'
// with the pivot blocks inverted explicitly (symmetric sweep operator).  A
// solve is then
//   c_k = b_k - G_k c_{k-1}  (forward),  d_k = S_k^-1 c_k,
//   x_k = d_k - G_{k+1}' x_{k+1}  (backward),
// 2 (nb - 1) dependent block steps of dense products.  z~ = A x~ as in the
// reduced form of the builtin's solve (qdldl_interface.c:431-466 gives the
// same x~ and z~ in exact arithmetic).
//
// The solve streams the factor through shared memory: each block's segment
// (gb_kkt_plan.h) is one bulk copy (cp.async.bulk, the TMA engine's untiled
// form) into a ring of `ring` slots, issued by one thread several segments
// ahead of use and tracked by one mbarrier per slot, so the dependent chain of
// block steps reads only shared memory.  Waits are bounded: a copy that does
// not arrive within the limit makes the solve read that segment from global
// memory instead (and records it in the pipe's error word).
//
// Everything is deterministic: each entry has one owner thread and a fixed
// summation order, so a QP's factor and solutions do not depend on the rest
// of a batch.  A pivot that is not positive and finite means K is not
// positive definite (the builtin's non-convexity test, qdldl_interface.c:
// 334-342, counts the positive pivots of the same factorisation).
#pragma once

#include "gb_common.cuh"
#include "gb_kkt_plan.h"

namespace gb {

// Lanes per row of the dense block products.
constexpr int kKktLanes = 8;

template <typename T>
struct KktView {
  int nb = 0, bmax = 0;          // nb == 0: no direct solve
  int ring = 0, segmax = 0;      // bulk-copy ring slots of the solve (0: no ring), largest segment
  const int* bs = nullptr;       // [nb + 1]
  const int* fo = nullptr;       // [nb + 1] forward segments
  const int* bo = nullptr;       // [nb + 1] backward segments
  const int* co = nullptr;       // [nb + 1] (positions in cr)
  const int* cr = nullptr;
  const int* perm = nullptr;     // permuted position -> variable
  const int* iperm = nullptr;    // variable -> permuted position
  T* F = nullptr;                // factor
};

// Factor K = P + sigma I + A' R A (scaled data) into F.  ws: on-chip
// workspace of kkt_factor_ws_elems(bmax) elements.  rho_vec == nullptr: the
// scalar rho.  Returns false when a pivot is not positive (K not positive
// definite in this precision).  All threads of the CTA call it.
template <typename T>
__device__ __noinline__ bool kkt_factor(const KktView<T>& kv, const CSR<T>& P, const CSR<T>& A, const CSR<T>& At,
                                        const T* rho_vec, T rho_s, T sigma, T* ws) {
  const int tid = threadIdx.x, nt = blockDim.x;
  const int lane = tid & 31, warp = tid >> 5, nwarps = nt >> 5;
  const int bm = kv.bmax;
  T* Sprev = ws;
  T* S = Sprev + bm * bm;
  T* S2 = S + bm * bm;
  T* Kc = S2 + bm * bm;
  T* G = Kc + bm * bm;
  T* tile = G + bm * bm;
  T* rhot = tile + kKktTileRows * 2 * bm;
  for (int k = 0; k < kv.nb; k++) {
    const int s0 = kv.bs[k], e0 = kv.bs[k + 1], b = e0 - s0;
    const int sp = k ? kv.bs[k - 1] : s0, bp = s0 - sp;
    const int W = bp + b;   // assembly columns: permuted positions [sp, e0)
    // ---- A' R A over the block's columns from the rows of A with two or
    // more entries, in chunks of kKktTileRows rows; every output entry has
    // one owner thread, so the sum order is fixed ----
    T acc[kKktOutMax];
#pragma unroll
    for (int q = 0; q < kKktOutMax; q++) acc[q] = T(0);
    const int nout = b * W;
    const int c0 = kv.co[k], c1 = kv.co[k + 1];
    for (int cb = c0; cb < c1; cb += kKktTileRows) {
      const int nr = min(kKktTileRows, c1 - cb);
      for (int e = tid; e < nr * W; e += nt) tile[e] = T(0);
      __syncthreads();
      for (int r = warp; r < nr; r += nwarps) {
        const int row = kv.cr[cb + r];
        const int kb = A.rowptr[row], ke = A.rowptr[row + 1];
        for (int f = kb + lane; f < ke; f += 32) {
          const int p = kv.iperm[A.col[f]] - sp;
          if (p >= 0 && p < W) tile[r * W + p] = A.val[f];
        }
        if (lane == 0) rhot[r] = rho_vec ? rho_vec[row] : rho_s;
      }
      __syncthreads();
#pragma unroll
      for (int q = 0; q < kKktOutMax; q++) {
        const int o = tid + q * nt;
        if (o < nout) {
          const int i = o / W, j = o - i * W;
          T a = acc[q];
          // (a_ri a_rj) rho_r: the same product for (i, j) and (j, i)
          for (int r = 0; r < nr; r++) a += (tile[r * W + bp + i] * tile[r * W + j]) * rhot[r];
          acc[q] = a;
        }
      }
      __syncthreads();
    }
#pragma unroll
    for (int q = 0; q < kKktOutMax; q++) {
      const int o = tid + q * nt;
      if (o < nout) {
        const int i = o / W, j = o - i * W;
        if (j < bp) Kc[i * bp + j] = acc[q];
        else S[i * b + (j - bp)] = acc[q];
      }
    }
    __syncthreads();
    // ---- P entries, sigma, and rows of A with a single entry: one warp per
    // variable (lanes over its entries; every P entry has its own target, the
    // single-entry rows are summed in a fixed shuffle order) ----
    for (int i = warp; i < b; i += nwarps) {
      const int v = kv.perm[s0 + i];
      const int pb0 = P.rowptr[v], pe0 = P.rowptr[v + 1];
      for (int e = pb0 + lane; e < pe0; e += 32) {
        const int p = kv.iperm[P.col[e]];
        if (p >= sp && p < s0) Kc[i * bp + (p - sp)] += P.val[e];
        else if (p >= s0 && p < e0 && p != s0 + i) S[i * b + (p - s0)] += P.val[e];
      }
      T dsum = T(0), pdiag = T(0);
      for (int e = pb0 + lane; e < pe0; e += 32)
        if (P.col[e] == v) pdiag = P.val[e];
      for (int e = At.rowptr[v] + lane; e < At.rowptr[v + 1]; e += 32) {
        const int row = At.col[e];
        if (A.rowptr[row + 1] - A.rowptr[row] == 1) {
          const T a = At.val[e];
          dsum += (a * a) * (rho_vec ? rho_vec[row] : rho_s);
        }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        dsum += __shfl_xor_sync(0xffffffffu, dsum, o);
        pdiag += __shfl_xor_sync(0xffffffffu, pdiag, o);   // one lane holds it
      }
      if (lane == 0) S[i * b + i] = ((S[i * b + i] + pdiag) + sigma) + dsum;
    }
    __syncthreads();
    T* Fk = kv.F + kv.fo[k];                         // forward segment: G_k, then S_k^-1
    T* Sg = Fk + kkt_pad4((long long)b * bp);
    if (k > 0) {
      // ---- G_k = K_{k,k-1} S_{k-1}^-1 ; S_k -= G_k K_{k,k-1}' (lower
      // triangle, mirrored: S_k stays exactly symmetric) ----
      for (int o = tid; o < b * bp; o += nt) {
        const int i = o / bp, j = o - i * bp;
        T a = T(0);
        for (int l = 0; l < bp; l++) a += Kc[i * bp + l] * Sprev[l * bp + j];
        G[o] = a;
      }
      __syncthreads();
      for (int o = tid; o < b * b; o += nt) {
        const int i = o / b, j = o - i * b;
        if (j > i) continue;
        T a = T(0);
        for (int l = 0; l < bp; l++) a += G[i * bp + l] * Kc[j * bp + l];
        const T v = S[i * b + j] - a;
        S[i * b + j] = v;
        S[j * b + i] = v;
      }
      T* Gg = Fk;
      T* GTg = kv.F + kv.bo[k];
      for (int o = tid; o < b * bp; o += nt) {
        Gg[o] = G[o];
        const int j = o / b, i = o - j * b;   // G' is bp x b
        GTg[o] = G[i * bp + j];
      }
      __syncthreads();
    }
    // ---- S_k^-1 by symmetric sweeps (double-buffered): -S^-1 after b sweeps ----
    T* src = S;
    T* dst = S2;
    bool bad = false;
    for (int kk = 0; kk < b; kk++) {
      const T piv = src[kk * b + kk];
      if (!(piv > T(0)) || !isfinite((double)piv)) { bad = true; break; }   // CTA-uniform
      const T d = T(1) / piv;
      for (int o = tid; o < b * b; o += nt) {
        const int i = o / b, j = o - i * b;
        const T aik = src[i * b + kk], akj = src[kk * b + j];
        T v;
        if (i == kk) v = (j == kk) ? -d : akj * d;
        else if (j == kk) v = aik * d;
        else v = src[o] - (aik * akj) * d;
        dst[o] = v;
      }
      __syncthreads();
      T* t = src; src = dst; dst = t;
    }
    if (bad) {
      __syncthreads();
      return false;
    }
    for (int o = tid; o < b * b; o += nt) {
      const T v = -src[o];
      Sg[o] = v;
      Sprev[o] = v;
    }
    __syncthreads();
  }
  // the solve reads the factor through the async (bulk-copy) proxy
  asm volatile("fence.proxy.async.global;" ::: "memory");
  __syncthreads();
  return true;
}

// fn(r, sum_j M[r][j] v[j]) for the rows r < rows of a row-major rows x cols
// block, by sub-warps of kKktLanes lanes over threads [t0, t0 + tn); fn runs
// on the sub-warp's first lane.  Loop bounds are uniform over each warp (t0
// and tn multiples of 32).
// Entries of a block row a lane loads before it multiplies (cols up to
// kKktLanes x kKktRowChunk per round): the loads of a round are independent,
// so a block row costs one memory latency per round, not one per entry.
constexpr int kKktRowChunk = 8;

template <typename T, typename FN>
__device__ __forceinline__ void kkt_block_rows(const T* __restrict__ M, const T* v, int rows, int cols, int t0,
                                               int tn, FN fn) {
  const int t = threadIdx.x - t0;
  const int sub = t / kKktLanes, sl = t % kKktLanes;
  const int per = tn / kKktLanes;
  for (int base = 0; base < rows; base += per) {
    const int r = base + sub;
    T a = T(0);
    if (r < rows) {
      const T* Mr = M + (size_t)r * cols;
      for (int j0 = sl; j0 < cols; j0 += kKktLanes * kKktRowChunk) {
        T mv[kKktRowChunk];
#pragma unroll
        for (int u = 0; u < kKktRowChunk; u++) {
          const int j = j0 + u * kKktLanes;
          mv[u] = j < cols ? Mr[j] : T(0);
        }
#pragma unroll
        for (int u = 0; u < kKktRowChunk; u++) {
          const int j = j0 + u * kKktLanes;
          if (j < cols) a += mv[u] * v[j];
        }
      }
    }
    a = subwarp_sum<kKktLanes>(a);
    if (r < rows && sl == 0) fn(r, a);
  }
}

// Copy the block starts and segment offsets (read at every block step) to
// on-chip memory `dst` (3 (nb + 1) ints) and point kv at the copies.
template <typename T>
__device__ __forceinline__ void kkt_plan_on_chip(KktView<T>& kv, int* dst) {
  const int w = kv.nb + 1;
  for (int k = threadIdx.x; k < w; k += blockDim.x) { dst[k] = kv.bs[k]; dst[w + k] = kv.fo[k]; dst[2 * w + k] = kv.bo[k]; }
  kv.bs = dst;
  kv.fo = dst + w;
  kv.bo = dst + 2 * w;
}

// ---------------------------------------------------------------------------
// Bulk-copy pipeline state of a CTA: one mbarrier per ring slot and the number
// of copies issued so far (copy Q goes to slot Q % ring; its wait parity is
// (Q / ring) & 1).  Lives in static shared memory; kkt_pipe_init once per
// kernel before the first solve.
// ---------------------------------------------------------------------------
struct KktPipe {
  unsigned long long bar[kKktRingMax];
  unsigned q;
  int err;
};

__device__ __forceinline__ unsigned kkt_smem(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void kkt_pipe_init(KktPipe* pp) {
  if (threadIdx.x == 0) {
    for (int s = 0; s < kKktRingMax; s++)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(kkt_smem(&pp->bar[s])) : "memory");
    pp->q = 0;
    pp->err = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
}

// Wait (bounded: about 50 ms of device time) for the phase of the given
// parity of an mbarrier.
constexpr unsigned long long kKktWaitNs = 50ull * 1000 * 1000;
__device__ __forceinline__ bool kkt_wait(unsigned long long* bar, unsigned parity) {
  const unsigned a = kkt_smem(bar);
  unsigned long long t0 = 0;
  for (unsigned i = 0;; i++) {
    unsigned ok;
    asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
                 " selp.u32 %0, 1, 0, p;\n}" : "=r"(ok) : "r"(a), "r"(parity) : "memory");
    if (ok) return true;
    if ((i & 31u) == 31u) {
      const unsigned long long t = global_ns();
      if (!t0) t0 = t;
      else if (t - t0 > kKktWaitNs) return false;
    }
  }
}

// One bulk copy global -> shared of `bytes` (multiple of 16, both addresses
// 16-byte aligned), completing a transaction on `bar`.  One thread.
__device__ __forceinline__ void kkt_bulk_load(void* dst, const void* src, unsigned bytes, unsigned long long* bar) {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" :: "r"(kkt_smem(bar)), "r"(bytes) : "memory");
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
               :: "r"(kkt_smem(dst)), "l"(src), "r"(bytes), "r"(kkt_smem(bar)) : "memory");
}

// The solve of kkt_solve with the factor streamed through `ring` (kv.ring
// slots of kv.segmax elements).  Copies j = 0..nb-1 are the forward segments,
// j = nb + t the backward segment of block nb - 1 - t.  A step may refill the
// slot of a copy no later step needs; at most kv.ring copies are ahead.
template <typename T, typename XO>
__device__ void kkt_solve_pipe(const KktView<T>& kv, KktPipe* pp, T* c, T* d, T* ring, XO xout,
                               unsigned long long* prof = nullptr) {
  // prof (thread 0 only, optional): cycles spent [0] waiting for segments, [1] in barriers
  long long tw = 0, tb = 0;
  auto sync = [&]() {
    const long long t = clock64();   // every thread takes the same barrier
    __syncthreads();
    if (prof) tb += clock64() - t;
  };
  const int nt = blockDim.x, half = nt >> 1;
  const bool lo = (int)threadIdx.x < half;
  const int nb = kv.nb, R = kv.ring, SM = kv.segmax;
  const unsigned q0 = pp->q;
  const int total = 2 * nb - 1;
  int issued = 0;                                     // thread 0's count
  auto seg = [&](int j, long long& elems) -> const T* {
    if (j < nb) {
      const long long b = kv.bs[j + 1] - kv.bs[j], bp = j ? kv.bs[j] - kv.bs[j - 1] : 0;
      elems = kkt_pad4(b * bp) + kkt_pad4(b * b);
      return kv.F + kv.fo[j];
    }
    const int k = nb - 1 - (j - nb);
    const long long b = kv.bs[k + 1] - kv.bs[k], bp = kv.bs[k] - kv.bs[k - 1];
    elems = kkt_pad4(b * bp);
    return kv.F + kv.bo[k];
  };
  auto slot = [&](int j) { return ring + (size_t)((q0 + (unsigned)j) % (unsigned)R) * SM; };
  auto issue_upto = [&](int lim) {
    if (threadIdx.x == 0) {
      const int end = lim < total ? lim : total;
      for (; issued < end; issued++) {
        long long el;
        const T* g = seg(issued, el);
        kkt_bulk_load(slot(issued), g, (unsigned)(el * sizeof(T)), &pp->bar[(q0 + (unsigned)issued) % (unsigned)R]);
      }
    }
  };
  // pointer to copy j's data: the ring slot, or global memory after a failed wait
  // (after one failed wait the CTA stops waiting and reads global memory)
  auto get = [&](int j) -> const T* {
    const unsigned Q = q0 + (unsigned)j;
    long long el;
    if (*(volatile int*)&pp->err) return seg(j, el);
    const long long t = prof ? clock64() : 0;
    const bool ok = kkt_wait(&pp->bar[Q % (unsigned)R], (Q / (unsigned)R) & 1u);
    if (prof) tw += clock64() - t;
    if (!ok) {
      *(volatile int*)&pp->err = 1;
      return seg(j, el);
    }
    return slot(j);
  };
  issue_upto(R);
  const T* cur = get(0);
  for (int k = 1; k < nb; k++) {
    const int s0 = kv.bs[k], b = kv.bs[k + 1] - s0, sp = kv.bs[k - 1], bp = s0 - sp;
    const int spp = k > 1 ? kv.bs[k - 2] : sp;
    issue_upto(k - 1 + R);            // copies < k - 1 are no longer needed
    const T* prev = cur;              // segment k - 1: S_{k-1}^-1 after G_{k-1}
    cur = get(k);                     // segment k: G_k first
    if (lo) {
      kkt_block_rows(cur, c + sp, b, bp, 0, half, [&](int r, T a) { c[s0 + r] -= a; });
    } else {
      const T* Si = prev + kkt_pad4((long long)bp * (sp - spp));
      kkt_block_rows(Si, c + sp, bp, bp, half, nt - half, [&](int r, T a) { d[sp + r] = a; });
    }
    sync();
  }
  {
    const int s0 = kv.bs[nb - 1], b = kv.bs[nb] - s0;
    const int bp = nb > 1 ? s0 - kv.bs[nb - 2] : 0;
    issue_upto(nb - 1 + R);
    const T* Si = cur + kkt_pad4((long long)b * bp);
    kkt_block_rows(Si, c + s0, b, b, 0, nt, [&](int r, T a) { d[s0 + r] = a; });
    sync();
  }
  for (int t = 0; t + 1 < nb; t++) {
    const int k = nb - 1 - t;
    const int s0 = kv.bs[k], b = kv.bs[k + 1] - s0, sp = kv.bs[k - 1], bp = s0 - sp;
    issue_upto(nb + t + R);           // copies < nb + t are no longer needed
    const T* GT = get(nb + t);
    if (lo) {
      kkt_block_rows(GT, d + s0, bp, b, 0, half, [&](int r, T a) { d[sp + r] -= a; });
    } else {
      for (int r = threadIdx.x - half; r < b; r += nt - half) xout(kv.perm[s0 + r], d[s0 + r]);
    }
    sync();
  }
  for (int r = threadIdx.x; r < kv.bs[1]; r += nt) xout(kv.perm[r], d[r]);
  if (threadIdx.x == 0) pp->q = q0 + (unsigned)total;
  sync();
  if (prof) { prof[0] += (unsigned long long)tw; prof[1] += (unsigned long long)tb; }
}

// Solve K x = b with the factor: c holds the permuted right-hand side on entry
// (c[iperm[i]] = b_i); d is a second permuted n-vector; x (unpermuted) is
// written through xout(i, value).  All threads of the CTA call it; blockDim.x
// is a multiple of 64.
template <typename T, typename XO>
__device__ void kkt_solve(const KktView<T>& kv, T* c, T* d, XO xout) {
  const int nt = blockDim.x, half = nt >> 1;
  const bool lo = (int)threadIdx.x < half;
  const int nb = kv.nb;
  // forward: c_k -= G_k c_{k-1} (lower half) while d_{k-1} = S_{k-1}^-1 c_{k-1} (upper half)
  for (int k = 1; k < nb; k++) {
    const int s0 = kv.bs[k], b = kv.bs[k + 1] - s0, sp = kv.bs[k - 1], bp = s0 - sp;
    const int spp = k > 1 ? kv.bs[k - 2] : sp;
    if (lo) {
      const T* G = kv.F + kv.fo[k];
      kkt_block_rows(G, c + sp, b, bp, 0, half, [&](int r, T a) { c[s0 + r] -= a; });
    } else {
      const T* Si = kv.F + kv.fo[k - 1] + kkt_pad4((long long)bp * (sp - spp));
      kkt_block_rows(Si, c + sp, bp, bp, half, nt - half, [&](int r, T a) { d[sp + r] = a; });
    }
    __syncthreads();
  }
  {
    const int s0 = kv.bs[nb - 1], b = kv.bs[nb] - s0;
    const int bp = nb > 1 ? s0 - kv.bs[nb - 2] : 0;
    kkt_block_rows(kv.F + kv.fo[nb - 1] + kkt_pad4((long long)b * bp), c + s0, b, b, 0, nt,
                   [&](int r, T a) { d[s0 + r] = a; });
    __syncthreads();
  }
  // backward: x_{k-1} = d_{k-1} - G_k' x_k (lower half) while block k is written out (upper half)
  for (int k = nb - 1; k >= 1; k--) {
    const int s0 = kv.bs[k], b = kv.bs[k + 1] - s0, sp = kv.bs[k - 1], bp = s0 - sp;
    if (lo) {
      const T* GT = kv.F + kv.bo[k];
      kkt_block_rows(GT, d + s0, bp, b, 0, half, [&](int r, T a) { d[sp + r] -= a; });
    } else {
      for (int r = threadIdx.x - half; r < b; r += nt - half) xout(kv.perm[s0 + r], d[s0 + r]);
    }
    __syncthreads();
  }
  for (int r = threadIdx.x; r < kv.bs[1]; r += nt) xout(kv.perm[r], d[r]);
  __syncthreads();
}

}  // namespace gb
