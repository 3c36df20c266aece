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
// A solve is a chain of dependent block steps, each a few small dense
// products, so it runs on a group of warps (two halves, Q lanes per block row,
// column-major blocks so that the lanes of a step read consecutive words)
// synchronised by a named barrier; the other warps of the CTA wait once at the
// end instead of taking every step's barrier.  The FP64 build stores the
// factor as double-float pairs and runs the block products on the FP32 pipe
// (see kKktDF below).  The factor streams through shared memory: each block's segment
// (gb_kkt_plan.h) is one bulk copy (cp.async.bulk, the TMA engine's untiled
// form) into a ring of `ring` slots, issued by a producer warp outside the
// group and tracked by a "full" mbarrier per slot; the group hands a slot back
// through its "empty" mbarrier when no later step needs it, so issuing never
// delays the chain.  Waits are bounded: a copy that does not arrive within the
// limit makes the solve read that segment from global memory instead (and
// records it in the pipe's error word).
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
  // diagonal-plus-dense-rows form (gb_kkt_plan.h; dr == 0 otherwise)
  int dr = 0;                    // dense rows r
  const int* drows = nullptr;    // [r] rows of A with two or more entries
  const int* didx = nullptr;     // [m] position of a row of A in drows, -1 for the others
  T* Cinv = nullptr;             // [r r] (R_d^-1 + A_d Dg^-1 A_d')^-1, row-major
  T* Dginv = nullptr;            // [n] 1 / Dg
};

// A direct solve of either form is set up.
template <typename T>
__host__ __device__ inline bool kkt_direct(const KktView<T>& kv) { return kv.nb > 0 || kv.dr > 0; }

// ---------------------------------------------------------------------------
// Double-float block solve of the FP64 build.
//
// GB300 runs FP64 at about 1/64 of the FP32 rate: an FP64 warp instruction
// takes 65-77 cycles of its SM sub-partition, and a block step is a chain of
// small dense products on a few warps.  The FP64 build therefore factors K in
// FP64 but stores the factor as double-float pairs (a float hi and a float
// lo with hi + lo = the FP64 entry to 48 significant bits), and runs the
// block solve in double-float on the FP32 pipe: the two solve vectors are
// (hi, lo) pairs, each product row is a compensated dot product (the exact
// product of the high parts by FMA plus the cross terms, partial sums kept
// error-free by TwoSum and their errors summed apart: the Dot2 scheme of
// Ogita, Rump and Oishi, "Accurate sum and dot product", SIAM J. Sci.
// Comput. 26 (2005)).  The right-hand side enters and the solution leaves in
// FP64.  A factor sub-array of len entries keeps its bytes: the hi words of
// all entries, then (after kkt_pad4(len) words) the lo words.
// ---------------------------------------------------------------------------
#ifndef GB_KKT_DF
#define GB_KKT_DF 1
#endif
template <typename T>
constexpr bool kKktDF = GB_KKT_DF && std::is_same<T, double>::value;

struct DF {
  float h, l;
};
__device__ __forceinline__ DF df_split(double v) {
  const float h = __double2float_rn(v);
  return DF{h, __double2float_rn(v - (double)h)};
}
__device__ __forceinline__ double df_join(DF a) { return (double)a.h + (double)a.l; }
// (s, e) = a + b exactly (Knuth's TwoSum)
__device__ __forceinline__ void df_two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
// a - b, renormalised
__device__ __forceinline__ DF df_sub(DF a, DF b) {
  float s, e;
  df_two_sum(a.h, -b.h, s, e);
  e = __fadd_rn(e, __fsub_rn(a.l, b.l));
  const float h = __fadd_rn(s, e);
  return DF{h, __fsub_rn(e, __fsub_rn(h, s))};
}

// Value type of one block-product row: T, or DF in the double-float solve.
template <typename T>
using kkt_val = typename std::conditional<kKktDF<T>, DF, T>::type;

// Entry o of a factor sub-array of len entries starting at base.
template <typename T>
__device__ __forceinline__ void kkt_fstore(T* base, long long len, long long o, T v) {
  if constexpr (kKktDF<T>) {
    float* f = reinterpret_cast<float*>(base);
    const DF s = df_split(v);
    f[o] = s.h;
    f[kkt_pad4(len) + o] = s.l;
  } else {
    base[o] = v;
  }
}

// The solve's permuted n-vectors (c, d): T values, or in the double-float
// solve the hi words of the n entries followed by their lo words (the same
// bytes as n doubles).
template <typename T>
__device__ __forceinline__ void kkt_vput(T* v, int n, int i, T x) {
  if constexpr (kKktDF<T>) {
    float* f = reinterpret_cast<float*>(v);
    const DF s = df_split(x);
    f[i] = s.h;
    f[n + i] = s.l;
  } else {
    v[i] = x;
  }
}
template <typename T>
__device__ __forceinline__ T kkt_vget(const T* v, int n, int i) {
  if constexpr (kKktDF<T>) {
    const float* f = reinterpret_cast<const float*>(v);
    return df_join(DF{f[i], f[n + i]});
  } else {
    return v[i];
  }
}
template <typename T>
__device__ __forceinline__ void kkt_vset(T* v, int n, int i, kkt_val<T> a) {
  if constexpr (kKktDF<T>) {
    float* f = reinterpret_cast<float*>(v);
    f[i] = a.h;
    f[n + i] = a.l;
  } else {
    v[i] = a;
  }
}
template <typename T>
__device__ __forceinline__ void kkt_vsub(T* v, int n, int i, kkt_val<T> a) {
  if constexpr (kKktDF<T>) {
    float* f = reinterpret_cast<float*>(v);
    const DF r = df_sub(DF{f[i], f[n + i]}, a);
    f[i] = r.h;
    f[n + i] = r.l;
  } else {
    v[i] -= a;
  }
}

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
      // forward segment: G_k column-major (entry (i, j) at j b + i); backward
      // segment: G_k' column-major, which is G_k row-major
      T* Gg = Fk;
      T* GTg = kv.F + kv.bo[k];
      for (int o = tid; o < b * bp; o += nt) {
        const int j = o / b, i = o - j * b;
        kkt_fstore(Gg, (long long)b * bp, o, G[i * bp + j]);
        kkt_fstore(GTg, (long long)b * bp, o, G[o]);
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
      kkt_fstore(Sg, (long long)b * b, o, v);
      Sprev[o] = v;
    }
    __syncthreads();
  }
  // the solve reads the factor through the async (bulk-copy) proxy
  asm volatile("fence.proxy.async.global;" ::: "memory");
  __syncthreads();
  return true;
}

// Threads in each half of the solve group: at least the largest block, a
// whole number of warps.
__host__ __device__ inline int kkt_half(int bmax) { return bmax <= 32 ? 32 : ((bmax + 31) & ~31); }

// Lanes per block row in the solve (Q): each row's product is split over Q
// consecutive lanes, so a step's chain of dependent multiply-adds is Q times
// shorter and more of the CTA's warps work on it.  The widest of 4, 2, 1
// whose group (two halves of kkt_group_half threads) leaves a warp for the
// producer.  Measured per step on batched MPC (blocks of ~34): one lane per
// row spent ~130 cycles per double-float term, latency rather than issue.
__host__ __device__ inline int kkt_group_half(int bmax, int q) {
  const int t = q * bmax;
  return t <= 32 ? 32 : ((t + 31) & ~31);
}
__host__ __device__ inline int kkt_lanes(int bmax, int threads) {
  for (int q = 4; q > 1; q >>= 1)
    if (2 * kkt_group_half(bmax, q) + 32 <= threads) return q;
  return 1;
}

__device__ __forceinline__ DF df_add(DF a, DF b) {
  float s, e;
  df_two_sum(a.h, b.h, s, e);
  e = __fadd_rn(e, __fadd_rn(a.l, b.l));
  const float h = __fadd_rn(s, e);
  return DF{h, __fsub_rn(e, __fsub_rn(h, s))};
}

// Row r of the column-major rows x cols block M times entries off.. of the
// solve vector v (n entries), by the Q consecutive lanes q = 0..Q-1 of a lane
// group: lane q takes columns q, q + Q, ... in two interleaved partial sums
// (compensated in the double-float solve), then the group adds its partials
// by xor shuffles, so every lane of the group gets the same value.  Every lane
// of the warp calls it; a lane group without a row passes active = false.
template <int Q, typename T>
__device__ __forceinline__ kkt_val<T> kkt_dot_q(const T* M, const T* v, int n, int off, int rows, int cols, int r,
                                               int q, bool active) {
  const int ce = active ? cols : 0;
  if constexpr (kKktDF<T>) {
    const float* __restrict__ Mh = reinterpret_cast<const float*>(M);
    const float* __restrict__ Ml = Mh + kkt_pad4((long long)rows * cols);
    const float* __restrict__ vh = reinterpret_cast<const float*>(v) + off;
    const float* __restrict__ vl = vh + n;
    float s0 = 0.f, s1 = 0.f, c0 = 0.f, c1 = 0.f;
    auto term = [&](int j, float& sa, float& ca) {
      const size_t o = (size_t)j * rows + r;
      const float mh = Mh[o], ml = Ml[o], xh = vh[j], xl = vl[j];
      const float p = __fmul_rn(mh, xh);
      const float e = __fmaf_rn(mh, xl, __fmaf_rn(ml, xh, __fmaf_rn(mh, xh, -p)));
      float t, es;
      df_two_sum(sa, p, t, es);
      sa = t;
      ca = __fadd_rn(ca, __fadd_rn(es, e));
    };
    int j = q;
    for (; j + Q < ce; j += 2 * Q) {
      term(j, s0, c0);
      term(j + Q, s1, c1);
    }
    if (j < ce) term(j, s0, c0);
    float S, es;
    df_two_sum(s0, s1, S, es);
    const float C = __fadd_rn(__fadd_rn(c0, c1), es);
    const float h = __fadd_rn(S, C);
    DF a{h, __fsub_rn(C, __fsub_rn(h, S))};
#pragma unroll
    for (int o = Q / 2; o > 0; o >>= 1)
      a = df_add(a, DF{__shfl_xor_sync(0xffffffffu, a.h, o), __shfl_xor_sync(0xffffffffu, a.l, o)});
    return a;
  } else {
    const T* __restrict__ x = v + off;
    T a0 = T(0), a1 = T(0);
    int j = q;
    for (; j + Q < ce; j += 2 * Q) {
      a0 += M[(size_t)j * rows + r] * x[j];
      a1 += M[(size_t)(j + Q) * rows + r] * x[j + Q];
    }
    if (j < ce) a0 += M[(size_t)j * rows + r] * x[j];
    T a = a0 + a1;
#pragma unroll
    for (int o = Q / 2; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
    return a;
  }
}

// Barrier of the solve group only (named barrier 1; `threads` a multiple of 32).
__device__ __forceinline__ void kkt_group_sync(int threads) {
  asm volatile("bar.sync 1, %0;" :: "r"(threads) : "memory");
}

// Copy the block starts and segment offsets (read at every block step) and
// the permutation of the n variables and its inverse (read by every
// right-hand side and solution) to on-chip memory `dst` (3 (nb + 1) + 2 n
// ints) and point kv at the copies.
template <typename T>
__device__ __forceinline__ void kkt_plan_on_chip(KktView<T>& kv, int* dst, int n) {
  const int w = kv.nb + 1;
  for (int k = threadIdx.x; k < w; k += blockDim.x) { dst[k] = kv.bs[k]; dst[w + k] = kv.fo[k]; dst[2 * w + k] = kv.bo[k]; }
  int* pm = dst + 3 * w;
  int* ip = pm + n;
  for (int i = threadIdx.x; i < n; i += blockDim.x) { pm[i] = kv.perm[i]; ip[i] = kv.iperm[i]; }
  kv.bs = dst;
  kv.fo = dst + w;
  kv.bo = dst + 2 * w;
  kv.perm = pm;
  kv.iperm = ip;
}

// ---------------------------------------------------------------------------
// Bulk-copy pipeline state of a CTA: per ring slot a "full" and an "empty"
// mbarrier and the number of phases each has completed before the current
// solve.  Copy j of a solve goes to slot j % ring and is the (fph[s] + j /
// ring)-th use of that slot, so its parities follow from these counts even
// when consecutive solves (QPs of different sizes) use different ring sizes.
// Lives in static shared memory; kkt_pipe_init once per kernel before the
// first solve.
// ---------------------------------------------------------------------------
struct KktPipe {
  unsigned long long bar[kKktRingMax];     // "full": copy landed in the slot
  unsigned long long empty[kKktRingMax];   // "empty": the group released the slot
  unsigned fph[kKktRingMax];               // completed phases of bar[s]
  unsigned eph[kKktRingMax];               // completed phases of empty[s]
  int err;                                 // a wait failed: read the factor from global memory
  int issued;                              // copies of the current solve issued so far
  int fail;                                // first copy of the current solve read from global memory
};

__device__ __forceinline__ unsigned kkt_smem(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void kkt_pipe_init(KktPipe* pp) {
  if (threadIdx.x == 0) {
    for (int s = 0; s < kKktRingMax; s++) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(kkt_smem(&pp->bar[s])) : "memory");
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(kkt_smem(&pp->empty[s])) : "memory");
      pp->fph[s] = 0;
      pp->eph[s] = 0;
    }
    pp->err = 0;
    pp->issued = 0;
    pp->fail = 0x7fffffff;
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
// 16-byte aligned), completing a transaction on `bar`.  One thread; earlier
// generic-proxy accesses of the slot are ordered before it by the "empty"
// handshake within a solve and by one fence.proxy.async per solve.
__device__ __forceinline__ void kkt_bulk_load(void* dst, const void* src, unsigned bytes, unsigned long long* bar) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" :: "r"(kkt_smem(bar)), "r"(bytes) : "memory");
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
               :: "r"(kkt_smem(dst)), "l"(src), "r"(bytes), "r"(kkt_smem(bar)) : "memory");
}

__device__ __forceinline__ void kkt_arrive(unsigned long long* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" :: "r"(kkt_smem(bar)) : "memory");
}

// The solve of kkt_solve with the factor streamed through `ring` (kv.ring
// slots of kv.segmax elements).  Copies j = 0..nb-1 are the forward segments,
// j = nb + t the backward segment of block nb - 1 - t; copy j goes to slot
// j % ring.  The producer (the first thread after the group) issues copy j
// once the group released copy j - ring; the group releases a copy after the
// step that last reads it, so every copy of a solve is released by its end.
// Needs blockDim.x >= 2 kkt_half(bmax) + 32 (kkt_lanes picks the lanes per
// row from the rest).
template <typename T, typename XO>
__device__ void kkt_solve_pipe(const KktView<T>& kv, KktPipe* pp, T* c, T* d, T* ring, XO xout,
                               unsigned long long* prof = nullptr, unsigned long long* prof_issue = nullptr,
                               unsigned long long* prof_dot = nullptr) {
  // the view's fields as locals: kv lives in memory that the stores through
  // the generic solve-vector pointers could alias, so every use would reload it
  const int* const bs = kv.bs;
  const int* const fo = kv.fo;
  const int* const bo = kv.bo;
  const int* const perm = kv.perm;
  const T* const F = kv.F;
  // prof (thread 0 only, optional): cycles spent [0] waiting for segments, [1]
  // in group barriers, [2] in the forward sweep, [3] in the backward sweep
  const int QL = kkt_lanes(kv.bmax, blockDim.x);
  const int H = kkt_group_half(kv.bmax, QL), GT = 2 * H;
  const int tid = threadIdx.x;
  const int nb = kv.nb, R = kv.ring, SM = kv.segmax;
  const int n = bs[nb];
  const int total = 2 * nb - 1;
  // parity of the wait for copy j (full) and of the release of copy j (empty)
  auto fpar = [&](int j) { return (pp->fph[j % R] + (unsigned)(j / R)) & 1u; };
  auto epar = [&](int j) { return (pp->eph[j % R] + (unsigned)(j / R)) & 1u; };
  auto seg = [&](int j, long long& elems) -> const T* {
    if (j < nb) {
      const long long b = bs[j + 1] - bs[j], bp = j ? bs[j] - bs[j - 1] : 0;
      elems = kkt_pad4(b * bp) + kkt_pad4(b * b);
      return F + fo[j];
    }
    const int k = nb - 1 - (j - nb);
    const long long b = bs[k + 1] - bs[k], bp = bs[k] - bs[k - 1];
    elems = kkt_pad4(b * bp);
    return F + bo[k];
  };
  auto slot = [&](int j) { return ring + (size_t)(j % R) * SM; };

  if (tid == GT) {
    // ---- producer ----
    const long long t0 = prof_issue ? clock64() : 0;
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    for (int j = 0; j < total; j++) {
      if (*(volatile int*)&pp->err) break;
      // the slot's previous copy of this solve must have been released (copies
      // of earlier solves were, before those solves ended)
      if (j >= R && !kkt_wait(&pp->empty[j % R], epar(j - R))) {
        *(volatile int*)&pp->err = 1;
        break;
      }
      long long el;
      const T* g = seg(j, el);
      kkt_bulk_load(slot(j), g, (unsigned)(el * sizeof(T)), &pp->bar[j % R]);
      *(volatile int*)&pp->issued = j + 1;
    }
    if (prof_issue) *prof_issue += (unsigned long long)(clock64() - t0);
  } else if (tid < GT) {
    // ---- the solve group: Q lanes per block row ----
    auto group = [&](auto Qc) {
      constexpr int Q = decltype(Qc)::value;
      const bool lo = tid < H;
      const int t = lo ? tid : tid - H;   // thread in its half
      const int r = t / Q, q = t % Q;     // block row, lane in the row's group
      long long tw = 0, tb = 0, td = 0;
      const long long t_start = prof ? clock64() : 0;
      long long t_fwd = 0;
      auto sync = [&]() {
        const long long t0 = prof ? clock64() : 0;
        kkt_group_sync(GT);
        if (prof) tb += clock64() - t0;
      };
      auto release = [&](int j) {
        if (tid == 0) kkt_arrive(&pp->empty[j % R]);
      };
      // copy j's data: the ring slot, or global memory after a failed wait
      // (after one failed wait the CTA stops waiting and reads global memory)
      auto get = [&](int j) -> const T* {
        long long el;
        bool ok = !*(volatile int*)&pp->err;
        if (ok) {
          const long long t0 = prof ? clock64() : 0;
          ok = kkt_wait(&pp->bar[j % R], fpar(j));
          if (prof) tw += clock64() - t0;
        }
        if (!ok) {
          *(volatile int*)&pp->err = 1;
          atomicMin(&pp->fail, j);
          return seg(j, el);
        }
        return slot(j);
      };
      const T* cur = get(0);
      for (int k = 1; k < nb; k++) {
        const int s0 = bs[k], b = bs[k + 1] - s0, sp = bs[k - 1], bp = s0 - sp;
        const int spp = k > 1 ? bs[k - 2] : sp;
        const T* prev = cur;              // segment k - 1: S_{k-1}^-1 after G_{k-1}
        cur = get(k);                     // segment k: G_k first
        if (lo) {
          const long long t0 = prof_dot ? clock64() : 0;
          const bool a = r < b;
          const kkt_val<T> v = kkt_dot_q<Q>(cur, c, n, sp, b, bp, a ? r : 0, q, a);
          if (a && q == 0) kkt_vsub(c, n, s0 + r, v);
          if (prof_dot) td += clock64() - t0;
        } else {
          const bool a = r < bp;
          const kkt_val<T> v = kkt_dot_q<Q>(prev + kkt_pad4((long long)bp * (sp - spp)), c, n, sp, bp, bp, a ? r : 0, q, a);
          if (a && q == 0) kkt_vset(d, n, sp + r, v);
        }
        sync();
        release(k - 1);
      }
      {
        const int s0 = bs[nb - 1], b = bs[nb] - s0;
        const int bp = nb > 1 ? s0 - bs[nb - 2] : 0;
        if (lo) {
          const bool a = r < b;
          const kkt_val<T> v = kkt_dot_q<Q>(cur + kkt_pad4((long long)b * bp), c, n, s0, b, b, a ? r : 0, q, a);
          if (a && q == 0) kkt_vset(d, n, s0 + r, v);
        }
        sync();
        release(nb - 1);
      }
      if (prof) t_fwd = clock64();
      for (int u = 0; u + 1 < nb; u++) {
        const int k = nb - 1 - u;
        const int s0 = bs[k], b = bs[k + 1] - s0, sp = bs[k - 1], bp = s0 - sp;
        const T* Gt = get(nb + u);
        if (lo) {
          const long long t0 = prof_dot ? clock64() : 0;
          const bool a = r < bp;
          const kkt_val<T> v = kkt_dot_q<Q>(Gt, d, n, s0, bp, b, a ? r : 0, q, a);
          if (a && q == 0) kkt_vsub(d, n, sp + r, v);
          if (prof_dot) td += clock64() - t0;
        } else {
          if (t < b) xout(perm[s0 + t], kkt_vget(d, n, s0 + t));
        }
        sync();
        release(nb + u);
      }
      for (int i = tid; i < bs[1]; i += GT) xout(perm[i], kkt_vget(d, n, i));
      if (prof) {
        const long long t_end = clock64();
        prof[0] += (unsigned long long)tw; prof[1] += (unsigned long long)tb;
        if (prof_dot) *prof_dot += (unsigned long long)td;
        prof[2] += (unsigned long long)(t_fwd - t_start); prof[3] += (unsigned long long)(t_end - t_fwd);
      }
    };
    if (QL == 4) group(std::integral_constant<int, 4>{});
    else if (QL == 2) group(std::integral_constant<int, 2>{});
    else group(std::integral_constant<int, 1>{});
  }
  __syncthreads();
  if (tid == 0) {
    if (*(volatile int*)&pp->err) {
      // copies issued but not waited for land before the CTA goes on; then,
      // with nothing in flight, the barriers start afresh.  A copy that
      // still does not land keeps the pipe off for the rest of the kernel.
      const int iss = *(volatile int*)&pp->issued;
      bool drained = true;
      for (int j = pp->fail; j < iss; j++) drained = kkt_wait(&pp->bar[j % R], fpar(j)) && drained;
      if (drained) {
        for (int q = 0; q < kKktRingMax; q++) {
          asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(kkt_smem(&pp->bar[q])) : "memory");
          asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(kkt_smem(&pp->empty[q])) : "memory");
          pp->fph[q] = 0;
          pp->eph[q] = 0;
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        pp->err = 0;
      }
    } else {
      // every copy of the solve landed and was released
      for (int q = 0; q < R && q < total; q++) {
        const unsigned uses = (unsigned)((total - 1 - q) / R + 1);
        pp->fph[q] += uses;
        pp->eph[q] += uses;
      }
    }
    pp->issued = 0;
    pp->fail = 0x7fffffff;
  }
  __syncthreads();
}

// Solve K x = b with the factor read from global memory: c holds the permuted
// right-hand side on entry (c[iperm[i]] = b_i); d is a second permuted
// n-vector; x (unpermuted) is written through xout(i, value).  All threads of
// the CTA call it; the solve group of kkt_solve_pipe does the block steps.
template <typename T, typename XO>
__device__ void kkt_solve(const KktView<T>& kv, T* c, T* d, XO xout) {
  // the view's fields as locals: kv lives in memory that the stores through
  // the generic solve-vector pointers could alias, so every use would reload it
  const int* const bs = kv.bs;
  const int* const fo = kv.fo;
  const int* const bo = kv.bo;
  const int* const perm = kv.perm;
  const T* const F = kv.F;
  const int QL = kkt_lanes(kv.bmax, blockDim.x);
  const int H = kkt_group_half(kv.bmax, QL), GT = 2 * H;
  const int tid = threadIdx.x;
  const int nb = kv.nb, n = bs[nb];
  auto group = [&](auto Qc) {
    constexpr int Q = decltype(Qc)::value;
    const bool lo = tid < H;
    const int t = lo ? tid : tid - H;
    const int r = t / Q, q = t % Q;
    // forward: c_k -= G_k c_{k-1} (lower half) while d_{k-1} = S_{k-1}^-1 c_{k-1} (upper half)
    for (int k = 1; k < nb; k++) {
      const int s0 = bs[k], b = bs[k + 1] - s0, sp = bs[k - 1], bp = s0 - sp;
      const int spp = k > 1 ? bs[k - 2] : sp;
      if (lo) {
        const bool a = r < b;
        const kkt_val<T> v = kkt_dot_q<Q>(F + fo[k], c, n, sp, b, bp, a ? r : 0, q, a);
        if (a && q == 0) kkt_vsub(c, n, s0 + r, v);
      } else {
        const bool a = r < bp;
        const kkt_val<T> v =
            kkt_dot_q<Q>(F + fo[k - 1] + kkt_pad4((long long)bp * (sp - spp)), c, n, sp, bp, bp, a ? r : 0, q, a);
        if (a && q == 0) kkt_vset(d, n, sp + r, v);
      }
      kkt_group_sync(GT);
    }
    {
      const int s0 = bs[nb - 1], b = bs[nb] - s0;
      const int bp = nb > 1 ? s0 - bs[nb - 2] : 0;
      if (lo) {
        const bool a = r < b;
        const kkt_val<T> v = kkt_dot_q<Q>(F + fo[nb - 1] + kkt_pad4((long long)b * bp), c, n, s0, b, b, a ? r : 0, q, a);
        if (a && q == 0) kkt_vset(d, n, s0 + r, v);
      }
      kkt_group_sync(GT);
    }
    // backward: x_{k-1} = d_{k-1} - G_k' x_k (lower half) while block k is written out (upper half)
    for (int k = nb - 1; k >= 1; k--) {
      const int s0 = bs[k], b = bs[k + 1] - s0, sp = bs[k - 1], bp = s0 - sp;
      if (lo) {
        const bool a = r < bp;
        const kkt_val<T> v = kkt_dot_q<Q>(F + bo[k], d, n, s0, bp, b, a ? r : 0, q, a);
        if (a && q == 0) kkt_vsub(d, n, sp + r, v);
      } else {
        if (t < b) xout(perm[s0 + t], kkt_vget(d, n, s0 + t));
      }
      kkt_group_sync(GT);
    }
    for (int i = tid; i < bs[1]; i += GT) xout(perm[i], kkt_vget(d, n, i));
  };
  if (tid < GT) {
    if (QL == 4) group(std::integral_constant<int, 4>{});
    else if (QL == 2) group(std::integral_constant<int, 2>{});
    else group(std::integral_constant<int, 1>{});
  }
  __syncthreads();
}

// ---------------------------------------------------------------------------
// Diagonal-plus-dense-rows form (gb_kkt_plan.h)
// ---------------------------------------------------------------------------

// Copy the dense-row list and the row map to on-chip memory `dst` (r + m ints).
template <typename T>
__device__ __forceinline__ void dr_on_chip(KktView<T>& kv, int* dst, int m) {
  int* rows = dst;
  int* didx = dst + kv.dr;
  for (int k = threadIdx.x; k < kv.dr; k += blockDim.x) rows[k] = kv.drows[k];
  for (int j = threadIdx.x; j < m; j += blockDim.x) didx[j] = kv.didx[j];
  kv.drows = rows;
  kv.didx = didx;
}

// Dg^-1 and C^-1 for the current rho (scaled data).  C is formed and inverted
// in place in kv.Cinv (global memory, L2-resident: r r elements); ws: on-chip
// workspace of n elements.  Returns false when Dg or C has a pivot that is
// not positive (K not positive definite).  All threads of the CTA call it;
// every entry has one owner and a fixed summation order.
template <typename T>
__device__ __noinline__ bool dr_factor(const KktView<T>& kv, int n, const CSR<T>& P, const CSR<T>& A,
                                       const CSR<T>& At, const T* rho_vec, T rho_s, T sigma, T* ws) {
  const int tid = threadIdx.x, nt = blockDim.x;
  const int lane = tid & 31, warp = tid >> 5, nwarps = nt >> 5;
  const int r = kv.dr;
  T* C = kv.Cinv;
  T* sv = ws;
  __shared__ int s_bad;
  if (tid == 0) s_bad = 0;
  __syncthreads();
  // Dg = P_ii + sigma + the single-entry rows' rho a^2: one warp per variable
  for (int i = warp; i < n; i += nwarps) {
    T pdiag = T(0), dsum = T(0);
    for (int e = P.rowptr[i] + lane; e < P.rowptr[i + 1]; e += 32)
      if (P.col[e] == i) pdiag = P.val[e];
    for (int e = At.rowptr[i] + lane; e < At.rowptr[i + 1]; e += 32) {
      const int row = At.col[e];
      if (kv.didx[row] < 0) {
        const T a = At.val[e];
        dsum += (a * a) * (rho_vec ? rho_vec[row] : rho_s);
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      dsum += __shfl_xor_sync(0xffffffffu, dsum, o);
      pdiag += __shfl_xor_sync(0xffffffffu, pdiag, o);   // one lane holds it
    }
    if (lane == 0) {
      const T d = (pdiag + sigma) + dsum;
      if (!(d > T(0)) || !isfinite((double)d)) s_bad = 1;
      kv.Dginv[i] = T(1) / d;
    }
  }
  __syncthreads();
  if (s_bad) return false;
  // C = R_d^-1 + A_d Dg^-1 A_d': row a of A_d scaled by Dg^-1 is scattered into
  // sv, then every C_ab (b >= a) is one warp's dot of row b with it
  for (int i = tid; i < n; i += nt) sv[i] = T(0);
  __syncthreads();
  for (int a = 0; a < r; a++) {
    const int ra = kv.drows[a];
    for (int e = A.rowptr[ra] + tid; e < A.rowptr[ra + 1]; e += nt) sv[A.col[e]] = A.val[e] * kv.Dginv[A.col[e]];
    __syncthreads();
    for (int b = a + warp; b < r; b += nwarps) {
      const int rb = kv.drows[b];
      Acc<T> acc;   // double-float in the FP32 build: a dense row sums many entries
      for (int e = A.rowptr[rb] + lane; e < A.rowptr[rb + 1]; e += 32) acc.add_prod(A.val[e], sv[A.col[e]]);
      warp_accT(acc);
      if (lane == 0) {
        double c = acc.value();
        if (b == a) c += 1.0 / (double)(rho_vec ? rho_vec[ra] : rho_s);
        C[(size_t)a * r + b] = (T)c;
        C[(size_t)b * r + a] = (T)c;
      }
    }
    __syncthreads();
    for (int e = A.rowptr[ra] + tid; e < A.rowptr[ra + 1]; e += nt) sv[A.col[e]] = T(0);
    __syncthreads();
  }
  // in-place symmetric sweeps (C stays exactly symmetric): -C^-1 after r sweeps
  for (int k = 0; k < r; k++) {
    const T piv = C[(size_t)k * r + k];
    if (!(piv > T(0)) || !isfinite((double)piv)) return false;   // CTA-uniform
    const T d = T(1) / piv;
    for (int o = tid; o < r * r; o += nt) {
      const int i = o / r, j = o - i * r;
      if (i != k && j != k) C[o] -= (C[(size_t)i * r + k] * C[(size_t)k * r + j]) * d;
    }
    __syncthreads();
    for (int o = tid; o < r; o += nt)
      if (o != k) { C[(size_t)o * r + k] *= d; C[(size_t)k * r + o] *= d; }
    if (tid == 0) C[(size_t)k * r + k] = -d;
    __syncthreads();
  }
  for (int o = tid; o < r * r; o += nt) C[o] = -C[o];
  __syncthreads();
  return true;
}

}  // namespace gb
