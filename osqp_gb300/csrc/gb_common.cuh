// gb_common.cuh -- shared device building blocks of the GB300 OSQP engine.
//
// * Group abstraction: the same device code runs an OSQP solve either on one
//   CTA (BlockGroup: batched instances, small problems; barrier =
//   __syncthreads) or on a cooperative persistent grid (GridGroup: one large
//   QP; barrier = bounded generation-counter grid barrier).
// * Deterministic reductions: every reduction is summed in FP64 in a fixed
//   order (warp shuffle tree, warps in index order, blocks in index order), so
//   a rerun reproduces every bit and all CTAs of a grid obtain identical
//   scalars, which lets each CTA keep its own copy of the solver's scalar state.
// * CSR row kernels with 1..32 lanes per row (sub-warp per row).
#pragma once

#include <cooperative_groups.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace gb {

constexpr int kMaxSum = 8;   // FP64 sum slots per reduction
constexpr int kMaxMax = 24;  // FP64 max slots per reduction
constexpr int kWarp = 32;

// Spin limit of the grid barrier: ~2^24 polls with 64 ns back-off is roughly
// one second of waiting before the kernel records an error and returns.
constexpr long long kBarrierSpinLimit = 1LL << 24;

// Error codes written to a kernel's error word (never a trap).
enum DevError : int {
  kErrNone = 0,
  kErrBarrierTimeout = 1,
  kErrBadShape = 2,
};

struct RedBuf {
  double sum[kMaxSum];
  double mx[kMaxMax];
};

// ---------------------------------------------------------------------------
// Warp helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
template <int L, typename T>
__device__ __forceinline__ T subwarp_sum(T v) {
#pragma unroll
  for (int o = L / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o, L);
  return v;
}


// ---------------------------------------------------------------------------
// Extended-precision sums without the FP64 pipe.
//
// GB300 executes FP64 at ~1/64 of the FP32 rate, so FP32-build reductions
// accumulate in "double-float": an unevaluated pair (hi, lo) of floats,
// updated with error-free transformations on the FP32 pipe --
// TwoProduct (p = a*b, e = fma(a,b,-p), exact) and TwoSum (Knuth) -- which
// carries ~48 significant bits, then widens to FP64 once per reduction.  The
// summation order is fixed, so results are bit-reproducible.  Max reductions
// of FP32 data are exact in FP32.  The FP64 build accumulates in double.
// ---------------------------------------------------------------------------
template <typename T> struct Acc;

template <> struct Acc<float> {
  float hi, lo;
  __device__ __forceinline__ Acc() : hi(0.f), lo(0.f) {}
  __device__ __forceinline__ static void two_sum(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  }
  __device__ __forceinline__ void add2(float h, float l) {
    float s, e;
    two_sum(hi, h, s, e);
    e = __fadd_rn(e, __fadd_rn(lo, l));
    hi = __fadd_rn(s, e);
    lo = __fsub_rn(e, __fsub_rn(hi, s));
  }
  __device__ __forceinline__ void add(float v) { add2(v, 0.f); }
  __device__ __forceinline__ void add_prod(float a, float b) {
    const float p = __fmul_rn(a, b);
    add2(p, __fmaf_rn(a, b, -p));
  }
  __device__ __forceinline__ void merge(const Acc& o) { add2(o.hi, o.lo); }
  __device__ __forceinline__ void shfl_merge(int off) {
    const float h = __shfl_xor_sync(0xffffffffu, hi, off);
    const float l = __shfl_xor_sync(0xffffffffu, lo, off);
    add2(h, l);
  }
  __device__ __forceinline__ double value() const { return (double)hi + (double)lo; }
};

template <> struct Acc<double> {
  double v;
  __device__ __forceinline__ Acc() : v(0.0) {}
  __device__ __forceinline__ void add(double a) { v += a; }
  __device__ __forceinline__ void add_prod(double a, double b) { v = fma(a, b, v); }
  __device__ __forceinline__ void merge(const Acc& o) { v += o.v; }
  __device__ __forceinline__ void shfl_merge(int off) { v += __shfl_xor_sync(0xffffffffu, v, off); }
  __device__ __forceinline__ double value() const { return v; }
};

template <typename T>
__device__ __forceinline__ T warp_maxT(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
template <typename T>
__device__ __forceinline__ void warp_accT(Acc<T>& a) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) a.shfl_merge(o);
}

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}

// ---------------------------------------------------------------------------
// Groups
// ---------------------------------------------------------------------------
// Shared scratch every group needs: per-warp partials and broadcast results.
struct GroupShared {
  double wsum[32][kMaxSum][2];   // per-warp partial sums (hi, lo) or (v, 0)
  double wmax[32][kMaxMax];      // per-warp partial maxima
  double rsum[kMaxSum];
  double rmax[kMaxMax];
  int flag;
  int parity;   // which half of the grid partial buffers the next reduction uses
  double csum[2][kMaxSum][2];  // cluster form: this CTA's partial sums (double-buffered)
  double cmax[2][kMaxMax];     // cluster form: this CTA's partial maxima
  int cidx;                    // cluster form: work item broadcast by rank 0
};

// Sum/max slot helpers shared by both group kinds.
template <typename T>
__device__ __forceinline__ void acc_store(double* dst, const Acc<T>& a);
template <>
__device__ __forceinline__ void acc_store<float>(double* dst, const Acc<float>& a) { dst[0] = a.hi; dst[1] = a.lo; }
template <>
__device__ __forceinline__ void acc_store<double>(double* dst, const Acc<double>& a) { dst[0] = a.v; dst[1] = 0.0; }
template <typename T>
__device__ __forceinline__ Acc<T> acc_load(const double* src);
template <>
__device__ __forceinline__ Acc<float> acc_load<float>(const double* src) { Acc<float> a; a.hi = (float)src[0]; a.lo = (float)src[1]; return a; }
template <>
__device__ __forceinline__ Acc<double> acc_load<double>(const double* src) { Acc<double> a; a.v = src[0]; return a; }

// One CTA cooperates on one problem.
struct BlockGroup {
  GroupShared* sh;
  __device__ int nthreads() const { return blockDim.x; }
  __device__ int tid() const { return threadIdx.x; }
  __device__ int nwarps() const { return blockDim.x >> 5; }
  __device__ int warp() const { return threadIdx.x >> 5; }
  __device__ bool sync() { __syncthreads(); return true; }
  __device__ bool ok() const { return true; }

  // Reduce NS sums and NM maxima across the CTA; every thread receives the
  // FP64 results in rs / rm.
  template <typename T, int NS, int NM>
  __device__ void reduce(Acc<T> (&s)[NS], T (&m)[NM], double (&rs)[NS], double (&rm)[NM]) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int i = 0; i < NS; i++) { warp_accT(s[i]); if (lane == 0) acc_store(sh->wsum[w][i], s[i]); }
#pragma unroll
    for (int i = 0; i < NM; i++) { T v = warp_maxT(m[i]); if (lane == 0) sh->wmax[w][i] = (double)v; }
    __syncthreads();
    const int nw = blockDim.x >> 5;
    if (threadIdx.x < NS) {
      Acc<T> a;
      for (int k = 0; k < nw; k++) a.merge(acc_load<T>(sh->wsum[k][threadIdx.x]));
      sh->rsum[threadIdx.x] = a.value();
    } else if (threadIdx.x >= 32 && threadIdx.x < 32 + NM) {
      const int i = threadIdx.x - 32;
      double a = sh->wmax[0][i];
      for (int k = 1; k < nw; k++) a = fmax(a, sh->wmax[k][i]);
      sh->rmax[i] = a;
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < NS; i++) rs[i] = sh->rsum[i];
#pragma unroll
    for (int i = 0; i < NM; i++) rm[i] = sh->rmax[i];
    __syncthreads();
  }
};


// The CTAs of one thread-block cluster cooperate on one problem: barriers are
// the hardware cluster barrier (no spinning), and each CTA reads the other
// CTAs' partial reductions straight from their shared memory (DSMEM) in rank
// order, so every CTA obtains identical results.
struct ClusterGroup {
  GroupShared* sh;
  unsigned rank, size;
  __device__ int nthreads() const { return blockDim.x * size; }
  __device__ int tid() const { return rank * blockDim.x + threadIdx.x; }
  __device__ int nwarps() const { return (blockDim.x >> 5) * size; }
  __device__ int warp() const { return rank * (blockDim.x >> 5) + (threadIdx.x >> 5); }
  __device__ bool sync() { cooperative_groups::this_cluster().sync(); return true; }
  __device__ bool ok() const { return true; }

  template <typename T, int NS, int NM>
  __device__ void reduce(Acc<T> (&s)[NS], T (&m)[NM], double (&rs)[NS], double (&rm)[NM]) {
    namespace cgr = cooperative_groups;
    cgr::cluster_group cl = cgr::this_cluster();
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int i = 0; i < NS; i++) { warp_accT(s[i]); if (lane == 0) acc_store(sh->wsum[w][i], s[i]); }
#pragma unroll
    for (int i = 0; i < NM; i++) { T v = warp_maxT(m[i]); if (lane == 0) sh->wmax[w][i] = (double)v; }
    __syncthreads();
    const int nw = blockDim.x >> 5;
    const int par = sh->parity;
    if (threadIdx.x < NS) {
      Acc<T> a;
      for (int k = 0; k < nw; k++) a.merge(acc_load<T>(sh->wsum[k][threadIdx.x]));
      acc_store(sh->csum[par][threadIdx.x], a);
    } else if (threadIdx.x >= 32 && threadIdx.x < 32 + NM) {
      const int i = threadIdx.x - 32;
      double a = sh->wmax[0][i];
      for (int k = 1; k < nw; k++) a = fmax(a, sh->wmax[k][i]);
      sh->cmax[par][i] = a;
    }
    cl.sync();
    if (threadIdx.x < NS) {
      Acc<T> a;
      for (unsigned r = 0; r < size; r++) {
        const double* src = cl.map_shared_rank(&sh->csum[par][threadIdx.x][0], r);
        double t2[2] = {src[0], src[1]};
        a.merge(acc_load<T>(t2));
      }
      sh->rsum[threadIdx.x] = a.value();
    } else if (threadIdx.x >= 32 && threadIdx.x < 32 + NM) {
      const int i = threadIdx.x - 32;
      double a = -INFINITY;
      for (unsigned r = 0; r < size; r++) a = fmax(a, *cl.map_shared_rank(&sh->cmax[par][i], r));
      sh->rmax[i] = a;
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < NS; i++) rs[i] = sh->rsum[i];
#pragma unroll
    for (int i = 0; i < NM; i++) rm[i] = sh->rmax[i];
    __syncthreads();
    // The other half of csum / cmax is written by the next reduction; no CTA
    // can overwrite this half before every CTA has passed the next cluster barrier.
    if (threadIdx.x == 0) sh->parity ^= 1;
    __syncthreads();
  }
};

// All CTAs of a cooperative launch cooperate on one problem.
struct GridSync {
  unsigned int* count;   // arrival counter
  unsigned int* gen;     // generation
  int* err;              // error word (kErrBarrierTimeout on a stuck barrier)
  double* partial_sum;   // [2][kMaxSum][gridDim.x][2] (double-buffered)
  double* partial_max;   // [2][kMaxMax][gridDim.x]
};

struct GridGroup {
  GroupShared* sh;
  GridSync gs;
  __device__ int nthreads() const { return blockDim.x * gridDim.x; }
  __device__ int tid() const { return blockIdx.x * blockDim.x + threadIdx.x; }
  __device__ int nwarps() const { return (blockDim.x >> 5) * gridDim.x; }
  __device__ int warp() const { return blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); }

  // Bounded barrier.  Returns false (in every CTA) once any CTA timed out.
  __device__ bool sync() {
    __syncthreads();
    if (threadIdx.x == 0) {
      volatile unsigned int* vgen = gs.gen;
      unsigned int my_gen = *vgen;
      __threadfence();
      unsigned int arrived = atomicAdd(gs.count, 1u);
      if (arrived == gridDim.x - 1) {
        atomicExch(gs.count, 0u);
        __threadfence();
        atomicAdd(gs.gen, 1u);
      } else {
        long long spins = 0;
        while (*vgen == my_gen) {
          if (++spins > kBarrierSpinLimit) { atomicExch(gs.err, (int)kErrBarrierTimeout); break; }
          if (*((volatile int*)gs.err) != 0) break;
          __nanosleep(64);
        }
      }
      __threadfence();
      sh->flag = *((volatile int*)gs.err);
    }
    __syncthreads();
    return sh->flag == 0;
  }
  __device__ bool ok() const { return sh->flag == 0; }

  template <typename T, int NS, int NM>
  __device__ void reduce(Acc<T> (&s)[NS], T (&m)[NM], double (&rs)[NS], double (&rm)[NM]) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int i = 0; i < NS; i++) { warp_accT(s[i]); if (lane == 0) acc_store(sh->wsum[w][i], s[i]); }
#pragma unroll
    for (int i = 0; i < NM; i++) { T v = warp_maxT(m[i]); if (lane == 0) sh->wmax[w][i] = (double)v; }
    __syncthreads();
    const int nw = blockDim.x >> 5, nb = gridDim.x;
    const int par = sh->parity;
    double* ps = gs.partial_sum + (size_t)par * kMaxSum * 2 * nb;   // [slot][block][2]
    double* pm = gs.partial_max + (size_t)par * kMaxMax * nb;       // [slot][block]
    if (threadIdx.x < NS) {
      Acc<T> a;
      for (int k = 0; k < nw; k++) a.merge(acc_load<T>(sh->wsum[k][threadIdx.x]));
      acc_store(ps + ((size_t)threadIdx.x * nb + blockIdx.x) * 2, a);
    } else if (threadIdx.x >= 32 && threadIdx.x < 32 + NM) {
      const int i = threadIdx.x - 32;
      double a = sh->wmax[0][i];
      for (int k = 1; k < nw; k++) a = fmax(a, sh->wmax[k][i]);
      pm[i * nb + blockIdx.x] = a;
    }
    sync();
    // Every CTA reduces the per-CTA partials in the same order.  The other
    // half of the buffers is written by the next reduction, so no CTA can
    // overwrite these values before every CTA has passed the next barrier.
    if (w == 0) {
      for (int i = 0; i < NS; i++) {
        Acc<T> a;
        for (int b = lane; b < nb; b += 32) {
          const volatile double* src = ps + ((size_t)i * nb + b) * 2;
          double tmp[2] = {src[0], src[1]};
          a.merge(acc_load<T>(tmp));
        }
        warp_accT(a);
        if (lane == 0) sh->rsum[i] = a.value();
      }
    } else if (w == 1) {
      for (int i = 0; i < NM; i++) {
        double a = -INFINITY;
        for (int b = lane; b < nb; b += 32) a = fmax(a, ((volatile double*)pm)[i * nb + b]);
        a = warp_max(a);
        if (lane == 0) sh->rmax[i] = a;
      }
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < NS; i++) rs[i] = sh->rsum[i];
#pragma unroll
    for (int i = 0; i < NM; i++) rm[i] = sh->rmax[i];
    __syncthreads();
    if (threadIdx.x == 0) sh->parity ^= 1;
    __syncthreads();
  }
};

// ---------------------------------------------------------------------------
// CSR matrices and row-parallel iteration
// ---------------------------------------------------------------------------
template <typename T>
struct CSR {
  const int* rowptr;
  const int* col;
  T* val;
  int rows;
  int cols;
  int lanes;  // lanes per row: 1,2,4,8,16,32
};


// Dot product of one CSR row segment handled by a sub-warp lane: entries
// b+sl, b+sl+L, ... < e.  Four entries are fetched per round before any is
// used, so each lane keeps four index/value loads and four gathers in flight.
template <int L, typename T, typename XF>
__device__ __forceinline__ T lane_row_dot(const int* __restrict__ col, const T* __restrict__ val,
                                          int b, int e, int sl, XF xf) {
  T acc = T(0);
  for (int k0 = b + sl; k0 < e; k0 += 4 * L) {
    int c[4];
    T v[4];
#pragma unroll
    for (int u = 0; u < 4; u++) {
      const int k = k0 + u * L;
      c[u] = k < e ? col[k] : -1;
      v[u] = k < e ? val[k] : T(0);
    }
    T x[4];
#pragma unroll
    for (int u = 0; u < 4; u++) x[u] = c[u] >= 0 ? xf(c[u]) : T(0);
#pragma unroll
    for (int u = 0; u < 4; u++) acc += v[u] * x[u];
  }
  return acc;
}

// Two products of the same row (shared index and value loads).
template <int L, typename T, typename XF1, typename XF2>
__device__ __forceinline__ void lane_row_dot2(const int* __restrict__ col, const T* __restrict__ val,
                                              int b, int e, int sl, XF1 xf1, XF2 xf2, T& a1, T& a2) {
  for (int k0 = b + sl; k0 < e; k0 += 4 * L) {
    int c[4];
    T v[4];
#pragma unroll
    for (int u = 0; u < 4; u++) {
      const int k = k0 + u * L;
      c[u] = k < e ? col[k] : -1;
      v[u] = k < e ? val[k] : T(0);
    }
    T x1[4], x2[4];
#pragma unroll
    for (int u = 0; u < 4; u++) {
      x1[u] = c[u] >= 0 ? xf1(c[u]) : T(0);
      x2[u] = c[u] >= 0 ? xf2(c[u]) : T(0);
    }
#pragma unroll
    for (int u = 0; u < 4; u++) { a1 += v[u] * x1[u]; a2 += v[u] * x2[u]; }
  }
}

// Visit every row of M; each sub-warp of L lanes computes sum_k val[k]*xf(col[k])
// for its row and calls fn(row, dot) on the sub-warp's lane 0.  Warp-uniform
// loop trip counts keep every shuffle convergent.
template <int L, typename T, typename G, typename XF, typename FN>
__device__ __forceinline__ void rows_apply_L(G& g, const CSR<T>& M, XF xf, FN fn) {
  const int lane = threadIdx.x & 31;
  const int sub = lane / L, sl = lane % L;
  constexpr int RPW = 32 / L;  // rows per warp step
  const int nw = g.nwarps(), w = g.warp();
  for (int base = w * RPW; base < M.rows; base += nw * RPW) {
    const int r = base + sub;
    T acc = T(0);
    if (r < M.rows) acc = lane_row_dot<L>(M.col, M.val, M.rowptr[r], M.rowptr[r + 1], sl, xf);
    acc = subwarp_sum<L>(acc);
    if (r < M.rows && sl == 0) fn(r, acc);
  }
}

template <typename T, typename G, typename XF, typename FN>
__device__ __forceinline__ void rows_apply(G& g, const CSR<T>& M, XF xf, FN fn) {
  switch (M.lanes) {
    case 1:  rows_apply_L<1>(g, M, xf, fn); break;
    case 2:  rows_apply_L<2>(g, M, xf, fn); break;
    case 4:  rows_apply_L<4>(g, M, xf, fn); break;
    case 8:  rows_apply_L<8>(g, M, xf, fn); break;
    case 16: rows_apply_L<16>(g, M, xf, fn); break;
    default: rows_apply_L<32>(g, M, xf, fn); break;
  }
}

// Two products with the same matrix in one pass (shared index loads).
template <int L, typename T, typename G, typename XF1, typename XF2, typename FN>
__device__ __forceinline__ void rows_apply2_L(G& g, const CSR<T>& M, XF1 xf1, XF2 xf2, FN fn) {
  const int lane = threadIdx.x & 31;
  const int sub = lane / L, sl = lane % L;
  constexpr int RPW = 32 / L;
  const int nw = g.nwarps(), w = g.warp();
  for (int base = w * RPW; base < M.rows; base += nw * RPW) {
    const int r = base + sub;
    T a1 = T(0), a2 = T(0);
    if (r < M.rows) lane_row_dot2<L>(M.col, M.val, M.rowptr[r], M.rowptr[r + 1], sl, xf1, xf2, a1, a2);
    a1 = subwarp_sum<L>(a1);
    a2 = subwarp_sum<L>(a2);
    if (r < M.rows && sl == 0) fn(r, a1, a2);
  }
}
template <typename T, typename G, typename XF1, typename XF2, typename FN>
__device__ __forceinline__ void rows_apply2(G& g, const CSR<T>& M, XF1 a, XF2 b, FN fn) {
  switch (M.lanes) {
    case 1:  rows_apply2_L<1>(g, M, a, b, fn); break;
    case 2:  rows_apply2_L<2>(g, M, a, b, fn); break;
    case 4:  rows_apply2_L<4>(g, M, a, b, fn); break;
    case 8:  rows_apply2_L<8>(g, M, a, b, fn); break;
    case 16: rows_apply2_L<16>(g, M, a, b, fn); break;
    default: rows_apply2_L<32>(g, M, a, b, fn); break;
  }
}

// Lanes per row from the mean row length: about four entries per lane
// (power of two, 1..32), so short rows pack several rows into a warp.
inline int pick_lanes(long long nnz, int rows) {
  if (rows <= 0) return 1;
  const double mean = (double)nnz / rows;
  int L = 1;
  while (L < 32 && L * 4 < mean) L <<= 1;
  return L;
}

// Element-wise loop over [b, e) across the group.
template <typename G, typename FN>
__device__ __forceinline__ void for_range(G& g, int b, int e, FN fn) {
  const int nt = g.nthreads();
  for (int i = b + g.tid(); i < e; i += nt) fn(i);
}

// Element-wise loop over [0, n) across the group.
template <typename G, typename FN>
__device__ __forceinline__ void for_each(G& g, int n, FN fn) {
  const int nt = g.nthreads();
  for (int i = g.tid(); i < n; i += nt) fn(i);
}

}  // namespace gb
