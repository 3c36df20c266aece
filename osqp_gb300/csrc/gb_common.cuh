// gb_common.cuh -- shared device building blocks of the GB300 OSQP engine.
//
// * Group abstraction: the same device code runs an OSQP solve on one CTA
//   (BlockGroup: batched instances, small problems; barrier = __syncthreads),
//   on a thread-block cluster (ClusterGroup: contiguous row slices per CTA,
//   hardware cluster barrier, partials exchanged through distributed shared
//   memory) or on a cooperative persistent grid (GridGroup: one large QP;
//   barrier = bounded generation-counter grid barrier).
// * Deterministic reductions: sums are accumulated in double-float (FP32
//   build) or FP64 and combined in a fixed order (lanes, warps, CTAs, ranks),
//   so a rerun reproduces every bit and all CTAs of a group obtain identical
//   scalars, which lets each CTA keep its own copy of the solver's scalar state.
// * CSR row kernels with 1..32 lanes per row (sub-warp per row), several rows
//   in flight per lane group; for the FP64 build, dense batches of 32 rows per
//   warp whose follow-up work runs one row per lane, and maxima and bound
//   tests on the integer pipe (FP64 instructions are slow on GB300).
#pragma once

#include <cooperative_groups.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

namespace gb {

constexpr int kMaxSum = 8;   // FP64 sum slots per reduction
constexpr int kMaxMax = 24;  // FP64 max slots per reduction
constexpr int kWarp = 32;
constexpr int kProfSlots = 16;   // per-phase cycle counters of a solve (DevSettings::profile)

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

// a / b for double-float a = (ah, al), b = (bh, bl), rounded to float: one
// correction step of the float quotient (Dekker's method; the remainder
// ah - q bh is exact with an FMA), on the FP32 pipe.
__device__ __forceinline__ float df_div(float ah, float al, float bh, float bl) {
  const float q1 = __fdiv_rn(ah, bh);
  const float r = __fmaf_rn(-q1, bh, ah) + (al - q1 * bl);
  return q1 + __fdiv_rn(r, bh);
}

template <typename T>
__device__ __forceinline__ T tmaxT(T a, T b) { return a > b ? a : (b == b ? b : a); }

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

// ---------------------------------------------------------------------------
// Maxima and bound tests on the integer pipe.
//
// GB300 issues an FP64 warp instruction in about 65-77 cycles of its SM
// sub-partition, whatever the number of active lanes, and the FP64 max and
// compare instructions (DMNMX, DSETP) go down that pipe too.  Maxima of |v|
// are therefore kept as bit patterns (nonnegative IEEE numbers order as
// their patterns) and reduced with integer compares; signed maxima use the
// usual order-preserving map of the pattern.  A NaN is ignored, as the
// reference's infinity norm ignores it (its test |v_i| > max is false for
// NaN).  Comparisons of a value with a positive threshold use the signed
// integer view of the pattern: for p > 0, v > p iff bits(v) > bits(p) and
// v < p iff bits(v) < bits(p), for every v that is not NaN.
// ---------------------------------------------------------------------------
template <typename T> struct FKey;
template <> struct FKey<double> {
  typedef unsigned long long U;
  typedef long long I;
  static constexpr U kAbs = 0x7fffffffffffffffull, kInf = 0x7ff0000000000000ull, kSign = 0x8000000000000000ull;
  static __device__ __forceinline__ I bits(double v) { return __double_as_longlong(v); }
  static __device__ __forceinline__ U absk(double v) {
    const U b = (U)bits(v) & kAbs;
    return b > kInf ? 0ull : b;
  }
  // order key of a signed value; NaN maps below every number
  static __device__ __forceinline__ U key(double v) {
    const U b = (U)bits(v);
    if ((b & kAbs) > kInf) return 0ull;
    return (b & kSign) ? ~b : (b | kSign);
  }
  static __device__ __forceinline__ U key_neg(double v) { return key(__longlong_as_double((I)((U)bits(v) ^ kSign))); }
  static __device__ __forceinline__ double from_absk(U k) { return __longlong_as_double((I)k); }
  static __device__ __forceinline__ double from_key(U k) { return __longlong_as_double((I)((k & kSign) ? (k & kAbs) : ~k)); }
  // v > p / v < p for p > 0 given pb = bits(p); the same for -v
  static __device__ __forceinline__ bool gt(double v, I pb) { return bits(v) > pb; }
  static __device__ __forceinline__ bool lt(double v, I pb) { return bits(v) < pb; }
  static __device__ __forceinline__ bool neg_gt(double v, I pb) { return (I)((U)bits(v) ^ kSign) > pb; }
  static __device__ __forceinline__ bool neg_lt(double v, I pb) { return (I)((U)bits(v) ^ kSign) < pb; }
  // |v| < p for p > 0
  static __device__ __forceinline__ bool abs_lt(double v, I pb) { return (I)((U)bits(v) & kAbs) < pb; }
  // max(v, 0) and min(v, 0) as `v > 0 ? v : 0` and `v < 0 ? v : 0`
  static __device__ __forceinline__ double pos(double v) { return bits(v) > 0 ? v : 0.0; }
  static __device__ __forceinline__ double neg(double v) { return (bits(v) < 0 && ((U)bits(v) << 1) != 0) ? v : 0.0; }
  // thresholds: bits of p for `v > p` and for `v < p` (p is a double)
  static __device__ __forceinline__ I thr_gt(double p) { return bits(p); }
  static __device__ __forceinline__ I thr_lt(double p) { return bits(p); }
};
template <> struct FKey<float> {
  typedef unsigned U;
  typedef int I;
  static constexpr U kAbs = 0x7fffffffu, kInf = 0x7f800000u, kSign = 0x80000000u;
  static __device__ __forceinline__ I bits(float v) { return __float_as_int(v); }
  static __device__ __forceinline__ U absk(float v) {
    const U b = (U)bits(v) & kAbs;
    return b > kInf ? 0u : b;
  }
  static __device__ __forceinline__ U key(float v) {
    const U b = (U)bits(v);
    if ((b & kAbs) > kInf) return 0u;
    return (b & kSign) ? ~b : (b | kSign);
  }
  static __device__ __forceinline__ U key_neg(float v) { return key(__int_as_float((I)((U)bits(v) ^ kSign))); }
  static __device__ __forceinline__ float from_absk(U k) { return __int_as_float((I)k); }
  static __device__ __forceinline__ float from_key(U k) { return __int_as_float((I)((k & kSign) ? (k & kAbs) : ~k)); }
  static __device__ __forceinline__ bool gt(float v, I pb) { return bits(v) > pb; }
  static __device__ __forceinline__ bool lt(float v, I pb) { return bits(v) < pb; }
  static __device__ __forceinline__ bool neg_gt(float v, I pb) { return (I)((U)bits(v) ^ kSign) > pb; }
  static __device__ __forceinline__ bool neg_lt(float v, I pb) { return (I)((U)bits(v) ^ kSign) < pb; }
  static __device__ __forceinline__ bool abs_lt(float v, I pb) { return (I)((U)bits(v) & kAbs) < pb; }
  static __device__ __forceinline__ float pos(float v) { return bits(v) > 0 ? v : 0.f; }
  static __device__ __forceinline__ float neg(float v) { return (bits(v) < 0 && ((U)bits(v) << 1) != 0) ? v : 0.f; }
  // a float v exceeds the double p iff it exceeds the largest float <= p, and
  // is below p iff it is below the smallest float >= p
  static __device__ __forceinline__ I thr_gt(double p) { return bits(__double2float_rd(p)); }
  static __device__ __forceinline__ I thr_lt(double p) { return bits(__double2float_ru(p)); }
};
template <typename U> __device__ __forceinline__ U umaxk(U a, U b) { return a > b ? a : b; }
template <typename U> __device__ __forceinline__ U warp_umax(U v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = umaxk(v, (U)__shfl_xor_sync(0xffffffffu, v, o));
  return v;
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
constexpr int kMaxRanks = 16;   // CTAs per cluster

struct GroupShared {
  // per-warp partials, one 64-bit word each in the iterate type's own bits
  // (acc_pack / max_pack: no FP64 conversion on the way)
  double wsum[32][kMaxSum];
  double wmax[32][kMaxMax];
  double rsum[kMaxSum];
  double rmax[kMaxMax];
  int flag;
  int parity;   // which half of the double-buffered partials the next reduction uses
  // cluster form: every CTA's per-CTA partials, pushed by their owners
  // (sum slots packed as one 64-bit word, then max slots)
  double recv[2][kMaxRanks][kMaxSum + kMaxMax];
  int cidx;                    // cluster form: work item broadcast by rank 0
  // scalars computed once per reduction by one thread and broadcast
  double bd[4];    // FP64 state
  double bdT[4];   // values of the iterate type (FP64 build)
  float bf[4];     // values of the iterate type (FP32 build)
  int bi[4];
  // one-barrier CTA reductions (reduce1): per-warp (hi, lo, max), double-buffered
  float r1[2][32][3];
};

// Broadcast slots of the iterate type T.
template <typename T> __device__ __forceinline__ T* bcast_slots(GroupShared* sh);
template <> __device__ __forceinline__ float* bcast_slots<float>(GroupShared* sh) { return sh->bf; }
template <> __device__ __forceinline__ double* bcast_slots<double>(GroupShared* sh) { return sh->bdT; }

// Reduction callback placeholder: no scalar follow-up.
struct NoFn {
  __device__ void operator()(const double*, const double*) const {}
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

// The part of a problem's index spaces a CTA works on: rows / entries
// [nlo, nhi) of the n-space (x, P, A') and [mlo, mhi) of the m-space (z, A).
// The defaults cover everything; a sliced cluster narrows them per CTA.
struct Spans {
  int nlo = 0, nhi = 0x7fffffff, mlo = 0, mhi = 0x7fffffff;
};
struct Rng { int lo, hi; };

// A sum slot packed into one 64-bit word (FP32 build: the two floats).
template <typename T> __device__ __forceinline__ double acc_pack(const Acc<T>& a);
template <> __device__ __forceinline__ double acc_pack<float>(const Acc<float>& a) {
  return __hiloint2double(__float_as_int(a.hi), __float_as_int(a.lo));
}
template <> __device__ __forceinline__ double acc_pack<double>(const Acc<double>& a) { return a.v; }
template <typename T> __device__ __forceinline__ Acc<T> acc_unpack(double w);
template <> __device__ __forceinline__ Acc<float> acc_unpack<float>(double w) {
  Acc<float> a; a.hi = __int_as_float(__double2hiint(w)); a.lo = __int_as_float(__double2loint(w)); return a;
}
template <> __device__ __forceinline__ Acc<double> acc_unpack<double>(double w) { Acc<double> a; a.v = w; return a; }
template <typename T> __device__ __forceinline__ double max_pack(T v);
template <> __device__ __forceinline__ double max_pack<float>(float v) { return __hiloint2double(0, __float_as_int(v)); }
template <> __device__ __forceinline__ double max_pack<double>(double v) { return v; }
template <typename T> __device__ __forceinline__ T max_unpack(double w);
template <> __device__ __forceinline__ float max_unpack<float>(double w) { return __int_as_float(__double2loint(w)); }
template <> __device__ __forceinline__ double max_unpack<double>(double w) { return w; }

// Slot `slot` of the per-warp partials reduced across the CTA's warps by the
// calling warp (lane k holds warp k's partial; fixed shuffle order).  Sum
// slots (slot < NS) return the packed Acc, max slots the maximum.
template <typename T, int NS>
__device__ __forceinline__ double cta_slot(GroupShared* sh, int slot) {
  const int lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  if (slot < NS) {
    Acc<T> a;
    if (lane < nw) a = acc_unpack<T>(sh->wsum[lane][slot]);
    warp_accT(a);
    return acc_pack<T>(a);
  }
  T a = lane < nw ? max_unpack<T>(sh->wmax[lane][slot - NS]) : T(-INFINITY);
  return max_pack<T>(warp_maxT(a));
}

// Per-warp partials of a CTA -> per-CTA values: sum slot i is reduced by
// warp i (lane k holds warp k's partial; fixed shuffle order), max slots by
// the following warps.  Sums go out as (hi, lo) pairs when sum2 is set, else
// as FP64 values in sumv.  At most 32 warps.
template <typename T, int NS, int NM>
__device__ __forceinline__ void cta_finish(GroupShared* sh, double (*sum2)[2], double* sumv, double* maxv) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int slot = w; slot < NS + NM; slot += nw) {
    if (slot < NS) {
      Acc<T> a;
      if (lane < nw) a = acc_unpack<T>(sh->wsum[lane][slot]);
      warp_accT(a);
      if (lane == 0) {
        if (sum2) acc_store(sum2[slot], a);
        else sumv[slot] = a.value();
      }
    } else {
      const int i = slot - NS;
      T a = lane < nw ? max_unpack<T>(sh->wmax[lane][i]) : T(-INFINITY);
      a = warp_maxT(a);
      if (lane == 0) maxv[i] = (double)a;
    }
  }
}

// One CTA cooperates on one problem.
struct BlockGroup {
  GroupShared* sh;
  Spans sp;
  __device__ int nthreads() const { return blockDim.x; }
  __device__ int tid() const { return threadIdx.x; }
  __device__ int nwarps() const { return blockDim.x >> 5; }
  __device__ int warp() const { return threadIdx.x >> 5; }
  // span iteration: first thread / warp and stride
  __device__ int t0() const { return threadIdx.x; }
  __device__ int ts() const { return blockDim.x; }
  __device__ int w0() const { return threadIdx.x >> 5; }
  __device__ int ws() const { return blockDim.x >> 5; }
  template <typename T> __device__ void put(T* v, int i, T val) const { v[i] = val; }
  __device__ bool sync() { __syncthreads(); return true; }
  __device__ bool ok() const { return true; }

  // One sum (double-float) and one maximum of the FP32 build across the CTA
  // with a single barrier: every warp finishes the reduction itself from the
  // per-warp partials (lane k reads warp k's; the same shuffle order in every
  // warp, so every thread obtains the same bits).  The partials are
  // double-buffered by `par` (flipped per call by every thread): a warp
  // writing the next reduction's partials cannot overwrite ones a slower warp
  // is still reading.
  __device__ void reduce1(Acc<float>& s, float& m, int& par) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    warp_accT(s);
    m = warp_maxT(m);
    if (lane == 0) { sh->r1[par][w][0] = s.hi; sh->r1[par][w][1] = s.lo; sh->r1[par][w][2] = m; }
    __syncthreads();
    Acc<float> a;
    float mm = 0.f;
    if (lane < nw) { a.hi = sh->r1[par][lane][0]; a.lo = sh->r1[par][lane][1]; mm = sh->r1[par][lane][2]; }
    warp_accT(a);
    s = a;
    m = warp_maxT(mm);
    par ^= 1;
  }

  // Reduce NS sums and NM maxima across the CTA; every thread receives the
  // FP64 results in rs / rm.  fn(rsum, rmax), if given, runs once (thread 0)
  // on the results before they are published, for scalar follow-up math
  // whose outputs go to shared memory (bd / bf / bi).
  // reduce_w: the same with maxima already reduced across each warp (every
  // lane holds its warp's maximum)
  template <typename T, int NS, int NM>
  __device__ void reduce_w(Acc<T> (&s)[NS], T (&m)[NM], double (&rs)[NS], double (&rm)[NM]) {
    reduce<T, NS, NM, NoFn, true>(s, m, rs, rm, NoFn());
  }
  template <typename T, int NS, int NM, typename FN = NoFn, bool WD = false>
  __device__ void reduce(Acc<T> (&s)[NS], T (&m)[NM], double (&rs)[NS], double (&rm)[NM], FN fn = FN()) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int i = 0; i < NS; i++) { warp_accT(s[i]); if (lane == 0) sh->wsum[w][i] = acc_pack<T>(s[i]); }
#pragma unroll
    for (int i = 0; i < NM; i++) { T v = WD ? m[i] : warp_maxT(m[i]); if (lane == 0) sh->wmax[w][i] = max_pack<T>(v); }
    __syncthreads();
    if constexpr (NS + NM <= 4) {
      // small reductions: warp 0 finishes every slot, lane 0 runs fn
      if (w == 0) {
#pragma unroll
        for (int slot = 0; slot < NS + NM; slot++) {
          const double v = cta_slot<T, NS>(sh, slot);
          if (lane == 0) {
            if (slot < NS) sh->rsum[slot] = acc_unpack<T>(v).value();
            else sh->rmax[slot - NS] = (double)max_unpack<T>(v);
          }
        }
        if (lane == 0) fn(sh->rsum, sh->rmax);
      }
    } else {
      cta_finish<T, NS, NM>(sh, nullptr, sh->rsum, sh->rmax);
      if constexpr (!std::is_same<FN, NoFn>::value) {
        __syncthreads();
        if (threadIdx.x == 0) fn(sh->rsum, sh->rmax);
      }
    }
    __syncthreads();
    // rsum / rmax / bd / bf / bi are rewritten only after the next
    // reduction's first barrier, which every thread reaches after reading them.
#pragma unroll
    for (int i = 0; i < NS; i++) rs[i] = sh->rsum[i];
#pragma unroll
    for (int i = 0; i < NM; i++) rm[i] = sh->rmax[i];
  }
};


// The CTAs of one thread-block cluster cooperate on one problem: barriers are
// the hardware cluster barrier (no spinning), and each CTA reads the other
// CTAs' partial reductions straight from their shared memory (DSMEM) in rank
// order, so every CTA obtains identical results.
struct ClusterGroup {
  GroupShared* sh;
  unsigned rank, size;
  Spans sp;
  bool sliced = false;   // spans are this CTA's own contiguous slices
  bool repl = false;     // put() writes every CTA's copy (replicated shared-memory vectors)
  __device__ int nthreads() const { return blockDim.x * size; }
  __device__ int tid() const { return rank * blockDim.x + threadIdx.x; }
  __device__ int nwarps() const { return (blockDim.x >> 5) * size; }
  __device__ int warp() const { return rank * (blockDim.x >> 5) + (threadIdx.x >> 5); }
  __device__ int t0() const { return sliced ? (int)threadIdx.x : tid(); }
  __device__ int ts() const { return sliced ? (int)blockDim.x : nthreads(); }
  __device__ int w0() const { return sliced ? (int)(threadIdx.x >> 5) : warp(); }
  __device__ int ws() const { return sliced ? (int)(blockDim.x >> 5) : nwarps(); }
  // Store v[i] = val; with replicated vectors every CTA of the cluster holds
  // a copy of v at the same shared-memory offset, and all copies are written.
  template <typename T> __device__ void put(T* v, int i, T val) const {
    if (!repl) { v[i] = val; return; }
    namespace cgr = cooperative_groups;
    cgr::cluster_group cl = cgr::this_cluster();
    for (unsigned r = 0; r < size; r++) *cl.map_shared_rank(v + i, r) = val;
  }
  __device__ bool sync() { cooperative_groups::this_cluster().sync(); return true; }
  __device__ bool ok() const { return true; }

  // Cluster reduction: each CTA reduces its warps (warp 0), pushes its
  // per-CTA partials into every CTA's `recv` (DSMEM stores), then after one
  // cluster barrier every CTA merges the ranks' partials in rank order from
  // its own shared memory, so all CTAs obtain identical values.
  // reduce_w: the same with maxima already reduced across each warp (every
  // lane holds its warp's maximum)
  template <typename T, int NS, int NM>
  __device__ void reduce_w(Acc<T> (&s)[NS], T (&m)[NM], double (&rs)[NS], double (&rm)[NM]) {
    reduce<T, NS, NM, NoFn, true>(s, m, rs, rm, NoFn());
  }
  template <typename T, int NS, int NM, typename FN = NoFn, bool WD = false>
  __device__ void reduce(Acc<T> (&s)[NS], T (&m)[NM], double (&rs)[NS], double (&rm)[NM], FN fn = FN()) {
    namespace cgr = cooperative_groups;
    cgr::cluster_group cl = cgr::this_cluster();
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    constexpr int NSL = NS + NM;
#pragma unroll
    for (int i = 0; i < NS; i++) { warp_accT(s[i]); if (lane == 0) sh->wsum[w][i] = acc_pack<T>(s[i]); }
#pragma unroll
    for (int i = 0; i < NM; i++) { T v = WD ? m[i] : warp_maxT(m[i]); if (lane == 0) sh->wmax[w][i] = max_pack<T>(v); }
    __syncthreads();
    const int par = sh->parity;
    if (w == 0) {
      // every lane ends with each slot's value (xor-butterfly reductions)
#pragma unroll
      for (int slot = 0; slot < NSL; slot++) {
        const double v = cta_slot<T, NS>(sh, slot);
        if (lane == slot) sh->recv[par][rank][slot] = v;
      }
      __syncwarp();
      // push this CTA's partials to the other ranks: lane handles (slot, rank) pairs
      for (int q = lane; q < NSL * (int)size; q += 32) {
        const int slot = q % NSL, r = q / NSL;
        if (r != (int)rank) *cl.map_shared_rank(&sh->recv[par][rank][slot], (unsigned)r) = sh->recv[par][rank][slot];
      }
    }
    cl.sync();
    if (w == 0) {
      if (lane < NS) {
        Acc<T> a;
        for (unsigned r = 0; r < size; r++) a.merge(acc_unpack<T>(sh->recv[par][r][lane]));
        sh->rsum[lane] = a.value();
      } else if (lane < NSL) {
        T a = T(-INFINITY);
        for (unsigned r = 0; r < size; r++) a = tmaxT(a, max_unpack<T>(sh->recv[par][r][lane]));
        sh->rmax[lane - NS] = (double)a;
      }
      __syncwarp();
      if (lane == 0) fn(sh->rsum, sh->rmax);
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < NS; i++) rs[i] = sh->rsum[i];
#pragma unroll
    for (int i = 0; i < NM; i++) rm[i] = sh->rmax[i];
    // The other half of recv is written by the next reduction; no CTA can
    // overwrite this half before every CTA has passed the next cluster
    // barrier.  rsum / rmax are rewritten only after the next reduction's
    // first block barrier, which every thread reaches after reading them.
    if (threadIdx.x == 0) sh->parity ^= 1;
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
  Spans sp;
  __device__ int nthreads() const { return blockDim.x * gridDim.x; }
  __device__ int tid() const { return blockIdx.x * blockDim.x + threadIdx.x; }
  __device__ int nwarps() const { return (blockDim.x >> 5) * gridDim.x; }
  __device__ int warp() const { return blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); }
  __device__ int t0() const { return tid(); }
  __device__ int ts() const { return nthreads(); }
  __device__ int w0() const { return warp(); }
  __device__ int ws() const { return nwarps(); }
  template <typename T> __device__ void put(T* v, int i, T val) const { v[i] = val; }

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

  // reduce_w: the same with maxima already reduced across each warp (every
  // lane holds its warp's maximum)
  template <typename T, int NS, int NM>
  __device__ void reduce_w(Acc<T> (&s)[NS], T (&m)[NM], double (&rs)[NS], double (&rm)[NM]) {
    reduce<T, NS, NM, NoFn, true>(s, m, rs, rm, NoFn());
  }
  template <typename T, int NS, int NM, typename FN = NoFn, bool WD = false>
  __device__ void reduce(Acc<T> (&s)[NS], T (&m)[NM], double (&rs)[NS], double (&rm)[NM], FN fn = FN()) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int i = 0; i < NS; i++) { warp_accT(s[i]); if (lane == 0) sh->wsum[w][i] = acc_pack<T>(s[i]); }
#pragma unroll
    for (int i = 0; i < NM; i++) { T v = WD ? m[i] : warp_maxT(m[i]); if (lane == 0) sh->wmax[w][i] = max_pack<T>(v); }
    __syncthreads();
    const int nw = blockDim.x >> 5, nb = gridDim.x;
    const int par = sh->parity;
    double* ps = gs.partial_sum + (size_t)par * kMaxSum * 2 * nb;   // [slot][block][2]
    double* pm = gs.partial_max + (size_t)par * kMaxMax * nb;       // [slot][block]
    if (threadIdx.x < NS) {
      Acc<T> a;
      for (int k = 0; k < nw; k++) a.merge(acc_unpack<T>(sh->wsum[k][threadIdx.x]));
      acc_store(ps + ((size_t)threadIdx.x * nb + blockIdx.x) * 2, a);
    } else if (threadIdx.x >= 32 && threadIdx.x < 32 + NM) {
      const int i = threadIdx.x - 32;
      T at = max_unpack<T>(sh->wmax[0][i]);
      for (int k = 1; k < nw; k++) at = tmaxT(at, max_unpack<T>(sh->wmax[k][i]));
      const double a = (double)at;
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
    if constexpr (!std::is_same<FN, NoFn>::value) {
      __syncthreads();
      if (threadIdx.x == 0) fn(sh->rsum, sh->rmax);
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
  // optional on-chip copy of the entries of rows [.., srow): scol / sval are
  // addressed by the same positions as col / val (the sparse-product loops
  // read them for rows below srow; everything else may keep reading col / val,
  // which hold the same values)
  const int* scol = nullptr;
  T* sval = nullptr;
  int srow = 0;
  // every row holds exactly one entry, on the diagonal (a diagonal P): the
  // product is one multiply per row, no sparse dot
  int diag = 0;
};


// Dot product of one CSR row segment handled by a sub-warp lane: entries
// b+sl, b+sl+L, ... < e.  Four entries are fetched per round before any is
// used, so each lane keeps four index/value loads and four gathers in flight.
// Entries per lane loaded before any is used: the index/value loads of a
// chunk are independent, so a row costs ceil(len / (kRowUnroll * L)) memory
// latencies.  The summation order (k ascending per lane) does not depend on
// it.  Measured on batched MPC (one box, alternating builds), with
// kRowsInFlight rows per lane group: (rows, unroll) = (2, 1) 523, (2, 2) 505,
// (4, 1) 491, (4, 2) 395, (2, 4) 426, (2, 8) 270 solves/s; short rows waste
// the predicated slots of a long unroll, and the kernel is issue-limited.
constexpr int kRowUnroll = 1;

template <int L, typename T, typename XF>
__device__ __forceinline__ T lane_row_dot(const int* __restrict__ col, const T* __restrict__ val,
                                          int b, int e, int sl, XF xf) {
  T acc = T(0);
  for (int k0 = b + sl; k0 < e; k0 += kRowUnroll * L) {
    int c[kRowUnroll];
    T v[kRowUnroll];
#pragma unroll
    for (int u = 0; u < kRowUnroll; u++) {
      const int k = k0 + u * L;
      c[u] = k < e ? col[k] : -1;
      v[u] = k < e ? val[k] : T(0);
    }
    T x[kRowUnroll];
#pragma unroll
    for (int u = 0; u < kRowUnroll; u++) x[u] = c[u] >= 0 ? xf(c[u]) : T(0);
#pragma unroll
    for (int u = 0; u < kRowUnroll; u++) acc += v[u] * x[u];
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
inline int pick_lanes(long long nnz, int rows, int per_lane = 4) {
  if (rows <= 0) return 1;
  const double mean = (double)nnz / rows;
  int L = 1;
  while (L < 32 && L * per_lane < mean) L <<= 1;
  return L;
}

// ---- loops over the CTA's part of a problem's index spaces (Spans) ----
template <typename G>
__device__ __forceinline__ Rng span_n(const G& g, int n) { return Rng{g.sp.nlo, n < g.sp.nhi ? n : g.sp.nhi}; }
template <typename G>
__device__ __forceinline__ Rng span_m(const G& g, int m) { return Rng{g.sp.mlo, m < g.sp.mhi ? m : g.sp.mhi}; }

template <typename G, typename FN>
__device__ __forceinline__ void for_rng(G& g, Rng r, FN fn) {
  for (int i = r.lo + g.t0(); i < r.hi; i += g.ts()) fn(i);
}
template <typename G, typename FN>
__device__ __forceinline__ void for_n(G& g, int n, FN fn) { for_rng(g, span_n(g, n), fn); }
template <typename G, typename FN>
__device__ __forceinline__ void for_m(G& g, int m, FN fn) { for_rng(g, span_m(g, m), fn); }

// Rows [rg.lo, rg.hi) of M, sub-warp per row (as rows_apply_L).
// Rows in flight per lane group: the chunk loads of all of them are issued
// before any is used, so a warp has kRowsInFlight times the memory requests
// in flight.  Each row's entries are still summed by the same lane in the
// same order.
constexpr int kRowsInFlight = 2;

template <int L, int NR, int U = kRowUnroll, typename T, typename XF>
__device__ __forceinline__ void lane_rows_dot(const int* const (&col)[NR], const T* const (&val)[NR],
                                              const int (&b)[NR], const int (&e)[NR], int sl, XF xf,
                                              T (&acc)[NR]) {
  int k[NR];
  bool more = false;
#pragma unroll
  for (int r = 0; r < NR; r++) { k[r] = b[r] + sl; more |= k[r] < e[r]; }
  while (more) {
    int c[NR][U];
    T v[NR][U];
#pragma unroll
    for (int r = 0; r < NR; r++)
#pragma unroll
      for (int u = 0; u < U; u++) {
        const int kk = k[r] + u * L;
        c[r][u] = kk < e[r] ? col[r][kk] : -1;
        v[r][u] = kk < e[r] ? val[r][kk] : T(0);
      }
    T x[NR][U];
#pragma unroll
    for (int r = 0; r < NR; r++)
#pragma unroll
      for (int u = 0; u < U; u++) x[r][u] = c[r][u] >= 0 ? xf(c[r][u]) : T(0);
    more = false;
#pragma unroll
    for (int r = 0; r < NR; r++) {
#pragma unroll
      for (int u = 0; u < U; u++) acc[r] += v[r][u] * x[r][u];
      k[r] += U * L;
      more |= k[r] < e[r];
    }
  }
}

// Row r's entry pointers: the on-chip copy below M.srow, else HBM.  (The
// row loops take their CSR descriptor by value: a descriptor inside a larger
// struct in memory would be reloaded after every store through the generic
// vector pointers, which could alias it.)
template <typename T>
__device__ __forceinline__ void row_ptrs(const CSR<T>& M, int r, bool valid, const int*& col, const T*& val,
                                         int& b, int& e) {
  const bool s = r < M.srow;
  col = s ? M.scol : M.col;
  val = s ? M.sval : M.val;
  b = valid ? M.rowptr[r] : 0;
  e = valid ? M.rowptr[r + 1] : 0;
}

template <int L, typename T, typename G, typename XF, typename FN>
__device__ __forceinline__ void rows_rng_L(G& g, Rng rg, const CSR<T> M, XF xf, FN fn) {
  constexpr int NR = kRowsInFlight;
  const int lane = threadIdx.x & 31;
  const int sub = lane / L, sl = lane % L;
  constexpr int RPW = 32 / L;
  const int step = g.ws() * RPW;
  for (int base = rg.lo + g.w0() * RPW; base < rg.hi; base += NR * step) {
    const int* col[NR];
    const T* val[NR];
    int b[NR], e[NR];
    T acc[NR];
#pragma unroll
    for (int r = 0; r < NR; r++) {
      row_ptrs(M, base + r * step + sub, base + r * step + sub < rg.hi, col[r], val[r], b[r], e[r]);
      acc[r] = T(0);
    }
    lane_rows_dot<L, NR>(col, val, b, e, sl, xf, acc);
#pragma unroll
    for (int r = 0; r < NR; r++) {
      const T a = subwarp_sum<L>(acc[r]);
      const int row = base + r * step + sub;
      if (row < rg.hi && sl == 0) fn(row, a);
    }
  }
}
template <typename T, typename G, typename XF, typename FN>
__device__ __forceinline__ void rows_rng(G& g, Rng rg, const CSR<T>& M, XF xf, FN fn) {
  switch (M.lanes) {
    case 1:  rows_rng_L<1>(g, rg, M, xf, fn); break;
    case 2:  rows_rng_L<2>(g, rg, M, xf, fn); break;
    case 4:  rows_rng_L<4>(g, rg, M, xf, fn); break;
    case 8:  rows_rng_L<8>(g, rg, M, xf, fn); break;
    case 16: rows_rng_L<16>(g, rg, M, xf, fn); break;
    default: rows_rng_L<32>(g, rg, M, xf, fn); break;
  }
}
template <int L, typename T, typename G, typename XF1, typename XF2, typename FN>
__device__ __forceinline__ void rows_rng2_L(G& g, Rng rg, const CSR<T> M, XF1 xf1, XF2 xf2, FN fn) {
  const int lane = threadIdx.x & 31;
  const int sub = lane / L, sl = lane % L;
  constexpr int RPW = 32 / L;
  const int ws = g.ws();
  for (int base = rg.lo + g.w0() * RPW; base < rg.hi; base += ws * RPW) {
    const int r = base + sub;
    T a1 = T(0), a2 = T(0);
    if (r < rg.hi) lane_row_dot2<L>(M.col, M.val, M.rowptr[r], M.rowptr[r + 1], sl, xf1, xf2, a1, a2);
    a1 = subwarp_sum<L>(a1);
    a2 = subwarp_sum<L>(a2);
    if (r < rg.hi && sl == 0) fn(r, a1, a2);
  }
}
template <typename T, typename G, typename XF1, typename XF2, typename FN>
__device__ __forceinline__ void rows_rng2(G& g, Rng rg, const CSR<T>& M, XF1 a, XF2 b, FN fn) {
  switch (M.lanes) {
    case 1:  rows_rng2_L<1>(g, rg, M, a, b, fn); break;
    case 2:  rows_rng2_L<2>(g, rg, M, a, b, fn); break;
    case 4:  rows_rng2_L<4>(g, rg, M, a, b, fn); break;
    case 8:  rows_rng2_L<8>(g, rg, M, a, b, fn); break;
    case 16: rows_rng2_L<16>(g, rg, M, a, b, fn); break;
    default: rows_rng2_L<32>(g, rg, M, a, b, fn); break;
  }
}

// ---- dense row batches: one row per lane for the follow-up work ----
//
// Rows [rg.lo, rg.hi) of M in batches of 32 consecutive rows per warp.  Each
// sub-warp of L lanes sums one row's entries exactly as rows_rng_L does (lane
// sl takes entries b+sl, b+sl+L, ... in order, then subwarp_sum), NR rows in
// flight per lane; the batch's 32 sums then move by shuffles so that lane t
// holds row base + t, and fn(row, value) runs on every lane that has a row.
// Element-wise follow-up work so issues one warp instruction per 32 rows
// instead of one per 32 / L rows, which matters for FP64 work on GB300 (an
// FP64 warp instruction costs the same whatever the number of active lanes).

// Two products of NR rows per lane (shared index and value loads), entries
// summed per lane in ascending order as lane_row_dot2.
template <int L, int NR, int U = 1, typename T, typename XF1, typename XF2>
__device__ __forceinline__ void lane_rows_dot2(const int* const (&col)[NR], const T* const (&val)[NR],
                                               const int (&b)[NR], const int (&e)[NR], int sl, XF1 xf1, XF2 xf2,
                                               T (&a1)[NR], T (&a2)[NR]) {
  int k[NR];
  bool more = false;
#pragma unroll
  for (int r = 0; r < NR; r++) { k[r] = b[r] + sl; more |= k[r] < e[r]; }
  while (more) {
    int c[NR][U];
    T v[NR][U];
#pragma unroll
    for (int r = 0; r < NR; r++)
#pragma unroll
      for (int u = 0; u < U; u++) {
        const int kk = k[r] + u * L;
        c[r][u] = kk < e[r] ? col[r][kk] : -1;
        v[r][u] = kk < e[r] ? val[r][kk] : T(0);
      }
    more = false;
#pragma unroll
    for (int r = 0; r < NR; r++) {
#pragma unroll
      for (int u = 0; u < U; u++) {
        const T x1 = c[r][u] >= 0 ? xf1(c[r][u]) : T(0);
        const T x2 = c[r][u] >= 0 ? xf2(c[r][u]) : T(0);
        a1[r] += v[r][u] * x1;
        a2[r] += v[r][u] * x2;
      }
      k[r] += U * L;
      more |= k[r] < e[r];
    }
  }
}

// Entries per lane loaded before any is used in the dense row batches: one
// product (rows_dense) takes four, two products (rows_dense2 / _pair) one.
// Measured on 4096 batched MPC QPs, FP64 direct solver (one box): four in
// both forms gave the single products -11 % / -16 % cycles and the
// termination's pairs +13 %.
constexpr int kDenseUnroll = 4;
constexpr int kDenseUnroll2 = 1;

template <int L>
struct DenseRows {
  static constexpr int RPW = 32 / L;            // rows per sub-iteration
  static constexpr int NR = L < 2 ? L : 2;      // rows in flight per lane
  // shuffle source lane and sub-iteration of this lane's row
  static __device__ __forceinline__ int src(int lane) { return (lane % RPW) * L; }
  static __device__ __forceinline__ int mine(int lane) { return lane / RPW; }
};

template <int L, typename T, typename G, typename XF, typename FN>
__device__ __forceinline__ void rows_dense_L(G& g, Rng rg, const CSR<T> M, XF xf, FN fn) {
  typedef DenseRows<L> D;
  constexpr int NR = D::NR;
  const int lane = threadIdx.x & 31, sub = lane / L, sl = lane % L;
  const int src = D::src(lane), mine = D::mine(lane);
  for (int base = rg.lo + g.w0() * 32; base < rg.hi; base += g.ws() * 32) {
    T res = T(0);
#pragma unroll 1
    for (int u0 = 0; u0 < L; u0 += NR) {
      const int* col[NR];
      const T* val[NR];
      int b[NR], e[NR];
      T acc[NR];
#pragma unroll
      for (int r = 0; r < NR; r++) {
        const int row = base + (u0 + r) * D::RPW + sub;
        row_ptrs(M, row, row < rg.hi, col[r], val[r], b[r], e[r]);
        acc[r] = T(0);
      }
      lane_rows_dot<L, NR, kDenseUnroll>(col, val, b, e, sl, xf, acc);
#pragma unroll
      for (int r = 0; r < NR; r++) {
        const T a = __shfl_sync(0xffffffffu, subwarp_sum<L>(acc[r]), src);
        if (mine == u0 + r) res = a;
      }
    }
    if (base + lane < rg.hi) fn(base + lane, res);
  }
}
template <typename T, typename G, typename XF, typename FN>
__device__ __forceinline__ void rows_dense(G& g, Rng rg, const CSR<T>& M, XF xf, FN fn) {
  switch (M.lanes) {
    case 1:  rows_dense_L<1>(g, rg, M, xf, fn); break;
    case 2:  rows_dense_L<2>(g, rg, M, xf, fn); break;
    case 4:  rows_dense_L<4>(g, rg, M, xf, fn); break;
    case 8:  rows_dense_L<8>(g, rg, M, xf, fn); break;
    case 16: rows_dense_L<16>(g, rg, M, xf, fn); break;
    default: rows_dense_L<32>(g, rg, M, xf, fn); break;
  }
}

template <int L, typename T, typename G, typename XF1, typename XF2, typename FN>
__device__ __forceinline__ void rows_dense2_L(G& g, Rng rg, const CSR<T> M, XF1 xf1, XF2 xf2, FN fn) {
  typedef DenseRows<L> D;
  constexpr int NR = D::NR;
  const int lane = threadIdx.x & 31, sub = lane / L, sl = lane % L;
  const int src = D::src(lane), mine = D::mine(lane);
  for (int base = rg.lo + g.w0() * 32; base < rg.hi; base += g.ws() * 32) {
    T r1 = T(0), r2 = T(0);
#pragma unroll 1
    for (int u0 = 0; u0 < L; u0 += NR) {
      const int* col[NR];
      const T* val[NR];
      int b[NR], e[NR];
      T a1[NR], a2[NR];
#pragma unroll
      for (int r = 0; r < NR; r++) {
        const int row = base + (u0 + r) * D::RPW + sub;
        row_ptrs(M, row, row < rg.hi, col[r], val[r], b[r], e[r]);
        a1[r] = T(0);
        a2[r] = T(0);
      }
      lane_rows_dot2<L, NR, kDenseUnroll2>(col, val, b, e, sl, xf1, xf2, a1, a2);
#pragma unroll
      for (int r = 0; r < NR; r++) {
        const T v1 = __shfl_sync(0xffffffffu, subwarp_sum<L>(a1[r]), src);
        const T v2 = __shfl_sync(0xffffffffu, subwarp_sum<L>(a2[r]), src);
        if (mine == u0 + r) { r1 = v1; r2 = v2; }
      }
    }
    if (base + lane < rg.hi) fn(base + lane, r1, r2);
  }
}
template <typename T, typename G, typename XF1, typename XF2, typename FN>
__device__ __forceinline__ void rows_dense2(G& g, Rng rg, const CSR<T>& M, XF1 a, XF2 b, FN fn) {
  switch (M.lanes) {
    case 1:  rows_dense2_L<1>(g, rg, M, a, b, fn); break;
    case 2:  rows_dense2_L<2>(g, rg, M, a, b, fn); break;
    case 4:  rows_dense2_L<4>(g, rg, M, a, b, fn); break;
    case 8:  rows_dense2_L<8>(g, rg, M, a, b, fn); break;
    case 16: rows_dense2_L<16>(g, rg, M, a, b, fn); break;
    default: rows_dense2_L<32>(g, rg, M, a, b, fn); break;
  }
}

// Dense row batches for the FP64 build on a CTA or a cluster, where the
// follow-up work is FP64 instructions; sub-warp rows (rows_rng) for the FP32
// build (its follow-up work is cheap on the FP32 pipe) and for the grid form
// (one large QP), where sub-warp rows spread more evenly over the grid's
// warps.  fn(row, value) alike in both.
template <typename T, typename G>
constexpr bool kDenseRows = std::is_same<T, double>::value && !std::is_same<G, GridGroup>::value;
template <typename T, typename G, typename XF, typename FN>
__device__ __forceinline__ void rows_auto(G& g, Rng rg, const CSR<T>& M, XF xf, FN fn) {
  if constexpr (kDenseRows<T, G>) rows_dense(g, rg, M, xf, fn);
  else rows_rng(g, rg, M, xf, fn);
}
template <typename T, typename G, typename XF1, typename XF2, typename FN>
__device__ __forceinline__ void rows_auto2(G& g, Rng rg, const CSR<T>& M, XF1 a, XF2 b, FN fn) {
  if constexpr (kDenseRows<T, G>) rows_dense2(g, rg, M, a, b, fn);
  else rows_rng2(g, rg, M, a, b, fn);
}

// Two matrices with the same rows (P and A'), two products each:
// fn(row, M1 x1, M1 x2, M2 y1, M2 y2) with one row per lane; L lanes per row
// for both matrices.
template <int L, typename T, typename G, typename XP1, typename XP2, typename XA1, typename XA2, typename FN>
__device__ __forceinline__ void rows_dense_pair_L(G& g, Rng rg, const CSR<T> M1, const CSR<T> M2, XP1 xp1, XP2 xp2,
                                                  XA1 xa1, XA2 xa2, FN fn) {
  typedef DenseRows<L> D;
  constexpr int NR = D::NR;
  const int lane = threadIdx.x & 31, sub = lane / L, sl = lane % L;
  const int src = D::src(lane), mine = D::mine(lane);
  for (int base = rg.lo + g.w0() * 32; base < rg.hi; base += g.ws() * 32) {
    T r1 = T(0), r2 = T(0), r3 = T(0), r4 = T(0);
#pragma unroll 1
    for (int u0 = 0; u0 < L; u0 += NR) {
      const int* col[NR];
      const T* val[NR];
      int b[NR], e[NR];
      T a1[NR], a2[NR], a3[NR], a4[NR];
#pragma unroll
      for (int r = 0; r < NR; r++) {
        const int row = base + (u0 + r) * D::RPW + sub;
        row_ptrs(M1, row, row < rg.hi, col[r], val[r], b[r], e[r]);
        a1[r] = a2[r] = a3[r] = a4[r] = T(0);
      }
      lane_rows_dot2<L, NR, kDenseUnroll2>(col, val, b, e, sl, xp1, xp2, a1, a2);
#pragma unroll
      for (int r = 0; r < NR; r++) {
        const int row = base + (u0 + r) * D::RPW + sub;
        row_ptrs(M2, row, row < rg.hi, col[r], val[r], b[r], e[r]);
      }
      lane_rows_dot2<L, NR, kDenseUnroll2>(col, val, b, e, sl, xa1, xa2, a3, a4);
#pragma unroll
      for (int r = 0; r < NR; r++) {
        const T v1 = __shfl_sync(0xffffffffu, subwarp_sum<L>(a1[r]), src);
        const T v2 = __shfl_sync(0xffffffffu, subwarp_sum<L>(a2[r]), src);
        const T v3 = __shfl_sync(0xffffffffu, subwarp_sum<L>(a3[r]), src);
        const T v4 = __shfl_sync(0xffffffffu, subwarp_sum<L>(a4[r]), src);
        if (mine == u0 + r) { r1 = v1; r2 = v2; r3 = v3; r4 = v4; }
      }
    }
    if (base + lane < rg.hi) fn(base + lane, r1, r2, r3, r4);
  }
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
