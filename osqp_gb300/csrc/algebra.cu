// algebra.cu -- OSQP's algebra / linear-system ABI on GB300 device memory.
//
// Replaces the reference's algebra/cuda backend (algebra/cuda/vector.cu,
// matrix.cu, algebra_libs.cu, lin_sys/indirect/cuda_pcg*.cu) behind the same
// C declarations (include/osqp_gb300_algebra.h):
//   * vectors are device arrays; element-wise operations are single kernels;
//     every reduction runs in one launch (grid partials + last-block finish,
//     fixed order, FP64-accurate accumulation) and returns a host scalar;
//   * matrices keep the caller's CSC as the master copy (value updates and
//     diagonal scalings act on it, as the reference's CSC semantics require)
//     plus row-major views built by deterministic stable-sort transposes:
//     CSR(A) and the CSC arrays read as CSR(A'), or the full symmetric CSR of
//     an upper-triangular P with an explicit diagonal;
//   * the linear system is the reduced-KKT PCG of gb_solver.cuh: one kernel
//     launch per solve (the reference issues ~16 launches and a host
//     synchronisation per CG iteration, cuda_pcg.cu:155-199).
#include <cuda_runtime.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "osqp_gb300_algebra.h"
#include "gb_solver.cuh"
#include "gb_structure.cuh"

using T = OSQPFloat;
using namespace gb;

namespace gba {

// ---------------------------------------------------------------------------
// Library context (refcounted; the reference keeps one global handle that
// every osqp_cleanup tears down, algebra/cuda/algebra_libs.cu:29-99)
// ---------------------------------------------------------------------------
struct Context {
  int refs = 0;
  int device = 0;
  cudaStream_t stream = nullptr;
  double* d_red = nullptr;      // reduction partials + result
  unsigned* d_ticket = nullptr;
  double* h_red = nullptr;      // pinned result
};
static Context g_ctx;

constexpr int kRedBlocks = 296;
constexpr int kRedThreads = 256;
constexpr int kEwThreads = 256;

static bool ensure_ctx() {
  if (g_ctx.stream) return true;
  if (cudaSetDevice(g_ctx.device) != cudaSuccess) return false;
  if (cudaStreamCreateWithFlags(&g_ctx.stream, cudaStreamNonBlocking) != cudaSuccess) return false;
  if (cudaMalloc((void**)&g_ctx.d_red, sizeof(double) * (3 * kRedBlocks + 4)) != cudaSuccess) return false;
  if (cudaMalloc((void**)&g_ctx.d_ticket, sizeof(unsigned)) != cudaSuccess) return false;
  if (cudaMemset(g_ctx.d_ticket, 0, sizeof(unsigned)) != cudaSuccess) return false;
  if (cudaMallocHost((void**)&g_ctx.h_red, sizeof(double) * 4) != cudaSuccess) return false;
  return true;
}
static cudaStream_t stream() { ensure_ctx(); return g_ctx.stream; }
static void check(cudaError_t e, const char* what) {
  if (e != cudaSuccess) fprintf(stderr, "osqp_gb300 algebra: %s: %s\n", what, cudaGetErrorString(e));
}
static int ew_blocks(long long n) { return (int)std::min<long long>(4096, (n + kEwThreads - 1) / kEwThreads); }

template <typename F>
__global__ void k_ew(int n, F f) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) f(i);
}
template <typename F>
static void ew(int n, F f) {
  if (n <= 0) return;
  k_ew<<<ew_blocks(n), kEwThreads, 0, stream()>>>(n, f);
  check(cudaGetLastError(), "element-wise kernel");
}

// One-launch reduction: every thread folds f(i, sum, max) over its indices;
// per-block partials are combined by the last block to finish, in block order.
template <typename F>
__global__ void __launch_bounds__(kRedThreads) k_reduce(int n, F f, double* part, unsigned* ticket) {
  Acc<T> s;
  T mx = T(0);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) f(i, s, mx);
  __shared__ double sh[3][kRedThreads / 32];
  __shared__ bool last;
  warp_accT(s);
  mx = warp_maxT(mx);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) { double t2[2]; acc_store(t2, s); sh[0][w] = t2[0]; sh[1][w] = t2[1]; sh[2][w] = (double)mx; }
  __syncthreads();
  if (threadIdx.x == 0) {
    Acc<T> a;
    double m2 = 0.0;
    for (int k = 0; k < kRedThreads / 32; k++) {
      double t2[2] = {sh[0][k], sh[1][k]};
      a.merge(acc_load<T>(t2));
      m2 = fmax(m2, sh[2][k]);
    }
    double t2[2];
    acc_store(t2, a);
    part[3 * blockIdx.x] = t2[0];
    part[3 * blockIdx.x + 1] = t2[1];
    part[3 * blockIdx.x + 2] = m2;
    __threadfence();
    last = atomicAdd(ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (last && threadIdx.x == 0) {
    __threadfence();
    Acc<T> a;
    double m2 = 0.0;
    for (int b = 0; b < (int)gridDim.x; b++) {
      double t2[2] = {((volatile double*)part)[3 * b], ((volatile double*)part)[3 * b + 1]};
      a.merge(acc_load<T>(t2));
      m2 = fmax(m2, ((volatile double*)part)[3 * b + 2]);
    }
    part[3 * gridDim.x] = a.value();
    part[3 * gridDim.x + 1] = m2;
    *ticket = 0;
  }
}
struct RedOut { double sum, max; };
template <typename F>
static RedOut reduce(int n, F f) {
  RedOut r{0.0, 0.0};
  if (n <= 0 || !ensure_ctx()) return r;
  const int blocks = std::min(kRedBlocks, std::max(1, (n + kRedThreads - 1) / kRedThreads));
  k_reduce<<<blocks, kRedThreads, 0, g_ctx.stream>>>(n, f, g_ctx.d_red, g_ctx.d_ticket);
  check(cudaMemcpyAsync(g_ctx.h_red, g_ctx.d_red + 3 * blocks, sizeof(double) * 2, cudaMemcpyDeviceToHost,
                        g_ctx.stream), "reduction result");
  check(cudaStreamSynchronize(g_ctx.stream), "reduction");
  r.sum = g_ctx.h_red[0];
  r.max = g_ctx.h_red[1];
  return r;
}

// Non-cooperative group for stand-alone row kernels (no barriers needed).
struct FlatGroup {
  __device__ int nwarps() const { return (blockDim.x >> 5) * gridDim.x; }
  __device__ int warp() const { return blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); }
};

template <typename TT>
__global__ void k_spmv(CSR<TT> M, const TT* x, TT* y, TT alpha, TT beta) {
  FlatGroup g;
  rows_apply(g, M, [&](int c) { return x[c]; }, [&](int r, TT v) {
    y[r] = (beta == TT(0)) ? alpha * v : alpha * v + beta * y[r];
  });
}

}  // namespace gba

using namespace gba;

// ---------------------------------------------------------------------------
// Vectors
// ---------------------------------------------------------------------------
struct OSQPVectorf_ { T* d_val; OSQPInt length; int owner; };
struct OSQPVectori_ { OSQPInt* d_val; OSQPInt length; };

extern "C" {

OSQPVectorf* OSQPVectorf_malloc(OSQPInt length) {
  if (length < 0 || !ensure_ctx()) return NULL;
  OSQPVectorf* v = (OSQPVectorf*)calloc(1, sizeof(OSQPVectorf));
  if (!v) return NULL;
  v->length = length;
  v->owner = 1;
  if (length > 0 && cudaMalloc((void**)&v->d_val, sizeof(T) * length) != cudaSuccess) { free(v); return NULL; }
  return v;
}
OSQPVectorf* OSQPVectorf_calloc(OSQPInt length) {
  OSQPVectorf* v = OSQPVectorf_malloc(length);
  if (v && length > 0) check(cudaMemsetAsync(v->d_val, 0, sizeof(T) * length, stream()), "calloc");
  return v;
}
OSQPVectori* OSQPVectori_malloc(OSQPInt length) {
  if (length < 0 || !ensure_ctx()) return NULL;
  OSQPVectori* v = (OSQPVectori*)calloc(1, sizeof(OSQPVectori));
  if (!v) return NULL;
  v->length = length;
  if (length > 0 && cudaMalloc((void**)&v->d_val, sizeof(OSQPInt) * length) != cudaSuccess) { free(v); return NULL; }
  return v;
}
OSQPVectori* OSQPVectori_calloc(OSQPInt length) {
  OSQPVectori* v = OSQPVectori_malloc(length);
  if (v && length > 0) check(cudaMemsetAsync(v->d_val, 0, sizeof(OSQPInt) * length, stream()), "calloc");
  return v;
}
void OSQPVectorf_from_raw(OSQPVectorf* b, const OSQPFloat* a) {
  if (!b || !a || b->length <= 0) return;
  check(cudaMemcpyAsync(b->d_val, a, sizeof(T) * b->length, cudaMemcpyDefault, stream()), "from_raw");
  check(cudaStreamSynchronize(stream()), "from_raw");
}
void OSQPVectori_from_raw(OSQPVectori* b, const OSQPInt* a) {
  if (!b || !a || b->length <= 0) return;
  check(cudaMemcpyAsync(b->d_val, a, sizeof(OSQPInt) * b->length, cudaMemcpyDefault, stream()), "from_raw");
  check(cudaStreamSynchronize(stream()), "from_raw");
}
void OSQPVectorf_to_raw(OSQPFloat* bv, const OSQPVectorf* a) {
  if (!bv || !a || a->length <= 0) return;
  check(cudaMemcpyAsync(bv, a->d_val, sizeof(T) * a->length, cudaMemcpyDefault, stream()), "to_raw");
  check(cudaStreamSynchronize(stream()), "to_raw");
}
void OSQPVectori_to_raw(OSQPInt* bv, const OSQPVectori* a) {
  if (!bv || !a || a->length <= 0) return;
  check(cudaMemcpyAsync(bv, a->d_val, sizeof(OSQPInt) * a->length, cudaMemcpyDefault, stream()), "to_raw");
  check(cudaStreamSynchronize(stream()), "to_raw");
}
OSQPVectorf* OSQPVectorf_new(const OSQPFloat* a, OSQPInt length) {
  OSQPVectorf* v = OSQPVectorf_malloc(length);
  if (v) OSQPVectorf_from_raw(v, a);
  return v;
}
OSQPVectori* OSQPVectori_new(const OSQPInt* a, OSQPInt length) {
  OSQPVectori* v = OSQPVectori_malloc(length);
  if (v) OSQPVectori_from_raw(v, a);
  return v;
}
void OSQPVectorf_copy(OSQPVectorf* b, const OSQPVectorf* a) {
  if (!a || !b || a->length <= 0) return;
  check(cudaMemcpyAsync(b->d_val, a->d_val, sizeof(T) * a->length, cudaMemcpyDeviceToDevice, stream()), "copy");
}
OSQPVectorf* OSQPVectorf_copy_new(const OSQPVectorf* a) {
  OSQPVectorf* v = OSQPVectorf_malloc(a->length);
  if (v) OSQPVectorf_copy(v, a);
  return v;
}
void OSQPVectorf_free(OSQPVectorf* a) {
  if (!a) return;
  if (a->owner && a->d_val) cudaFree(a->d_val);
  free(a);
}
void OSQPVectori_free(OSQPVectori* a) {
  if (!a) return;
  if (a->d_val) cudaFree(a->d_val);
  free(a);
}
OSQPVectorf* OSQPVectorf_view(const OSQPVectorf* a, OSQPInt head, OSQPInt length) {
  OSQPVectorf* v = (OSQPVectorf*)calloc(1, sizeof(OSQPVectorf));
  if (v) OSQPVectorf_view_update(v, a, head, length);
  return v;
}
void OSQPVectorf_view_update(OSQPVectorf* a, const OSQPVectorf* b, OSQPInt head, OSQPInt length) {
  a->length = length;
  a->d_val = b->d_val ? b->d_val + head : NULL;
  a->owner = 0;
}
void OSQPVectorf_view_free(OSQPVectorf* a) { free(a); }
OSQPInt OSQPVectorf_length(const OSQPVectorf* a) { return a->length; }
OSQPInt OSQPVectori_length(const OSQPVectori* a) { return a->length; }
OSQPFloat* OSQPVectorf_data(const OSQPVectorf* a) { return a->d_val; }

void OSQPVectorf_subvector_assign(OSQPVectorf* A, OSQPFloat* b, OSQPInt start, OSQPInt length, OSQPFloat multiplier) {
  if (length <= 0) return;
  T* tmp = NULL;
  check(cudaMallocAsync((void**)&tmp, sizeof(T) * length, stream()), "subvector_assign");
  check(cudaMemcpyAsync(tmp, b, sizeof(T) * length, cudaMemcpyDefault, stream()), "subvector_assign");
  T* d = A->d_val + start;
  const T mlt = multiplier;
  ew(length, [=] __device__(int i) { d[i] = mlt * tmp[i]; });
  cudaFreeAsync(tmp, stream());
  check(cudaStreamSynchronize(stream()), "subvector_assign");
}
void OSQPVectorf_subvector_assign_scalar(OSQPVectorf* A, OSQPFloat sc, OSQPInt start, OSQPInt length) {
  T* d = A->d_val + start;
  const T v = sc;
  ew(length, [=] __device__(int i) { d[i] = v; });
}
OSQPVectorf* OSQPVectorf_subvector_byrows(const OSQPVectorf* A, const OSQPVectori* rows) {
  std::vector<T> a(A->length > 0 ? A->length : 1);
  std::vector<OSQPInt> r(rows->length > 0 ? rows->length : 1);
  OSQPVectorf_to_raw(a.data(), A);
  OSQPVectori_to_raw(r.data(), rows);
  std::vector<T> out;
  for (OSQPInt i = 0; i < A->length; i++) if (r[i]) out.push_back(a[i]);
  return OSQPVectorf_new(out.data(), (OSQPInt)out.size());
}
OSQPVectorf* OSQPVectorf_concat(const OSQPVectorf* A, const OSQPVectorf* B) {
  OSQPVectorf* v = OSQPVectorf_malloc(A->length + B->length);
  if (!v) return NULL;
  if (A->length) check(cudaMemcpyAsync(v->d_val, A->d_val, sizeof(T) * A->length, cudaMemcpyDeviceToDevice, stream()), "concat");
  if (B->length) check(cudaMemcpyAsync(v->d_val + A->length, B->d_val, sizeof(T) * B->length, cudaMemcpyDeviceToDevice, stream()), "concat");
  return v;
}

void OSQPVectorf_set_scalar(OSQPVectorf* a, OSQPFloat sc) {
  T* d = a->d_val; const T v = sc;
  ew(a->length, [=] __device__(int i) { d[i] = v; });
}
void OSQPVectorf_set_scalar_conditional(OSQPVectorf* a, const OSQPVectori* test, OSQPFloat neg, OSQPFloat zero, OSQPFloat pos) {
  T* d = a->d_val; const OSQPInt* t = test->d_val;
  const T vn = neg, vz = zero, vp = pos;
  ew(a->length, [=] __device__(int i) { d[i] = t[i] < 0 ? vn : (t[i] == 0 ? vz : vp); });
}
void OSQPVectorf_round_to_zero(OSQPVectorf* a, OSQPFloat tol) {
  T* d = a->d_val; const T tl = tol;
  ew(a->length, [=] __device__(int i) { if (fabs(d[i]) < tl) d[i] = T(0); });
}
void OSQPVectorf_mult_scalar(OSQPVectorf* a, OSQPFloat sc) {
  T* d = a->d_val; const T v = sc;
  ew(a->length, [=] __device__(int i) { d[i] *= v; });
}
void OSQPVectorf_plus(OSQPVectorf* x, const OSQPVectorf* a, const OSQPVectorf* b) {
  T* xd = x->d_val; const T* ad = a->d_val; const T* bd = b->d_val;
  ew(a->length, [=] __device__(int i) { xd[i] = ad[i] + bd[i]; });
}
void OSQPVectorf_minus(OSQPVectorf* x, const OSQPVectorf* a, const OSQPVectorf* b) {
  T* xd = x->d_val; const T* ad = a->d_val; const T* bd = b->d_val;
  ew(a->length, [=] __device__(int i) { xd[i] = ad[i] - bd[i]; });
}
void OSQPVectorf_add_scaled(OSQPVectorf* x, OSQPFloat sca, const OSQPVectorf* a, OSQPFloat scb, const OSQPVectorf* b) {
  T* xd = x->d_val; const T* ad = a->d_val; const T* bd = b->d_val;
  const T ca = sca, cb = scb;
  ew(x->length, [=] __device__(int i) { xd[i] = ca * ad[i] + cb * bd[i]; });
}
void OSQPVectorf_add_scaled3(OSQPVectorf* x, OSQPFloat sca, const OSQPVectorf* a, OSQPFloat scb, const OSQPVectorf* b,
                             OSQPFloat scc, const OSQPVectorf* c) {
  T* xd = x->d_val; const T* ad = a->d_val; const T* bd = b->d_val; const T* cd = c->d_val;
  const T ca = sca, cb = scb, cc = scc;
  ew(x->length, [=] __device__(int i) { xd[i] = ca * ad[i] + cb * bd[i] + cc * cd[i]; });
}
void OSQPVectorf_ew_prod(OSQPVectorf* c, const OSQPVectorf* a, const OSQPVectorf* b) {
  T* cd = c->d_val; const T* ad = a->d_val; const T* bd = b->d_val;
  ew(a->length, [=] __device__(int i) { cd[i] = ad[i] * bd[i]; });
}
void OSQPVectorf_ew_bound_vec(OSQPVectorf* x, const OSQPVectorf* z, const OSQPVectorf* l, const OSQPVectorf* u) {
  T* xd = x->d_val; const T* zd = z->d_val; const T* ld = l->d_val; const T* ud = u->d_val;
  ew(x->length, [=] __device__(int i) { xd[i] = tmin(tmax(zd[i], ld[i]), ud[i]); });
}
void OSQPVectorf_project_polar_reccone(OSQPVectorf* y, const OSQPVectorf* l, const OSQPVectorf* u, OSQPFloat infval) {
  T* yd = y->d_val; const T* ld = l->d_val; const T* ud = u->d_val; const T inf = infval;
  ew(y->length, [=] __device__(int i) {
    if (ud[i] > inf) yd[i] = (ld[i] < -inf) ? T(0) : tmin(yd[i], T(0));
    else if (ld[i] < -inf) yd[i] = tmax(yd[i], T(0));
  });
}
void OSQPVectorf_ew_reciprocal(OSQPVectorf* b, const OSQPVectorf* a) {
  T* bd = b->d_val; const T* ad = a->d_val;
  ew(a->length, [=] __device__(int i) { bd[i] = T(1) / ad[i]; });
}
void OSQPVectorf_ew_sqrt(OSQPVectorf* a) {
  T* d = a->d_val;
  ew(a->length, [=] __device__(int i) { d[i] = sqrt(d[i]); });
}
void OSQPVectorf_ew_max_vec(OSQPVectorf* c, const OSQPVectorf* a, const OSQPVectorf* b) {
  T* cd = c->d_val; const T* ad = a->d_val; const T* bd = b->d_val;
  ew(a->length, [=] __device__(int i) { cd[i] = tmax(ad[i], bd[i]); });
}
void OSQPVectorf_ew_min_vec(OSQPVectorf* c, const OSQPVectorf* a, const OSQPVectorf* b) {
  T* cd = c->d_val; const T* ad = a->d_val; const T* bd = b->d_val;
  ew(a->length, [=] __device__(int i) { cd[i] = tmin(ad[i], bd[i]); });
}
void OSQPVectorf_set_scalar_if_lt(OSQPVectorf* x, const OSQPVectorf* z, OSQPFloat testval, OSQPFloat newval) {
  T* xd = x->d_val; const T* zd = z->d_val; const T tv = testval, nv = newval;
  ew(x->length, [=] __device__(int i) { xd[i] = zd[i] < tv ? nv : zd[i]; });
}
void OSQPVectorf_set_scalar_if_gt(OSQPVectorf* x, const OSQPVectorf* z, OSQPFloat testval, OSQPFloat newval) {
  T* xd = x->d_val; const T* zd = z->d_val; const T tv = testval, nv = newval;
  ew(x->length, [=] __device__(int i) { xd[i] = zd[i] > tv ? nv : zd[i]; });
}

// ---- reductions ----
OSQPFloat OSQPVectorf_norm_inf(const OSQPVectorf* v) {
  const T* d = v->d_val;
  return (OSQPFloat)reduce(v->length, [=] __device__(int i, Acc<T>&, T& m) { m = tmax(m, (T)fabs(d[i])); }).max;
}
OSQPFloat OSQPVectorf_scaled_norm_inf(const OSQPVectorf* S, const OSQPVectorf* v) {
  const T* s = S->d_val; const T* d = v->d_val;
  return (OSQPFloat)reduce(v->length, [=] __device__(int i, Acc<T>&, T& m) { m = tmax(m, (T)fabs(s[i] * d[i])); }).max;
}
OSQPFloat OSQPVectorf_norm_inf_diff(const OSQPVectorf* a, const OSQPVectorf* b) {
  const T* x = a->d_val; const T* y = b->d_val;
  return (OSQPFloat)reduce(a->length, [=] __device__(int i, Acc<T>&, T& m) { m = tmax(m, (T)fabs(x[i] - y[i])); }).max;
}
OSQPFloat OSQPVectorf_norm_2(const OSQPVectorf* v) {
  const T* d = v->d_val;
  return (OSQPFloat)sqrt(reduce(v->length, [=] __device__(int i, Acc<T>& s, T&) { s.add_prod(d[i], d[i]); }).sum);
}
OSQPFloat OSQPVectorf_norm_1(const OSQPVectorf* v) {
  const T* d = v->d_val;
  return (OSQPFloat)reduce(v->length, [=] __device__(int i, Acc<T>& s, T&) { s.add((T)fabs(d[i])); }).sum;
}
OSQPFloat OSQPVectorf_dot_prod(const OSQPVectorf* a, const OSQPVectorf* b) {
  const T* x = a->d_val; const T* y = b->d_val;
  return (OSQPFloat)reduce(a->length, [=] __device__(int i, Acc<T>& s, T&) { s.add_prod(x[i], y[i]); }).sum;
}
OSQPFloat OSQPVectorf_dot_prod_signed(const OSQPVectorf* a, const OSQPVectorf* b, OSQPInt sign) {
  const T* x = a->d_val; const T* y = b->d_val;
  if (sign == 1) return (OSQPFloat)reduce(a->length, [=] __device__(int i, Acc<T>& s, T&) { s.add_prod(x[i], tmax(y[i], T(0))); }).sum;
  if (sign == -1) return (OSQPFloat)reduce(a->length, [=] __device__(int i, Acc<T>& s, T&) { s.add_prod(x[i], tmin(y[i], T(0))); }).sum;
  return OSQPVectorf_dot_prod(a, b);
}
OSQPInt OSQPVectorf_is_eq(const OSQPVectorf* A, const OSQPVectorf* B, OSQPFloat tol) {
  if (A->length != B->length) return 0;
  const T* x = A->d_val; const T* y = B->d_val; const T tl = tol;
  return reduce(A->length, [=] __device__(int i, Acc<T>&, T& m) { if (fabs(x[i] - y[i]) > tl) m = T(1); }).max == 0.0;
}
OSQPInt OSQPVectorf_all_leq(const OSQPVectorf* l, const OSQPVectorf* u) {
  const T* x = l->d_val; const T* y = u->d_val;
  return reduce(l->length, [=] __device__(int i, Acc<T>&, T& m) { if (x[i] > y[i]) m = T(1); }).max == 0.0;
}
OSQPInt OSQPVectorf_in_reccone(const OSQPVectorf* y, const OSQPVectorf* l, const OSQPVectorf* u, OSQPFloat infval, OSQPFloat tol) {
  const T* yd = y->d_val; const T* ld = l->d_val; const T* ud = u->d_val; const T inf = infval, tl = tol;
  return reduce(y->length, [=] __device__(int i, Acc<T>&, T& m) {
    if ((ud[i] < inf && yd[i] > tl) || (ld[i] > -inf && yd[i] < -tl)) m = T(1);
  }).max == 0.0;
}
OSQPInt OSQPVectorf_ew_bounds_type(OSQPVectori* iseq, const OSQPVectorf* l, const OSQPVectorf* u, OSQPFloat tol, OSQPFloat infval) {
  OSQPInt* t = iseq->d_val; const T* ld = l->d_val; const T* ud = u->d_val; const T tl = tol, inf = infval;
  return reduce(iseq->length, [=] __device__(int i, Acc<T>&, T& m) {
    const OSQPInt old = t[i];
    OSQPInt nt;
    if (ld[i] < -inf && ud[i] > inf) nt = -1;
    else if (ud[i] - ld[i] < tl) nt = 1;
    else nt = 0;
    t[i] = nt;
    if (nt != old) m = T(1);
  }).max != 0.0;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Matrices
// ---------------------------------------------------------------------------
struct OSQPMatrix_ {
  OSQPInt m, n, nnz;
  int triu;             // upper-triangular storage of a symmetric matrix
  OSQPInt *p, *i;       // CSC master (device)
  T* x;
  int* ecol;            // column of every CSC entry
  CSR<T> S;             // rows of the represented matrix (full symmetric if triu)
  int* src;             // S.val[k] = x[src[k]], or 0 for a structural diagonal
  int* diag;            // triu: position of (j,j) in S
  int nnzS;
  CSR<T> At;            // non-triu: the CSC arrays read as CSR of the transpose
};

namespace gba {

__global__ void k_gather_vals(T* dst, const T* src, const int* idx, int n) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const int s = idx[k];
    dst[k] = s >= 0 ? src[s] : T(0);
  }
}
static void refresh(OSQPMatrix* M) {
  if (M->nnzS > 0) k_gather_vals<<<ew_blocks(M->nnzS), kEwThreads, 0, stream()>>>(M->S.val, M->x, M->src, M->nnzS);
}

// Row-major view of a CSC matrix (CSR of the represented matrix).
static int build_rows(OSQPMatrix* M) {
  cudaStream_t s = stream();
  const int n = M->n, m = M->m, nnz = M->nnz;
  if (!M->triu) {
    M->nnzS = nnz;
    if (cudaMalloc((void**)&M->S.rowptr, sizeof(int) * (m + 1)) != cudaSuccess) return 1;
    if (cudaMalloc((void**)&M->S.col, sizeof(int) * (nnz > 0 ? nnz : 1)) != cudaSuccess) return 1;
    if (cudaMalloc((void**)&M->S.val, sizeof(T) * (nnz > 0 ? nnz : 1)) != cudaSuccess) return 1;
    if (cudaMalloc((void**)&M->src, sizeof(int) * (nnz > 0 ? nnz : 1)) != cudaSuccess) return 1;
    int *keys_out = nullptr, *idx = nullptr;
    check(cudaMallocAsync((void**)&keys_out, sizeof(int) * (nnz > 0 ? nnz : 1), s), "build");
    check(cudaMallocAsync((void**)&idx, sizeof(int) * (nnz > 0 ? nnz : 1), s), "build");
    if (nnz) {
      k_iota<<<ew_blocks(nnz), kEwThreads, 0, s>>>(idx, nnz);
      void* tmp = nullptr; size_t tb = 0;
      const int bits = bits_for((unsigned long long)(m > 0 ? m : 1));
      cub::DeviceRadixSort::SortPairs(tmp, tb, (const int*)M->i, keys_out, idx, M->src, nnz, 0, bits, s);
      check(cudaMallocAsync(&tmp, tb ? tb : 1, s), "build");
      check(cub::DeviceRadixSort::SortPairs(tmp, tb, (const int*)M->i, keys_out, idx, M->src, nnz, 0, bits, s), "sort");
      k_gather_int<<<ew_blocks(nnz), kEwThreads, 0, s>>>(M->ecol, M->src, nnz, (int*)M->S.col);
      cudaFreeAsync(tmp, s);
    }
    k_rowptr_from_sorted<<<std::max(1, ew_blocks(nnz + 1)), kEwThreads, 0, s>>>(keys_out, nnz, m, (int*)M->S.rowptr);
    cudaFreeAsync(keys_out, s); cudaFreeAsync(idx, s);
    M->S.rows = m; M->S.cols = n; M->S.lanes = pick_lanes(nnz, m);
    M->At = CSR<T>{(const int*)M->p, (const int*)M->i, M->x, n, m, pick_lanes(nnz, n)};
  } else {
    std::vector<OSQPInt> hp(n + 1), hi(nnz > 0 ? nnz : 1);
    check(cudaMemcpy(hp.data(), M->p, sizeof(OSQPInt) * (n + 1), cudaMemcpyDeviceToHost), "pattern");
    if (nnz) check(cudaMemcpy(hi.data(), M->i, sizeof(OSQPInt) * nnz, cudaMemcpyDeviceToHost), "pattern");
    int ndiag = 0;
    for (int j = 0; j < n; j++)
      for (int k = hp[j]; k < hp[j + 1]; k++) if (hi[k] == j) { ndiag++; break; }
    const int nnzF = 2 * nnz - 2 * ndiag + n;
    M->nnzS = nnzF;
    if (cudaMalloc((void**)&M->S.rowptr, sizeof(int) * (n + 1)) != cudaSuccess) return 1;
    if (cudaMalloc((void**)&M->S.col, sizeof(int) * nnzF) != cudaSuccess) return 1;
    if (cudaMalloc((void**)&M->S.val, sizeof(T) * nnzF) != cudaSuccess) return 1;
    if (cudaMalloc((void**)&M->src, sizeof(int) * nnzF) != cudaSuccess) return 1;
    if (cudaMalloc((void**)&M->diag, sizeof(int) * (n > 0 ? n : 1)) != cudaSuccess) return 1;
    const int slots = 2 * nnz + n;
    unsigned long long *k_in = nullptr, *k_out = nullptr;
    int *s_in = nullptr, *s_out = nullptr;
    check(cudaMallocAsync((void**)&k_in, sizeof(unsigned long long) * slots, s), "build");
    check(cudaMallocAsync((void**)&k_out, sizeof(unsigned long long) * slots, s), "build");
    check(cudaMallocAsync((void**)&s_in, sizeof(int) * slots, s), "build");
    check(cudaMallocAsync((void**)&s_out, sizeof(int) * slots, s), "build");
    k_triu_expand<<<std::max(1, (n + 255) / 256), 256, 0, s>>>((const int*)M->p, (const int*)M->i, n, nnz, k_in, s_in);
    void* tmp = nullptr; size_t tb = 0;
    cub::DeviceRadixSort::SortPairs(tmp, tb, k_in, k_out, s_in, s_out, slots, 0, 64, s);
    check(cudaMallocAsync(&tmp, tb ? tb : 1, s), "build");
    check(cub::DeviceRadixSort::SortPairs(tmp, tb, k_in, k_out, s_in, s_out, slots, 0, 64, s), "sort");
    k_full_from_sorted<<<std::max(1, (nnzF + 256) / 256), 256, 0, s>>>(k_out, nnzF, n, (int*)M->S.col, (int*)M->S.rowptr, M->diag);
    check(cudaMemcpyAsync(M->src, s_out, sizeof(int) * nnzF, cudaMemcpyDeviceToDevice, s), "build");
    cudaFreeAsync(tmp, s); cudaFreeAsync(k_in, s); cudaFreeAsync(k_out, s); cudaFreeAsync(s_in, s); cudaFreeAsync(s_out, s);
    M->S.rows = n; M->S.cols = n; M->S.lanes = pick_lanes(nnzF, n);
    M->At = M->S;
  }
  refresh(M);
  return cudaStreamSynchronize(s) != cudaSuccess;
}

}  // namespace gba

extern "C" {

void OSQPMatrix_free(OSQPMatrix* M) {
  if (!M) return;
  cudaFree(M->p); cudaFree(M->i); cudaFree(M->x); cudaFree(M->ecol);
  cudaFree((void*)M->S.rowptr); cudaFree((void*)M->S.col); cudaFree(M->S.val);
  cudaFree(M->src); cudaFree(M->diag);
  free(M);
}

OSQPMatrix* OSQPMatrix_new_from_csc(const OSQPCscMatrix* A, OSQPInt is_triu) {
  if (!A || !ensure_ctx()) return NULL;
  OSQPMatrix* M = (OSQPMatrix*)calloc(1, sizeof(OSQPMatrix));
  if (!M) return NULL;
  M->m = A->m; M->n = A->n; M->triu = is_triu ? 1 : 0;
  OSQPInt nnz = 0;
  if (cudaMemcpy(&nnz, A->p + A->n, sizeof(OSQPInt), cudaMemcpyDefault) != cudaSuccess) { free(M); return NULL; }
  M->nnz = nnz;
  cudaStream_t s = stream();
  if (cudaMalloc((void**)&M->p, sizeof(OSQPInt) * (A->n + 1)) != cudaSuccess ||
      cudaMalloc((void**)&M->i, sizeof(OSQPInt) * (nnz > 0 ? nnz : 1)) != cudaSuccess ||
      cudaMalloc((void**)&M->x, sizeof(T) * (nnz > 0 ? nnz : 1)) != cudaSuccess ||
      cudaMalloc((void**)&M->ecol, sizeof(int) * (nnz > 0 ? nnz : 1)) != cudaSuccess) {
    OSQPMatrix_free(M);
    return NULL;
  }
  check(cudaMemcpyAsync(M->p, A->p, sizeof(OSQPInt) * (A->n + 1), cudaMemcpyDefault, s), "csc");
  if (nnz) {
    check(cudaMemcpyAsync(M->i, A->i, sizeof(OSQPInt) * nnz, cudaMemcpyDefault, s), "csc");
    check(cudaMemcpyAsync(M->x, A->x, sizeof(T) * nnz, cudaMemcpyDefault, s), "csc");
  }
  k_csc_entry_cols<<<std::max(1, (A->n + 255) / 256), 256, 0, s>>>((const int*)M->p, A->n, M->ecol);
  if (build_rows(M)) { OSQPMatrix_free(M); return NULL; }
  return M;
}

OSQPInt OSQPMatrix_get_m(const OSQPMatrix* M) { return M->m; }
OSQPInt OSQPMatrix_get_n(const OSQPMatrix* M) { return M->n; }
OSQPFloat* OSQPMatrix_get_x(const OSQPMatrix* M) { return M->x; }
OSQPInt* OSQPMatrix_get_i(const OSQPMatrix* M) { return M->i; }
OSQPInt* OSQPMatrix_get_p(const OSQPMatrix* M) { return M->p; }
OSQPInt OSQPMatrix_get_nz(const OSQPMatrix* M) { return M->nnz; }

OSQPInt osqp_gb300_matrix_rows(const OSQPMatrix* M, OSQPInt* rowptr, OSQPInt* col, OSQPInt* src, OSQPInt* diag) {
  if (!M) return -1;
  const int rows = M->S.rows, nz = M->nnzS;
  if (rowptr && cudaMemcpy(rowptr, M->S.rowptr, sizeof(int) * (rows + 1), cudaMemcpyDeviceToHost) != cudaSuccess) return -1;
  if (col && nz && cudaMemcpy(col, M->S.col, sizeof(int) * nz, cudaMemcpyDeviceToHost) != cudaSuccess) return -1;
  if (src && nz && cudaMemcpy(src, M->src, sizeof(int) * nz, cudaMemcpyDeviceToHost) != cudaSuccess) return -1;
  if (diag && M->triu && M->n && cudaMemcpy(diag, M->diag, sizeof(int) * M->n, cudaMemcpyDeviceToHost) != cudaSuccess) return -1;
  return nz;
}

void OSQPMatrix_update_values(OSQPMatrix* M, const OSQPFloat* Mx_new, const OSQPInt* Mx_new_idx, OSQPInt M_new_n) {
  if (M_new_n <= 0 || !Mx_new) return;
  cudaStream_t s = stream();
  if (!Mx_new_idx) {
    check(cudaMemcpyAsync(M->x, Mx_new, sizeof(T) * M_new_n, cudaMemcpyDefault, s), "update_values");
  } else {
    T* v = NULL; OSQPInt* idx = NULL;
    check(cudaMallocAsync((void**)&v, sizeof(T) * M_new_n, s), "update_values");
    check(cudaMallocAsync((void**)&idx, sizeof(OSQPInt) * M_new_n, s), "update_values");
    check(cudaMemcpyAsync(v, Mx_new, sizeof(T) * M_new_n, cudaMemcpyDefault, s), "update_values");
    check(cudaMemcpyAsync(idx, Mx_new_idx, sizeof(OSQPInt) * M_new_n, cudaMemcpyDefault, s), "update_values");
    T* x = M->x;
    ew(M_new_n, [=] __device__(int k) { x[idx[k]] = v[k]; });
    cudaFreeAsync(v, s); cudaFreeAsync(idx, s);
  }
  refresh(M);
  check(cudaStreamSynchronize(s), "update_values");
}
void OSQPMatrix_mult_scalar(OSQPMatrix* A, OSQPFloat sc) {
  T* x = A->x; const T v = sc;
  ew(A->nnz, [=] __device__(int k) { x[k] *= v; });
  refresh(A);
}
void OSQPMatrix_lmult_diag(OSQPMatrix* A, const OSQPVectorf* L) {
  T* x = A->x; const OSQPInt* ri = A->i; const T* d = L->d_val;
  ew(A->nnz, [=] __device__(int k) { x[k] *= d[ri[k]]; });
  refresh(A);
}
void OSQPMatrix_rmult_diag(OSQPMatrix* A, const OSQPVectorf* R) {
  T* x = A->x; const int* ec = A->ecol; const T* d = R->d_val;
  ew(A->nnz, [=] __device__(int k) { x[k] *= d[ec[k]]; });
  refresh(A);
}
void OSQPMatrix_extract_diag(const OSQPMatrix* A, OSQPVectorf* d) {
  T* out = d->d_val;
  if (A->triu) {
    const T* v = A->S.val; const int* dg = A->diag;
    ew(A->n, [=] __device__(int j) { out[j] = v[dg[j]]; });
  } else {
    const OSQPInt* p = A->p; const OSQPInt* ri = A->i; const T* x = A->x;
    ew(A->n, [=] __device__(int j) {
      T a = T(0);
      for (OSQPInt k = p[j]; k < p[j + 1]; k++) if (ri[k] == j) a += x[k];
      out[j] = a;
    });
  }
}
void OSQPMatrix_AtDA_extract_diag(const OSQPMatrix* A, const OSQPVectorf* D, OSQPVectorf* d) {
  const OSQPInt* p = A->p; const OSQPInt* ri = A->i; const T* x = A->x; const T* dv = D->d_val; T* out = d->d_val;
  ew(A->n, [=] __device__(int j) {
    T a = T(0);
    for (OSQPInt k = p[j]; k < p[j + 1]; k++) a += x[k] * x[k] * dv[ri[k]];
    out[j] = a;
  });
}
void OSQPMatrix_Axpy(const OSQPMatrix* A, const OSQPVectorf* x, OSQPVectorf* y, OSQPFloat alpha, OSQPFloat beta) {
  if (!y || y->length <= 0) return;
  if (!x || x->length <= 0 || A->nnzS == 0) {  // y = beta y
    T* yd = y->d_val; const T b = beta;
    ew(y->length, [=] __device__(int i) { yd[i] = (b == T(0)) ? T(0) : b * yd[i]; });
    return;
  }
  k_spmv<T><<<std::min(4096, std::max(1, A->S.rows * A->S.lanes / 256 + 1)), 256, 0, stream()>>>(A->S, x->d_val, y->d_val, (T)alpha, (T)beta);
  check(cudaGetLastError(), "Axpy");
}
void OSQPMatrix_Atxpy(const OSQPMatrix* A, const OSQPVectorf* x, OSQPVectorf* y, OSQPFloat alpha, OSQPFloat beta) {
  if (!y || y->length <= 0) return;
  if (!x || x->length <= 0 || A->nnz == 0) {
    T* yd = y->d_val; const T b = beta;
    ew(y->length, [=] __device__(int i) { yd[i] = (b == T(0)) ? T(0) : b * yd[i]; });
    return;
  }
  k_spmv<T><<<std::min(4096, std::max(1, A->At.rows * A->At.lanes / 256 + 1)), 256, 0, stream()>>>(A->At, x->d_val, y->d_val, (T)alpha, (T)beta);
  check(cudaGetLastError(), "Atxpy");
}
// col_norm_inf: CUDA-backend semantics (algebra/cuda/matrix.cu:130-135): rows of
// the transpose, i.e. of the full symmetric matrix for P.
void OSQPMatrix_col_norm_inf(const OSQPMatrix* M, OSQPVectorf* E) {
  const CSR<T> R = M->At;
  T* out = E->d_val;
  ew(R.rows, [=] __device__(int r) {
    T a = T(0);
    for (int k = R.rowptr[r]; k < R.rowptr[r + 1]; k++) a = tmax(a, (T)fabs(R.val[k]));
    out[r] = a;
  });
}
void OSQPMatrix_row_norm_inf(const OSQPMatrix* M, OSQPVectorf* E) {
  const CSR<T> R = M->S;
  T* out = E->d_val;
  ew(R.rows, [=] __device__(int r) {
    T a = T(0);
    for (int k = R.rowptr[r]; k < R.rowptr[r + 1]; k++) a = tmax(a, (T)fabs(R.val[k]));
    out[r] = a;
  });
}
OSQPMatrix* OSQPMatrix_submatrix_byrows(const OSQPMatrix* A, const OSQPVectori* rows) {
  if (A->triu) return NULL;  // as the reference: no row selection of a triangular matrix
  std::vector<OSQPInt> hp(A->n + 1), hi(A->nnz > 0 ? A->nnz : 1), fl(A->m > 0 ? A->m : 1);
  std::vector<T> hx(A->nnz > 0 ? A->nnz : 1);
  check(cudaMemcpy(hp.data(), A->p, sizeof(OSQPInt) * (A->n + 1), cudaMemcpyDeviceToHost), "submatrix");
  if (A->nnz) {
    check(cudaMemcpy(hi.data(), A->i, sizeof(OSQPInt) * A->nnz, cudaMemcpyDeviceToHost), "submatrix");
    check(cudaMemcpy(hx.data(), A->x, sizeof(T) * A->nnz, cudaMemcpyDeviceToHost), "submatrix");
  }
  if (A->m) OSQPVectori_to_raw(fl.data(), rows);
  std::vector<OSQPInt> map(A->m > 0 ? A->m : 1, -1);
  OSQPInt mr = 0;
  for (OSQPInt r = 0; r < A->m; r++) if (fl[r]) map[r] = mr++;
  std::vector<OSQPInt> np(A->n + 1, 0), ni;
  std::vector<T> nx;
  for (OSQPInt j = 0; j < A->n; j++) {
    for (OSQPInt k = hp[j]; k < hp[j + 1]; k++)
      if (map[hi[k]] >= 0) { ni.push_back(map[hi[k]]); nx.push_back(hx[k]); }
    np[j + 1] = (OSQPInt)ni.size();
  }
  if (ni.empty()) { ni.push_back(0); nx.push_back(T(0)); }
  OSQPCscMatrix C;
  C.m = mr; C.n = A->n; C.p = np.data(); C.i = ni.data(); C.x = nx.data(); C.nzmax = np[A->n]; C.nz = -1; C.owned = 0;
  return OSQPMatrix_new_from_csc(&C, 0);
}
OSQPInt OSQPMatrix_is_eq(const OSQPMatrix* A, const OSQPMatrix* B, OSQPFloat tol) {
  if (A->m != B->m || A->n != B->n || A->nnz != B->nnz || A->triu != B->triu) return 0;
  std::vector<OSQPInt> pa(A->n + 1), pb(A->n + 1), ia(A->nnz + 1), ib(A->nnz + 1);
  std::vector<T> xa(A->nnz + 1), xb(A->nnz + 1);
  cudaMemcpy(pa.data(), A->p, sizeof(OSQPInt) * (A->n + 1), cudaMemcpyDeviceToHost);
  cudaMemcpy(pb.data(), B->p, sizeof(OSQPInt) * (A->n + 1), cudaMemcpyDeviceToHost);
  if (A->nnz) {
    cudaMemcpy(ia.data(), A->i, sizeof(OSQPInt) * A->nnz, cudaMemcpyDeviceToHost);
    cudaMemcpy(ib.data(), B->i, sizeof(OSQPInt) * A->nnz, cudaMemcpyDeviceToHost);
    cudaMemcpy(xa.data(), A->x, sizeof(T) * A->nnz, cudaMemcpyDeviceToHost);
    cudaMemcpy(xb.data(), B->x, sizeof(T) * A->nnz, cudaMemcpyDeviceToHost);
  }
  for (OSQPInt j = 0; j <= A->n; j++) if (pa[j] != pb[j]) return 0;
  for (OSQPInt k = 0; k < A->nnz; k++) if (ia[k] != ib[k] || fabs((double)xa[k] - (double)xb[k]) > tol) return 0;
  return 1;
}

// ---------------------------------------------------------------------------
// Backend
// ---------------------------------------------------------------------------
OSQPInt osqp_algebra_linsys_supported(void) { return OSQP_CAPABILITY_INDIRECT_SOLVER; }
enum osqp_linsys_solver_type osqp_algebra_default_linsys(void) { return OSQP_INDIRECT_SOLVER; }
OSQPInt osqp_algebra_init_libs(OSQPInt device) {
  if (g_ctx.refs == 0) g_ctx.device = device;
  if (cudaSetDevice(device) != cudaSuccess) return 1;
  if (!ensure_ctx()) return 1;
  g_ctx.refs++;
  return 0;
}
void osqp_algebra_free_libs(void) {
  // Buffers stay alive while any solver might still use them; the context is
  // released with the process.  (The reference frees its global handle on
  // every osqp_cleanup, which breaks concurrent solvers.)
  if (g_ctx.refs > 0) g_ctx.refs--;
}
OSQPInt osqp_algebra_name(char* name, OSQPInt nameLen) {
  const char* s = sizeof(T) == 4 ? "GB300 sm_103a (FP32, FP64 reductions)" : "GB300 sm_103a (FP64)";
  snprintf(name, nameLen, "%s", s);
  return (OSQPInt)strlen(name) + 1;
}
OSQPInt osqp_algebra_device_name(char* name, OSQPInt nameLen) {
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, g_ctx.device) != cudaSuccess) return 0;
  snprintf(name, nameLen, "%s (SMs: %d)", prop.name, prop.multiProcessorCount);
  return (OSQPInt)strlen(name) + 1;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Linear system: reduced-KKT PCG (cuda_pcg_interface.cu:99-361)
// ---------------------------------------------------------------------------
namespace gba {

constexpr int kLsBlockThreads = 1024;

__global__ void __launch_bounds__(kLsBlockThreads, 1)
k_linsys(DevProblem<T> pr, DevSettings s, int kktL, T* b, int admm_iter, int polishing, double spr, double sdr) {
  __shared__ GroupShared gsh;
  __shared__ SolverScalars ssc;
  if (threadIdx.x == 0) { gsh.parity = 0; gsh.flag = 0; ssc = *pr.st; }
  __syncthreads();
  BlockGroup g{&gsh};
  Solver<T> S{pr, s, &ssc, kktL};
  S.linsys_solve(g, b, admm_iter, polishing != 0, spr, sdr);
  __syncthreads();
  if (threadIdx.x == 0) *pr.st = ssc;
}
__global__ void __launch_bounds__(kLsBlockThreads, 1)
k_linsys_grid(DevProblem<T> pr, DevSettings s, int kktL, T* b, int admm_iter, int polishing, double spr, double sdr,
              GridSync gs) {
  __shared__ GroupShared gsh;
  __shared__ SolverScalars ssc;
  if (threadIdx.x == 0) { gsh.parity = 0; gsh.flag = 0; ssc = *pr.st; }
  __syncthreads();
  GridGroup g{&gsh, gs};
  Solver<T> S{pr, s, &ssc, kktL};
  bool ok = S.linsys_solve(g, b, admm_iter, polishing != 0, spr, sdr);
  __syncthreads();
  if (ok && blockIdx.x == 0 && threadIdx.x == 0) *pr.st = ssc;
}
__global__ void k_ls_precond(DevProblem<T> pr, double sigma, double rho, int rho_vec, int precond) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < pr.n; i += gridDim.x * blockDim.x) {
    if (precond == 0) { pr.Minv[i] = T(1); continue; }
    T d = T(0);
    for (int k = pr.At.rowptr[i]; k < pr.At.rowptr[i + 1]; k++) {
      const T a = pr.At.val[k];
      d += rho_vec ? a * a * pr.rho_vec[pr.At.col[k]] : a * a;
    }
    if (!rho_vec) d *= (T)rho;
    pr.Minv[i] = T(1) / ((T)sigma + pr.P.val[pr.Pdiag[i]] + d);
  }
}

struct GbPcg {
  LinSysSolver base;
  int n, m, polishing, use_grid, grid_blocks;
  DevProblem<T> pr;
  DevSettings ds;
  int kktL;
  char* arena;
  SolverScalars* d_st;
  SolverScalars h_st;
  OSQPFloat *spr, *sdr;
  unsigned* bar;
  int* err;
  double* partials;
  int rho_vec;
  double rho;
};

static const char* ls_name(LinSysSolver* self) {
  GbPcg* s = (GbPcg*)self;
  if (s->ds.cg_precond == kPrecondBlockDiagonal) return "GB300 reduced-KKT PCG - Block-diagonal preconditioner";
  return s->ds.cg_precond ? "GB300 reduced-KKT PCG - Diagonal preconditioner" : "GB300 reduced-KKT PCG - No preconditioner";
}
// Block-Jacobi storage, allocated when cg_precond = 2 is first asked for.
static int ls_ensure_blocks(GbPcg* s) {
  if (s->pr.Binv || s->ds.cg_precond != kPrecondBlockDiagonal) return 0;
  T* p = nullptr;
  if (cudaMalloc((void**)&p, sizeof(T) * block_precond_elems(s->n)) != cudaSuccess) return 1;
  s->pr.Binv = p;
  return 0;
}
static void ls_precond(GbPcg* s) {
  k_ls_precond<<<ew_blocks(s->n), kEwThreads, 0, stream()>>>(s->pr, s->ds.sigma, s->rho, s->rho_vec, s->ds.cg_precond);
  if (s->ds.cg_precond == kPrecondBlockDiagonal && s->pr.Binv && s->n > 0)
    k_block_precond<T><<<block_precond_grid(s->n), kBlockPrecondThreads, 0, stream()>>>(s->pr, s->ds.sigma, s->rho,
                                                                                       s->rho_vec);
}
static OSQPInt ls_solve(LinSysSolver* self, OSQPVectorf* b, OSQPInt admm_iter) {
  GbPcg* s = (GbPcg*)self;
  const double spr = s->spr ? (double)*s->spr : 0.0, sdr = s->sdr ? (double)*s->sdr : 0.0;
  cudaStream_t st = stream();
  if (s->use_grid) {
    cudaMemsetAsync(s->bar, 0, sizeof(unsigned) * 4 + sizeof(int) * 4, st);
    GridSync gs{s->bar, s->bar + 1, s->err, s->partials, s->partials + (size_t)4 * kMaxSum * s->grid_blocks};
    T* bp = b->d_val;
    int it = admm_iter, pol = s->polishing;
    void* args[] = {(void*)&s->pr, (void*)&s->ds, (void*)&s->kktL, (void*)&bp, (void*)&it, (void*)&pol,
                    (void*)&spr, (void*)&sdr, (void*)&gs};
    check(cudaLaunchCooperativeKernel((void*)k_linsys_grid, dim3(s->grid_blocks), dim3(kLsBlockThreads), args, 0, st), "linsys");
  } else {
    k_linsys<<<1, kLsBlockThreads, 0, st>>>(s->pr, s->ds, s->kktL, b->d_val, admm_iter, s->polishing, spr, sdr);
  }
  return cudaStreamSynchronize(st) != cudaSuccess;
}
static void ls_update_settings(LinSysSolver* self, const OSQPSettings* st) {
  GbPcg* s = (GbPcg*)self;
  s->ds.cg_max_iter = st->cg_max_iter;
  s->ds.cg_tol_reduction = st->cg_tol_reduction;
  s->ds.cg_tol_fraction = st->cg_tol_fraction;
  if (s->ds.cg_precond != (int)st->cg_precond) {
    const int before = s->ds.cg_precond;
    s->ds.cg_precond = (int)st->cg_precond;
    if (ls_ensure_blocks(s)) {
      // no room for the blocks: the solver keeps its previous preconditioner
      fprintf(stderr, "osqp_gb300 linsys: no device memory for the block-diagonal preconditioner\n");
      s->ds.cg_precond = before;
    }
    ls_precond(s);
  }
}
static void ls_warm_start(LinSysSolver* self, const OSQPVectorf* x) {
  GbPcg* s = (GbPcg*)self;
  if (x->length > 0) check(cudaMemcpyAsync(s->pr.xp, x->d_val, sizeof(T) * x->length, cudaMemcpyDeviceToDevice, stream()), "warm_start");
}
static OSQPInt ls_adjoint(LinSysSolver*) { return OSQP_FUNC_NOT_IMPLEMENTED; }
static void ls_free(LinSysSolver* self) {
  GbPcg* s = (GbPcg*)self;
  if (!s) return;
  if (s->arena) cudaFree(s->arena);
  if (s->pr.Binv) cudaFree(s->pr.Binv);
  free(s);
}
static OSQPInt ls_update_matrices(LinSysSolver* self, const OSQPMatrix*, const OSQPInt*, OSQPInt, const OSQPMatrix*,
                                  const OSQPInt*, OSQPInt) {
  // the solver views the matrices' device arrays; only the preconditioner changes
  ls_precond((GbPcg*)self);
  return 0;
}
static OSQPInt ls_update_rho_vec(LinSysSolver* self, const OSQPVectorf*, OSQPFloat rho_sc) {
  GbPcg* s = (GbPcg*)self;
  s->rho = rho_sc;
  check(cudaMemcpyAsync(&s->d_st->rho, &s->rho, sizeof(double), cudaMemcpyHostToDevice, stream()), "rho");
  check(cudaStreamSynchronize(stream()), "rho");
  ls_precond(s);
  return 0;
}

}  // namespace gba

extern "C" OSQPInt osqp_algebra_init_linsys_solver(LinSysSolver** sp, const OSQPMatrix* P, const OSQPMatrix* A,
                                                   const OSQPVectorf* rho_vec, const OSQPSettings* settings,
                                                   OSQPFloat* scaled_prim_res, OSQPFloat* scaled_dual_res,
                                                   OSQPInt polishing) {
  if (!sp || !P || !A || !settings || !ensure_ctx()) return OSQP_LINSYS_SOLVER_INIT_ERROR;
  *sp = NULL;
  GbPcg* s = (GbPcg*)calloc(1, sizeof(GbPcg));
  if (!s) return OSQP_LINSYS_SOLVER_INIT_ERROR;
  const int n = P->n, m = A->m;
  s->n = n; s->m = m; s->polishing = polishing ? 1 : 0;
  s->spr = scaled_prim_res; s->sdr = scaled_dual_res;
  s->rho_vec = (!polishing && rho_vec) ? 1 : 0;
  s->rho = polishing ? 1.0 / settings->delta : settings->rho;
  DevSettings& d = s->ds;
  memset(&d, 0, sizeof(d));
  d.sigma = polishing ? settings->delta : settings->sigma;
  d.rho = s->rho;
  d.rho_is_vec = s->rho_vec;
  d.cg_max_iter = settings->cg_max_iter;
  d.cg_tol_reduction = settings->cg_tol_reduction;
  d.cg_tol_fraction = settings->cg_tol_fraction;
  d.cg_precond = (int)settings->cg_precond;
  d.infty = (double)OSQP_INFTY;
  // device vectors: xp r p0 p1 Kp yv rhs Minv (n), t (m), scalars, grid buffers
  const long long sms = 152;
  size_t off = 0;
  auto take = [&](size_t bytes) { off = (off + 255) & ~size_t(255); size_t o = off; off += bytes > 0 ? bytes : 1; return o; };
  size_t o_vn[8];
  for (int k = 0; k < 8; k++) o_vn[k] = take(sizeof(T) * n);
  size_t o_t = take(sizeof(T) * m), o_st = take(sizeof(SolverScalars)), o_bar = take(64);
  size_t o_part = take(sizeof(double) * (4 * kMaxSum + 2 * kMaxMax) * sms * 2);
  if (cudaMalloc((void**)&s->arena, off) != cudaSuccess) { free(s); return OSQP_LINSYS_SOLVER_INIT_ERROR; }
  cudaMemsetAsync(s->arena, 0, off, stream());
  char* a = s->arena;
  DevProblem<T>& pr = s->pr;
  memset(&pr, 0, sizeof(pr));
  pr.n = n; pr.m = m;
  pr.P = P->S; pr.A = A->S; pr.At = A->At; pr.Pdiag = P->diag;
  pr.rho_vec = s->rho_vec ? rho_vec->d_val : NULL;
  pr.xp = (T*)(a + o_vn[0]); pr.r = (T*)(a + o_vn[1]); pr.p0 = (T*)(a + o_vn[2]); pr.p1 = (T*)(a + o_vn[3]);
  pr.Kp = (T*)(a + o_vn[4]); pr.yv = (T*)(a + o_vn[5]); pr.rhs = (T*)(a + o_vn[6]); pr.Minv = (T*)(a + o_vn[7]);
  pr.t = (T*)(a + o_t);
  pr.Arow_g = pr.A.rowptr; pr.Acol_g = pr.A.col; pr.Aval_g = pr.A.val;
  if (ls_ensure_blocks(s)) { ls_free(&s->base); return OSQP_LINSYS_SOLVER_INIT_ERROR; }
  s->d_st = (SolverScalars*)(a + o_st);
  pr.st = s->d_st;
  s->bar = (unsigned*)(a + o_bar); s->err = (int*)(s->bar + 4);
  s->partials = (double*)(a + o_part);
  memset(&s->h_st, 0, sizeof(SolverScalars));
  s->h_st.rho = s->rho;
  s->h_st.reduction_factor = settings->cg_tol_fraction;
  s->h_st.eps_prev = 1.0;
  check(cudaMemcpyAsync(s->d_st, &s->h_st, sizeof(SolverScalars), cudaMemcpyHostToDevice, stream()), "linsys init");
  s->kktL = pick_lanes((long long)P->nnzS + A->nnz, n);
  const long long work = (long long)P->nnzS + 2LL * A->nnz + n + m;
  s->use_grid = work > 200000;
  if (s->use_grid) {
    int per_sm = 0, nsm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_linsys_grid, kLsBlockThreads, 0);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, g_ctx.device);
    if (per_sm < 1 || nsm > sms) s->use_grid = 0;
    else s->grid_blocks = nsm;
  }
  LinSysSolver& b = s->base;
  b.type = OSQP_INDIRECT_SOLVER;
  b.name = ls_name;
  b.solve = ls_solve;
  b.update_settings = ls_update_settings;
  b.warm_start = ls_warm_start;
  b.adjoint_derivative = ls_adjoint;
  b.free = ls_free;
  b.update_matrices = ls_update_matrices;
  b.update_rho_vec = ls_update_rho_vec;
  b.nthreads = 1;
  ls_precond(s);
  if (cudaStreamSynchronize(stream()) != cudaSuccess) { ls_free(&s->base); return OSQP_LINSYS_SOLVER_INIT_ERROR; }
  *sp = &s->base;
  return 0;
}

// ---------------------------------------------------------------------------
// Allocation-free reduced-KKT solve
//
// For callers that cannot allocate device memory at the point of the call:
// real-time control loops whose device memory is fixed before the loop starts
// (an allocation can block or fail at a moment the loop cannot afford), and
// host programs that share the GPU under a memory budget granted up front.
// The PCG work vectors live in the file-scope array below
// (kNoAllocScratchBytes per device, held by every GPU that loads the library
// until the process exits) instead of a per-solver cudaMalloc.
// ---------------------------------------------------------------------------
namespace gba {

constexpr size_t kNoAllocScratchBytes = size_t(4) << 20;   // 4 MiB per device
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];
static void* g_noalloc_addr[64];   // device address of g_noalloc_scratch, per device

// Bytes of scratch a solve with n variables and m constraints needs: eight
// n-vectors and one m-vector, each on a 256-byte boundary, then the
// block-Jacobi blocks when `blocks` is set.
static size_t noalloc_bytes(long long n, long long m, bool blocks) {
  auto r = [](size_t b) { return (b + 255) & ~size_t(255); };
  return 8 * r(sizeof(T) * (size_t)(n > 0 ? n : 1)) + r(sizeof(T) * (size_t)(m > 0 ? m : 1)) +
         (blocks ? r(sizeof(T) * block_precond_elems(n)) : 0);
}

__global__ void __launch_bounds__(kLsBlockThreads, 1)
k_linsys_noalloc(DevProblem<T> pr, DevSettings s, int kktL, T* b, double rho) {
  __shared__ GroupShared gsh;
  __shared__ SolverScalars ssc;
  if (threadIdx.x == 0) {
    // fresh solver state: the scratch keeps whatever the previous call left
    unsigned char* raw = reinterpret_cast<unsigned char*>(&ssc);
    for (size_t k = 0; k < sizeof(SolverScalars); k++) raw[k] = 0;
    ssc.rho = rho;
    ssc.reduction_factor = s.cg_tol_fraction;
    ssc.eps_prev = 1.0;
    gsh.parity = 0;
    gsh.flag = 0;
  }
  __syncthreads();
  BlockGroup g{&gsh};
  Solver<T> S{pr, s, &ssc, kktL};
  // the iterate and search directions start at zero on every call
  for_each(g, pr.n, [&](int i) { pr.xp[i] = T(0); pr.p0[i] = T(0); pr.p1[i] = T(0); });
  S.update_precond(g);
  __syncthreads();
  S.linsys_solve(g, b, 1, false, 0.0, 0.0);
}

}  // namespace gba

extern "C" OSQPInt osqp_gb300_linsys_solve_noalloc(const OSQPMatrix* P, const OSQPMatrix* A,
                                                   const OSQPVectorf* rho_vec, const OSQPSettings* settings,
                                                   OSQPVectorf* b) {
  if (!P || !A || !settings || !b) return OSQP_DATA_VALIDATION_ERROR;
  const int n = P->n, m = A->m;
  if (b->length != n + m || A->n != n) return OSQP_DATA_VALIDATION_ERROR;
  const bool blocks = settings->cg_precond == (osqp_precond_type)kPrecondBlockDiagonal;
  const size_t need = noalloc_bytes(n, m, blocks);
  if (need > kNoAllocScratchBytes) {
    fprintf(stderr,
            "osqp_gb300_linsys_solve_noalloc: n=%d, m=%d needs %zu bytes of scratch; the fixed maximum is %zu bytes\n",
            n, m, need, kNoAllocScratchBytes);
    return OSQP_DATA_VALIDATION_ERROR;
  }
  // the matrices live on the library's device: make it current, so that the
  // scratch address and the launch belong to the same device
  if (!ensure_ctx()) return OSQP_ALGEBRA_LOAD_ERROR;
  const int dev = g_ctx.device;
  if (dev < 0 || dev >= 64 || cudaSetDevice(dev) != cudaSuccess) return OSQP_ALGEBRA_LOAD_ERROR;
  // set-up, once per device, with that device current: the host-side name of
  // the array is not a device address, so ask the runtime for the address
  if (!g_noalloc_addr[dev]) {
    void* ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess || !ptr) {
      fprintf(stderr, "osqp_gb300_linsys_solve_noalloc: cudaGetSymbolAddress failed: %s\n", cudaGetErrorString(e));
      return OSQP_ALGEBRA_LOAD_ERROR;
    }
    g_noalloc_addr[dev] = ptr;
  }
  char* base = (char*)g_noalloc_addr[dev];
  auto r = [](size_t v) { return (v + 255) & ~size_t(255); };
  const size_t vn = r(sizeof(T) * (size_t)(n > 0 ? n : 1));
  DevProblem<T> pr;
  memset(&pr, 0, sizeof(pr));
  pr.n = n; pr.m = m;
  pr.P = P->S; pr.A = A->S; pr.At = A->At; pr.Pdiag = P->diag;
  pr.rho_vec = rho_vec ? rho_vec->d_val : NULL;
  pr.xp = (T*)(base + 0 * vn); pr.r = (T*)(base + 1 * vn); pr.p0 = (T*)(base + 2 * vn); pr.p1 = (T*)(base + 3 * vn);
  pr.Kp = (T*)(base + 4 * vn); pr.yv = (T*)(base + 5 * vn); pr.rhs = (T*)(base + 6 * vn); pr.Minv = (T*)(base + 7 * vn);
  pr.t = (T*)(base + 8 * vn);
  pr.Arow_g = pr.A.rowptr; pr.Acol_g = pr.A.col; pr.Aval_g = pr.A.val;
  pr.Binv = blocks ? (T*)(base + 8 * vn + r(sizeof(T) * (size_t)(m > 0 ? m : 1))) : nullptr;
  DevSettings d;
  memset(&d, 0, sizeof(d));
  d.sigma = settings->sigma;
  d.rho_is_vec = rho_vec ? 1 : 0;
  d.cg_max_iter = settings->cg_max_iter;
  d.cg_tol_reduction = settings->cg_tol_reduction;
  d.cg_tol_fraction = settings->cg_tol_fraction;
  d.cg_precond = (int)settings->cg_precond;
  d.infty = (double)OSQP_INFTY;
  const int kktL = pick_lanes((long long)P->nnzS + A->nnz, n);
  // on the library's stream, which the call then waits for
  cudaStream_t st = g_ctx.stream;
  k_linsys_noalloc<<<1, kLsBlockThreads, 0, st>>>(pr, d, kktL, b->d_val, (double)settings->rho);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    fprintf(stderr, "osqp_gb300_linsys_solve_noalloc: %s\n", cudaGetErrorString(e));
    return OSQP_ALGEBRA_LOAD_ERROR;
  }
  return 0;
}
