/*
 * Test infrastructure: FP64 CPU restatement of OSQP 1.0 (oracle).
 *
 * Only tests/, the package smoke check and bench.py's CPU-baseline leg load
 * this file's library; the GB300 product never links or calls it.
 *
 * Each section names the reference code whose behaviour it restates.  The
 * restatement is pinned against the reference itself (oracle/_ref, built from
 * the reference sources) by tests/test_oracle_pin.py and the committed
 * fixtures in tests/golden/.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "osqp_oracle.h"

/* The LDL^T module is shared with the reference build (ref_compat/). */
#define OSQP_ORACLE_QDLDL_TYPES_H
typedef OSQPInt   QDLDL_int;
typedef OSQPFloat QDLDL_float;
typedef int       QDLDL_bool;
#define QDLDL_INT_MAX 2147483647
#include "ref_compat/ldl_compat.c"

/* builtin-algebra defaults (include/public/osqp_api_constants.h:111-178) */
#define ORC_RHO_IS_VEC           1
#define ORC_ADAPTIVE_RHO_TOL     5.0
#define ORC_CHECK_TERMINATION    25
#define ORC_CHECK_DUALGAP        1
#define ORC_INF                  1e30
#define ORC_DIV_TOL              (1.0 / ORC_INF)
#define ORC_ZERO_DEADZONE        1e-15

static double dmin(double a, double b) { return a < b ? a : b; }
static double dmax(double a, double b) { return a > b ? a : b; }

static double now_s(void) {
  struct timespec t;
  clock_gettime(CLOCK_MONOTONIC, &t);
  return (double)t.tv_sec + 1e-9 * (double)t.tv_nsec;
}

/* ======================================================================
 * Status / error strings (src/auxil.c:785-799, src/error.c)
 * ====================================================================== */
const char* OSQP_STATUS_MESSAGE[] = {
  "", "solved", "solved inaccurate", "primal infeasible",
  "primal infeasible inaccurate", "dual infeasible", "dual infeasible inaccurate",
  "maximum iterations reached", "run time limit reached", "problem non convex",
  "interrupted", "unsolved"
};
const char* OSQP_ERROR_MESSAGE[] = {
  "", "Problem data validation.", "Solver settings validation.",
  "Linear system solver initialization.", "KKT matrix factorization.",
  "Memory allocation.", "Solver workspace not initialized.",
  "Algebra library loading.", "File open.", "Invalid defines for codegen.",
  "Vector/matrix not initialized.", "Function not implemented."
};

/* ======================================================================
 * Compressed-column matrices (algebra/_common/csc_math.c, csc_utils.c)
 * ====================================================================== */
typedef struct { OSQPInt m, n; OSQPInt* p; OSQPInt* i; double* x; } ocsc;

static ocsc* csc_alloc(OSQPInt m, OSQPInt n, OSQPInt nnz) {
  ocsc* M = (ocsc*)calloc(1, sizeof(ocsc));
  M->m = m; M->n = n;
  M->p = (OSQPInt*)calloc((size_t)n + 1, sizeof(OSQPInt));
  M->i = (OSQPInt*)calloc((size_t)(nnz > 0 ? nnz : 1), sizeof(OSQPInt));
  M->x = (double*)calloc((size_t)(nnz > 0 ? nnz : 1), sizeof(double));
  return M;
}
static void csc_free(ocsc* M) { if (M) { free(M->p); free(M->i); free(M->x); free(M); } }
static OSQPInt csc_nnz(const ocsc* M) { return M->p[M->n]; }
static ocsc* csc_from_api(const OSQPCscMatrix* S) {
  OSQPInt nnz = S->p[S->n];
  ocsc* M = csc_alloc(S->m, S->n, nnz);
  memcpy(M->p, S->p, sizeof(OSQPInt) * ((size_t)S->n + 1));
  if (nnz) { memcpy(M->i, S->i, sizeof(OSQPInt) * nnz); memcpy(M->x, S->x, sizeof(double) * nnz); }
  return M;
}

/* y = alpha*M*x + beta*y ; sym_triu: M holds the upper triangle of a symmetric matrix */
static void csc_axpy(const ocsc* M, const double* x, double* y, double alpha, double beta, int sym_triu) {
  OSQPInt j, k, rows = M->m;
  if (beta == 0.0) { for (j = 0; j < rows; j++) y[j] = 0.0; }
  else if (beta != 1.0) { for (j = 0; j < rows; j++) y[j] *= beta; }
  for (j = 0; j < M->n; j++) {
    for (k = M->p[j]; k < M->p[j + 1]; k++) {
      OSQPInt i = M->i[k];
      y[i] += alpha * M->x[k] * x[j];
      if (sym_triu && i != j) y[j] += alpha * M->x[k] * x[i];
    }
  }
}
/* y = alpha*M'*x + beta*y */
static void csc_atxpy(const ocsc* M, const double* x, double* y, double alpha, double beta) {
  OSQPInt j, k;
  for (j = 0; j < M->n; j++) {
    double acc = 0.0;
    for (k = M->p[j]; k < M->p[j + 1]; k++) acc += M->x[k] * x[M->i[k]];
    y[j] = (beta == 0.0 ? 0.0 : beta * y[j]) + alpha * acc;
  }
}
static void csc_col_norm_inf(const ocsc* M, double* out, int sym_triu) {
  OSQPInt j, k;
  for (j = 0; j < M->n; j++) out[j] = 0.0;
  for (j = 0; j < M->n; j++) {
    for (k = M->p[j]; k < M->p[j + 1]; k++) {
      double a = fabs(M->x[k]);
      out[j] = dmax(out[j], a);
      if (sym_triu && M->i[k] != j) out[M->i[k]] = dmax(out[M->i[k]], a);
    }
  }
}
static void csc_row_norm_inf(const ocsc* M, double* out) {
  OSQPInt j, k;
  for (j = 0; j < M->m; j++) out[j] = 0.0;
  for (j = 0; j < M->n; j++)
    for (k = M->p[j]; k < M->p[j + 1]; k++) out[M->i[k]] = dmax(out[M->i[k]], fabs(M->x[k]));
}
static void csc_lmult(ocsc* M, const double* d) {
  OSQPInt k; for (k = 0; k < csc_nnz(M); k++) M->x[k] *= d[M->i[k]];
}
static void csc_rmult(ocsc* M, const double* d) {
  OSQPInt j, k;
  for (j = 0; j < M->n; j++) for (k = M->p[j]; k < M->p[j + 1]; k++) M->x[k] *= d[j];
}
static void csc_scale(ocsc* M, double s) { OSQPInt k; for (k = 0; k < csc_nnz(M); k++) M->x[k] *= s; }

/* rows of A with flag != 0, in row order (algebra/builtin/matrix.c submatrix_byrows) */
static ocsc* csc_rows(const ocsc* A, const OSQPInt* flags, OSQPInt* n_out) {
  OSQPInt r, j, k, nr = 0, cnt = 0;
  OSQPInt* map = (OSQPInt*)malloc(sizeof(OSQPInt) * (A->m > 0 ? A->m : 1));
  for (r = 0; r < A->m; r++) map[r] = flags[r] ? nr++ : -1;
  for (k = 0; k < csc_nnz(A); k++) if (map[A->i[k]] >= 0) cnt++;
  ocsc* R = csc_alloc(nr, A->n, cnt);
  cnt = 0;
  for (j = 0; j < A->n; j++) {
    R->p[j] = cnt;
    for (k = A->p[j]; k < A->p[j + 1]; k++) {
      OSQPInt mr = map[A->i[k]];
      if (mr >= 0) { R->i[cnt] = mr; R->x[cnt] = A->x[k]; cnt++; }
    }
  }
  R->p[A->n] = cnt;
  free(map);
  *n_out = nr;
  return R;
}

/* ======================================================================
 * Vector helpers (algebra/builtin/vector.c)
 * ====================================================================== */
static double* vnew(OSQPInt n) { return (double*)calloc((size_t)(n > 0 ? n : 1), sizeof(double)); }
static double vnorm_inf(const double* v, OSQPInt n) {
  double r = 0.0; OSQPInt i; for (i = 0; i < n; i++) r = dmax(r, fabs(v[i])); return r;
}
static double vscaled_norm_inf(const double* s, const double* v, OSQPInt n) {
  double r = 0.0; OSQPInt i; for (i = 0; i < n; i++) r = dmax(r, fabs(s[i] * v[i])); return r;
}
static double vdot(const double* a, const double* b, OSQPInt n) {
  double r = 0.0; OSQPInt i; for (i = 0; i < n; i++) r += a[i] * b[i]; return r;
}
/* sum a_i*max(b_i,0) (sign>0) or a_i*min(b_i,0) (sign<0); vector.c:591-617 */
static double vdot_signed(const double* a, const double* b, OSQPInt n, int sign) {
  double r = 0.0; OSQPInt i;
  for (i = 0; i < n; i++) r += a[i] * (sign > 0 ? dmax(b[i], 0.0) : dmin(b[i], 0.0));
  return r;
}
/* vector.c:676-702 */
static void vproject_polar_reccone(double* y, const double* l, const double* u, OSQPInt n, double infval) {
  OSQPInt i;
  for (i = 0; i < n; i++) {
    if (u[i] > infval) y[i] = (l[i] < -infval) ? 0.0 : dmin(y[i], 0.0);
    else if (l[i] < -infval) y[i] = dmax(y[i], 0.0);
  }
}
/* vector.c:704-727 */
static int vin_reccone(const double* y, const double* l, const double* u, OSQPInt n, double infval, double tol) {
  OSQPInt i;
  for (i = 0; i < n; i++)
    if ((u[i] < infval && y[i] > tol) || (l[i] > -infval && y[i] < -tol)) return 0;
  return 1;
}
/* constraint types: -1 loose, 1 equality, 0 inequality; vector.c:885-921 */
static int vbounds_type(OSQPInt* t, const double* l, const double* u, OSQPInt n, double tol, double infval) {
  OSQPInt i; int changed = 0;
  for (i = 0; i < n; i++) {
    OSQPInt old = t[i];
    if (l[i] < -infval && u[i] > infval) t[i] = -1;
    else if (u[i] - l[i] < tol) t[i] = 1;
    else t[i] = 0;
    changed = changed || (t[i] != old);
  }
  return changed;
}
static double limit_scaling(double v) {  /* scaling.c:8-12 */
  v = v < OSQP_MIN_SCALING ? 1.0 : v;
  return v > OSQP_MAX_SCALING ? OSQP_MAX_SCALING : v;
}

/* ======================================================================
 * Minimum-degree ordering for the KKT pattern (used by the direct solver;
 * the reference uses SuiteSparse AMD, qdldl_interface.c:137-212).  Explicit
 * elimination graph, Rose/Tinney-Walker minimum degree, ties by index.
 * ====================================================================== */
typedef struct { OSQPInt* v; OSQPInt len, cap; } ivec;
static void ivec_push(ivec* a, OSQPInt x) {
  if (a->len == a->cap) { a->cap = a->cap ? 2 * a->cap : 8; a->v = (OSQPInt*)realloc(a->v, sizeof(OSQPInt) * a->cap); }
  a->v[a->len++] = x;
}

/* K: upper-triangular CSC of the KKT matrix (N x N).  perm[k] = original index at position k. */
static void min_degree_order(const ocsc* K, OSQPInt* perm) {
  OSQPInt N = K->n, j, k, t, s;
  ivec* adj = (ivec*)calloc((size_t)N, sizeof(ivec));
  char* gone = (char*)calloc((size_t)N, 1);
  OSQPInt* mark = (OSQPInt*)malloc(sizeof(OSQPInt) * N);
  OSQPInt* nbr  = (OSQPInt*)malloc(sizeof(OSQPInt) * N);
  for (j = 0; j < N; j++) mark[j] = -1;
  for (j = 0; j < N; j++)
    for (k = K->p[j]; k < K->p[j + 1]; k++) {
      OSQPInt i = K->i[k];
      if (i != j) { ivec_push(&adj[i], j); ivec_push(&adj[j], i); }
    }
  /* Bucket structure keyed by (approximate) degree with lazy deletion */
  OSQPInt* deg = (OSQPInt*)malloc(sizeof(OSQPInt) * N);
  OSQPInt stamp_next = -2;   /* unique negative stamps, one per list rebuild */
  for (j = 0; j < N; j++) deg[j] = adj[j].len;
  for (t = 0; t < N; t++) {
    /* pick the live node of least degree (linear scan; sizes here are moderate) */
    OSQPInt best = -1, bd = 0;
    for (j = 0; j < N; j++) if (!gone[j] && (best < 0 || deg[j] < bd)) { best = j; bd = deg[j]; }
    perm[t] = best;
    gone[best] = 1;
    /* live neighbours of best, deduplicated */
    OSQPInt nn = 0;
    for (k = 0; k < adj[best].len; k++) {
      OSQPInt u = adj[best].v[k];
      if (!gone[u] && mark[u] != best) { mark[u] = best; nbr[nn++] = u; }
    }
    /* form the clique on the neighbours */
    for (s = 0; s < nn; s++) {
      OSQPInt u = nbr[s], w, cnt = 0;
      /* compact u's list to live nodes and dedupe, then add clique members */
      OSQPInt stamp = stamp_next--;
      ivec* a = &adj[u];
      OSQPInt out = 0;
      for (k = 0; k < a->len; k++) {
        w = a->v[k];
        if (!gone[w] && mark[w] != stamp) { mark[w] = stamp; a->v[out++] = w; }
      }
      a->len = out;
      for (k = 0; k < nn; k++) {
        w = nbr[k];
        if (w != u && mark[w] != stamp) { mark[w] = stamp; ivec_push(a, w); }
      }
      cnt = a->len;
      deg[u] = cnt;
      /* restore the marks of the clique so the next neighbour sees them as fresh */
      for (k = 0; k < nn; k++) mark[nbr[k]] = best;
    }
    free(adj[best].v); adj[best].v = NULL; adj[best].len = adj[best].cap = 0;
  }
  for (j = 0; j < N; j++) free(adj[j].v);
  free(adj); free(gone); free(mark); free(nbr); free(deg);
}

/* ======================================================================
 * Linear system solvers (LinSysSolver, include/private/types.h:243-279)
 * ====================================================================== */
typedef struct {
  int type;            /* OSQP_DIRECT_SOLVER / OSQP_INDIRECT_SOLVER */
  OSQPInt n, m;
  int polishing;
  double sigma;
  /* direct: permuted upper KKT + factor (qdldl_interface.c:216-526) */
  ocsc* KKT;
  OSQPInt *perm, *pinv, *rho_pos, *Pval_pos, *Aval_pos, *Pdiag_pos;
  OSQPInt *Lp, *Li, *etree, *Lnz, *iwork; int* bwork;
  double *Lx, *D, *Dinv, *fwork, *bp, *sol;
  double rho_inv; double* rho_inv_vec;
  /* indirect: reduced-KKT PCG (cuda_pcg.cu:50-285, cuda_pcg_interface.cu:32-361) */
  const ocsc* P; const ocsc* A; const double* rho_vec; double rho;
  double *x, *p, *Kp, *yv, *r, *rhs, *zt, *Pdiag, *precond_inv;
  double *binv, *bwork_m;   /* block-Jacobi (cg_precond = 2): 32 x 32 blocks, dense scatter of A columns */
  OSQPInt max_iter, reduction_threshold, zero_pcg_iters, precond_type;
  double tol_fraction, reduction_factor, eps_prev;
  const double *scaled_prim_res, *scaled_dual_res;
  OSQPInt last_pcg_iters;
} oc_ls;

/* --- direct --- */
/* KKT = [P + sigma I, A'; A, -diag(param2)] upper triangle, with index maps
 * (algebra/_common/kkt.c:293-347, form_KKT) */
static ocsc* form_kkt(const ocsc* P, const ocsc* A, double sigma, const double* p2vec, double p2,
                      OSQPInt* Pmap, OSQPInt* Amap, OSQPInt* rhomap, OSQPInt* Pdiag) {
  OSQPInt n = P->n, m = A->m, N = n + m, j, k;
  /* count entries: P upper + missing diagonals, A' entries, m diagonals */
  OSQPInt nzP = 0;
  for (j = 0; j < n; j++) {
    int has = 0;
    for (k = P->p[j]; k < P->p[j + 1]; k++) { nzP++; if (P->i[k] == j) has = 1; }
    if (!has) nzP++;
  }
  OSQPInt nnz = nzP + csc_nnz(A) + m;
  ocsc* K = csc_alloc(N, N, nnz);
  /* column counts for the A' block: column n+r holds row r of A */
  OSQPInt* cnt = (OSQPInt*)calloc((size_t)N + 1, sizeof(OSQPInt));
  for (k = 0; k < csc_nnz(A); k++) cnt[n + A->i[k]]++;
  OSQPInt pos = 0;
  for (j = 0; j < n; j++) {
    K->p[j] = pos;
    int has = 0;
    for (k = P->p[j]; k < P->p[j + 1]; k++) {
      K->i[pos] = P->i[k];
      K->x[pos] = P->x[k] + (P->i[k] == j ? sigma : 0.0);
      if (Pmap) Pmap[k] = pos;
      if (P->i[k] == j) { has = 1; if (Pdiag) Pdiag[j] = pos; }
      pos++;
    }
    if (!has) { K->i[pos] = j; K->x[pos] = sigma; if (Pdiag) Pdiag[j] = pos; pos++; }
  }
  /* A' block columns: fill order by column of A */
  OSQPInt* start = (OSQPInt*)malloc(sizeof(OSQPInt) * ((size_t)m + 1));
  OSQPInt acc = pos;
  for (j = 0; j < m; j++) { start[j] = acc; acc += cnt[n + j] + 1; }
  for (j = 0; j < m; j++) K->p[n + j] = start[j];
  K->p[N] = acc;
  OSQPInt* fill = (OSQPInt*)malloc(sizeof(OSQPInt) * ((size_t)m + 1));
  for (j = 0; j < m; j++) fill[j] = start[j];
  for (j = 0; j < n; j++)
    for (k = A->p[j]; k < A->p[j + 1]; k++) {
      OSQPInt r = A->i[k];
      K->i[fill[r]] = j; K->x[fill[r]] = A->x[k];
      if (Amap) Amap[k] = fill[r];
      fill[r]++;
    }
  for (j = 0; j < m; j++) {
    K->i[fill[j]] = n + j;
    K->x[fill[j]] = -(p2vec ? p2vec[j] : p2);
    if (rhomap) rhomap[j] = fill[j];
  }
  free(cnt); free(start); free(fill);
  return K;
}

/* Permute the upper-triangular KKT: K' = K(perm,perm), kept upper (qdldl_interface.c permute_KKT) */
static ocsc* permute_upper(const ocsc* K, const OSQPInt* pinv, OSQPInt* map) {
  OSQPInt N = K->n, j, k, nnz = csc_nnz(K);
  ocsc* C = csc_alloc(N, N, nnz);
  OSQPInt* cnt = (OSQPInt*)calloc((size_t)N + 1, sizeof(OSQPInt));
  for (j = 0; j < N; j++)
    for (k = K->p[j]; k < K->p[j + 1]; k++) {
      OSQPInt a = pinv[K->i[k]], b = pinv[j];
      cnt[a > b ? a : b]++;
    }
  C->p[0] = 0;
  for (j = 0; j < N; j++) C->p[j + 1] = C->p[j] + cnt[j];
  for (j = 0; j < N; j++) cnt[j] = C->p[j];
  for (j = 0; j < N; j++)
    for (k = K->p[j]; k < K->p[j + 1]; k++) {
      OSQPInt a = pinv[K->i[k]], b = pinv[j];
      OSQPInt col = a > b ? a : b, row = a > b ? b : a;
      OSQPInt q = cnt[col]++;
      C->i[q] = row; C->x[q] = K->x[k];
      map[k] = q;
    }
  free(cnt);
  return C;
}

static int direct_factor(oc_ls* s) {
  OSQPInt N = s->n + s->m;
  OSQPInt r = QDLDL_factor(N, s->KKT->p, s->KKT->i, s->KKT->x, s->Lp, s->Li, s->Lx, s->D, s->Dinv,
                           s->Lnz, s->etree, s->bwork, s->iwork, s->fwork);
  if (r < 0) return -1;
  if (r < s->n) return -2;
  return 0;
}

static void ls_free(oc_ls* s);

static int direct_init(oc_ls* s, const ocsc* P, const ocsc* A, const double* rho_vec, double rho, double sigma) {
  OSQPInt n = P->n, m = A->m, N = n + m, k;
  OSQPInt* Pmap = (OSQPInt*)malloc(sizeof(OSQPInt) * (csc_nnz(P) + 1));
  OSQPInt* Amap = (OSQPInt*)malloc(sizeof(OSQPInt) * (csc_nnz(A) + 1));
  OSQPInt* rmap = (OSQPInt*)malloc(sizeof(OSQPInt) * (m + 1));
  OSQPInt* Pdg  = (OSQPInt*)malloc(sizeof(OSQPInt) * (n + 1));
  double p2 = 0.0;
  if (s->polishing) { p2 = sigma; }
  else if (rho_vec) {
    s->rho_inv_vec = vnew(m);
    for (k = 0; k < m; k++) s->rho_inv_vec[k] = 1.0 / rho_vec[k];
  } else { s->rho_inv = 1.0 / rho; p2 = s->rho_inv; }
  ocsc* K0 = form_kkt(P, A, sigma, s->polishing ? NULL : s->rho_inv_vec, p2, Pmap, Amap, rmap, Pdg);
  s->perm = (OSQPInt*)malloc(sizeof(OSQPInt) * N);
  s->pinv = (OSQPInt*)malloc(sizeof(OSQPInt) * N);
  min_degree_order(K0, s->perm);
  for (k = 0; k < N; k++) s->pinv[s->perm[k]] = k;
  OSQPInt* kmap = (OSQPInt*)malloc(sizeof(OSQPInt) * (csc_nnz(K0) + 1));
  s->KKT = permute_upper(K0, s->pinv, kmap);
  s->Pval_pos = (OSQPInt*)malloc(sizeof(OSQPInt) * (csc_nnz(P) + 1));
  s->Aval_pos = (OSQPInt*)malloc(sizeof(OSQPInt) * (csc_nnz(A) + 1));
  s->rho_pos  = (OSQPInt*)malloc(sizeof(OSQPInt) * (m + 1));
  s->Pdiag_pos = (OSQPInt*)malloc(sizeof(OSQPInt) * (n + 1));
  for (k = 0; k < csc_nnz(P); k++) s->Pval_pos[k] = kmap[Pmap[k]];
  for (k = 0; k < csc_nnz(A); k++) s->Aval_pos[k] = kmap[Amap[k]];
  for (k = 0; k < m; k++) s->rho_pos[k] = kmap[rmap[k]];
  for (k = 0; k < n; k++) s->Pdiag_pos[k] = kmap[Pdg[k]];
  csc_free(K0); free(kmap); free(Pmap); free(Amap); free(rmap); free(Pdg);

  s->etree = (OSQPInt*)malloc(sizeof(OSQPInt) * N);
  s->Lnz   = (OSQPInt*)malloc(sizeof(OSQPInt) * N);
  s->iwork = (OSQPInt*)malloc(sizeof(OSQPInt) * 3 * N);
  s->bwork = (int*)malloc(sizeof(int) * N);
  s->fwork = vnew(N);
  s->Lp = (OSQPInt*)malloc(sizeof(OSQPInt) * (N + 1));
  OSQPInt lnz = QDLDL_etree(N, s->KKT->p, s->KKT->i, s->iwork, s->Lnz, s->etree);
  if (lnz < 0) return OSQP_LINSYS_SOLVER_INIT_ERROR;
  s->Li = (OSQPInt*)malloc(sizeof(OSQPInt) * (lnz + 1));
  s->Lx = vnew(lnz + 1);
  s->D = vnew(N); s->Dinv = vnew(N); s->bp = vnew(N); s->sol = vnew(N);
  if (direct_factor(s) < 0) return OSQP_NONCVX_ERROR;
  return 0;
}

static void ldl_solve_perm(oc_ls* s, double* x, const double* b) {
  OSQPInt N = s->n + s->m, j;
  for (j = 0; j < N; j++) s->bp[j] = b[s->perm[j]];
  QDLDL_solve(N, s->Lp, s->Li, s->Lx, s->Dinv, s->bp);
  for (j = 0; j < N; j++) x[s->perm[j]] = s->bp[j];
}

/* qdldl_interface.c:418-461 */
static void direct_solve(oc_ls* s, double* b) {
  OSQPInt j, n = s->n, m = s->m;
  if (s->polishing) { ldl_solve_perm(s, b, b); return; }
  ldl_solve_perm(s, s->sol, b);
  for (j = 0; j < n; j++) b[j] = s->sol[j];
  for (j = 0; j < m; j++) b[n + j] += (s->rho_inv_vec ? s->rho_inv_vec[j] : s->rho_inv) * s->sol[n + j];
}

/* --- indirect: reduced KKT  K = P + sigma I + A' diag(rho) A --- */
static void pcg_rho_apply(const oc_ls* s, double* v) {
  OSQPInt j;
  if (s->rho_vec) for (j = 0; j < s->m; j++) v[j] *= s->rho_vec[j];
  else            for (j = 0; j < s->m; j++) v[j] *= s->rho;
}
/* cuda_pcg.cu:50-106 */
static void pcg_matvec(oc_ls* s, const double* x, double* y) {
  OSQPInt j;
  for (j = 0; j < s->n; j++) y[j] = s->sigma * x[j];
  csc_axpy(s->P, x, y, 1.0, 1.0, 1);
  if (s->m == 0) return;
  csc_axpy(s->A, x, s->zt, 1.0, 0.0, 0);
  pcg_rho_apply(s, s->zt);
  csc_atxpy(s->A, s->zt, y, 1.0, 1.0);
}
/* Block-Jacobi preconditioner of the GB300 solver (cg_precond = 2; the
 * reference's PCG has the diagonal one only).  Blocks are the variables
 * [32 b, 32 b + 32); block b of M^-1 = inverse of the block of
 * K = P + sigma I + A' R A, stored densely at binv + 1024 b (row-major, the
 * block is symmetric).  Inverted through a Cholesky factorisation; a block
 * with a non-positive pivot keeps 1 / K_ii on its diagonal. */
#define OC_PBLK 32
static void pcg_block_precond(oc_ls* s) {
  OSQPInt n = s->n, b, nblk = (n + OC_PBLK - 1) / OC_PBLK;
  double K[OC_PBLK][OC_PBLK], L[OC_PBLK][OC_PBLK], W[OC_PBLK][OC_PBLK];
  for (b = 0; b < nblk; b++) {
    OSQPInt i0 = b * OC_PBLK, nb = (n - i0 < OC_PBLK) ? n - i0 : OC_PBLK, a, c, k, e;
    double* Bb = s->binv + (size_t)b * OC_PBLK * OC_PBLK;
    int ok = 1;
    memset(K, 0, sizeof(K));
    /* P from its upper triangle */
    for (c = 0; c < nb; c++)
      for (k = s->P->p[i0 + c]; k < s->P->p[i0 + c + 1]; k++) {
        OSQPInt r = s->P->i[k] - i0;
        if (r < 0 || r >= nb) continue;
        K[r][c] += s->P->x[k];
        if (r != c) K[c][r] += s->P->x[k];
      }
    /* A' R A: column c of A scattered densely, dotted with columns a >= c */
    for (c = 0; c < nb; c++) {
      for (k = s->A->p[i0 + c]; k < s->A->p[i0 + c + 1]; k++) s->bwork_m[s->A->i[k]] = s->A->x[k];
      for (a = c; a < nb; a++) {
        double d = 0.0;
        for (e = s->A->p[i0 + a]; e < s->A->p[i0 + a + 1]; e++) {
          OSQPInt row = s->A->i[e];
          double rr = s->rho_vec ? s->rho_vec[row] : s->rho;
          d += rr * s->bwork_m[row] * s->A->x[e];
        }
        K[a][c] += d;
        if (a != c) K[c][a] += d;
      }
      for (k = s->A->p[i0 + c]; k < s->A->p[i0 + c + 1]; k++) s->bwork_m[s->A->i[k]] = 0.0;
    }
    for (c = 0; c < nb; c++) K[c][c] += s->sigma;
    /* K = L L' */
    memset(L, 0, sizeof(L));
    for (c = 0; c < nb && ok; c++) {
      double d = K[c][c];
      for (k = 0; k < c; k++) d -= L[c][k] * L[c][k];
      if (!(d > 0.0) || !isfinite(d)) { ok = 0; break; }
      L[c][c] = sqrt(d);
      for (a = c + 1; a < nb; a++) {
        double v = K[a][c];
        for (k = 0; k < c; k++) v -= L[a][k] * L[c][k];
        L[a][c] = v / L[c][c];
      }
    }
    memset(Bb, 0, sizeof(double) * OC_PBLK * OC_PBLK);
    if (!ok) {
      for (c = 0; c < nb; c++) Bb[c * OC_PBLK + c] = 1.0 / K[c][c];
      continue;
    }
    /* W = L^-1 (forward substitution on unit vectors), M^-1 = W' W */
    memset(W, 0, sizeof(W));
    for (c = 0; c < nb; c++)
      for (a = c; a < nb; a++) {
        double v = (a == c) ? 1.0 : 0.0;
        for (k = c; k < a; k++) v -= L[a][k] * W[k][c];
        W[a][c] = v / L[a][a];
      }
    for (a = 0; a < nb; a++)
      for (c = 0; c < nb; c++) {
        double v = 0.0;
        for (k = (a > c ? a : c); k < nb; k++) v += W[k][a] * W[k][c];
        Bb[a * OC_PBLK + c] = v;
      }
  }
}
static void pcg_block_apply(const oc_ls* s, const double* r, double* y) {
  OSQPInt n = s->n, i, j;
  for (i = 0; i < n; i++) {
    OSQPInt b0 = i - i % OC_PBLK, nb = (n - b0 < OC_PBLK) ? n - b0 : OC_PBLK;
    const double* row = s->binv + (size_t)b0 * OC_PBLK + (size_t)(i - b0) * OC_PBLK;
    double v = 0.0;
    for (j = 0; j < nb; j++) v += row[j] * r[b0 + j];
    y[i] = v;
  }
}

/* cuda_pcg.cu:211-285 */
static void pcg_update_precond(oc_ls* s) {
  OSQPInt j, k;
  if (s->precond_type == 2) {
    if (!s->binv) {
      s->binv = vnew(((s->n + OC_PBLK - 1) / OC_PBLK) * OC_PBLK * OC_PBLK);
      s->bwork_m = vnew(s->m > 0 ? s->m : 1);
    }
    pcg_block_precond(s);
  }
  if (s->precond_type == OSQP_NO_PRECONDITIONER) {
    for (j = 0; j < s->n; j++) s->precond_inv[j] = 1.0;
    return;
  }
  for (j = 0; j < s->n; j++) s->Pdiag[j] = 0.0;
  for (j = 0; j < s->n; j++)
    for (k = s->P->p[j]; k < s->P->p[j + 1]; k++) if (s->P->i[k] == j) s->Pdiag[j] += s->P->x[k];
  for (j = 0; j < s->n; j++) {
    double d = 0.0;
    for (k = s->A->p[j]; k < s->A->p[j + 1]; k++) {
      double rr = s->rho_vec ? s->rho_vec[s->A->i[k]] : s->rho;
      d += s->A->x[k] * s->A->x[k] * rr;
    }
    s->precond_inv[j] = 1.0 / (s->sigma + s->Pdiag[j] + d);
  }
}
/* cuda_pcg_interface.cu:32-64 */
static double pcg_tolerance(oc_ls* s, OSQPInt admm_iter) {
  double rn = vnorm_inf(s->rhs, s->n), eps;
  if (s->polishing) return dmax(rn * OSQP_CG_POLISH_TOL, OSQP_CG_TOL_MIN);
  if (admm_iter == 1) {
    s->reduction_factor = s->tol_fraction;
    s->eps_prev = (rn < OSQP_CG_TOL_MIN) ? 1.0 : rn * s->reduction_factor;
    return s->eps_prev;
  }
  if (s->zero_pcg_iters >= s->reduction_threshold) {
    s->reduction_factor /= 2;
    s->zero_pcg_iters = 0;
  }
  eps = s->reduction_factor * sqrt((*s->scaled_prim_res) * (*s->scaled_dual_res));
  eps = dmax(dmin(eps, s->eps_prev), OSQP_CG_TOL_MIN);
  s->eps_prev = eps;
  return eps;
}
/* cuda_pcg.cu:113-208 (warm-started x, inf-norm stopping) */
static OSQPInt pcg_run(oc_ls* s, double eps) {
  OSQPInt n = s->n, j, it = 0;
  double rTy, rTy_prev, pKp, alpha, beta, rnorm;
  pcg_matvec(s, s->x, s->r);
  for (j = 0; j < n; j++) s->r[j] -= s->rhs[j];
  rnorm = vnorm_inf(s->r, n);
  if (s->precond_type == 2) pcg_block_apply(s, s->r, s->yv);
  else for (j = 0; j < n; j++) s->yv[j] = s->precond_inv[j] * s->r[j];
  for (j = 0; j < n; j++) s->p[j] = -s->yv[j];
  rTy = vdot(s->yv, s->r, n);
  while (rnorm > eps && it < s->max_iter) {
    pcg_matvec(s, s->p, s->Kp);
    pKp = vdot(s->p, s->Kp, n);
    alpha = rTy / pKp;
    for (j = 0; j < n; j++) { s->x[j] += alpha * s->p[j]; s->r[j] += alpha * s->Kp[j]; }
    if (s->precond_type == 2) pcg_block_apply(s, s->r, s->yv);
    else for (j = 0; j < n; j++) s->yv[j] = s->precond_inv[j] * s->r[j];
    rTy_prev = rTy;
    rTy = vdot(s->yv, s->r, n);
    rnorm = vnorm_inf(s->r, n);
    beta = rTy / rTy_prev;
    for (j = 0; j < n; j++) s->p[j] = beta * s->p[j] - s->yv[j];
    it++;
  }
  return it;
}
/* cuda_pcg_interface.cu:229-273 */
static void indirect_solve(oc_ls* s, double* b, OSQPInt admm_iter) {
  OSQPInt n = s->n, m = s->m, j, it;
  double eps;
  for (j = 0; j < n; j++) s->rhs[j] = b[j];
  if (m) {
    for (j = 0; j < m; j++) s->zt[j] = b[n + j];
    pcg_rho_apply(s, s->zt);
    csc_atxpy(s->A, s->zt, s->rhs, 1.0, 1.0);
  }
  eps = pcg_tolerance(s, admm_iter);
  it = pcg_run(s, eps);
  s->last_pcg_iters = it;
  for (j = 0; j < n; j++) b[j] = s->x[j];
  if (m) {
    if (!s->polishing) {
      csc_axpy(s->A, s->x, b + n, 1.0, 0.0, 0);
    } else {
      csc_axpy(s->A, s->x, s->zt, 1.0, 0.0, 0);
      for (j = 0; j < m; j++) b[n + j] = (s->zt[j] - b[n + j]) * s->rho;
    }
  }
  if (it == 0) s->zero_pcg_iters++; else s->zero_pcg_iters = 0;
}

static int ls_init(oc_ls** out, const ocsc* P, const ocsc* A, const double* rho_vec, double rho,
                   const OSQPSettings* st, const double* spr, const double* sdr, int polishing) {
  oc_ls* s = (oc_ls*)calloc(1, sizeof(oc_ls));
  int rc = 0;
  *out = s;
  s->type = st->linsys_solver;
  s->n = P->n; s->m = A->m; s->polishing = polishing;
  s->sigma = polishing ? st->delta : st->sigma;
  if (s->type == OSQP_DIRECT_SOLVER) {
    rc = direct_init(s, P, A, polishing ? NULL : rho_vec, rho, s->sigma);
  } else {
    s->P = P; s->A = A;
    s->rho_vec = polishing ? NULL : rho_vec;
    s->rho = polishing ? 1.0 / st->delta : rho;
    s->x = vnew(s->n); s->p = vnew(s->n); s->Kp = vnew(s->n); s->yv = vnew(s->n);
    s->r = vnew(s->n); s->rhs = vnew(s->n); s->zt = vnew(s->m);
    s->Pdiag = vnew(s->n); s->precond_inv = vnew(s->n);
    s->max_iter = st->cg_max_iter; s->reduction_threshold = st->cg_tol_reduction;
    s->tol_fraction = st->cg_tol_fraction; s->reduction_factor = st->cg_tol_fraction;
    s->precond_type = st->cg_precond;
    /* the GB300 polish runs its PCG with the diagonal preconditioner */
    if (polishing && s->precond_type == 2) s->precond_type = OSQP_DIAGONAL_PRECONDITIONER;
    s->scaled_prim_res = spr; s->scaled_dual_res = sdr;
    pcg_update_precond(s);
  }
  return rc;
}
static void ls_solve(oc_ls* s, double* b, OSQPInt admm_iter) {
  if (s->type == OSQP_DIRECT_SOLVER) direct_solve(s, b); else indirect_solve(s, b, admm_iter);
}
static void ls_warm_start(oc_ls* s, const double* x) {
  if (s->type == OSQP_INDIRECT_SOLVER) memcpy(s->x, x, sizeof(double) * s->n);
}
/* qdldl_interface.c:496-526 / cuda_pcg_interface.cu:352-361 */
static int ls_update_rho(oc_ls* s, const double* rho_vec, double rho_sc) {
  OSQPInt j;
  if (s->type == OSQP_DIRECT_SOLVER) {
    if (s->rho_inv_vec) for (j = 0; j < s->m; j++) s->rho_inv_vec[j] = 1.0 / rho_vec[j];
    else s->rho_inv = 1.0 / rho_sc;
    for (j = 0; j < s->m; j++)
      s->KKT->x[s->rho_pos[j]] = -(s->rho_inv_vec ? s->rho_inv_vec[j] : s->rho_inv);
    return direct_factor(s) == -1;
  }
  s->rho = rho_sc;
  pcg_update_precond(s);
  return 0;
}
/* qdldl_interface.c:468-494 / cuda_pcg_interface.cu:337-349 (full value refresh) */
static int ls_update_matrices(oc_ls* s, const ocsc* P, const ocsc* A) {
  OSQPInt k;
  if (s->type == OSQP_DIRECT_SOLVER) {
    for (k = 0; k < s->n; k++) s->KKT->x[s->Pdiag_pos[k]] = s->sigma;
    /* rewrite values: diagonal entries keep sigma added */
    for (k = 0; k < csc_nnz(P); k++) s->KKT->x[s->Pval_pos[k]] = 0.0;
    for (k = 0; k < s->n; k++) s->KKT->x[s->Pdiag_pos[k]] = s->sigma;
    for (k = 0; k < csc_nnz(P); k++) s->KKT->x[s->Pval_pos[k]] += P->x[k];
    for (k = 0; k < csc_nnz(A); k++) s->KKT->x[s->Aval_pos[k]] = A->x[k];
    return direct_factor(s) == 0 ? 0 : 1;
  }
  pcg_update_precond(s);
  return 0;
}
static void ls_free(oc_ls* s) {
  if (!s) return;
  csc_free(s->KKT);
  free(s->perm); free(s->pinv); free(s->rho_pos); free(s->Pval_pos); free(s->Aval_pos); free(s->Pdiag_pos);
  free(s->Lp); free(s->Li); free(s->etree); free(s->Lnz); free(s->iwork); free(s->bwork);
  free(s->Lx); free(s->D); free(s->Dinv); free(s->fwork); free(s->bp); free(s->sol); free(s->rho_inv_vec);
  free(s->x); free(s->p); free(s->Kp); free(s->yv); free(s->r); free(s->rhs); free(s->zt);
  free(s->Pdiag); free(s->precond_inv); free(s->binv); free(s->bwork_m);
  free(s);
}

/* ======================================================================
 * Workspace (include/private/types.h:99-238)
 * ====================================================================== */
struct OSQPWorkspace_ {
  OSQPInt n, m;
  ocsc *P, *A;
  double *q, *l, *u;
  double *rho_vec, *rho_inv_vec; OSQPInt* constr_type; double rho_inv;
  double *x, *y, *z, *xz, *x_prev, *z_prev;
  double *Ax, *Px, *Aty, *delta_y, *Atdelta_y, *delta_x, *Pdelta_x, *Adelta_x;
  double *D_temp, *D_temp_A, *E_temp;
  int scaled; double *D, *Dinv, *E, *Einv, c, cinv;
  double xtPx, qtx, SC, scaled_dual_gap, scaled_prim_res, scaled_dual_res;
  oc_ls* ls;
  /* polish */
  OSQPInt* active; double *pol_x, *pol_z, *pol_y; OSQPInt n_active;
  double pol_obj, pol_dobj, pol_gap, pol_prim, pol_dual;
  /* timing */
  double t0; int first_run, clear_update_time, rho_update_from_solve;
  int rho_updated; double last_rel_kkt;
  OSQPInt pcg_iters_total;
};

static void update_status(OSQPInfo* info, OSQPInt s) {
  info->status_val = s;
  strncpy(info->status, OSQP_STATUS_MESSAGE[s], 31);
  info->status[31] = 0;
}

/* ---- scaling (src/scaling.c:48-208) ----
 * Column inf-norms of P: the builtin algebra takes them over the stored upper
 * triangle only (algebra/builtin/matrix.c:194-197 -> csc_col_norm_inf), the
 * CUDA algebra over the full symmetric matrix (algebra/cuda/matrix.cu:130-135).
 * The direct mode restates the builtin backend, the indirect mode the CUDA one. */
static void scale_data(OSQPSolver* solver) {
  OSQPWorkspace* w = solver->work;
  OSQPInt n = w->n, m = w->m, i, k;
  const int sym = solver->settings->linsys_solver == OSQP_INDIRECT_SOLVER;
  w->c = 1.0;
  for (k = 0; k < n; k++) { w->D[k] = 1.0; w->Dinv[k] = 1.0; }
  for (k = 0; k < m; k++) { w->E[k] = 1.0; w->Einv[k] = 1.0; }
  for (i = 0; i < solver->settings->scaling; i++) {
    csc_col_norm_inf(w->P, w->D_temp, sym);
    csc_col_norm_inf(w->A, w->D_temp_A, 0);
    for (k = 0; k < n; k++) w->D_temp[k] = dmax(w->D_temp[k], w->D_temp_A[k]);
    csc_row_norm_inf(w->A, w->E_temp);
    for (k = 0; k < n; k++) w->D_temp[k] = 1.0 / sqrt(limit_scaling(w->D_temp[k]));
    for (k = 0; k < m; k++) w->E_temp[k] = 1.0 / sqrt(limit_scaling(w->E_temp[k]));
    csc_lmult(w->P, w->D_temp); csc_rmult(w->P, w->D_temp);
    csc_lmult(w->A, w->E_temp); csc_rmult(w->A, w->D_temp);
    for (k = 0; k < n; k++) { w->q[k] *= w->D_temp[k]; w->D[k] *= w->D_temp[k]; }
    for (k = 0; k < m; k++) w->E[k] *= w->E_temp[k];
    csc_col_norm_inf(w->P, w->D_temp, sym);
    double ct = 0.0;
    for (k = 0; k < n; k++) ct += fabs(w->D_temp[k]);
    ct /= n;
    double nq = limit_scaling(vnorm_inf(w->q, n));
    ct = limit_scaling(dmax(ct, nq));
    ct = 1.0 / ct;
    csc_scale(w->P, ct);
    for (k = 0; k < n; k++) w->q[k] *= ct;
    w->c *= ct;
  }
  w->cinv = 1.0 / w->c;
  for (k = 0; k < n; k++) w->Dinv[k] = 1.0 / w->D[k];
  for (k = 0; k < m; k++) { w->Einv[k] = 1.0 / w->E[k]; w->l[k] *= w->E[k]; w->u[k] *= w->E[k]; }
}
static void unscale_data(OSQPSolver* solver) {
  OSQPWorkspace* w = solver->work;
  OSQPInt k;
  csc_scale(w->P, w->cinv);
  csc_lmult(w->P, w->Dinv); csc_rmult(w->P, w->Dinv);
  for (k = 0; k < w->n; k++) w->q[k] = w->q[k] * w->cinv * w->Dinv[k];
  csc_lmult(w->A, w->Einv); csc_rmult(w->A, w->Dinv);
  for (k = 0; k < w->m; k++) { w->l[k] *= w->Einv[k]; w->u[k] *= w->Einv[k]; }
}

/* ---- rho vector (src/auxil.c:76-122) ---- */
static int set_rho_vec(OSQPSolver* solver) {
  OSQPWorkspace* w = solver->work;
  OSQPSettings* st = solver->settings;
  OSQPInt k;
  st->rho = dmin(dmax(st->rho, OSQP_RHO_MIN), OSQP_RHO_MAX);
  int changed = vbounds_type(w->constr_type, w->l, w->u, w->m, OSQP_RHO_TOL, ORC_INF * OSQP_MIN_SCALING);
  for (k = 0; k < w->m; k++) {
    w->rho_vec[k] = w->constr_type[k] < 0 ? OSQP_RHO_MIN
                  : (w->constr_type[k] == 0 ? st->rho : OSQP_RHO_EQ_OVER_RHO_INEQ * st->rho);
    w->rho_inv_vec[k] = 1.0 / w->rho_vec[k];
  }
  return changed;
}

/* ---- residuals, objective, termination (src/auxil.c:231-945) ---- */
static void obj_val_dual_gap(OSQPSolver* solver, const double* x, const double* y,
                             double* pobj, double* dobj, double* gap) {
  OSQPWorkspace* w = solver->work;
  OSQPInt k, m = w->m;
  double quad = vdot(w->Px, x, w->n), lin = vdot(w->q, x, w->n), sup;
  memcpy(w->z_prev, y, sizeof(double) * m);
  vproject_polar_reccone(w->z_prev, w->l, w->u, m, ORC_INF * OSQP_MIN_SCALING);
  for (k = 0; k < m; k++) if (fabs(w->z_prev[k]) < ORC_ZERO_DEADZONE) w->z_prev[k] = 0.0;
  sup = vdot_signed(w->u, w->z_prev, m, +1) + vdot_signed(w->l, w->z_prev, m, -1);
  *pobj = 0.5 * quad + lin;
  *dobj = -0.5 * quad - sup;
  w->scaled_dual_gap = quad + lin + sup;
  if (solver->settings->scaling) {
    *pobj *= w->cinv; *dobj *= w->cinv; *gap = w->cinv * w->scaled_dual_gap;
  } else *gap = w->scaled_dual_gap;
  w->xtPx = quad; w->qtx = lin; w->SC = sup;
}
static int unscaled_term(const OSQPSolver* s) { return s->settings->scaling && !s->settings->scaled_termination; }

static double prim_res(OSQPSolver* solver, const double* x, const double* z) {
  OSQPWorkspace* w = solver->work;
  OSQPInt k;
  csc_axpy(w->A, x, w->Ax, 1.0, 0.0, 0);
  for (k = 0; k < w->m; k++) w->z_prev[k] = w->Ax[k] - z[k];
  w->scaled_prim_res = vnorm_inf(w->z_prev, w->m);
  return unscaled_term(solver) ? vscaled_norm_inf(w->Einv, w->z_prev, w->m) : w->scaled_prim_res;
}
static double dual_res(OSQPSolver* solver, const double* x, const double* y) {
  OSQPWorkspace* w = solver->work;
  OSQPInt k;
  memcpy(w->x_prev, w->q, sizeof(double) * w->n);
  csc_axpy(w->P, x, w->Px, 1.0, 0.0, 1);
  for (k = 0; k < w->n; k++) w->x_prev[k] += w->Px[k];
  if (w->m) {
    csc_atxpy(w->A, y, w->Aty, 1.0, 0.0);
    for (k = 0; k < w->n; k++) w->x_prev[k] += w->Aty[k];
  }
  w->scaled_dual_res = vnorm_inf(w->x_prev, w->n);
  return unscaled_term(solver) ? w->cinv * vscaled_norm_inf(w->Dinv, w->x_prev, w->n) : w->scaled_dual_res;
}
static double prim_tol(OSQPSolver* solver, double ea, double er) {
  OSQPWorkspace* w = solver->work;
  double r;
  if (unscaled_term(solver))
    r = dmax(vscaled_norm_inf(w->Einv, w->z, w->m), vscaled_norm_inf(w->Einv, w->Ax, w->m));
  else r = dmax(vnorm_inf(w->z, w->m), vnorm_inf(w->Ax, w->m));
  return ea + er * r;
}
static double dual_tol(OSQPSolver* solver, double ea, double er) {
  OSQPWorkspace* w = solver->work;
  double r;
  if (unscaled_term(solver)) {
    r = dmax(vscaled_norm_inf(w->Dinv, w->q, w->n), vscaled_norm_inf(w->Dinv, w->Aty, w->n));
    r = dmax(r, vscaled_norm_inf(w->Dinv, w->Px, w->n));
    r *= w->cinv;
  } else {
    r = dmax(dmax(vnorm_inf(w->q, w->n), vnorm_inf(w->Aty, w->n)), vnorm_inf(w->Px, w->n));
  }
  return ea + er * r;
}
static double gap_tol(OSQPSolver* solver, double ea, double er) {
  OSQPWorkspace* w = solver->work;
  double r = dmax(dmax(fabs(w->xtPx), fabs(w->qtx)), fabs(w->SC));
  if (unscaled_term(solver)) r *= w->cinv;
  return ea + er * r;
}
static int primal_infeasible(OSQPSolver* solver, double eps) {
  OSQPWorkspace* w = solver->work;
  OSQPInt k;
  double nrm, lhs;
  vproject_polar_reccone(w->delta_y, w->l, w->u, w->m, ORC_INF * OSQP_MIN_SCALING);
  if (unscaled_term(solver)) {
    for (k = 0; k < w->m; k++) w->Adelta_x[k] = w->E[k] * w->delta_y[k];
    nrm = vnorm_inf(w->Adelta_x, w->m);
  } else nrm = vnorm_inf(w->delta_y, w->m);
  if (nrm > ORC_DIV_TOL) {
    lhs = vdot_signed(w->u, w->delta_y, w->m, +1) + vdot_signed(w->l, w->delta_y, w->m, -1);
    if (lhs < 0.0) {
      csc_atxpy(w->A, w->delta_y, w->Atdelta_y, 1.0, 0.0);
      if (unscaled_term(solver)) for (k = 0; k < w->n; k++) w->Atdelta_y[k] *= w->Dinv[k];
      return vnorm_inf(w->Atdelta_y, w->n) < eps * nrm;
    }
  }
  return 0;
}
static int dual_infeasible(OSQPSolver* solver, double eps) {
  OSQPWorkspace* w = solver->work;
  OSQPInt k;
  double nrm, cs;
  if (unscaled_term(solver)) { nrm = vscaled_norm_inf(w->D, w->delta_x, w->n); cs = w->c; }
  else { nrm = vnorm_inf(w->delta_x, w->n); cs = 1.0; }
  if (nrm > ORC_DIV_TOL) {
    if (vdot(w->q, w->delta_x, w->n) < 0.0) {
      csc_axpy(w->P, w->delta_x, w->Pdelta_x, 1.0, 0.0, 1);
      if (unscaled_term(solver)) for (k = 0; k < w->n; k++) w->Pdelta_x[k] *= w->Dinv[k];
      if (vnorm_inf(w->Pdelta_x, w->n) < cs * eps * nrm) {
        csc_axpy(w->A, w->delta_x, w->Adelta_x, 1.0, 0.0, 0);
        if (unscaled_term(solver)) for (k = 0; k < w->m; k++) w->Adelta_x[k] *= w->Einv[k];
        return vin_reccone(w->Adelta_x, w->l, w->u, w->m, ORC_INF * OSQP_MIN_SCALING, eps * nrm);
      }
    }
  }
  return 0;
}

static void update_info(OSQPSolver* solver, OSQPInt iter, int polishing) {
  OSQPWorkspace* w = solver->work;
  OSQPInfo* info = solver->info;
  const double *x, *y, *z;
  double *po, *dob, *gap, *pr, *dr;
  if (polishing) {
    x = w->pol_x; y = w->pol_y; z = w->pol_z;
    po = &w->pol_obj; dob = &w->pol_dobj; gap = &w->pol_gap; pr = &w->pol_prim; dr = &w->pol_dual;
  } else {
    x = w->x; y = w->y; z = w->z;
    po = &info->obj_val; dob = &info->dual_obj_val; gap = &info->duality_gap;
    pr = &info->prim_res; dr = &info->dual_res;
    info->iter = iter;
  }
  *pr = (w->m == 0) ? 0.0 : prim_res(solver, x, z);
  *dr = dual_res(solver, x, y);
  obj_val_dual_gap(solver, x, y, po, dob, gap);
  if (!polishing) info->primdual_int += fabs(*gap);
  if (polishing) info->polish_time = now_s() - w->t0;
  else info->solve_time = now_s() - w->t0;
  info->rel_kkt_error = dmax(dmax(*dr, *pr), *gap);
}

static int check_termination(OSQPSolver* solver, int approximate) {
  OSQPWorkspace* w = solver->work;
  OSQPInfo* info = solver->info;
  OSQPSettings* st = solver->settings;
  double ea = st->eps_abs, er = st->eps_rel, epi = st->eps_prim_inf, edi = st->eps_dual_inf;
  int prc = 0, drc = 0, pic = 0, dic = 0, gc = 0;
  OSQPInt k;
  if (info->prim_res > ORC_INF || info->dual_res > ORC_INF) {
    update_status(info, OSQP_NON_CVX);
    info->obj_val = NAN;
    return 1;
  }
  if (approximate) { ea *= 10; er *= 10; epi *= 10; edi *= 10; }
  if (w->m == 0) prc = 1;
  else {
    if (info->prim_res < prim_tol(solver, ea, er)) prc = 1;
    else pic = primal_infeasible(solver, epi);
  }
  if (info->dual_res < dual_tol(solver, ea, er)) drc = 1;
  else dic = dual_infeasible(solver, edi);
  if (st->check_dualgap) {
    double gt = gap_tol(solver, ea, er);
    double g = unscaled_term(solver) ? info->duality_gap : w->scaled_dual_gap;
    gc = fabs(g) < gt;
  } else gc = 1;
  if (prc && drc && gc) {
    update_status(info, approximate ? OSQP_SOLVED_INACCURATE : OSQP_SOLVED);
    return 1;
  }
  if (pic) {
    update_status(info, approximate ? OSQP_PRIMAL_INFEASIBLE_INACCURATE : OSQP_PRIMAL_INFEASIBLE);
    if (unscaled_term(solver)) for (k = 0; k < w->m; k++) w->delta_y[k] *= w->E[k];
    info->obj_val = ORC_INF;
    return 1;
  }
  if (dic) {
    update_status(info, approximate ? OSQP_DUAL_INFEASIBLE_INACCURATE : OSQP_DUAL_INFEASIBLE);
    if (unscaled_term(solver)) for (k = 0; k < w->n; k++) w->delta_x[k] *= w->D[k];
    info->obj_val = -ORC_INF;
    return 1;
  }
  return 0;
}

static double rho_estimate(OSQPSolver* solver) {
  OSQPWorkspace* w = solver->work;
  double pr = w->scaled_prim_res, dr = w->scaled_dual_res, pn, dn, r;
  pn = dmax(vnorm_inf(w->z, w->m), vnorm_inf(w->Ax, w->m));
  pr /= (pn + ORC_DIV_TOL);
  dn = dmax(dmax(vnorm_inf(w->q, w->n), vnorm_inf(w->Aty, w->n)), vnorm_inf(w->Px, w->n));
  dr /= (dn + ORC_DIV_TOL);
  r = solver->settings->rho * sqrt(pr / dr);
  return dmin(dmax(r, OSQP_RHO_MIN), OSQP_RHO_MAX);
}

OSQPInt osqp_update_rho(OSQPSolver* solver, OSQPFloat rho_new) {
  OSQPWorkspace* w;
  OSQPInt k;
  if (!solver || !solver->work) return OSQP_WORKSPACE_NOT_INIT_ERROR;
  w = solver->work;
  if (rho_new <= 0) return 1;
  solver->settings->rho = dmin(dmax(rho_new, OSQP_RHO_MIN), OSQP_RHO_MAX);
  if (solver->settings->rho_is_vec) {
    for (k = 0; k < w->m; k++) {
      w->rho_vec[k] = w->constr_type[k] < 0 ? OSQP_RHO_MIN
                    : (w->constr_type[k] == 0 ? solver->settings->rho
                                              : OSQP_RHO_EQ_OVER_RHO_INEQ * solver->settings->rho);
      w->rho_inv_vec[k] = 1.0 / w->rho_vec[k];
    }
  } else w->rho_inv = 1.0 / solver->settings->rho;
  return ls_update_rho(w->ls, w->rho_vec, solver->settings->rho);
}

static int adapt_rho(OSQPSolver* solver) {
  double r = rho_estimate(solver);
  int rc = 0;
  solver->info->rho_estimate = r;
  if (r > solver->settings->rho * solver->settings->adaptive_rho_tolerance ||
      r < solver->settings->rho / solver->settings->adaptive_rho_tolerance) {
    rc = (int)osqp_update_rho(solver, r);
    solver->info->rho_updates += 1;
    solver->work->rho_updated = 1;
  }
  return rc;
}

/* ======================================================================
 * Public API (src/osqp_api.c)
 * ====================================================================== */
OSQPInt osqp_capabilities(void) { return OSQP_CAPABILITY_DIRECT_SOLVER | OSQP_CAPABILITY_INDIRECT_SOLVER | OSQP_CAPABILITY_UPDATE_MATRICES; }
const char* osqp_version(void) { return "1.0.0-oracle"; }
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
  st->linsys_solver = OSQP_DIRECT_SOLVER;
  st->allocate_solution = 1;
  st->verbose = OSQP_VERBOSE;
  st->profiler_level = 0;
  st->warm_starting = OSQP_WARM_STARTING;
  st->scaling = OSQP_SCALING;
  st->polishing = OSQP_POLISHING;
  st->rho = OSQP_RHO;
  st->rho_is_vec = ORC_RHO_IS_VEC;
  st->sigma = OSQP_SIGMA;
  st->alpha = OSQP_ALPHA;
  st->cg_max_iter = OSQP_CG_MAX_ITER;
  st->cg_tol_reduction = OSQP_CG_TOL_REDUCTION;
  st->cg_tol_fraction = OSQP_CG_TOL_FRACTION;
  st->cg_precond = OSQP_DIAGONAL_PRECONDITIONER;
  st->adaptive_rho = OSQP_ADAPTIVE_RHO_UPDATE_DEFAULT;
  st->adaptive_rho_interval = OSQP_ADAPTIVE_RHO_INTERVAL;
  st->adaptive_rho_fraction = OSQP_ADAPTIVE_RHO_FRACTION;
  st->adaptive_rho_tolerance = ORC_ADAPTIVE_RHO_TOL;
  st->max_iter = OSQP_MAX_ITER;
  st->eps_abs = OSQP_EPS_ABS;
  st->eps_rel = OSQP_EPS_REL;
  st->eps_prim_inf = OSQP_EPS_PRIM_INF;
  st->eps_dual_inf = OSQP_EPS_DUAL_INF;
  st->scaled_termination = OSQP_SCALED_TERMINATION;
  st->check_termination = ORC_CHECK_TERMINATION;
  st->check_dualgap = ORC_CHECK_DUALGAP;
  st->time_limit = OSQP_TIME_LIMIT;
  st->delta = OSQP_DELTA;
  st->polish_refine_iter = OSQP_POLISH_REFINE_ITER;
}

OSQPSettings* OSQPSettings_new(void) {
  OSQPSettings* s = (OSQPSettings*)calloc(1, sizeof(OSQPSettings));
  osqp_set_default_settings(s);
  return s;
}
void OSQPSettings_free(OSQPSettings* s) { free(s); }

/* validate_data / validate_settings: src/auxil.c:950-1223 */
static int validate_data(const OSQPCscMatrix* P, const OSQPFloat* q, const OSQPCscMatrix* A,
                         const OSQPFloat* l, const OSQPFloat* u, OSQPInt m, OSQPInt n) {
  OSQPInt j, k;
  if (!P || !A || !q) return 1;
  if (n <= 0 || m < 0) return 1;
  if (P->m != n || P->m != P->n) return 1;
  for (j = 0; j < n; j++) for (k = P->p[j]; k < P->p[j + 1]; k++) if (P->i[k] > j) return 1;
  if (A->m != m || A->n != n) return 1;
  for (j = 0; j < m; j++) if (l[j] > u[j]) return 1;
  return 0;
}
static int validate_settings(const OSQPSettings* s, int from_setup) {
  if (!s) return 1;
  if (from_setup && s->linsys_solver != OSQP_DIRECT_SOLVER && s->linsys_solver != OSQP_INDIRECT_SOLVER) return 1;
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

void osqp_cold_start(OSQPSolver* solver) {
  OSQPWorkspace* w = solver->work;
  memset(w->x, 0, sizeof(double) * w->n);
  memset(w->z, 0, sizeof(double) * (w->m ? w->m : 1));
  memset(w->y, 0, sizeof(double) * (w->m ? w->m : 1));
  ls_warm_start(w->ls, w->x);
}

static void reset_info(OSQPInfo* info) {
  info->solve_time = 0.0;
  info->polish_time = 0.0;
  update_status(info, OSQP_UNSOLVED);
  info->rho_updates = 0;
}

OSQPInt osqp_setup(OSQPSolver** solverp, const OSQPCscMatrix* P, const OSQPFloat* q,
                   const OSQPCscMatrix* A, const OSQPFloat* l, const OSQPFloat* u,
                   OSQPInt m, OSQPInt n, const OSQPSettings* settings) {
  OSQPSolver* solver;
  OSQPWorkspace* w;
  OSQPInt k;
  int rc;
  double t0 = now_s();
  if (validate_data(P, q, A, l, u, m, n)) return OSQP_DATA_VALIDATION_ERROR;
  if (validate_settings(settings, 1)) return OSQP_SETTINGS_VALIDATION_ERROR;
  solver = (OSQPSolver*)calloc(1, sizeof(OSQPSolver));
  *solverp = solver;
  w = (OSQPWorkspace*)calloc(1, sizeof(OSQPWorkspace));
  solver->work = w;
  solver->info = (OSQPInfo*)calloc(1, sizeof(OSQPInfo));
  solver->settings = (OSQPSettings*)malloc(sizeof(OSQPSettings));
  memcpy(solver->settings, settings, sizeof(OSQPSettings));
  w->n = n; w->m = m;
  w->P = csc_from_api(P);
  w->A = csc_from_api(A);
  w->q = vnew(n); memcpy(w->q, q, sizeof(double) * n);
  w->l = vnew(m); w->u = vnew(m);
  if (m) { memcpy(w->l, l, sizeof(double) * m); memcpy(w->u, u, sizeof(double) * m); }
  if (settings->rho_is_vec) {
    w->rho_vec = vnew(m); w->rho_inv_vec = vnew(m);
    w->constr_type = (OSQPInt*)calloc((size_t)(m ? m : 1), sizeof(OSQPInt));
  }
  w->x = vnew(n); w->z = vnew(m); w->xz = vnew(n + m);
  w->x_prev = vnew(n); w->z_prev = vnew(m); w->y = vnew(m);
  w->Ax = vnew(m); w->Px = vnew(n); w->Aty = vnew(n);
  w->delta_y = vnew(m); w->Atdelta_y = vnew(n);
  w->delta_x = vnew(n); w->Pdelta_x = vnew(n); w->Adelta_x = vnew(m);
  w->D = vnew(n); w->Dinv = vnew(n); w->E = vnew(m); w->Einv = vnew(m);
  w->D_temp = vnew(n); w->D_temp_A = vnew(n); w->E_temp = vnew(m);
  w->c = 1.0; w->cinv = 1.0;
  for (k = 0; k < n; k++) { w->D[k] = 1.0; w->Dinv[k] = 1.0; }
  for (k = 0; k < m; k++) { w->E[k] = 1.0; w->Einv[k] = 1.0; }
  if (settings->scaling) scale_data(solver);
  if (settings->rho_is_vec) set_rho_vec(solver);
  else {
    solver->settings->rho = dmin(dmax(settings->rho, OSQP_RHO_MIN), OSQP_RHO_MAX);
    w->rho_inv = 1.0 / solver->settings->rho;
  }
  rc = ls_init(&w->ls, w->P, w->A, w->rho_vec, solver->settings->rho, solver->settings,
               &w->scaled_prim_res, &w->scaled_dual_res, 0);
  if (rc == OSQP_NONCVX_ERROR) { update_status(solver->info, OSQP_NON_CVX); return rc; }
  if (rc) return rc;
  osqp_cold_start(solver);
  w->active = (OSQPInt*)calloc((size_t)(m ? m : 1), sizeof(OSQPInt));
  w->pol_x = vnew(n); w->pol_z = vnew(m); w->pol_y = vnew(m);
  if (settings->allocate_solution) {
    solver->solution = (OSQPSolution*)calloc(1, sizeof(OSQPSolution));
    solver->solution->x = (OSQPFloat*)calloc((size_t)n, sizeof(double));
    solver->solution->y = (OSQPFloat*)calloc((size_t)(m ? m : 1), sizeof(double));
    solver->solution->prim_inf_cert = (OSQPFloat*)calloc((size_t)(m ? m : 1), sizeof(double));
    solver->solution->dual_inf_cert = (OSQPFloat*)calloc((size_t)n, sizeof(double));
  }
  solver->info->status_polish = OSQP_POLISH_NOT_PERFORMED;
  update_status(solver->info, OSQP_UNSOLVED);
  solver->info->setup_time = now_s() - t0;
  w->first_run = 1;
  solver->info->rho_updates = 0;
  solver->info->rho_estimate = solver->settings->rho;
  solver->info->obj_val = ORC_INF;
  solver->info->prim_res = ORC_INF;
  solver->info->dual_res = ORC_INF;
  solver->info->rel_kkt_error = ORC_INF;
  w->last_rel_kkt = ORC_INF;
  if (solver->settings->adaptive_rho == OSQP_ADAPTIVE_RHO_UPDATE_ITERATIONS &&
      solver->settings->adaptive_rho_interval == 0) {
    solver->settings->adaptive_rho_interval = solver->settings->check_termination
        ? OSQP_ADAPTIVE_RHO_MULTIPLE_TERMINATION * solver->settings->check_termination
        : OSQP_ADAPTIVE_RHO_FIXED;
  }
  if (solver->settings->adaptive_rho == OSQP_ADAPTIVE_RHO_UPDATE_KKT_ERROR &&
      solver->settings->adaptive_rho_interval == 0)
    solver->settings->adaptive_rho_interval = 1;
  return 0;
}

static int has_solution(const OSQPInfo* info) {
  return info->status_val != OSQP_PRIMAL_INFEASIBLE && info->status_val != OSQP_PRIMAL_INFEASIBLE_INACCURATE &&
         info->status_val != OSQP_DUAL_INFEASIBLE && info->status_val != OSQP_DUAL_INFEASIBLE_INACCURATE &&
         info->status_val != OSQP_NON_CVX;
}

/* store_solution: src/auxil.c:598-674 */
static void store_solution(OSQPSolver* solver, OSQPSolution* sol) {
  OSQPWorkspace* w = solver->work;
  OSQPInfo* info = solver->info;
  OSQPInt k, n = w->n, m = w->m;
  if (!sol) return;
  if (has_solution(info)) {
    if (solver->settings->scaling) {
      for (k = 0; k < n; k++) sol->x[k] = w->D[k] * w->x[k];
      for (k = 0; k < m; k++) sol->y[k] = w->E[k] * w->y[k] * w->cinv;
    } else {
      memcpy(sol->x, w->x, sizeof(double) * n);
      if (m) memcpy(sol->y, w->y, sizeof(double) * m);
    }
    for (k = 0; k < m; k++) { w->delta_y[k] = NAN; sol->prim_inf_cert[k] = NAN; }
    for (k = 0; k < n; k++) { w->delta_x[k] = NAN; sol->dual_inf_cert[k] = NAN; }
  } else {
    for (k = 0; k < n; k++) sol->x[k] = NAN;
    for (k = 0; k < m; k++) sol->y[k] = NAN;
    osqp_cold_start(solver);
    if (info->status_val == OSQP_PRIMAL_INFEASIBLE || info->status_val == OSQP_PRIMAL_INFEASIBLE_INACCURATE) {
      double nv = vnorm_inf(w->delta_y, m);
      for (k = 0; k < m; k++) { w->delta_y[k] *= 1.0 / nv; sol->prim_inf_cert[k] = w->delta_y[k]; }
      for (k = 0; k < n; k++) { w->delta_x[k] = NAN; sol->dual_inf_cert[k] = NAN; }
    }
    if (info->status_val == OSQP_DUAL_INFEASIBLE || info->status_val == OSQP_DUAL_INFEASIBLE_INACCURATE) {
      double nv = vnorm_inf(w->delta_x, n);
      for (k = 0; k < n; k++) { w->delta_x[k] *= 1.0 / nv; sol->dual_inf_cert[k] = w->delta_x[k]; }
      for (k = 0; k < m; k++) { w->delta_y[k] = NAN; sol->prim_inf_cert[k] = NAN; }
    }
  }
}

/* polish: src/polish.c:19-515 */
static void polish(OSQPSolver* solver) {
  OSQPWorkspace* w = solver->work;
  OSQPInfo* info = solver->info;
  OSQPSettings* st = solver->settings;
  OSQPInt j, n = w->n, m = w->m, cnt = 0, mred, i;
  oc_ls* pl = NULL;
  double t0 = now_s();
  w->n_active = 0;
  for (j = 0; j < m; j++) {
    if ((w->z[j] - w->l[j] < -w->y[j]) || (w->l[j] == w->u[j])) { w->active[j] = -1; w->n_active++; }
    else if (w->u[j] - w->z[j] < w->y[j]) { w->active[j] = 1; w->n_active++; }
    else w->active[j] = 0;
  }
  ocsc* Ared = csc_rows(w->A, w->active, &mred);
  if (w->n_active == 0) {
    info->status_polish = OSQP_POLISH_NO_ACTIVE_SET_FOUND;
    csc_free(Ared);
    return;
  }
  double w_t0 = w->t0;
  if (ls_init(&pl, w->P, Ared, NULL, 0.0, st, NULL, NULL, 1)) {
    info->status_polish = OSQP_POLISH_LINSYS_ERROR;
    ls_free(pl); csc_free(Ared);
    return;
  }
  double* rhs = vnew(n + mred);
  double* sol = vnew(n + mred);
  double* tmp = vnew(n + mred);
  for (j = 0; j < n; j++) rhs[j] = -w->q[j];
  for (j = 0; j < m; j++) {
    if (w->active[j] == -1) rhs[n + cnt++] = w->l[j];
    else if (w->active[j] == 1) rhs[n + cnt++] = w->u[j];
  }
  memcpy(sol, rhs, sizeof(double) * (n + mred));
  ls_warm_start(pl, w->x);
  ls_solve(pl, sol, 1);
  for (i = 0; i < st->polish_refine_iter; i++) {
    memcpy(tmp, rhs, sizeof(double) * (n + mred));
    csc_axpy(w->P, sol, tmp, -1.0, 1.0, 1);
    csc_atxpy(Ared, sol + n, tmp, -1.0, 1.0);
    csc_axpy(Ared, sol, tmp + n, -1.0, 1.0, 0);
    ls_solve(pl, tmp, 1);
    for (j = 0; j < n + mred; j++) sol[j] += tmp[j];
  }
  memcpy(w->pol_x, sol, sizeof(double) * n);
  csc_axpy(w->A, w->pol_x, w->pol_z, 1.0, 0.0, 0);
  cnt = 0;
  for (j = 0; j < m; j++) w->pol_y[j] = (w->active[j] == 0) ? 0.0 : sol[n + cnt++];
  for (j = 0; j < m; j++) {
    double yz = w->pol_y[j] + w->pol_z[j];
    w->pol_z[j] = dmin(dmax(yz, w->l[j]), w->u[j]);
    w->pol_y[j] = yz - w->pol_z[j];
  }
  w->t0 = t0;
  update_info(solver, 0, 1);
  w->t0 = w_t0;
  int ok = (w->pol_prim < info->prim_res && w->pol_dual < info->dual_res) ||
           (w->pol_prim < info->prim_res && info->dual_res < 1e-10) ||
           (w->pol_dual < info->dual_res && info->prim_res < 1e-10);
  if (ok) {
    info->obj_val = w->pol_obj; info->dual_obj_val = w->pol_dobj; info->duality_gap = w->pol_gap;
    info->prim_res = w->pol_prim; info->dual_res = w->pol_dual;
    info->status_polish = OSQP_POLISH_SUCCESS;
    memcpy(w->x, w->pol_x, sizeof(double) * n);
    if (m) { memcpy(w->z, w->pol_z, sizeof(double) * m); memcpy(w->y, w->pol_y, sizeof(double) * m); }
  } else info->status_polish = OSQP_POLISH_FAILED;
  ls_free(pl); csc_free(Ared);
  free(rhs); free(sol); free(tmp);
}

OSQPInt osqp_solve(OSQPSolver* solver) {
  OSQPWorkspace* w;
  OSQPSettings* st;
  OSQPInfo* info;
  OSQPInt iter, k, n, m;
  int can_check = 0, can_adapt = 0;
  double* t;
  if (!solver || !solver->work) return OSQP_WORKSPACE_NOT_INIT_ERROR;
  w = solver->work; st = solver->settings; info = solver->info;
  n = w->n; m = w->m;
  if (w->clear_update_time) info->update_time = 0.0;
  w->rho_update_from_solve = 1;
  w->t0 = now_s();
  if (!st->warm_starting) osqp_cold_start(solver);
  w->pcg_iters_total = 0;
  for (iter = 1; iter <= st->max_iter; iter++) {
    t = w->x; w->x = w->x_prev; w->x_prev = t;
    t = w->z; w->z = w->z_prev; w->z_prev = t;
    /* compute_rhs + linsys solve: src/auxil.c:136-170 */
    for (k = 0; k < n; k++) w->xz[k] = st->sigma * w->x_prev[k] - w->q[k];
    if (st->rho_is_vec) for (k = 0; k < m; k++) w->xz[n + k] = w->z_prev[k] - w->rho_inv_vec[k] * w->y[k];
    else for (k = 0; k < m; k++) w->xz[n + k] = w->z_prev[k] - w->rho_inv * w->y[k];
    ls_solve(w->ls, w->xz, iter);
    if (w->ls->type == OSQP_INDIRECT_SOLVER) w->pcg_iters_total += w->ls->last_pcg_iters;
    /* update_x, update_z, update_y: src/auxil.c:172-229 */
    for (k = 0; k < n; k++) {
      w->x[k] = st->alpha * w->xz[k] + (1.0 - st->alpha) * w->x_prev[k];
      w->delta_x[k] = w->x[k] - w->x_prev[k];
    }
    for (k = 0; k < m; k++) {
      double ri = st->rho_is_vec ? w->rho_inv_vec[k] : w->rho_inv;
      double rr = st->rho_is_vec ? w->rho_vec[k] : st->rho;
      double zr = st->alpha * w->xz[n + k] + (1.0 - st->alpha) * w->z_prev[k];
      double zz = zr + ri * w->y[k];
      w->z[k] = dmin(dmax(zz, w->l[k]), w->u[k]);
      w->delta_y[k] = rr * (zr - w->z[k]);
      w->y[k] += w->delta_y[k];
    }
    if (st->time_limit && (now_s() - w->t0 + (w->first_run ? info->setup_time : info->update_time)) >= st->time_limit) {
      update_status(info, OSQP_TIME_LIMIT_REACHED);
      break;
    }
    can_check = st->check_termination && (iter % st->check_termination == 0);
    can_adapt = 0;
    if (st->adaptive_rho == OSQP_ADAPTIVE_RHO_UPDATE_ITERATIONS ||
        st->adaptive_rho == OSQP_ADAPTIVE_RHO_UPDATE_KKT_ERROR)
      can_adapt = st->adaptive_rho_interval && (iter % st->adaptive_rho_interval == 0);
    if (can_check || can_adapt || iter == 1) update_info(solver, iter, 0);
    if (can_check && check_termination(solver, 0)) break;
    w->rho_updated = 0;
    if (can_adapt && st->adaptive_rho == OSQP_ADAPTIVE_RHO_UPDATE_KKT_ERROR)
      can_adapt = info->rel_kkt_error <= st->adaptive_rho_fraction * w->last_rel_kkt;
    if (can_adapt && adapt_rho(solver)) return 1;
    if (w->rho_updated) w->last_rel_kkt = info->rel_kkt_error;
  }
  if (!can_check) {
    update_info(solver, iter - 1, 0);
    check_termination(solver, 0);
  }
  if (has_solution(info))
    obj_val_dual_gap(solver, w->x, w->y, &info->obj_val, &info->dual_obj_val, &info->duality_gap);
  if (info->status_val == OSQP_UNSOLVED) {
    if (!check_termination(solver, 1)) update_status(info, OSQP_MAX_ITER_REACHED);
  }
  if (info->status_val == OSQP_TIME_LIMIT_REACHED) {
    if (!check_termination(solver, 1)) update_status(info, OSQP_TIME_LIMIT_REACHED);
  }
  info->rho_estimate = rho_estimate(solver);
  info->solve_time = now_s() - w->t0;
  if (st->polishing && info->status_val == OSQP_SOLVED) polish(solver);
  info->run_time = (w->first_run ? info->setup_time : info->update_time) + info->solve_time + info->polish_time;
  w->first_run = 0;
  w->clear_update_time = 1;
  w->rho_update_from_solve = 0;
  store_solution(solver, solver->solution);
  return 0;
}

OSQPInt osqp_get_solution(OSQPSolver* solver, OSQPSolution* solution) {
  if (!solver || !solver->work || !solution) return OSQP_WORKSPACE_NOT_INIT_ERROR;
  store_solution(solver, solution);
  return 0;
}

OSQPInt osqp_cleanup(OSQPSolver* solver) {
  OSQPWorkspace* w;
  if (!solver) return 0;
  w = solver->work;
  if (w) {
    csc_free(w->P); csc_free(w->A);
    free(w->q); free(w->l); free(w->u); free(w->rho_vec); free(w->rho_inv_vec); free(w->constr_type);
    free(w->x); free(w->y); free(w->z); free(w->xz); free(w->x_prev); free(w->z_prev);
    free(w->Ax); free(w->Px); free(w->Aty); free(w->delta_y); free(w->Atdelta_y);
    free(w->delta_x); free(w->Pdelta_x); free(w->Adelta_x);
    free(w->D_temp); free(w->D_temp_A); free(w->E_temp);
    free(w->D); free(w->Dinv); free(w->E); free(w->Einv);
    ls_free(w->ls);
    free(w->active); free(w->pol_x); free(w->pol_z); free(w->pol_y);
    free(w);
  }
  if (solver->solution) {
    free(solver->solution->x); free(solver->solution->y);
    free(solver->solution->prim_inf_cert); free(solver->solution->dual_inf_cert);
    free(solver->solution);
  }
  free(solver->settings); free(solver->info); free(solver);
  return 0;
}

/* osqp_api.c:1184-1257 */
OSQPInt osqp_update_data_vec(OSQPSolver* solver, const OSQPFloat* q_new, const OSQPFloat* l_new, const OSQPFloat* u_new) {
  OSQPWorkspace* w;
  OSQPInt k, bad = 0;
  double t0 = now_s();
  if (!solver || !solver->work) return OSQP_WORKSPACE_NOT_INIT_ERROR;
  w = solver->work;
  if (w->clear_update_time) { w->clear_update_time = 0; solver->info->update_time = 0.0; }
  if (l_new || u_new) {
    double* lt = w->z_prev;
    double* ut = w->delta_y;
    if (l_new) for (k = 0; k < w->m; k++) lt[k] = l_new[k] * (solver->settings->scaling ? w->E[k] : 1.0);
    if (u_new) for (k = 0; k < w->m; k++) ut[k] = u_new[k] * (solver->settings->scaling ? w->E[k] : 1.0);
    const double* lc = l_new ? lt : w->l;
    const double* uc = u_new ? ut : w->u;
    for (k = 0; k < w->m; k++) if (lc[k] > uc[k]) bad = 1;
    if (bad) return OSQP_DATA_VALIDATION_ERROR;
    if (l_new) { w->z_prev = w->l; w->l = lt; }
    if (u_new) { w->delta_y = w->u; w->u = ut; }
    if (solver->settings->rho_is_vec) {
      if (set_rho_vec(solver)) bad = ls_update_rho(w->ls, w->rho_vec, solver->settings->rho);
    }
  }
  if (q_new) {
    for (k = 0; k < w->n; k++)
      w->q[k] = solver->settings->scaling ? q_new[k] * w->D[k] * w->c : q_new[k];
  }
  reset_info(solver->info);
  solver->info->update_time += now_s() - t0;
  return bad;
}

/* osqp_api.c:1260-1293 */
OSQPInt osqp_warm_start(OSQPSolver* solver, const OSQPFloat* x, const OSQPFloat* y) {
  OSQPWorkspace* w;
  OSQPInt k;
  if (!solver || !solver->work) return OSQP_WORKSPACE_NOT_INIT_ERROR;
  w = solver->work;
  if (!solver->settings->warm_starting) solver->settings->warm_starting = 1;
  if (x) for (k = 0; k < w->n; k++) w->x[k] = solver->settings->scaling ? x[k] * w->Dinv[k] : x[k];
  if (y) for (k = 0; k < w->m; k++) w->y[k] = solver->settings->scaling ? y[k] * w->Einv[k] * w->c : y[k];
  if (x) csc_axpy(w->A, w->x, w->z, 1.0, 0.0, 0);
  ls_warm_start(w->ls, w->x);
  return 0;
}

/* osqp_api.c:1309-1409 */
OSQPInt osqp_update_data_mat(OSQPSolver* solver, const OSQPFloat* Px_new, const OSQPInt* Px_new_idx, OSQPInt P_new_n,
                             const OSQPFloat* Ax_new, const OSQPInt* Ax_new_idx, OSQPInt A_new_n) {
  OSQPWorkspace* w;
  OSQPInt k, nnzP, nnzA;
  int rc;
  double t0 = now_s();
  if (!solver || !solver->work) return OSQP_WORKSPACE_NOT_INIT_ERROR;
  w = solver->work;
  if (w->clear_update_time) { w->clear_update_time = 0; solver->info->update_time = 0.0; }
  nnzP = csc_nnz(w->P); nnzA = csc_nnz(w->A);
  if (P_new_n > nnzP || P_new_n < 0) return 1;
  if (!Px_new_idx && P_new_n != 0 && P_new_n != nnzP) return 1;
  if (P_new_n == 0) P_new_n = nnzP;
  if (A_new_n > nnzA || A_new_n < 0) return 2;
  if (!Ax_new_idx && A_new_n != 0 && A_new_n != nnzA) return 2;
  if (A_new_n == 0) A_new_n = nnzA;
  if (solver->settings->scaling) unscale_data(solver);
  if (Px_new) for (k = 0; k < P_new_n; k++) w->P->x[Px_new_idx ? Px_new_idx[k] : k] = Px_new[k];
  if (Ax_new) for (k = 0; k < A_new_n; k++) w->A->x[Ax_new_idx ? Ax_new_idx[k] : k] = Ax_new[k];
  if (solver->settings->scaling) scale_data(solver);
  rc = ls_update_matrices(w->ls, w->P, w->A);
  reset_info(solver->info);
  solver->info->update_time += now_s() - t0;
  return rc;
}

/* osqp_api.c:1474-1530 */
OSQPInt osqp_update_settings(OSQPSolver* solver, const OSQPSettings* ns) {
  OSQPSettings* s;
  if (!solver || !solver->work) return OSQP_WORKSPACE_NOT_INIT_ERROR;
  if (validate_settings(ns, 0)) return OSQP_SETTINGS_VALIDATION_ERROR;
  s = solver->settings;
  s->profiler_level = ns->profiler_level; s->verbose = ns->verbose; s->warm_starting = ns->warm_starting;
  s->polishing = ns->polishing; s->alpha = ns->alpha;
  s->cg_max_iter = ns->cg_max_iter; s->cg_tol_reduction = ns->cg_tol_reduction;
  s->cg_tol_fraction = ns->cg_tol_fraction; s->cg_precond = ns->cg_precond;
  s->max_iter = ns->max_iter; s->eps_abs = ns->eps_abs; s->eps_rel = ns->eps_rel;
  s->eps_prim_inf = ns->eps_prim_inf; s->eps_dual_inf = ns->eps_dual_inf;
  s->scaled_termination = ns->scaled_termination; s->check_termination = ns->check_termination;
  s->check_dualgap = ns->check_dualgap; s->time_limit = ns->time_limit;
  s->delta = ns->delta; s->polish_refine_iter = ns->polish_refine_iter;
  if (solver->work->ls->type == OSQP_INDIRECT_SOLVER) {
    oc_ls* l = solver->work->ls;
    l->max_iter = s->cg_max_iter; l->reduction_threshold = s->cg_tol_reduction;
    l->tol_fraction = s->cg_tol_fraction;
    if (l->precond_type != s->cg_precond) { l->precond_type = s->cg_precond; pcg_update_precond(l); }
  }
  return 0;
}

/* Total PCG iterations of the last solve (oracle diagnostics only). */
OSQPInt oracle_last_pcg_iters(OSQPSolver* solver) { return solver && solver->work ? solver->work->pcg_iters_total : 0; }
/* The block-Jacobi blocks (cg_precond = 2, indirect solver): copies
 * ceil(n / 32) * 1024 values into out; returns how many, 0 when there are none. */
OSQPInt oracle_block_inverse(OSQPSolver* solver, double* out) {
  oc_ls* l;
  size_t cnt;
  if (!solver || !solver->work || !(l = solver->work->ls) || l->type != OSQP_INDIRECT_SOLVER || !l->binv) return 0;
  cnt = (size_t)((l->n + OC_PBLK - 1) / OC_PBLK) * OC_PBLK * OC_PBLK;
  if (out) memcpy(out, l->binv, sizeof(double) * cnt);
  return (OSQPInt)cnt;
}
