/*
 * osqp_gb300_algebra.h -- the algebra / linear-system ABI of OSQP 1.0,
 * implemented on GB300 device memory by libosqp_gb300_algebra.so (FP32) and
 * libosqp_gb300_algebra_f64.so (FP64).
 *
 * This is the drop-in boundary for OSQP's unmodified C core (src/osqp_api.c,
 * src/auxil.c, src/scaling.c, src/polish.c): the core calls only these
 * functions, so linking it against this library instead of the reference's
 * algebra/cuda backend runs every vector, matrix and linear-system operation
 * on the hand-written sm_103a kernels.  Each declaration names the reference
 * declaration it replaces.  Semantics follow the reference's CUDA backend:
 * raw pointers given to *_from_raw, *_to_raw and OSQPMatrix_new_from_csc may
 * be host or device memory; reductions return host scalars (accumulated in
 * FP64-accurate arithmetic); errors are reported, never exit().
 */
#ifndef OSQP_GB300_ALGEBRA_H
#define OSQP_GB300_ALGEBRA_H

#include "osqp_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct OSQPVectori_ OSQPVectori;
typedef struct OSQPVectorf_ OSQPVectorf;
typedef struct OSQPMatrix_ OSQPMatrix;
typedef struct linsys_solver LinSysSolver;

/* ---- vectors: include/private/algebra_vector.h ---- */
OSQPInt      OSQPVectorf_is_eq(const OSQPVectorf* A, const OSQPVectorf* B, OSQPFloat tol);   /* :28 */
OSQPVectorf* OSQPVectorf_malloc(OSQPInt length);                                              /* :33 */
OSQPVectorf* OSQPVectorf_calloc(OSQPInt length);                                              /* :34 */
OSQPVectori* OSQPVectori_malloc(OSQPInt length);                                              /* :35 */
OSQPVectori* OSQPVectori_calloc(OSQPInt length);                                              /* :36 */
OSQPVectorf* OSQPVectorf_new(const OSQPFloat* a, OSQPInt length);                             /* :39 */
OSQPVectori* OSQPVectori_new(const OSQPInt* a, OSQPInt length);                               /* :43 */
OSQPVectorf* OSQPVectorf_copy_new(const OSQPVectorf* a);                                      /* :47 */
void         OSQPVectorf_free(OSQPVectorf* a);                                                /* :50 */
void         OSQPVectori_free(OSQPVectori* a);                                                /* :53 */
void         OSQPVectorf_subvector_assign(OSQPVectorf* A, OSQPFloat* b, OSQPInt start,
                                          OSQPInt length, OSQPFloat multiplier);              /* :58 */
void         OSQPVectorf_subvector_assign_scalar(OSQPVectorf* A, OSQPFloat sc, OSQPInt start,
                                                 OSQPInt length);                             /* :67 */
OSQPVectorf* OSQPVectorf_subvector_byrows(const OSQPVectorf* A, const OSQPVectori* rows);    /* :72 */
OSQPVectorf* OSQPVectorf_concat(const OSQPVectorf* A, const OSQPVectorf* B);                 /* :75 */
OSQPVectorf* OSQPVectorf_view(const OSQPVectorf* a, OSQPInt head, OSQPInt length);           /* :81 */
void         OSQPVectorf_view_update(OSQPVectorf* a, const OSQPVectorf* b, OSQPInt head,
                                     OSQPInt length);                                         /* :88 */
void         OSQPVectorf_view_free(OSQPVectorf* a);                                           /* :91 */
OSQPInt      OSQPVectorf_length(const OSQPVectorf* a);                                        /* :97 */
OSQPInt      OSQPVectori_length(const OSQPVectori* a);                                        /* :100 */
OSQPFloat*   OSQPVectorf_data(const OSQPVectorf* a);                                          /* :103 (device pointer) */
void         OSQPVectorf_copy(OSQPVectorf* b, const OSQPVectorf* a);                          /* :106 */
void         OSQPVectorf_from_raw(OSQPVectorf* b, const OSQPFloat* a);                        /* :110 */
void         OSQPVectori_from_raw(OSQPVectori* b, const OSQPInt* a);                          /* :114 */
void         OSQPVectorf_to_raw(OSQPFloat* bv, const OSQPVectorf* a);                         /* :118 */
void         OSQPVectori_to_raw(OSQPInt* bv, const OSQPVectori* a);                           /* :122 */
void         OSQPVectorf_set_scalar(OSQPVectorf* a, OSQPFloat sc);                            /* :126 */
void         OSQPVectorf_set_scalar_conditional(OSQPVectorf* a, const OSQPVectori* test,
                                                OSQPFloat val_if_neg, OSQPFloat val_if_zero,
                                                OSQPFloat val_if_pos);                        /* :130 */
void         OSQPVectorf_round_to_zero(OSQPVectorf* a, OSQPFloat tol);                        /* :139 */
void         OSQPVectorf_mult_scalar(OSQPVectorf* a, OSQPFloat sc);                           /* :143 */
void         OSQPVectorf_plus(OSQPVectorf* x, const OSQPVectorf* a, const OSQPVectorf* b);    /* :147 */
void         OSQPVectorf_minus(OSQPVectorf* x, const OSQPVectorf* a, const OSQPVectorf* b);   /* :152 */
void         OSQPVectorf_add_scaled(OSQPVectorf* x, OSQPFloat sca, const OSQPVectorf* a,
                                    OSQPFloat scb, const OSQPVectorf* b);                     /* :157 */
void         OSQPVectorf_add_scaled3(OSQPVectorf* x, OSQPFloat sca, const OSQPVectorf* a,
                                     OSQPFloat scb, const OSQPVectorf* b, OSQPFloat scc,
                                     const OSQPVectorf* c);                                   /* :164 */
OSQPFloat    OSQPVectorf_norm_inf(const OSQPVectorf* v);                                      /* :173 */
OSQPFloat    OSQPVectorf_scaled_norm_inf(const OSQPVectorf* S, const OSQPVectorf* v);         /* :176 */
OSQPFloat    OSQPVectorf_norm_inf_diff(const OSQPVectorf* a, const OSQPVectorf* b);           /* :180 */
OSQPFloat    OSQPVectorf_norm_2(const OSQPVectorf* v);                                        /* :184 */
OSQPFloat    OSQPVectorf_norm_1(const OSQPVectorf* a);                                        /* :187 */
OSQPFloat    OSQPVectorf_dot_prod(const OSQPVectorf* a, const OSQPVectorf* b);                /* :190 */
OSQPFloat    OSQPVectorf_dot_prod_signed(const OSQPVectorf* a, const OSQPVectorf* b,
                                         OSQPInt sign);                                       /* :198 */
void         OSQPVectorf_ew_prod(OSQPVectorf* c, const OSQPVectorf* a, const OSQPVectorf* b); /* :203 */
OSQPInt      OSQPVectorf_all_leq(const OSQPVectorf* l, const OSQPVectorf* u);                 /* :210 */
void         OSQPVectorf_ew_bound_vec(OSQPVectorf* x, const OSQPVectorf* z, const OSQPVectorf* l,
                                      const OSQPVectorf* u);                                  /* :217 */
void         OSQPVectorf_project_polar_reccone(OSQPVectorf* y, const OSQPVectorf* l,
                                               const OSQPVectorf* u, OSQPFloat infval);       /* :227 */
OSQPInt      OSQPVectorf_in_reccone(const OSQPVectorf* y, const OSQPVectorf* l, const OSQPVectorf* u,
                                    OSQPFloat infval, OSQPFloat tol);                         /* :237 */
void         OSQPVectorf_ew_reciprocal(OSQPVectorf* b, const OSQPVectorf* a);                 /* :246 */
void         OSQPVectorf_ew_sqrt(OSQPVectorf* a);                                             /* :250 */
void         OSQPVectorf_ew_max_vec(OSQPVectorf* c, const OSQPVectorf* a, const OSQPVectorf* b); /* :253 */
void         OSQPVectorf_ew_min_vec(OSQPVectorf* c, const OSQPVectorf* a, const OSQPVectorf* b); /* :258 */
OSQPInt      OSQPVectorf_ew_bounds_type(OSQPVectori* iseq, const OSQPVectorf* l, const OSQPVectorf* u,
                                        OSQPFloat tol, OSQPFloat infval);                     /* :269 */
void         OSQPVectorf_set_scalar_if_lt(OSQPVectorf* x, const OSQPVectorf* z, OSQPFloat testval,
                                          OSQPFloat newval);                                  /* :279 */
void         OSQPVectorf_set_scalar_if_gt(OSQPVectorf* x, const OSQPVectorf* z, OSQPFloat testval,
                                          OSQPFloat newval);                                  /* :287 */

/* ---- matrices: include/private/algebra_matrix.h ---- */
OSQPInt     OSQPMatrix_is_eq(const OSQPMatrix* A, const OSQPMatrix* B, OSQPFloat tol);       /* :26 */
OSQPMatrix* OSQPMatrix_new_from_csc(const OSQPCscMatrix* A, OSQPInt is_triu);                /* :34 */
void        OSQPMatrix_update_values(OSQPMatrix* M, const OSQPFloat* Mx_new, const OSQPInt* Mx_new_idx,
                                     OSQPInt M_new_n);                                        /* :60 */
OSQPInt     OSQPMatrix_get_m(const OSQPMatrix* M);                                            /* :66 */
OSQPInt     OSQPMatrix_get_n(const OSQPMatrix* M);                                            /* :69 */
OSQPFloat*  OSQPMatrix_get_x(const OSQPMatrix* M);                                            /* :72 (device) */
OSQPInt*    OSQPMatrix_get_i(const OSQPMatrix* M);                                            /* :75 (device) */
OSQPInt*    OSQPMatrix_get_p(const OSQPMatrix* M);                                            /* :78 (device) */
OSQPInt     OSQPMatrix_get_nz(const OSQPMatrix* M);                                           /* :81 */
void        OSQPMatrix_mult_scalar(OSQPMatrix* A, OSQPFloat sc);                             /* :86 */
void        OSQPMatrix_lmult_diag(OSQPMatrix* A, const OSQPVectorf* L);                      /* :90 */
void        OSQPMatrix_rmult_diag(OSQPMatrix* A, const OSQPVectorf* R);                      /* :94 */
void        OSQPMatrix_AtDA_extract_diag(const OSQPMatrix* A, const OSQPVectorf* D, OSQPVectorf* d); /* :98 */
void        OSQPMatrix_extract_diag(const OSQPMatrix* A, OSQPVectorf* d);                    /* :103 */
void        OSQPMatrix_Axpy(const OSQPMatrix* A, const OSQPVectorf* x, OSQPVectorf* y, OSQPFloat alpha,
                            OSQPFloat beta);                                                  /* :107 */
void        OSQPMatrix_Atxpy(const OSQPMatrix* A, const OSQPVectorf* x, OSQPVectorf* y, OSQPFloat alpha,
                             OSQPFloat beta);                                                 /* :114 */
void        OSQPMatrix_col_norm_inf(const OSQPMatrix* M, OSQPVectorf* E);                    /* :125 */
void        OSQPMatrix_row_norm_inf(const OSQPMatrix* M, OSQPVectorf* E);                    /* :128 */
void        OSQPMatrix_free(OSQPMatrix* M);                                                   /* :135 */
OSQPMatrix* OSQPMatrix_submatrix_byrows(const OSQPMatrix* A, const OSQPVectori* rows);       /* :137 */

/* ---- backend and linear system: include/private/lin_alg.h ---- */
OSQPInt osqp_algebra_linsys_supported(void);                                                  /* :13 */
enum osqp_linsys_solver_type osqp_algebra_default_linsys(void);                               /* :16 */
OSQPInt osqp_algebra_init_libs(OSQPInt device);                                               /* :19 */
void    osqp_algebra_free_libs(void);                                                         /* :22 */
OSQPInt osqp_algebra_name(char* name, OSQPInt nameLen);                                       /* :25 */
OSQPInt osqp_algebra_device_name(char* name, OSQPInt nameLen);                                /* :28 */
OSQPInt osqp_algebra_init_linsys_solver(LinSysSolver** s, const OSQPMatrix* P, const OSQPMatrix* A,
                                        const OSQPVectorf* rho_vec, const OSQPSettings* settings,
                                        OSQPFloat* scaled_prim_res, OSQPFloat* scaled_dual_res,
                                        OSQPInt polishing);                                   /* :46 */
/* settings->cg_precond: 0 none, 1 diagonal (as the reference's CUDA PCG,
 * cuda_pcg_interface.cu:133), 2 the 32 x 32 block-Jacobi preconditioner of
 * this library (blocks of P + sigma I + A' R A, rebuilt by update_rho_vec and
 * update_matrices; also selectable later through update_settings). */

/* One reduced-KKT solve that allocates nothing (no counterpart in the
 * reference).  For callers that cannot call cudaMalloc where they solve --
 * real-time control loops whose device memory is fixed before the loop
 * starts, because an allocation may block or fail at a moment the loop cannot
 * afford, and programs that share the GPU under a memory budget granted up
 * front -- this solves (P + sigma I + A' R A) x = b1 + A' R b2 by
 * PCG from x = 0 (R = diag(rho_vec), or settings->rho when rho_vec is NULL;
 * CG tolerance of the first ADMM iteration) and writes [x; A x] over b
 * (length n + m), exactly as a freshly initialised LinSysSolver's
 * solve(b, 1) does.  Its work vectors live in a fixed 4 MiB device array
 * inside the library (each GPU that loads the library holds it until the
 * process exits), so 8 n-vectors plus one m-vector (plus, with
 * settings->cg_precond = 2, the ceil(n / 32) * 1024 values of the
 * block-Jacobi blocks), each rounded up to 256 bytes, must fit in 4 MiB;
 * larger problems return
 * OSQP_DATA_VALIDATION_ERROR.  The call runs on the library's device (the
 * one the matrices were created on), launches one kernel on the library's own
 * stream and waits for it before returning.  The first call on a device looks
 * up that array's device address; make it before any stream capture begins.
 * All calls share the one array, which keeps the last call's contents (the
 * kernel clears what must start at zero): calls that overlap on the GPU
 * (other threads, other processes' streams of the same library) race and
 * must be serialised by the caller. */
/* Row structure derived from a matrix's CSC arrays (host copies; no
 * reference counterpart -- the reference keeps the same arrays inside its
 * csr_t, algebra/cuda/include/csr_type.h:27-40, built by csr_triu_to_full /
 * csr_transpose, algebra/cuda/src/cuda_csr.cu:489-628): CSR rowptr (rows + 1),
 * col and src (nnz each; value k of the rows is CSC value src[k], or -1 for a
 * structural diagonal added to a symmetric matrix) and, for upper-triangular
 * storage, diag (n: position of (j, j) in the rows).  The rows are those of
 * the represented matrix: full symmetric with an explicit diagonal for
 * is_triu, else of A itself.  Any pointer may be NULL.  Returns the number of
 * row entries, or -1. */
OSQPInt osqp_gb300_matrix_rows(const OSQPMatrix* M, OSQPInt* rowptr, OSQPInt* col, OSQPInt* src, OSQPInt* diag);

OSQPInt osqp_gb300_linsys_solve_noalloc(const OSQPMatrix* P, const OSQPMatrix* A, const OSQPVectorf* rho_vec,
                                        const OSQPSettings* settings, OSQPVectorf* b);

/* Linear-system object (include/private/types.h:243-279; layout is ABI). */
struct linsys_solver {
  enum osqp_linsys_solver_type type;
  const char* (*name)(LinSysSolver* self);
  OSQPInt (*solve)(LinSysSolver* self, OSQPVectorf* b, OSQPInt admm_iter);
  void (*update_settings)(LinSysSolver* self, const OSQPSettings* settings);
  void (*warm_start)(LinSysSolver* self, const OSQPVectorf* x);
  OSQPInt (*adjoint_derivative)(LinSysSolver* self);
  void (*free)(LinSysSolver* self);
  OSQPInt (*update_matrices)(LinSysSolver* self, const OSQPMatrix* P, const OSQPInt* Px_new_idx,
                             OSQPInt P_new_n, const OSQPMatrix* A, const OSQPInt* Ax_new_idx,
                             OSQPInt A_new_n);
  OSQPInt (*update_rho_vec)(LinSysSolver* self, const OSQPVectorf* rho_vec, OSQPFloat rho_sc);
  OSQPInt nthreads;
};

#ifdef __cplusplus
}
#endif

#endif /* OSQP_GB300_ALGEBRA_H */
