/*
 * osqp_gb300_ext.h -- entry points of the GB300 library beyond OSQP's API.
 *
 * These have no counterpart in the reference's public API; they expose what
 * the device engine measures or adds (statistics of the last solve, the
 * batched many-QP solver, the request-serving loop).
 */
#ifndef OSQP_GB300_EXT_H
#define OSQP_GB300_EXT_H

#include "osqp_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Statistics of the last osqp_solve: ADMM iterations, total PCG iterations,
 * device time of the solve kernel (ms) and the execution form used
 * (0 = one CTA, 1 = cooperative grid, k > 1 = one cluster of k CTAs).
 * Returns 0 on success. */
OSQPInt osqp_gb300_solve_stats(OSQPSolver* solver, OSQPInt* admm_iter, long long* pcg_iter,
                               double* kernel_ms, OSQPInt* grid_form);

/* ---- Batched solver --------------------------------------------------------
 * Many independent QPs of uneven size solved in one persistent launch: one
 * CTA runs the complete OSQP algorithm (scaling, ADMM, reduced-KKT PCG,
 * termination, adaptive rho) for one QP at a time, pulling QPs from a device
 * work queue ordered by decreasing size.  Results are identical to solving
 * each QP alone with the same settings (same launch shape per QP).
 *
 * Packed input: for QP k with sizes n[k], m[k]
 *   P: upper-triangular CSC, column pointers Pp (n[k]+1 entries, starting at 0)
 *      concatenated over k; row indices Pi and values Px concatenated.
 *   A: CSC, likewise Ap / Ai / Ax.
 *   q concatenated (sum n), l and u concatenated (sum m).
 * Pointers may be host or device memory.  Settings apply to every QP
 * (linsys_solver must be OSQP_INDIRECT_SOLVER). */
typedef struct OSQPBatch_ OSQPBatch;

OSQPInt osqp_gb300_batch_setup(OSQPBatch** batchp, OSQPInt count, const OSQPInt* n, const OSQPInt* m,
                               const OSQPInt* Pp, const OSQPInt* Pi, const OSQPFloat* Px,
                               const OSQPInt* Ap, const OSQPInt* Ai, const OSQPFloat* Ax,
                               const OSQPFloat* q, const OSQPFloat* l, const OSQPFloat* u,
                               const OSQPSettings* settings);

/* New q / l / u for every QP (packed as in setup; any may be NULL).  Bounds are
 * checked per QP; returns OSQP_DATA_VALIDATION_ERROR if some l > u, leaving
 * the previous vectors in place. */
OSQPInt osqp_gb300_batch_update_data_vec(OSQPBatch* batch, const OSQPFloat* q, const OSQPFloat* l,
                                         const OSQPFloat* u);

/* Solve all QPs (cold or warm start per settings->warm_starting). */
OSQPInt osqp_gb300_batch_solve(OSQPBatch* batch);

/* Packed results: x (sum n), y (sum m), and per-QP status, iterations,
 * objective, primal and dual residual.  Any pointer may be NULL; pointers may
 * be host or device memory. */
OSQPInt osqp_gb300_batch_get_solution(OSQPBatch* batch, OSQPFloat* x, OSQPFloat* y, OSQPInt* status,
                                      OSQPInt* iter, OSQPFloat* obj_val, OSQPFloat* prim_res,
                                      OSQPFloat* dual_res);

/* Device time of the last batch solve (ms), total ADMM and PCG iterations. */
OSQPInt osqp_gb300_batch_stats(OSQPBatch* batch, double* kernel_ms, long long* admm_iter,
                               long long* pcg_iter);

/* Device time (ms) from the start of the last osqp_gb300_batch_update_data_vec
 * to the end of the following solve (equals the solve time without an update). */
OSQPInt osqp_gb300_batch_step_ms(OSQPBatch* batch, double* step_ms);

/* PCG iterations of every QP in the last batch solve (count entries, host memory). */
OSQPInt osqp_gb300_batch_pcg_iters(OSQPBatch* batch, long long* pcg_iter);

OSQPInt osqp_gb300_batch_cleanup(OSQPBatch* batch);

#ifdef __cplusplus
}
#endif

#endif
