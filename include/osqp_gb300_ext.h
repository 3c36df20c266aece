/*
 * osqp_gb300_ext.h -- entry points of the GB300 library beyond OSQP's API.
 *
 * These have no counterpart in the reference's public API; they expose what
 * the device engine measures or adds (statistics of the last solve, the
 * block-Jacobi preconditioner, the batched many-QP solver, the
 * request-serving loop).
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

/* Interrupt the solve running on `solver` (from another thread): the solve
 * stops at its next ADMM iteration with status OSQP_SIGINT, stores no
 * solution and osqp_solve returns 1, as after Ctrl-C (osqp_api.c:728-737).
 * osqp_solve itself turns a SIGINT that arrives while it runs into the same
 * request; the previous SIGINT handler is restored when it returns.  A request
 * counts for the solve in progress only.  Returns 0 on success. */
OSQPInt osqp_gb300_interrupt(OSQPSolver* solver);

/* Row structure the set-up derived from the caller's CSC arrays (host
 * copies, for inspection; no reference counterpart -- the reference builds
 * the same arrays with csr_triu_to_full / csr_transpose,
 * algebra/cuda/src/cuda_csr.cu:489-628): which = 0 the full symmetric P with an
 * explicit diagonal (n rows), 1 the rows of A (m rows).  rowptr (rows + 1),
 * col and src (entries: row entry e holds input value src[e] of the upper
 * triangle of P / of A, or -1 for a structural diagonal), diag (which = 0: n
 * positions of the diagonal entries).  Any pointer may be NULL.  Returns the
 * number of entries, or -1. */
OSQPInt osqp_gb300_structure(OSQPSolver* solver, OSQPInt which, OSQPInt* rowptr, OSQPInt* col, OSQPInt* src,
                             OSQPInt* diag);

/* ---- Block-Jacobi preconditioner -------------------------------------------
 * settings->cg_precond = OSQP_GB300_BLOCK_DIAGONAL_PRECONDITIONER (an
 * extension of osqp_precond_type, include/public/osqp_api_constants.h:66-69,
 * which has the none and diagonal values only) preconditions the reduced-KKT
 * PCG with the inverted 32 x 32 diagonal blocks of K = P + sigma I + A' R A
 * (variables [32 b, 32 b + 32)), rebuilt on the device whenever rho changes.
 * Accepted by osqp_setup, osqp_update_settings, the batched solver and the
 * algebra library's linear-system solver.  The polish keeps the diagonal
 * preconditioner. */
#define OSQP_GB300_BLOCK_DIAGONAL_PRECONDITIONER 2

/* Copies the current block-Jacobi blocks of M^-1 (scaled problem) into `out`
 * (host or device memory; ceil(n / 32) * 1024 values, block b at 1024 b,
 * entry (j, i) at 32 j + i, zeros past n) and returns the number of values; `out` NULL
 * returns the count only.  Returns 0 when the solver has no blocks. */
OSQPInt osqp_gb300_precond_blocks(OSQPSolver* solver, OSQPFloat* out);

/* ---- Batched solver --------------------------------------------------------
 * Many independent QPs of uneven size solved in one persistent launch: a CTA
 * (or a thread-block cluster) runs the complete OSQP algorithm (scaling, ADMM,
 * reduced-KKT PCG, termination, adaptive rho) for one QP at a time, pulling
 * QPs from a device work queue ordered by decreasing size; QPs still running
 * after a fixed ADMM iteration continue on a cluster of CTAs.  A QP's result
 * does not depend on the other QPs of the batch.
 *
 * Packed input: for QP k with sizes n[k], m[k]
 *   P: upper-triangular CSC, column pointers Pp (n[k]+1 entries, starting at 0)
 *      concatenated over k; row indices Pi and values Px concatenated.
 *   A: CSC, likewise Ap / Ai / Ax.
 *   q concatenated (sum n), l and u concatenated (sum m).
 * Pointers may be host or device memory.  Settings apply to every QP.
 * linsys_solver selects the linear-system solver of every QP:
 *   OSQP_INDIRECT_SOLVER  the reduced-KKT PCG of the reference's CUDA backend
 *                         (algebra/cuda/lin_sys/indirect/cuda_pcg.cu:113-208);
 *   OSQP_DIRECT_SOLVER    an exact factorisation of K = P + sigma I + A' R A,
 *                         refreshed on every rho change, as the builtin backend
 *                         factors its KKT matrix (algebra/_common/lin_sys/qdldl/
 *                         qdldl_interface.c:216-530): a block-tridiagonal LDL'
 *                         in a level-set ordering, held per QP in device memory
 *                         and factored / applied by the QP's CTA on chip.  Set-up
 *                         returns OSQP_LINSYS_SOLVER_INIT_ERROR when a QP's
 *                         ordering has a block larger than the on-chip limit
 *                         (about 100 variables: dense couplings such as a budget
 *                         row over all assets); such QPs take the indirect solver.
 *                         A non-positive pivot (K not positive definite) ends
 *                         that QP with status OSQP_NON_CVX.
 * A batch is used by one host thread at a time (the server below owns the
 * pools it serves). */
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

/* New values of QP k's P entries (upper triangle, in the order given at setup)
 * and A entries; replaces osqp_update_data_mat (include/public/osqp_api_functions.h,
 * src/osqp_api.c:1309-1409) for one QP of a batch, with its arguments: NULL
 * values leave a matrix unchanged, NULL indices with a count of 0 or of all
 * entries update every entry in order.  Returns 1 / 2 for a bad P / A count
 * (as the reference), OSQP_DATA_VALIDATION_ERROR for k or an index out of
 * range (nothing changed).  QP k is re-scaled and refactored (direct solver)
 * or its preconditioner rebuilt, with rho and its iterates kept.  A pool of a
 * server may be updated while none of its requests is in flight. */
OSQPInt osqp_gb300_batch_update_data_mat(OSQPBatch* batch, OSQPInt k, const OSQPFloat* Px_new,
                                         const OSQPInt* Px_new_idx, OSQPInt P_new_n, const OSQPFloat* Ax_new,
                                         const OSQPInt* Ax_new_idx, OSQPInt A_new_n);

/* Solve all QPs (cold or warm start per settings->warm_starting). */
OSQPInt osqp_gb300_batch_solve(OSQPBatch* batch);

/* Packed results: x (sum n), y (sum m), and per-QP status, iterations,
 * objective, primal and dual residual.  Any pointer may be NULL; pointers may
 * be host or device memory. */
OSQPInt osqp_gb300_batch_get_solution(OSQPBatch* batch, OSQPFloat* x, OSQPFloat* y, OSQPInt* status,
                                      OSQPInt* iter, OSQPFloat* obj_val, OSQPFloat* prim_res,
                                      OSQPFloat* dual_res);

/* SpMV tile autotuner: times a short solve (probe_iter ADMM iterations; <= 0
 * means 60) of a sample of the batch for several targets of matrix entries
 * per lane of a row's sub-warp (8, 4, 16), keeps the fastest for every later
 * solve (the default 8 unless another is more than 3 % faster) and returns it
 * in *per_lane (may be NULL).  Every iterate and scalar of the
 * batch is restored afterwards.  The tile changes the summation order inside
 * a row, so results are reproducible for a given tile; the default tile
 * (OSQP_GB300_LANE_TARGET, 8) does not depend on the batch. */
OSQPInt osqp_gb300_batch_autotune(OSQPBatch* batch, OSQPInt probe_iter, OSQPInt* per_lane);

/* Device time of the last batch solve (ms), total ADMM and PCG iterations. */
OSQPInt osqp_gb300_batch_stats(OSQPBatch* batch, double* kernel_ms, long long* admm_iter,
                               long long* pcg_iter);

/* Device time (ms) from the start of the last osqp_gb300_batch_update_data_vec
 * to the end of the following solve (equals the solve time without an update). */
OSQPInt osqp_gb300_batch_step_ms(OSQPBatch* batch, double* step_ms);

/* Device time of every QP's last solve in seconds, from its first ADMM
 * iteration to its last (count entries, host memory; a QP that moved to the
 * tail form counts the time in between). */
OSQPInt osqp_gb300_batch_qp_seconds(OSQPBatch* batch, double* seconds);

/* PCG iterations of every QP in the last batch solve (count entries, host memory). */
OSQPInt osqp_gb300_batch_pcg_iters(OSQPBatch* batch, long long* pcg_iter);

/* The row structure of QP k of a batch, as osqp_gb300_structure describes
 * (positions relative to the QP's own arrays). */
OSQPInt osqp_gb300_batch_structure(OSQPBatch* batch, OSQPInt k, OSQPInt which, OSQPInt* rowptr, OSQPInt* col,
                                   OSQPInt* src, OSQPInt* diag);

/* SM clock cycles of the last batch solve summed over its QPs, per phase of
 * the ADMM iteration: right-hand side, linear solve, x / z / y updates,
 * residuals and termination, refactorisation; of the direct solve's block
 * steps the waits for factor segments, the barriers, the forward and the
 * backward sweep; the sparse products of the right-hand side and of the
 * updates; the issuing of the direct solve's bulk copies (cycles[0..11],
 * thread 0's view, the last by the issuing thread), then counts of direct
 * solves: all, through the bulk-copy ring, and of those the ones that read
 * the factor from global memory after a failed wait (cycles[12..14]), and
 * the cycles thread 0 spends in the block products of the sweeps
 * (cycles[15]); zeros unless the
 * batch was set up with OSQP_GB300_PROFILE=1 in the environment).  No
 * reference counterpart (the reference's profiler_level times host phases). */
OSQPInt osqp_gb300_batch_phase_cycles(OSQPBatch* batch, double* cycles);

/* rho updates of every QP in the last batch solve (count entries, host memory;
 * OSQPInfo.rho_updates, include/public/osqp_api_types.h:165). */
OSQPInt osqp_gb300_batch_rho_updates(OSQPBatch* batch, OSQPInt* rho_updates);

/* Elements of every QP's direct-solver factor (count entries, host memory; 0
 * for the indirect solver): the bytes one direct solve reads, over the value
 * width.  No reference counterpart. */
OSQPInt osqp_gb300_batch_factor_elems(OSQPBatch* batch, long long* elems);

/* Direct solver in the diagonal-plus-dense-rows form (a QP whose constraint
 * rows couple too many variables for the block-tridiagonal ordering, with a
 * diagonal P): for QP k of a batch, *r = its dense rows (rows of A with two or
 * more entries; 0 when the QP uses the block form or the PCG), and, where the
 * pointers are not NULL, the rows (r entries), the inverse capacitance matrix
 * (R_d^-1 + A_d Dg^-1 A_d')^-1 (r x r, row-major) and Dg^-1 (n entries) of the
 * scaled problem for the current rho.  No reference counterpart. */
OSQPInt osqp_gb300_batch_dense_rows(OSQPBatch* batch, OSQPInt k, OSQPInt* r, OSQPInt* rows, OSQPFloat* cinv,
                                    OSQPFloat* dginv);

OSQPInt osqp_gb300_batch_cleanup(OSQPBatch* batch);

/* Ordering of the direct solver for one QP (host memory; no device work):
 * P upper-triangular CSC (Pp, Pi), A CSC (Ap, Ai) with m rows.  On return
 * *nblocks blocks, block_start[0..*nblocks] (n + 1 entries of room) and perm
 * (n entries: permuted position -> variable).  In this order every entry of
 * P + A'A lies in a diagonal block or a first off-diagonal block.  Returns 0,
 * 1 when a block would exceed bmax_limit variables, 2 on inconsistent input.
 * No reference counterpart: the builtin orders its KKT matrix with AMD
 * (algebra/_common/lin_sys/qdldl/qdldl_interface.c:94-116). */
OSQPInt osqp_gb300_kkt_plan(OSQPInt n, OSQPInt m, const OSQPInt* Pp, const OSQPInt* Pi, const OSQPInt* Ap,
                            const OSQPInt* Ai, OSQPInt bmax_limit, OSQPInt* nblocks, OSQPInt* block_start,
                            OSQPInt* perm);

/* ---- Request serving (continuous batching) ---------------------------------
 * A server owns a worker thread and `concurrency` CUDA streams.  QPs are made
 * resident as pools (batches set up with osqp_gb300_batch_setup; set-up is
 * refused with OSQP_MEM_ALLOC_ERROR when free device memory does not hold the
 * pool): structures, scaling, preconditioner and warm-start iterates stay in
 * device memory between requests.  A request names a pool, a QP of it and
 * optional new q / l / u (host memory, QP-sized; NULL keeps the current
 * vector).  Requests that arrive while others are on the device are launched
 * as soon as a stream is free: every free stream takes the waiting requests of
 * one pool (at most one per QP at a time, at most the pool's resident CTA
 * slots / concurrency) as one launch, so work from different arrivals
 * overlaps on the device.  A request's result is the same whatever
 * else is in flight.  Pools may be added while the server runs: a QP of a
 * structure no pool holds is admitted by setting it up as a one-QP pool (the
 * per-request counterpart of osqp_setup).  A pool served by a server must not
 * be used through the batch calls while any of its requests is in flight. */
typedef struct OSQPServer_ OSQPServer;

OSQPInt osqp_gb300_server_create(OSQPServer** server, OSQPInt concurrency);

/* Register a pool; returns its id in *pool_id. */
OSQPInt osqp_gb300_server_add_pool(OSQPServer* server, OSQPBatch* pool, OSQPInt* pool_id);

/* Queue a solve of QP `qp` of pool `pool_id`; returns a ticket.  The vectors
 * are copied before the call returns. */
OSQPInt osqp_gb300_server_submit(OSQPServer* server, OSQPInt pool_id, OSQPInt qp, const OSQPFloat* q,
                                 const OSQPFloat* l, const OSQPFloat* u, long long* ticket);

/* Wait for a ticket; copies x (QP-sized, host memory, may be NULL), status,
 * iterations, objective and the request's latency in ms (submission to
 * results on the host).  Each ticket can be waited for once.  Returns 0, or
 * OSQP_ALGEBRA_LOAD_ERROR once a launch of the server has failed: from then
 * on every waiting and later request completes with status OSQP_UNSOLVED. */
OSQPInt osqp_gb300_server_wait(OSQPServer* server, long long ticket, OSQPFloat* x, OSQPInt* status,
                               OSQPInt* iter, OSQPFloat* obj_val, double* latency_ms);

/* Stop the worker after the queued requests complete and free the server
 * (the pools stay owned by the caller).  Call it after every ticket has been
 * waited for; tickets not waited for are discarded. */
OSQPInt osqp_gb300_server_destroy(OSQPServer* server);

#ifdef __cplusplus
}
#endif

#endif
