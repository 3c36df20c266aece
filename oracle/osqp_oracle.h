/*
 * Test infrastructure: FP64 CPU oracle for OSQP.  Only tests/, the package's
 * smoke check and bench.py's CPU-baseline leg load it; the GB300 library never
 * links it.
 *
 * liboracle.so exports the same public API as OSQP 1.0
 * (include/public/osqp_api_functions.h) with OSQPFloat = double and
 * OSQPInt = int32, so one ctypes binding drives the oracle, the reference
 * build in oracle/_ref and the GB300 library alike.
 *
 * Defaults are those of the reference's builtin algebra (rho_is_vec 1,
 * check_termination 25, adaptive_rho_tolerance 5, OSQP_INFTY 1e30;
 * include/public/osqp_api_constants.h:111-178).  Both linear-system modes
 * exist: OSQP_DIRECT_SOLVER factors the quasi-definite KKT matrix with a
 * sparse LDL^T after a minimum-degree ordering (as builtin QDLDL does after
 * AMD), OSQP_INDIRECT_SOLVER runs the reduced-KKT preconditioned CG with the
 * tolerance policy of algebra/cuda/lin_sys/indirect/cuda_pcg_interface.cu:32-64.
 */
#ifndef OSQP_ORACLE_H
#define OSQP_ORACLE_H
#include "../include/osqp_gb300.h"
#endif
