/*
 * Test infrastructure (oracle only; never linked into the GB300 library).
 *
 * Sparse LDL^T interface with the call signatures that OSQP's direct linear
 * system solver uses (algebra/_common/lin_sys/qdldl/qdldl_interface.c:94,116,409).
 * QDLDL v0.1.8 itself is a FetchContent download
 * (algebra/_common/lin_sys/qdldl/qdldl.cmake:6-10) that is not available
 * offline, so the three entry points are re-implemented in ldl_compat.c from
 * the published up-looking LDL^T method (T. A. Davis, "Direct Methods for
 * Sparse Linear Systems", SIAM 2006, ch. 4: elimination tree, row patterns by
 * tree reach, column-by-column fill of L).
 */
#ifndef OSQP_ORACLE_QDLDL_H
#define OSQP_ORACLE_QDLDL_H

#include "qdldl_types.h"

#define QDLDL_VERSION_MAJOR 0
#define QDLDL_VERSION_MINOR 1
#define QDLDL_VERSION_PATCH 8

#ifdef __cplusplus
extern "C" {
#endif

/* Elimination tree and column counts of L for an upper-triangular CSC matrix.
 * Returns sum(Lnz), -1 if an entry lies below the diagonal or a column is
 * empty, -2 if the count overflows QDLDL_int. */
QDLDL_int QDLDL_etree(const QDLDL_int n, const QDLDL_int* Ap, const QDLDL_int* Ai,
                      QDLDL_int* work, QDLDL_int* Lnz, QDLDL_int* etree);

/* Numeric factorisation A = L D L^T (L unit lower triangular, stored without
 * its diagonal).  Returns the number of positive entries of D, or -1 if a
 * zero pivot occurs. */
QDLDL_int QDLDL_factor(const QDLDL_int n, const QDLDL_int* Ap, const QDLDL_int* Ai,
                       const QDLDL_float* Ax, QDLDL_int* Lp, QDLDL_int* Li,
                       QDLDL_float* Lx, QDLDL_float* D, QDLDL_float* Dinv,
                       const QDLDL_int* Lnz, const QDLDL_int* etree,
                       QDLDL_bool* bwork, QDLDL_int* iwork, QDLDL_float* fwork);

/* In-place solve x <- (L D L^T)^{-1} x. */
void QDLDL_solve(const QDLDL_int n, const QDLDL_int* Lp, const QDLDL_int* Li,
                 const QDLDL_float* Lx, const QDLDL_float* Dinv, QDLDL_float* x);

#ifdef __cplusplus
}
#endif

#endif
