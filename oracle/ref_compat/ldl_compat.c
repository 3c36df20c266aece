/*
 * Test infrastructure (oracle only; never linked into the GB300 library).
 *
 * Up-looking sparse LDL^T (Davis 2006, ch. 4) behind the QDLDL v0.1.8 entry
 * points declared in qdldl.h.  Used when building OSQP's builtin algebra
 * from the reference sources (oracle/Makefile, target "ref") and by the
 * oracle restatement (oracle/osqp_oracle.c) through the same file.
 *
 *   etree  : for every column k, walk the elimination tree upward from each
 *            off-diagonal row index i < k of A(:,k) until a node already
 *            visited for k; every node on the walk gains one entry L(k,node).
 *   factor : row k of L solves L(0:k-1,0:k-1) D y = A(0:k-1,k) on the pattern
 *            given by the same tree walk, visited in topological order.
 *   solve  : forward substitution with L, scaling by D^{-1}, backward with L^T.
 */
#include "qdldl.h"

#define LDL_UNUSED (-1)

QDLDL_int QDLDL_etree(const QDLDL_int n, const QDLDL_int* Ap, const QDLDL_int* Ai,
                      QDLDL_int* work, QDLDL_int* Lnz, QDLDL_int* etree) {
  QDLDL_int k, p, i;
  QDLDL_int total = 0;

  for (k = 0; k < n; k++) {
    work[k]  = LDL_UNUSED;  /* last column that visited node k */
    Lnz[k]   = 0;
    etree[k] = LDL_UNUSED;
  }

  for (k = 0; k < n; k++) {
    if (Ap[k] == Ap[k + 1]) return -1;   /* column without any entry */
    work[k] = k;
    for (p = Ap[k]; p < Ap[k + 1]; p++) {
      i = Ai[p];
      if (i > k) return -1;              /* entry below the diagonal */
      /* climb until a node already reached from column k */
      while (work[i] != k) {
        if (etree[i] == LDL_UNUSED) etree[i] = k;
        Lnz[i]++;
        work[i] = k;
        i = etree[i];
      }
    }
  }

  for (k = 0; k < n; k++) {
    if (total > QDLDL_INT_MAX - Lnz[k]) return -2;
    total += Lnz[k];
  }
  return total;
}

QDLDL_int QDLDL_factor(const QDLDL_int n, const QDLDL_int* Ap, const QDLDL_int* Ai,
                       const QDLDL_float* Ax, QDLDL_int* Lp, QDLDL_int* Li,
                       QDLDL_float* Lx, QDLDL_float* D, QDLDL_float* Dinv,
                       const QDLDL_int* Lnz, const QDLDL_int* etree,
                       QDLDL_bool* bwork, QDLDL_int* iwork, QDLDL_float* fwork) {
  /* Workspace split: iwork = [ pattern (n) | path stack (n) | fill cursor (n) ] */
  QDLDL_int*   pattern = iwork;
  QDLDL_int*   stack   = iwork + n;
  QDLDL_int*   cursor  = iwork + 2 * n;
  QDLDL_bool*  seen    = bwork;
  QDLDL_float* y       = fwork;
  QDLDL_int k, p, i, t, depth, npat, col, q, positives = 0;
  QDLDL_float yc, lk;

  Lp[0] = 0;
  for (k = 0; k < n; k++) {
    Lp[k + 1] = Lp[k] + Lnz[k];
    cursor[k] = Lp[k];
    seen[k]   = 0;
    y[k]      = 0.0;
  }

  for (k = 0; k < n; k++) {
    npat = 0;
    D[k] = 0.0;

    /* Scatter column k of A and collect the row pattern of L(k,:) */
    for (p = Ap[k]; p < Ap[k + 1]; p++) {
      i = Ai[p];
      if (i == k) { D[k] = Ax[p]; continue; }
      y[i] = Ax[p];
      depth = 0;
      while (i != LDL_UNUSED && i < k && !seen[i]) {
        seen[i] = 1;
        stack[depth++] = i;
        i = etree[i];
      }
      /* append the walk so that descendants end up after their ancestors */
      for (t = depth - 1; t >= 0; t--) pattern[npat++] = stack[t];
    }

    /* Sparse triangular solve on the pattern, descendants first */
    for (t = npat - 1; t >= 0; t--) {
      col = pattern[t];
      yc  = y[col];
      for (q = Lp[col]; q < cursor[col]; q++) {
        y[Li[q]] -= Lx[q] * yc;
      }
      lk = yc * Dinv[col];
      Li[cursor[col]] = k;
      Lx[cursor[col]] = lk;
      cursor[col]++;
      D[k] -= yc * lk;
      y[col]    = 0.0;
      seen[col] = 0;
    }

    if (D[k] == 0.0) return -1;
    if (D[k] > 0.0) positives++;
    Dinv[k] = 1.0 / D[k];
  }
  return positives;
}

void QDLDL_solve(const QDLDL_int n, const QDLDL_int* Lp, const QDLDL_int* Li,
                 const QDLDL_float* Lx, const QDLDL_float* Dinv, QDLDL_float* x) {
  QDLDL_int i, q;
  for (i = 0; i < n; i++) {
    QDLDL_float xi = x[i];
    for (q = Lp[i]; q < Lp[i + 1]; q++) x[Li[q]] -= Lx[q] * xi;
  }
  for (i = 0; i < n; i++) x[i] *= Dinv[i];
  for (i = n - 1; i >= 0; i--) {
    QDLDL_float acc = x[i];
    for (q = Lp[i]; q < Lp[i + 1]; q++) acc -= Lx[q] * x[Li[q]];
    x[i] = acc;
  }
}
