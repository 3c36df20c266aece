// gb_kkt_plan.h -- host-side symbolic analysis of the direct KKT solve.
//
// The direct linear-system solver (linsys_solver = OSQP_DIRECT_SOLVER)
// factors the reduced KKT matrix K = P + sigma I + A' R A of every ADMM step
// exactly (reference: the builtin QDLDL path factors the quasi-definite
// [P + sigma I, A'; A, -R^-1], algebra/_common/lin_sys/qdldl/qdldl_interface.c:
// 216-382; eliminating its constraint block first gives this K, whose
// factorisation gives the same x~ and z~ = A x~, qdldl_interface.c:394-466).
//
// Ordering.  The variables are split into consecutive blocks such that K is
// block tridiagonal: the level sets of a breadth-first search of K's graph
// (variables adjacent when P couples them or a row of A holds both) from a
// pseudo-peripheral variable (George & Liu, "An implementation of a
// pseudoperipheral node finder", ACM TOMS 5, 1979).  Edges of a BFS only join
// equal or neighbouring levels, so every entry of K lies in a diagonal or
// first off-diagonal block.  Two refinements: a variable whose neighbours all
// lie in the previous level may move two levels down (the ends of a
// horizon in MPC, which BFS from the far end files one stage late), and
// neighbouring blocks are merged while they stay small.  On a stacked MPC QP
// the blocks are the stages (x_k, u_k), so the factor costs
// O(T (nx + nu)^3) and each solve O(T (nx + nu)^2).
//
// Storage of the factor (elements of OSQPFloat; every segment padded to a
// multiple of 4 elements, so each starts on a 16-byte boundary and can be
// fetched by one bulk copy), block k of size b_k after one of size b_{k-1}:
//   forward segment k   [ G_k (b_k x b_{k-1}) | S_k^-1 (b_k x b_k) ]   at fo[k]
//   backward segment k  [ G_k' (b_{k-1} x b_k) ]                        at bo[k]
// with G_k = K_{k,k-1} S_{k-1}^-1 and S_k = K_kk - G_k K_{k,k-1}' (block LDL').
// The forward sweep of a solve reads the forward segments in order, the
// backward sweep the backward segments in reverse order.
#pragma once

#include <algorithm>
#include <cstdint>
#include <cstdlib>
#include <vector>

#if defined(__CUDACC__)
#define GB_KKT_HD __host__ __device__
#else
#define GB_KKT_HD
#endif

namespace gb {

// Constraint rows gathered per assembly pass of a block, and the largest
// number of block entries one thread accumulates (kKktOutMax x threads >=
// b_k (b_k + b_{k-1})).
constexpr int kKktTileRows = 32;
constexpr int kKktOutMax = 24;
// Blocks are merged while the merged block stays at or below this size.
constexpr int kKktMergeTo = 32;

// Factor segments hold multiples of 4 elements.
GB_KKT_HD inline long long kkt_pad4(long long e) { return (e + 3) & ~3LL; }
// Ring slots of the solve's bulk-copy pipeline (0: the solve reads the factor
// from global memory directly).
constexpr int kKktRingMax = 16;

// On-chip workspace of the block factorisation (elements): S_{k-1}^-1, S_k,
// its sweep buffer, K_{k,k-1}, G_k, the assembly tile and its rho values.
GB_KKT_HD inline long long kkt_factor_ws_elems(int bmax) {
  return 5LL * bmax * bmax + (long long)kKktTileRows * 2 * bmax + kKktTileRows;
}
// Whole on-chip workspace of a direct solve: the factorisation's, or the
// ADMM iteration's, whichever is larger.  The iteration's: two permuted
// n-vectors of the block solve, `ring` slots of segmax elements, then the
// vectors the sparse products gather -- x~ (n) and w = rho z - y (m).
GB_KKT_HD inline long long kkt_iter_ws_elems(int n, int m, int segmax, int ring) {
  return kkt_pad4(2LL * n) + (long long)ring * segmax + kkt_pad4(n) + kkt_pad4(m);
}
GB_KKT_HD inline long long kkt_ws_elems(int n, int m, int bmax, int segmax, int ring) {
  const long long f = kkt_factor_ws_elems(bmax), v = kkt_iter_ws_elems(n, m, segmax, ring);
  return kkt_pad4(f > v ? f : v);
}
// Bytes of the whole workspace: the elements above, then copies of the block
// starts and the forward / backward segment offsets (3 (nb + 1) ints) that
// every block step reads, and of the permutation and its inverse (2 n ints)
// that every right-hand side and solution passes through.
GB_KKT_HD inline long long kkt_ws_bytes(int n, int m, int bmax, int nb, int segmax, int ring, int elem) {
  return kkt_ws_elems(n, m, bmax, segmax, ring) * elem + 12LL * (nb + 1) + 8LL * n;
}

struct KktPlan {
  int n = 0, nb = 0, bmax = 0;
  std::vector<int> perm;    // permuted position -> variable
  std::vector<int> iperm;   // variable -> permuted position
  std::vector<int> bs;      // [nb + 1] block starts (permuted positions)
  std::vector<int> fo;      // [nb + 1] forward segment offsets (elements); fo[nb] = start of the backward ones
  std::vector<int> bo;      // [nb + 1] backward segment offsets (bo[0] unused)
  int segmax = 0;           // largest segment (elements)
  std::vector<int> co;      // [nb + 1] offsets of the blocks' constraint lists in cr
  std::vector<int> cr;      // per block, ascending: rows of A with >= 2 entries touching it
  long long fsize = 0;      // factor elements
};

// Build the plan of one QP.  P: upper-triangular CSC (Pp, Pi), A: m x n CSC
// (Ap, Ai).  Returns 0, or 1 when a block would exceed bmax_limit variables
// (the direct solver does not apply), 2 on inconsistent structure.
inline int kkt_plan_build(int n, int m, const int* Pp, const int* Pi, const int* Ap, const int* Ai,
                          int bmax_limit, KktPlan& pl) {
  pl = KktPlan();
  pl.n = n;
  if (n <= 0 || m < 0) return 2;
  // rows of A (CSR pattern), ascending columns
  std::vector<int> rp(m + 1, 0), rc((size_t)Ap[n]);
  for (int j = 0; j < n; j++)
    for (int e = Ap[j]; e < Ap[j + 1]; e++) {
      if (Ai[e] < 0 || Ai[e] >= m) return 2;
      rp[Ai[e] + 1]++;
    }
  for (int r = 0; r < m; r++) rp[r + 1] += rp[r];
  {
    std::vector<int> fill(rp.begin(), rp.end() - 1);
    for (int j = 0; j < n; j++)
      for (int e = Ap[j]; e < Ap[j + 1]; e++) rc[fill[Ai[e]]++] = j;
  }
  // off-diagonal adjacency of P (both directions)
  std::vector<int> pp(n + 1, 0);
  for (int j = 0; j < n; j++)
    for (int e = Pp[j]; e < Pp[j + 1]; e++) {
      const int i = Pi[e];
      if (i < 0 || i > j) return 2;
      if (i != j) { pp[i + 1]++; pp[j + 1]++; }
    }
  for (int i = 0; i < n; i++) pp[i + 1] += pp[i];
  std::vector<int> pc((size_t)pp[n]);
  {
    std::vector<int> fill(pp.begin(), pp.end() - 1);
    for (int j = 0; j < n; j++)
      for (int e = Pp[j]; e < Pp[j + 1]; e++) {
        const int i = Pi[e];
        if (i != j) { pc[fill[i]++] = j; pc[fill[j]++] = i; }
      }
  }
  auto rowlen = [&](int r) { return rp[r + 1] - rp[r]; };
  // degree estimate: P neighbours plus the other entries of its rows
  std::vector<long long> deg(n, 0);
  for (int v = 0; v < n; v++) {
    long long d = pp[v + 1] - pp[v];
    for (int e = Ap[v]; e < Ap[v + 1]; e++) d += rowlen(Ai[e]) - 1;
    deg[v] = d;
  }

  // BFS over the variables; a row of A is expanded once per search.
  std::vector<int> vstamp(n, 0), rstamp(m, 0), level(n, -1);
  int stamp = 0;
  std::vector<char> done(n, 0);
  std::vector<int> order;          // BFS order of the current search
  std::vector<int> lstart;         // level starts in `order`
  auto bfs = [&](int root) {
    stamp++;
    order.clear(); lstart.clear();
    order.push_back(root); vstamp[root] = stamp;
    lstart.push_back(0);
    size_t head = 0;
    while (head < order.size()) {
      const size_t lend = order.size();
      lstart.push_back((int)lend);
      for (; head < lend; head++) {
        const int v = order[head];
        for (int e = pp[v]; e < pp[v + 1]; e++) {
          const int w = pc[e];
          if (!done[w] && vstamp[w] != stamp) { vstamp[w] = stamp; order.push_back(w); }
        }
        for (int e = Ap[v]; e < Ap[v + 1]; e++) {
          const int r = Ai[e];
          if (rstamp[r] == stamp || rowlen(r) < 2) continue;
          rstamp[r] = stamp;
          for (int f = rp[r]; f < rp[r + 1]; f++) {
            const int w = rc[f];
            if (!done[w] && vstamp[w] != stamp) { vstamp[w] = stamp; order.push_back(w); }
          }
        }
      }
      if (order.size() == lend) { lstart.pop_back(); break; }
    }
    lstart.push_back((int)order.size());
    return (int)lstart.size() - 1;   // number of levels
  };

  std::vector<std::vector<int>> blocks;
  std::vector<int> by_deg(n);
  for (int v = 0; v < n; v++) by_deg[v] = v;
  std::stable_sort(by_deg.begin(), by_deg.end(), [&](int a, int b) { return deg[a] < deg[b]; });
  size_t next_start = 0;
  int remaining = n;
  while (remaining > 0) {
    // start: unplaced variable of smallest degree
    while (done[by_deg[next_start]]) next_start++;
    const int start = by_deg[next_start];
    int root = start, nlev = bfs(root);
    for (int it = 0; it < 4; it++) {
      int cand = -1;
      for (int p = lstart[nlev - 1]; p < lstart[nlev]; p++) {
        const int v = order[p];
        if (cand < 0 || deg[v] < deg[cand]) cand = v;
      }
      const int nl2 = bfs(cand);
      if (nl2 <= nlev) { bfs(root); break; }
      root = cand; nlev = nl2;
    }
    // levels of this component (order / lstart hold the search from root)
    std::vector<std::vector<int>> lev(nlev);
    for (int l = 0; l < nlev; l++)
      for (int p = lstart[l]; p < lstart[l + 1]; p++) { lev[l].push_back(order[p]); level[order[p]] = l; }
    // refinement: a variable of level l >= 2 whose neighbours are all in
    // level l - 1 may move to level l - 2 (its neighbours then lie in the
    // level above it); moved while that balances the two levels
    for (int l = 2; l < nlev; l++) {
      std::vector<int> movable;
      for (int v : lev[l]) {
        bool ok = true;
        for (int e = pp[v]; e < pp[v + 1] && ok; e++) ok = level[pc[e]] == l - 1;
        for (int e = Ap[v]; e < Ap[v + 1] && ok; e++) {
          const int r = Ai[e];
          for (int f = rp[r]; f < rp[r + 1] && ok; f++) {
            const int w = rc[f];
            if (w != v && level[w] != l - 1) ok = false;
          }
        }
        if (ok) movable.push_back(v);
      }
      const long long take = std::min<long long>((long long)movable.size(),
                                                 ((long long)lev[l].size() - (long long)lev[l - 2].size()) / 2);
      if (take <= 0) continue;
      for (long long t = 0; t < take; t++) {
        const int v = movable[t];
        level[v] = l - 2;
        lev[l - 2].push_back(v);
      }
      std::vector<int> keep;
      for (int v : lev[l]) if (level[v] == l) keep.push_back(v);
      lev[l].swap(keep);
    }
    for (auto& L : lev) {
      if (L.empty()) continue;
      std::sort(L.begin(), L.end());
      for (int v : L) { done[v] = 1; remaining--; }
      blocks.push_back(L);
    }
  }
  // merge neighbouring small blocks
  std::vector<std::vector<int>> merged;
  for (auto& B : blocks) {
    if (!merged.empty() && merged.back().size() + B.size() <= (size_t)kKktMergeTo)
      merged.back().insert(merged.back().end(), B.begin(), B.end());
    else
      merged.push_back(B);
  }
  pl.nb = (int)merged.size();
  pl.perm.reserve(n);
  pl.bs.push_back(0);
  for (auto& B : merged) {
    pl.bmax = std::max(pl.bmax, (int)B.size());
    pl.perm.insert(pl.perm.end(), B.begin(), B.end());
    pl.bs.push_back((int)pl.perm.size());
  }
  if ((int)pl.perm.size() != n) return 2;
  if (pl.bmax > bmax_limit) return 1;
  pl.iperm.assign(n, -1);
  for (int p = 0; p < n; p++) pl.iperm[pl.perm[p]] = p;
  std::vector<int> blk(n);
  for (int k = 0; k < pl.nb; k++)
    for (int p = pl.bs[k]; p < pl.bs[k + 1]; p++) blk[pl.perm[p]] = k;
  // every entry of K in a diagonal or first off-diagonal block
  for (int r = 0; r < m; r++) {
    if (rowlen(r) < 2) continue;
    int lo = pl.nb, hi = -1;
    for (int f = rp[r]; f < rp[r + 1]; f++) { lo = std::min(lo, blk[rc[f]]); hi = std::max(hi, blk[rc[f]]); }
    if (hi - lo > 1) return 2;
  }
  for (int v = 0; v < n; v++)
    for (int e = pp[v]; e < pp[v + 1]; e++)
      if (std::abs(blk[v] - blk[pc[e]]) > 1) return 2;
  // factor offsets: the forward segments, then the backward ones
  pl.fo.assign(pl.nb + 1, 0);
  pl.bo.assign(pl.nb + 1, 0);
  long long off = 0, smax = 0;
  for (int k = 0; k < pl.nb; k++) {
    const long long b = pl.bs[k + 1] - pl.bs[k], bp = k ? pl.bs[k] - pl.bs[k - 1] : 0;
    pl.fo[k] = (int)off;
    const long long seg = kkt_pad4(b * bp) + kkt_pad4(b * b);
    smax = std::max(smax, seg);
    off += seg;
    if (off > INT32_MAX) return 1;
  }
  pl.fo[pl.nb] = (int)off;
  for (int k = 1; k < pl.nb; k++) {
    const long long b = pl.bs[k + 1] - pl.bs[k], bp = pl.bs[k] - pl.bs[k - 1];
    pl.bo[k] = (int)off;
    off += kkt_pad4(b * bp);
    if (off > INT32_MAX) return 1;
  }
  pl.bo[0] = (int)off;
  pl.fsize = off;
  pl.segmax = (int)smax;
  // constraint rows (two or more entries) touching each block, ascending
  pl.co.assign(pl.nb + 1, 0);
  std::vector<int> rmark(m, -1);
  for (int k = 0; k < pl.nb; k++) {
    pl.co[k] = (int)pl.cr.size();
    std::vector<int> rows;
    for (int p = pl.bs[k]; p < pl.bs[k + 1]; p++) {
      const int v = pl.perm[p];
      for (int e = Ap[v]; e < Ap[v + 1]; e++) {
        const int r = Ai[e];
        if (rowlen(r) >= 2 && rmark[r] != k) { rmark[r] = k; rows.push_back(r); }
      }
    }
    std::sort(rows.begin(), rows.end());
    pl.cr.insert(pl.cr.end(), rows.begin(), rows.end());
  }
  pl.co[pl.nb] = (int)pl.cr.size();
  return 0;
}

// Largest block the device factorisation handles with `threads` threads and
// `ws_bytes` of on-chip workspace for elements of `elem` bytes.
inline int kkt_bmax_limit(int threads, long long ws_bytes, int elem) {
  int b = 1;
  while (true) {
    const int c = b + 1;
    if ((long long)c * 2 * c > (long long)kKktOutMax * threads) break;
    // the solve group (two halves of at least c threads, whole warps) and a producer warp
    if (2 * (c <= 32 ? 32 : ((c + 31) & ~31)) + 32 > threads) break;
    if (kkt_factor_ws_elems(c) * elem > ws_bytes) break;
    b = c;
  }
  return b;
}

// ---------------------------------------------------------------------------
// Diagonal-plus-dense-rows form (Woodbury).  When the block ordering does not
// apply -- a row of A couples most variables, as a budget row or the factor
// rows of a factor model do -- but P is diagonal, K splits into a diagonal and
// the rows of A with two or more entries ("dense rows"):
//   K = Dg + A_d' R_d A_d,   Dg = diag(P) + sigma + sum over single-entry rows
//                                  of rho_j a_j^2,
// and the builtin's quasi-definite KKT system restricted to the dense rows is
// solved by eliminating x:  C nu = A_d Dg^-1 b_s - (z_d - R_d^-1 y_d),
// x~ = Dg^-1 (b_s - A_d' nu),  C = R_d^-1 + A_d Dg^-1 A_d'  (b_s: the
// right-hand side without the dense rows), with C (r x r, r dense rows)
// inverted once per factorisation.  A solve is then two sparse products over
// the dense rows and one dense r x r product.
// ---------------------------------------------------------------------------
// Most dense rows of the form: C^-1 holds r^2 values per QP and a
// factorisation costs about r^3 + r nnz(A_d) multiply-adds.
constexpr int kDrMaxRows = 512;

struct DrPlan {
  int r = 0;
  std::vector<int> rows;   // ascending rows of A with two or more entries
};

// 0 on success; 1 when P has an off-diagonal entry or there are more than rmax
// dense rows (the form does not apply); 2 on inconsistent structure.
inline int dr_plan_build(int n, int m, const int* Pp, const int* Pi, const int* Ap, const int* Ai, int rmax,
                         DrPlan& pl) {
  pl = DrPlan();
  if (n <= 0 || m < 0) return 2;
  for (int j = 0; j < n; j++)
    for (int e = Pp[j]; e < Pp[j + 1]; e++) {
      if (Pi[e] < 0 || Pi[e] > j) return 2;
      if (Pi[e] != j) return 1;
    }
  std::vector<int> len(m, 0);
  for (int j = 0; j < n; j++)
    for (int e = Ap[j]; e < Ap[j + 1]; e++) {
      if (Ai[e] < 0 || Ai[e] >= m) return 2;
      len[Ai[e]]++;
    }
  for (int r = 0; r < m; r++)
    if (len[r] >= 2) pl.rows.push_back(r);
  pl.r = (int)pl.rows.size();
  if (pl.r == 0 || pl.r > rmax) return 1;
  return 0;
}

// Elements of the on-chip workspace: the factorisation's (a scatter vector of
// n; C itself is formed in global memory), or the iteration's (right-hand
// side and its second vector, x~ (n), w = rho z - y (m), then the (hi, lo)
// pairs of t and nu, r each).
GB_KKT_HD inline long long dr_ws_elems(int n, int m, int r) {
  const long long f = kkt_pad4(n);
  const long long v = kkt_pad4(2LL * n) + kkt_pad4(n) + kkt_pad4(m) + kkt_pad4(4LL * r);
  return kkt_pad4(f > v ? f : v);
}
// Bytes: the elements, then on-chip copies of the dense-row list (r ints) and
// of the row -> dense-row map (m ints).
GB_KKT_HD inline long long dr_ws_bytes(int n, int m, int r, int elem) {
  return dr_ws_elems(n, m, r) * elem + 4LL * (r + m);
}

}  // namespace gb
