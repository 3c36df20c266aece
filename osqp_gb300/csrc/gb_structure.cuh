// gb_structure.cuh -- deterministic sparse structure conversions on the device.
//
//   CSC(A) -> CSR(A)            (reference: cuda_csr.cu:559-628, csr_transpose /
//                                cuda_mat_init_A, which sorts COO by row with
//                                cusparseXcoosortByRow)
//   triu CSC(P) -> full CSR(P)  (reference: cuda_csr.cu:489-607, csr_triu_to_full,
//                                with an explicit diagonal and the triu->full map)
//
// Both use a stable LSD radix sort (CUB) keyed by row (CSC order is already
// column-major, so stability yields increasing column order inside each
// row): the output index arrays are a pure function of the input pattern,
// bit-identical from run to run.  The value maps (Asrc, Psrc) let later value
// updates and rescalings gather into the CSR arrays without another sort.
#pragma once

#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

namespace gb {
// Kernels have internal linkage: every translation unit gets its own copy.

// entry k of a CSC matrix -> its column
static __global__ void k_csc_entry_cols(const int* __restrict__ colptr, int ncols, int* __restrict__ entcol) {
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < ncols; j += gridDim.x * blockDim.x)
    for (int k = colptr[j]; k < colptr[j + 1]; k++) entcol[k] = j;
}

static __global__ void k_iota(int* __restrict__ v, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) v[i] = i;
}

// rowptr from sorted row keys: rowptr[r] = first k with key[k] >= r
static __global__ void k_rowptr_from_sorted(const int* __restrict__ keys, int nnz, int rows, int* __restrict__ rowptr) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k <= nnz; k += gridDim.x * blockDim.x) {
    const int prev = (k == 0) ? -1 : keys[k - 1];
    const int cur = (k == nnz) ? rows : keys[k];
    for (int r = prev + 1; r <= cur; r++) rowptr[r] = k;
  }
}

static __global__ void k_gather_int(const int* __restrict__ src, const int* __restrict__ idx, int n, int* __restrict__ dst) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) dst[i] = src[idx[i]];
}

// Symmetric expansion of an upper-triangular CSC P into COO with 64-bit keys
// row*n+col.  Slot layout: [0, nnzT) the stored entries; [nnzT, 2 nnzT) their
// mirrors (key = UINT64_MAX for diagonal entries, which have no mirror);
// [2 nnzT, 2 nnzT + n) a structural zero diagonal for columns without one.
static __global__ void k_triu_expand(const int* __restrict__ Pp, const int* __restrict__ Pi, int n, int nnzT,
                              unsigned long long* __restrict__ keys, int* __restrict__ src) {
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
    bool has_diag = false;
    for (int k = Pp[j]; k < Pp[j + 1]; k++) {
      const int i = Pi[k];
      keys[k] = (unsigned long long)i * n + j;
      src[k] = k;
      if (i == j) {
        has_diag = true;
        keys[nnzT + k] = ~0ull;
        src[nnzT + k] = -1;
      } else {
        keys[nnzT + k] = (unsigned long long)j * n + i;
        src[nnzT + k] = k;
      }
    }
    keys[2 * nnzT + j] = has_diag ? ~0ull : (unsigned long long)j * n + j;
    src[2 * nnzT + j] = -1;
  }
}

// From sorted 64-bit keys (valid prefix of length nnzF): CSR col, rowptr, diag position.
static __global__ void k_full_from_sorted(const unsigned long long* __restrict__ keys, int nnzF, int n,
                                   int* __restrict__ col, int* __restrict__ rowptr, int* __restrict__ diag) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k <= nnzF; k += gridDim.x * blockDim.x) {
    if (k < nnzF) {
      const int r = (int)(keys[k] / (unsigned long long)n);
      const int c = (int)(keys[k] % (unsigned long long)n);
      col[k] = c;
      if (r == c) diag[r] = k;
    }
    const int prev = (k == 0) ? -1 : (int)(keys[k - 1] / (unsigned long long)n);
    const int cur = (k == nnzF) ? n : (int)(keys[k] / (unsigned long long)n);
    for (int r = prev + 1; r <= cur; r++) rowptr[r] = k;
  }
}

inline int bits_for(unsigned long long v) {
  int b = 1;
  while (b < 64 && (1ull << b) <= v) b++;
  return b;
}

}  // namespace gb
