// The row-major form of a sparse matrix that the dense-vector SpMV runs on
// (spmv.cu), shared with the sparse-vector multiplies that fold rows in
// column order (spmspv_sr.cu).
#pragma once
#include "gbc_internal.cuh"

namespace gbc {

struct SpmvPlan {
    Context *ctx = nullptr;
    int64_t m = 0, n = 0, nnz = 0;
    int vt = 0;
    int64_t *rowptr = nullptr;  // [m+1]
    int32_t *col = nullptr;     // [nnz]
    void *val = nullptr;        // [nnz]
    int64_t nchunks = 0, nlong = 0;
    int64_t *chunk_start = nullptr;  // [nchunks]
    int32_t *chunk_row = nullptr;    // [nchunks]
    int8_t *partial_slot = nullptr;  // [nchunks] -1: the row's only chunk, 1: part of a longer row
    int64_t *chunk_end = nullptr;    // [nchunks]
    int64_t nshort = 0;
    int32_t *short_rows = nullptr;   // [nshort] rows of 1..kShort entries
    int32_t *long_row = nullptr;     // [nlong] rows of more than one chunk
    int64_t *long_first = nullptr, *long_end = nullptr;  // their chunk ranges
    void *partial = nullptr;         // [nchunks] chunk results of long rows
};

// Build p (p->ctx and p->vt set) from A: rows ascending, each row's entries
// in ascending column order, by a stable device radix sort.
int spmv_plan_build(SpmvPlan *p, const gbc_matrix *A);
// Free p's device arrays (p itself stays).
void spmv_plan_release(SpmvPlan *p);

}  // namespace gbc
