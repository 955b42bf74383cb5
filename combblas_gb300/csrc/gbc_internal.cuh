// Internal declarations shared by the translation units of libgbcomb.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/gbcomb.h"

namespace gbc {

// ----------------------------------------------------------------- errors
void set_error(const std::string &msg);
int fail(int code, const std::string &msg);

#define GBC_CUDA_TRY(expr)                                                                          \
    do {                                                                                            \
        cudaError_t _e = (expr);                                                                    \
        if (_e != cudaSuccess) {                                                                    \
            return ::gbc::fail(_e == cudaErrorMemoryAllocation ? GBC_ENOMEM : GBC_ECUDA,           \
                               std::string(#expr) + ": " + cudaGetErrorString(_e));               \
        }                                                                                           \
    } while (0)

#define GBC_TRY(expr)            \
    do {                         \
        int _s = (expr);         \
        if (_s != GBC_OK) return _s; \
    } while (0)

// Count of kernel launches issued by this library (all contexts, this
// process); reported by gbc_launch_count().
void note_launch();
// Adjust the count by n (graph captures record kernels without running them;
// each replay then runs them).
void note_launches(long long n);
long long launch_count();

// ---------------------------------------------------------------- context
struct Context {
    int device = 0;
    int num_sms = 0;
    size_t smem_optin = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    cudaEvent_t ev[8] = {};
    int32_t *d_flag = nullptr;  // device error/overflow flags (8 ints)
    void *mlp = nullptr;        // sizing model used by GBC_SIZING_LEARNED (gbc_mlp*)
    void *pinned = nullptr;     // small pinned staging for scalar reads
    int fold = GBC_FOLD_EXACT;  // PlusTimes fp64 accumulation (gbc_context_set_fold)
};

// Stream-ordered device allocations; everything taken through a Workspace
// is released when the Workspace goes out of scope (on the same stream).
struct Workspace {
    Context *ctx;
    std::vector<void *> ptrs;
    explicit Workspace(Context *c) : ctx(c) {}
    ~Workspace();
    int alloc(void **p, size_t bytes);
    template <typename T>
    int alloc_n(T **p, size_t n)
    {
        return alloc(reinterpret_cast<void **>(p), n * sizeof(T) + 16);
    }
};

int device_alloc(Context *ctx, void **p, size_t bytes);
void device_free(Context *ctx, void *p);
// Synchronous scalar read of a device value (used where a size decides an
// allocation, the same place the reference allocates after its symbolic pass).
int read_i64(Context *ctx, const int64_t *dptr, int64_t *out);

// -------------------------------------------------------------- result
struct Result {
    int64_t nrow = 0, ncol = 0, nzc = 0, nnz = 0;
    int valtype = GBC_F64;
    int64_t *cp = nullptr, *jc = nullptr, *ir = nullptr;
    void *num = nullptr;
    Context *ctx = nullptr;
};

size_t value_size(int vt);

// ----------------------------------------------------------- device views
// Device-resident CSC/DCSC with int64 indices as handed over by the caller.
struct DevMatrix {
    int64_t nrow = 0, ncol = 0, nzc = 0, nnz = 0;
    const int64_t *cp = nullptr;  // [nzc+1]
    const int64_t *jc = nullptr;  // [nzc] or nullptr (CSC)
    const int64_t *ir = nullptr;  // [nnz]
    const void *num = nullptr;    // [nnz] or nullptr (all ones)
};

// Bring a gbc_matrix onto the device (copies host arrays into `ws`).
int upload(Workspace &ws, const gbc_matrix *M, int vt, DevMatrix *out);

// --------------------------------------------------------------- scans
// Exclusive scan of n int64 values (out may alias in); out[n] = total.
int exclusive_scan_i64(Workspace &ws, const int64_t *in, int64_t *out, int64_t n, cudaStream_t s);
// Allocation-free form (graph-capturable); tmp holds scan_tmp_elems(n) int64s.
int64_t scan_tmp_elems(int64_t n);
int exclusive_scan_i64_tmp(const int64_t *in, int64_t *out, int64_t n, int64_t *tmp, cudaStream_t s);

}  // namespace gbc

struct gbc_context : gbc::Context {};
struct gbc_result : gbc::Result {};
