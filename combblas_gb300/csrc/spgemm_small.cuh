// Warp-per-column SpGEMM kernels for columns with few multiplications
// (flop <= FS).  Used for sparse outputs where the block/tile kernel's
// per-tile overhead would dominate (MCL expansion, small R-MAT products,
// frontier matrices of multi-source BFS).
//
//  k_small_count    symbolic: distinct rows of the column through a warp-local
//                   open-addressing table in shared memory (order does not
//                   matter for a count).
//  k_small_numeric  gathers the column's products (row, A(row,k)*B(k,j)) in
//                   k-major order, sorts them by row with a stable LSD radix
//                   sort (ranks within a 32-item chunk from eight ballots,
//                   so equal digits keep their order), then folds each run of
//                   equal rows left to right: acc = add(mrhs, acc) over k
//                   ascending, the reference's hash-path order.  Rows come out
//                   ascending.
#pragma once

#include <type_traits>

#include "spgemm_exact.cuh"
#include "spgemm_kernels.cuh"

namespace gbc {

// Warp-cooperative walk over the products of one B column: calls
// fn(row, idx_in_A, b_entry_position) for product slots in k-major order,
// slot by slot, 32 at a time; `pos` is the product's position in that
// order.  All 32 lanes must call this together.
template <class Fn>
__device__ __forceinline__ void warp_products(const SpgemmArgs &a, int64_t bs, int64_t be, Fn fn)
{
    const int lane = threadIdx.x & 31;
    int base = 0;  // products before this chunk of B entries
    for (int64_t cb = bs; cb < be; cb += 32) {
        const int64_t b = cb + lane;
        int64_t s = 0;
        int len = 0;
        if (b < be) {
            const int k = a.brow[b];
            s = a.acp[k];
            len = (int)(a.acp[k + 1] - s);
        }
        int incl = len;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        const int excl = incl - len;
        const int tot = __shfl_sync(0xffffffffu, incl, 31);
        for (int j0 = 0; j0 < tot; j0 += 32) {
            const int j = j0 + lane;
            // owner lane: largest l with excl(l) <= j (and len(l) > 0)
            int lo = 0, hi = 32;
            while (hi - lo > 1) {
                const int mid = (lo + hi) >> 1;
                const int em = __shfl_sync(0xffffffffu, excl, mid);
                if (em <= j)
                    lo = mid;
                else
                    hi = mid;
            }
            // zero-length entries share their successor's offset; step past them
            const int el = __shfl_sync(0xffffffffu, excl, lo);
            const int64_t sl = __shfl_sync(0xffffffffu, s, lo);
            const int64_t bl = cb + lo;
            fn(j < tot, j < tot ? a.arow[sl + (j - el)] : 0, sl + (j - el), bl, base + j);
        }
        base += tot;
    }
}

// Warp hash count of distinct rows; table of TS slots per warp.
template <int TS, int WPB>
__global__ void __launch_bounds__(WPB * 32) k_small_count(const SpgemmArgs *args, const int64_t *items, int64_t ncols,
                                                          int64_t *cnt)
{
    extern __shared__ int32_t tabs[];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int32_t *t = tabs + (size_t)w * TS;
    for (int64_t ci = int64_t(blockIdx.x) * WPB + w; ci < ncols; ci += int64_t(gridDim.x) * WPB) {
        const SpgemmArgs &a = args[item_pid(items[ci])];
        const int64_t i = item_col(items[ci]);
        for (int s = lane; s < TS; s += 32) t[s] = -1;
        __syncwarp();
        int mine = 0;
        warp_products(a, a.bcp[i], a.bcp[i + 1], [&](bool act, int row, int64_t, int64_t, int) {
            if (act) {
                uint32_t h = ((uint32_t)row * 2654435761u) & (TS - 1);
                for (int probe = 0; probe < TS; ++probe) {
                    const int32_t old = atomicCAS(&t[h], -1, row);
                    if (old == -1) {
                        ++mine;
                        break;
                    }
                    if (old == row) break;
                    h = (h + 1) & (TS - 1);
                }
            }
        });
#pragma unroll
        for (int o = 16; o; o >>= 1) mine += __shfl_xor_sync(0xffffffffu, mine, o);
        if (lane == 0) cnt[a.col_base + i] = mine;
        __syncwarp();
    }
}

// Gather of one B column's products into shared memory in k-major order:
// keys[p] = row (or row << 12 | p when PACK), vals[p] = A(row,k) * B(k,j).
// Four product slots per lane are resolved before their loads are issued.
template <class SR, bool PACK>
__device__ __forceinline__ int warp_gather(const SpgemmArgs &a, const typename SR::V *aval,
                                           const typename SR::V *bval, int64_t bs, int64_t be, uint32_t *keys,
                                           typename SR::V *vals, int FS)
{
    typedef typename SR::V V;
    const int lane = threadIdx.x & 31;
    int base = 0;
    for (int64_t cb = bs; cb < be; cb += 32) {
        const int64_t b = cb + lane;
        int64_t s = 0;
        int len = 0;
        V bv = SR::one();
        if (b < be) {
            const int k = a.brow[b];
            s = a.acp[k];
            len = (int)(a.acp[k + 1] - s);
            if (bval) bv = bval[b];
        }
        int incl = len;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        const int excl = incl - len;
        const int tot = __shfl_sync(0xffffffffu, incl, 31);
        for (int j0 = 0; j0 < tot; j0 += 128) {
            int64_t idx[4];
            V bvu[4];
            bool act[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int j = j0 + u * 32 + lane;
                int lo = 0, hi = 32;
                while (hi - lo > 1) {
                    const int mid = (lo + hi) >> 1;
                    if (__shfl_sync(0xffffffffu, excl, mid) <= j)
                        lo = mid;
                    else
                        hi = mid;
                }
                const int el = __shfl_sync(0xffffffffu, excl, lo);
                const int64_t sl = __shfl_sync(0xffffffffu, s, lo);
                bvu[u] = __shfl_sync(0xffffffffu, bv, lo);
                act[u] = j < tot && base + j < FS;
                idx[u] = sl + (j - el);
            }
            int32_t row[4];
            V av[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                row[u] = act[u] ? a.arow[idx[u]] : 0;
                av[u] = (act[u] && aval) ? aval[idx[u]] : SR::one();
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                if (act[u]) {
                    const int p = base + j0 + u * 32 + lane;
                    keys[p] = PACK ? (((uint32_t)row[u] << 12) | (uint32_t)p) : (uint32_t)row[u];
                    vals[p] = SR::mul(av[u], bvu[u]);
                }
            }
        }
        base += tot;
    }
    return base;
}

// Numeric for small columns.  `cap` (optional): per-column capacity in the
// output (learned sizing); when given, the column writes at ccp[i - base]
// and a column whose distinct rows exceed cap[i] writes nothing and is
// flagged in overflow[i].  Without `cap` the exact count must equal the
// column's ccp range.  PACK (rows < 2^20): sort keys carry the product's
// position in their low 12 bits and values stay in place; otherwise values
// move with the keys.
template <class SR, int FS, int WPB, bool PACK>
__global__ void __launch_bounds__(WPB * 32) k_small_numeric(const SpgemmArgs *args, const int64_t *items,
                                                            int64_t ncols, const int64_t *ccp, int64_t ccp_base,
                                                            const int64_t *cap, int64_t *out_cnt, int32_t *overflow,
                                                            int64_t *cir, void *cval_v)
{
    typedef typename SR::V V;
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const unsigned lt = (1u << lane) - 1;
    constexpr size_t per_warp = PACK ? (size_t)FS * (8 + sizeof(V)) + 1024 : (size_t)FS * (8 + 2 * sizeof(V)) + 1024;
    unsigned char *basep = smem + (size_t)w * ((per_warp + 15) & ~size_t(15));
    V *vals0 = reinterpret_cast<V *>(basep);
    V *vals1 = PACK ? vals0 : vals0 + FS;
    uint32_t *keys0 = reinterpret_cast<uint32_t *>(vals0 + (PACK ? FS : 2 * FS));
    uint32_t *keys1 = keys0 + FS;
    int32_t *hist = reinterpret_cast<int32_t *>(keys1 + FS);
    V *cval = static_cast<V *>(cval_v);
    const int shift0 = PACK ? 12 : 0;

    for (int64_t ci = int64_t(blockIdx.x) * WPB + w; ci < ncols; ci += int64_t(gridDim.x) * WPB) {
        const SpgemmArgs &a = args[item_pid(items[ci])];
        const int64_t i = item_col(items[ci]);
        const int64_t g = a.col_base + i;
        const int key_bits = a.key_bits;
        const V *aval = static_cast<const V *>(a.aval);
        const V *bval = static_cast<const V *>(a.bval);
        // 1. gather products in k-major order
        const int n = warp_gather<SR, PACK>(a, aval, bval, a.bcp[i], a.bcp[i + 1], keys0, vals0, FS);
        if (n > FS) {  // the column was binned by its flop count, so this cannot happen
            if (lane == 0) atomicOr(a.err, 256);
            continue;
        }
        __syncwarp();
        // 2. stable LSD radix sort by row, 8 bits per pass
        uint32_t *ks = keys0, *kd = keys1;
        V *vs = vals0, *vd = vals1;
        for (int shift = shift0; shift < shift0 + key_bits; shift += 8) {
            for (int d = lane; d < 256; d += 32) hist[d] = 0;
            __syncwarp();
            for (int p = lane; p < n; p += 32) atomicAdd(&hist[(ks[p] >> shift) & 255], 1);
            __syncwarp();
            {  // exclusive scan of 256 counters: 8 per lane
                int loc[8], sum = 0;
#pragma unroll
                for (int u = 0; u < 8; ++u) {
                    loc[u] = hist[lane * 8 + u];
                    sum += loc[u];
                }
                int incl = sum;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int y = __shfl_up_sync(0xffffffffu, incl, o);
                    if (lane >= o) incl += y;
                }
                int run = incl - sum;
#pragma unroll
                for (int u = 0; u < 8; ++u) {
                    hist[lane * 8 + u] = run;
                    run += loc[u];
                }
            }
            __syncwarp();
            for (int p0 = 0; p0 < n; p0 += 32) {
                const int p = p0 + lane;
                const bool act = p < n;
                const uint32_t key = act ? ks[p] : 0u;
                const int dg = act ? (int)((key >> shift) & 255) : 0;
                // lanes holding the same digit: eight ballots (much cheaper
                // than __match_any_sync on this part)
                unsigned grp = __ballot_sync(0xffffffffu, act);
#pragma unroll
                for (int bit = 0; bit < 8; ++bit) {
                    const unsigned bb = __ballot_sync(0xffffffffu, act && ((dg >> bit) & 1));
                    grp &= ((dg >> bit) & 1) ? bb : ~bb;
                }
                if (act) {
                    const int dst = hist[dg] + __popc(grp & lt);
                    kd[dst] = key;
                    if (!PACK) vd[dst] = vs[p];
                }
                __syncwarp();
                if (act && (grp & lt) == 0) hist[dg] += __popc(grp);
                __syncwarp();
            }
            uint32_t *tk = ks;
            ks = kd;
            kd = tk;
            if (!PACK) {
                V *tv = vs;
                vs = vd;
                vd = tv;
            }
        }
        // PlusTimes fp64 with exact accumulation: the column's exponent
        // window (the same admission as the block kernel's)
        int ebase = 0;
        bool xact = false;
        if constexpr (std::is_same<SR, PlusTimes<double>>::value) {
            if (a.aexp) {
                int emin = 1 << 30, emax = -(1 << 30);
                for (int64_t b = a.bcp[i] + lane; b < a.bcp[i + 1]; b += 32)
                    x_window(a.aexp[a.brow[b]], bval ? (double)bval[b] : 1.0, bval != nullptr, emin, emax);
                ebase = __reduce_min_sync(0xffffffffu, emin);
                emax = __reduce_max_sync(0xffffffffu, emax);
                xact = x_admit(ebase, emax, a.bcp[i + 1] - a.bcp[i]);
            }
        }
        // 3. fold runs of equal rows in order and write them
        const int64_t out0 = ccp[g - ccp_base];
        const int64_t room = cap ? cap[g] : (ccp[g - ccp_base + 1] - out0);
        int64_t heads = 0;  // output entries before this chunk
        bool over = false;
        for (int p0 = 0; p0 < n; p0 += 32) {
            const int p = p0 + lane;
            const bool act = p < n;
            const uint32_t kk = act ? ks[p] : 0u;
            const int row = act ? (int)(PACK ? (kk >> 12) : kk) : -1;
            const bool head = act && (p == 0 || (int)(PACK ? (ks[p - 1] >> 12) : ks[p - 1]) != row);
            const unsigned hm = __ballot_sync(0xffffffffu, head);
            if (head) {
                V v = PACK ? vs[kk & 4095] : vs[p];
                if (xact) {
                    // exact sum of the run, rounded once (PlusTimes fp64)
                    uint64_t hi = 0, lo = 0;
                    uint32_t fl = 0;
                    bool ok = true;
                    for (int q = p; q < n; ++q) {
                        const uint32_t kq = ks[q];
                        if ((int)(PACK ? (kq >> 12) : kq) != row) break;
                        ok &= x_acc128(hi, lo, fl, (double)(PACK ? vs[kq & 4095] : vs[q]), ebase);
                    }
                    v = (V)x_round(hi, lo, fl, ebase);
                    if (!ok) atomicOr(a.err, 512);
                } else {
                    for (int q = p + 1; q < n; ++q) {
                        const uint32_t kq = ks[q];
                        if ((int)(PACK ? (kq >> 12) : kq) != row) break;
                        v = SR::add(PACK ? vs[kq & 4095] : vs[q], v);
                    }
                }
                const int64_t pos = heads + __popc(hm & lt);
                if (pos < room) {
                    cir[out0 + pos] = (int64_t)row;
                    cval[out0 + pos] = v;
                } else {
                    over = true;
                }
            }
            heads += __popc(hm);
        }
        over = __any_sync(0xffffffffu, over);
        if (lane == 0) {
            if (out_cnt) out_cnt[g] = heads;
            if (over) {
                if (overflow)
                    overflow[g] = 1;
                else
                    atomicOr(a.err, 128);
            }
        }
        __syncwarp();
    }
}

template <int FS, class V, bool PACK>
constexpr size_t small_warp_smem()
{
    return ((PACK ? (size_t)FS * (8 + sizeof(V)) + 1024 : (size_t)FS * (8 + 2 * sizeof(V)) + 1024) + 15) &
           ~size_t(15);
}

}  // namespace gbc
