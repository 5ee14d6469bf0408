// Transpose, SpGEMM and the Galerkin product P^T A P.
//
// Reference: utopia::ptap -> PETSc MatPtAP (utopia/backend/petsc/eval/utopia_petsc_Eval_Multiply.cpp:12-61)
// and the explicit R = transpose(I) of IPRTransfer
// (utopia/solvers/multilevel/transfer/utopia_IPRTransfer.hpp:28-39).
//
// SpGEMM C = A B keeps the full symbolic structure (every structurally produced
// entry, numerical zeros included) with ascending columns.  Each output row is
// owned by one warp (or one CTA for long rows) with an open-addressing hash table
// in shared memory.  Products are enumerated j-by-j in A-row order; within one j the
// columns of B_j are distinct, so lanes never collide on a value slot and every
// output entry sums its terms in A-row order: the result is deterministic and uses
// the same summation order as the CPU oracle.
#include <algorithm>

#include "abi_util.cuh"
#include "device_util.cuh"

namespace ugpu {

namespace {

// ------------------------------------------------------------------------------------
// exclusive scan of int64 (3 phases: per-CTA scan, scan of CTA sums, add)
// ------------------------------------------------------------------------------------
constexpr int kScanBlock = 512;
constexpr int kScanItems = 8;

__device__ __forceinline__ int64_t block_exclusive_scan(int64_t v, int64_t &total) {
    __shared__ int64_t sh[32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    int64_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int64_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) sh[w] = x;
    __syncthreads();
    if (w == 0) {
        int64_t s = lane < nw ? sh[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int64_t y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        if (lane < nw) sh[lane] = s;
    }
    __syncthreads();
    int64_t before = (w > 0 ? sh[w - 1] : 0) + x - v;
    total = sh[nw - 1];
    __syncthreads();
    return before;
}

// in: n values; out: n+1 values (out[0] = 0, out[n] = total); block sums to bsum
__global__ void k_scan_local(const int64_t *in, int64_t *out, int64_t n, int64_t *bsum) {
    const int64_t base = int64_t(blockIdx.x) * kScanBlock * kScanItems;
    int64_t loc[kScanItems];
    int64_t s = 0;
#pragma unroll
    for (int q = 0; q < kScanItems; ++q) {
        int64_t i = base + int64_t(threadIdx.x) * kScanItems + q;
        loc[q] = (i < n) ? in[i] : 0;
        s += loc[q];
    }
    int64_t total;
    int64_t pre = block_exclusive_scan(s, total);
#pragma unroll
    for (int q = 0; q < kScanItems; ++q) {
        int64_t i = base + int64_t(threadIdx.x) * kScanItems + q;
        if (i < n) out[i] = pre;
        pre += loc[q];
    }
    if (threadIdx.x == 0) bsum[blockIdx.x] = total;
}

__global__ void k_scan_add(int64_t *out, int64_t n, const int64_t *boff) {
    const int64_t base = int64_t(blockIdx.x) * kScanBlock * kScanItems;
    int64_t add = boff[blockIdx.x];
    for (int q = 0; q < kScanItems; ++q) {
        int64_t i = base + int64_t(threadIdx.x) * kScanItems + q;
        if (i < n) out[i] += add;
    }
}

__global__ void k_i64_to_i32(const int64_t *in, int32_t *out, int64_t n) {
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
        out[i] = int32_t(in[i]);
}

// ------------------------------------------------------------------------------------
// transpose
// ------------------------------------------------------------------------------------
__global__ void k_col_count(const int32_t *ci, int64_t nnz, int64_t *cnt) {
    for (int64_t k = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; k < nnz; k += int64_t(gridDim.x) * blockDim.x)
        atomicAdd(reinterpret_cast<unsigned long long *>(cnt + ci[k]), 1ull);
}

template <class V>
__global__ void k_transpose_scatter(const int32_t *rp, const int32_t *ci, const V *cv, int64_t n, int64_t *fill,
                                    const int64_t *tp, int32_t *tci, V *tcv) {
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
        for (int32_t k = rp[i]; k < rp[i + 1]; ++k) {
            int32_t c = ci[k];
            int64_t pos = tp[c] + int64_t(atomicAdd(reinterpret_cast<unsigned long long *>(fill + c), 1ull));
            tci[pos] = int32_t(i);
            tcv[pos] = cv[k];
        }
    }
}

// sort every row by column (insertion sort; rows of transposed transfer operators are short)
template <class V>
__global__ void k_sort_rows(const int64_t *tp, int64_t n, int32_t *tci, V *tcv) {
    // a warp per row: rows of at most 32 entries are placed by rank (the keys of a row are
    // distinct: they are the source rows of one column), longer rows by one lane's insertion sort
    const int lane = threadIdx.x & 31;
    const int64_t nw = (int64_t(gridDim.x) * blockDim.x) >> 5;
    for (int64_t r = (blockIdx.x * int64_t(blockDim.x) + threadIdx.x) >> 5; r < n; r += nw) {
        const int64_t a = tp[r], b = tp[r + 1];
        const int64_t len = b - a;
        if (len <= 1) continue;
        if (len <= 32) {
            const int32_t key = lane < len ? tci[a + lane] : INT32_MAX;
            const V val = lane < len ? tcv[a + lane] : V{};
            int rank = 0;
            for (int t = 0; t < int(len); ++t) rank += __shfl_sync(0xffffffffu, key, t) < key ? 1 : 0;
            if (lane < len) {
                tci[a + rank] = key;
                tcv[a + rank] = val;
            }
        } else if (lane == 0) {
            for (int64_t i = a + 1; i < b; ++i) {
                const int32_t key = tci[i];
                const V val = tcv[i];
                int64_t j = i - 1;
                while (j >= a && tci[j] > key) {
                    tci[j + 1] = tci[j];
                    tcv[j + 1] = tcv[j];
                    --j;
                }
                tci[j + 1] = key;
                tcv[j + 1] = val;
            }
        }
        __syncwarp();
    }
}

// ------------------------------------------------------------------------------------
// SpGEMM
// ------------------------------------------------------------------------------------
// per-row upper bound of the product's row length, and their maximum (one atomic per warp)
__global__ void k_row_upper_bound(const int32_t *arp, const int32_t *aci, const int32_t *brp, int64_t m,
                                  int64_t *ub, unsigned long long *max_ub) {
    unsigned long long mx = 0;
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < m; i += int64_t(gridDim.x) * blockDim.x) {
        int64_t s = 0;
        for (int32_t k = arp[i]; k < arp[i + 1]; ++k) {
            int32_t j = aci[k];
            s += brp[j + 1] - brp[j];
        }
        ub[i] = s;
        mx = s > int64_t(mx) ? (unsigned long long)s : mx;
    }
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long v = __shfl_xor_sync(0xffffffffu, mx, o);
        mx = v > mx ? v : mx;
    }
    if ((threadIdx.x & 31) == 0 && mx) atomicMax(max_ub, mx);
}

constexpr int kWarpTable = 2048;      // max slots per warp (rows with upper bound <= 1024)
constexpr int kWarpRowsUb = 1024;
constexpr int kWarpsPerCta = 4;
constexpr int kCtaTable = 8192;       // slots per CTA (rows with upper bound <= 4096)
constexpr int kCtaRowsUb = 4096;
constexpr int kCtaThreads = 256;

__device__ __forceinline__ uint32_t hash_col(int32_t c, int mask) { return (uint32_t(c) * 2654435761u) & mask; }

// insert column c; concurrent inserters hold distinct columns.  Returns the slot.
__device__ __forceinline__ int hash_insert(int32_t *keys, int mask, int32_t c, int *n_unique) {
    volatile int32_t *vk = keys;
    uint32_t h = hash_col(c, mask);
    while (true) {
        int32_t k = vk[h];
        if (k == c) return int(h);
        if (k == -1) {
            int32_t old = atomicCAS(&keys[h], -1, c);
            if (old == -1) {
                if (n_unique) atomicAdd(n_unique, 1);
                return int(h);
            }
            if (old == c) return int(h);
        }
        h = (h + 1) & mask;
    }
}

// the group's barrier: the CTA, or the lanes of gmask within a warp (a whole warp or a sub-warp group)
template <bool CTA>
__device__ __forceinline__ void group_sync(unsigned gmask) {
    if constexpr (CTA) __syncthreads();
    else __syncwarp(gmask);
}

// table size for a row: power of two >= 2 * upper bound (load factor <= 1/2)
__device__ __forceinline__ int table_size(int64_t ub, int cap) {
    int t = 64;
    while (t < 2 * ub && t < cap) t <<= 1;
    return t;
}

// One output row with G cooperating threads.  NUMERIC = false: count unique columns;
// true: accumulate values and write the row sorted by column.
template <class V, bool NUMERIC, bool CTA>
__device__ void row_product(int64_t i, int tid, int G, int TS, int32_t *keys, double *vals, int32_t *lkeys,
                            double *lvals, int *s_count, const int32_t *arp, const int32_t *aci, const V *acv,
                            const int32_t *brp, const int32_t *bci, const V *bcv, int64_t *cnt_out,
                            const int32_t *crp, int32_t *cci, V *ccv, unsigned gmask = 0xffffffffu) {
    const int mask = TS - 1;
    for (int s = tid; s < TS; s += G) {
        keys[s] = -1;
        if (NUMERIC) vals[s] = 0.0;
    }
    if (tid == 0) *s_count = 0;
    group_sync<CTA>(gmask);
    for (int32_t ka = arp[i]; ka < arp[i + 1]; ++ka) {
        const int32_t j = aci[ka];
        const double a = NUMERIC ? cvt<double>(acv[ka]) : 0.0;
        const int32_t b1 = brp[j + 1];
        for (int32_t kb = brp[j] + tid; kb < b1; kb += G) {
            const int slot = hash_insert(keys, mask, bci[kb], NUMERIC ? nullptr : s_count);
            if (NUMERIC) vals[slot] = fma(a, cvt<double>(bcv[kb]), vals[slot]);
        }
        group_sync<CTA>(gmask);  // every product of this j lands before the next j
    }
    if (!NUMERIC) {
        if (tid == 0) cnt_out[i] = *s_count;
        group_sync<CTA>(gmask);
        return;
    }
    // compact the occupied slots, then place each entry at its rank (sorted by column)
    for (int s = tid; s < TS; s += G) {
        const int32_t k = keys[s];
        if (k >= 0) {
            const int p = atomicAdd(s_count, 1);
            lkeys[p] = k;
            lvals[p] = vals[s];
        }
    }
    group_sync<CTA>(gmask);
    const int u = *s_count;
    const int32_t base = crp[i];
    for (int e = tid; e < u; e += G) {
        const int32_t k = lkeys[e];
        int rank = 0;
        for (int t = 0; t < u; ++t) rank += (lkeys[t] < k);
        cci[base + rank] = k;
        ccv[base + rank] = cvt<V>(lvals[e]);
    }
    group_sync<CTA>(gmask);
}

constexpr size_t kWarpSmem = (sizeof(int32_t) + sizeof(double)) * (kWarpTable + kWarpRowsUb) * kWarpsPerCta;
constexpr size_t kCtaSmem = (sizeof(int32_t) + sizeof(double)) * (kCtaTable + kCtaRowsUb);

// Warp tiers: each warp takes whole rows whose upper bound u lies in (LO, ROWS_UB], with a
// hash table of TABLE slots; the small tiers keep the shared memory per warp small so that
// many warps share an SM (the typical Galerkin row has a few tens of products).  The last
// warp tier lists the rows beyond it for the CTA kernels (symbolic phase).
constexpr int kTier0Table = 64, kTier0Ub = 32, kTier0Warps = 8;
constexpr int kTier1Table = 256, kTier1Ub = 128, kTier1Warps = 8;
template <int TABLE, int ROWS_UB, int WARPS>
constexpr size_t tier_smem() {
    return (sizeof(int32_t) + sizeof(double)) * size_t(TABLE + ROWS_UB) * WARPS;
}

template <class V, bool NUMERIC, int TABLE, int ROWS_UB, int WARPS, bool APPEND>
__global__ void __launch_bounds__(WARPS * 32) k_spgemm_warp(int64_t m, int64_t lo, const int64_t *ub,
                                                            const int32_t *arp, const int32_t *aci, const V *acv,
                                                            const int32_t *brp, const int32_t *bci, const V *bcv,
                                                            int64_t *cnt, const int32_t *crp, int32_t *cci, V *ccv,
                                                            int *big_rows, int *n_big) {
    extern __shared__ unsigned char smem[];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    double *vals = reinterpret_cast<double *>(smem) + size_t(w) * TABLE;
    double *lvals = reinterpret_cast<double *>(smem) + size_t(WARPS) * TABLE + size_t(w) * ROWS_UB;
    int32_t *ibase = reinterpret_cast<int32_t *>(smem + sizeof(double) * (TABLE + ROWS_UB) * WARPS);
    int32_t *keys = ibase + size_t(w) * TABLE;
    int32_t *lkeys = ibase + size_t(WARPS) * TABLE + size_t(w) * ROWS_UB;
    __shared__ int s_count[WARPS];
    const int64_t gw = int64_t(blockIdx.x) * WARPS + w;
    const int64_t nw = int64_t(gridDim.x) * WARPS;
    for (int64_t i = gw; i < m; i += nw) {
        const int64_t u = ub[i];
        if (u <= lo) continue;
        if (u > ROWS_UB) {
            if (APPEND && !NUMERIC && lane == 0) big_rows[atomicAdd(n_big, 1)] = int(i);
            continue;
        }
        row_product<V, NUMERIC, false>(i, lane, 32, table_size(u, TABLE), keys, vals, lkeys, lvals, &s_count[w],
                                       arp, aci, acv, brp, bci, bcv, cnt, crp, cci, ccv);
    }
}

// Tier 0 with sub-warp groups: rows of at most kTier0Ub products (the A P rows of a Galerkin product
// have a few to a few dozen) take a group of kSubLanes lanes each, kSubGroups groups per warp, each
// with its own table; a whole warp per such row left most of its lanes idle.  The same per-column
// accumulation order as the warp form (products land in A-row order), so the same bits.
constexpr int kSubLanes = 8, kSubGroups = 32 / kSubLanes, kSubWarps = 8;
constexpr size_t kSubSmem = (sizeof(int32_t) + sizeof(double)) * size_t(kTier0Table + kTier0Ub) * kSubWarps * kSubGroups;

template <class V, bool NUMERIC>
__global__ void __launch_bounds__(kSubWarps * 32) k_spgemm_sub(int64_t m, const int64_t *ub, const int32_t *arp,
                                                             const int32_t *aci, const V *acv, const int32_t *brp,
                                                             const int32_t *bci, const V *bcv, int64_t *cnt,
                                                             const int32_t *crp, int32_t *cci, V *ccv) {
    extern __shared__ unsigned char smem[];
    constexpr int NG = kSubWarps * kSubGroups;  // groups per CTA
    const int lane = threadIdx.x & 31;
    const int g = threadIdx.x / kSubLanes;  // group within the CTA
    const int tid = lane % kSubLanes;
    const unsigned gmask = ((1u << kSubLanes) - 1u) << (lane & ~(kSubLanes - 1));
    double *vals = reinterpret_cast<double *>(smem) + size_t(g) * kTier0Table;
    double *lvals = reinterpret_cast<double *>(smem) + size_t(NG) * kTier0Table + size_t(g) * kTier0Ub;
    int32_t *ibase = reinterpret_cast<int32_t *>(smem + sizeof(double) * (kTier0Table + kTier0Ub) * NG);
    int32_t *keys = ibase + size_t(g) * kTier0Table;
    int32_t *lkeys = ibase + size_t(NG) * kTier0Table + size_t(g) * kTier0Ub;
    __shared__ int s_count[NG];
    const int64_t ng = int64_t(gridDim.x) * NG;
    for (int64_t i = int64_t(blockIdx.x) * NG + g; i < m; i += ng) {
        const int64_t u = ub[i];
        if (u > kTier0Ub) continue;  // the group's lanes agree: one row per group
        row_product<V, NUMERIC, false>(i, tid, kSubLanes, table_size(u, kTier0Table), keys, vals, lkeys, lvals,
                                       &s_count[g], arp, aci, acv, brp, bci, bcv, cnt, crp, cci, ccv, gmask);
    }
}

// The mid tier: rows of 129..1024 products whose distinct columns number at most 128 (a
// Galerkin row has a few hundred products landing on a few dozen columns).  Sized by the
// distinct count, a warp's table is 256 slots and its compaction buffer 128 entries (4.5 KB, 48
// warps per SM) where sizing by the product count took 36 KB per warp (4 warps per SM).  The
// symbolic pass tries every such row at that size and sends the rows that exceed 128 distinct
// columns to a list for the full-size tier; the numeric pass picks the tier by the row's length.
constexpr int kMidTable = 256, kMidCap = 128, kMidWarps = 8;
constexpr size_t kMidSmem = (sizeof(int32_t) + sizeof(double)) * size_t(kMidTable + kMidCap) * kMidWarps;

// hash_insert with a bounded probe sequence: -1 when the table is full
__device__ __forceinline__ int hash_insert_bounded(int32_t *keys, int mask, int32_t c, int *n_unique) {
    volatile int32_t *vk = keys;
    uint32_t h = hash_col(c, mask);
    for (int p = 0; p <= mask; ++p) {
        const int32_t k = vk[h];
        if (k == c) return int(h);
        if (k == -1) {
            const int32_t old = atomicCAS(&keys[h], -1, c);
            if (old == -1) {
                atomicAdd(n_unique, 1);
                return int(h);
            }
            if (old == c) return int(h);
        }
        h = (h + 1) & mask;
    }
    return -1;
}

// distinct columns of row i of A B with one warp and a table of TS slots, or -1 past cap
__device__ int row_count_capped(int64_t i, int lane, int TS, int cap, int32_t *keys, int *s_count, int *s_over,
                                const int32_t *arp, const int32_t *aci, const int32_t *brp, const int32_t *bci) {
    const int mask = TS - 1;
    for (int t = lane; t < TS; t += 32) keys[t] = -1;
    if (lane == 0) {
        *s_count = 0;
        *s_over = 0;
    }
    __syncwarp();
    bool over = false;
    for (int32_t ka = arp[i]; ka < arp[i + 1] && !over; ++ka) {
        const int32_t j = aci[ka];
        const int32_t b1 = brp[j + 1];
        for (int32_t kb = brp[j] + lane; kb < b1; kb += 32) {
            if (*reinterpret_cast<volatile int *>(s_count) > cap) break;
            if (hash_insert_bounded(keys, mask, bci[kb], s_count) < 0) {
                *s_over = 1;
                break;
            }
        }
        __syncwarp();
        over = *reinterpret_cast<volatile int *>(s_count) > cap || *reinterpret_cast<volatile int *>(s_over) != 0;
        __syncwarp();  // every lane reads before any lane inserts again: `over` is warp-uniform
    }
    const int c = *reinterpret_cast<volatile int *>(s_count);
    __syncwarp();
    return over ? -1 : c;
}

// symbolic mid tier: rows with kTier1Ub < ub <= kWarpRowsUb counted at the small size; those past
// kMidCap distinct columns go to over[], rows beyond kWarpRowsUb products to big[] (for the CTA kernels)
__global__ void __launch_bounds__(kMidWarps * 32) k_spgemm_mid_sym(int64_t m, const int64_t *ub, const int32_t *arp,
                                                                 const int32_t *aci, const int32_t *brp,
                                                                 const int32_t *bci, int64_t *cnt, int *over,
                                                                 int *n_over, int *big, int *n_big) {
    __shared__ int32_t s_keys[kMidWarps][kMidTable];
    __shared__ int s_count[kMidWarps], s_over[kMidWarps];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t nw = int64_t(gridDim.x) * kMidWarps;
    for (int64_t i = int64_t(blockIdx.x) * kMidWarps + w; i < m; i += nw) {
        const int64_t u = ub[i];
        if (u <= kTier1Ub) continue;
        if (u > kWarpRowsUb) {
            if (lane == 0) big[atomicAdd(n_big, 1)] = int(i);
            continue;
        }
        const int c = row_count_capped(i, lane, kMidTable, kMidCap, s_keys[w], &s_count[w], &s_over[w], arp, aci,
                                       brp, bci);
        if (lane == 0) {
            if (c >= 0) cnt[i] = c;
            else over[atomicAdd(n_over, 1)] = int(i);
        }
    }
}

// numeric mid tier: rows with kTier1Ub < ub <= kWarpRowsUb and at most kMidCap entries
template <class V>
__global__ void __launch_bounds__(kMidWarps * 32) k_spgemm_mid_num(int64_t m, const int64_t *ub, const int32_t *arp,
                                                                 const int32_t *aci, const V *acv,
                                                                 const int32_t *brp, const int32_t *bci,
                                                                 const V *bcv, const int32_t *crp, int32_t *cci,
                                                                 V *ccv) {
    extern __shared__ unsigned char smem[];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    double *vals = reinterpret_cast<double *>(smem) + size_t(w) * kMidTable;
    double *lvals = reinterpret_cast<double *>(smem) + size_t(kMidWarps) * kMidTable + size_t(w) * kMidCap;
    int32_t *ibase = reinterpret_cast<int32_t *>(smem + sizeof(double) * (kMidTable + kMidCap) * kMidWarps);
    int32_t *keys = ibase + size_t(w) * kMidTable;
    int32_t *lkeys = ibase + size_t(kMidWarps) * kMidTable + size_t(w) * kMidCap;
    __shared__ int s_count[kMidWarps];
    const int64_t nw = int64_t(gridDim.x) * kMidWarps;
    for (int64_t i = int64_t(blockIdx.x) * kMidWarps + w; i < m; i += nw) {
        const int64_t u = ub[i];
        const int nz = crp[i + 1] - crp[i];
        if (u <= kTier1Ub || u > kWarpRowsUb || nz > kMidCap) continue;
        row_product<V, true, false>(i, lane, 32, table_size(nz, kMidTable), keys, vals, lkeys, lvals, &s_count[w],
                                    arp, aci, acv, brp, bci, bcv, nullptr, crp, cci, ccv);
    }
}

// the full-size warp tier over a list of rows (the mid tier's overflow)
template <class V, bool NUMERIC>
__global__ void __launch_bounds__(kWarpsPerCta * 32) k_spgemm_warp_list(const int *rows, int nrows, const int64_t *ub,
                                                                       const int32_t *arp, const int32_t *aci,
                                                                       const V *acv, const int32_t *brp,
                                                                       const int32_t *bci, const V *bcv,
                                                                       int64_t *cnt, const int32_t *crp,
                                                                       int32_t *cci, V *ccv) {
    extern __shared__ unsigned char smem[];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    double *vals = reinterpret_cast<double *>(smem) + size_t(w) * kWarpTable;
    double *lvals = reinterpret_cast<double *>(smem) + size_t(kWarpsPerCta) * kWarpTable + size_t(w) * kWarpRowsUb;
    int32_t *ibase = reinterpret_cast<int32_t *>(smem + sizeof(double) * (kWarpTable + kWarpRowsUb) * kWarpsPerCta);
    int32_t *keys = ibase + size_t(w) * kWarpTable;
    int32_t *lkeys = ibase + size_t(kWarpsPerCta) * kWarpTable + size_t(w) * kWarpRowsUb;
    __shared__ int s_count[kWarpsPerCta];
    const int nw = gridDim.x * kWarpsPerCta;
    for (int b = blockIdx.x * kWarpsPerCta + w; b < nrows; b += nw) {
        const int64_t i = rows[b];
        row_product<V, NUMERIC, false>(i, lane, 32, table_size(ub[i], kWarpTable), keys, vals, lkeys, lvals,
                                       &s_count[w], arp, aci, acv, brp, bci, bcv, cnt, crp, cci, ccv);
    }
}

template <class V, bool NUMERIC>
__global__ void __launch_bounds__(kCtaThreads) k_spgemm_cta(const int *big_rows, int n_big, const int64_t *ub,
                                                            const int32_t *arp, const int32_t *aci, const V *acv,
                                                            const int32_t *brp, const int32_t *bci, const V *bcv,
                                                            int64_t *cnt, const int32_t *crp, int32_t *cci, V *ccv) {
    extern __shared__ unsigned char smem[];
    double *vals = reinterpret_cast<double *>(smem);
    double *lvals = vals + kCtaTable;
    int32_t *keys = reinterpret_cast<int32_t *>(lvals + kCtaRowsUb);
    int32_t *lkeys = keys + kCtaTable;
    __shared__ int s_count;
    for (int b = blockIdx.x; b < n_big; b += gridDim.x) {
        const int64_t i = big_rows[b];
        if (ub[i] > kCtaRowsUb) continue;  // wide row: k_spgemm_wide
        row_product<V, NUMERIC, true>(i, threadIdx.x, blockDim.x, table_size(ub[i], kCtaTable), keys, vals, lkeys,
                                      lvals, &s_count, arp, aci, acv, brp, bci, bcv, cnt, crp, cci, ccv);
    }
}

// Rows with more than kCtaRowsUb intermediate products (wide Galerkin rows of deep algebraic-
// multigrid levels): one CTA per row walks the row's column range in windows of kWideWindow
// columns, with a dense shared-memory accumulator per window.  Products are added in A-row order
// (one B row at a time, each column owned by one thread, a barrier between B rows), so the sums
// are deterministic; a block-wide scan of the window's occupancy flags writes the entries in
// column order.  NUMERIC = false counts the row's distinct columns.
constexpr int kWideWindow = 8192;
constexpr int kWideThreads = 256;
constexpr size_t kWideSmem = (sizeof(double) + sizeof(int)) * kWideWindow;

template <bool NUMERIC>
__global__ void __launch_bounds__(kWideThreads) k_spgemm_wide(const int *big_rows, int n_big, const int64_t *ub,
                                                              const int32_t *arp, const int32_t *aci,
                                                              const double *acv, const int32_t *brp,
                                                              const int32_t *bci, const double *bcv, int64_t *cnt,
                                                              const int32_t *crp, int32_t *cci, double *ccv) {
    extern __shared__ unsigned char smem[];
    double *acc = reinterpret_cast<double *>(smem);
    int *flag = reinterpret_cast<int *>(acc + kWideWindow);
    __shared__ int s_min, s_max, s_base, s_warp[kWideThreads / 32];
    const int tid = threadIdx.x;
    for (int b = blockIdx.x; b < n_big; b += gridDim.x) {
        const int64_t i = big_rows[b];
        if (ub[i] <= kCtaRowsUb) continue;  // a shared-memory hash row
        // column range of the row's products
        int lo = INT_MAX, hi = -1;
        for (int32_t ka = arp[i]; ka < arp[i + 1]; ++ka) {
            const int32_t j = aci[ka];
            for (int32_t kb = brp[j] + tid; kb < brp[j + 1]; kb += kWideThreads) {
                lo = min(lo, bci[kb]);
                hi = max(hi, bci[kb]);
            }
        }
        if (tid == 0) {
            s_min = INT_MAX;
            s_max = -1;
            s_base = 0;
        }
        __syncthreads();
        atomicMin(&s_min, lo);
        atomicMax(&s_max, hi);
        __syncthreads();
        const int cmin = s_min, cmax = s_max;
        int64_t written = 0;
        for (int64_t c0 = cmin; c0 <= cmax; c0 += kWideWindow) {
            for (int s = tid; s < kWideWindow; s += kWideThreads) {
                acc[s] = 0.0;
                flag[s] = 0;
            }
            __syncthreads();
            for (int32_t ka = arp[i]; ka < arp[i + 1]; ++ka) {
                const int32_t j = aci[ka];
                const double a = NUMERIC ? acv[ka] : 0.0;
                for (int32_t kb = brp[j] + tid; kb < brp[j + 1]; kb += kWideThreads) {
                    const int64_t c = bci[kb] - c0;
                    if (c >= 0 && c < kWideWindow) {
                        flag[c] = 1;
                        if (NUMERIC) acc[c] = fma(a, bcv[kb], acc[c]);
                    }
                }
                __syncthreads();  // every product of this B row lands before the next row's
            }
            // block-wide exclusive scan of the flags: thread t owns kWideWindow / kWideThreads
            // consecutive columns
            constexpr int per = kWideWindow / kWideThreads;
            int mine = 0;
            for (int q = 0; q < per; ++q) mine += flag[tid * per + q];
            int incl = mine;
            const int lane = tid & 31, warp = tid >> 5;
            for (int o = 1; o < 32; o <<= 1) {
                const int t = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += t;
            }
            if (lane == 31) s_warp[warp] = incl;
            __syncthreads();
            int wofs = 0;
            for (int w = 0; w < warp; ++w) wofs += s_warp[w];
            int pos = wofs + incl - mine;
            if (NUMERIC) {
                const int64_t base = int64_t(crp[i]) + written;
                for (int q = 0; q < per; ++q) {
                    const int s = tid * per + q;
                    if (flag[s]) {
                        cci[base + pos] = int32_t(c0 + s);
                        ccv[base + pos] = acc[s];
                        ++pos;
                    }
                }
            }
            int total = 0;
            for (int w = 0; w < kWideThreads / 32; ++w) total += s_warp[w];
            written += total;
            __syncthreads();  // the window's arrays are reused
        }
        if (!NUMERIC && tid == 0) cnt[i] = written;
        __syncthreads();
    }
}

}  // namespace

// host: exclusive scan of n int64 -> out[0..n] (out[n] = total: `out` holds n + 1 entries); returns total
int64_t device_exclusive_scan(Context &ctx, const int64_t *in, int64_t *out, int64_t n) {
    const int64_t per = int64_t(kScanBlock) * kScanItems;
    const int64_t nb = (n + per - 1) / per;
    if (n == 0) {
        UGPU_CUDA(cudaMemsetAsync(out, 0, sizeof(int64_t), ctx.stream));
        return 0;
    }
    Buffer bsum, boff;
    bsum.alloc(sizeof(int64_t) * nb);
    boff.alloc(sizeof(int64_t) * (nb + 1));
    k_scan_local<<<int(nb), kScanBlock, 0, ctx.stream>>>(in, out, n, bsum.as<int64_t>());
    ctx.launches++;
    UGPU_LAUNCH_CHECK();
    if (nb > 1) {
        device_exclusive_scan(ctx, bsum.as<int64_t>(), boff.as<int64_t>(), nb);
        k_scan_add<<<int(nb), kScanBlock, 0, ctx.stream>>>(out, n, boff.as<int64_t>());
        ctx.launches++;
        UGPU_LAUNCH_CHECK();
    } else {
        UGPU_CUDA(cudaMemsetAsync(boff.ptr, 0, sizeof(int64_t), ctx.stream));
    }
    // total = last exclusive value + last input
    int64_t last_ex = 0, last_in = 0;
    UGPU_CUDA(cudaMemcpyAsync(&last_ex, out + n - 1, sizeof(int64_t), cudaMemcpyDeviceToHost, ctx.stream));
    UGPU_CUDA(cudaMemcpyAsync(&last_in, in + n - 1, sizeof(int64_t), cudaMemcpyDeviceToHost, ctx.stream));
    UGPU_CUDA(cudaStreamSynchronize(ctx.stream));
    int64_t total = last_ex + last_in;
    UGPU_CUDA(cudaMemcpyAsync(out + n, &total, sizeof(int64_t), cudaMemcpyHostToDevice, ctx.stream));
    UGPU_CUDA(cudaStreamSynchronize(ctx.stream));
    return total;
}

std::unique_ptr<Mat> transpose(const Mat &A, bool finalize) {
    Context &ctx = *A.ctx;
    Buffer cnt, tp64, fill;
    cnt.alloc(sizeof(int64_t) * std::max<int64_t>(A.ncols, 1));
    tp64.alloc(sizeof(int64_t) * (A.ncols + 1));
    fill.alloc(sizeof(int64_t) * std::max<int64_t>(A.ncols, 1));
    UGPU_CUDA(cudaMemsetAsync(cnt.ptr, 0, cnt.bytes, ctx.stream));
    UGPU_CUDA(cudaMemsetAsync(fill.ptr, 0, fill.bytes, ctx.stream));
    if (A.nnz) {
        k_col_count<<<stream_grid(ctx, A.nnz), kBlock, 0, ctx.stream>>>(A.colidx.as<int32_t>(), A.nnz,
                                                                        cnt.as<int64_t>());
        ctx.launches++;
        UGPU_LAUNCH_CHECK();
    }
    device_exclusive_scan(ctx, cnt.as<int64_t>(), tp64.as<int64_t>(), A.ncols);
    auto T = make_csr_device(ctx, A.ncols, A.nrows, A.nnz, A.vdtype);
    auto go = [&](auto tag) {
        using V = decltype(tag);
        if (A.nrows)
            k_transpose_scatter<V><<<stream_grid(ctx, A.nrows), kBlock, 0, ctx.stream>>>(
                A.rowptr.as<int32_t>(), A.colidx.as<int32_t>(), A.vals.as<V>(), A.nrows, fill.as<int64_t>(),
                tp64.as<int64_t>(), T->colidx.as<int32_t>(), T->vals.as<V>());
        if (A.ncols)
            k_sort_rows<V><<<stream_grid(ctx, A.ncols * 32), kBlock, 0, ctx.stream>>>(tp64.as<int64_t>(), A.ncols,
                                                                                T->colidx.as<int32_t>(),
                                                                                T->vals.as<V>());
        ctx.launches += 2;
    };
    if (A.vdtype == UGPU_F64) go(double{});
    else if (A.vdtype == UGPU_F32) go(float{});
    else go(__nv_bfloat16{});
    UGPU_LAUNCH_CHECK();
    k_i64_to_i32<<<stream_grid(ctx, A.ncols + 1), kBlock, 0, ctx.stream>>>(tp64.as<int64_t>(),
                                                                           T->rowptr.as<int32_t>(), A.ncols + 1);
    ctx.launches++;
    UGPU_LAUNCH_CHECK();
    UGPU_CUDA(cudaStreamSynchronize(ctx.stream));
    if (finalize) finalize_matrix(*T);
    return T;
}

namespace {

void spgemm_set_attributes() {
    const size_t warp_smem = kWarpSmem;
    const size_t cta_smem = kCtaSmem;
    static bool attr_done = false;
    if (!attr_done) {
        UGPU_CUDA(cudaFuncSetAttribute(
            k_spgemm_warp<double, false, kWarpTable, kWarpRowsUb, kWarpsPerCta, true>,
            cudaFuncAttributeMaxDynamicSharedMemorySize, int(warp_smem)));
        UGPU_CUDA(cudaFuncSetAttribute(
            k_spgemm_warp<double, true, kWarpTable, kWarpRowsUb, kWarpsPerCta, true>,
            cudaFuncAttributeMaxDynamicSharedMemorySize, int(warp_smem)));
        UGPU_CUDA(cudaFuncSetAttribute(k_spgemm_warp_list<double, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       int(warp_smem)));
        UGPU_CUDA(cudaFuncSetAttribute(k_spgemm_warp_list<double, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       int(warp_smem)));
        UGPU_CUDA(cudaFuncSetAttribute(k_spgemm_cta<double, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       int(cta_smem)));
        UGPU_CUDA(cudaFuncSetAttribute(k_spgemm_cta<double, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       int(cta_smem)));
        UGPU_CUDA(cudaFuncSetAttribute(k_spgemm_wide<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       int(kWideSmem)));
        UGPU_CUDA(cudaFuncSetAttribute(k_spgemm_wide<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       int(kWideSmem)));
        attr_done = true;
    }
}

// the warp tiers (rows up to kWarpRowsUb products); tiers above the largest row are skipped.
// Symbolic (N = false): row counts into cnt, rows beyond the warp tiers listed in big/nbig.
// Symbolic: the mid tier's overflow rows go to over[] (count in *nover on the device, returned in
// *h_nover_out); numeric: the list from the symbolic pass (h_nover_in rows).
template <bool N>
void launch_warp_tiers(Context &ctx, const Mat &A, const Mat &B, unsigned long long max_ub, const int64_t *ub,
                       int64_t *cnt, const int32_t *crp, int32_t *cci, double *ccv, int *big, int *nbig, int *over,
                       int *nover, int h_nover_in, int *h_nover_out) {
    const int64_t m = A.nrows;
    if (!m) return;
    const int32_t *arp = A.rowptr.as<int32_t>(), *aci = A.colidx.as<int32_t>();
    const int32_t *brp = B.rowptr.as<int32_t>(), *bci = B.colidx.as<int32_t>();
    const double *acv = A.vals.as<double>(), *bcv = B.vals.as<double>();
    auto grid = [&](int warps, int per_sm) {
        return int(std::max<int64_t>(1, std::min<int64_t>((m + warps - 1) / warps, int64_t(ctx.sms) * per_sm)));
    };
    k_spgemm_sub<double, N><<<grid(kSubWarps * kSubGroups, 8), kSubWarps * 32, kSubSmem, ctx.stream>>>(
        m, ub, arp, aci, acv, brp, bci, bcv, cnt, crp, cci, ccv);
    ctx.launches++;
    if (max_ub > (unsigned long long)kTier0Ub) {
        k_spgemm_warp<double, N, kTier1Table, kTier1Ub, kTier1Warps, false>
            <<<grid(kTier1Warps, 6), kTier1Warps * 32, tier_smem<kTier1Table, kTier1Ub, kTier1Warps>(),
               ctx.stream>>>(m, kTier0Ub, ub, arp, aci, acv, brp, bci, bcv, cnt, crp, cci, ccv, nullptr, nullptr);
        ctx.launches++;
    }
    if (max_ub > (unsigned long long)kTier1Ub) {
        if constexpr (!N) {
            k_spgemm_mid_sym<<<grid(kMidWarps, 6), kMidWarps * 32, 0, ctx.stream>>>(m, ub, arp, aci, brp, bci, cnt,
                                                                                   over, nover, big, nbig);
        } else {
            k_spgemm_mid_num<double><<<grid(kMidWarps, 6), kMidWarps * 32, kMidSmem, ctx.stream>>>(
                m, ub, arp, aci, acv, brp, bci, bcv, crp, cci, ccv);
        }
        ctx.launches++;
        UGPU_LAUNCH_CHECK();
        // the mid tier's overflow rows at the full warp-table size
        int h_nover = h_nover_in;
        if constexpr (!N) {
            UGPU_CUDA(cudaMemcpyAsync(&h_nover, nover, sizeof(int), cudaMemcpyDeviceToHost, ctx.stream));
            UGPU_CUDA(cudaStreamSynchronize(ctx.stream));
            *h_nover_out = h_nover;
        }
        if (h_nover > 0) {
            k_spgemm_warp_list<double, N><<<std::max(1, std::min((h_nover + kWarpsPerCta - 1) / kWarpsPerCta,
                                                                 ctx.sms * 16)),
                                            kWarpsPerCta * 32, kWarpSmem, ctx.stream>>>(
                over, h_nover, ub, arp, aci, acv, brp, bci, bcv, cnt, crp, cci, ccv);
            ctx.launches++;
        }
    }
    UGPU_LAUNCH_CHECK();
}

// rows beyond the warp tiers: one CTA per row (hash table), then the windowed wide rows
template <bool N>
void launch_big_rows(Context &ctx, const Mat &A, const Mat &B, unsigned long long max_ub, const int64_t *ub,
                     const int *big, int h_nbig, int64_t *cnt, const int32_t *crp, int32_t *cci, double *ccv) {
    if (!h_nbig) return;
    const int32_t *arp = A.rowptr.as<int32_t>(), *aci = A.colidx.as<int32_t>();
    const int32_t *brp = B.rowptr.as<int32_t>(), *bci = B.colidx.as<int32_t>();
    const double *acv = A.vals.as<double>(), *bcv = B.vals.as<double>();
    k_spgemm_cta<double, N><<<std::min(h_nbig, ctx.sms * 2), kCtaThreads, kCtaSmem, ctx.stream>>>(
        big, h_nbig, ub, arp, aci, acv, brp, bci, bcv, cnt, crp, cci, ccv);
    ctx.launches++;
    UGPU_LAUNCH_CHECK();
    if (max_ub > (unsigned long long)kCtaRowsUb) {
        k_spgemm_wide<N><<<std::min(h_nbig, ctx.sms * 2), kWideThreads, kWideSmem, ctx.stream>>>(
            big, h_nbig, ub, arp, aci, acv, brp, bci, bcv, cnt, crp, cci, ccv);
        ctx.launches++;
        UGPU_LAUNCH_CHECK();
    }
}

}  // namespace

std::unique_ptr<Mat> spgemm(const Mat &A, const Mat &B, bool finalize, SpgemmPlan *plan) {
    Context &ctx = *A.ctx;
    UGPU_CHECK(A.ncols == B.nrows, UGPU_ERR_ARG, "spgemm: inner dimensions differ");
    UGPU_CHECK(A.vdtype == UGPU_F64 && B.vdtype == UGPU_F64, UGPU_ERR_UNSUPPORTED, "spgemm: FP64 operands");
    const int64_t m = A.nrows;
    Buffer ub, cnt, crp64, big, nbig, over, nover;
    ub.alloc(sizeof(int64_t) * std::max<int64_t>(m, 1));
    over.alloc(sizeof(int) * std::max<int64_t>(m, 1));
    nover.alloc(sizeof(int));
    UGPU_CUDA(cudaMemsetAsync(nover.ptr, 0, sizeof(int), ctx.stream));
    cnt.alloc(sizeof(int64_t) * std::max<int64_t>(m, 1));
    crp64.alloc(sizeof(int64_t) * (m + 1));
    big.alloc(sizeof(int) * std::max<int64_t>(m, 1));
    nbig.alloc(sizeof(unsigned long long));  // the maximum upper bound, then the count of big rows
    UGPU_CUDA(cudaMemsetAsync(nbig.ptr, 0, sizeof(int), ctx.stream));
    spgemm_set_attributes();
    // largest per-row upper bound decides whether every row fits a shared-memory table
    unsigned long long max_ub = 0;
    if (m) {
        UGPU_CUDA(cudaMemsetAsync(nbig.ptr, 0, sizeof(unsigned long long), ctx.stream));
        k_row_upper_bound<<<stream_grid(ctx, m), kBlock, 0, ctx.stream>>>(
            A.rowptr.as<int32_t>(), A.colidx.as<int32_t>(), B.rowptr.as<int32_t>(), m, ub.as<int64_t>(),
            nbig.as<unsigned long long>());
        ctx.launches++;
        UGPU_LAUNCH_CHECK();
        UGPU_CUDA(cudaMemcpyAsync(&max_ub, nbig.ptr, sizeof(max_ub), cudaMemcpyDeviceToHost, ctx.stream));
        UGPU_CUDA(cudaMemsetAsync(nbig.ptr, 0, sizeof(int), ctx.stream));
        UGPU_CUDA(cudaStreamSynchronize(ctx.stream));
    }
    // symbolic
    int h_nover = 0;
    launch_warp_tiers<false>(ctx, A, B, max_ub, ub.as<int64_t>(), cnt.as<int64_t>(), nullptr, nullptr, nullptr,
                             big.as<int>(), nbig.as<int>(), over.as<int>(), nover.as<int>(), 0, &h_nover);
    int h_nbig = 0;
    UGPU_CUDA(cudaMemcpyAsync(&h_nbig, nbig.ptr, sizeof(int), cudaMemcpyDeviceToHost, ctx.stream));
    UGPU_CUDA(cudaStreamSynchronize(ctx.stream));
    launch_big_rows<false>(ctx, A, B, max_ub, ub.as<int64_t>(), big.as<int>(), h_nbig, cnt.as<int64_t>(), nullptr,
                           nullptr, nullptr);
    int64_t nnz = device_exclusive_scan(ctx, cnt.as<int64_t>(), crp64.as<int64_t>(), m);
    UGPU_CHECK(nnz < (1ll << 31), UGPU_ERR_UNSUPPORTED, "spgemm: product has more than 2^31 entries");
    auto C = make_csr_device(ctx, m, B.ncols, nnz, UGPU_F64);
    k_i64_to_i32<<<stream_grid(ctx, m + 1), kBlock, 0, ctx.stream>>>(crp64.as<int64_t>(), C->rowptr.as<int32_t>(),
                                                                     m + 1);
    ctx.launches++;
    UGPU_LAUNCH_CHECK();
    // numeric
    launch_warp_tiers<true>(ctx, A, B, max_ub, ub.as<int64_t>(), nullptr, C->rowptr.as<int32_t>(),
                            C->colidx.as<int32_t>(), C->vals.as<double>(), nullptr, nullptr, over.as<int>(), nullptr,
                            h_nover, nullptr);
    launch_big_rows<true>(ctx, A, B, max_ub, ub.as<int64_t>(), big.as<int>(), h_nbig, nullptr,
                          C->rowptr.as<int32_t>(), C->colidx.as<int32_t>(), C->vals.as<double>());
    UGPU_CUDA(cudaStreamSynchronize(ctx.stream));
    if (plan) {
        plan->ub = std::move(ub);
        plan->big = std::move(big);
        plan->h_nbig = h_nbig;
        plan->over = std::move(over);
        plan->h_nover = h_nover;
        plan->max_ub = max_ub;
    }
    if (finalize) finalize_matrix(*C);
    return C;
}

// values of C = A B again, for A and B with the structure the plan was made from
void spgemm_numeric(const Mat &A, const Mat &B, Mat &C, const SpgemmPlan &plan) {
    Context &ctx = *A.ctx;
    launch_warp_tiers<true>(ctx, A, B, plan.max_ub, plan.ub.as<int64_t>(), nullptr, C.rowptr.as<int32_t>(),
                            C.colidx.as<int32_t>(), C.vals.as<double>(), nullptr, nullptr,
                            const_cast<int *>(plan.over.as<int>()), nullptr, plan.h_nover, nullptr);
    launch_big_rows<true>(ctx, A, B, plan.max_ub, plan.ub.as<int64_t>(), plan.big.as<int>(), plan.h_nbig, nullptr,
                          C.rowptr.as<int32_t>(), C.colidx.as<int32_t>(), C.vals.as<double>());
}

std::unique_ptr<Mat> ptap(const Mat &A, const Mat &P) {
    UGPU_CHECK(A.nrows == A.ncols && P.nrows == A.nrows, UGPU_ERR_ARG, "ptap: dimension mismatch");
    auto R = transpose(P, false);   // CSR operands only: no SpMV layout for the intermediates
    auto AP = spgemm(A, P, false);
    return spgemm(*R, *AP);
}

// ------------------------------------------------------------------------------------
// Galerkin products with a kept structure: ptap_with_plan keeps what a later numeric-only
// product needs (the transpose's entry permutation, the A P intermediate and both products'
// row bounds and long-row lists); ptap_numeric recomputes the values of the same product in
// place after the values of A and P changed.  A structure digest of A and P guards the reuse.
// ------------------------------------------------------------------------------------
namespace {

__global__ void k_iota_f64(int64_t n, double *out) {
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
        out[i] = double(i);
}

__global__ void k_f64_to_i64(int64_t n, const double *in, int64_t *out) {
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
        out[i] = int64_t(in[i]);
}

__global__ void k_gather_f64(int64_t n, const double *__restrict__ src, const int64_t *__restrict__ perm,
                             double *__restrict__ dst) {
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
        dst[i] = src[perm[i]];
}

__device__ __forceinline__ unsigned long long mix64(unsigned long long x) {
    x ^= x >> 33;
    x *= 0xff51afd7ed558ccdull;
    x ^= x >> 33;
    x *= 0xc4ceb9fe1a85ec53ull;
    x ^= x >> 33;
    return x;
}

// order-independent digest of (rowptr, colidx): a wrapping sum of mixed (position, value) pairs
__global__ void k_structure_digest(const int32_t *rp, const int32_t *ci, int64_t n, int64_t nnz,
                                   unsigned long long *out) {
    unsigned long long acc = 0;
    const int64_t stride = int64_t(gridDim.x) * blockDim.x;
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i <= n; i += stride)
        acc += mix64((unsigned long long)(i) * 0x9e3779b97f4a7c15ull ^ (unsigned long long)(uint32_t(rp[i])));
    for (int64_t k = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; k < nnz; k += stride)
        acc += mix64(((unsigned long long)(k) << 1 | 1ull) * 0xbf58476d1ce4e5b9ull ^
                     (unsigned long long)(uint32_t(ci[k])));
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(out, acc);
}

}  // namespace

unsigned long long structure_digest(const Mat &A) {
    Context &ctx = *A.ctx;
    Buffer d;
    d.alloc(sizeof(unsigned long long));
    UGPU_CUDA(cudaMemsetAsync(d.ptr, 0, sizeof(unsigned long long), ctx.stream));
    k_structure_digest<<<stream_grid(ctx, std::max<int64_t>(A.nnz, A.nrows + 1)), kBlock, 0, ctx.stream>>>(
        A.rowptr.as<int32_t>(), A.colidx.as<int32_t>(), A.nrows, A.nnz, d.as<unsigned long long>());
    ctx.launches++;
    UGPU_LAUNCH_CHECK();
    unsigned long long h = 0;
    UGPU_CUDA(cudaMemcpyAsync(&h, d.ptr, sizeof(h), cudaMemcpyDeviceToHost, ctx.stream));
    UGPU_CUDA(cudaStreamSynchronize(ctx.stream));
    return h ^ (unsigned long long)(A.nrows) * 31ull ^ (unsigned long long)(A.ncols) << 20;
}

// T = P^T and perm with T.vals[k] = P.vals[perm[k]] (the transpose of P's entry positions)
std::unique_ptr<Mat> transpose_with_perm(const Mat &P, Buffer &perm, bool finalize) {
    UGPU_CHECK(P.vdtype == UGPU_F64, UGPU_ERR_UNSUPPORTED, "transpose_with_perm: FP64 matrix");
    Context &ctx = *P.ctx;
    Mat idx;
    idx.ctx = &ctx;
    idx.nrows = P.nrows;
    idx.ncols = P.ncols;
    idx.nnz = P.nnz;
    idx.vdtype = UGPU_F64;
    idx.rowptr.borrow(P.rowptr.ptr, P.rowptr.bytes);
    idx.colidx.borrow(P.colidx.ptr, P.colidx.bytes);
    idx.vals.alloc(sizeof(double) * std::max<int64_t>(P.nnz, 1));
    k_iota_f64<<<stream_grid(ctx, P.nnz), kBlock, 0, ctx.stream>>>(P.nnz, idx.vals.as<double>());
    ctx.launches++;
    auto T = transpose(idx, false);  // synchronises before it returns
    perm.ensure(sizeof(int64_t) * std::max<int64_t>(P.nnz, 1));
    k_f64_to_i64<<<stream_grid(ctx, P.nnz), kBlock, 0, ctx.stream>>>(P.nnz, T->vals.as<double>(),
                                                                     perm.as<int64_t>());
    ctx.launches++;
    gather_values(ctx, P.nnz, P.vals.as<double>(), perm.as<int64_t>(), T->vals.as<double>());
    if (finalize) {
        UGPU_CUDA(cudaStreamSynchronize(ctx.stream));
        finalize_matrix(*T);
    }
    return T;
}

void gather_values(Context &ctx, int64_t n, const double *src, const int64_t *perm, double *dst) {
    if (n == 0) return;
    k_gather_f64<<<stream_grid(ctx, n), kBlock, 0, ctx.stream>>>(n, src, perm, dst);
    ctx.launches++;
    UGPU_LAUNCH_CHECK();
}

struct PtapPlan {
    unsigned long long a_digest = 0, p_digest = 0;
    int64_t p_nnz = 0;
    std::unique_ptr<Mat> R, AP;  // P^T (values gathered from P through rperm) and A P
    Buffer rperm;
    SpgemmPlan s1, s2;           // A P and R (A P)
};

std::unique_ptr<Mat> ptap_with_plan(const Mat &A, const Mat &P, std::shared_ptr<PtapPlan> &plan) {
    UGPU_CHECK(A.nrows == A.ncols && P.nrows == A.nrows, UGPU_ERR_ARG, "ptap: dimension mismatch");
    UGPU_CHECK(A.vdtype == UGPU_F64 && P.vdtype == UGPU_F64, UGPU_ERR_UNSUPPORTED, "ptap: FP64 operands");
    auto pl = std::make_shared<PtapPlan>();
    pl->a_digest = structure_digest(A);
    pl->p_digest = structure_digest(P);
    pl->p_nnz = P.nnz;
    pl->R = transpose_with_perm(P, pl->rperm, false);
    pl->AP = spgemm(A, P, false, &pl->s1);
    auto C = spgemm(*pl->R, *pl->AP, true, &pl->s2);
    plan = std::move(pl);
    return C;
}

bool ptap_numeric(const Mat &A, const Mat &P, Mat &Ac, PtapPlan &pl, bool finalize) {
    Context &ctx = *A.ctx;
    if (P.nnz != pl.p_nnz || A.nrows != pl.AP->nrows || P.ncols != pl.R->nrows || Ac.nrows != pl.R->nrows)
        return false;
    if (structure_digest(A) != pl.a_digest || structure_digest(P) != pl.p_digest) return false;
    gather_values(ctx, P.nnz, P.vals.as<double>(), pl.rperm.as<int64_t>(), pl.R->vals.as<double>());
    spgemm_numeric(A, P, *pl.AP, pl.s1);
    spgemm_numeric(*pl.R, *pl.AP, Ac, pl.s2);
    Ac.has_diag = false;
    if (finalize) refresh_values(Ac);
    return true;
}

}  // namespace ugpu

using namespace ugpu;

extern "C" {

int ugpu_transpose(const ugpu_mat *A, ugpu_mat **out) {
    UGPU_ABI_BEGIN
    UGPU_REQUIRE(A);
    UGPU_REQUIRE(out);
    auto T = transpose(A->impl);
    auto h = new ugpu_mat;
    h->impl = std::move(*T);
    *out = h;
    UGPU_ABI_END(A ? A->impl.ctx : nullptr)
}

int ugpu_spgemm(const ugpu_mat *A, const ugpu_mat *B, ugpu_mat **out) {
    UGPU_ABI_BEGIN
    UGPU_REQUIRE(A);
    UGPU_REQUIRE(B);
    UGPU_REQUIRE(out);
    auto C = spgemm(A->impl, B->impl);
    auto h = new ugpu_mat;
    h->impl = std::move(*C);
    *out = h;
    UGPU_ABI_END(A ? A->impl.ctx : nullptr)
}

int ugpu_ptap(const ugpu_mat *A, const ugpu_mat *P, ugpu_mat **out) {
    UGPU_ABI_BEGIN
    UGPU_REQUIRE(A);
    UGPU_REQUIRE(P);
    UGPU_REQUIRE(out);
    auto C = ptap(A->impl, P->impl);
    auto h = new ugpu_mat;
    h->impl = std::move(*C);
    *out = h;
    UGPU_ABI_END(A ? A->impl.ctx : nullptr)
}

int ugpu_ptap_reuse(const ugpu_mat *A, const ugpu_mat *P, int reuse, ugpu_mat **out) {
    UGPU_ABI_BEGIN
    UGPU_REQUIRE(A);
    UGPU_REQUIRE(P);
    UGPU_REQUIRE(out);
    UGPU_CHECK(reuse == 0 || reuse == 1, UGPU_ERR_ARG, "reuse: 0 (initial matrix) or 1 (reuse matrix)");
    if (reuse == 1) {
        UGPU_CHECK(*out && (*out)->impl.ptap_plan, UGPU_ERR_ARG,
                   "reuse: the matrix must come from an earlier ugpu_ptap_reuse(..., 0, ...)");
        Mat &Ac = (*out)->impl;
        UGPU_CHECK(ptap_numeric(A->impl, P->impl, Ac, *Ac.ptap_plan, true), UGPU_ERR_ARG,
                   "reuse: A or P no longer has the structure the product was formed from");
    } else {
        std::shared_ptr<PtapPlan> plan;
        auto C = ptap_with_plan(A->impl, P->impl, plan);
        C->ptap_plan = std::move(plan);
        auto h = new ugpu_mat;
        h->impl = std::move(*C);
        *out = h;
    }
    UGPU_ABI_END(A ? A->impl.ctx : nullptr)
}

}  // extern "C"
