// convert.cu -- CSR -> row-window block-condensed format on the GPU.
//
// Bit-identical to the reference CPU conversion blockProcess_fp16_balance /
// blockProcess_tf32_balance (gcn/Block_gcn/example.cpp:48-348) and extends it
// with the GAT slot->edge maps (ATT_Block*.blockProcess_sddmm_balance_gnn
// [_trans], Block/include/example.h:4-6).  Where the reference builds a
// std::set per window on the CPU and concatenates serially
// (example.cpp:61-175), this is an integer sort / scan / compaction pipeline:
//
//   plan  k_unique_small   one CTA per window of <= kSmallCap edges: bitonic
//                          sort in shared memory, de-duplicate, compact
//         k_unique_large   windows above the cap: per-CTA column bitmap in
//                          global scratch (L2-resident), popcount-scan compaction
//         k_window_counts  padded width and part count per window
//         exclusive scans  column offsets and part offsets (int64, 3 kernels)
//   fill  k_fill_structure one warp per window: condensed column list with -1
//                          padding, rowptr pairs, window id, atomic flag
//         k_fill_edges     one thread per CSR edge: binary-search its condensed
//                          column, write value / slot->edge map / mirrored map
//
// All integer work; HBM- and L2-latency bound.
#include "att_common.cuh"

namespace att {
namespace {

constexpr int kSmallCap = 4096;     // windows up to this many edges sort in smem
constexpr int kSmallThreads = 512;  // kSmallCap / 8
constexpr int kLargeThreads = 512;
constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;
constexpr int kMaxBitmapCtas = 128;
constexpr size_t kBitmapBudget = 256ull << 20;  // bytes of bitmap scratch at most

enum { FLAG_BAD_COL = 1, FLAG_BAD_ROWPTR = 2, FLAG_UNSORTED = 4, FLAG_OVERFLOW = 8 };

struct Workspace {
    int32_t *ucols;      // [nnz]      sorted distinct columns, at each window's edge offset
    int32_t *ucount;     // [n_win]    distinct columns per window
    int64_t *col_off;    // [n_win+1]  exclusive scan of padded widths
    int64_t *part_off;   // [n_win+1]  exclusive scan of part counts
    int64_t *scan_tmp;   // [2*nblk]
    int32_t *flags;      // [4]
    int64_t *summary;    // [3]  n_condensed, n_parts, flags (the plan's result)
    uint32_t *bitmap;    // [n_bitmap_ctas * words]
    int n_bitmap_ctas;
    int64_t words;
};

int64_t n_windows(int64_t n_rows, int window) { return n_rows / window; }

int bitmap_ctas(int64_t n_cols) {
    int64_t words = (n_cols + 31) / 32;
    int64_t by_budget = (int64_t)(kBitmapBudget / (size_t)((words > 0 ? words : 1) * 4));
    if (by_budget < 1) by_budget = 1;
    return (int)(by_budget < kMaxBitmapCtas ? by_budget : kMaxBitmapCtas);
}

size_t workspace_layout(int64_t n_rows, int64_t nnz, int64_t n_cols, int window, Workspace *ws,
                        char *base) {
    int64_t nw = n_windows(n_rows, window);
    int64_t nblk = (nw + 1 + kScanTile - 1) / kScanTile;
    int64_t words = (n_cols + 31) / 32;
    int nb = bitmap_ctas(n_cols);
    size_t off = 0;
    auto take = [&](size_t bytes) {
        size_t o = off;
        off = align_up(off + bytes, 256);
        return o;
    };
    size_t o_ucols = take((size_t)(nnz > 0 ? nnz : 1) * 4);
    size_t o_ucount = take((size_t)(nw + 1) * 4);
    size_t o_col = take((size_t)(nw + 1) * 8);
    size_t o_part = take((size_t)(nw + 1) * 8);
    size_t o_scan = take((size_t)(2 * nblk + 2) * 8);
    size_t o_flags = take(16);
    size_t o_sum = take(24);
    size_t o_bitmap = take((size_t)nb * (size_t)(words > 0 ? words : 1) * 4);
    if (ws && base) {
        ws->ucols = (int32_t *)(base + o_ucols);
        ws->ucount = (int32_t *)(base + o_ucount);
        ws->col_off = (int64_t *)(base + o_col);
        ws->part_off = (int64_t *)(base + o_part);
        ws->scan_tmp = (int64_t *)(base + o_scan);
        ws->flags = (int32_t *)(base + o_flags);
        ws->summary = (int64_t *)(base + o_sum);
        ws->bitmap = (uint32_t *)(base + o_bitmap);
        ws->n_bitmap_ctas = nb;
        ws->words = words;
    }
    return off;
}

// ---- block-wide exclusive scan of one int per thread ----------------------
template <int THREADS>
__device__ __forceinline__ int block_exclusive_scan(int v, int *total, int *sh /*[THREADS/32+1]*/) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) sh[wid] = x;
    __syncthreads();
    if (wid == 0) {
        int s = lane < THREADS / 32 ? sh[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        if (lane < THREADS / 32) sh[lane] = s;  // inclusive warp totals
    }
    __syncthreads();
    int warp_prefix = wid > 0 ? sh[wid - 1] : 0;
    int res = warp_prefix + x - v;
    *total = sh[THREADS / 32 - 1];
    __syncthreads();
    return res;
}

__device__ __forceinline__ bool window_range(const int32_t *rowptr, int64_t w, int window,
                                             int64_t nnz, int64_t *b0, int64_t *b1,
                                             int32_t *flags) {
    int64_t s = rowptr[w * window], e = rowptr[(w + 1) * window];
    if (s < 0 || e < s || e > nnz) {
        atomicOr(flags, FLAG_BAD_ROWPTR);
        *b0 = *b1 = 0;
        return false;
    }
    *b0 = s;
    *b1 = e;
    return true;
}

// ---- plan: distinct sorted columns per window ------------------------------
// Windows of at most kWarpCap edges (most windows of a sparse graph): one warp
// each, a bitonic sort of the window's column ids in the warp's own slice of
// shared memory (warp-synchronous, no block barriers), then de-duplication
// and a warp scan to compact.
constexpr int kWarpCap = 256;
constexpr int kWarpSortWarps = 8;

__global__ void __launch_bounds__(kWarpSortWarps * 32) k_unique_warp(
    const int32_t *__restrict__ rowptr, const int32_t *__restrict__ col, int64_t n_win,
    int window, int64_t nnz, int64_t n_cols, Workspace ws) {
    __shared__ int keys_all[kWarpSortWarps][kWarpCap];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    int *keys = keys_all[wib];
    const int64_t nwarps = (int64_t)gridDim.x * kWarpSortWarps;
    for (int64_t w = (int64_t)blockIdx.x * kWarpSortWarps + wib; w < n_win; w += nwarps) {
        int64_t b0, b1;
        window_range(rowptr, w, window, nnz, &b0, &b1, ws.flags);
        const int64_t E = b1 - b0;
        if (E > kWarpCap) continue;  // k_unique_small / k_unique_large
        int n = 32;
        while (n < E) n <<= 1;
        for (int t = lane; t < n; t += 32) {
            int c = INT32_MAX;
            if (t < E) {
                c = col[b0 + t];
                if (c < 0 || c >= n_cols) {
                    atomicOr(ws.flags, FLAG_BAD_COL);
                    c = INT32_MAX;
                }
            }
            keys[t] = c;
        }
        __syncwarp();
        for (int k = 2; k <= n; k <<= 1) {
            for (int j = k >> 1; j > 0; j >>= 1) {
                for (int t = lane; t < (n >> 1); t += 32) {
                    const int i = 2 * t - (t & (j - 1)), l = i + j;  // pair (i, i + j)
                    const int a = keys[i], b = keys[l];
                    if ((a > b) == ((i & k) == 0)) {
                        keys[i] = b;
                        keys[l] = a;
                    }
                }
                __syncwarp();
            }
        }
        // de-duplicate: lane owns n / 32 consecutive sorted keys
        const int per = n >> 5, base = lane * per;
        int cnt = 0;
        for (int q = 0; q < per; ++q) {
            const int kk = base + q;
            if (kk < E) {
                const int v = keys[kk];
                if (v != INT32_MAX && (kk == 0 || keys[kk - 1] != v)) cnt++;
            }
        }
        int x = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        const int total = __shfl_sync(0xffffffffu, x, 31);
        int pos = x - cnt;
        for (int q = 0; q < per; ++q) {
            const int kk = base + q;
            if (kk < E) {
                const int v = keys[kk];
                if (v != INT32_MAX && (kk == 0 || keys[kk - 1] != v)) ws.ucols[b0 + pos++] = v;
            }
        }
        if (lane == 0) ws.ucount[w] = total;
        __syncwarp();
    }
}

// Windows of kWarpCap+1 .. kSmallCap edges: one CTA each, bitonic sort in
// shared memory across the block.
__global__ void __launch_bounds__(kSmallThreads) k_unique_small(
    const int32_t *__restrict__ rowptr, const int32_t *__restrict__ col, int64_t n_win,
    int window, int64_t nnz, int64_t n_cols, Workspace ws) {
    __shared__ int keys[kSmallCap];
    __shared__ int sh[kSmallThreads / 32 + 1];
    for (int64_t w = blockIdx.x; w < n_win; w += gridDim.x) {
        int64_t b0, b1;
        window_range(rowptr, w, window, nnz, &b0, &b1, ws.flags);
        int64_t E = b1 - b0;
        if (E > kSmallCap || E <= kWarpCap) continue;  // k_unique_large / k_unique_warp
        int n = 1;
        while (n < E) n <<= 1;
        for (int t = threadIdx.x; t < n; t += kSmallThreads) {
            int c = INT32_MAX;
            if (t < E) {
                c = col[b0 + t];
                if (c < 0 || c >= n_cols) {
                    atomicOr(ws.flags, FLAG_BAD_COL);
                    c = INT32_MAX;
                }
            }
            keys[t] = c;
        }
        __syncthreads();
        // bitonic sort, ascending
        for (int k = 2; k <= n; k <<= 1) {
            for (int j = k >> 1; j > 0; j >>= 1) {
                for (int t = threadIdx.x; t < (n >> 1); t += kSmallThreads) {
                    int i = 2 * t - (t & (j - 1));  // (t / j) * 2j + t % j, j a power of two
                    int l = i + j;
                    int a = keys[i], b = keys[l];
                    bool up = (i & k) == 0;
                    if ((a > b) == up) {
                        keys[i] = b;
                        keys[l] = a;
                    }
                }
                __syncthreads();
            }
        }
        // de-duplicate: each thread owns 8 consecutive sorted keys
        int base = threadIdx.x * 8, cnt = 0;
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            int k = base + q;
            if (k < E) {
                int v = keys[k];
                if (v != INT32_MAX && (k == 0 || keys[k - 1] != v)) cnt++;
            }
        }
        int total;
        int pos = block_exclusive_scan<kSmallThreads>(cnt, &total, sh);
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            int k = base + q;
            if (k < E) {
                int v = keys[k];
                if (v != INT32_MAX && (k == 0 || keys[k - 1] != v)) ws.ucols[b0 + pos++] = v;
            }
        }
        if (threadIdx.x == 0) ws.ucount[w] = total;
        __syncthreads();
    }
}

__global__ void __launch_bounds__(kLargeThreads) k_unique_large(
    const int32_t *__restrict__ rowptr, const int32_t *__restrict__ col, int64_t n_win,
    int window, int64_t nnz, int64_t n_cols, Workspace ws) {
    __shared__ int sh[kLargeThreads / 32 + 1];
    uint32_t *bm = ws.bitmap + (int64_t)blockIdx.x * ws.words;
    const int64_t words = ws.words;
    const int64_t chunk = (words + kLargeThreads - 1) / kLargeThreads;
    for (int64_t w = blockIdx.x; w < n_win; w += gridDim.x) {
        int64_t b0 = rowptr[w * window], b1 = rowptr[(w + 1) * window];
        if (b0 < 0 || b1 < b0 || b1 > nnz) continue;  // flagged by k_unique_small
        if (b1 - b0 <= kSmallCap) continue;
        for (int64_t t = threadIdx.x; t < words; t += kLargeThreads) bm[t] = 0u;
        __syncthreads();
        for (int64_t e = b0 + threadIdx.x; e < b1; e += kLargeThreads) {
            int c = col[e];
            if (c < 0 || c >= n_cols) {
                atomicOr(ws.flags, FLAG_BAD_COL);
                continue;
            }
            atomicOr(&bm[c >> 5], 1u << (c & 31));
        }
        __syncthreads();
        int64_t w0 = (int64_t)threadIdx.x * chunk;
        int64_t w1 = w0 + chunk < words ? w0 + chunk : words;
        int cnt = 0;
        for (int64_t q = w0; q < w1; ++q) cnt += __popc(bm[q]);
        int total;
        int pos = block_exclusive_scan<kLargeThreads>(cnt, &total, sh);
        for (int64_t q = w0; q < w1; ++q) {
            uint32_t bits = bm[q];
            while (bits) {
                int b = __ffs(bits) - 1;
                ws.ucols[b0 + pos++] = (int32_t)(q * 32 + b);
                bits &= bits - 1;
            }
        }
        if (threadIdx.x == 0) ws.ucount[w] = total;
        __syncthreads();
    }
}

// padded width and part count per window -> col_off / part_off (before scan)
__global__ void k_window_counts(int64_t n_win, int wide, int part, int emit_empty, Workspace ws) {
    int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (w > n_win) return;
    if (w == n_win) {
        ws.col_off[w] = 0;
        ws.part_off[w] = 0;
        return;
    }
    int64_t u = ws.ucount[w];
    int64_t pad = (u + wide - 1) / wide * wide;
    int64_t blocks = pad / wide;
    int64_t np = blocks == 0 ? (emit_empty ? 1 : 0) : (blocks + part - 1) / part;
    ws.col_off[w] = pad;
    ws.part_off[w] = np;
}

// ---- int64 exclusive scan (in place), three kernels ------------------------
__device__ __forceinline__ int64_t block_scan64(int64_t v, int64_t *total, int64_t *sh) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int64_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int64_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) sh[wid] = x;
    __syncthreads();
    if (wid == 0) {
        int64_t s = lane < kScanThreads / 32 ? sh[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int64_t y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        if (lane < kScanThreads / 32) sh[lane] = s;
    }
    __syncthreads();
    int64_t res = (wid > 0 ? sh[wid - 1] : 0) + x - v;
    *total = sh[kScanThreads / 32 - 1];
    __syncthreads();
    return res;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_reduce(const int64_t *a, int64_t n,
                                                              int64_t *sums) {
    __shared__ int64_t sh[kScanThreads / 32];
    int64_t base = (int64_t)blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    int64_t s = 0;
#pragma unroll
    for (int q = 0; q < kScanItems; ++q)
        if (base + q < n) s += a[base + q];
    int64_t total;
    block_scan64(s, &total, sh);
    if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_sums(int64_t *sums, int64_t nblk) {
    __shared__ int64_t sh[kScanThreads / 32];
    int64_t carry = 0;
    for (int64_t b0 = 0; b0 < nblk; b0 += kScanThreads) {
        int64_t i = b0 + threadIdx.x;
        int64_t v = i < nblk ? sums[i] : 0;
        int64_t total;
        int64_t ex = block_scan64(v, &total, sh);
        if (i < nblk) sums[i] = carry + ex;
        carry += total;
    }
}

__global__ void __launch_bounds__(kScanThreads) k_scan_apply(int64_t *a, int64_t n,
                                                             const int64_t *sums) {
    __shared__ int64_t sh[kScanThreads / 32];
    int64_t base = (int64_t)blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    int64_t v[kScanItems];
    int64_t s = 0;
#pragma unroll
    for (int q = 0; q < kScanItems; ++q) {
        v[q] = base + q < n ? a[base + q] : 0;
        s += v[q];
    }
    int64_t total;
    int64_t ex = block_scan64(s, &total, sh) + sums[blockIdx.x];
#pragma unroll
    for (int q = 0; q < kScanItems; ++q) {
        if (base + q < n) a[base + q] = ex;
        ex += v[q];
    }
}

int exclusive_scan64(int64_t *a, int64_t n, int64_t *tmp, cudaStream_t st) {
    int64_t nblk = (n + kScanTile - 1) / kScanTile;
    if (nblk == 0) return ATT_OK;
    k_scan_reduce<<<(unsigned)nblk, kScanThreads, 0, st>>>(a, n, tmp);
    k_scan_sums<<<1, kScanThreads, 0, st>>>(tmp, nblk);
    k_scan_apply<<<(unsigned)nblk, kScanThreads, 0, st>>>(a, n, tmp);
    return launch_status("exclusive_scan64");
}

// ---- fill: structure ---------------------------------------------------------
__global__ void k_fill_structure(int64_t n_win, int window, int wide, int part, int emit_empty,
                                 Workspace ws, const int32_t *__restrict__ rowptr,
                                 int32_t *__restrict__ out_rowptr, int32_t *__restrict__ out_col,
                                 int32_t *__restrict__ out_window,
                                 int32_t *__restrict__ out_atomic) {
    const int lane = threadIdx.x & 31;
    int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (w == 0 && lane == 0) out_rowptr[0] = 0;
    if (w >= n_win) return;
    int64_t u = ws.ucount[w];
    int64_t cbase = ws.col_off[w];
    int64_t pad = ws.col_off[w + 1] - cbase;
    int64_t pbase = ws.part_off[w];
    int64_t np = ws.part_off[w + 1] - pbase;
    int64_t b0 = rowptr[w * window];
    for (int64_t k = lane; k < pad; k += 32) out_col[cbase + k] = k < u ? ws.ucols[b0 + k] : -1;
    int64_t blocks = pad / wide;
    int64_t padamt = pad - u;
    for (int64_t p = lane; p < np; p += 32) {
        int64_t r_end, p_end;
        if (blocks == 0) {
            r_end = p_end = cbase;
        } else {
            int64_t nb = blocks - p * part < part ? blocks - p * part : part;
            int64_t start = cbase + p * part * wide;
            p_end = start + nb * wide;
            r_end = p_end - (p == np - 1 ? padamt : 0);
        }
        out_rowptr[2 * (pbase + p) + 1] = (int32_t)r_end;
        out_rowptr[2 * (pbase + p) + 2] = (int32_t)p_end;
        out_window[pbase + p] = (int32_t)w;
        out_atomic[pbase + p] = np > 1 ? 1 : 0;
    }
}

// ---- fill: per-edge values and maps -----------------------------------------------
template <typename VT>
__device__ __forceinline__ VT from_f32(float x);
template <>
__device__ __forceinline__ __half from_f32<__half>(float x) { return __float2half_rn(x); }
template <>
__device__ __forceinline__ __nv_bfloat16 from_f32<__nv_bfloat16>(float x) {
    return __float2bfloat16_rn(x);
}
template <>
__device__ __forceinline__ float from_f32<float>(float x) { return x; }

__device__ __forceinline__ float deg_at(const void *deg, int deg_dtype, int64_t i) {
    if (deg_dtype == ATT_F16) return __half2float(((const __half *)deg)[i]);
    return ((const float *)deg)[i];
}

template <typename VT>
__global__ void k_fill_edges(const int32_t *__restrict__ rowptr, const int32_t *__restrict__ col,
                             int64_t n_rows_used, int window, int wide, int64_t n_cols,
                             int64_t n_rows, Workspace ws, const void *__restrict__ deg,
                             int deg_dtype, VT *__restrict__ out_val, int32_t *__restrict__ out_map,
                             int32_t *__restrict__ out_map_t, int32_t *__restrict__ out_edge_slot,
                             int64_t nnz) {
    const int64_t e0 = rowptr[0], e_end = rowptr[n_rows_used];
    int64_t e = e0 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e0 < 0 || e_end > nnz || e_end < e0) return;
    if (e >= e_end) return;  // edges of dropped trailing rows keep slot -1
    // row of edge e: last r with rowptr[r] <= e
    int64_t lo = 0, hi = n_rows_used - 1;
    while (lo < hi) {
        int64_t mid = (lo + hi + 1) >> 1;
        if (rowptr[mid] <= e) lo = mid; else hi = mid - 1;
    }
    const int64_t row = lo;
    const int32_t c = col[e];
    if (c < 0 || c >= n_cols) {
        if (out_edge_slot) out_edge_slot[e] = -1;
        return;  // flagged during plan
    }
    if (e > rowptr[row] && col[e - 1] > c) atomicOr(ws.flags, FLAG_UNSORTED);
    const int64_t w = row / window, r = row - w * window;
    const int64_t b0 = rowptr[w * window];
    const int64_t u = ws.ucount[w];
    const int32_t *uc = ws.ucols + b0;
    int64_t a = 0, b = u;
    while (a < b) {
        int64_t m = (a + b) >> 1;
        if (uc[m] < c) a = m + 1; else b = m;
    }
    const int64_t ci = a;
    const int64_t slot = (ws.col_off[w] + (ci / wide) * wide) * window + r * wide + (ci % wide);
    if (out_val) {
        float v = deg_at(deg, deg_dtype, row) * deg_at(deg, deg_dtype, c);
        out_val[slot] = from_f32<VT>(v);
    }
    if (out_map) atomicMax(&out_map[slot], (int32_t)e);
    if (out_edge_slot) out_edge_slot[e] = (int32_t)slot;
    if (out_map_t) {
        int32_t t = -1;
        if (c < n_rows) {
            // last position in row c with col <= row (rows sorted ascending)
            int64_t s0 = rowptr[c], s1 = rowptr[c + 1];
            int64_t x = s0, y = s1;
            while (x < y) {
                int64_t m = (x + y) >> 1;
                if (col[m] <= row) x = m + 1; else y = m;
            }
            if (x > s0 && col[x - 1] == row) t = (int32_t)(x - 1);
        }
        // duplicates of (row,c) share a slot and compute the same t
        out_map_t[slot] = t;
    }
}

// {n_condensed, n_parts, flags} of a finished plan, for one copy to the host
__global__ void k_plan_summary(Workspace ws, int64_t nw) {
    ws.summary[0] = ws.col_off[nw];
    ws.summary[1] = ws.part_off[nw];
    ws.summary[2] = ws.flags[0];
}
}  // namespace

size_t scan64_tmp_bytes(int64_t n) {
    return (size_t)((n + kScanTile - 1) / kScanTile + 1) * sizeof(int64_t);
}
int scan64_exclusive(int64_t *a, int64_t n, int64_t *tmp, cudaStream_t st) {
    return exclusive_scan64(a, n, tmp, st);
}
}  // namespace att

using namespace att;

extern "C" size_t att_block_workspace_bytes(int64_t n_rows, int64_t nnz, int64_t n_cols,
                                            int window) {
    if (window <= 0 || n_rows < 0) return 0;
    return workspace_layout(n_rows, nnz, n_cols, window, nullptr, nullptr);
}

static int check_conv_args(const int32_t *rowptr, const int32_t *col, int64_t n_rows, int64_t nnz,
                           int64_t n_cols, int window, int wide, int part) {
    ATT_CHECK(rowptr != nullptr, ATT_ERR_INVALID, "rowptr is null");
    ATT_CHECK(nnz == 0 || col != nullptr, ATT_ERR_INVALID, "col is null");
    ATT_CHECK(n_rows >= 0 && nnz >= 0 && n_cols >= 0, ATT_ERR_INVALID, "negative size");
    ATT_CHECK(window > 0 && window <= 64, ATT_ERR_INVALID, "window must be in [1,64], got %d",
              window);
    ATT_CHECK(wide > 0 && wide <= 64, ATT_ERR_INVALID, "wide must be in [1,64], got %d", wide);
    ATT_CHECK(part > 0, ATT_ERR_INVALID, "partSize must be positive, got %d", part);
    ATT_CHECK(nnz <= INT32_MAX, ATT_ERR_OVERFLOW, "nnz %lld exceeds int32 edge ids",
              (long long)nnz);
    return ATT_OK;
}

// Enqueue phase 1 on `st`, ending with the summary {n_condensed, n_parts,
// flags} in ws.summary.
static int plan_enqueue(const int32_t *rowptr, const int32_t *col, int64_t n_rows, int64_t nnz,
                 int64_t n_cols, int window, int wide, int part, int emit_empty, void *workspace,
                 size_t workspace_bytes, Workspace &ws, cudaStream_t st) {
    int s = check_conv_args(rowptr, col, n_rows, nnz, n_cols, window, wide, part);
    if (s != ATT_OK) return s;
    size_t need = workspace_layout(n_rows, nnz, n_cols, window, nullptr, nullptr);
    ATT_CHECK(workspace != nullptr && workspace_bytes >= need, ATT_ERR_WORKSPACE,
              "workspace %zu bytes < %zu needed", workspace_bytes, need);
    workspace_layout(n_rows, nnz, n_cols, window, &ws, (char *)workspace);
    const int64_t nw = n_windows(n_rows, window);
    ATT_CUDA(cudaMemsetAsync(ws.flags, 0, 16, st), "memset flags");
    if (nw > 0) {
        ATT_CUDA(cudaMemsetAsync(ws.ucount, 0, (size_t)nw * 4, st), "memset ucount");
        int sms = sm_count();
        int64_t g_small = nw < (int64_t)sms * 32 ? nw : (int64_t)sms * 32;
        const int64_t g_warp0 = (nw + kWarpSortWarps - 1) / kWarpSortWarps;
        const int64_t g_warp = g_warp0 < (int64_t)sms * 16 ? g_warp0 : (int64_t)sms * 16;
        k_unique_warp<<<(unsigned)g_warp, kWarpSortWarps * 32, 0, st>>>(rowptr, col, nw, window,
                                                                          nnz, n_cols, ws);
        ATT_CUDA(cudaGetLastError(), "k_unique_warp");
        k_unique_small<<<(unsigned)g_small, kSmallThreads, 0, st>>>(rowptr, col, nw, window, nnz,
                                                                     n_cols, ws);
        int64_t g_large = nw < ws.n_bitmap_ctas ? nw : ws.n_bitmap_ctas;
        k_unique_large<<<(unsigned)g_large, kLargeThreads, 0, st>>>(rowptr, col, nw, window, nnz,
                                                                     n_cols, ws);
        s = launch_status("k_unique");
        if (s != ATT_OK) return s;
    }
    k_window_counts<<<(unsigned)((nw + 1 + 255) / 256), 256, 0, st>>>(nw, wide, part, emit_empty,
                                                                       ws);
    s = launch_status("k_window_counts");
    if (s != ATT_OK) return s;
    s = exclusive_scan64(ws.col_off, nw + 1, ws.scan_tmp, st);
    if (s != ATT_OK) return s;
    s = exclusive_scan64(ws.part_off, nw + 1, ws.scan_tmp, st);
    if (s != ATT_OK) return s;
    k_plan_summary<<<1, 1, 0, st>>>(ws, nw);
    return launch_status("k_plan_summary");
}

static int plan_check(const int64_t *sum, int window, int64_t n_cols, int64_t *n_parts_out,
               int64_t *n_condensed_out) {
    const int64_t flags = sum[2];
    ATT_CHECK(!(flags & FLAG_BAD_ROWPTR), ATT_ERR_FORMAT, "rowptr is not monotone or exceeds nnz");
    ATT_CHECK(!(flags & FLAG_BAD_COL), ATT_ERR_FORMAT, "column id outside [0, %lld)",
              (long long)n_cols);
    ATT_CHECK(sum[0] * window <= INT32_MAX && 2 * sum[1] + 1 <= INT32_MAX, ATT_ERR_OVERFLOW,
              "block format would exceed int32 indexing (%lld condensed columns)",
              (long long)sum[0]);
    *n_condensed_out = sum[0];
    *n_parts_out = sum[1];
    return ATT_OK;
}

extern "C" int att_block_plan(const int32_t *rowptr, const int32_t *col, int64_t n_rows,
                              int64_t nnz, int64_t n_cols, int window, int wide, int part,
                              int emit_empty, void *workspace, size_t workspace_bytes,
                              int64_t *n_parts_out, int64_t *n_condensed_out, void *stream) {
    clear_error();
    ATT_CHECK(n_parts_out && n_condensed_out, ATT_ERR_INVALID, "null size outputs");
    cudaStream_t st = (cudaStream_t)stream;
    Workspace ws;
    int s = plan_enqueue(rowptr, col, n_rows, nnz, n_cols, window, wide, part, emit_empty,
                         workspace, workspace_bytes, ws, st);
    if (s != ATT_OK) return s;
    int64_t sum[3];
    ATT_CUDA(cudaMemcpyAsync(sum, ws.summary, sizeof(sum), cudaMemcpyDeviceToHost, st), "d2h");
    ATT_CUDA(cudaStreamSynchronize(st), "plan sync");
    return plan_check(sum, window, n_cols, n_parts_out, n_condensed_out);
}

extern "C" int att_block_plan_async(const int32_t *rowptr, const int32_t *col, int64_t n_rows,
                                    int64_t nnz, int64_t n_cols, int window, int wide, int part,
                                    int emit_empty, void *workspace, size_t workspace_bytes,
                                    int64_t *summary, void *stream) {
    clear_error();
    ATT_CHECK(summary != nullptr, ATT_ERR_INVALID, "null summary");
    cudaStream_t st = (cudaStream_t)stream;
    Workspace ws;
    int s = plan_enqueue(rowptr, col, n_rows, nnz, n_cols, window, wide, part, emit_empty,
                         workspace, workspace_bytes, ws, st);
    if (s != ATT_OK) return s;
    ATT_CUDA(cudaMemcpyAsync(summary, ws.summary, 3 * sizeof(int64_t), cudaMemcpyDefault, st),
             "summary copy");
    return ATT_OK;
}

extern "C" int att_block_plan_result(const int64_t *summary, int64_t n_cols, int window,
                                     int64_t *n_parts_out, int64_t *n_condensed_out) {
    clear_error();
    ATT_CHECK(summary && n_parts_out && n_condensed_out && window > 0, ATT_ERR_INVALID,
              "null argument");
    return plan_check(summary, window, n_cols, n_parts_out, n_condensed_out);
}

extern "C" int att_block_fill(const int32_t *rowptr, const int32_t *col, int64_t n_rows,
                              int64_t nnz, int64_t n_cols, int window, int wide, int part,
                              int emit_empty, const void *deg, int deg_dtype,
                              const void *workspace, size_t workspace_bytes, int32_t *out_rowptr,
                              int32_t *out_col, void *out_val, int val_dtype, int32_t *out_map,
                              int32_t *out_map_t, int32_t *out_edge_slot, int32_t *out_window,
                              int32_t *out_atomic, void *stream) {
    clear_error();
    int s = check_conv_args(rowptr, col, n_rows, nnz, n_cols, window, wide, part);
    if (s != ATT_OK) return s;
    size_t need = workspace_layout(n_rows, nnz, n_cols, window, nullptr, nullptr);
    ATT_CHECK(workspace != nullptr && workspace_bytes >= need, ATT_ERR_WORKSPACE,
              "workspace %zu bytes < %zu needed", workspace_bytes, need);
    ATT_CHECK(out_rowptr != nullptr, ATT_ERR_INVALID, "rowptr output is null");
    if (out_val) {
        ATT_CHECK(deg != nullptr && (deg_dtype == ATT_F16 || deg_dtype == ATT_F32),
                  ATT_ERR_INVALID, "values need fp16 or fp32 degrees");
        ATT_CHECK(val_dtype == ATT_F16 || val_dtype == ATT_BF16 || val_dtype == ATT_F32,
                  ATT_ERR_INVALID, "val_dtype must be f16, bf16 or f32");
    }
    Workspace ws;
    workspace_layout(n_rows, nnz, n_cols, window, &ws, (char *)workspace);
    cudaStream_t st = (cudaStream_t)stream;
    const int64_t nw = n_windows(n_rows, window);
    int64_t tot[2] = {0, 0};
    ATT_CUDA(cudaMemcpyAsync(&tot[0], ws.col_off + nw, 8, cudaMemcpyDeviceToHost, st), "d2h");
    ATT_CUDA(cudaMemcpyAsync(&tot[1], ws.part_off + nw, 8, cudaMemcpyDeviceToHost, st), "d2h");
    ATT_CUDA(cudaStreamSynchronize(st), "fill sync");
    const int64_t n_cond = tot[0], n_parts = tot[1];
    ATT_CHECK(n_cond == 0 || out_col != nullptr, ATT_ERR_INVALID, "col output is null");
    ATT_CHECK(n_parts == 0 || (out_window && out_atomic), ATT_ERR_INVALID,
              "window/atomic output is null");
    const size_t nslot = (size_t)n_cond * (size_t)window;
    size_t vbytes = val_dtype == ATT_F32 ? 4 : 2;
    if (out_val && nslot) ATT_CUDA(cudaMemsetAsync(out_val, 0, nslot * vbytes, st), "memset val");
    if (out_map && nslot) ATT_CUDA(cudaMemsetAsync(out_map, 0xff, nslot * 4, st), "memset map");
    if (out_map_t && nslot)
        ATT_CUDA(cudaMemsetAsync(out_map_t, 0xff, nslot * 4, st), "memset map_t");
    if (out_edge_slot && nnz) ATT_CUDA(cudaMemsetAsync(out_edge_slot, 0xff, (size_t)nnz * 4, st),
                                       "memset edge_slot");
    ATT_CUDA(cudaMemsetAsync(ws.flags, 0, 16, st), "memset flags");
    {
        int64_t threads = (nw > 0 ? nw : 1) * 32;
        k_fill_structure<<<(unsigned)((threads + 255) / 256), 256, 0, st>>>(
            nw, window, wide, part, emit_empty, ws, rowptr, out_rowptr, out_col, out_window,
            out_atomic);
        s = launch_status("k_fill_structure");
        if (s != ATT_OK) return s;
    }
    if (nw > 0 && (out_val || out_map || out_map_t || out_edge_slot)) {
        int64_t rows_used = nw * window;
        // upper bound of edges in used rows is nnz; threads beyond the range exit
        int64_t n_threads = nnz > 0 ? nnz : 1;
        unsigned grid = (unsigned)((n_threads + 255) / 256);
        if (!out_val || val_dtype == ATT_F16) {
            k_fill_edges<__half><<<grid, 256, 0, st>>>(rowptr, col, rows_used, window, wide,
                                                       n_cols, n_rows, ws, deg, deg_dtype,
                                                       (__half *)out_val, out_map, out_map_t,
                                                       out_edge_slot, nnz);
        } else if (val_dtype == ATT_BF16) {
            k_fill_edges<__nv_bfloat16><<<grid, 256, 0, st>>>(
                rowptr, col, rows_used, window, wide, n_cols, n_rows, ws, deg, deg_dtype,
                (__nv_bfloat16 *)out_val, out_map, out_map_t, out_edge_slot, nnz);
        } else {
            k_fill_edges<float><<<grid, 256, 0, st>>>(rowptr, col, rows_used, window, wide,
                                                      n_cols, n_rows, ws, deg, deg_dtype,
                                                      (float *)out_val, out_map, out_map_t,
                                                      out_edge_slot, nnz);
        }
        s = launch_status("k_fill_edges");
        if (s != ATT_OK) return s;
    }
    int32_t flags[4];
    ATT_CUDA(cudaMemcpyAsync(flags, ws.flags, 16, cudaMemcpyDeviceToHost, st), "d2h");
    ATT_CUDA(cudaStreamSynchronize(st), "fill sync");
    ATT_CHECK(!(out_map_t && (flags[0] & FLAG_UNSORTED)), ATT_ERR_FORMAT,
              "mirrored-edge map needs every CSR row sorted by column");
    return ATT_OK;
}
