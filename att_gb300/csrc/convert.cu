// convert.cu -- CSR -> row-window block-condensed format on the GPU.
//
// Bit-identical to the reference CPU conversion blockProcess_fp16_balance /
// blockProcess_tf32_balance (gcn/Block_gcn/example.cpp:48-348) and extends it
// with the GAT slot->edge maps (ATT_Block*.blockProcess_sddmm_balance_gnn
// [_trans], Block/include/example.h:4-6).  Where the reference builds a
// std::set per window on the CPU and concatenates serially
// (example.cpp:61-175), this is an integer sort / merge / scan / compaction
// pipeline:
//
//   plan  k_unique_warp    one warp per window of <= kWarpCap edges (two
//                          launches by size class): bitonic sort of (column,
//                          edge index) keys in registers, de-duplicate,
//                          warp-scan compact; each edge's rank among its
//                          window's distinct columns falls out of the sort
//         k_chunk_rows     row holding the first edge of each 2048-edge chunk
//         k_merge_rank     larger windows, thread per edge: its position in
//                          the merge of the window's sorted rows (binary
//                          searches in the other rows) and whether it is its
//                          column's first occurrence
//         scan32           inclusive scan of those flags (all edges)
//         k_merge_emit     thread per edge: rank = flags up to its merged
//                          position; first occurrences emit the columns
//         k_unique_warp / k_unique_small / k_unique_large
//                          only windows with an unsorted row (the merge needs
//                          sorted rows): warp sort up to 1024 edges, CTA sort
//                          up to kSmallCap, else a column bitmap per CTA with
//                          a summary bitmap of its touched words
//         k_window_counts  padded width and part count per window
//         exclusive scans  column offsets and part offsets (int64, 3 kernels)
//   fill  k_col_chunk_windows  window holding each 2048-column chunk's start
//         k_fill_cols      CTA per 2048 condensed columns: sorted distinct
//                          columns with -1 padding (coalesced, whatever the
//                          window sizes)
//         k_fill_parts     thread per part: rowptr pair, window id, atomic flag
//         k_fill_edges     CTA per 2048-edge chunk: each edge's row from the
//                          chunk's slice of rowptr, its rank from the plan;
//                          writes value / slot->edge map / mirrored map /
//                          edge->slot
//
// All integer work; HBM- and L2-latency bound.
#include "att_common.cuh"

#include <mutex>

namespace att {
namespace {

constexpr int kSmallCap = 4096;     // windows up to this many edges sort in smem
constexpr int kSmallThreads = 512;  // kSmallCap / 8
constexpr int kLargeThreads = 1024;
constexpr int kEdgeChunk = 2048;    // CSR edges per CTA of the edge-chunk kernels
constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;
constexpr int kColChunkW = 2048;   // condensed columns per CTA of k_fill_cols
constexpr int kS32Threads = 256;
constexpr int kS32Items = 8;
constexpr int kS32Tile = kS32Threads * kS32Items;
constexpr int kMaxBitmapCtas = 304;
constexpr size_t kBitmapBudget = 256ull << 20;  // bytes of bitmap scratch at most

enum { FLAG_BAD_COL = 1, FLAG_BAD_ROWPTR = 2, FLAG_UNSORTED = 4, FLAG_OVERFLOW = 8 };

struct Workspace {
    int32_t *ucols;      // [nnz]      sorted distinct columns, at each window's edge offset
    int32_t *erank;      // [nnz]      rank of each edge's column among its window's distinct ones
    int32_t *ucount;     // [n_win]    distinct columns per window
    int64_t *col_off;    // [n_win+1]  exclusive scan of padded widths
    int64_t *part_off;   // [n_win+1]  exclusive scan of part counts
    int64_t *scan_tmp;   // [2*nblk]
    int32_t *flags;      // [4]
    int64_t *summary;    // [3]  n_condensed, n_parts, flags (the plan's result)
    uint32_t *bitmap;    // [n_bitmap_ctas * words]   column bits (zero between windows)
    uint32_t *bsum;      // [n_bitmap_ctas * swords]  touched-word bits (zero between windows)
    int32_t *wpre;       // [n_bitmap_ctas * words]   rank of a touched word's first column
    int32_t *chunk_row;  // [nnz / kEdgeChunk + 2]    row holding each edge chunk's first edge
    int32_t *mval;       // [nnz]  column at each merged position of windows above kWarpCap edges
    int32_t *mscan;      // [nnz]  first-occurrence flags at merged positions, then their scan
    int32_t *wflag;      // [n_win] 1 when a window above kWarpCap edges has an unsorted row
    int32_t *wlist;      // [n_win] the flagged windows, in no particular order
    int32_t *wlist_n;    // [1]     their count
    int32_t *chunk_win;  // [cond_chunks + 1]  window holding each column chunk's first column
    int32_t *scan32_tmp; // tile sums of the int32 scan, every level
    int n_bitmap_ctas;
    int64_t words, swords;
};

int64_t n_windows(int64_t n_rows, int window) { return n_rows / window; }

int bitmap_ctas(int64_t n_cols) {
    const int64_t words = (n_cols + 31) / 32, swords = (words + 31) / 32;
    const int64_t per_cta = (words > 0 ? words : 1) * 8 + swords * 4;
    int64_t by_budget = (int64_t)(kBitmapBudget / (size_t)per_cta);
    if (by_budget < 1) by_budget = 1;
    return (int)(by_budget < kMaxBitmapCtas ? by_budget : kMaxBitmapCtas);
}

// ints of tile sums an inclusive scan of n int32 needs, over all its levels
size_t scan32_tmp_ints(int64_t n) {
    size_t total = 0;
    for (int64_t m = n; m > kS32Tile;) {
        m = (m + kS32Tile - 1) / kS32Tile;
        total += (size_t)m + 1;
    }
    return total + 1;
}

size_t workspace_layout(int64_t n_rows, int64_t nnz, int64_t n_cols, int window, Workspace *ws,
                        char *base) {
    int64_t nw = n_windows(n_rows, window);
    int64_t nblk = (nw + 1 + kScanTile - 1) / kScanTile;
    int64_t words = (n_cols + 31) / 32;
    int64_t swords = (words + 31) / 32;
    int nb = bitmap_ctas(n_cols);
    size_t off = 0;
    auto take = [&](size_t bytes) {
        size_t o = off;
        off = align_up(off + bytes, 256);
        return o;
    };
    const size_t edges = (size_t)(nnz > 0 ? nnz : 1);
    size_t o_ucols = take(edges * 4);
    size_t o_erank = take(edges * 4);
    size_t o_ucount = take((size_t)(nw + 1) * 4);
    size_t o_col = take((size_t)(nw + 1) * 8);
    size_t o_part = take((size_t)(nw + 1) * 8);
    size_t o_scan = take((size_t)(2 * nblk + 2) * 8);
    size_t o_flags = take(16);
    size_t o_sum = take(24);
    size_t o_bitmap = take((size_t)nb * (size_t)(words > 0 ? words : 1) * 4);
    size_t o_bsum = take((size_t)nb * (size_t)(swords > 0 ? swords : 1) * 4);
    size_t o_wpre = take((size_t)nb * (size_t)(words > 0 ? words : 1) * 4);
    size_t o_crow = take((size_t)(nnz / kEdgeChunk + 2) * 4);
    size_t o_mval = take(edges * 4);
    size_t o_mscan = take(edges * 4);
    size_t o_wflag = take((size_t)(nw + 1) * 4);
    size_t o_wlist = take((size_t)(nw + 1) * 4);
    size_t o_wlist_n = take(16);
    // condensed columns are at most nnz plus under `wide` (<= 64) padding per window
    size_t o_cwin = take((size_t)((nnz + 64 * nw) / kColChunkW + 2) * 4);
    size_t o_s32 = take(scan32_tmp_ints(nnz) * 4);
    if (ws && base) {
        ws->ucols = (int32_t *)(base + o_ucols);
        ws->erank = (int32_t *)(base + o_erank);
        ws->ucount = (int32_t *)(base + o_ucount);
        ws->col_off = (int64_t *)(base + o_col);
        ws->part_off = (int64_t *)(base + o_part);
        ws->scan_tmp = (int64_t *)(base + o_scan);
        ws->flags = (int32_t *)(base + o_flags);
        ws->summary = (int64_t *)(base + o_sum);
        ws->bitmap = (uint32_t *)(base + o_bitmap);
        ws->bsum = (uint32_t *)(base + o_bsum);
        ws->wpre = (int32_t *)(base + o_wpre);
        ws->chunk_row = (int32_t *)(base + o_crow);
        ws->mval = (int32_t *)(base + o_mval);
        ws->mscan = (int32_t *)(base + o_mscan);
        ws->wflag = (int32_t *)(base + o_wflag);
        ws->wlist = (int32_t *)(base + o_wlist);
        ws->wlist_n = (int32_t *)(base + o_wlist_n);
        ws->chunk_win = (int32_t *)(base + o_cwin);
        ws->scan32_tmp = (int32_t *)(base + o_s32);
        ws->n_bitmap_ctas = nb;
        ws->words = words;
        ws->swords = swords;
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

// ---- plan: distinct sorted columns per window, and each edge's rank --------
// Keys are (column << IB) | index-of-the-edge-in-its-window, unsigned, so a
// sort orders the window's edges by column and keeps who is who; the
// sentinel (all ones) sorts last.  32-bit keys when the columns fit in
// 32 - IB bits, else 64-bit.
template <typename KT>
__device__ __forceinline__ KT key_sentinel() { return ~(KT)0; }

// Bitonic sort (ascending) of n keys (n a power of two) in shared memory by
// the calling warp alone.
template <typename KT>
__device__ __forceinline__ void warp_bitonic(KT *keys, int n, int lane) {
    for (int k = 2; k <= n; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int t = lane; t < (n >> 1); t += 32) {
                const int i = 2 * t - (t & (j - 1)), l = i + j;  // pair (i, i + j)
                const KT x = keys[i], y = keys[l];
                if ((x > y) == ((i & k) == 0)) {
                    keys[i] = y;
                    keys[l] = x;
                }
            }
            __syncwarp();
        }
    }
}

// Bitonic sort (ascending) of 32 * PER keys held by a warp in registers: key
// i = lane * PER + q sits in v[q].  Compare distances below PER swap
// registers of one lane; larger ones exchange with lane ^ (distance / PER).
template <typename KT, int PER>
__device__ __forceinline__ void warp_bitonic_regs(KT (&v)[PER], int lane) {
#pragma unroll
    for (int k = 2; k <= 32 * PER; k <<= 1) {
#pragma unroll
        for (int j = k >> 1; j > 0; j >>= 1) {
            if (j < PER) {
#pragma unroll
                for (int q = 0; q < PER; ++q) {
                    if ((q & j) == 0) {
                        const bool asc = ((lane * PER + q) & k) == 0;
                        const KT x = v[q], y = v[q + j];
                        const bool sw = asc ? (x > y) : (x < y);
                        v[q] = sw ? y : x;
                        v[q + j] = sw ? x : y;
                    }
                }
            } else {
                const int lj = j / PER;
                const bool lower = (lane & lj) == 0;
#pragma unroll
                for (int q = 0; q < PER; ++q) {
                    const bool asc = ((lane * PER + q) & k) == 0;
                    const KT o = __shfl_xor_sync(0xffffffffu, v[q], lj);
                    const KT mn = v[q] < o ? v[q] : o, mx = v[q] < o ? o : v[q];
                    v[q] = lower == asc ? mn : mx;
                }
            }
        }
    }
}

// One window of 1 .. 32 * PER edges by the calling warp, in registers: sort
// the (column, edge) keys, then each lane de-duplicates its PER consecutive
// sorted keys (the key before its first comes from the lane below), a warp
// scan places the distinct columns, and every edge gets its column's rank.
template <typename KT, int PER, int IB>
__device__ __forceinline__ void unique_window_regs(const int32_t *__restrict__ col, int64_t b0,
                                                   int E, int64_t n_cols, const Workspace &ws,
                                                   int64_t w, int lane) {
    KT v[PER];
#pragma unroll
    for (int q = 0; q < PER; ++q) {
        const int t = lane * PER + q;
        v[q] = key_sentinel<KT>();
        if (t < E) {
            const int c = col[b0 + t];
            if (c < 0 || c >= n_cols) atomicOr(ws.flags, FLAG_BAD_COL);
            else v[q] = ((KT)c << IB) | (KT)t;
        }
    }
    warp_bitonic_regs<KT, PER>(v, lane);
    const KT below = __shfl_up_sync(0xffffffffu, v[PER - 1], 1);
    bool fl[PER];
    int cnt = 0;
#pragma unroll
    for (int q = 0; q < PER; ++q) {
        const KT prv = q == 0 ? below : v[q - 1];
        fl[q] = v[q] != key_sentinel<KT>() &&
                ((lane == 0 && q == 0) || (prv >> IB) != (v[q] >> IB));
        cnt += fl[q] ? 1 : 0;
    }
    int x = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    const int total = __shfl_sync(0xffffffffu, x, 31);
    int pos = x - cnt;  // distinct columns before this lane's keys
#pragma unroll
    for (int q = 0; q < PER; ++q) {
        if (v[q] != key_sentinel<KT>()) {
            if (fl[q]) ws.ucols[b0 + pos++] = (int32_t)(v[q] >> IB);
            ws.erank[b0 + (int64_t)(v[q] & (KT)((1u << IB) - 1))] = pos - 1;
        }
    }
    if (lane == 0) ws.ucount[w] = total;
}

// Windows of LO+1 .. CAP edges: one warp each.  Up to kWarpCap edges the keys
// sort in registers (unique_window_regs); larger windows sort in the warp's
// own slice of shared memory (warp-synchronous, no block barriers).  Then the
// window is de-duplicated and compacted with a warp scan; the rank of every
// edge's column is written to erank.  With `unsorted_only`, only windows the
// merge path flagged.
constexpr int kWarpSortWarps = 8;
constexpr int kWarpCap = 256;  // windows up to this many edges: warp sort; above: merge
constexpr int kMidCap = 1024;

template <typename KT, int CAP, int LO>
__global__ void __launch_bounds__(kWarpSortWarps * 32) k_unique_warp(
    const int32_t *__restrict__ rowptr, const int32_t *__restrict__ col, int64_t n_win,
    int window, int64_t nnz, int64_t n_cols, int unsorted_only, Workspace ws) {
    constexpr int IB = CAP <= 256 ? 8 : (CAP <= 1024 ? 10 : 12);
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    KT *keys = reinterpret_cast<KT *>(smem_raw) + wib * CAP;
    const int64_t nwarps = (int64_t)gridDim.x * kWarpSortWarps;
    // all windows, or (unsorted_only) the list of windows the merge path flagged
    const int64_t n_it = unsorted_only ? *ws.wlist_n : n_win;
    for (int64_t it = (int64_t)blockIdx.x * kWarpSortWarps + wib; it < n_it; it += nwarps) {
        const int64_t w = unsorted_only ? ws.wlist[it] : it;
        int64_t b0, b1;
        window_range(rowptr, w, window, nnz, &b0, &b1, ws.flags);
        const int64_t E = b1 - b0;
        if (E > CAP || E <= LO) continue;  // another kernel's window
        if constexpr (CAP <= kWarpCap) {
            // only the networks of this launch's size class are compiled in
            // (one unrolled network per kernel keeps instruction fetch short)
            if constexpr (LO < 32) {
                if (E <= 32) {
                    unique_window_regs<KT, 1, IB>(col, b0, (int)E, n_cols, ws, w, lane);
                    continue;
                }
            }
            if constexpr (LO < 64 && CAP > 32) {
                if (E <= 64) {
                    unique_window_regs<KT, 2, IB>(col, b0, (int)E, n_cols, ws, w, lane);
                    continue;
                }
            }
            if constexpr (LO < 128 && CAP > 64) {
                if (E <= 128) {
                    unique_window_regs<KT, 4, IB>(col, b0, (int)E, n_cols, ws, w, lane);
                    continue;
                }
            }
            if constexpr (CAP > 128) unique_window_regs<KT, 8, IB>(col, b0, (int)E, n_cols, ws, w, lane);
            continue;
        }
        int n = 32;
        while (n < E) n <<= 1;
        for (int t = lane; t < n; t += 32) {
            KT k = key_sentinel<KT>();
            if (t < E) {
                const int c = col[b0 + t];
                if (c < 0 || c >= n_cols) atomicOr(ws.flags, FLAG_BAD_COL);
                else k = ((KT)c << IB) | (KT)t;
            }
            keys[t] = k;
        }
        __syncwarp();
        warp_bitonic(keys, n, lane);
        // de-duplicate: lane owns n / 32 consecutive sorted keys
        const int per = n >> 5, base = lane * per;
        int cnt = 0;
        for (int q = 0; q < per; ++q) {
            const int kk = base + q;
            const KT v = keys[kk];
            if (kk < E && v != key_sentinel<KT>() &&
                (kk == 0 || (keys[kk - 1] >> IB) != (v >> IB)))
                cnt++;
        }
        int x = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        const int total = __shfl_sync(0xffffffffu, x, 31);
        int pos = x - cnt;  // distinct columns before this lane's keys
        for (int q = 0; q < per; ++q) {
            const int kk = base + q;
            const KT v = keys[kk];
            if (kk < E && v != key_sentinel<KT>()) {
                const bool first = kk == 0 || (keys[kk - 1] >> IB) != (v >> IB);
                if (first) ws.ucols[b0 + pos++] = (int32_t)(v >> IB);
                ws.erank[b0 + (int64_t)(v & (KT)((1u << IB) - 1))] = pos - 1;
            }
        }
        if (lane == 0) ws.ucount[w] = total;
        __syncwarp();
    }
}

// Windows of kMidCap+1 .. kSmallCap edges: one CTA each, bitonic sort in
// shared memory across the block (64-bit keys).
__global__ void __launch_bounds__(kSmallThreads) k_unique_small(
    const int32_t *__restrict__ rowptr, const int32_t *__restrict__ col, int64_t n_win,
    int window, int64_t nnz, int64_t n_cols, int unsorted_only, Workspace ws) {
    constexpr int IB = 12;
    __shared__ unsigned long long keys[kSmallCap];
    __shared__ int sh[kSmallThreads / 32 + 1];
    const int64_t n_it = unsorted_only ? *ws.wlist_n : n_win;
    for (int64_t it = blockIdx.x; it < n_it; it += gridDim.x) {
        const int64_t w = unsorted_only ? ws.wlist[it] : it;
        int64_t b0, b1;
        window_range(rowptr, w, window, nnz, &b0, &b1, ws.flags);
        int64_t E = b1 - b0;
        if (E > kSmallCap || E <= kMidCap) continue;  // another kernel's window
        int n = 1;
        while (n < E) n <<= 1;
        for (int t = threadIdx.x; t < n; t += kSmallThreads) {
            unsigned long long k = ~0ull;
            if (t < E) {
                const int c = col[b0 + t];
                if (c < 0 || c >= n_cols) atomicOr(ws.flags, FLAG_BAD_COL);
                else k = ((unsigned long long)c << IB) | (unsigned long long)t;
            }
            keys[t] = k;
        }
        __syncthreads();
        for (int k = 2; k <= n; k <<= 1) {
            for (int j = k >> 1; j > 0; j >>= 1) {
                for (int t = threadIdx.x; t < (n >> 1); t += kSmallThreads) {
                    const int i = 2 * t - (t & (j - 1)), l = i + j;
                    const unsigned long long x = keys[i], y = keys[l];
                    if ((x > y) == ((i & k) == 0)) {
                        keys[i] = y;
                        keys[l] = x;
                    }
                }
                __syncthreads();
            }
        }
        // de-duplicate: each thread owns 8 consecutive sorted keys
        const int base = threadIdx.x * 8;
        int cnt = 0;
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const int kk = base + q;
            if (kk < E) {
                const unsigned long long v = keys[kk];
                if (v != ~0ull && (kk == 0 || (keys[kk - 1] >> IB) != (v >> IB))) cnt++;
            }
        }
        int total;
        int pos = block_exclusive_scan<kSmallThreads>(cnt, &total, sh);
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const int kk = base + q;
            if (kk < E) {
                const unsigned long long v = keys[kk];
                if (v != ~0ull) {
                    if (kk == 0 || (keys[kk - 1] >> IB) != (v >> IB))
                        ws.ucols[b0 + pos++] = (int32_t)(v >> IB);
                    ws.erank[b0 + (int64_t)(v & ((1ull << IB) - 1))] = pos - 1;
                }
            }
        }
        if (threadIdx.x == 0) ws.ucount[w] = total;
        __syncthreads();
    }
}

// Windows above kSmallCap edges: one CTA per window at a time, with its own
// column bitmap `bm` (n_cols bits) and summary bitmap `bs` (one bit per
// bitmap word) in global scratch, both all-zero between windows.  Each edge
// sets its column's bit and its word's summary bit; the CTA then walks only
// the summary's set bits (n_cols / 1024 words) to count, emit the sorted
// columns and record each touched word's first rank; each edge's rank is
// that plus a popcount; finally each edge clears its word and summary word.
__global__ void __launch_bounds__(kLargeThreads) k_unique_large(
    const int32_t *__restrict__ rowptr, const int32_t *__restrict__ col, int64_t n_win,
    int window, int64_t nnz, int64_t n_cols, int unsorted_only, Workspace ws) {
    __shared__ int sh[kLargeThreads / 32 + 1];
    uint32_t *bm = ws.bitmap + (int64_t)blockIdx.x * ws.words;
    uint32_t *bs = ws.bsum + (int64_t)blockIdx.x * ws.swords;
    int32_t *wp = ws.wpre + (int64_t)blockIdx.x * ws.words;
    const int64_t swords = ws.swords;
    const int64_t chunk = (swords + kLargeThreads - 1) / kLargeThreads;
    const int64_t n_it = unsorted_only ? *ws.wlist_n : n_win;
    for (int64_t it = blockIdx.x; it < n_it; it += gridDim.x) {
        const int64_t w = unsorted_only ? ws.wlist[it] : it;
        const int64_t b0 = rowptr[w * window], b1 = rowptr[(w + 1) * window];
        if (b0 < 0 || b1 < b0 || b1 > nnz) continue;  // flagged by the other plan kernels
        if (b1 - b0 <= kSmallCap) continue;           // another kernel's window
        for (int64_t e = b0 + threadIdx.x; e < b1; e += kLargeThreads) {
            const int c = col[e];
            if (c < 0 || c >= n_cols) {
                atomicOr(ws.flags, FLAG_BAD_COL);
                continue;
            }
            atomicOr(&bm[c >> 5], 1u << (c & 31));
            atomicOr(&bs[c >> 10], 1u << ((c >> 5) & 31));
        }
        __syncthreads();
        // count the distinct columns under this thread's summary words
        const int64_t s0 = (int64_t)threadIdx.x * chunk;
        const int64_t s1 = s0 + chunk < swords ? s0 + chunk : swords;
        int cnt = 0;
        for (int64_t q2 = s0; q2 < s1; ++q2) {
            uint32_t sb = bs[q2];
            while (sb) {
                const int b = __ffs(sb) - 1;
                sb &= sb - 1;
                cnt += __popc(bm[q2 * 32 + b]);
            }
        }
        int total;
        int pos = block_exclusive_scan<kLargeThreads>(cnt, &total, sh);
        for (int64_t q2 = s0; q2 < s1; ++q2) {
            uint32_t sb = bs[q2];
            while (sb) {
                const int b = __ffs(sb) - 1;
                sb &= sb - 1;
                const int64_t q = q2 * 32 + b;
                uint32_t bits = bm[q];
                wp[q] = pos;
                while (bits) {
                    const int bb = __ffs(bits) - 1;
                    bits &= bits - 1;
                    ws.ucols[b0 + pos++] = (int32_t)(q * 32 + bb);
                }
            }
        }
        if (threadIdx.x == 0) ws.ucount[w] = total;
        __syncthreads();
        for (int64_t e = b0 + threadIdx.x; e < b1; e += kLargeThreads) {
            const int c = col[e];
            if (c < 0 || c >= n_cols) continue;
            const uint32_t bits = bm[c >> 5];
            ws.erank[e] = wp[c >> 5] + __popc(bits & ((1u << (c & 31)) - 1u));
        }
        __syncthreads();
        for (int64_t e = b0 + threadIdx.x; e < b1; e += kLargeThreads) {
            const int c = col[e];
            if (c < 0 || c >= n_cols) continue;
            bm[c >> 5] = 0u;
            bs[c >> 10] = 0u;
        }
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

// ---- shared by the fill and merge kernels ------------------------------------
// Largest index i in [lo, hi] with a[i] <= x (a non-decreasing, a[lo] <= x).
template <typename T>
__device__ __forceinline__ int64_t last_le(const T *a, int64_t lo, int64_t hi, int64_t x) {
    while (lo < hi) {
        const int64_t mid = (lo + hi + 1) >> 1;
        if ((int64_t)a[mid] <= x) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// Row of each 2048-edge chunk's first edge: thread per row, writing the chunks
// whose first edge the row holds (no search).
__global__ void k_chunk_rows(const int32_t *__restrict__ rowptr, int64_t n_rows_used,
                             int64_t n_chunks, Workspace ws) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n_rows_used) return;
    const int64_t e0 = rowptr[0];
    const int64_t s = rowptr[r] - e0, e = rowptr[r + 1] - e0;
    if (s < 0 || e <= s) return;
    const int64_t c_hi = (e + kEdgeChunk - 1) / kEdgeChunk;
    for (int64_t c = (s + kEdgeChunk - 1) / kEdgeChunk; c < c_hi && c < n_chunks; ++c)
        ws.chunk_row[c] = (int32_t)r;
}

// The edge-chunk kernels run a CTA of kEdgeThreads threads per kEdgeChunk CSR
// edges of the used rows.  A chunk's rows run from the row of its first edge
// to the row of the next chunk's first edge.  When that slice of rowptr fits
// in shared memory, the CTA builds the row of every edge of the chunk there
// (EdgeRows): each row marks its first edge inside the chunk, and a max-scan
// carries the mark over the row's edges.  Otherwise each edge searches
// rowptr.
constexpr int kEdgeThreads = 256;
constexpr int kEdgeStage = 2048;
constexpr int kEdgePer = kEdgeChunk / kEdgeThreads;  // scan entries per thread
static_assert(kEdgePer == 8, "EdgeRows scans two int4 per thread");

struct EdgeChunk {
    int64_t eb, ee, r0, r1, nr;
    bool staged;
};

struct EdgeRows {
    int32_t rp[kEdgeStage];                    // rowptr[r0 .. r0 + nr - 1]
    __align__(16) int32_t row[kEdgeChunk];     // row of edge eb + j, minus r0
    int warp_max[kEdgeThreads / 32];
};

// Row of every edge of a staged chunk.  A row's first edge inside the chunk
// (edge eb for rows starting at or before it) gets the row's index; the
// largest index wins, so an empty row loses to the non-empty row sharing its
// start.  An inclusive max-scan then gives every edge the last row that
// starts at or before it, which is the row holding it.
__device__ __forceinline__ void edge_rows_build(EdgeRows &sh, const EdgeChunk &c) {
    const int len = (int)(c.ee - c.eb);
    const int t = threadIdx.x, lane = t & 31, wid = t >> 5;
    int4 *row4 = reinterpret_cast<int4 *>(sh.row);
    for (int j = t; j < kEdgeChunk / 4; j += kEdgeThreads)
        row4[j] = make_int4(j == 0 ? 0 : -1, -1, -1, -1);
    __syncthreads();
    for (int i = t; i < (int)c.nr; i += kEdgeThreads) {
        const int64_t st = (int64_t)sh.rp[i] - c.eb;
        if (st < len) atomicMax(&sh.row[st > 0 ? st : 0], i);
    }
    __syncthreads();
    int4 lo = row4[2 * t], hi = row4[2 * t + 1];
    lo.y = max(lo.y, lo.x);
    lo.z = max(lo.z, lo.y);
    lo.w = max(lo.w, lo.z);
    hi.x = max(hi.x, lo.w);
    hi.y = max(hi.y, hi.x);
    hi.z = max(hi.z, hi.y);
    hi.w = max(hi.w, hi.z);
    int run = hi.w;  // inclusive max-scan of the thread totals
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, run, o);
        if (lane >= o) run = max(run, y);
    }
    if (lane == 31) sh.warp_max[wid] = run;
    __syncthreads();
    int pre = __shfl_up_sync(0xffffffffu, run, 1);
    if (lane == 0) pre = -1;
    for (int k = 0; k < wid; ++k) pre = max(pre, sh.warp_max[k]);
    lo = make_int4(max(lo.x, pre), max(lo.y, pre), max(lo.z, pre), max(lo.w, pre));
    hi = make_int4(max(hi.x, pre), max(hi.y, pre), max(hi.z, pre), max(hi.w, pre));
    row4[2 * t] = lo;
    row4[2 * t + 1] = hi;
    __syncthreads();
}

// Returns false (for the whole CTA) when the CTA has no edges.
__device__ __forceinline__ bool edge_chunk(const int32_t *__restrict__ rowptr, int64_t n_rows_used,
                                           int64_t nnz, const Workspace &ws, EdgeRows &sh,
                                           EdgeChunk &c) {
    const int64_t e0 = rowptr[0], e_end = rowptr[n_rows_used];
    if (e0 < 0 || e_end > nnz || e_end < e0) return false;  // flagged during plan
    const int64_t n_chunks = (e_end - e0 + kEdgeChunk - 1) / kEdgeChunk;
    const int64_t cidx = blockIdx.x;
    if (cidx >= n_chunks) return false;
    c.eb = e0 + cidx * kEdgeChunk;
    c.ee = c.eb + kEdgeChunk < e_end ? c.eb + kEdgeChunk : e_end;
    c.r0 = ws.chunk_row[cidx];
    c.r1 = cidx + 1 < n_chunks ? ws.chunk_row[cidx + 1] : n_rows_used - 1;
    if (c.r0 < 0 || c.r1 < c.r0 || c.r1 >= n_rows_used) {  // not from a plan of this CSR
        c.r0 = 0;
        c.r1 = n_rows_used - 1;
    }
    c.nr = c.r1 - c.r0 + 1;
    c.staged = c.nr <= kEdgeStage;
    if (c.staged) {
        for (int64_t i = threadIdx.x; i < c.nr; i += kEdgeThreads) sh.rp[i] = rowptr[c.r0 + i];
        edge_rows_build(sh, c);  // its first barrier orders these stores
    }
    return true;
}

__device__ __forceinline__ int64_t chunk_row_of(const int32_t *__restrict__ rowptr,
                                                const EdgeRows &sh, const EdgeChunk &c,
                                                int64_t e) {
    return c.staged ? c.r0 + sh.row[e - c.eb] : last_le(rowptr, c.r0, c.r1, e);
}

// ---- plan, windows above kWarpCap edges: merge ranks ---------------------------
// CSR rows are sorted, so a window's distinct sorted columns are the
// de-duplicated merge of its rows.  An edge's position in that merge (ties
// ordered by row) is its position in its own row plus, for every other row of
// the window, the number of that row's columns before it -- found by binary
// search, so every edge is placed independently, whatever the window sizes.
// The edge is the first occurrence of its column when its row holds no equal
// column before it and no earlier row holds the column.  Its column and that
// flag go to the merged position; one scan of the flags then gives every
// merged position its rank among distinct columns (k_merge_emit).  A window
// with an unsorted row is flagged and redone by the sorting kernels.
// Elements of the sorted a[0, n) below x (LE: at or below x), n < 2^31.
// Branch-free halving: the answer stays in [base, base + n] and every probe
// a[base + half] is inside the array.
template <bool LE>
__device__ __forceinline__ int count_below(const int32_t *__restrict__ a, int n, int32_t x) {
    if (n <= 0) return 0;
    int base = 0;
    while (n > 1) {
        const int half = n >> 1;
        const int32_t v = a[base + half];
        base = (LE ? v <= x : v < x) ? base + half : base;
        n -= half;
    }
    const int32_t v = a[base];
    return base + ((LE ? v <= x : v < x) ? 1 : 0);
}

// Mark window w as holding an unsorted row and list it once.
__device__ __forceinline__ void flag_unsorted(const Workspace &ws, int64_t w) {
    if (atomicOr(&ws.wflag[w], 1) == 0) ws.wlist[atomicAdd(ws.wlist_n, 1)] = (int32_t)w;
}

__global__ void __launch_bounds__(kEdgeThreads) k_merge_rank(
    const int32_t *__restrict__ rowptr, const int32_t *__restrict__ col, int64_t n_rows_used,
    int window, int64_t nnz, int64_t n_cols, Workspace ws) {
    __shared__ EdgeRows sh;
    EdgeChunk c;
    if (!edge_chunk(rowptr, n_rows_used, nnz, ws, sh, c)) return;
    for (int64_t e = c.eb + threadIdx.x; e < c.ee; e += kEdgeThreads) {
        const int64_t row = chunk_row_of(rowptr, sh, c, e);
        const int64_t w = row / window, wb = w * window;
        const int i = (int)(row - wb);
        const int64_t b0 = rowptr[wb], b1 = rowptr[wb + window];
        if (b1 - b0 <= kWarpCap) continue;  // k_unique_warp's window (flags stay 0)
        const int32_t x = col[e];
        if (x < 0 || x >= n_cols) atomicOr(ws.flags, FLAG_BAD_COL);
        // positions are below 2^31 (int32 rowptr)
        const int p = (int)(e - rowptr[row]);
        bool first = true;
        if (p > 0) {
            const int32_t prev = col[e - 1];
            if (prev > x) flag_unsorted(ws, w);
            first = prev != x;
        }
        int64_t m = p;
        for (int k = 0; k < window; ++k) {
            if (k == i) continue;
            const int32_t rs = rowptr[wb + k];
            const int len = rowptr[wb + k + 1] - rs;
            if (len <= 0) continue;
            const int32_t *rk = col + rs;
            if (k < i) {
                const int ub = count_below<true>(rk, len, x);
                m += ub;
                if (ub > 0 && rk[ub - 1] == x) first = false;
            } else {
                m += count_below<false>(rk, len, x);
            }
        }
        if (m < 0 || m >= b1 - b0) {  // only when a row is unsorted
            flag_unsorted(ws, w);
            continue;
        }
        ws.mval[b0 + m] = x;
        ws.mscan[b0 + m] = first ? 1 : 0;
        ws.erank[e] = (int32_t)m;
    }
}

// After the scan: rank = distinct columns up to the edge's merged position,
// within its window; first occurrences emit the window's sorted columns.
__global__ void __launch_bounds__(kEdgeThreads) k_merge_emit(
    const int32_t *__restrict__ rowptr, int64_t n_rows_used, int window, int64_t nnz,
    Workspace ws) {
    __shared__ EdgeRows sh;
    EdgeChunk c;
    if (!edge_chunk(rowptr, n_rows_used, nnz, ws, sh, c)) return;
    for (int64_t e = c.eb + threadIdx.x; e < c.ee; e += kEdgeThreads) {
        const int64_t row = chunk_row_of(rowptr, sh, c, e);
        const int64_t w = row / window, wb = w * window;
        const int64_t b0 = rowptr[wb], b1 = rowptr[wb + window];
        if (b1 - b0 <= kWarpCap || ws.wflag[w]) continue;
        // differences of the scan within the window (unsigned: exact modulo
        // 2^32 whatever the prefix before it)
        const uint32_t base = b0 > 0 ? (uint32_t)ws.mscan[b0 - 1] : 0u;
        const int64_t q = b0 + ws.erank[e];
        const uint32_t incl = (uint32_t)ws.mscan[q];
        const uint32_t prev = q > 0 ? (uint32_t)ws.mscan[q - 1] : 0u;
        const int64_t rank = (int64_t)(incl - base) - 1;
        ws.erank[e] = (int32_t)rank;
        if (incl - prev == 1u) ws.ucols[b0 + rank] = ws.mval[q];
        if (e == b0) ws.ucount[w] = (int32_t)((uint32_t)ws.mscan[b1 - 1] - base);
    }
}

// ---- int32 scan (in place), tiles of kS32Tile, tile sums scanned recursively --
__global__ void __launch_bounds__(kS32Threads) k_scan32_reduce(const int32_t *__restrict__ a,
                                                               int64_t n, int32_t *sums) {
    __shared__ int sh[kS32Threads / 32 + 1];
    const int64_t base = (int64_t)blockIdx.x * kS32Tile + threadIdx.x * kS32Items;
    int s = 0;
    if (base + kS32Items <= n && ((uintptr_t)(a + base) & 15) == 0) {
        const int4 lo = *reinterpret_cast<const int4 *>(a + base);
        const int4 hi = *reinterpret_cast<const int4 *>(a + base + 4);
        s = lo.x + lo.y + lo.z + lo.w + hi.x + hi.y + hi.z + hi.w;
    } else {
#pragma unroll
        for (int q = 0; q < kS32Items; ++q)
            if (base + q < n) s += a[base + q];
    }
    int total;
    block_exclusive_scan<kS32Threads>(s, &total, sh);
    if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

// inclusive (or exclusive) scan of each tile plus its offset (the exclusive
// prefix of the tile sums; none for a single tile)
__global__ void __launch_bounds__(kS32Threads) k_scan32_apply(int32_t *a, int64_t n,
                                                              const int32_t *offs,
                                                              int inclusive) {
    __shared__ int sh[kS32Threads / 32 + 1];
    const int64_t base = (int64_t)blockIdx.x * kS32Tile + threadIdx.x * kS32Items;
    int v[kS32Items];
    // a thread's 8 items as two 16-byte loads when they are whole and aligned
    const bool vec = base + kS32Items <= n && ((uintptr_t)(a + base) & 15) == 0;
    if (vec) {
        const int4 lo = *reinterpret_cast<const int4 *>(a + base);
        const int4 hi = *reinterpret_cast<const int4 *>(a + base + 4);
        v[0] = lo.x; v[1] = lo.y; v[2] = lo.z; v[3] = lo.w;
        v[4] = hi.x; v[5] = hi.y; v[6] = hi.z; v[7] = hi.w;
    } else {
#pragma unroll
        for (int q = 0; q < kS32Items; ++q) v[q] = base + q < n ? a[base + q] : 0;
    }
    int s = 0;
#pragma unroll
    for (int q = 0; q < kS32Items; ++q) s += v[q];
    int total;
    int run = block_exclusive_scan<kS32Threads>(s, &total, sh) + (offs ? offs[blockIdx.x] : 0);
#pragma unroll
    for (int q = 0; q < kS32Items; ++q) {
        const int x = v[q];
        if (inclusive) run += x;
        v[q] = run;
        if (!inclusive) run += x;
    }
    if (vec) {
        *reinterpret_cast<int4 *>(a + base) = make_int4(v[0], v[1], v[2], v[3]);
        *reinterpret_cast<int4 *>(a + base + 4) = make_int4(v[4], v[5], v[6], v[7]);
    } else {
#pragma unroll
        for (int q = 0; q < kS32Items; ++q)
            if (base + q < n) a[base + q] = v[q];
    }
}

int scan32(int32_t *a, int64_t n, int32_t *tmp, int inclusive, cudaStream_t st) {
    if (n <= 0) return ATT_OK;
    const int64_t nblk = (n + kS32Tile - 1) / kS32Tile;
    if (nblk == 1) {
        k_scan32_apply<<<1, kS32Threads, 0, st>>>(a, n, nullptr, inclusive);
        return launch_status("k_scan32_apply");
    }
    k_scan32_reduce<<<(unsigned)nblk, kS32Threads, 0, st>>>(a, n, tmp);
    int s = launch_status("k_scan32_reduce");
    if (s != ATT_OK) return s;
    s = scan32(tmp, nblk, tmp + nblk + 1, 0, st);  // exclusive tile offsets
    if (s != ATT_OK) return s;
    k_scan32_apply<<<(unsigned)nblk, kS32Threads, 0, st>>>(a, n, tmp, inclusive);
    return launch_status("k_scan32_apply");
}

// ---- fill: structure ---------------------------------------------------------
// Window holding the first condensed column of each column chunk: thread per
// window, writing the chunks whose first column the window holds.
__global__ void k_col_chunk_windows(int64_t n_win, int64_t n_chunks, Workspace ws) {
    const int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= n_win) return;
    const int64_t s = ws.col_off[w], e = ws.col_off[w + 1];
    if (e <= s) return;
    const int64_t c_hi = (e + kColChunkW - 1) / kColChunkW;
    for (int64_t c = (s + kColChunkW - 1) / kColChunkW; c < c_hi && c < n_chunks; ++c)
        ws.chunk_win[c] = (int32_t)w;
}

// Condensed columns: CTA per kColChunkW output positions.  The chunk's windows
// run from the window of its first column to the window of the next chunk's
// first column; their offsets and first edges are staged in shared memory
// when they fit (else searched in global memory), so every position is
// written by its own thread, coalesced, however long the windows are.
constexpr int kColThreads = 256;
constexpr int kColStage = 512;

__global__ void __launch_bounds__(kColThreads) k_fill_cols(int64_t n_win, int64_t total, int window,
                                                           Workspace ws,
                                                           const int32_t *__restrict__ rowptr,
                                                           int32_t *__restrict__ out_col) {
    __shared__ int64_t s_off[kColStage + 1];
    __shared__ int64_t s_b0[kColStage];
    const int64_t n_chunks = (total + kColChunkW - 1) / kColChunkW;
    const int64_t cidx = blockIdx.x;
    const int64_t start = cidx * kColChunkW;
    if (start >= total) return;
    const int64_t end = start + kColChunkW < total ? start + kColChunkW : total;
    int64_t w0 = ws.chunk_win[cidx];
    int64_t w1 = cidx + 1 < n_chunks ? ws.chunk_win[cidx + 1] : n_win - 1;
    if (w0 < 0 || w1 < w0 || w1 >= n_win) {  // not from a plan of this CSR
        w0 = 0;
        w1 = n_win - 1;
    }
    const int64_t nw = w1 - w0 + 1;
    const bool staged = nw <= kColStage;
    if (staged) {
        for (int64_t i = threadIdx.x; i <= nw; i += kColThreads) {
            s_off[i] = ws.col_off[w0 + i];
            if (i < nw) s_b0[i] = rowptr[(w0 + i) * window];
        }
    }
    __syncthreads();
    for (int64_t k = start + threadIdx.x; k < end; k += kColThreads) {
        int64_t w, cb, b0;
        if (staged) {
            const int64_t i = last_le(s_off, 0, nw - 1, k);
            w = w0 + i;
            cb = s_off[i];
            b0 = s_b0[i];
        } else {
            w = last_le(ws.col_off, w0, w1, k);
            cb = ws.col_off[w];
            b0 = rowptr[w * window];
        }
        const int64_t j = k - cb;
        out_col[k] = j < ws.ucount[w] ? ws.ucols[b0 + j] : -1;
    }
}

// Parts: thread per part; its window from the part offsets.
__global__ void k_fill_parts(int64_t n_win, int64_t n_parts, int wide, int part, Workspace ws,
                             int32_t *__restrict__ out_rowptr, int32_t *__restrict__ out_window,
                             int32_t *__restrict__ out_atomic) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p == 0) out_rowptr[0] = 0;
    if (p >= n_parts) return;
    const int64_t w = last_le(ws.part_off, 0, n_win - 1, p);
    const int64_t pl = p - ws.part_off[w];
    const int64_t np = ws.part_off[w + 1] - ws.part_off[w];
    const int64_t cbase = ws.col_off[w];
    const int64_t pad = ws.col_off[w + 1] - cbase;
    const int64_t blocks = pad / wide;
    int64_t r_end, p_end;
    if (blocks == 0) {
        r_end = p_end = cbase;  // the (0, 0) part of an empty window (emit_empty)
    } else {
        const int64_t nb = blocks - pl * part < part ? blocks - pl * part : part;
        p_end = cbase + pl * part * wide + nb * wide;
        r_end = p_end - (pl == np - 1 ? pad - (int64_t)ws.ucount[w] : 0);
    }
    out_rowptr[2 * p + 1] = (int32_t)r_end;
    out_rowptr[2 * p + 2] = (int32_t)p_end;
    out_window[p] = (int32_t)w;
    out_atomic[p] = np > 1 ? 1 : 0;
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
__device__ __forceinline__ void fill_edge(
    int64_t e, int64_t row, const int32_t *__restrict__ rowptr, const int32_t *__restrict__ col,
    int window, int wide, int64_t n_cols, int64_t n_rows, const Workspace &ws,
    const void *__restrict__ deg, int deg_dtype, VT *__restrict__ out_val,
    int32_t *__restrict__ out_map, int32_t *__restrict__ out_map_t,
    int32_t *__restrict__ out_edge_slot, int64_t n_slots) {
    const int32_t c = col[e];
    if (c < 0 || c >= n_cols) {
        if (out_edge_slot) out_edge_slot[e] = -1;
        return;  // flagged during plan
    }
    if (e > rowptr[row] && col[e - 1] > c) atomicOr(ws.flags, FLAG_UNSORTED);
    const int64_t w = row / window, r = row - w * window;
    const int64_t ci = ws.erank[e];
    const int64_t slot = (ws.col_off[w] + (ci / wide) * wide) * window + r * wide + (ci % wide);
    if (ci < 0 || ci >= ws.ucount[w] || slot < 0 || slot >= n_slots) {
        atomicOr(ws.flags, FLAG_OVERFLOW);  // no plan of this CSR in the workspace
        return;
    }
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

template <typename VT>
__global__ void __launch_bounds__(kEdgeThreads) k_fill_edges(
    const int32_t *__restrict__ rowptr, const int32_t *__restrict__ col, int64_t n_rows_used,
    int window, int wide, int64_t n_cols, int64_t n_rows, Workspace ws,
    const void *__restrict__ deg, int deg_dtype, VT *__restrict__ out_val,
    int32_t *__restrict__ out_map, int32_t *__restrict__ out_map_t,
    int32_t *__restrict__ out_edge_slot, int64_t nnz, int64_t n_slots) {
    __shared__ EdgeRows sh;
    EdgeChunk c;
    if (!edge_chunk(rowptr, n_rows_used, nnz, ws, sh, c)) return;
    for (int64_t e = c.eb + threadIdx.x; e < c.ee; e += kEdgeThreads)
        fill_edge<VT>(e, chunk_row_of(rowptr, sh, c, e), rowptr, col, window, wide, n_cols,
                      n_rows, ws, deg, deg_dtype, out_val, out_map, out_map_t, out_edge_slot,
                      n_slots);
}

// {n_condensed, n_parts, flags} of a finished plan, for one copy to the host
__global__ void k_plan_summary(Workspace ws, int64_t nw) {
    ws.summary[0] = ws.col_off[nw];
    ws.summary[1] = ws.part_off[nw];
    ws.summary[2] = ws.flags[0];
}
}  // namespace

// one warp per window of LO+1..CAP edges; dynamic shared memory of 8 warps x
// CAP keys (above the 48 KB default for 64-bit keys at CAP 1024)
template <typename KT, int CAP, int LO>
int launch_unique_warp(unsigned grid, const int32_t *rowptr, const int32_t *col, int64_t nw,
                       int window, int64_t nnz, int64_t n_cols, int unsorted_only, Workspace ws,
                       cudaStream_t st) {
    // register sort up to kWarpCap edges: no shared memory
    constexpr size_t smem = CAP <= kWarpCap ? 0 : (size_t)kWarpSortWarps * CAP * sizeof(KT);
    auto kernel = k_unique_warp<KT, CAP, LO>;
    if (smem > 48 * 1024) {
        static std::once_flag once;
        static cudaError_t e = cudaSuccess;
        std::call_once(once, [&] {
            e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        });
        ATT_CUDA(e, "k_unique_warp shared memory");
    }
    kernel<<<grid, kWarpSortWarps * 32, smem, st>>>(rowptr, col, nw, window, nnz, n_cols,
                                                    unsorted_only, ws);
    return launch_status("k_unique_warp");
}

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
        ATT_CUDA(cudaMemsetAsync(ws.wflag, 0, (size_t)nw * 4, st), "memset window flags");
        ATT_CUDA(cudaMemsetAsync(ws.wlist_n, 0, 4, st), "memset flagged count");
        // the large-window bitmaps start all-zero (each window clears its own bits)
        ATT_CUDA(cudaMemsetAsync(ws.bitmap, 0, (size_t)ws.n_bitmap_ctas * ws.words * 4, st),
                 "memset bitmap");
        ATT_CUDA(cudaMemsetAsync(ws.bsum, 0, (size_t)ws.n_bitmap_ctas * ws.swords * 4, st),
                 "memset bitmap summary");
        const int sms = sm_count();
        const int64_t g_warp0 = (nw + kWarpSortWarps - 1) / kWarpSortWarps;
        const unsigned g_warp = (unsigned)(g_warp0 < (int64_t)sms * 16 ? g_warp0 : (int64_t)sms * 16);
        const unsigned g_mid = (unsigned)(g_warp0 < (int64_t)sms * 8 ? g_warp0 : (int64_t)sms * 8);
        // 32-bit keys while (column << index bits) stays below the sentinel
        const bool narrow256 = n_cols <= (1ll << 24) - 1;
        const bool narrow1024 = n_cols <= (1ll << 22) - 1;
        // windows of <= kWarpCap edges: warp sorts in registers, one launch
        // per size class (up to 128 edges, then 129-256)
        s = narrow256 ? launch_unique_warp<uint32_t, 128, 0>(g_warp, rowptr, col, nw, window, nnz,
                                                            n_cols, 0, ws, st)
                      : launch_unique_warp<unsigned long long, 128, 0>(
                            g_warp, rowptr, col, nw, window, nnz, n_cols, 0, ws, st);
        if (s != ATT_OK) return s;
        s = narrow256 ? launch_unique_warp<uint32_t, kWarpCap, 128>(g_warp, rowptr, col, nw, window,
                                                                   nnz, n_cols, 0, ws, st)
                      : launch_unique_warp<unsigned long long, kWarpCap, 128>(
                            g_warp, rowptr, col, nw, window, nnz, n_cols, 0, ws, st);
        if (s != ATT_OK) return s;
        // larger windows: merge ranks, edge-parallel
        const int64_t rows_used = nw * window;
        const int64_t n_chunks = (nnz + kEdgeChunk - 1) / kEdgeChunk;
        k_chunk_rows<<<(unsigned)((rows_used + 255) / 256), 256, 0, st>>>(rowptr, rows_used,
                                                                          n_chunks, ws);
        s = launch_status("k_chunk_rows");
        if (s != ATT_OK) return s;
        if (nnz > 0) {
            ATT_CUDA(cudaMemsetAsync(ws.mscan, 0, (size_t)nnz * 4, st), "memset merge flags");
            k_merge_rank<<<(unsigned)n_chunks, kEdgeThreads, 0, st>>>(rowptr, col, rows_used,
                                                                      window, nnz, n_cols, ws);
            s = launch_status("k_merge_rank");
            if (s != ATT_OK) return s;
            s = scan32(ws.mscan, nnz, ws.scan32_tmp, 1, st);
            if (s != ATT_OK) return s;
            k_merge_emit<<<(unsigned)n_chunks, kEdgeThreads, 0, st>>>(rowptr, rows_used, window,
                                                                      nnz, ws);
            s = launch_status("k_merge_emit");
            if (s != ATT_OK) return s;
        }
        // windows with an unsorted row: sort (warp / CTA) or column bitmap
        s = narrow1024 ? launch_unique_warp<uint32_t, kMidCap, kWarpCap>(
                             g_mid, rowptr, col, nw, window, nnz, n_cols, 1, ws, st)
                       : launch_unique_warp<unsigned long long, kMidCap, kWarpCap>(
                             g_mid, rowptr, col, nw, window, nnz, n_cols, 1, ws, st);
        if (s != ATT_OK) return s;
        const int64_t g_small = nw < (int64_t)sms * 4 ? nw : (int64_t)sms * 4;
        k_unique_small<<<(unsigned)g_small, kSmallThreads, 0, st>>>(rowptr, col, nw, window, nnz,
                                                                     n_cols, 1, ws);
        s = launch_status("k_unique_small");
        if (s != ATT_OK) return s;
        const int64_t g_large = nw < ws.n_bitmap_ctas ? nw : ws.n_bitmap_ctas;
        k_unique_large<<<(unsigned)g_large, kLargeThreads, 0, st>>>(rowptr, col, nw, window, nnz,
                                                                     n_cols, 1, ws);
        s = launch_status("k_unique_large");
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

namespace {
// Argument checks shared by the fill entry points; lays out `ws`.
int fill_checks(const int32_t *rowptr, const int32_t *col, int64_t n_rows, int64_t nnz,
                int64_t n_cols, int window, int wide, int part, const void *deg, int deg_dtype,
                const void *workspace, size_t workspace_bytes, int32_t *out_rowptr,
                const void *out_val, int val_dtype, Workspace &ws) {
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
    workspace_layout(n_rows, nnz, n_cols, window, &ws, (char *)workspace);
    return ATT_OK;
}


// Enqueue the fill of a plan with n_cond condensed columns and n_parts parts
// (the plan's own sizes) on `st`; no synchronisation.
int fill_enqueue(const int32_t *rowptr, const int32_t *col, int64_t n_rows, int64_t nnz,
                 int64_t n_cols, int window, int wide, int part, const void *deg, int deg_dtype,
                 const Workspace &ws, int64_t n_cond, int64_t n_parts, int32_t *out_rowptr,
                 int32_t *out_col, void *out_val, int val_dtype, int32_t *out_map,
                 int32_t *out_map_t, int32_t *out_edge_slot, int32_t *out_window,
                 int32_t *out_atomic, cudaStream_t st) {
    int s = ATT_OK;
    const int64_t nw = n_windows(n_rows, window);
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
    if (n_cond > 0) {
        const int64_t n_cchunks = (n_cond + kColChunkW - 1) / kColChunkW;
        ATT_CHECK(n_cchunks <= (nnz + 64 * nw) / kColChunkW + 1, ATT_ERR_WORKSPACE,
                  "condensed columns beyond the workspace's bound");
        k_col_chunk_windows<<<(unsigned)((nw + 255) / 256), 256, 0, st>>>(nw, n_cchunks, ws);
        s = launch_status("k_col_chunk_windows");
        if (s != ATT_OK) return s;
        k_fill_cols<<<(unsigned)n_cchunks, kColThreads, 0, st>>>(nw, n_cond, window, ws, rowptr,
                                                                 out_col);
        s = launch_status("k_fill_cols");
        if (s != ATT_OK) return s;
    }
    {
        const int64_t threads = n_parts > 0 ? n_parts : 1;
        k_fill_parts<<<(unsigned)((threads + 255) / 256), 256, 0, st>>>(
            nw, n_parts, wide, part, ws, out_rowptr, out_window, out_atomic);
        s = launch_status("k_fill_parts");
        if (s != ATT_OK) return s;
    }
    if (nw > 0 && nnz > 0 && (out_val || out_map || out_map_t || out_edge_slot)) {
        const int64_t rows_used = nw * window;
        // chunk rows come from the plan; CTAs past the used edges exit
        const unsigned grid = (unsigned)((nnz + kEdgeChunk - 1) / kEdgeChunk);
        const int64_t n_slots = (int64_t)nslot;
        if (!out_val || val_dtype == ATT_F16) {
            k_fill_edges<__half><<<grid, kEdgeThreads, 0, st>>>(
                rowptr, col, rows_used, window, wide, n_cols, n_rows, ws, deg, deg_dtype,
                (__half *)out_val, out_map, out_map_t, out_edge_slot, nnz, n_slots);
        } else if (val_dtype == ATT_BF16) {
            k_fill_edges<__nv_bfloat16><<<grid, kEdgeThreads, 0, st>>>(
                rowptr, col, rows_used, window, wide, n_cols, n_rows, ws, deg, deg_dtype,
                (__nv_bfloat16 *)out_val, out_map, out_map_t, out_edge_slot, nnz, n_slots);
        } else {
            k_fill_edges<float><<<grid, kEdgeThreads, 0, st>>>(
                rowptr, col, rows_used, window, wide, n_cols, n_rows, ws, deg, deg_dtype,
                (float *)out_val, out_map, out_map_t, out_edge_slot, nnz, n_slots);
        }
        s = launch_status("k_fill_edges");
        if (s != ATT_OK) return s;
    }
    return ATT_OK;
}

// Status of a fill from its device-side flags.
int fill_flags_status(const int32_t *flags, int want_map_t) {
    ATT_CHECK(!(want_map_t && (flags[0] & FLAG_UNSORTED)), ATT_ERR_FORMAT,
              "mirrored-edge map needs every CSR row sorted by column");
    ATT_CHECK(!(flags[0] & FLAG_OVERFLOW), ATT_ERR_FORMAT,
              "the workspace does not hold a plan of this CSR (run att_block_plan first)");
    return ATT_OK;
}
}  // namespace

extern "C" int att_block_fill(const int32_t *rowptr, const int32_t *col, int64_t n_rows,
                              int64_t nnz, int64_t n_cols, int window, int wide, int part,
                              int emit_empty, const void *deg, int deg_dtype,
                              const void *workspace, size_t workspace_bytes, int32_t *out_rowptr,
                              int32_t *out_col, void *out_val, int val_dtype, int32_t *out_map,
                              int32_t *out_map_t, int32_t *out_edge_slot, int32_t *out_window,
                              int32_t *out_atomic, void *stream) {
    clear_error();
    (void)emit_empty;  // the plan decided the parts
    Workspace ws;
    int s = fill_checks(rowptr, col, n_rows, nnz, n_cols, window, wide, part, deg, deg_dtype,
                        workspace, workspace_bytes, out_rowptr, out_val, val_dtype, ws);
    if (s != ATT_OK) return s;
    cudaStream_t st = (cudaStream_t)stream;
    const int64_t nw = n_windows(n_rows, window);
    int64_t tot[2] = {0, 0};
    ATT_CUDA(cudaMemcpyAsync(&tot[0], ws.col_off + nw, 8, cudaMemcpyDeviceToHost, st), "d2h");
    ATT_CUDA(cudaMemcpyAsync(&tot[1], ws.part_off + nw, 8, cudaMemcpyDeviceToHost, st), "d2h");
    ATT_CUDA(cudaStreamSynchronize(st), "fill sync");
    const int64_t n_cond = tot[0], n_parts = tot[1];
    s = fill_enqueue(rowptr, col, n_rows, nnz, n_cols, window, wide, part, deg, deg_dtype, ws,
                     n_cond, n_parts, out_rowptr, out_col, out_val, val_dtype, out_map, out_map_t,
                     out_edge_slot, out_window, out_atomic, st);
    if (s != ATT_OK) return s;
    int32_t flags[4];
    ATT_CUDA(cudaMemcpyAsync(flags, ws.flags, 16, cudaMemcpyDeviceToHost, st), "d2h");
    ATT_CUDA(cudaStreamSynchronize(st), "fill sync");
    return fill_flags_status(flags, out_map_t != nullptr);
}

extern "C" int att_block_fill_async(const int32_t *rowptr, const int32_t *col, int64_t n_rows,
                                    int64_t nnz, int64_t n_cols, int window, int wide, int part,
                                    int emit_empty, const void *deg, int deg_dtype,
                                    const void *workspace, size_t workspace_bytes,
                                    int64_t n_parts, int64_t n_condensed, int32_t *out_rowptr,
                                    int32_t *out_col, void *out_val, int val_dtype,
                                    int32_t *out_map, int32_t *out_map_t, int32_t *out_edge_slot,
                                    int32_t *out_window, int32_t *out_atomic, int32_t *flags,
                                    void *stream) {
    clear_error();
    (void)emit_empty;
    ATT_CHECK(flags != nullptr && n_parts >= 0 && n_condensed >= 0, ATT_ERR_INVALID,
              "null flags or negative sizes");
    Workspace ws;
    int s = fill_checks(rowptr, col, n_rows, nnz, n_cols, window, wide, part, deg, deg_dtype,
                        workspace, workspace_bytes, out_rowptr, out_val, val_dtype, ws);
    if (s != ATT_OK) return s;
    cudaStream_t st = (cudaStream_t)stream;
    s = fill_enqueue(rowptr, col, n_rows, nnz, n_cols, window, wide, part, deg, deg_dtype, ws,
                     n_condensed, n_parts, out_rowptr, out_col, out_val, val_dtype, out_map,
                     out_map_t, out_edge_slot, out_window, out_atomic, st);
    if (s != ATT_OK) return s;
    ATT_CUDA(cudaMemcpyAsync(flags, ws.flags, 16, cudaMemcpyDeviceToHost, st), "d2h flags");
    return ATT_OK;
}

extern "C" int att_block_fill_result(const int32_t *flags, int with_map_t) {
    clear_error();
    ATT_CHECK(flags != nullptr, ATT_ERR_INVALID, "null flags");
    return fill_flags_status(flags, with_map_t);
}
