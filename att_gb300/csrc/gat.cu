// gat.cu -- the GAT operators on the row-window block format with a
// slot -> edge map (the form ATT_Block*.blockProcess_sddmm_balance_gnn
// returns).  They replace the reference's ATT_SDDMM_v{1,3,4} and
// ATT_SpMM_v{1,3,4} extension ops, whose CUDA source is not in the reference
// tree; their meaning is pinned by the reference's tests
// (benchmark-v3/{sddmm,spmm}-benchmark/test/*) and callers
// (end2end_ori/gat_final/mgat_csr/mgat_conv.py, end2end_head/gat_final/mgat_csr/mgat_conv.py).
//
// Every edge-valued tensor is addressed as base[h * stride_h + e * stride_e]
// and every node-valued tensor as base[h * stride_h + node * stride_n], so the
// [h, nnz] / [nnz, h] and [h, M, F] / [M, h, F] layouts of the v1/v3/v4 ops
// are all views.
//
//   k_node_scores     s[h][m] = X[h][m] . a[h]                (warp per node row)
//   k_slot_edges      per slot with an edge: additive score s0[row]+s1[col]
//                     or row broadcast g[row]; written at the edge id
//   k_sddmm16/_tf32   blocked SDDMM S = B_cols . A_rows^T on tensor cores
//                     (mma.sync m16n8k16 / 3xTF32 m16n8k8), gathered rows
//                     staged by cp.async, results scattered to edge ids
//   k_gather_slots    dense block values from per-edge values through the map
//   k_rowsum_slots    per-row sums of per-edge values through the map
#include "att_common.cuh"

#include <mutex>

namespace att {
namespace {

template <typename T>
__device__ __forceinline__ float ld_f(const void *p, int64_t i);
template <>
__device__ __forceinline__ float ld_f<__half>(const void *p, int64_t i) {
    return __half2float(((const __half *)p)[i]);
}
template <>
__device__ __forceinline__ float ld_f<__nv_bfloat16>(const void *p, int64_t i) {
    return __bfloat162float(((const __nv_bfloat16 *)p)[i]);
}
template <>
__device__ __forceinline__ float ld_f<float>(const void *p, int64_t i) {
    return ((const float *)p)[i];
}

__device__ __forceinline__ float ld_any(const void *p, int dt, int64_t i) {
    if (dt == ATT_F16) return ld_f<__half>(p, i);
    if (dt == ATT_BF16) return ld_f<__nv_bfloat16>(p, i);
    return ld_f<float>(p, i);
}
__device__ __forceinline__ void st_any(void *p, int dt, int64_t i, float v) {
    if (dt == ATT_F16) ((__half *)p)[i] = __float2half_rn(v);
    else if (dt == ATT_BF16) ((__nv_bfloat16 *)p)[i] = __float2bfloat16_rn(v);
    else ((float *)p)[i] = v;
}

// slot index of (window row r, global condensed column g)
__device__ __forceinline__ int64_t slot_of(int64_t g, int r, int W, int wide) {
    return (g - g % wide) * W + (int64_t)r * wide + g % wide;
}

// ---- node scores ------------------------------------------------------------
__global__ void k_node_scores(const void *__restrict__ X, int xdt, int64_t H, int64_t M, int64_t F,
                              int64_t xsh, int64_t xsm, const void *__restrict__ a, int adt,
                              int64_t ash, float *__restrict__ s, int64_t ssh) {
    const int lane = threadIdx.x & 31;
    const int64_t wid = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (wid >= H * M) return;
    const int64_t h = wid / M, m = wid - h * M;
    float acc = 0.f;
    for (int64_t f = lane; f < F; f += 32)
        acc += ld_any(X, xdt, h * xsh + m * xsm + f) * ld_any(a, adt, h * ash + f);
    acc = warp_sum(acc);
    if (lane == 0) s[h * ssh + m] = acc;
}

// s0[h][m] = X[h][m] . a0[h] and s1[h][m] = X[h][m] . a1[h] in one pass over X
// (16-bit X, fp32 attention vectors): LPR = F / 8 lanes per node row, each
// loading 8 features with one 16-byte load; the row's partial sums meet by
// shuffles within its lanes.
template <typename T, int LPR>
__global__ void k_node_scores_pair(const T *__restrict__ X, int64_t H, int64_t M, int64_t xsh,
                                   int64_t xsm, const float *__restrict__ a0,
                                   const float *__restrict__ a1, int64_t ash,
                                   float *__restrict__ s0, float *__restrict__ s1, int64_t ssh) {
    constexpr int RPW = 32 / LPR;  // node rows per warp
    const int lane = threadIdx.x & 31, sub = lane % LPR;
    const int64_t row = (((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * RPW + lane / LPR;
    const bool ok = row < H * M;
    const int64_t h = ok ? row / M : 0, m = ok ? row - h * M : 0;
    float acc0 = 0.f, acc1 = 0.f;
    if (ok) {
        const uint4 v = *reinterpret_cast<const uint4 *>(X + h * xsh + m * xsm + sub * 8);
        const T *x = reinterpret_cast<const T *>(&v);
        const float4 p0 = *reinterpret_cast<const float4 *>(a0 + h * ash + sub * 8);
        const float4 q0 = *reinterpret_cast<const float4 *>(a0 + h * ash + sub * 8 + 4);
        const float4 p1 = *reinterpret_cast<const float4 *>(a1 + h * ash + sub * 8);
        const float4 q1 = *reinterpret_cast<const float4 *>(a1 + h * ash + sub * 8 + 4);
        const float w0[8] = {p0.x, p0.y, p0.z, p0.w, q0.x, q0.y, q0.z, q0.w};
        const float w1[8] = {p1.x, p1.y, p1.z, p1.w, q1.x, q1.y, q1.z, q1.w};
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const float xv = ld_f<T>(x, k);
            acc0 += xv * w0[k];
            acc1 += xv * w1[k];
        }
    }
#pragma unroll
    for (int o = LPR / 2; o > 0; o >>= 1) {
        acc0 += __shfl_xor_sync(0xffffffffu, acc0, o);
        acc1 += __shfl_xor_sync(0xffffffffu, acc1, o);
    }
    if (ok && sub == 0) {
        s0[h * ssh + m] = acc0;
        s1[h * ssh + m] = acc1;
    }
}

// ---- per-slot edge values -----------------------------------------------------
// mode 0: out[e] = s0[row] + s1[col]      mode 1: out[e] = g[row]
struct SlotEdgeArgs {
    const int32_t *rowptr, *col, *map, *win;
    int64_t n_parts;
    int W, wide;
    int mode;
    const float *s0, *s1;
    int64_t ssh;
    const void *g;
    int gdt;
    int64_t gsh, gsn;
    void *out;
    int odt;
    int64_t osh, ose;
    int64_t H, n_nodes;
};

__global__ void k_slot_edges(SlotEdgeArgs A) {
    const int lane = threadIdx.x & 31;
    const int64_t wid = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (wid >= A.n_parts * A.H) return;
    const int64_t p = wid / A.H, h = wid - p * A.H;
    const int64_t start = A.rowptr[2 * p], end_real = A.rowptr[2 * p + 1];
    const int64_t pend = (end_real + A.wide - 1) / A.wide * A.wide;
    const int64_t win = A.win[p];
    const int64_t nslot = (pend - start) * A.W;
    for (int64_t q = lane; q < nslot; q += 32) {
        const int64_t s = start * A.W + q;
        const int32_t e = A.map[s];
        if (e < 0) continue;
        const int64_t inb = q % ((int64_t)A.W * A.wide);
        const int r = (int)(inb / A.wide);
        const int64_t g = start + (q / ((int64_t)A.W * A.wide)) * A.wide + inb % A.wide;
        const int64_t row = win * A.W + r;
        float v;
        if (A.mode == 0) {
            const int32_t c = A.col[g];
            v = (row < A.n_nodes ? A.s0[h * A.ssh + row] : 0.f) +
                (c >= 0 && c < A.n_nodes ? A.s1[h * A.ssh + c] : 0.f);
        } else {
            v = row < A.n_nodes ? ld_any(A.g, A.gdt, h * A.gsh + row * A.gsn) : 0.f;
        }
        st_any(A.out, A.odt, h * A.osh + (int64_t)e * A.ose, v);
    }
}

// ---- dense block values through the map ------------------------------------------
// out is in the layout of block width out_wide, the map in that of map_wide
// (W, map_wide and out_wide are powers of two, given as log2); heads on y
__global__ void k_gather_slots(const int32_t *__restrict__ map, int64_t n_slots, int lw,
                               int lmw, int low, const void *vals, int vdt, int64_t vsh,
                               int64_t vse, void *out, int odt, int64_t osh) {
    const int64_t h = blockIdx.y;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < n_slots; s += stride) {
        int64_t ms = s;
        if (lmw != low) {
            const int64_t blk = s >> (lw + low), inb = s & ((1 << (lw + low)) - 1);
            const int r = (int)(inb >> low);
            const int64_t g = (blk << low) | (inb & ((1 << low) - 1));
            ms = ((g >> lmw) << (lmw + lw)) | ((int64_t)r << lmw) | (g & ((1 << lmw) - 1));
        }
        const int32_t e = map[ms];
        const float v = e >= 0 ? ld_any(vals, vdt, h * vsh + (int64_t)e * vse) : 0.f;
        st_any(out, odt, h * osh + s, v);
    }
}

// ---- row sums through the map -----------------------------------------------------------
template <int W>
__global__ void k_rowsum_slots(const int32_t *__restrict__ rowptr, const int32_t *__restrict__ map,
                               const int32_t *__restrict__ win, const int32_t *__restrict__ atomic,
                               int64_t n_parts, int wide, const void *vals, int vdt, int64_t vsh,
                               int64_t vse, int64_t H, float *out, int64_t osh, int64_t osm,
                               int64_t m_out) {
    const int lane = threadIdx.x & 31;
    const int64_t wid = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (wid >= n_parts * H) return;
    const int64_t p = wid / H, h = wid - p * H;
    const int64_t start = rowptr[2 * p], end_real = rowptr[2 * p + 1];
    const int64_t pend = (end_real + wide - 1) / wide * wide;
    const int64_t nslot = (pend - start) * W;
    float acc[W];
#pragma unroll
    for (int r = 0; r < W; ++r) acc[r] = 0.f;
    for (int64_t q = lane; q < nslot; q += 32) {
        const int32_t e = map[start * W + q];
        if (e < 0) continue;
        const int r = (int)((q % ((int64_t)W * wide)) / wide);
        const float v = ld_any(vals, vdt, h * vsh + (int64_t)e * vse);
#pragma unroll
        for (int rr = 0; rr < W; ++rr)
            if (rr == r) acc[rr] += v;
    }
#pragma unroll
    for (int r = 0; r < W; ++r) acc[r] = warp_sum(acc[r]);
    const bool add = atomic[p] != 0;
    const int64_t row0 = (int64_t)win[p] * W;
    if (lane < W) {
        float v = 0.f;
#pragma unroll
        for (int r = 0; r < W; ++r)
            if (r == lane) v = acc[r];
        const int64_t row = row0 + lane;
        if (row >= 0 && row < m_out) {
            float *dst = out + h * osh + row * osm;
            if (add) red_add_f32(dst, v);
            else *dst = v;
        }
    }
}

// zero the rows no unsplit part writes (all heads)
__global__ void k_zero_rows_heads(const int32_t *__restrict__ win, const int32_t *__restrict__ atomic,
                                  int64_t n_parts, int W, float *out, int64_t osh, int64_t osm,
                                  int64_t m_out, int64_t H) {
    const int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t n_w = (m_out + W - 1) / W;
    if (w >= n_w) return;
    int64_t lo = 0, hi = n_parts;
    while (lo < hi) {
        int64_t mid = (lo + hi) >> 1;
        if (win[mid] < w) lo = mid + 1; else hi = mid;
    }
    if (lo < n_parts && win[lo] == w && atomic[lo] == 0) return;
    const int64_t r1 = (w + 1) * W < m_out ? (w + 1) * W : m_out;
    for (int64_t h = 0; h < H; ++h)
        for (int64_t r = w * W; r < r1; ++r) out[h * osh + r * osm] = 0.f;
}

// ---- blocked SDDMM on tensor cores -----------------------------------------------
constexpr int kSWarps = 4;
constexpr int kSThreads = kSWarps * 32;
constexpr int kSStages = 3;

struct SddmmArgs {
    const int32_t *rowptr, *col, *map, *win;
    int64_t n_parts;
    int wide;
    const void *A;  // window rows (the "query" side):  A[h*ash + row*asn + f]
    int64_t ash, asn, n_a;
    const void *B;  // gathered columns:                 B[h*bsh + col*bsn + f]
    int64_t bsh, bsn, n_b;
    int64_t F, H;
    void *out;
    int odt;
    int64_t osh, ose;
    int32_t *err;
};

template <int ROW_BYTES>
__device__ __forceinline__ int sswz(int r) {
    if constexpr (ROW_BYTES >= 128) return r & 7;
    else return (r >> 1) & 3;
}

template <typename T, int W, int FC>
struct SCfg {
    static constexpr int ES = sizeof(T);
    static constexpr int XROW = FC * ES;
    static constexpr int XSTAGE = 16 * XROW;
    static constexpr int MSTAGE = 16 * W * 4;  // the step's map entries
    static constexpr int STAGE = XSTAGE + MSTAGE;
    static constexpr int WARP_SMEM = kSStages * STAGE;
    static constexpr int SMEM = kSWarps * WARP_SMEM;
    static constexpr int CPR = XROW / 16;
    static constexpr int RPP = 32 / CPR > 0 ? 32 / CPR : 1;
    static constexpr int PASSES = 16 * CPR / 32;
    static constexpr int NT = W / 8;
};

// 16-bit operands: S[col][row] = sum_f B[col][f] * A[row][f]  (m16n8k16)
template <typename T, int W, int FC>
__global__ void __launch_bounds__(kSThreads) k_sddmm16(SddmmArgs P) {
    using C = SCfg<T, W, FC>;
    static_assert(C::CPR <= 32, "row too wide");
    extern __shared__ __align__(128) unsigned char smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t sbase = smem_u32(smem) + warp * C::WARP_SMEM;
    const unsigned char *sgen = smem + warp * C::WARP_SMEM;
    const int gid = lane >> 2, tig = lane & 3;
    const int64_t n_items = P.n_parts * P.H;
    const int64_t stride = (int64_t)gridDim.x * kSWarps;
    const T *A = (const T *)P.A;
    const T *B = (const T *)P.B;

    // slot of (step column cl, window row r) relative to the step's first slot:
    // fixed per lane, since every step starts on a multiple of wide (4, 8, 16)
    int lsl[C::NT][4];
#pragma unroll
    for (int t = 0; t < C::NT; ++t)
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int cl = gid + 8 * (u >> 1), r = t * 8 + 2 * tig + (u & 1);
            lsl[t][u] = (cl - cl % P.wide) * W + r * P.wide + cl % P.wide;
        }
    for (int64_t item = (int64_t)blockIdx.x * kSWarps + warp; item < n_items; item += stride) {
        const int64_t part = item / P.H, h = item - part * P.H;
        const int start = P.rowptr[2 * part];
        const int e_real = P.rowptr[2 * part + 1];
        const int nreal = e_real > start ? e_real - start : 0;
        const int nsteps = (nreal + 15) >> 4;
        if (nsteps == 0) continue;
        const int64_t wrow = (int64_t)P.win[part] * W;
        // B fragments (window rows) for every 16-feature k-step, all n-tiles
        uint32_t bq[FC / 16][C::NT][2];
#pragma unroll
        for (int kk = 0; kk < FC / 16; ++kk)
#pragma unroll
            for (int t = 0; t < C::NT; ++t)
#pragma unroll
                for (int u = 0; u < 2; ++u) {
                    const int64_t row = wrow + t * 8 + gid;
                    const int64_t f = 16 * kk + 2 * tig + 8 * u;
                    uint32_t v = 0;
                    if (row < P.n_a && f < P.F) {
                        const T *src = A + h * P.ash + row * P.asn + f;
                        if (f + 1 < P.F) v = *(const uint32_t *)src;
                        else v = (uint32_t)(*(const uint16_t *)src);
                    }
                    bq[kk][t][u] = v;
                }
        auto issue = [&](int stage, int step) {
            const uint32_t xs = sbase + stage * C::STAGE;
            const uint32_t ms = xs + C::XSTAGE;
            const int c0 = step * 16;
            int myc = -1;
            if (c0 + (lane & 15) < nreal) myc = P.col[start + c0 + (lane & 15)];
#pragma unroll
            for (int i = 0; i < C::PASSES; ++i) {
                const int idx = i * 32 + lane;
                const int r = idx / C::CPR, ch = idx % C::CPR;
                const int cidx = __shfl_sync(0xffffffffu, myc, r);
                const int64_t f = (int64_t)ch * (16 / C::ES);
                bool ok = cidx >= 0 && cidx < P.n_b && f < P.F;
                if (cidx >= P.n_b || cidx < -1) {
                    if (P.err) atomicOr(P.err, 1);
                }
                const T *src = ok ? B + h * P.bsh + (int64_t)cidx * P.bsn + f : B;
                cp_async16(xs + r * C::XROW + ((ch ^ sswz<C::XROW>(r)) << 4), src, ok ? 16 : 0);
            }
            // the step's map entries are contiguous: 16 columns x W rows
            for (int q = lane; q < 16 * W / 4; q += 32) {
                const int blk = (q * 4) / (W * P.wide);
                const bool ok = c0 + blk * P.wide < nreal;
                const int32_t *src = P.map + (int64_t)(start + c0) * W + q * 4;
                cp_async16(ms + q * 16, ok ? (const void *)src : (const void *)P.map, ok ? 16 : 0);
            }
        };
#pragma unroll
        for (int s = 0; s < kSStages - 1; ++s) {
            if (s < nsteps) issue(s, s);
            cp_async_commit();
        }
        for (int step = 0; step < nsteps; ++step) {
            cp_async_wait<kSStages - 2>();
            __syncwarp();
            const int stage = step % kSStages;
            const uint32_t xs = sbase + stage * C::STAGE;
            const int32_t *ms = (const int32_t *)(sgen + stage * C::STAGE + C::XSTAGE);
            float acc[C::NT][4];
#pragma unroll
            for (int t = 0; t < C::NT; ++t) acc[t][0] = acc[t][1] = acc[t][2] = acc[t][3] = 0.f;
#pragma unroll
            for (int kk = 0; kk < FC / 16; ++kk) {
                const int q = lane >> 3, rr = lane & 7;
                const int m = (q & 1) * 8 + rr;
                const int ch = 2 * kk + (q >> 1);
                uint32_t a[4];
                ldsm_x4(xs + m * C::XROW + ((ch ^ sswz<C::XROW>(m)) << 4), a[0], a[1], a[2], a[3]);
#pragma unroll
                for (int t = 0; t < C::NT; ++t) mma_16816<T>(acc[t], a, bq[kk][t][0], bq[kk][t][1]);
            }
            // scatter S[col][row] to the edge ids of the step's slots
            const int c0 = step * 16;
#pragma unroll
            for (int t = 0; t < C::NT; ++t)
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int cl = gid + 8 * (u >> 1);
                    const int r = t * 8 + 2 * tig + (u & 1);
                    if (c0 + cl < nreal) {
                        const int32_t e = ms[lsl[t][u]];
                        if (e >= 0) st_any(P.out, P.odt, h * P.osh + (int64_t)e * P.ose, acc[t][u]);
                    }
                }
            __syncwarp();
            if (step + kSStages - 1 < nsteps) issue((step + kSStages - 1) % kSStages, step + kSStages - 1);
            cp_async_commit();
        }
        cp_async_wait<0>();
        __syncwarp();
    }
}

// fp32 operands, 3xTF32: S[col][row] with m16n8k8

// the fp32 kernel also keeps each warp's window rows (W x FC, rows padded by
// 4 floats against bank conflicts) in shared memory, after the stage ring
template <int W, int FC>
struct STf32 {
    static constexpr int QROW = FC + 4;
    static constexpr int QTILE = W * QROW * 4;
    static constexpr int SMEM = SCfg<float, W, FC>::SMEM + kSWarps * QTILE;
};

template <int W, int FC>
__global__ void __launch_bounds__(kSThreads) k_sddmm_tf32(SddmmArgs P) {
    using C = SCfg<float, W, FC>;
    using Q = STf32<W, FC>;
    extern __shared__ __align__(128) unsigned char smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t sbase = smem_u32(smem) + warp * C::WARP_SMEM;
    const unsigned char *sgen = smem + warp * C::WARP_SMEM;
    float *qs = (float *)(smem + C::SMEM + warp * Q::QTILE);
    const int gid = lane >> 2, tig = lane & 3;
    const int64_t n_items = P.n_parts * P.H;
    const int64_t stride = (int64_t)gridDim.x * kSWarps;
    const float *A = (const float *)P.A;
    const float *B = (const float *)P.B;

    // slot of (step column cl, window row r) relative to the step's first slot:
    // fixed per lane, since every step starts on a multiple of wide (4, 8, 16)
    int lsl[C::NT][4];
#pragma unroll
    for (int t = 0; t < C::NT; ++t)
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int cl = gid + 8 * (u >> 1), r = t * 8 + 2 * tig + (u & 1);
            lsl[t][u] = (cl - cl % P.wide) * W + r * P.wide + cl % P.wide;
        }
    for (int64_t item = (int64_t)blockIdx.x * kSWarps + warp; item < n_items; item += stride) {
        const int64_t part = item / P.H, h = item - part * P.H;
        const int start = P.rowptr[2 * part];
        const int e_real = P.rowptr[2 * part + 1];
        const int nreal = e_real > start ? e_real - start : 0;
        const int nsteps = (nreal + 15) >> 4;
        if (nsteps == 0) continue;
        const int64_t wrow = (int64_t)P.win[part] * W;
        // the window rows (the B side), staged once per item
        __syncwarp();
        for (int q = lane; q < W * FC; q += 32) {
            const int rr = q / FC, f = q % FC;
            const int64_t row = wrow + rr;
            qs[rr * Q::QROW + f] = (row < P.n_a && f < P.F) ? A[h * P.ash + row * P.asn + f] : 0.f;
        }
        __syncwarp();
        auto issue = [&](int stage, int step) {
            const uint32_t xs = sbase + stage * C::STAGE;
            const uint32_t ms = xs + C::XSTAGE;
            const int c0 = step * 16;
            int myc = -1;
            if (c0 + (lane & 15) < nreal) myc = P.col[start + c0 + (lane & 15)];
#pragma unroll
            for (int i = 0; i < C::PASSES; ++i) {
                const int idx = i * 32 + lane;
                const int r = idx / C::CPR, ch = idx % C::CPR;
                const int cidx = __shfl_sync(0xffffffffu, myc, r);
                const int64_t f = (int64_t)ch * 4;
                bool ok = cidx >= 0 && cidx < P.n_b && f < P.F;
                if (cidx >= P.n_b || cidx < -1) {
                    if (P.err) atomicOr(P.err, 1);
                }
                const float *src = ok ? B + h * P.bsh + (int64_t)cidx * P.bsn + f : B;
                cp_async16(xs + r * C::XROW + ((ch ^ (r & 7)) << 4), src, ok ? 16 : 0);
            }
            for (int q = lane; q < 16 * W / 4; q += 32) {
                const int blk = (q * 4) / (W * P.wide);
                const bool ok = c0 + blk * P.wide < nreal;
                const int32_t *src = P.map + (int64_t)(start + c0) * W + q * 4;
                cp_async16(ms + q * 16, ok ? (const void *)src : (const void *)P.map, ok ? 16 : 0);
            }
        };
#pragma unroll
        for (int s = 0; s < kSStages - 1; ++s) {
            if (s < nsteps) issue(s, s);
            cp_async_commit();
        }
        for (int step = 0; step < nsteps; ++step) {
            cp_async_wait<kSStages - 2>();
            __syncwarp();
            const int stage = step % kSStages;
            const float *xsg = (const float *)(sgen + stage * C::STAGE);
            const int32_t *ms = (const int32_t *)(sgen + stage * C::STAGE + C::XSTAGE);
            float acc[C::NT][4];
#pragma unroll
            for (int t = 0; t < C::NT; ++t) acc[t][0] = acc[t][1] = acc[t][2] = acc[t][3] = 0.f;
#pragma unroll 2
            for (int kk = 0; kk < FC / 8; ++kk) {
                uint32_t ah[4], al[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int m = gid + 8 * (u & 1);
                    const int f = 8 * kk + tig + 4 * (u >> 1);
                    const float x = xsg[m * FC + (((f >> 2) ^ (m & 7)) << 2) + (f & 3)];
                    split_tf32x3(x, ah[u], al[u]);
                }
#pragma unroll
                for (int t = 0; t < C::NT; ++t) {
                    uint32_t bh[2], bl[2];
                    const float *qr = qs + (t * 8 + gid) * Q::QROW + 8 * kk + tig;
                    split_tf32x3(qr[0], bh[0], bl[0]);
                    split_tf32x3(qr[4], bh[1], bl[1]);
                    mma_1688_tf32(acc[t], al[0], al[1], al[2], al[3], bh[0], bh[1]);
                    mma_1688_tf32(acc[t], ah[0], ah[1], ah[2], ah[3], bl[0], bl[1]);
                    mma_1688_tf32(acc[t], ah[0], ah[1], ah[2], ah[3], bh[0], bh[1]);
                }
            }
            const int c0 = step * 16;
#pragma unroll
            for (int t = 0; t < C::NT; ++t)
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int cl = gid + 8 * (u >> 1);
                    const int r = t * 8 + 2 * tig + (u & 1);
                    if (c0 + cl < nreal) {
                        const int32_t e = ms[lsl[t][u]];
                        if (e >= 0) st_any(P.out, P.odt, h * P.osh + (int64_t)e * P.ose, acc[t][u]);
                    }
                }
            __syncwarp();
            if (step + kSStages - 1 < nsteps) issue((step + kSStages - 1) % kSStages, step + kSStages - 1);
            cp_async_commit();
        }
        cp_async_wait<0>();
        __syncwarp();
    }
}

template <typename K>
int sddmm_launch(K kernel, int smem, int64_t items, const SddmmArgs &P, cudaStream_t st,
                 std::once_flag &once, int &prep) {
    std::call_once(once, [&] {
        prep = cuda_status(
            cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem),
            "cudaFuncSetAttribute");
    });
    if (prep != ATT_OK) return prep;
    if (items == 0) return ATT_OK;
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kSThreads, smem);
    if (per_sm < 1) per_sm = 1;
    int64_t want = (items + kSWarps - 1) / kSWarps;
    int64_t cap = (int64_t)sm_count() * per_sm;
    int grid = (int)(want < cap ? want : cap);
    kernel<<<grid, kSThreads, smem, st>>>(P);
    return launch_status("k_sddmm");
}

template <typename T, int W, int FC>
int run_sddmm16(const SddmmArgs &P, cudaStream_t st) {
    static std::once_flag once;
    static int prep = ATT_OK;
    return sddmm_launch(k_sddmm16<T, W, FC>, SCfg<T, W, FC>::SMEM, P.n_parts * P.H, P, st, once,
                        prep);
}
template <int W, int FC>
int run_sddmm32(const SddmmArgs &P, cudaStream_t st) {
    static std::once_flag once;
    static int prep = ATT_OK;
    return sddmm_launch(k_sddmm_tf32<W, FC>, STf32<W, FC>::SMEM, P.n_parts * P.H, P, st,
                        once, prep);
}

template <typename T, int W>
int dispatch_sddmm16(const SddmmArgs &P, cudaStream_t st) {
    if (P.F <= 32) return run_sddmm16<T, W, 32>(P, st);
    if (P.F <= 64) return run_sddmm16<T, W, 64>(P, st);
    if (P.F <= 128) return run_sddmm16<T, W, 128>(P, st);
    return run_sddmm16<T, W, 256>(P, st);
}
template <int W>
int dispatch_sddmm32(const SddmmArgs &P, cudaStream_t st) {
    if (P.F <= 32) return run_sddmm32<W, 32>(P, st);
    if (P.F <= 64) return run_sddmm32<W, 64>(P, st);
    return run_sddmm32<W, 128>(P, st);
}

}  // namespace
}  // namespace att

using namespace att;

extern "C" int att_node_scores(const void *X, int x_dtype, int64_t n_heads, int64_t n_nodes,
                               int64_t F, int64_t x_stride_h, int64_t x_stride_n, const void *a,
                               int a_dtype, int64_t a_stride_h, float *scores,
                               int64_t s_stride_h, void *stream) {
    clear_error();
    ATT_CHECK(n_heads >= 0 && n_nodes >= 0 && F >= 0, ATT_ERR_INVALID, "negative size");
    ATT_CHECK(x_dtype >= ATT_F32 && x_dtype <= ATT_BF16 && a_dtype >= ATT_F32 && a_dtype <= ATT_BF16,
              ATT_ERR_UNSUPPORTED, "X and a must be f32, f16 or bf16");
    const int64_t warps = n_heads * n_nodes;
    if (warps == 0) return ATT_OK;
    ATT_CHECK(X && a && scores, ATT_ERR_INVALID, "null pointer");
    k_node_scores<<<(unsigned)((warps * 32 + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
        X, x_dtype, n_heads, n_nodes, F, x_stride_h, x_stride_n, a, a_dtype, a_stride_h, scores,
        s_stride_h);
    return launch_status("k_node_scores");
}

extern "C" int att_node_scores_pair(const void *X, int x_dtype, int64_t n_heads, int64_t n_nodes,
                                    int64_t F, int64_t x_stride_h, int64_t x_stride_n,
                                    const float *a0, const float *a1, int64_t a_stride_h,
                                    float *s0, float *s1, int64_t s_stride_h, void *stream) {
    clear_error();
    ATT_CHECK(n_heads >= 0 && n_nodes >= 0 && F >= 0, ATT_ERR_INVALID, "negative size");
    const int64_t rows = n_heads * n_nodes;
    if (rows == 0) return ATT_OK;
    ATT_CHECK(X && a0 && a1 && s0 && s1, ATT_ERR_INVALID, "null pointer");
    const bool v16 = (x_dtype == ATT_F16 || x_dtype == ATT_BF16) &&
                     (F == 8 || F == 16 || F == 32 || F == 64 || F == 128 || F == 256) &&
                     x_stride_h % 8 == 0 && x_stride_n % 8 == 0 && ((uintptr_t)X & 15) == 0 &&
                     a_stride_h % 8 == 0 && ((uintptr_t)a0 & 15) == 0 && ((uintptr_t)a1 & 15) == 0;
    cudaStream_t st = (cudaStream_t)stream;
    if (!v16) {  // any layout: two passes of the generic kernel
        int s = att_node_scores(X, x_dtype, n_heads, n_nodes, F, x_stride_h, x_stride_n, a0,
                                ATT_F32, a_stride_h, s0, s_stride_h, stream);
        if (s != ATT_OK) return s;
        return att_node_scores(X, x_dtype, n_heads, n_nodes, F, x_stride_h, x_stride_n, a1,
                               ATT_F32, a_stride_h, s1, s_stride_h, stream);
    }
    const int lpr = (int)(F / 8);
    const int64_t warps = (rows * lpr + 31) / 32;
    const unsigned grid = (unsigned)((warps * 32 + 255) / 256);
#define ATT_NSP(T, L)                                                                           \
    k_node_scores_pair<T, L><<<grid, 256, 0, st>>>((const T *)X, n_heads, n_nodes, x_stride_h, \
                                                   x_stride_n, a0, a1, a_stride_h, s0, s1,     \
                                                   s_stride_h)
#define ATT_NSP_T(T)                                  \
    switch (lpr) {                                    \
        case 1: ATT_NSP(T, 1); break;                 \
        case 2: ATT_NSP(T, 2); break;                 \
        case 4: ATT_NSP(T, 4); break;                 \
        case 8: ATT_NSP(T, 8); break;                 \
        case 16: ATT_NSP(T, 16); break;               \
        default: ATT_NSP(T, 32); break;               \
    }
    if (x_dtype == ATT_F16) { ATT_NSP_T(__half) } else { ATT_NSP_T(__nv_bfloat16) }
#undef ATT_NSP_T
#undef ATT_NSP
    return launch_status("k_node_scores_pair");
}

extern "C" int att_slot_edges(const int32_t *rowptr, const int32_t *col, const int32_t *map,
                              const int32_t *window_of_part, int64_t n_parts, int window,
                              int wide, int mode, const float *s0, const float *s1,
                              int64_t s_stride_h, const void *g, int g_dtype, int64_t g_stride_h,
                              int64_t g_stride_n, int64_t n_nodes, int64_t n_heads, void *out,
                              int out_dtype, int64_t out_stride_h, int64_t out_stride_e,
                              void *stream) {
    clear_error();
    ATT_CHECK(window > 0 && wide > 0, ATT_ERR_INVALID, "bad window/wide");
    ATT_CHECK(mode == 0 || mode == 1, ATT_ERR_INVALID, "mode must be 0 (score) or 1 (row)");
    ATT_CHECK(mode == 1 || (s0 && s1), ATT_ERR_INVALID, "scores are null");
    ATT_CHECK(mode == 0 || g, ATT_ERR_INVALID, "row values are null");
    const int64_t warps = n_parts * n_heads;
    if (warps == 0) return ATT_OK;
    SlotEdgeArgs A{rowptr, col, map, window_of_part, n_parts, window, wide, mode, s0, s1,
                   s_stride_h, g, g_dtype, g_stride_h, g_stride_n, out, out_dtype, out_stride_h,
                   out_stride_e, n_heads, n_nodes};
    k_slot_edges<<<(unsigned)((warps * 32 + 255) / 256), 256, 0, (cudaStream_t)stream>>>(A);
    return launch_status("k_slot_edges");
}

extern "C" int att_sddmm(const int32_t *rowptr, const int32_t *col, const int32_t *map,
                         const int32_t *window_of_part, int64_t n_parts, int window, int wide,
                         const void *A, const void *B, int dtype, int64_t n_heads, int64_t F,
                         int64_t a_stride_h, int64_t a_stride_n, int64_t n_a,
                         int64_t b_stride_h, int64_t b_stride_n, int64_t n_b, void *out,
                         int out_dtype, int64_t out_stride_h, int64_t out_stride_e,
                         int32_t *err_flag, void *stream) {
    clear_error();
    ATT_CHECK(window == 8 || window == 16, ATT_ERR_UNSUPPORTED, "window must be 8 or 16");
    ATT_CHECK(wide == 4 || wide == 8 || wide == 16, ATT_ERR_UNSUPPORTED,
              "SDDMM needs wide 4, 8 or 16 (a 16-column step must span whole blocks)");
    ATT_CHECK(F > 0 && F <= 256, ATT_ERR_UNSUPPORTED, "SDDMM feature dim must be in [1, 256]");
    ATT_CHECK(out_dtype >= ATT_F32 && out_dtype <= ATT_BF16, ATT_ERR_INVALID, "bad out dtype");
    const int64_t items = n_parts * n_heads;
    if (items == 0) return ATT_OK;
    ATT_CHECK(rowptr && col && map && window_of_part && A && B && out, ATT_ERR_INVALID,
              "null pointer");
    SddmmArgs P{rowptr, col, map, window_of_part, n_parts, wide, A, a_stride_h, a_stride_n, n_a,
                B, b_stride_h, b_stride_n, n_b, F, n_heads, out, out_dtype, out_stride_h,
                out_stride_e, err_flag};
    cudaStream_t st = (cudaStream_t)stream;
    if (dtype == ATT_F16 || dtype == ATT_BF16) {
        ATT_CHECK(F % 8 == 0 && b_stride_n % 8 == 0 && b_stride_h % 8 == 0 &&
                      ((uintptr_t)B & 15) == 0 && a_stride_n % 2 == 0 && a_stride_h % 2 == 0 &&
                      ((uintptr_t)A & 3) == 0,
                  ATT_ERR_UNSUPPORTED,
                  "16-bit SDDMM needs F and the column strides multiples of 8 and 16-byte "
                  "aligned operands");
        if (dtype == ATT_F16) {
            if (window == 8) return dispatch_sddmm16<__half, 8>(P, st);
            return dispatch_sddmm16<__half, 16>(P, st);
        }
        if (window == 8) return dispatch_sddmm16<__nv_bfloat16, 8>(P, st);
        return dispatch_sddmm16<__nv_bfloat16, 16>(P, st);
    }
    if (dtype == ATT_F32) {
        ATT_CHECK(F % 4 == 0 && b_stride_n % 4 == 0 && b_stride_h % 4 == 0 &&
                      ((uintptr_t)B & 15) == 0 && F <= 128,
                  ATT_ERR_UNSUPPORTED,
                  "fp32 SDDMM needs F <= 128, F and the column strides multiples of 4, 16-byte "
                  "aligned columns");
        if (window == 8) return dispatch_sddmm32<8>(P, st);
        return dispatch_sddmm32<16>(P, st);
    }
    set_error("unsupported dtype %d", dtype);
    return ATT_ERR_UNSUPPORTED;
}

extern "C" int att_gather_slot_values(const int32_t *map, int64_t n_slots, int window,
                                      int map_wide, int out_wide, const void *vals, int v_dtype,
                                      int64_t v_stride_h, int64_t v_stride_e, int64_t n_heads,
                                      void *out, int out_dtype, int64_t out_stride_h,
                                      void *stream) {
    clear_error();
    ATT_CHECK(window > 0 && map_wide > 0 && out_wide > 0, ATT_ERR_INVALID, "bad layout");
    ATT_CHECK(n_slots % ((int64_t)window * (map_wide > out_wide ? map_wide : out_wide)) == 0,
              ATT_ERR_INVALID, "slot count is not a whole number of blocks");
    auto lg2 = [](int v) { int l = 0; while ((1 << l) < v) ++l; return (1 << l) == v ? l : -1; };
    const int lw = lg2(window), lmw = lg2(map_wide), low = lg2(out_wide);
    ATT_CHECK(lw >= 0 && lmw >= 0 && low >= 0, ATT_ERR_UNSUPPORTED,
              "window and block widths must be powers of two");
    ATT_CHECK(n_heads < 65536, ATT_ERR_UNSUPPORTED, "too many heads");
    if (n_slots == 0 || n_heads == 0) return ATT_OK;
    ATT_CHECK(map && vals && out, ATT_ERR_INVALID, "null pointer");
    const int64_t want = (n_slots + 255) / 256, cap = (int64_t)sm_count() * 16;
    const dim3 grid((unsigned)(want < cap ? want : cap), (unsigned)n_heads);
    k_gather_slots<<<grid, 256, 0, (cudaStream_t)stream>>>(map, n_slots, lw, lmw, low, vals,
                                                          v_dtype, v_stride_h, v_stride_e, out,
                                                          out_dtype, out_stride_h);
    return launch_status("k_gather_slots");
}

extern "C" int att_rowsum(const int32_t *rowptr, const int32_t *map,
                          const int32_t *window_of_part, const int32_t *atomic, int64_t n_parts,
                          int window, int wide, const void *vals, int v_dtype,
                          int64_t v_stride_h, int64_t v_stride_e, int64_t n_heads, float *out,
                          int64_t out_stride_h, int64_t out_stride_n, int64_t m_out,
                          void *stream) {
    clear_error();
    ATT_CHECK(window == 8 || window == 16, ATT_ERR_UNSUPPORTED, "window must be 8 or 16");
    ATT_CHECK(wide > 0, ATT_ERR_INVALID, "bad wide");
    cudaStream_t st = (cudaStream_t)stream;
    if (m_out == 0 || n_heads == 0) return ATT_OK;
    ATT_CHECK(out != nullptr, ATT_ERR_INVALID, "null output");
    const int64_t n_w = (m_out + window - 1) / window;
    k_zero_rows_heads<<<(unsigned)((n_w + 255) / 256), 256, 0, st>>>(
        window_of_part, atomic, n_parts, window, out, out_stride_h, out_stride_n, m_out, n_heads);
    int s = launch_status("k_zero_rows_heads");
    if (s != ATT_OK) return s;
    const int64_t warps = n_parts * n_heads;
    if (warps == 0) return ATT_OK;
    ATT_CHECK(rowptr && map && window_of_part && atomic && vals, ATT_ERR_INVALID, "null pointer");
    const unsigned grid = (unsigned)((warps * 32 + 255) / 256);
    if (window == 8)
        k_rowsum_slots<8><<<grid, 256, 0, st>>>(rowptr, map, window_of_part, atomic, n_parts, wide,
                                                vals, v_dtype, v_stride_h, v_stride_e, n_heads,
                                                out, out_stride_h, out_stride_n, m_out);
    else
        k_rowsum_slots<16><<<grid, 256, 0, st>>>(rowptr, map, window_of_part, atomic, n_parts,
                                                 wide, vals, v_dtype, v_stride_h, v_stride_e,
                                                 n_heads, out, out_stride_h, out_stride_n, m_out);
    return launch_status("k_rowsum_slots");
}

// ---------------------------------------------------------------------------
// Edge softmax over CSR rows (the unfused chain's softmax in one kernel)
// ---------------------------------------------------------------------------
namespace att {
namespace {

// One warp per (head, row): lanes stride the row's edges keeping an online
// (max, sum) pair, merged across the warp; a second sweep writes
// exp(e - max) / sum.  Optional LeakyReLU on the logits first.
__global__ void k_edge_softmax(const int32_t *__restrict__ rowptr, int64_t n_rows,
                               const float *__restrict__ logits, int64_t lsh, int64_t H,
                               float slope, int leaky, void *out, int odt, int64_t osh,
                               float *row_max, float *row_sum) {
    const int lane = threadIdx.x & 31;
    const int64_t wid = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (wid >= n_rows * H) return;
    const int64_t h = wid / n_rows, r = wid - h * n_rows;
    const int64_t b = rowptr[r], e = rowptr[r + 1];
    const float *L = logits + h * lsh;
    float m = -INFINITY, s = 0.f;
    for (int64_t i = b + lane; i < e; i += 32) {
        float x = L[i];
        if (leaky) x = x > 0.f ? x : slope * x;
        if (x > m) {
            s = s * __expf(m - x) + 1.f;
            m = x;
        } else {
            s += __expf(x - m);
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float m2 = __shfl_xor_sync(0xffffffffu, m, o);
        const float s2 = __shfl_xor_sync(0xffffffffu, s, o);
        const float mn = fmaxf(m, m2);
        s = (m == -INFINITY ? 0.f : s * __expf(m - mn)) + (m2 == -INFINITY ? 0.f : s2 * __expf(m2 - mn));
        m = mn;
    }
    const float inv = s > 0.f ? 1.f / s : 0.f;
    for (int64_t i = b + lane; i < e; i += 32) {
        float x = L[i];
        if (leaky) x = x > 0.f ? x : slope * x;
        st_any(out, odt, h * osh + i, __expf(x - m) * inv);
    }
    if (lane == 0) {
        if (row_max) row_max[h * n_rows + r] = m;
        if (row_sum) row_sum[h * n_rows + r] = s;
    }
}

}  // namespace
}  // namespace att

extern "C" int att_edge_softmax(const int32_t *rowptr, int64_t n_rows, const float *logits,
                                int64_t logit_stride_h, int64_t n_heads, float slope, int leaky,
                                void *out, int out_dtype, int64_t out_stride_h, float *row_max,
                                float *row_sum, void *stream) {
    using namespace att;
    clear_error();
    ATT_CHECK(n_rows >= 0 && n_heads > 0, ATT_ERR_INVALID, "bad sizes");
    ATT_CHECK(out_dtype == ATT_F32 || out_dtype == ATT_F16 || out_dtype == ATT_BF16,
              ATT_ERR_UNSUPPORTED, "edge softmax writes fp32, fp16 or bf16");
    if (n_rows == 0) return ATT_OK;
    ATT_CHECK(rowptr && logits && out, ATT_ERR_INVALID, "null pointer");
    const int64_t threads = n_rows * n_heads * 32;
    k_edge_softmax<<<(unsigned)((threads + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
        rowptr, n_rows, logits, logit_stride_h, n_heads, slope, leaky, out, out_dtype,
        out_stride_h, row_max, row_sum);
    return launch_status("k_edge_softmax");
}
