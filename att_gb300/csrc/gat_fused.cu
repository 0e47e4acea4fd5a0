// gat_fused.cu -- one-pass GAT attention layer on the row-window block format.
//
// Replaces the reference's chain of separate ops for a GAT layer
// (end2end_ori/gat_final/mgat_csr/mgat_conv.py:173-198: att/SDDMM ->
// LeakyReLU -> exp -> row sums -> SpMM -> divide, each a kernel with an
// nnz-sized intermediate) by one kernel that never materialises per-edge
// values.  Per 8-row window and 16 condensed columns at a time:
//
//   logits  mode 0 (dot):      S[c][r] = X'_c . X'_r  -- mma.sync m16n8k16, K = F
//           mode 1 (additive): S[c][r] = s0[r] + s1[c] -- GAT's a0/a1 scores
//   e = LeakyReLU(S) on occupied slots (per-slot bitmap), -inf elsewhere
//   online softmax: running row max m and sum l in fp32 registers, reduced
//     across the 8 lanes of a row with shuffles; the accumulator is rescaled
//     by exp(m_old - m_new) whenever the max grows
//   P = exp(e - m) -> fp16/bf16, transposed in registers (movmatrix) into the
//     B operand of acc[f][r] += X'^T[f][c] . P[c][r]  -- mma.sync m16n8k16
//
// X' rows of the 16 columns are gathered once per step (16-byte cp.async into
// a 4-stage per-warp ring, XOR-swizzled) and feed both products.
// A work item is a chunk of up to `parts_per_chunk` consecutive parts of one
// window; a window covered by one chunk is finalised in place (out = acc/l,
// plus the row max and sum for the backward pass); a window spread over
// several chunks writes (m, l, acc) partials that k_gat_combine merges.
#include "att_common.cuh"

#include <mutex>

namespace att {
namespace {

constexpr int kGWarps = 4;
constexpr int kGThreads = kGWarps * 32;
constexpr int kGStages = 3;
constexpr int kW = 8;  // window rows

__device__ __forceinline__ uint32_t movmatrix_trans(uint32_t x) {
    uint32_t y;
    asm volatile("movmatrix.sync.aligned.m8n8.trans.b16 %0, %1;\n" : "=r"(y) : "r"(x));
    return y;
}

template <typename T>
__device__ __forceinline__ float2 unpack2(uint32_t v);
template <>
__device__ __forceinline__ float2 unpack2<__half>(uint32_t v) {
    return __half22float2(*reinterpret_cast<__half2 *>(&v));
}
template <>
__device__ __forceinline__ float2 unpack2<__nv_bfloat16>(uint32_t v) {
    return __bfloat1622float2(*reinterpret_cast<__nv_bfloat162 *>(&v));
}

template <typename T>
__device__ __forceinline__ uint32_t pack2(float lo, float hi);
template <>
__device__ __forceinline__ uint32_t pack2<__half>(float lo, float hi) {
    __half2 h = __floats2half2_rn(lo, hi);
    return *reinterpret_cast<uint32_t *>(&h);
}
template <>
__device__ __forceinline__ uint32_t pack2<__nv_bfloat16>(float lo, float hi) {
    __nv_bfloat162 h = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t *>(&h);
}

__device__ __forceinline__ void cp_async8(uint32_t dst, const void *src, int src_bytes) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(dst), "l"(src),
                 "r"(src_bytes));
}
__device__ __forceinline__ void cp_async4(uint32_t dst, const void *src, int src_bytes) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(dst), "l"(src),
                 "r"(src_bytes));
}

struct GatArgs {
    const int32_t *rowptr, *col, *win;
    const uint32_t *mask;         // occupancy bit per slot
    const int32_t *chunk_begin;   // [n_chunks + 1] part ranges
    const int32_t *chunk_slot;    // [n_chunks] partial slot or -1 (whole window)
    int64_t n_chunks;
    int wide;
    const void *X;                // X' rows: X + node * ldx + head * F
    int64_t n_nodes, H, F, ldx;
    int mode;
    const float *s0, *s1;         // [H][n_nodes] node scores (mode 1)
    float slope;
    float *out;                   // [n_nodes, H*F] rows of ldo
    int64_t ldo;
    float *row_max, *row_sum;     // [H][n_nodes] or null
    float *partial;               // [n_partial][H][kW][F + 2]
    int32_t *err;
};

template <int F>
__device__ __forceinline__ int swz_row(int r) {
    if constexpr (F * 2 >= 128) return r & 7;
    else return (r >> 1) & 3;
}

template <typename T, int F, int MODE>
struct GCfg {
    static constexpr bool F32 = sizeof(T) == 4;  // fp32 X': 3xTF32 products
    static constexpr int XROW = F * (int)sizeof(T);
    static constexpr int XSTAGE = 16 * XROW;
    static constexpr int MSTAGE = 16;            // 128 occupancy bits
    static constexpr int SSTAGE = MODE == 1 ? 64 : 0;  // s1 of the 16 columns
    static constexpr int STAGE = XSTAGE + MSTAGE + SSTAGE;
    static constexpr int PTILE = F32 ? 16 * kW * 4 : 0;  // the step's P, re-read transposed
    static constexpr int WARP_SMEM = kGStages * STAGE + PTILE;
    static constexpr int SMEM = kGWarps * WARP_SMEM;
    static constexpr int CPR = XROW / 16;
    static constexpr int EPC = 16 / (int)sizeof(T);  // elements per 16-byte chunk
    static constexpr int PASSES = (16 * CPR + 31) / 32;
    static constexpr int MT = F / 16;
};

// XOR swizzle of 16-byte chunks by row, for rows of ROW_BYTES bytes
template <int ROW_BYTES>
__device__ __forceinline__ int swz_rb(int r) {
    if constexpr (ROW_BYTES >= 128) return r & 7;
    else return (r >> 1) & 3;
}


// PSPLIT: aggregate with P as a hi + lo pair of 16-bit values (fp32-accurate
// output); the training path needs it so that dout . out matches the
// backward's recomputed probabilities.
// IT: index type of items and element offsets (int32_t when every offset fits)
// fp32 X' with at most 64 features: registers bounded for 3 CTAs per SM
// (200 registers would leave room for 2), without spills
template <typename T, int F, int MODE, bool PSPLIT, typename IT>
__global__ void __launch_bounds__(kGThreads, (sizeof(T) == 4 && F <= 64) ? 3 : 1)
    k_gat_fused(GatArgs A) {
    using C = GCfg<T, F, MODE>;
    extern __shared__ __align__(128) unsigned char smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t sbase = smem_u32(smem) + warp * C::WARP_SMEM;
    const unsigned char *sgen = smem + warp * C::WARP_SMEM;
    const int gid = lane >> 2, tig = lane & 3;
    const IT n_items = (IT)(A.n_chunks * A.H);
    const IT stride = (IT)gridDim.x * kGWarps;
    const IT H = (IT)A.H, n_nodes = (IT)A.n_nodes, ldx = (IT)A.ldx, ldo = (IT)A.ldo;
    const T *X = (const T *)A.X;
    const float NEG_INF = -INFINITY;
    // logits may exceed a row's reference by this much before it moves
    constexpr float kLazy = 8.f;
    float *ptile = (float *)(smem + warp * C::WARP_SMEM + kGStages * C::STAGE);  // fp32 only
    (void)ptile;

    // ---- producer: (item, part, step) cursor ----
    IT p_item = (IT)blockIdx.x * kGWarps + warp;
    IT p_h = 0;
    int p_part = 0, p_part_end = 0, p_start = 0, p_nreal = 0, p_pend = 0, p_step = 0;
    int p_myc = -1;  // column ids of the producer's position, fetched one step ahead
    auto p_set_part = [&]() {  // returns with p_part < p_part_end and a non-empty part, or exhausted
        while (true) {
            while (p_part < p_part_end) {
                p_start = A.rowptr[2 * p_part];
                const int e = A.rowptr[2 * p_part + 1];
                p_pend = A.rowptr[2 * p_part + 2];
                p_nreal = e > p_start ? e - p_start : 0;
                if ((p_start % A.wide) != 0 || (p_pend % A.wide) != 0 || p_pend < p_start + p_nreal) {
                    if (A.err) atomicOr(A.err, 2);
                    p_nreal = 0;
                }
                p_step = 0;
                if (p_nreal > 0) return;
                ++p_part;
            }
            p_item += stride;
            if (p_item >= n_items) return;
            const IT ch = p_item / H;
            p_h = p_item - ch * H;
            p_part = A.chunk_begin[ch];
            p_part_end = A.chunk_begin[ch + 1];
        }
    };
    auto p_begin = [&]() {
        if (p_item < n_items) {
            const IT ch = p_item / H;
            p_h = p_item - ch * H;
            p_part = A.chunk_begin[ch];
            p_part_end = A.chunk_begin[ch + 1];
            p_set_part();
        }
    };
    auto issue = [&](int stage) {
        const uint32_t xs = sbase + stage * C::STAGE;
        const uint32_t ms = xs + C::XSTAGE;
        const uint32_t ss = ms + C::MSTAGE;
        const int c0 = p_step * 16;
        int myc = p_myc;
        if ((uint64_t)(int64_t)(myc + 1) > (uint64_t)n_nodes) {  // valid: -1 .. n_nodes - 1
            if (A.err) atomicOr(A.err, 1);
            myc = -1;
        }
#pragma unroll
        for (int i = 0; i < C::PASSES; ++i) {
            const int idx = i * 32 + lane;
            const int r = idx / C::CPR, ch = idx % C::CPR;
            const int cidx = __shfl_sync(0xffffffffu, myc, r & 15);
            if (idx < 16 * C::CPR) {
                const bool ok = cidx >= 0;
                const IT off = ok ? (IT)cidx * ldx + p_h * F + ch * C::EPC : (IT)0;
                cp_async16(xs + r * C::XROW + ((ch ^ swz_rb<C::XROW>(r)) << 4), X + off, ok ? 16 : 0);
            }
        }
        // occupancy bits of the step's 16 x 8 slots, one 8-byte piece per
        // 8-column half (a half past the part's padded end is zero-filled)
        if (lane < 2) {
            const bool ok = c0 + 8 * lane < p_pend - p_start;
            const int64_t bit0 = (int64_t)(p_start + c0 + 8 * lane) * kW;  // bit index: 64-bit always
            const uint32_t *src = ok ? A.mask + (bit0 >> 5) : A.mask;
            cp_async8(ms + 8 * lane, src, ok ? 8 : 0);
        }
        if constexpr (MODE == 1) {
            if (lane < 16) {
                const int c = __shfl_sync(0x0000ffffu, myc, lane);
                const bool ok = c >= 0;
                cp_async4(ss + 4 * lane, ok ? (const void *)(A.s1 + (p_h * n_nodes + c))
                                            : (const void *)A.s1,
                          ok ? 4 : 0);
            }
        } else {
            (void)ss;
        }
    };
    auto p_fetch = [&]() {
        p_myc = -1;
        if (p_item < n_items && p_step * 16 + (lane & 15) < p_nreal)
            p_myc = A.col[p_start + p_step * 16 + (lane & 15)];
    };
    auto p_advance = [&]() {
        if (++p_step * 16 >= p_nreal) {
            ++p_part;
            p_set_part();
        }
        p_fetch();
    };

    p_begin();
    p_fetch();
#pragma unroll
    for (int s = 0; s < kGStages - 1; ++s) {
        if (p_item < n_items) {
            issue(s);
            p_advance();
        }
        cp_async_commit();
    }

    // occupancy-bit positions of this lane's four (column, row) slots within
    // a step's 16 x 8 block run: fixed per lane (wide is a power of two)
    const int wmask = A.wide - 1;
    int mbit[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        const int c = gid + 8 * (u >> 1), r = 2 * tig + (u & 1);
        mbit[u] = (c & ~wmask) * kW + r * A.wide + (c & wmask);
    }
    int cstage = 0, pstage = kGStages - 1;
    for (IT c_item = (IT)blockIdx.x * kGWarps + warp; c_item < n_items; c_item += stride) {
        const IT chunk = c_item / H;
        const IT h = c_item - chunk * H;
        const int part0 = A.chunk_begin[chunk], part1 = A.chunk_begin[chunk + 1];
        if (part1 <= part0) continue;
        const IT wrow = (IT)A.win[part0] * kW;
        // query side of the window: B fragments (mode 0) or row scores (mode 1);
        // fp32: the B values of every 8-feature k-step, split at use
        uint32_t bq[C::MT][2];
        float bqf[C::F32 ? F / 8 : 1][2];
        float s0r[2] = {0.f, 0.f};
        if constexpr (MODE == 0 && !C::F32) {
#pragma unroll
            for (int kk = 0; kk < C::MT; ++kk)
#pragma unroll
                for (int u = 0; u < 2; ++u) {
                    const IT row = wrow + gid;
                    const int f = 16 * kk + 2 * tig + 8 * u;
                    bq[kk][u] = row < n_nodes ? *(const uint32_t *)(X + (row * ldx + h * F + f)) : 0u;
                }
        } else if constexpr (MODE == 0) {
#pragma unroll
            for (int kk = 0; kk < F / 8; ++kk)
#pragma unroll
                for (int u = 0; u < 2; ++u) {
                    const IT row = wrow + gid;
                    const int f = 8 * kk + tig + 4 * u;
                    bqf[kk][u] = row < n_nodes ? (float)X[row * ldx + h * F + f] : 0.f;
                }
        } else {
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                const IT row = wrow + 2 * tig + u;
                s0r[u] = row < n_nodes ? A.s0[h * n_nodes + row] : 0.f;
            }
        }
        float m_run[2] = {NEG_INF, NEG_INF}, l_run[2] = {0.f, 0.f};
        float acc[C::MT][4];
#pragma unroll
        for (int j = 0; j < C::MT; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;

        for (int part = part0; part < part1; ++part) {
            const int start = A.rowptr[2 * part];
            const int e = A.rowptr[2 * part + 1];
            const int pend = A.rowptr[2 * part + 2];
            int nreal = e > start ? e - start : 0;
            if ((start & wmask) != 0 || (pend & wmask) != 0 || pend < start + nreal) nreal = 0;
            const int nsteps = (nreal + 15) >> 4;
            for (int step = 0; step < nsteps; ++step) {
                cp_async_wait<kGStages - 2>();
                __syncwarp();
                const uint32_t xs = sbase + cstage * C::STAGE;
                const uint32_t *mw = (const uint32_t *)(sgen + cstage * C::STAGE + C::XSTAGE);
                // logits S[col][row]: this lane holds cols (gid, gid+8) x rows (2tig, 2tig+1)
                float sv[4];
                if constexpr (MODE == 0 && !C::F32) {
                    sv[0] = sv[1] = sv[2] = sv[3] = 0.f;
#pragma unroll
                    for (int kk = 0; kk < C::MT; ++kk) {
                        const int q = lane >> 3, rr = lane & 7;
                        const int mrow = (q & 1) * 8 + rr;
                        const int ch = 2 * kk + (q >> 1);
                        uint32_t a[4];
                        ldsm_x4(xs + mrow * C::XROW + ((ch ^ swz_rb<C::XROW>(mrow)) << 4), a[0], a[1],
                                a[2], a[3]);
                        mma_16816<T>(sv, a, bq[kk][0], bq[kk][1]);
                    }
                } else if constexpr (MODE == 0) {
                    // 8 features per k-step; ldmatrix of 16-byte rows hands each
                    // lane the fp32 element (row gid, feature tig) of every 8 x 4
                    // matrix: the m16n8k8 A fragment.  3xTF32: lo.hi + hi.lo + hi.hi
                    sv[0] = sv[1] = sv[2] = sv[3] = 0.f;
#pragma unroll
                    for (int kk = 0; kk < F / 8; ++kk) {
                        const int q = lane >> 3, rr = lane & 7;
                        const int mrow = (q & 1) * 8 + rr;
                        const int ch = 2 * kk + (q >> 1);
                        uint32_t a[4], ah[4], al[4], bh[2], bl[2];
                        ldsm_x4(xs + mrow * C::XROW + ((ch ^ swz_rb<C::XROW>(mrow)) << 4), a[0], a[1],
                                a[2], a[3]);
#pragma unroll
                        for (int u = 0; u < 4; ++u) split_tf32x3(__uint_as_float(a[u]), ah[u], al[u]);
                        split_tf32x3(bqf[kk][0], bh[0], bl[0]);
                        split_tf32x3(bqf[kk][1], bh[1], bl[1]);
                        mma_1688_tf32(sv, al[0], al[1], al[2], al[3], bh[0], bh[1]);
                        mma_1688_tf32(sv, ah[0], ah[1], ah[2], ah[3], bl[0], bl[1]);
                        mma_1688_tf32(sv, ah[0], ah[1], ah[2], ah[3], bh[0], bh[1]);
                    }
                } else {
                    const float *s1s = (const float *)(sgen + cstage * C::STAGE + C::XSTAGE + C::MSTAGE);
                    const float c_lo = s1s[gid], c_hi = s1s[gid + 8];
                    sv[0] = s0r[0] + c_lo;
                    sv[1] = s0r[1] + c_lo;
                    sv[2] = s0r[0] + c_hi;
                    sv[3] = s0r[1] + c_hi;
                }
                // LeakyReLU on occupied slots, -inf on empty ones
                const int c0 = step * 16;
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int c = gid + 8 * (u >> 1);
                    const bool occ = c0 + c < nreal && ((mw[mbit[u] >> 5] >> (mbit[u] & 31)) & 1u);
                    const float x = sv[u];
                    sv[u] = occ ? (x > 0.f ? x : A.slope * x) : NEG_INF;
                }
                // online softmax, rows 2tig (u even) and 2tig+1 (u odd), with
                // lazy rescaling: a row's reference m_run moves (max over the
                // row's lanes, accumulators and partial sums rescaled) only on
                // its first occupied slot or when a logit exceeds it by more
                // than kLazy, so most steps run no reduction at all; the
                // probabilities stay below e^kLazy, well inside the 16-bit P
                // range.  Each lane sums its own columns' probabilities
                // (l_run holds that partial until the end of the item).
                const bool up = sv[0] > m_run[0] + kLazy || sv[2] > m_run[0] + kLazy ||
                                sv[1] > m_run[1] + kLazy || sv[3] > m_run[1] + kLazy;
                if (__any_sync(0xffffffffu, up)) {
                    float mx[2] = {fmaxf(sv[0], sv[2]), fmaxf(sv[1], sv[3])};
#pragma unroll
                    for (int o = 4; o < 32; o <<= 1) {
                        mx[0] = fmaxf(mx[0], __shfl_xor_sync(0xffffffffu, mx[0], o));
                        mx[1] = fmaxf(mx[1], __shfl_xor_sync(0xffffffffu, mx[1], o));
                    }
                    float alpha[2];
#pragma unroll
                    for (int u = 0; u < 2; ++u) {
                        const float mn = fmaxf(m_run[u], mx[u]);
                        alpha[u] = mn == NEG_INF ? 1.f : __expf(m_run[u] - mn);
                        l_run[u] *= alpha[u];
                        m_run[u] = mn;
                    }
#pragma unroll
                    for (int j = 0; j < C::MT; ++j) {
                        acc[j][0] *= alpha[0];
                        acc[j][1] *= alpha[1];
                        acc[j][2] *= alpha[0];
                        acc[j][3] *= alpha[1];
                    }
                }
                const float mref[2] = {m_run[0] == NEG_INF ? 0.f : m_run[0],
                                       m_run[1] == NEG_INF ? 0.f : m_run[1]};
                float p[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) p[u] = __expf(sv[u] - mref[u & 1]);
                l_run[0] += p[0] + p[2];
                l_run[1] += p[1] + p[3];
                if constexpr (!C::F32) {
                    // P^T into B fragments: (col gid, rows 2tig..) -> (row gid, cols 2tig..)
                    const uint32_t h01 = pack2<T>(p[0], p[1]), h23 = pack2<T>(p[2], p[3]);
                    const uint32_t b0 = movmatrix_trans(h01);
                    const uint32_t b1 = movmatrix_trans(h23);
                    uint32_t bl0 = 0, bl1 = 0;
                    if constexpr (PSPLIT) {
                        const float2 r01 = unpack2<T>(h01), r23 = unpack2<T>(h23);
                        bl0 = movmatrix_trans(pack2<T>(p[0] - r01.x, p[1] - r01.y));
                        bl1 = movmatrix_trans(pack2<T>(p[2] - r23.x, p[3] - r23.y));
                    }
#pragma unroll
                    for (int j = 0; j < C::MT; ++j) {
                        const int q = lane >> 3, rr = lane & 7;
                        const int k = (q >> 1) * 8 + rr;
                        const int ch = 2 * j + (q & 1);
                        uint32_t a[4];
                        ldsm_x4_trans(xs + k * C::XROW + ((ch ^ swz_rb<C::XROW>(k)) << 4), a[0], a[1],
                                      a[2], a[3]);
                        mma_16816<T>(acc[j], a, b0, b1);
                        if constexpr (PSPLIT) mma_16816<T>(acc[j], a, bl0, bl1);
                    }
                } else {
                    // P through shared memory: written as (col, row), read back as the
                    // m16n8k8 B fragment (col tig (+4), row gid) of each 8-column k-step
#pragma unroll
                    for (int u = 0; u < 4; ++u)
                        ptile[(gid + 8 * (u >> 1)) * kW + 2 * tig + (u & 1)] = p[u];
                    __syncwarp();
                    uint32_t ph[2][2], pl[2][2];
#pragma unroll
                    for (int ks = 0; ks < 2; ++ks) {
                        split_tf32x3(ptile[(8 * ks + tig) * kW + gid], ph[ks][0], pl[ks][0]);
                        split_tf32x3(ptile[(8 * ks + tig + 4) * kW + gid], ph[ks][1], pl[ks][1]);
                    }
                    const float *xt = (const float *)(sgen + cstage * C::STAGE);
#pragma unroll
                    for (int j = 0; j < C::MT; ++j) {
#pragma unroll
                        for (int ks = 0; ks < 2; ++ks) {
                            // A = X'^T: (feature 16j + gid (+8), column 8ks + tig (+4))
                            uint32_t ah[4], al[4];
#pragma unroll
                            for (int u = 0; u < 4; ++u) {
                                const int c = 8 * ks + tig + 4 * (u >> 1);
                                const int f = 16 * j + gid + 8 * (u & 1);
                                const float x = xt[c * F + (((f >> 2) ^ swz_rb<C::XROW>(c)) << 2) + (f & 3)];
                                split_tf32x3(x, ah[u], al[u]);
                            }
                            mma_1688_tf32(acc[j], al[0], al[1], al[2], al[3], ph[ks][0], ph[ks][1]);
                            mma_1688_tf32(acc[j], ah[0], ah[1], ah[2], ah[3], pl[ks][0], pl[ks][1]);
                            mma_1688_tf32(acc[j], ah[0], ah[1], ah[2], ah[3], ph[ks][0], ph[ks][1]);
                        }
                    }
                }
                __syncwarp();
                if (p_item < n_items) {
                    issue(pstage);
                    p_advance();
                }
                cp_async_commit();
                cstage = cstage + 1 == kGStages ? 0 : cstage + 1;
                pstage = pstage + 1 == kGStages ? 0 : pstage + 1;
            }
        }
        // row sums: the lanes' partial sums over their own columns
#pragma unroll
        for (int o = 4; o < 32; o <<= 1) {
            l_run[0] += __shfl_xor_sync(0xffffffffu, l_run[0], o);
            l_run[1] += __shfl_xor_sync(0xffffffffu, l_run[1], o);
        }
        // ---- epilogue: acc[j] = (feature 16j+gid (+8), rows 2tig, 2tig+1) ----
        const int slot = A.chunk_slot[chunk];
        if (slot < 0) {
            float inv[2] = {l_run[0] > 0.f ? 1.f / l_run[0] : 0.f, l_run[1] > 0.f ? 1.f / l_run[1] : 0.f};
#pragma unroll
            for (int j = 0; j < C::MT; ++j)
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const IT row = wrow + 2 * tig + (u & 1);
                    const int f = 16 * j + gid + 8 * (u >> 1);
                    if (row < n_nodes) A.out[row * ldo + h * F + f] = acc[j][u] * inv[u & 1];
                }
            if (gid == 0) {
#pragma unroll
                for (int u = 0; u < 2; ++u) {
                    const IT row = wrow + 2 * tig + u;
                    if (row < n_nodes) {
                        if (A.row_max) A.row_max[h * n_nodes + row] = m_run[u];
                        if (A.row_sum) A.row_sum[h * n_nodes + row] = l_run[u];
                    }
                }
            }
        } else {
            float *pp = A.partial + ((IT)slot * H + h) * kW * (F + 2);
#pragma unroll
            for (int j = 0; j < C::MT; ++j)
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int r = 2 * tig + (u & 1);
                    const int f = 16 * j + gid + 8 * (u >> 1);
                    pp[r * (F + 2) + f] = acc[j][u];
                }
            if (gid == 0) {
#pragma unroll
                for (int u = 0; u < 2; ++u) {
                    const int r = 2 * tig + u;
                    pp[r * (F + 2) + F] = m_run[u];
                    pp[r * (F + 2) + F + 1] = l_run[u];
                }
            }
        }
    }
    cp_async_wait<0>();
}

// Merge the partials of windows spread over several chunks: one block per
// (window, head), one warp per window row; the window's chunks are
// [multi[2i], multi[2i+1]).  Row max and sum are reduced across the chunks
// lane-parallel, then each lane merges its features over the chunks.
__global__ void __launch_bounds__(kW * 32) k_gat_combine(
    const int32_t *__restrict__ multi_chunk_begin, const int32_t *__restrict__ chunk_slot,
    const int32_t *__restrict__ chunk_begin, const int32_t *__restrict__ win, int64_t n_multi,
    int64_t H, int64_t F, int64_t n_nodes, const float *__restrict__ partial,
    float *__restrict__ out, int64_t ldo, float *row_max, float *row_sum) {
    const int lane = threadIdx.x & 31, r = threadIdx.x >> 5;
    const int64_t wid = blockIdx.x;
    if (wid >= n_multi * H) return;
    const int64_t mwin = wid / H, h = wid - mwin * H;
    const int cb = multi_chunk_begin[2 * mwin], ce = multi_chunk_begin[2 * mwin + 1];
    const int64_t row = (int64_t)win[chunk_begin[cb]] * kW + r;
    if (row >= n_nodes) return;
    const int64_t pitch = kW * (F + 2);
    auto part_row = [&](int c) {
        return partial + ((int64_t)chunk_slot[c] * H + h) * pitch + r * (F + 2);
    };
    float m = -INFINITY;
    for (int c = cb + lane; c < ce; c += 32) m = fmaxf(m, part_row(c)[F]);
    m = warp_max(m);
    const float mref = m == -INFINITY ? 0.f : m;
    float l = 0.f;
    for (int c = cb + lane; c < ce; c += 32) {
        const float *pp = part_row(c);
        l += __expf(pp[F] - mref) * pp[F + 1];
    }
    l = warp_sum(l);
    const float inv = l > 0.f ? 1.f / l : 0.f;
    for (int64_t f = lane; f < F; f += 32) {
        float a = 0.f;
        for (int c = cb; c < ce; ++c) {
            const float *pp = part_row(c);
            a += __expf(pp[F] - mref) * pp[f];
        }
        out[row * ldo + h * F + f] = a * inv;
    }
    if (lane == 0) {
        if (row_max) row_max[h * n_nodes + row] = m;
        if (row_sum) row_sum[h * n_nodes + row] = l;
    }
}

// rows of windows that own no part (and rows past the last window): zero
__global__ void k_gat_zero_rows(const int32_t *__restrict__ win, int64_t n_parts, int64_t n_nodes,
                                int64_t H, int64_t F, float *out, int64_t ldo, float *row_max,
                                float *row_sum) {
    const int lane = threadIdx.x & 31;
    const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t n_w = (n_nodes + kW - 1) / kW;
    if (w >= n_w) return;
    int64_t lo = 0, hi = n_parts;
    while (lo < hi) {
        int64_t mid = (lo + hi) >> 1;
        if (win[mid] < w) lo = mid + 1; else hi = mid;
    }
    if (lo < n_parts && win[lo] == w) return;
    for (int64_t r = w * kW; r < (w + 1) * kW && r < n_nodes; ++r) {
        for (int64_t f = lane; f < H * F; f += 32) out[r * ldo + f] = 0.f;
        if (lane < H) {
            if (row_max) row_max[lane * n_nodes + r] = -INFINITY;
            if (row_sum) row_sum[lane * n_nodes + r] = 0.f;
        }
    }
}

// occupancy bitmap from the per-edge slot index
__global__ void k_slot_mask(const int32_t *__restrict__ edge_slot, int64_t nnz, uint32_t *mask) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nnz) return;
    const int32_t s = edge_slot[e];
    if (s >= 0) atomicOr(mask + (s >> 5), 1u << (s & 31));
}

template <typename T, int F, int MODE, bool PSPLIT>
int run_gat(const GatArgs &P, cudaStream_t st, int64_t n_partial) {
    using C = GCfg<T, F, MODE>;
    const int64_t items = P.n_chunks * P.H;
    if (items == 0) return ATT_OK;
    // 32-bit offsets when X', the output, the statistics, the partials and
    // the items all stay below 2^31 elements
    const int64_t lim = INT32_MAX - (1 << 22);
    const bool small = P.n_nodes * P.ldx < lim && P.n_nodes * P.ldo < lim &&
                       P.H * P.n_nodes < lim && n_partial * P.H * kW * (P.F + 2) < lim &&
                       items < lim;
    auto run = [&](auto kernel) {
        static std::once_flag once;
        static int prep = ATT_OK;
        std::call_once(once, [&] {
            prep = cuda_status(
                cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM),
                "cudaFuncSetAttribute");
        });
        if (prep != ATT_OK) return prep;
        int per_sm = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kGThreads, C::SMEM);
        if (per_sm < 1) per_sm = 1;
        const int64_t want = (items + kGWarps - 1) / kGWarps;
        const int64_t cap = (int64_t)sm_count() * per_sm;
        kernel<<<(unsigned)(want < cap ? want : cap), kGThreads, C::SMEM, st>>>(P);
        return launch_status("k_gat_fused");
    };
    if (small) return run(k_gat_fused<T, F, MODE, PSPLIT, int32_t>);
    return run(k_gat_fused<T, F, MODE, PSPLIT, int64_t>);
}

template <typename T, int MODE>
int dispatch_gat_f(const GatArgs &P, cudaStream_t st, int64_t np) {
    // statistics requested: training path (16-bit P as hi + lo); fp32 X'
    // always runs 3xTF32 products
    const bool split = P.row_sum != nullptr && sizeof(T) == 2;
    if constexpr (sizeof(T) == 4) {
        switch (P.F) {
            case 32: return run_gat<T, 32, MODE, false>(P, st, np);
            case 64: return run_gat<T, 64, MODE, false>(P, st, np);
            case 128: return run_gat<T, 128, MODE, false>(P, st, np);
            default:
                set_error("fused GAT supports F in {32, 64, 128}, got %lld", (long long)P.F);
                return ATT_ERR_UNSUPPORTED;
        }
    } else {
        switch (P.F) {
            case 32: return split ? run_gat<T, 32, MODE, true>(P, st, np) : run_gat<T, 32, MODE, false>(P, st, np);
            case 64: return split ? run_gat<T, 64, MODE, true>(P, st, np) : run_gat<T, 64, MODE, false>(P, st, np);
            case 128: return split ? run_gat<T, 128, MODE, true>(P, st, np) : run_gat<T, 128, MODE, false>(P, st, np);
            default:
                set_error("fused GAT supports F in {32, 64, 128}, got %lld", (long long)P.F);
                return ATT_ERR_UNSUPPORTED;
        }
    }
}

// ---------------------------------------------------------------------------
// Backward of the additive GAT layer, fused.  With the forward's row max m and
// sum l saved, and c_i = dout_i . out_i, every edge term is local:
//   p_ij  = exp(LeakyReLU(s0_i + s1_j) - m_i) / l_i
//   dp_ij = dout_i . X'_j
//   dz_ij = p_ij (dp_ij - c_i) LeakyReLU'(s0_i + s1_j)
//   dX'_j += p_ij dout_i      (the SpMM adjoint)
//   ds1_j += dz_ij,  ds0_i += dz_ij
// One pass over the block format of the TRANSPOSED graph: window rows are the
// j's, condensed columns the i's.  Per 16 columns: the dout rows of the i's
// are gathered (cp.async ring) and feed dp (mma, K = F) and the adjoint
// product (mma after a movmatrix transpose of p); ds1 is a register row sum,
// ds0 one atomic add per (window, column).  All outputs are accumulated with
// red.global.add into zeroed buffers.
struct GatBwdArgs {
    const int32_t *rowptr, *col, *win;
    const uint32_t *mask;
    int64_t n_parts;
    int wide;
    const void *Xp;    // X'[j][h*F + f]  (rows of the transposed windows)
    const void *dout;     // dout[i][h*F + f] (gathered)
    const void *dout_lo;  // dout - dout (rounded), same layout, or null
    int64_t n_nodes, H, F, ldx, ldd;
    const float *s0, *s1, *m, *l, *c;  // [H][n_nodes]
    float slope;
    float *dXp;  // [n_nodes][H*F] fp32, ld ldg
    int64_t ldg;
    float *ds0, *ds1;  // [H][n_nodes]
    int32_t *err;
};

// the backward's ring depth: 2 stages leave room for 6 CTAs per SM where 3
// stages allowed 4 (the kernel is latency-bound: warps matter more than depth)
constexpr int kBStages = 2;

template <typename T, int F, bool SPLIT>
struct BCfg {
    static constexpr int XROW = F * 2;
    static constexpr int TILE = 16 * XROW;
    static constexpr int XSTAGE = (SPLIT ? 2 : 1) * TILE;
    static constexpr int MSTAGE = 16;
    static constexpr int CSTAGE = 5 * 64;  // s0, m, l, c and the ids of the 16 columns
    static constexpr int STAGE = XSTAGE + MSTAGE + CSTAGE;
    static constexpr int WARP_SMEM = kBStages * STAGE;
    static constexpr int SMEM = kGWarps * WARP_SMEM;
    static constexpr int CPR = XROW / 16;
    static constexpr int PASSES = (16 * CPR + 31) / 32;
    static constexpr int MT = F / 16;
};

// IT: index type of items and element offsets (int32_t when every offset fits)
template <typename T, int F, bool SPLIT, typename IT>
__global__ void __launch_bounds__(kGThreads) k_gat_backward(GatBwdArgs A) {
    using C = BCfg<T, F, SPLIT>;
    const IT H = (IT)A.H, n_nodes = (IT)A.n_nodes, ldd = (IT)A.ldd, ldx = (IT)A.ldx,
             ldg = (IT)A.ldg;
    extern __shared__ __align__(128) unsigned char smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t sbase = smem_u32(smem) + warp * C::WARP_SMEM;
    const unsigned char *sgen = smem + warp * C::WARP_SMEM;
    const int gid = lane >> 2, tig = lane & 3;
    const IT n_items = (IT)(A.n_parts * A.H);
    const IT stride = (IT)gridDim.x * kGWarps;
    const T *Xq = (const T *)A.Xp;
    const T *D = (const T *)A.dout;
    const T *DL = (const T *)A.dout_lo;

    IT p_item = (IT)blockIdx.x * kGWarps + warp;
    IT p_h = 0;
    int p_start = 0, p_nreal = 0, p_pend = 0, p_step = 0, p_myc = -1;
    auto p_load = [&]() {
        while (p_item < n_items) {
            const IT part = p_item / H;
            p_h = p_item - part * H;
            p_start = A.rowptr[2 * part];
            const int e = A.rowptr[2 * part + 1];
            p_pend = A.rowptr[2 * part + 2];
            p_nreal = e > p_start ? e - p_start : 0;
            if ((p_start % A.wide) != 0 || (p_pend % A.wide) != 0 || p_pend < p_start + p_nreal) {
                if (A.err) atomicOr(A.err, 2);
                p_nreal = 0;
            }
            p_step = 0;
            if (p_nreal > 0) return;
            p_item += stride;
        }
    };
    auto issue = [&](int stage) {
        const uint32_t xs = sbase + stage * C::STAGE;
        const uint32_t ms = xs + C::XSTAGE;
        const uint32_t cs = ms + C::MSTAGE;
        const int c0 = p_step * 16;
        int myc = p_myc;  // fetched one step ahead
        if (myc >= n_nodes || myc < -1) {
            if (A.err) atomicOr(A.err, 1);
            myc = -1;
        }
#pragma unroll
        for (int i = 0; i < C::PASSES; ++i) {
            const int idx = i * 32 + lane;
            const int r = idx / C::CPR, ch = idx % C::CPR;
            const int cidx = __shfl_sync(0xffffffffu, myc, r & 15);
            if (idx < 16 * C::CPR) {
                const bool ok = cidx >= 0;
                const IT o = (IT)cidx * ldd + p_h * F + ch * 8;
                const uint32_t d = r * C::XROW + ((ch ^ swz_row<F>(r)) << 4);
                cp_async16(xs + d, ok ? D + o : D, ok ? 16 : 0);
                if constexpr (SPLIT) cp_async16(xs + C::TILE + d, ok ? DL + o : DL, ok ? 16 : 0);
            }
        }
        if (lane < 2) {
            const bool ok = c0 + 8 * lane < p_pend - p_start;
            const int64_t bit0 = (int64_t)(p_start + c0 + 8 * lane) * kW;  // bit index: 64-bit always
            cp_async8(ms + 8 * lane, ok ? (const void *)(A.mask + (bit0 >> 5)) : (const void *)A.mask,
                      ok ? 8 : 0);
        }
        if (lane < 16) {
            const bool ok = myc >= 0;
            const IT o = p_h * n_nodes + (ok ? myc : 0);
            const float *arrs[4] = {A.s0, A.m, A.l, A.c};
#pragma unroll
            for (int a = 0; a < 4; ++a)
                cp_async4(cs + a * 64 + 4 * lane, arrs[a] + o, ok ? 4 : 0);
            // the column ids themselves, for the ds0 scatter (-1: none)
            asm volatile("st.shared.u32 [%0], %1;\n" ::"r"(cs + 4 * 64 + 4 * lane), "r"(myc)
                         : "memory");
        }
    };
    auto p_fetch = [&]() {
        p_myc = -1;
        if (p_item < n_items && p_step * 16 + (lane & 15) < p_nreal)
            p_myc = A.col[p_start + p_step * 16 + (lane & 15)];
    };
    auto p_advance = [&]() {
        if (++p_step * 16 >= p_nreal) {
            p_item += stride;
            p_load();
        }
        p_fetch();
    };

    p_load();
    p_fetch();
#pragma unroll
    for (int s = 0; s < kBStages - 1; ++s) {
        if (p_item < n_items) {
            issue(s);
            p_advance();
        }
        cp_async_commit();
    }

    const int wmask = A.wide - 1;  // wide is a power of two
    int mbit[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        const int c = gid + 8 * (u >> 1), r = 2 * tig + (u & 1);
        mbit[u] = (c & ~wmask) * kW + r * A.wide + (c & wmask);
    }
    int cstage = 0, pstage = kBStages - 1;
    for (IT c_item = (IT)blockIdx.x * kGWarps + warp; c_item < n_items; c_item += stride) {
        const IT part = c_item / H;
        const IT h = c_item - part * H;
        const int start = A.rowptr[2 * part];
        const int e = A.rowptr[2 * part + 1];
        const int pend = A.rowptr[2 * part + 2];
        int nreal = e > start ? e - start : 0;
        if ((start & wmask) != 0 || (pend & wmask) != 0 || pend < start + nreal) nreal = 0;
        const int nsteps = (nreal + 15) >> 4;
        if (nsteps == 0) continue;
        const IT wrow = (IT)A.win[part] * kW;
        uint32_t bq[C::MT][2];
#pragma unroll
        for (int kk = 0; kk < C::MT; ++kk)
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                const IT row = wrow + gid;
                const int f = 16 * kk + 2 * tig + 8 * u;
                bq[kk][u] = row < n_nodes ? *(const uint32_t *)(Xq + row * ldx + h * F + f) : 0u;
            }
        float s1r[2];
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            const IT row = wrow + 2 * tig + u;
            s1r[u] = row < n_nodes ? A.s1[h * n_nodes + row] : 0.f;
        }
        float ds1_acc[2] = {0.f, 0.f};
        float acc[C::MT][4];
#pragma unroll
        for (int j = 0; j < C::MT; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;

        for (int step = 0; step < nsteps; ++step) {
            cp_async_wait<kBStages - 2>();
            __syncwarp();
            const uint32_t xs = sbase + cstage * C::STAGE;
            const uint32_t *mw = (const uint32_t *)(sgen + cstage * C::STAGE + C::XSTAGE);
            const float *cv = (const float *)(sgen + cstage * C::STAGE + C::XSTAGE + C::MSTAGE);
            // dp[c][r] = dout_c . X'_r
            float dp[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
            for (int kk = 0; kk < C::MT; ++kk) {
                const int q = lane >> 3, rr = lane & 7;
                const int mrow = (q & 1) * 8 + rr;
                const int ch = 2 * kk + (q >> 1);
                const uint32_t ad = mrow * C::XROW + ((ch ^ swz_row<F>(mrow)) << 4);
                uint32_t a[4];
                ldsm_x4(xs + ad, a[0], a[1], a[2], a[3]);
                mma_16816<T>(dp, a, bq[kk][0], bq[kk][1]);
                if constexpr (SPLIT) {
                    ldsm_x4(xs + C::TILE + ad, a[0], a[1], a[2], a[3]);
                    mma_16816<T>(dp, a, bq[kk][0], bq[kk][1]);
                }
            }
            const int c0 = step * 16;
            float p[4], dz[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int c = gid + 8 * (u >> 1);
                const bool occ = c0 + c < nreal && ((mw[mbit[u] >> 5] >> (mbit[u] & 31)) & 1u);
                const float s0c = cv[c], mc = cv[16 + c], lc = cv[32 + c], cc = cv[48 + c];
                const float z = s0c + s1r[u & 1];
                const float lr = z > 0.f ? z : A.slope * z;
                const float pv = occ && lc > 0.f ? __fdividef(__expf(lr - mc), lc) : 0.f;
                p[u] = pv;
                dz[u] = pv * (dp[u] - cc) * (z > 0.f ? 1.f : A.slope);
            }
            // ds1 (rows): each lane sums its own columns; the row's lanes are
            // reduced once per work item
            ds1_acc[0] += dz[0] + dz[2];
            ds1_acc[1] += dz[1] + dz[3];
            // ds0 (columns): sum over the 8 rows, one atomic per column
            float c_lo = dz[0] + dz[1], c_hi = dz[2] + dz[3];
#pragma unroll
            for (int o = 1; o < 4; o <<= 1) {
                c_lo += __shfl_xor_sync(0xffffffffu, c_lo, o);
                c_hi += __shfl_xor_sync(0xffffffffu, c_hi, o);
            }
            if (tig == 0) {
#pragma unroll
                for (int u = 0; u < 2; ++u) {
                    const int ci = ((const int *)(cv + 64))[gid + 8 * u];  // -1 past nreal
                    if (ci >= 0 && ci < n_nodes)
                        red_add_f32(A.ds0 + h * n_nodes + ci, u ? c_hi : c_lo);
                }
            }
            // dX'_r += sum_c p[c][r] dout_c
            const uint32_t b0 = movmatrix_trans(pack2<T>(p[0], p[1]));
            const uint32_t b1 = movmatrix_trans(pack2<T>(p[2], p[3]));
#pragma unroll
            for (int j = 0; j < C::MT; ++j) {
                const int q = lane >> 3, rr = lane & 7;
                const int k = (q >> 1) * 8 + rr;
                const int ch = 2 * j + (q & 1);
                const uint32_t ad = k * C::XROW + ((ch ^ swz_row<F>(k)) << 4);
                uint32_t a[4];
                ldsm_x4_trans(xs + ad, a[0], a[1], a[2], a[3]);
                mma_16816<T>(acc[j], a, b0, b1);
                if constexpr (SPLIT) {
                    ldsm_x4_trans(xs + C::TILE + ad, a[0], a[1], a[2], a[3]);
                    mma_16816<T>(acc[j], a, b0, b1);
                }
            }
            __syncwarp();
            if (p_item < n_items) {
                issue(pstage);
                p_advance();
            }
            cp_async_commit();
            cstage = cstage + 1 == kBStages ? 0 : cstage + 1;
            pstage = pstage + 1 == kBStages ? 0 : pstage + 1;
        }
#pragma unroll
        for (int j = 0; j < C::MT; ++j)
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const IT row = wrow + 2 * tig + (u & 1);
                const int f = 16 * j + gid + 8 * (u >> 1);
                if (row < n_nodes) red_add_f32(A.dXp + row * ldg + h * F + f, acc[j][u]);
            }
#pragma unroll
        for (int o = 4; o < 32; o <<= 1) {
            ds1_acc[0] += __shfl_xor_sync(0xffffffffu, ds1_acc[0], o);
            ds1_acc[1] += __shfl_xor_sync(0xffffffffu, ds1_acc[1], o);
        }
        if (gid == 0) {
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                const IT row = wrow + 2 * tig + u;
                if (row < n_nodes) red_add_f32(A.ds1 + h * n_nodes + row, ds1_acc[u]);
            }
        }
    }
    cp_async_wait<0>();
}

template <typename T, int F, bool SPLIT>
int run_gat_bwd(const GatBwdArgs &P, cudaStream_t st) {
    using C = BCfg<T, F, SPLIT>;
    const int64_t items = P.n_parts * P.H;
    if (items == 0) return ATT_OK;
    auto run = [&](auto kernel) {
        static std::once_flag once;
        static int prep = ATT_OK;
        std::call_once(once, [&] {
            prep = cuda_status(
                cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM),
                "cudaFuncSetAttribute");
        });
        if (prep != ATT_OK) return prep;
        int per_sm = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kGThreads, C::SMEM);
        if (per_sm < 1) per_sm = 1;
        const int64_t want = (items + kGWarps - 1) / kGWarps;
        const int64_t cap = (int64_t)sm_count() * per_sm;
        kernel<<<(unsigned)(want < cap ? want : cap), kGThreads, C::SMEM, st>>>(P);
        return launch_status("k_gat_backward");
    };
    // 32-bit offsets when rows of X', dout and dXp, the per-head node arrays
    // and the item count (plus one grid stride) all stay below 2^31
    const int64_t lim = INT32_MAX - (1 << 22);
    int64_t ld = P.ldx > P.ldd ? P.ldx : P.ldd;
    ld = ld > P.ldg ? ld : P.ldg;
    const bool small = P.n_nodes * ld < lim && P.n_nodes * P.H < lim && items < lim;
    if (small) return run(k_gat_backward<T, F, SPLIT, int32_t>);
    return run(k_gat_backward<T, F, SPLIT, int64_t>);
}

template <typename T>
int dispatch_gat_bwd(const GatBwdArgs &P, cudaStream_t st) {
    const bool split = P.dout_lo != nullptr;
    switch (P.F) {
        case 32: return split ? run_gat_bwd<T, 32, true>(P, st) : run_gat_bwd<T, 32, false>(P, st);
        case 64: return split ? run_gat_bwd<T, 64, true>(P, st) : run_gat_bwd<T, 64, false>(P, st);
        case 128: return split ? run_gat_bwd<T, 128, true>(P, st) : run_gat_bwd<T, 128, false>(P, st);
        default:
            set_error("fused GAT backward supports F in {32, 64, 128}, got %lld", (long long)P.F);
            return ATT_ERR_UNSUPPORTED;
    }
}

}  // namespace
}  // namespace att

using namespace att;

extern "C" int att_slot_mask(const int32_t *edge_slot, int64_t nnz, uint32_t *mask,
                             int64_t n_words, void *stream) {
    clear_error();
    cudaStream_t st = (cudaStream_t)stream;
    if (n_words > 0) {
        ATT_CHECK(mask != nullptr, ATT_ERR_INVALID, "null mask");
        ATT_CUDA(cudaMemsetAsync(mask, 0, (size_t)n_words * 4, st), "memset mask");
    }
    if (nnz == 0) return ATT_OK;
    ATT_CHECK(edge_slot != nullptr, ATT_ERR_INVALID, "null edge_slot");
    k_slot_mask<<<(unsigned)((nnz + 255) / 256), 256, 0, st>>>(edge_slot, nnz, mask);
    return launch_status("k_slot_mask");
}

extern "C" int att_gat_forward(const int32_t *rowptr, const int32_t *col, const uint32_t *slot_mask,
                               const int32_t *window_of_part, int64_t n_parts,
                               const int32_t *chunk_begin, const int32_t *chunk_slot,
                               int64_t n_chunks, const int32_t *multi_chunk_begin,
                               int64_t n_multi, int window, int wide, const void *Xp, int x_dtype,
                               int64_t n_nodes, int64_t n_heads, int64_t F, int64_t ldx, int mode,
                               const float *s0, const float *s1, float slope, float *out,
                               int64_t ldo, float *row_max, float *row_sum, float *partial,
                               int32_t *err_flag, void *stream) {
    clear_error();
    ATT_CHECK(window == kW, ATT_ERR_UNSUPPORTED, "fused GAT needs 8-row windows");
    ATT_CHECK(wide == 4 || wide == 8 || wide == 16, ATT_ERR_UNSUPPORTED, "wide must be 4, 8 or 16");
    ATT_CHECK(mode == 0 || mode == 1, ATT_ERR_INVALID, "mode must be 0 (dot) or 1 (additive)");
    ATT_CHECK(x_dtype == ATT_F16 || x_dtype == ATT_BF16 || x_dtype == ATT_F32, ATT_ERR_UNSUPPORTED,
              "fused GAT takes fp16, bf16 or fp32 (3xTF32) features");
    ATT_CHECK(n_heads > 0 && n_heads <= 32 && F > 0, ATT_ERR_INVALID, "bad heads / features");
    ATT_CHECK(ldx % (x_dtype == ATT_F32 ? 4 : 8) == 0 && ((uintptr_t)Xp & 15) == 0 &&
                  ldx >= n_heads * F,
              ATT_ERR_UNSUPPORTED, "X' rows must be 16-byte aligned with ldx >= heads*F");
    ATT_CHECK(ldo >= n_heads * F, ATT_ERR_INVALID, "ldo < heads*F");
    ATT_CHECK(mode == 0 || (s0 && s1), ATT_ERR_INVALID, "additive mode needs node scores");
    cudaStream_t st = (cudaStream_t)stream;
    if (n_nodes == 0) return ATT_OK;
    {
        const int64_t threads = (n_nodes + kW - 1) / kW * 32;
        k_gat_zero_rows<<<(unsigned)((threads + 255) / 256), 256, 0, st>>>(
            window_of_part, n_parts, n_nodes, n_heads, F, out, ldo, row_max, row_sum);
        int s = launch_status("k_gat_zero_rows");
        if (s != ATT_OK) return s;
    }
    if (n_chunks == 0) return ATT_OK;
    ATT_CHECK(rowptr && col && slot_mask && window_of_part && chunk_begin && chunk_slot,
              ATT_ERR_INVALID, "null format pointer");
    ATT_CHECK(n_multi == 0 || (partial && multi_chunk_begin), ATT_ERR_INVALID,
              "split windows need the partial buffer");
    GatArgs P{rowptr, col, window_of_part, slot_mask, chunk_begin, chunk_slot, n_chunks, wide, Xp,
              n_nodes, n_heads, F, ldx, mode, s0, s1, slope, out, ldo, row_max, row_sum, partial,
              err_flag};
    int s;
    // partial slots are at most one per chunk
    const int64_t np = P.n_chunks;
    if (x_dtype == ATT_F16)
        s = mode == 0 ? dispatch_gat_f<__half, 0>(P, st, np) : dispatch_gat_f<__half, 1>(P, st, np);
    else if (x_dtype == ATT_F32)
        s = mode == 0 ? dispatch_gat_f<float, 0>(P, st, np) : dispatch_gat_f<float, 1>(P, st, np);
    else
        s = mode == 0 ? dispatch_gat_f<__nv_bfloat16, 0>(P, st, np)
                      : dispatch_gat_f<__nv_bfloat16, 1>(P, st, np);
    if (s != ATT_OK) return s;
    if (n_multi > 0) {
        k_gat_combine<<<(unsigned)(n_multi * n_heads), kW * 32, 0, st>>>(
            multi_chunk_begin, chunk_slot, chunk_begin, window_of_part, n_multi, n_heads, F,
            n_nodes, partial, out, ldo, row_max, row_sum);
        s = launch_status("k_gat_combine");
    }
    return s;
}

extern "C" int att_gat_backward(const int32_t *rowptr_t, const int32_t *col_t,
                                const uint32_t *slot_mask_t, const int32_t *window_of_part_t,
                                int64_t n_parts_t, int window, int wide, const void *Xp,
                                const void *dout, const void *dout_lo, int x_dtype, int64_t n_nodes, int64_t n_heads,
                                int64_t F, int64_t ldx, int64_t ldd, const float *s0,
                                const float *s1, const float *row_max, const float *row_sum,
                                const float *c, float slope, float *dXp, int64_t ldg, float *ds0,
                                float *ds1, int32_t *err_flag, void *stream) {
    clear_error();
    ATT_CHECK(window == kW, ATT_ERR_UNSUPPORTED, "fused GAT backward needs 8-row windows");
    ATT_CHECK(wide == 4 || wide == 8 || wide == 16, ATT_ERR_UNSUPPORTED, "wide must be 4, 8 or 16");
    ATT_CHECK(x_dtype == ATT_F16 || x_dtype == ATT_BF16, ATT_ERR_UNSUPPORTED,
              "fused GAT backward takes fp16 or bf16 X' and dout");
    ATT_CHECK(n_heads > 0 && F > 0, ATT_ERR_INVALID, "bad heads / features");
    ATT_CHECK(ldx % 8 == 0 && ldd % 8 == 0 && ((uintptr_t)Xp & 15) == 0 &&
                  ((uintptr_t)dout & 15) == 0 && ((uintptr_t)dout_lo & 15) == 0,
              ATT_ERR_UNSUPPORTED, "X' and dout rows must be 16-byte aligned");
    ATT_CHECK(s0 && s1 && row_max && row_sum && c && dXp && ds0 && ds1, ATT_ERR_INVALID,
              "null pointer");
    if (n_parts_t == 0 || n_nodes == 0) return ATT_OK;
    ATT_CHECK(rowptr_t && col_t && slot_mask_t && window_of_part_t, ATT_ERR_INVALID,
              "null format pointer");
    GatBwdArgs P{rowptr_t, col_t, window_of_part_t, slot_mask_t, n_parts_t, wide, Xp, dout,
                 dout_lo, n_nodes, n_heads, F, ldx, ldd, s0, s1, row_max, row_sum, c, slope, dXp, ldg,
                 ds0, ds1, err_flag};
    cudaStream_t st = (cudaStream_t)stream;
    return x_dtype == ATT_F16 ? dispatch_gat_bwd<__half>(P, st) : dispatch_gat_bwd<__nv_bfloat16>(P, st);
}

// ---------------------------------------------------------------------------
// Elementwise ends of the fused GAT backward (one pass each over [N, H*F])
// ---------------------------------------------------------------------------
namespace att {
namespace {

template <typename T>
__device__ __forceinline__ T to_t(float v);
template <>
__device__ __forceinline__ __half to_t<__half>(float v) { return __float2half_rn(v); }
template <>
__device__ __forceinline__ __nv_bfloat16 to_t<__nv_bfloat16>(float v) {
    return __float2bfloat16_rn(v);
}
template <typename T>
__device__ __forceinline__ float from_t(T v);
template <>
__device__ __forceinline__ float from_t<__half>(__half v) { return __half2float(v); }
template <>
__device__ __forceinline__ float from_t<__nv_bfloat16>(__nv_bfloat16 v) {
    return __bfloat162float(v);
}

// One warp per node row: c[h][n] = dout[n, h] . out[n, h] (fp32), and dout
// split into a 16-bit hi part and the 16-bit rounding of its remainder.
template <typename T>
__global__ void k_gat_grad_prepare(const float *__restrict__ dout, int64_t ldd,
                                   const float *__restrict__ out, int64_t ldo, int64_t n_nodes,
                                   int64_t H, int64_t F, T *__restrict__ hi, T *__restrict__ lo,
                                   int64_t ldh, float *__restrict__ c) {
    const int lane = threadIdx.x & 31;
    const int64_t n = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (n >= n_nodes) return;
    for (int64_t h = 0; h < H; ++h) {
        float s = 0.f;
        for (int64_t f = lane; f < F; f += 32) {
            const int64_t col = h * F + f;
            const float d = dout[n * ldd + col];
            s += d * out[n * ldo + col];
            const T dh = to_t<T>(d);
            hi[n * ldh + col] = dh;
            lo[n * ldh + col] = to_t<T>(d - from_t<T>(dh));
        }
        s = warp_sum(s);
        if (lane == 0) c[h * n_nodes + n] = s;
    }
}

// dX[n, hF+f] = cast(dXp[n, hF+f] + ds0[h][n] a0[h][f] + ds1[h][n] a1[h][f]);
// da0[h][f] += sum_n ds0[h][n] X'[n, hF+f], da1 likewise (fp32 atomics, one
// per column per thread).  A block covers 256 columns of several rows per
// sweep (256 / HF rows when HF <= 256).
template <typename T>
__global__ void __launch_bounds__(256) k_gat_grad_finish(
    const float *__restrict__ dXp, int64_t ldg, const float *__restrict__ ds0,
    const float *__restrict__ ds1, const float *__restrict__ a0, const float *__restrict__ a1,
    const T *__restrict__ Xp, int64_t ldx, int64_t n_nodes, int64_t H, int64_t F,
    T *__restrict__ dX, int64_t ldo, float *__restrict__ da0, float *__restrict__ da1) {
    const int64_t HF = H * F;
    const int t = threadIdx.x;
    const int64_t cols = HF < 256 ? HF : 256;
    const int64_t rows = 256 / cols;  // rows per sweep of the block
    const int64_t roff = t / cols;
    if (roff >= rows) return;
    for (int64_t cb = 0; cb < HF; cb += 256) {
        const int64_t col = cb + t % cols;
        if (col >= HF) continue;
        const int64_t h = col / F;
        const float w0 = a0[col], w1 = a1[col];
        float acc0 = 0.f, acc1 = 0.f;
        for (int64_t n = (int64_t)blockIdx.x * rows + roff; n < n_nodes; n += (int64_t)gridDim.x * rows) {
            const float g0 = ds0[h * n_nodes + n], g1 = ds1[h * n_nodes + n];
            const float x = from_t<T>(Xp[n * ldx + col]);
            dX[n * ldo + col] = to_t<T>(dXp[n * ldg + col] + g0 * w0 + g1 * w1);
            acc0 += g0 * x;
            acc1 += g1 * x;
        }
        atomicAdd(da0 + col, acc0);
        atomicAdd(da1 + col, acc1);
    }
}

}  // namespace
}  // namespace att

extern "C" int att_gat_grad_prepare(const float *dout, int64_t ldd, const float *out, int64_t ldo,
                                    int64_t n_nodes, int64_t n_heads, int64_t F, void *dout_hi,
                                    void *dout_lo, int dtype, int64_t ldh, float *c, void *stream) {
    using namespace att;
    clear_error();
    ATT_CHECK(dtype == ATT_F16 || dtype == ATT_BF16, ATT_ERR_UNSUPPORTED,
              "dout splits into fp16 or bf16");
    ATT_CHECK(n_nodes >= 0 && n_heads > 0 && F > 0, ATT_ERR_INVALID, "bad sizes");
    ATT_CHECK(ldd >= n_heads * F && ldo >= n_heads * F && ldh >= n_heads * F, ATT_ERR_INVALID,
              "row strides shorter than heads x F");
    if (n_nodes == 0) return ATT_OK;
    ATT_CHECK(dout && out && dout_hi && dout_lo && c, ATT_ERR_INVALID, "null pointer");
    cudaStream_t st = (cudaStream_t)stream;
    const int64_t threads = n_nodes * 32;
    const unsigned grid = (unsigned)((threads + 255) / 256);
    if (dtype == ATT_F16)
        k_gat_grad_prepare<__half><<<grid, 256, 0, st>>>(dout, ldd, out, ldo, n_nodes, n_heads, F,
                                                         (__half *)dout_hi, (__half *)dout_lo, ldh, c);
    else
        k_gat_grad_prepare<__nv_bfloat16><<<grid, 256, 0, st>>>(
            dout, ldd, out, ldo, n_nodes, n_heads, F, (__nv_bfloat16 *)dout_hi,
            (__nv_bfloat16 *)dout_lo, ldh, c);
    return launch_status("k_gat_grad_prepare");
}

extern "C" int att_gat_grad_finish(const float *dXp, int64_t ldg, const float *ds0, const float *ds1,
                                   const float *a0, const float *a1, const void *Xp, int dtype,
                                   int64_t ldx, int64_t n_nodes, int64_t n_heads, int64_t F, void *dX,
                                   int64_t ld_dx, float *da0, float *da1, void *stream) {
    using namespace att;
    clear_error();
    ATT_CHECK(dtype == ATT_F16 || dtype == ATT_BF16, ATT_ERR_UNSUPPORTED,
              "X' and dX are fp16 or bf16");
    ATT_CHECK(n_nodes >= 0 && n_heads > 0 && F > 0, ATT_ERR_INVALID, "bad sizes");
    ATT_CHECK(ldg >= n_heads * F && ldx >= n_heads * F && ld_dx >= n_heads * F, ATT_ERR_INVALID,
              "row strides shorter than heads x F");
    if (n_nodes == 0) return ATT_OK;
    ATT_CHECK(dXp && ds0 && ds1 && a0 && a1 && Xp && dX && da0 && da1, ATT_ERR_INVALID,
              "null pointer");
    cudaStream_t st = (cudaStream_t)stream;
    const int64_t HF = n_heads * F;
    const int64_t rows = 256 / (HF < 256 ? HF : 256);
    int64_t want = (n_nodes + rows - 1) / rows;
    const int64_t cap = (int64_t)sm_count() * 8;
    const unsigned grid = (unsigned)(want < cap ? want : cap);
    if (dtype == ATT_F16)
        k_gat_grad_finish<__half><<<grid, 256, 0, st>>>(dXp, ldg, ds0, ds1, a0, a1,
                                                        (const __half *)Xp, ldx, n_nodes, n_heads,
                                                        F, (__half *)dX, ld_dx, da0, da1);
    else
        k_gat_grad_finish<__nv_bfloat16><<<grid, 256, 0, st>>>(
            dXp, ldg, ds0, ds1, a0, a1, (const __nv_bfloat16 *)Xp, ldx, n_nodes, n_heads, F,
            (__nv_bfloat16 *)dX, ld_dx, da0, da1);
    return launch_status("k_gat_grad_finish");
}
