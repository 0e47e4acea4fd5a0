// spmm.cu -- blocked SpMM Y = A_blocks * X on the row-window block format.
//
// Replaces the reference's GCN SpMM kernels (gcn/SpMM/src/spmmKernel.cu:158-265
// fp16, :959-1075 tf32, :2066-2330 the "_acc" variants) behind
// SpMM_sr_bcrs.forward_{fp16,tf32}_gnn[_acc] (gcn/SpMM/src/benchmark.cpp:35-335).
//
// Design (sm_103a):
//  * One warp owns one work item = (part, chunk of FC features) at a time and
//    walks its items in a persistent grid-stride sequence.  Each k-step is 16
//    condensed columns: the 16 gathered X rows (FC features each) and the
//    16 x W value block are copied global->shared with 16-byte cp.async into
//    an S-stage ring; the producer cursor runs S-1 steps ahead of the
//    consumer across item boundaries, so the gather stream never drains.
//  * The contraction is D[feature, row] += X^T[feature, col] * V[col, row]:
//    M = 16 features, N = 8 window rows, K = 16 columns, so the sparse block
//    is the dense B operand and the gathered rows are A.  ldmatrix.trans
//    turns the row-major gathered X tile into the A fragment; the value tile
//    feeds B through a plain ldmatrix.  fp32 accumulators stay in registers.
//    (The reference uses m16n8k8 with fp16 accumulation; this accumulates in
//    fp32.)  Shared rows are XOR-swizzled per 16-byte chunk so both ldmatrix
//    forms are bank-conflict free.
//  * TF32 runs m16n8k8 as a 3xTF32 split (hi*hi + hi*lo + lo*hi), which gives
//    fp32-level accuracy at no cost on a gather-bound kernel.
//  * Output: a part of an unsplit window stores its whole W-row tile with
//    plain stores; parts of split windows add with red.global.add.f32.  A
//    small pre-pass zeroes only rows that no unsplit part writes (split
//    windows, windows without parts, trailing rows), so Y needs no memset.
#include "att_common.cuh"

#include <cuda.h>
#include <cudaTypedefs.h>

#include <atomic>
#include <mutex>
#include <string.h>
#include <type_traits>

namespace att {
namespace {

constexpr int kWarps = 4;
constexpr int kThreads = kWarps * 32;
constexpr int kStages = 4;

struct PartInfo {
    int start, nreal, nsteps;
};

// A part must start and end on a block boundary of the layout the kernel
// reads (the value tile of a 16-column step is read whole); a part that does
// not is flagged and skipped instead of read past its end.
template <int WIDE>
__device__ __forceinline__ PartInfo part_info(const int32_t *__restrict__ rowptr, int64_t p,
                                              int32_t *err) {
    PartInfo pi;
    pi.start = __ldg(rowptr + 2 * p);
    const int e = __ldg(rowptr + 2 * p + 1);
    const int pend = __ldg(rowptr + 2 * p + 2);
    pi.nreal = e > pi.start ? e - pi.start : 0;
    if ((pi.start % WIDE) != 0 || (pend % WIDE) != 0 || pend < pi.start + pi.nreal) {
        if (err) atomicOr(err, 2);
        pi.nreal = 0;
    }
    pi.nsteps = (pi.nreal + 15) >> 4;
    return pi;
}

// XOR swizzle of the 16-byte chunk index within a shared row of `row_bytes`
template <int ROW_BYTES>
__device__ __forceinline__ int swz(int r) {
    if constexpr (ROW_BYTES >= 128) return r & 7;
    else return (r >> 1) & 3;  // 64-byte rows: two rows share a 128-byte bank window
}

// ---------------------------------------------------------------------------
// 16-bit operand kernel (fp16 / bf16 values and features)
// ---------------------------------------------------------------------------
template <typename T, int W, int FC, int WIDE, int S = kStages>
struct Cfg16 {
    static constexpr int XROW = FC * 2;                 // bytes per gathered row in smem
    static constexpr int XSTAGE = 16 * XROW;            // 16 rows per k-step
    static constexpr int VSTAGE = 16 * W * 2;           // 16 cols x W rows
    static constexpr int STAGE = XSTAGE + VSTAGE;
    static constexpr int WARP_SMEM = S * STAGE;
    static constexpr int SMEM = kWarps * WARP_SMEM;
    static constexpr int CPR = FC / 8;                  // 16-byte chunks per row
    static constexpr int RPP = 32 / CPR;                // rows per warp pass
    static constexpr int MT = FC / 16;                  // m16 tiles
    static constexpr int NT = W / 8;                    // n8 tiles
    static constexpr int VCH = VSTAGE / 16;             // value chunks per step
    // 8-row windows with <= 64 features: as many CTAs per SM as shared memory
    // allows (228 KB per SM, 1 KB reserved per CTA; 8 for the default shape)
    // bound the registers; other shapes keep the compiler's choice
    static constexpr int MINB_RAW = (228 * 1024) / (SMEM + 1024);
    static constexpr int MINB =
        (W != 8 || FC > 64) ? 1 : (MINB_RAW < 1 ? 1 : (MINB_RAW > 8 ? 8 : MINB_RAW));
};

// IT: index type of items and element offsets -- int32_t when every offset
// into X, Y and the values fits (the common case: fewer instructions per
// gathered row; the kernel is issue-bound), else int64_t.
// FULL: F is a multiple of FC (every chunk whole; no per-feature bounds checks)
template <typename T, int W, int FC, int WIDE, int S, typename IT, bool FULL>
__global__ void __launch_bounds__(kThreads, (Cfg16<T, W, FC, WIDE, S>::MINB)) k_spmm16(
    const int32_t *__restrict__ rowptr, const int32_t *__restrict__ col,
    const T *__restrict__ val, const int32_t *__restrict__ win,
    const int32_t *__restrict__ atomic, int64_t n_parts, const T *__restrict__ X, int64_t n_x_,
    int64_t F_, int64_t ldx_, float *__restrict__ Y, int64_t m_out_, int64_t ldy_, int n_chunks,
    int32_t *__restrict__ err) {
    using C = Cfg16<T, W, FC, WIDE, S>;
    extern __shared__ __align__(128) unsigned char smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t sbase = smem_u32(smem) + warp * C::WARP_SMEM;
    const IT n_x = (IT)n_x_, F = (IT)F_, ldx = (IT)ldx_, m_out = (IT)m_out_, ldy = (IT)ldy_;
    const IT n_items = (IT)(n_parts * n_chunks);
    const IT stride = (IT)gridDim.x * kWarps;
    const int gid = lane >> 2, tig = lane & 3;

    // ---- producer cursor ----
    IT p_item = (IT)blockIdx.x * kWarps + warp;
    int p_step = 0, p_myc = -1;
    PartInfo p_pi = {0, 0, 0};
    int p_fc = 0;
    auto p_load = [&]() {
        while (p_item < n_items) {
            const IT part = p_item / n_chunks;
            p_fc = (int)(p_item - part * n_chunks);
            p_pi = part_info<WIDE>(rowptr, part, err);
            p_step = 0;
            if (p_pi.nsteps > 0) return;
            p_item += stride;
        }
    };
    auto issue = [&](int stage) {
        const uint32_t xs = sbase + stage * C::STAGE;
        const uint32_t vs = xs + C::XSTAGE;
        const int c0 = p_step * 16;
        int myc = p_myc;  // loaded one step ahead
        // valid ids are -1 (padding) .. n_x - 1; an id outside is flagged and
        // gathered as padding (zeros) -- checked once per id, not per chunk
        if ((uint64_t)(int64_t)(myc + 1) > (uint64_t)n_x) {
            if (err) atomicOr(err, 1);
            myc = -1;
        }
        const IT fbase = (IT)p_fc * FC;
        const bool full = FULL || fbase + FC <= F;  // the whole chunk is inside F (uniform)
        // CPR lanes copy one row's FC features per pass (whole 128-byte lines
        // per instruction; spreading a row over lane pairs measured 2.4x
        // slower on the 2.45M-node graph)
#pragma unroll
        for (int i = 0; i < 16 / C::RPP; ++i) {
            const int r = i * C::RPP + lane / C::CPR;
            const int ch = lane % C::CPR;
            const int cidx = __shfl_sync(0xffffffffu, myc, r);
            const IT f = fbase + ch * 8;
            const bool ok = cidx >= 0 && (full || f < F);
            // padding: src-size 0 fills zeros (the source stays X's base)
            const IT off = ok ? (IT)cidx * ldx + f : (IT)0;
            cp_async16(xs + r * C::XROW + ((ch ^ swz<C::XROW>(r)) << 4), X + off, ok ? 16 : 0);
        }
#pragma unroll
        for (int q = lane; q < C::VCH; q += 32) {
            const int e = q * 8;                       // element offset within the step's block run
            const int blk = e / (W * WIDE);
            const bool ok = c0 + blk * WIDE < p_pi.nreal;
            const T *src = val + ((IT)(p_pi.start + c0) * W + e);
            cp_async16(vs + q * 16, ok ? (const void *)src : (const void *)val, ok ? 16 : 0);
        }
    };
    // column ids of the producer's position, fetched one step ahead so the
    // load latency overlaps the consumer's work instead of stalling issue()
    auto p_fetch = [&]() {
        p_myc = -1;
        if (p_item < n_items && p_step * 16 + (lane & 15) < p_pi.nreal)
            p_myc = __ldg(col + p_pi.start + p_step * 16 + (lane & 15));
    };
    auto p_advance = [&]() {
        if (++p_step >= p_pi.nsteps) {
            p_item += stride;
            p_load();
        }
        p_fetch();
    };

    p_load();
    p_fetch();
#pragma unroll
    for (int s = 0; s < S - 1; ++s) {
        if (p_item < n_items) {
            issue(s);
            p_advance();
        }
        cp_async_commit();
    }

    // ---- consumer ----
    float acc[C::MT][C::NT][4];
#pragma unroll
    for (int j = 0; j < C::MT; ++j)
#pragma unroll
        for (int t = 0; t < C::NT; ++t) acc[j][t][0] = acc[j][t][1] = acc[j][t][2] = acc[j][t][3] = 0.f;

    int cstage = 0, pstage = S - 1;
    for (IT c_item = (IT)blockIdx.x * kWarps + warp; c_item < n_items; c_item += stride) {
        const IT part = c_item / n_chunks;
        const int fc = (int)(c_item - part * n_chunks);
        const PartInfo pi = part_info<WIDE>(rowptr, part, err);
        for (int step = 0; step < pi.nsteps; ++step) {
            cp_async_wait<S - 2>();
            __syncwarp();
            const uint32_t xs = sbase + cstage * C::STAGE;
            const uint32_t vs = xs + C::XSTAGE;
            // B fragments: value tile rows = window rows, 8 columns per matrix
            uint32_t b[C::NT][2];
            {
                const int q = lane >> 3, rr = lane & 7;
                if constexpr (C::NT == 2) {
                    const int kb = q & 1, r = (q >> 1) * 8 + rr;
                    const int e = (kb * 8 / WIDE) * W * WIDE + r * WIDE + (kb * 8) % WIDE;
                    ldsm_x4(vs + e * 2, b[0][0], b[0][1], b[1][0], b[1][1]);
                } else {
                    const int kb = q & 1, r = rr;
                    const int e = (kb * 8 / WIDE) * W * WIDE + r * WIDE + (kb * 8) % WIDE;
                    ldsm_x2(vs + e * 2, b[0][0], b[0][1]);
                }
            }
#pragma unroll
            for (int j = 0; j < C::MT; ++j) {
                const int q = lane >> 3, rr = lane & 7;
                const int k = (q >> 1) * 8 + rr;
                const int ch = 2 * j + (q & 1);
                uint32_t a[4];
                ldsm_x4_trans(xs + k * C::XROW + ((ch ^ swz<C::XROW>(k)) << 4), a[0], a[1], a[2],
                              a[3]);
#pragma unroll
                for (int t = 0; t < C::NT; ++t) mma_16816<T>(acc[j][t], a, b[t][0], b[t][1]);
            }
            __syncwarp();
            if (p_item < n_items) {
                issue(pstage);
                p_advance();
            }
            cp_async_commit();
            cstage = cstage + 1 == S ? 0 : cstage + 1;
            pstage = pstage + 1 == S ? 0 : pstage + 1;
        }
        // ---- epilogue: the W x FC tile of this part ----
        const int wrow = __ldg(win + part);
        const bool add = __ldg(atomic + part) != 0;
        const IT f0 = (IT)fc * FC;
        const bool full = FULL || f0 + FC <= F;
#pragma unroll
        for (int t = 0; t < C::NT; ++t) {
            const IT r0 = (IT)wrow * W + t * 8 + 2 * tig;
#pragma unroll
            for (int j = 0; j < C::MT; ++j) {
                const IT fa = f0 + 16 * j + gid;
#pragma unroll
                for (int h = 0; h < 4; ++h) {
                    const IT r = r0 + (h & 1);
                    const IT f = fa + (h >> 1) * 8;
                    if (r < m_out && (full || f < F)) {
                        float *dst = Y + (r * ldy + f);
                        // Y is written once: a streaming store leaves L2 to the X rows
                        if (add) red_add_f32(dst, acc[j][t][h]);
                        else __stcs(dst, acc[j][t][h]);
                    }
                    acc[j][t][h] = 0.f;
                }
            }
        }
    }
    cp_async_wait<0>();
}

constexpr uint32_t kMaxPolls = 1u << 24;  // bounded mbarrier waits

// ---------------------------------------------------------------------------
// 16-bit operand kernel with bulk row copies (8-row windows, 8-wide blocks,
// 64-feature chunks)
// ---------------------------------------------------------------------------
// Same contraction and epilogue as k_spmm16; the producer moves each gathered
// row's 128 bytes with one cp.async.bulk (lanes 0-15, one row each) instead of
// eight 16-byte cp.async spread over the warp, so the issue cost per gathered
// row drops.  Rows sit at a 144-byte pitch: the 16-byte pad keeps
// ldmatrix.trans conflict-free without a swizzle (a bulk copy cannot swizzle)
// and holds one 16-byte chunk of the step's value tile (chunk r = block r / 8,
// window row r % 8), so a stage stays 16 x 144 bytes.  Each stage completes on
// its own mbarrier (32 arrivals + the copied bytes); waits are bounded and a
// timeout sets error bit 4.  Padding rows (column -1) and value blocks past
// the part's real columns are zero-filled with shared stores instead of read.
constexpr int kBulkPitch = 144;

template <typename T, int S, typename IT>
__global__ void __launch_bounds__(kThreads) k_spmm16_bulk(
    const int32_t *__restrict__ rowptr, const int32_t *__restrict__ col,
    const T *__restrict__ val, const int32_t *__restrict__ win,
    const int32_t *__restrict__ atomic, int64_t n_parts, const T *__restrict__ X, int64_t n_x_,
    int64_t F_, int64_t ldx_, float *__restrict__ Y, int64_t m_out_, int64_t ldy_, int n_chunks,
    int32_t *__restrict__ err) {
    constexpr int W = 8, WIDE = 8, FC = 64, MT = FC / 16;
    constexpr int STAGE = 16 * kBulkPitch;
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ __align__(8) uint64_t bars[kWarps][S];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t sbase = smem_u32(smem) + warp * (S * STAGE);
    const uint32_t bar0 = smem_u32(&bars[warp][0]);
    const IT n_x = (IT)n_x_, F = (IT)F_, ldx = (IT)ldx_, m_out = (IT)m_out_, ldy = (IT)ldy_;
    const IT n_items = (IT)(n_parts * n_chunks);
    const IT stride = (IT)gridDim.x * kWarps;
    const int gid = lane >> 2, tig = lane & 3;

    if (lane == 0)
        for (int s = 0; s < S; ++s) mbar_init(bar0 + 8 * s, 32);
    mbar_fence_init();
    __syncwarp();

    IT p_item = (IT)blockIdx.x * kWarps + warp;
    int p_step = 0, p_myc = -1;
    PartInfo p_pi = {0, 0, 0};
    int p_fc = 0;
    auto p_load = [&]() {
        while (p_item < n_items) {
            const IT part = p_item / n_chunks;
            p_fc = (int)(p_item - part * n_chunks);
            p_pi = part_info<WIDE>(rowptr, part, err);
            p_step = 0;
            if (p_pi.nsteps > 0) return;
            p_item += stride;
        }
    };
    auto issue = [&](int stage) {
        const uint32_t xs = sbase + stage * STAGE;
        const uint32_t bar = bar0 + 8 * stage;
        uint32_t bytes = 0;
        if (lane < 16) {
            const int r = lane;
            int cidx = p_myc;  // this lane's own column id (row r of the step)
            if ((uint64_t)(int64_t)(cidx + 1) > (uint64_t)n_x) {
                if (err) atomicOr(err, 1);
                cidx = -1;
            }
            const IT fbase = (IT)p_fc * FC;
            const uint32_t dst = xs + r * kBulkPitch;
            fence_proxy_async_smem();  // earlier generic reads of this stage before the async writes
            if (cidx >= 0) {
                const uint32_t nb = (uint32_t)(fbase + FC <= F ? FC * 2 : (F - fbase) * 2);
                bulk_g2s(dst, X + ((IT)cidx * ldx + fbase), nb, bar);
                bytes += nb;
            } else {
#pragma unroll
                for (int q = 0; q < FC * 2 / 16; ++q)
                    asm volatile("st.shared.v4.b32 [%0], {%1, %1, %1, %1};\n" ::"r"(dst + 16 * q), "r"(0)
                                 : "memory");
            }
            const int c0 = p_step * 16;
            const int blk = r >> 3;  // value chunk r: block r / 8, window row r % 8
            if (c0 + blk * WIDE < p_pi.nreal) {
                bulk_g2s(dst + 128, val + ((IT)(p_pi.start + c0) * W + r * 8), 16, bar);
                bytes += 16;
            } else {
                asm volatile("st.shared.v4.b32 [%0], {%1, %1, %1, %1};\n" ::"r"(dst + 128), "r"(0)
                             : "memory");
            }
        }
        if (bytes)
            mbar_arrive_expect_tx(bar, bytes);
        else
            asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(bar) : "memory");
    };
    auto p_fetch = [&]() {
        p_myc = -1;
        if (p_item < n_items && p_step * 16 + (lane & 15) < p_pi.nreal)
            p_myc = __ldg(col + p_pi.start + p_step * 16 + (lane & 15));
    };
    auto p_advance = [&]() {
        if (++p_step >= p_pi.nsteps) {
            p_item += stride;
            p_load();
        }
        p_fetch();
    };

    p_load();
    p_fetch();
#pragma unroll
    for (int s = 0; s < S - 1; ++s)
        if (p_item < n_items) {
            issue(s);
            p_advance();
        }

    float acc[MT][4];
#pragma unroll
    for (int j = 0; j < MT; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;

    uint32_t phase = 0;  // bit s: parity of stage s's next completion
    int cstage = 0, pstage = S - 1;
    for (IT c_item = (IT)blockIdx.x * kWarps + warp; c_item < n_items; c_item += stride) {
        const IT part = c_item / n_chunks;
        const int fc = (int)(c_item - part * n_chunks);
        const PartInfo pi = part_info<WIDE>(rowptr, part, nullptr);
        for (int step = 0; step < pi.nsteps; ++step) {
            if (!mbar_wait_bounded(bar0 + 8 * cstage, (phase >> cstage) & 1u, kMaxPolls)) {
                if (err) atomicOr(err, 4);
            }
            phase ^= 1u << cstage;
            __syncwarp();
            const uint32_t xs = sbase + cstage * STAGE;
            uint32_t b0, b1;
            {
                // B: value tile rows = window rows; matrix kb = block kb
                const int kb = (lane >> 3) & 1, rr = lane & 7;
                ldsm_x2(xs + (kb * 8 + rr) * kBulkPitch + 128, b0, b1);
            }
#pragma unroll
            for (int j = 0; j < MT; ++j) {
                const int q = lane >> 3, rr = lane & 7;
                const int k = (q >> 1) * 8 + rr;
                const int ch = 2 * j + (q & 1);
                uint32_t a[4];
                ldsm_x4_trans(xs + k * kBulkPitch + ch * 16, a[0], a[1], a[2], a[3]);
                mma_16816<T>(acc[j], a, b0, b1);
            }
            __syncwarp();
            if (p_item < n_items) {
                issue(pstage);
                p_advance();
            }
            cstage = cstage + 1 == S ? 0 : cstage + 1;
            pstage = pstage + 1 == S ? 0 : pstage + 1;
        }
        const int wrow = __ldg(win + part);
        const bool add = __ldg(atomic + part) != 0;
        const IT f0 = (IT)fc * FC;
        const bool full = f0 + FC <= F;
        const IT r0 = (IT)wrow * W + 2 * tig;
#pragma unroll
        for (int j = 0; j < MT; ++j) {
            const IT fa = f0 + 16 * j + gid;
#pragma unroll
            for (int h = 0; h < 4; ++h) {
                const IT r = r0 + (h & 1);
                const IT f = fa + (h >> 1) * 8;
                if (r < m_out && (full || f < F)) {
                    float *dst = Y + (r * ldy + f);
                    if (add) red_add_f32(dst, acc[j][h]);
                    else *dst = acc[j][h];
                }
                acc[j][h] = 0.f;
            }
        }
    }
}

// ---------------------------------------------------------------------------
// 16-bit operand kernel fed by TMA: tile::gather4 row gathers
// ---------------------------------------------------------------------------
// Same contraction and epilogue as k_spmm16; the producer is one bulk-tensor
// instruction per 4 gathered rows and 64 features instead of 16 cp.async per
// lane.  X is described by a 2-D tensor map (features x rows) with an
// 80 x 1 box and no swizzle: a gathered row occupies 160 bytes, so the 8 rows
// an ldmatrix reads fall on distinct 32-byte bank groups within a 4-row group
// (two groups share them: 2-way), and 4 rows (640 bytes) keep every TMA
// destination 128-byte aligned without padding.  Of the 80 features, the 64
// wanted plus 16 chosen outside [0, F) where possible (left of feature 0, or
// right of the last), which TMA zero-fills without reading memory.  Rows of
// padding columns are fetched from row n_x, outside the tensor, also
// zero-filled.  The step's value tile is one contiguous bulk copy.  Each
// stage completes on an mbarrier carrying the byte count; every wait is
// bounded, and a timeout raises bit 4 of err and ends the warp after draining
// its copies in flight.
constexpr int kBox = 80;            // features per TMA box
constexpr int kPitch = kBox * 2;    // bytes per gathered row in shared memory
constexpr int kGroup = 4 * kPitch;  // one gather4 destination (640 B, 128-aligned)

template <int W, int FC, int S>
struct CfgTma {
    static constexpr int FCH = FC / 64;            // 64-feature boxes per gathered row
    static constexpr int CHUNK = 4 * kGroup;       // 16 rows of one box
    static constexpr int XSTAGE = FCH * CHUNK;
    static constexpr int VSTAGE = 16 * W * 2;
    static constexpr int STAGE = (XSTAGE + VSTAGE + 127) / 128 * 128;
    static constexpr int WARP_SMEM = (S * STAGE + S * 8 + 127) / 128 * 128;
    static constexpr int SMEM = kWarps * WARP_SMEM + 128;  // + alignment slack
    static constexpr int MT = FC / 16;
    static constexpr int NT = W / 8;
};

// 16 of the 80 features of a box are extra: to the left of `fb` (box starts
// at fb - 16) unless the right side is past F (box starts at fb)
__device__ __forceinline__ bool box_left(int64_t fb, int64_t F) { return fb == 0 || fb + 64 < F; }

template <typename T, int W, int FC, int WIDE, int S>
__global__ void __launch_bounds__(kThreads) k_spmm16_tma(
    const __grid_constant__ CUtensorMap tmX, const int32_t *__restrict__ rowptr,
    const int32_t *__restrict__ col, const T *__restrict__ val, const int32_t *__restrict__ win,
    const int32_t *__restrict__ atomic, int64_t n_parts, int64_t n_x, int64_t F,
    float *__restrict__ Y, int64_t m_out, int64_t ldy, int n_chunks, int32_t *__restrict__ err) {
    using C = CfgTma<W, FC, S>;
    extern __shared__ __align__(128) unsigned char smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t sbase = ((smem_u32(smem) + 127u) & ~127u) + warp * C::WARP_SMEM;
    const int64_t n_items = n_parts * n_chunks;
    const int64_t stride = (int64_t)gridDim.x * kWarps;
    const int gid = lane >> 2, tig = lane & 3;
    const int oob_row = (int)n_x;  // one past the last row: zero-filled by TMA
    auto xstage = [&](int stage) { return sbase + stage * C::STAGE; };
    auto vtile = [&](int stage) { return sbase + stage * C::STAGE + C::XSTAGE; };
    auto sbar = [&](int stage) { return sbase + S * C::STAGE + 8 * stage; };

    // value tiles start zeroed (a tile whose second block lies past its part
    // keeps finite data that only ever meets zero rows); barriers armed once
    for (int st = 0; st < S; ++st)
        for (int i = lane; i < C::VSTAGE / 4; i += 32)
            asm volatile("st.shared.u32 [%0], %1;\n" ::"r"(vtile(st) + 4 * i), "r"(0) : "memory");
    if (lane == 0) {
        for (int st = 0; st < S; ++st) mbar_init(sbar(st), 1);
        mbar_fence_init();
    }
    fence_proxy_async_smem();
    __syncwarp();

    int64_t p_item = (int64_t)blockIdx.x * kWarps + warp;
    int p_step = 0, p_fc = 0, p_pend = 0, p_myc = -1;
    PartInfo p_pi = {0, 0, 0};
    auto p_load = [&]() {
        while (p_item < n_items) {
            int64_t part = p_item / n_chunks;
            p_fc = (int)(p_item - part * n_chunks);
            p_pi = part_info<WIDE>(rowptr, part, err);
            p_pend = __ldg(rowptr + 2 * part + 2);
            p_step = 0;
            if (p_pi.nsteps > 0) return;
            p_item += stride;
        }
    };
    auto issue = [&](int stage) {
        const uint32_t bar = sbar(stage);
        const int c0 = p_step * 16;
        const int vcols = min(16, p_pend - p_pi.start - c0);
        const uint32_t vbytes = (uint32_t)(vcols * W * 2);
        if (lane == 0) mbar_arrive_expect_tx(bar, C::FCH * 4 * 4 * kPitch + vbytes);
        int y[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {  // ids of rows 4*lane+i (prefetched one step ahead)
            int cidx = __shfl_sync(0xffffffffu, p_myc, (4 * lane + i) & 15);
            if (cidx >= n_x || cidx < -1) {
                if (err && lane < 4) atomicOr(err, 1);
                cidx = -1;
            }
            y[i] = cidx >= 0 ? cidx : oob_row;
        }
        (void)c0;
        __syncwarp();
        if (lane < 4) {
#pragma unroll
            for (int ch = 0; ch < C::FCH; ++ch) {
                const int64_t fb = (int64_t)p_fc * FC + 64 * ch;
                const int x = (int)(box_left(fb, F) ? fb - 16 : fb);
                tma_gather4(xstage(stage) + ch * C::CHUNK + lane * kGroup, &tmX, x, y[0], y[1], y[2],
                            y[3], bar);
            }
        } else if (lane == 4) {
            bulk_g2s(vtile(stage), val + (int64_t)(p_pi.start + c0) * W, vbytes, bar);
        }
    };
    // column ids of the producer's position, fetched one step ahead so the
    // load latency overlaps the consumer's work instead of stalling issue()
    auto p_fetch = [&]() {
        p_myc = -1;
        if (p_item < n_items && p_step * 16 + (lane & 15) < p_pi.nreal)
            p_myc = __ldg(col + p_pi.start + p_step * 16 + (lane & 15));
    };
    auto p_advance = [&]() {
        if (++p_step >= p_pi.nsteps) {
            p_item += stride;
            p_load();
        }
        p_fetch();
    };

    p_load();
    p_fetch();
    int inflight = 0;
#pragma unroll
    for (int s = 0; s < S - 1; ++s) {
        if (p_item < n_items) {
            issue(s);
            p_advance();
            ++inflight;
        }
    }

    float acc[C::MT][C::NT][4];
#pragma unroll
    for (int j = 0; j < C::MT; ++j)
#pragma unroll
        for (int t = 0; t < C::NT; ++t) acc[j][t][0] = acc[j][t][1] = acc[j][t][2] = acc[j][t][3] = 0.f;

    uint32_t phase = 0;  // bit s: parity of stage s's next completion
    int cstage = 0, pstage = S - 1;
    for (int64_t c_item = (int64_t)blockIdx.x * kWarps + warp; c_item < n_items; c_item += stride) {
        const int64_t part = c_item / n_chunks;
        const int fc = (int)(c_item - part * n_chunks);
        const PartInfo pi = part_info<WIDE>(rowptr, part, nullptr);
        for (int step = 0; step < pi.nsteps; ++step) {
            const uint32_t bar = sbar(cstage);
            if (!mbar_wait_bounded(bar, (phase >> cstage) & 1u, kMaxPolls)) {
                // give up: record it, drain the copies still in flight, leave
                if (lane == 0 && err) atomicOr(err, 4);
                for (int k = 1; k < inflight; ++k) {
                    const int s2 = (cstage + k) % S;
                    mbar_wait_bounded(sbar(s2), (phase >> s2) & 1u, kMaxPolls);
                }
                return;
            }
            phase ^= 1u << cstage;
            --inflight;
            const uint32_t vs = vtile(cstage);
            uint32_t b[C::NT][2];
            {
                const int q = lane >> 3, rr = lane & 7;
                if constexpr (C::NT == 2) {
                    const int kb = q & 1, r = (q >> 1) * 8 + rr;
                    const int e = (kb * 8 / WIDE) * W * WIDE + r * WIDE + (kb * 8) % WIDE;
                    ldsm_x4(vs + e * 2, b[0][0], b[0][1], b[1][0], b[1][1]);
                } else {
                    const int kb = q & 1, r = rr;
                    const int e = (kb * 8 / WIDE) * W * WIDE + r * WIDE + (kb * 8) % WIDE;
                    ldsm_x2(vs + e * 2, b[0][0], b[0][1]);
                }
            }
#pragma unroll
            for (int j = 0; j < C::MT; ++j) {
                const int q = lane >> 3, rr = lane & 7;
                const int k = (q >> 1) * 8 + rr;
                const int bx = j >> 2;  // 64-feature box
                const int fo = (box_left((int64_t)fc * FC + 64 * bx, F) ? 16 : 0) + (j & 3) * 16 +
                               (q & 1) * 8;
                uint32_t a[4];
                ldsm_x4_trans(xstage(cstage) + bx * C::CHUNK + (k >> 2) * kGroup + (k & 3) * kPitch +
                                  fo * 2,
                              a[0], a[1], a[2], a[3]);
#pragma unroll
                for (int t = 0; t < C::NT; ++t) mma_16816<T>(acc[j][t], a, b[t][0], b[t][1]);
            }
            __syncwarp();
            if (p_item < n_items) {
                fence_proxy_async_smem();
                issue(pstage);
                p_advance();
                ++inflight;
            }
            cstage = cstage + 1 == S ? 0 : cstage + 1;
            pstage = pstage + 1 == S ? 0 : pstage + 1;
        }
        const int wrow = __ldg(win + part);
        const bool add = __ldg(atomic + part) != 0;
        const int64_t f0 = (int64_t)fc * FC;
#pragma unroll
        for (int t = 0; t < C::NT; ++t) {
            const int64_t r0 = (int64_t)wrow * W + t * 8 + 2 * tig;
#pragma unroll
            for (int j = 0; j < C::MT; ++j) {
                const int64_t fa = f0 + 16 * j + gid;
#pragma unroll
                for (int h = 0; h < 4; ++h) {
                    const int64_t r = r0 + (h & 1);
                    const int64_t f = fa + (h >> 1) * 8;
                    if (r >= 0 && r < m_out && f < F) {
                        float *dst = Y + r * ldy + f;
                        if (add) red_add_f32(dst, acc[j][t][h]);
                        else *dst = acc[j][t][h];
                    }
                    acc[j][t][h] = 0.f;
                }
            }
        }
    }
}

// ---------------------------------------------------------------------------
// fp32 operand kernel: 3xTF32 m16n8k8
// ---------------------------------------------------------------------------
template <int W, int FC, int WIDE, int S = kStages>
struct CfgTF32 {
    static constexpr int XROW = FC * 4;
    static constexpr int XSTAGE = 16 * XROW;
    static constexpr int VSTAGE = 16 * W * 4;
    static constexpr int STAGE = XSTAGE + VSTAGE;
    static constexpr int WARP_SMEM = S * STAGE;
    static constexpr int SMEM = kWarps * WARP_SMEM;
    static constexpr int CPR = FC / 4;
    static constexpr int RPP = 32 / CPR;
    static constexpr int MT = FC / 16;
    static constexpr int NT = W / 8;
    static constexpr int VCH = VSTAGE / 16;
};


template <int W, int FC, int WIDE, int S>
__global__ void __launch_bounds__(kThreads) k_spmm_tf32(
    const int32_t *__restrict__ rowptr, const int32_t *__restrict__ col,
    const float *__restrict__ val, const int32_t *__restrict__ win,
    const int32_t *__restrict__ atomic, int64_t n_parts, const float *__restrict__ X, int64_t n_x,
    int64_t F, int64_t ldx, float *__restrict__ Y, int64_t m_out, int64_t ldy, int n_chunks,
    int32_t *__restrict__ err) {
    using C = CfgTF32<W, FC, WIDE, S>;
    extern __shared__ __align__(128) unsigned char smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t sbase = smem_u32(smem) + warp * C::WARP_SMEM;
    const unsigned char *sgen = smem + warp * C::WARP_SMEM;
    const int64_t n_items = n_parts * n_chunks;
    const int64_t stride = (int64_t)gridDim.x * kWarps;
    const int gid = lane >> 2, tig = lane & 3;

    int64_t p_item = (int64_t)blockIdx.x * kWarps + warp;
    int p_step = 0, p_fc = 0, p_myc = -1;
    PartInfo p_pi = {0, 0, 0};
    auto p_load = [&]() {
        while (p_item < n_items) {
            int64_t part = p_item / n_chunks;
            p_fc = (int)(p_item - part * n_chunks);
            p_pi = part_info<WIDE>(rowptr, part, err);
            p_step = 0;
            if (p_pi.nsteps > 0) return;
            p_item += stride;
        }
    };
    auto issue = [&](int stage) {
        const uint32_t xs = sbase + stage * C::STAGE;
        const uint32_t vs = xs + C::XSTAGE;
        const int c0 = p_step * 16;
        int myc = p_myc;  // loaded one step ahead
        const int64_t fbase = (int64_t)p_fc * FC;
#pragma unroll
        for (int i = 0; i < 16 / C::RPP; ++i) {
            const int r = i * C::RPP + lane / C::CPR;
            const int ch = lane % C::CPR;
            const int cidx = __shfl_sync(0xffffffffu, myc, r);
            const int64_t f = fbase + ch * 4;
            bool ok = cidx >= 0 && f < F;
            if (cidx >= n_x || cidx < -1) {
                if (err) atomicOr(err, 1);
                ok = false;
            }
            const float *src = ok ? X + (int64_t)cidx * ldx + f : X;
            cp_async16(xs + r * C::XROW + ((ch ^ ((r & 3) << 1)) << 4), src, ok ? 16 : 0);
        }
#pragma unroll
        for (int q = lane; q < C::VCH; q += 32) {
            const int e = q * 4;
            const int blk = e / (W * WIDE);
            const bool ok = c0 + blk * WIDE < p_pi.nreal;
            const float *src = val + ((int64_t)(p_pi.start + c0) * W + e);
            cp_async16(vs + q * 16, ok ? (const void *)src : (const void *)val, ok ? 16 : 0);
        }
    };
    // column ids of the producer's position, fetched one step ahead so the
    // load latency overlaps the consumer's work instead of stalling issue()
    auto p_fetch = [&]() {
        p_myc = -1;
        if (p_item < n_items && p_step * 16 + (lane & 15) < p_pi.nreal)
            p_myc = __ldg(col + p_pi.start + p_step * 16 + (lane & 15));
    };
    auto p_advance = [&]() {
        if (++p_step >= p_pi.nsteps) {
            p_item += stride;
            p_load();
        }
        p_fetch();
    };

    p_load();
    p_fetch();
#pragma unroll
    for (int s = 0; s < S - 1; ++s) {
        if (p_item < n_items) {
            issue(s);
            p_advance();
        }
        cp_async_commit();
    }

    float acc[C::MT][C::NT][4];
#pragma unroll
    for (int j = 0; j < C::MT; ++j)
#pragma unroll
        for (int t = 0; t < C::NT; ++t) acc[j][t][0] = acc[j][t][1] = acc[j][t][2] = acc[j][t][3] = 0.f;

    int cstage = 0, pstage = S - 1;
    for (int64_t c_item = (int64_t)blockIdx.x * kWarps + warp; c_item < n_items; c_item += stride) {
        const int64_t part = c_item / n_chunks;
        const int fc = (int)(c_item - part * n_chunks);
        const PartInfo pi = part_info<WIDE>(rowptr, part, err);
        for (int step = 0; step < pi.nsteps; ++step) {
            cp_async_wait<S - 2>();
            __syncwarp();
            const float *xsg = (const float *)(sgen + cstage * C::STAGE);
            const float *vsg = (const float *)(sgen + cstage * C::STAGE + C::XSTAGE);
#pragma unroll
            for (int h = 0; h < 2; ++h) {  // two k8 steps per 16-column stage
                uint32_t bh[C::NT][2], bl[C::NT][2];
#pragma unroll
                for (int t = 0; t < C::NT; ++t) {
#pragma unroll
                    for (int u = 0; u < 2; ++u) {
                        const int c = 8 * h + tig + 4 * u;
                        const int r = t * 8 + gid;
                        const float v = vsg[(c / WIDE) * W * WIDE + r * WIDE + c % WIDE];
                        split_tf32x3(v, bh[t][u], bl[t][u]);
                    }
                }
#pragma unroll
                for (int j = 0; j < C::MT; ++j) {
                    uint32_t ah[4], al[4];
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        const int k = 8 * h + tig + ((u >> 1) << 2);
                        const int f = 16 * j + gid + ((u & 1) << 3);
                        const int ch = f >> 2;
                        const float x = xsg[k * FC + (((ch ^ ((k & 3) << 1))) << 2) + (f & 3)];
                        split_tf32x3(x, ah[u], al[u]);
                    }
#pragma unroll
                    for (int t = 0; t < C::NT; ++t) {
                        mma_1688_tf32(acc[j][t], al[0], al[1], al[2], al[3], bh[t][0], bh[t][1]);
                        mma_1688_tf32(acc[j][t], ah[0], ah[1], ah[2], ah[3], bl[t][0], bl[t][1]);
                        mma_1688_tf32(acc[j][t], ah[0], ah[1], ah[2], ah[3], bh[t][0], bh[t][1]);
                    }
                }
            }
            __syncwarp();
            if (p_item < n_items) {
                issue(pstage);
                p_advance();
            }
            cp_async_commit();
            cstage = cstage + 1 == S ? 0 : cstage + 1;
            pstage = pstage + 1 == S ? 0 : pstage + 1;
        }
        const int wrow = __ldg(win + part);
        const bool add = __ldg(atomic + part) != 0;
        const int64_t f0 = (int64_t)fc * FC;
#pragma unroll
        for (int t = 0; t < C::NT; ++t) {
            const int64_t r0 = (int64_t)wrow * W + t * 8 + 2 * tig;
#pragma unroll
            for (int j = 0; j < C::MT; ++j) {
                const int64_t fa = f0 + 16 * j + gid;
#pragma unroll
                for (int h = 0; h < 4; ++h) {
                    const int64_t r = r0 + (h & 1);
                    const int64_t f = fa + (h >> 1) * 8;
                    if (r >= 0 && r < m_out && f < F) {
                        float *dst = Y + r * ldy + f;
                        if (add) red_add_f32(dst, acc[j][t][h]);
                        else *dst = acc[j][t][h];
                    }
                    acc[j][t][h] = 0.f;
                }
            }
        }
    }
    cp_async_wait<0>();
}

// ---------------------------------------------------------------------------
// FP8 E4M3 features with per-row fp32 scales (values fp16)
// ---------------------------------------------------------------------------
// The gathered rows are e4m3 (half the bytes of fp16), staged by 16-byte
// cp.async in a deep ring; the consumer dequantizes the step's 16 rows into
// one fp16 tile per warp -- cvt e4m3x2 -> f16x2 is exact, then one multiply by
// the row's scale (done here on X, where it cannot underflow to fp16
// subnormals as it could on the small block values) -- and runs the fp16
// ldmatrix.trans + mma.sync path with fp32 accumulation.
constexpr int kF8Stages = 3;

template <int W, int FC, int S = kF8Stages>
struct CfgF8 {
    static constexpr int XROW8 = FC;             // bytes per gathered e4m3 row
    static constexpr int XSTAGE = 16 * XROW8;
    static constexpr int VSTAGE = 16 * W * 2;
    static constexpr int SSTAGE = 64;            // 16 fp32 scales
    static constexpr int STAGE = XSTAGE + VSTAGE + SSTAGE;
    static constexpr int XROW16 = FC * 2;        // dequantized fp16 tile row
    static constexpr int TILE16 = 16 * XROW16;
    static constexpr int WARP_SMEM = S * STAGE + TILE16;
    static constexpr int SMEM = kWarps * WARP_SMEM;
    static constexpr int CPR = FC / 16;          // 16-byte e4m3 chunks per row
    static constexpr int MT = FC / 16;
    static constexpr int NT = W / 8;
    static constexpr int VCH = VSTAGE / 16;
};

__device__ __forceinline__ uint32_t e4m3x2_to_f16x2(uint16_t v) {
    uint32_t r;
    asm("cvt.rn.f16x2.e4m3x2 %0, %1;\n" : "=r"(r) : "h"(v));
    return r;
}

// IT: index type of items and element offsets (int32_t when they fit)
template <int W, int FC, int WIDE, typename IT>
__global__ void __launch_bounds__(kThreads) k_spmm_fp8(
    const int32_t *__restrict__ rowptr, const int32_t *__restrict__ col,
    const __half *__restrict__ val, const int32_t *__restrict__ win,
    const int32_t *__restrict__ atomic, int64_t n_parts, const uint8_t *__restrict__ X,
    const float *__restrict__ xscale, int64_t n_x_, int64_t F_, int64_t ldx_, float *__restrict__ Y,
    int64_t m_out_, int64_t ldy_, int n_chunks, int32_t *__restrict__ err) {
    const IT n_x = (IT)n_x_, F = (IT)F_, ldx = (IT)ldx_, m_out = (IT)m_out_, ldy = (IT)ldy_;
    using C = CfgF8<W, FC>;
    constexpr int S = kF8Stages;
    static_assert(C::WARP_SMEM == S * C::STAGE + C::TILE16, "layout");
    extern __shared__ __align__(128) unsigned char smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t sbase = smem_u32(smem) + warp * C::WARP_SMEM;
    const unsigned char *sgen = smem + warp * C::WARP_SMEM;
    const uint32_t tile = sbase + S * C::STAGE;
    const IT n_items = (IT)(n_parts * n_chunks);
    const IT stride = (IT)gridDim.x * kWarps;
    const int gid = lane >> 2, tig = lane & 3;

    IT p_item = (IT)blockIdx.x * kWarps + warp;
    int p_step = 0, p_fc = 0, p_myc = -1;
    PartInfo p_pi = {0, 0, 0};
    auto p_load = [&]() {
        while (p_item < n_items) {
            const IT part = p_item / n_chunks;
            p_fc = (int)(p_item - part * n_chunks);
            p_pi = part_info<WIDE>(rowptr, part, err);
            p_step = 0;
            if (p_pi.nsteps > 0) return;
            p_item += stride;
        }
    };
    auto issue = [&](int stage) {
        const uint32_t xs = sbase + stage * C::STAGE;
        const uint32_t vs = xs + C::XSTAGE;
        const uint32_t ss = vs + C::VSTAGE;
        const int c0 = p_step * 16;
        int myc = p_myc;  // loaded one step ahead
        if ((uint64_t)(int64_t)(myc + 1) > (uint64_t)n_x) {  // valid: -1 .. n_x - 1
            if (err) atomicOr(err, 1);
            myc = -1;
        }
        const IT fbase = (IT)p_fc * FC;
        const bool full = fbase + FC <= F;
#pragma unroll
        for (int i = 0; i < 16 * C::CPR / 32; ++i) {
            const int idx = i * 32 + lane;
            const int r = idx / C::CPR, ch = idx % C::CPR;
            const int cidx = __shfl_sync(0xffffffffu, myc, r);
            const IT f = fbase + ch * 16;
            const bool ok = cidx >= 0 && (full || f < F);
            const IT off = ok ? (IT)cidx * ldx + f : (IT)0;
            cp_async16(xs + r * C::XROW8 + ch * 16, X + off, ok ? 16 : 0);
        }
#pragma unroll
        for (int q = lane; q < C::VCH; q += 32) {
            const int e = q * 8;
            const int blk = e / (W * WIDE);
            const bool ok = c0 + blk * WIDE < p_pi.nreal;
            const __half *src = val + ((IT)(p_pi.start + c0) * W + e);
            cp_async16(vs + q * 16, ok ? (const void *)src : (const void *)val, ok ? 16 : 0);
        }
        if (lane < 16) {
            const bool ok = myc >= 0;
            asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(ss + 4 * lane),
                         "l"(ok ? xscale + myc : xscale), "r"(ok ? 4 : 0));
        }
    };
    // column ids of the producer's position, fetched one step ahead so the
    // load latency overlaps the consumer's work instead of stalling issue()
    auto p_fetch = [&]() {
        p_myc = -1;
        if (p_item < n_items && p_step * 16 + (lane & 15) < p_pi.nreal)
            p_myc = __ldg(col + p_pi.start + p_step * 16 + (lane & 15));
    };
    auto p_advance = [&]() {
        if (++p_step >= p_pi.nsteps) {
            p_item += stride;
            p_load();
        }
        p_fetch();
    };

    p_load();
    p_fetch();
#pragma unroll
    for (int s = 0; s < S - 1; ++s) {
        if (p_item < n_items) {
            issue(s);
            p_advance();
        }
        cp_async_commit();
    }

    float acc[C::MT][C::NT][4];
#pragma unroll
    for (int j = 0; j < C::MT; ++j)
#pragma unroll
        for (int t = 0; t < C::NT; ++t) acc[j][t][0] = acc[j][t][1] = acc[j][t][2] = acc[j][t][3] = 0.f;

    int cstage = 0, pstage = S - 1;
    for (IT c_item = (IT)blockIdx.x * kWarps + warp; c_item < n_items; c_item += stride) {
        const IT part = c_item / n_chunks;
        const int fc = (int)(c_item - part * n_chunks);
        const PartInfo pi = part_info<WIDE>(rowptr, part, nullptr);
        for (int step = 0; step < pi.nsteps; ++step) {
            cp_async_wait<S - 2>();
            __syncwarp();
            const unsigned char *x8 = sgen + cstage * C::STAGE;
            const float *sc = (const float *)(x8 + C::XSTAGE + C::VSTAGE);
            const uint32_t vs = sbase + cstage * C::STAGE + C::XSTAGE;
            // dequantize: 8 lanes per row, one 16-byte e4m3 chunk each
#pragma unroll
            for (int i = 0; i < 16 * C::CPR / 32; ++i) {
                const int idx = i * 32 + lane;
                const int r = idx / C::CPR, ch = idx % C::CPR;
                const uint4 raw = *reinterpret_cast<const uint4 *>(x8 + r * C::XROW8 + ch * 16);
                const __half2 s2 = __float2half2_rn(sc[r]);
                const uint32_t w[4] = {raw.x, raw.y, raw.z, raw.w};
                uint32_t h[8];
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    uint32_t lo = e4m3x2_to_f16x2((uint16_t)(w[k] & 0xffffu));
                    uint32_t hi = e4m3x2_to_f16x2((uint16_t)(w[k] >> 16));
                    __half2 l2 = __hmul2(*reinterpret_cast<__half2 *>(&lo), s2);
                    __half2 h2 = __hmul2(*reinterpret_cast<__half2 *>(&hi), s2);
                    h[2 * k] = *reinterpret_cast<uint32_t *>(&l2);
                    h[2 * k + 1] = *reinterpret_cast<uint32_t *>(&h2);
                }
                // fp16 chunks 2ch, 2ch+1 of row r, XOR-swizzled as in k_spmm16
#pragma unroll
                for (int u = 0; u < 2; ++u) {
                    const int c16 = 2 * ch + u;
                    const uint32_t dst = tile + r * C::XROW16 + ((c16 ^ swz<C::XROW16>(r)) << 4);
                    asm volatile("st.shared.v4.u32 [%0], {%1, %2, %3, %4};\n" ::"r"(dst),
                                 "r"(h[4 * u]), "r"(h[4 * u + 1]), "r"(h[4 * u + 2]),
                                 "r"(h[4 * u + 3])
                                 : "memory");
                }
            }
            __syncwarp();
            uint32_t b[C::NT][2];
            {
                const int q = lane >> 3, rr = lane & 7;
                if constexpr (C::NT == 2) {
                    const int kb = q & 1, r = (q >> 1) * 8 + rr;
                    const int e = (kb * 8 / WIDE) * W * WIDE + r * WIDE + (kb * 8) % WIDE;
                    ldsm_x4(vs + e * 2, b[0][0], b[0][1], b[1][0], b[1][1]);
                } else {
                    const int kb = q & 1, r = rr;
                    const int e = (kb * 8 / WIDE) * W * WIDE + r * WIDE + (kb * 8) % WIDE;
                    ldsm_x2(vs + e * 2, b[0][0], b[0][1]);
                }
            }
#pragma unroll
            for (int j = 0; j < C::MT; ++j) {
                const int q = lane >> 3, rr = lane & 7;
                const int k = (q >> 1) * 8 + rr;
                const int ch = 2 * j + (q & 1);
                uint32_t a[4];
                ldsm_x4_trans(tile + k * C::XROW16 + ((ch ^ swz<C::XROW16>(k)) << 4), a[0], a[1],
                              a[2], a[3]);
#pragma unroll
                for (int t = 0; t < C::NT; ++t) mma_16816<__half>(acc[j][t], a, b[t][0], b[t][1]);
            }
            __syncwarp();
            if (p_item < n_items) {
                issue(pstage);
                p_advance();
            }
            cp_async_commit();
            cstage = cstage + 1 == S ? 0 : cstage + 1;
            pstage = pstage + 1 == S ? 0 : pstage + 1;
        }
        const int wrow = __ldg(win + part);
        const bool add = __ldg(atomic + part) != 0;
        const IT f0 = (IT)fc * FC;
        const bool full = f0 + FC <= F;
#pragma unroll
        for (int t = 0; t < C::NT; ++t) {
            const IT r0 = (IT)wrow * W + t * 8 + 2 * tig;
#pragma unroll
            for (int j = 0; j < C::MT; ++j) {
                const IT fa = f0 + 16 * j + gid;
#pragma unroll
                for (int h = 0; h < 4; ++h) {
                    const IT r = r0 + (h & 1);
                    const IT f = fa + (h >> 1) * 8;
                    if (r < m_out && (full || f < F)) {
                        float *dst = Y + (r * ldy + f);
                        if (add) red_add_f32(dst, acc[j][t][h]);
                        else *dst = acc[j][t][h];
                    }
                    acc[j][t][h] = 0.f;
                }
            }
        }
    }
    cp_async_wait<0>();
}

// ---------------------------------------------------------------------------
// FP8 E4M3 features dequantized in registers (values fp16)
// ---------------------------------------------------------------------------
// Same staging ring as k_spmm_fp8, without the fp16 tile: ldmatrix.trans
// reads the e4m3 rows as 16-bit feature pairs, so each register holds
// features (f, f+1) of two gathered rows (c, c+1).  One byte permute regroups
// it into (f: c, c+1) | (f+1: c, c+1), and two cvt.e4m3x2 -> f16x2 give the A
// fragments of two MMA rows.  The per-row scales are folded into the B
// fragment (the step's block values, 16 gathered rows x 8 or 16 window rows):
// B' = fp16(V * s * 2^15), a few multiplies per step instead of one per A
// register, and the fp32 accumulators are multiplied by 2^-15 at the store
// (both factors are powers of two, so exact).  A step whose scaled values
// would leave fp16's normal range scales A by fp16(s) instead.  The MMA rows
// are a permutation of the features (row m < 8 is feature 2m of its
// 16-feature tile, row m + 8 is feature 2m + 1), which the epilogue undoes:
// each lane ends up owning two adjacent features of two window rows and
// stores them as float2.  This removes the shared-memory round trip of the
// fp16 tile (4 KB of shared traffic and four 16-byte stores per lane per
// step) and lets one work item cover 128 features.
constexpr float kF8Shift = 32768.f;
constexpr float kF8Unshift = 1.f / 32768.f;

__device__ __forceinline__ bool f16_normal_or_zero(float x) {
    const float a = fabsf(x);
    return a == 0.f || (a >= 6.103515625e-05f && a <= 65504.f);
}

template <int W, int FC, int S = kF8Stages>
struct CfgF8R {
    static constexpr int XROW = FC;              // bytes per gathered e4m3 row
    static constexpr int XSTAGE = 16 * XROW;
    static constexpr int VSTAGE = 16 * W * 2;
    static constexpr int SSTAGE = 64;            // 16 fp32 scales
    static constexpr int STAGE = XSTAGE + VSTAGE + SSTAGE;
    static constexpr int WARP_SMEM = S * STAGE;
    static constexpr int SMEM = kWarps * WARP_SMEM;
    static constexpr int CPR = FC / 16;          // 16-byte chunks per row
    static constexpr int RPP = 32 / CPR;         // rows per warp pass
    static constexpr int MT = FC / 16;           // 16-feature MMA tiles
    static constexpr int NT = W / 8;
    static constexpr int VCH = VSTAGE / 16;
};

__device__ __forceinline__ uint32_t hmul2_u32(uint32_t a, __half2 s) {
    __half2 r = __hmul2(*reinterpret_cast<__half2 *>(&a), s);
    return *reinterpret_cast<uint32_t *>(&r);
}

template <int W, int FC, int WIDE, typename IT, bool FULL>
__global__ void __launch_bounds__(kThreads) k_spmm_fp8r(
    const int32_t *__restrict__ rowptr, const int32_t *__restrict__ col,
    const __half *__restrict__ val, const int32_t *__restrict__ win,
    const int32_t *__restrict__ atomic, int64_t n_parts, const uint8_t *__restrict__ X,
    const float *__restrict__ xscale, int64_t n_x_, int64_t F_, int64_t ldx_, float *__restrict__ Y,
    int64_t m_out_, int64_t ldy_, int n_chunks, int vec_out, int32_t *__restrict__ err) {
    const IT n_x = (IT)n_x_, F = (IT)F_, ldx = (IT)ldx_, m_out = (IT)m_out_, ldy = (IT)ldy_;
    using C = CfgF8R<W, FC>;
    constexpr int S = kF8Stages;
    extern __shared__ __align__(128) unsigned char smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t sbase = smem_u32(smem) + warp * C::WARP_SMEM;
    const unsigned char *sgen = smem + warp * C::WARP_SMEM;
    const IT n_items = (IT)(n_parts * n_chunks);
    const IT stride = (IT)gridDim.x * kWarps;
    const int gid = lane >> 2, tig = lane & 3;

    IT p_item = (IT)blockIdx.x * kWarps + warp;
    int p_step = 0, p_fc = 0, p_myc = -1;
    PartInfo p_pi = {0, 0, 0};
    auto p_load = [&]() {
        while (p_item < n_items) {
            const IT part = p_item / n_chunks;
            p_fc = (int)(p_item - part * n_chunks);
            p_pi = part_info<WIDE>(rowptr, part, err);
            p_step = 0;
            if (p_pi.nsteps > 0) return;
            p_item += stride;
        }
    };
    auto issue = [&](int stage) {
        const uint32_t xs = sbase + stage * C::STAGE;
        const uint32_t vs = xs + C::XSTAGE;
        const uint32_t ss = vs + C::VSTAGE;
        const int c0 = p_step * 16;
        int myc = p_myc;  // loaded one step ahead
        if ((uint64_t)(int64_t)(myc + 1) > (uint64_t)n_x) {  // valid: -1 .. n_x - 1
            if (err) atomicOr(err, 1);
            myc = -1;
        }
        const IT fbase = (IT)p_fc * FC;
        const bool full = FULL || fbase + FC <= F;
#pragma unroll
        for (int i = 0; i < 16 / C::RPP; ++i) {
            const int r = i * C::RPP + lane / C::CPR;
            const int ch = lane % C::CPR;
            const int cidx = __shfl_sync(0xffffffffu, myc, r);
            const IT f = fbase + ch * 16;
            const bool ok = cidx >= 0 && (full || f < F);
            const IT off = ok ? (IT)cidx * ldx + f : (IT)0;
            cp_async16(xs + r * C::XROW + ((ch ^ swz<C::XROW>(r)) << 4), X + off, ok ? 16 : 0);
        }
#pragma unroll
        for (int q = lane; q < C::VCH; q += 32) {
            const int e = q * 8;
            const int blk = e / (W * WIDE);
            const bool ok = c0 + blk * WIDE < p_pi.nreal;
            const __half *src = val + ((IT)(p_pi.start + c0) * W + e);
            cp_async16(vs + q * 16, ok ? (const void *)src : (const void *)val, ok ? 16 : 0);
        }
        if (lane < 16) {
            const bool ok = myc >= 0;
            asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(ss + 4 * lane),
                         "l"(ok ? xscale + myc : xscale), "r"(ok ? 4 : 0));
        }
    };
    auto p_fetch = [&]() {
        p_myc = -1;
        if (p_item < n_items && p_step * 16 + (lane & 15) < p_pi.nreal)
            p_myc = __ldg(col + p_pi.start + p_step * 16 + (lane & 15));
    };
    auto p_advance = [&]() {
        if (++p_step >= p_pi.nsteps) {
            p_item += stride;
            p_load();
        }
        p_fetch();
    };

    p_load();
    p_fetch();
#pragma unroll
    for (int s = 0; s < S - 1; ++s) {
        if (p_item < n_items) {
            issue(s);
            p_advance();
        }
        cp_async_commit();
    }

    float acc[C::MT][C::NT][4];
#pragma unroll
    for (int j = 0; j < C::MT; ++j)
#pragma unroll
        for (int t = 0; t < C::NT; ++t) acc[j][t][0] = acc[j][t][1] = acc[j][t][2] = acc[j][t][3] = 0.f;

    // ldmatrix lane roles: matrix mi = lane / 8 holds gathered rows
    // (mi / 2) * 8 + lane % 8 and 16-feature chunk (mi % 2) of a 32-feature pair
    const int lm_k = ((lane >> 4) << 3) + (lane & 7);
    const int lm_h = (lane >> 3) & 1;
    int cstage = 0, pstage = S - 1;
    for (IT c_item = (IT)blockIdx.x * kWarps + warp; c_item < n_items; c_item += stride) {
        const IT part = c_item / n_chunks;
        const int fc = (int)(c_item - part * n_chunks);
        const PartInfo pi = part_info<WIDE>(rowptr, part, nullptr);
        for (int step = 0; step < pi.nsteps; ++step) {
            cp_async_wait<S - 2>();
            __syncwarp();
            const uint32_t xs = sbase + cstage * C::STAGE;
            const uint32_t vs = xs + C::XSTAGE;
            const float *sc = (const float *)(sgen + cstage * C::STAGE + C::XSTAGE + C::VSTAGE);
            // scale pairs of the gathered rows this lane's A fragments hold:
            // rows (2 tig, 2 tig + 1) and (8 + 2 tig, 9 + 2 tig)
            const float2 s_lo = *reinterpret_cast<const float2 *>(sc + 2 * tig);
            const float2 s_hi = *reinterpret_cast<const float2 *>(sc + 8 + 2 * tig);
            uint32_t b[C::NT][2];
            {
                const int q = lane >> 3, rr = lane & 7;
                if constexpr (C::NT == 2) {
                    const int kb = q & 1, r = (q >> 1) * 8 + rr;
                    const int e = (kb * 8 / WIDE) * W * WIDE + r * WIDE + (kb * 8) % WIDE;
                    ldsm_x4(vs + e * 2, b[0][0], b[0][1], b[1][0], b[1][1]);
                } else {
                    const int kb = q & 1, r = rr;
                    const int e = (kb * 8 / WIDE) * W * WIDE + r * WIDE + (kb * 8) % WIDE;
                    ldsm_x2(vs + e * 2, b[0][0], b[0][1]);
                }
            }
            // The row scales go on the B fragment: b[t][0] holds the values of
            // gathered rows (2 tig, 2 tig + 1), b[t][1] of (8 + 2 tig, 9 + 2 tig),
            // exactly the rows of the lane's scale pairs.  V * s is multiplied
            // by kF8Shift (2^15) into fp16's normal range, so the accumulators
            // hold 2^15 * Y until the store; if any scaled value of the step
            // would be neither zero nor a normal fp16, the warp scales A
            // instead for that step (accumulators brought back to 1 * Y around
            // it, exact: powers of two).
            uint32_t bs[C::NT][2];
            bool ok = true;
#pragma unroll
            for (int t = 0; t < C::NT; ++t) {
#pragma unroll
                for (int g = 0; g < 2; ++g) {
                    const float2 v = __half22float2(*reinterpret_cast<const __half2 *>(&b[t][g]));
                    const float2 sg = g == 0 ? s_lo : s_hi;
                    const float p0 = v.x * sg.x * kF8Shift, p1 = v.y * sg.y * kF8Shift;
                    ok = ok && f16_normal_or_zero(p0) && f16_normal_or_zero(p1);
                    const __half2 hp = __floats2half2_rn(p0, p1);
                    bs[t][g] = *reinterpret_cast<const uint32_t *>(&hp);
                }
            }
            const bool bside = __all_sync(0xffffffffu, ok);
            __half2 h_lo, h_hi;
            if (!bside) {
                h_lo = __floats2half2_rn(s_lo.x, s_lo.y);
                h_hi = __floats2half2_rn(s_hi.x, s_hi.y);
#pragma unroll
                for (int j = 0; j < C::MT; ++j)
#pragma unroll
                    for (int t = 0; t < C::NT; ++t)
#pragma unroll
                        for (int q = 0; q < 4; ++q) acc[j][t][q] *= kF8Unshift;
            }
#pragma unroll
            for (int jp = 0; jp < C::MT / 2; ++jp) {
                const int ch = 2 * jp + lm_h;
                uint32_t R[4];  // (rows 0-7 | 8-15) x (tile 2jp | 2jp+1)
                ldsm_x4_trans(xs + lm_k * C::XROW + ((ch ^ swz<C::XROW>(lm_k)) << 4), R[0], R[1],
                              R[2], R[3]);
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    // bytes (f: c, f+1: c, f: c+1, f+1: c+1) -> (f: c, c+1 | f+1: c, c+1)
                    const uint32_t p0 = __byte_perm(R[h], 0, 0x3120);      // rows 2tig, 2tig+1
                    const uint32_t p1 = __byte_perm(R[h + 2], 0, 0x3120);  // rows 8+2tig, 9+2tig
                    uint32_t a[4];
                    a[0] = e4m3x2_to_f16x2((uint16_t)(p0 & 0xffffu));
                    a[1] = e4m3x2_to_f16x2((uint16_t)(p0 >> 16));
                    a[2] = e4m3x2_to_f16x2((uint16_t)(p1 & 0xffffu));
                    a[3] = e4m3x2_to_f16x2((uint16_t)(p1 >> 16));
                    if (bside) {
#pragma unroll
                        for (int t = 0; t < C::NT; ++t)
                            mma_16816<__half>(acc[2 * jp + h][t], a, bs[t][0], bs[t][1]);
                    } else {
                        a[0] = hmul2_u32(a[0], h_lo);
                        a[1] = hmul2_u32(a[1], h_lo);
                        a[2] = hmul2_u32(a[2], h_hi);
                        a[3] = hmul2_u32(a[3], h_hi);
#pragma unroll
                        for (int t = 0; t < C::NT; ++t)
                            mma_16816<__half>(acc[2 * jp + h][t], a, b[t][0], b[t][1]);
                    }
                }
            }
            if (!bside) {
#pragma unroll
                for (int j = 0; j < C::MT; ++j)
#pragma unroll
                    for (int t = 0; t < C::NT; ++t)
#pragma unroll
                        for (int q = 0; q < 4; ++q) acc[j][t][q] *= kF8Shift;
            }
            __syncwarp();
            if (p_item < n_items) {
                issue(pstage);
                p_advance();
            }
            cp_async_commit();
            cstage = cstage + 1 == S ? 0 : cstage + 1;
            pstage = pstage + 1 == S ? 0 : pstage + 1;
        }
        // epilogue: tile j, lane -> features f0 + 16 j + 2 gid (+1), window
        // rows t * 8 + 2 tig (+1); F is a multiple of 16, so both features of
        // a pair are inside F together
        const int wrow = __ldg(win + part);
        const bool add = __ldg(atomic + part) != 0;
        const IT f0 = (IT)fc * FC;
#pragma unroll
        for (int t = 0; t < C::NT; ++t) {
            const IT r0 = (IT)wrow * W + t * 8 + 2 * tig;
#pragma unroll
            for (int j = 0; j < C::MT; ++j) {
                const IT f = f0 + 16 * j + 2 * gid;
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const IT r = r0 + h;
                    const float v0 = acc[j][t][h] * kF8Unshift, v1 = acc[j][t][h + 2] * kF8Unshift;
                    if (r < m_out && (FULL || f < F)) {
                        float *dst = Y + (r * ldy + f);
                        if (add) {
                            red_add_f32(dst, v0);
                            red_add_f32(dst + 1, v1);
                        } else if (vec_out) {
                            *reinterpret_cast<float2 *>(dst) = make_float2(v0, v1);
                        } else {
                            dst[0] = v0;
                            dst[1] = v1;
                        }
                    }
                    acc[j][t][h] = acc[j][t][h + 2] = 0.f;
                }
            }
        }
    }
    cp_async_wait<0>();
}

// ---------------------------------------------------------------------------
// Batched SpMM over many graphs in one launch (the serving loop's kernel)
// ---------------------------------------------------------------------------
// The job table lives in device memory: a header {n_jobs, total items, total
// empty windows, total multi-group windows, work counter} and, per job, the
// block format, its groups, X and Y of one graph plus exclusive prefixes of its
// work items (groups x feature chunks), empty windows and multi-group windows.
// Launch parameters are only the table pointers, so one launch captured in a
// CUDA graph can be replayed every scheduler tick after the table is
// rewritten.  A group (<= group_parts consecutive parts of one window, chosen
// when the groups are built) is one contiguous run of condensed columns, so it
// streams like one long part.  Warps take work items from a queue (the
// counter header[4]): the first item of each warp is fixed, the rest come
// from an atomic counter, which evens out items of very different lengths
// (one step to 16 x group_parts steps).  The per-warp cp.async pipeline runs
// across item and job boundaries as in k_spmm16; a small per-warp ring in
// shared memory hands the producer's item sequence to the consumer.

// find the job whose [begin, next begin) range of `which` (0 items, 1 empty
// windows, 2 multi-group windows) holds v
__device__ __forceinline__ int64_t find_prefix(const att_spmm_job *__restrict__ jobs, int64_t n_jobs,
                                               int64_t v, int which) {
    int64_t lo = 0, hi = n_jobs - 1;
    while (lo < hi) {
        const int64_t mid = (lo + hi + 1) >> 1;
        const int64_t b = which == 0 ? jobs[mid].item_begin
                          : which == 1 ? jobs[mid].empty_begin : jobs[mid].red_begin;
        if (b <= v) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// Condensed-column run of parts [p0, p1) of one window.  At least one step
// (an item whose run is empty -- only a malformed part -- streams one step
// of zeros and stores zeros).
template <int WIDE>
__device__ __forceinline__ PartInfo group_info(const int32_t *__restrict__ rowptr, int64_t p0,
                                               int64_t p1, int32_t *err) {
    PartInfo pi;
    pi.start = __ldg(rowptr + 2 * p0);
    const int e = __ldg(rowptr + 2 * (p1 - 1) + 1);
    const int pend = __ldg(rowptr + 2 * p1);
    pi.nreal = e > pi.start ? e - pi.start : 0;
    if ((pi.start % WIDE) != 0 || (pend % WIDE) != 0 || pend < pi.start + pi.nreal) {
        if (err) atomicOr(err, 2);
        pi.nreal = 0;
    }
    pi.nsteps = pi.nreal > 0 ? (pi.nreal + 15) >> 4 : 1;
    return pi;
}

constexpr int kRing = 8;  // >= S + 2 items in flight per warp

// A job's element offsets (X rows, Y rows, partial slots) fit in 31 bits:
// the batched kernel computes them in 32-bit arithmetic and skips (error bit
// 8) a job that does not fit instead of addressing it.
__device__ __forceinline__ bool job_small(const att_spmm_job *j) {
    const int64_t lim = (int64_t)INT32_MAX - 4096;
    return j->n_x * j->ldx < lim && j->m_out * j->ldy < lim && j->n_slots * 8 * j->F < lim &&
           j->F < lim && j->ldx < lim && j->ldy < lim;
}

// 8 CTAs per SM (64 registers): like k_spmm16, throughput follows resident warps
template <int W, int FC, int WIDE, int S>
__global__ void __launch_bounds__(kThreads, 8) k_spmm16_batched(const att_spmm_job *__restrict__ jobs,
                                                                int64_t *__restrict__ header,
                                                                int32_t *__restrict__ err) {
    static_assert(kRing >= S + 2, "item ring too small");
    using T = __half;
    using C = Cfg16<T, W, FC, WIDE, S>;
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ int ring[kWarps][kRing];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t sbase = smem_u32(smem) + warp * C::WARP_SMEM;
    const int64_t n_jobs = header[0];
    const int n_fixed = (int)gridDim.x * kWarps;
    if (header[1] > (int64_t)INT32_MAX - n_fixed - 1) {  // items must be 32-bit
        if (err && threadIdx.x == 0 && blockIdx.x == 0) atomicOr(err, 8);
        return;
    }
    const int n_items = (int)header[1];
    unsigned int *const counter = reinterpret_cast<unsigned int *>(header + 4);
    const int gid = lane >> 2, tig = lane & 3;
    int pq = 0, cq = 0;

    auto next_item = [&]() -> int {
        unsigned int v = 0;
        if (lane == 0) v = atomicAdd(counter, 1u);
        v = __shfl_sync(0xffffffffu, v, 0);
        return n_fixed + (int)v;
    };

    // producer cursor and the fields of its job it uses every step
    int p_item = (int)blockIdx.x * kWarps + warp;
    int p_step = 0, p_fc = 0, p_myc = -1;
    PartInfo p_pi = {0, 0, 0};
    const T *p_X = nullptr, *p_val = nullptr;  // p_val: the group's first value
    const int32_t *p_col = nullptr;             // the group's first column id
    int p_ldx = 0, p_nx = 0, p_F = 0;
    // load item p_item (or the end marker) and hand it to the consumer
    auto p_load = [&]() {
        ring[warp][pq % kRing] = p_item;  // every lane writes the same value and reads its own
        ++pq;
        if (p_item >= n_items) return;
        const att_spmm_job *pj = jobs + find_prefix(jobs, n_jobs, p_item, 0);
        const int local = (int)(p_item - pj->item_begin);
        p_F = (int)pj->F;
        const int nch = (p_F + FC - 1) / FC;
        const int g = local / nch;
        p_fc = local - g * nch;
        p_X = (const T *)pj->X;
        p_ldx = (int)pj->ldx;
        p_nx = (int)pj->n_x;
        p_pi = group_info<WIDE>(pj->rowptr, __ldg(pj->group_part + g), __ldg(pj->group_part + g + 1),
                                err);
        p_val = (const T *)pj->val + p_pi.start * W;
        p_col = pj->col + p_pi.start;
        if (!job_small(pj)) {  // not addressed: one zero step, no store
            if (err) atomicOr(err, 8);
            p_pi.nreal = 0;
            p_pi.nsteps = 1;
        }
        p_step = 0;
    };
    auto p_fetch = [&]() {
        p_myc = -1;
        if (p_item < n_items && p_step * 16 + (lane & 15) < p_pi.nreal)
            p_myc = __ldg(p_col + p_step * 16 + (lane & 15));
    };
    auto issue = [&](int stage) {
        const uint32_t xs = sbase + stage * C::STAGE;
        const uint32_t vs = xs + C::XSTAGE;
        const int c0 = p_step * 16;
        int myc = p_myc;
        // valid ids are -1 (padding) .. n_x - 1: checked once per id
        if ((unsigned)(myc + 1) > (unsigned)p_nx) {
            if (err) atomicOr(err, 1);
            myc = -1;
        }
        const int fbase = p_fc * FC;
        const bool full = fbase + FC <= p_F;
#pragma unroll
        for (int i = 0; i < 16 / C::RPP; ++i) {
            const int r = i * C::RPP + lane / C::CPR;
            const int ch = lane % C::CPR;
            const int cidx = __shfl_sync(0xffffffffu, myc, r);
            const int f = fbase + ch * 8;
            const bool ok = cidx >= 0 && (full || f < p_F);
            const int off = ok ? cidx * p_ldx + f : 0;
            cp_async16(xs + r * C::XROW + ((ch ^ swz<C::XROW>(r)) << 4), p_X + off, ok ? 16 : 0);
        }
#pragma unroll
        for (int q = lane; q < C::VCH; q += 32) {
            const int e = q * 8;
            const int blk = e / (W * WIDE);
            const bool ok = c0 + blk * WIDE < p_pi.nreal;
            const T *src = p_val + (c0 * W + e);
            cp_async16(vs + q * 16, ok ? (const void *)src : (const void *)p_val, ok ? 16 : 0);
        }
    };
    auto p_advance = [&]() {
        if (++p_step >= p_pi.nsteps) {
            p_item = next_item();
            p_load();
        }
        p_fetch();
    };

    p_load();
    p_fetch();
#pragma unroll
    for (int s = 0; s < S - 1; ++s) {
        if (p_item < n_items) {
            issue(s);
            p_advance();
        }
        cp_async_commit();
    }

    float acc[C::MT][C::NT][4];
#pragma unroll
    for (int j = 0; j < C::MT; ++j)
#pragma unroll
        for (int t = 0; t < C::NT; ++t) acc[j][t][0] = acc[j][t][1] = acc[j][t][2] = acc[j][t][3] = 0.f;

    int cstage = 0, pstage = S - 1;
    for (;;) {
        const int c_item = ring[warp][cq % kRing];
        ++cq;
        if (c_item >= n_items) break;
        const att_spmm_job *cj = jobs + find_prefix(jobs, n_jobs, c_item, 0);
        const int local = (int)(c_item - cj->item_begin);
        const int F = (int)cj->F;
        const int nch = (F + FC - 1) / FC;
        const int g = local / nch;
        const int fc = local - g * nch;
        const int gp0 = __ldg(cj->group_part + g);
        PartInfo pi = group_info<WIDE>(cj->rowptr, gp0, __ldg(cj->group_part + g + 1), nullptr);
        const bool small = job_small(cj);
        if (!small) pi.nsteps = 1;  // the producer streamed one zero step
        for (int step = 0; step < pi.nsteps; ++step) {
            cp_async_wait<S - 2>();
            __syncwarp();
            const uint32_t xs = sbase + cstage * C::STAGE;
            const uint32_t vs = xs + C::XSTAGE;
            uint32_t b[C::NT][2];
            {
                const int q = lane >> 3, rr = lane & 7;
                if constexpr (C::NT == 2) {
                    const int kb = q & 1, r = (q >> 1) * 8 + rr;
                    const int e = (kb * 8 / WIDE) * W * WIDE + r * WIDE + (kb * 8) % WIDE;
                    ldsm_x4(vs + e * 2, b[0][0], b[0][1], b[1][0], b[1][1]);
                } else {
                    const int kb = q & 1, r = rr;
                    const int e = (kb * 8 / WIDE) * W * WIDE + r * WIDE + (kb * 8) % WIDE;
                    ldsm_x2(vs + e * 2, b[0][0], b[0][1]);
                }
            }
#pragma unroll
            for (int j = 0; j < C::MT; ++j) {
                const int q = lane >> 3, rr = lane & 7;
                const int k = (q >> 1) * 8 + rr;
                const int ch = 2 * j + (q & 1);
                uint32_t a[4];
                ldsm_x4_trans(xs + k * C::XROW + ((ch ^ swz<C::XROW>(k)) << 4), a[0], a[1], a[2],
                              a[3]);
#pragma unroll
                for (int t = 0; t < C::NT; ++t) mma_16816<T>(acc[j][t], a, b[t][0], b[t][1]);
            }
            __syncwarp();
            if (p_item < n_items) {
                issue(pstage);
                p_advance();
            }
            cp_async_commit();
            cstage = cstage + 1 == S ? 0 : cstage + 1;
            pstage = pstage + 1 == S ? 0 : pstage + 1;
        }
        const int wrow = __ldg(cj->window_of_part + gp0);
        const int slot = __ldg(cj->group_slot + g);
        const int f0 = fc * FC;
        const bool full = f0 + FC <= F;
        const int m_out = (int)cj->m_out;
        // whole window: rows of Y; else rows of partial slot `slot` ([8, F], ld F)
        float *const base = slot < 0 ? cj->Y + wrow * W * (int)cj->ldy : cj->partial + slot * W * F;
        const int ld = slot < 0 ? (int)cj->ldy : F;
#pragma unroll
        for (int t = 0; t < C::NT; ++t) {
            const int rl0 = t * 8 + 2 * tig;
#pragma unroll
            for (int j = 0; j < C::MT; ++j) {
                const int fa = f0 + 16 * j + gid;
#pragma unroll
                for (int h = 0; h < 4; ++h) {
                    const int rl = rl0 + (h & 1);
                    const int f = fa + (h >> 1) * 8;
                    if (small && rl < W && wrow * W + rl < m_out && (full || f < F))
                        base[rl * ld + f] = acc[j][t][h];
                    acc[j][t][h] = 0.f;
                }
            }
        }
    }
    cp_async_wait<0>();
}

// First pass of the batched SpMM: resets the work counter and zeroes the
// rows of windows that own no part (listed per job in empty_win; one warp per
// window).
template <int W>
__global__ void k_zero_empty_batched(const att_spmm_job *__restrict__ jobs, int64_t *__restrict__ header) {
    if (blockIdx.x == 0 && threadIdx.x == 0) header[4] = 0;
    const int lane = threadIdx.x & 31;
    const int64_t n_jobs = header[0], n_e = header[2];
    const int64_t wstride = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t ge = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; ge < n_e; ge += wstride) {
        const att_spmm_job *j = jobs + find_prefix(jobs, n_jobs, ge, 1);
        const int64_t w = __ldg(j->empty_win + (ge - j->empty_begin));
        const int64_t r1 = (w + 1) * W < j->m_out ? (w + 1) * W : j->m_out;
        for (int64_t r = w * W; r < r1; ++r)
            for (int64_t f = lane; f < j->F; f += 32) j->Y[r * j->ldy + f] = 0.f;
    }
}

// Last pass: Y rows of a multi-group window = sum of its groups' partial slots
// in group order.  One CTA per window; a thread per (row, 4 features).  The
// window's slots are consecutive: [group_slot[first group], group_slot[first
// group of the next multi-group window]) (n_slots after the last).
template <int W>
__global__ void __launch_bounds__(256) k_reduce_groups_batched(const att_spmm_job *__restrict__ jobs,
                                                               const int64_t *__restrict__ header) {
    const int64_t n_jobs = header[0], n_r = header[3];
    for (int64_t gr = blockIdx.x; gr < n_r; gr += gridDim.x) {
        const att_spmm_job *j = jobs + find_prefix(jobs, n_jobs, gr, 2);
        if (!job_small(j)) continue;  // skipped by the main pass (error bit 8)
        const int64_t k = gr - j->red_begin;
        const int g0 = __ldg(j->red_first + k);
        const int64_t w = __ldg(j->window_of_part + __ldg(j->group_part + g0));
        const int s0 = __ldg(j->group_slot + g0);
        const int s1 = k + 1 < j->n_red ? __ldg(j->group_slot + __ldg(j->red_first + k + 1))
                                        : (int)j->n_slots;
        const int64_t F = j->F, F4 = F >> 2;
        const float4 *part = reinterpret_cast<const float4 *>(j->partial);
        for (int64_t u = threadIdx.x; u < W * F4; u += blockDim.x) {
            const int64_t rl = u / F4, f4 = u - rl * F4;
            const int64_t r = w * W + rl;
            if (r >= j->m_out) continue;
            float4 s = make_float4(0.f, 0.f, 0.f, 0.f);
            int sl = s0;
#pragma unroll 4
            for (; sl < s1; ++sl) {
                const float4 v = __ldg(part + ((int64_t)sl * W + rl) * F4 + f4);
                s.x += v.x;
                s.y += v.y;
                s.z += v.z;
                s.w += v.w;
            }
            float *y = j->Y + r * j->ldy + f4 * 4;
            y[0] = s.x;
            y[1] = s.y;
            y[2] = s.z;
            y[3] = s.w;
        }
    }
}

// ---- groups of a block format -------------------------------------------------
// Per part p of window w (parts of a window are consecutive): rank = p - first
// part of w, np = parts of w.  p starts a group when rank % G == 0; a window
// with np > G is multi-group: each of its groups owns a partial slot and its
// first group opens a reduction entry.  The three flags are packed in 21-bit
// fields of one int64 and scanned together.  Empty windows (no part) below
// n_windows are listed by a second scan.
constexpr int kFieldBits = 21;
constexpr int64_t kFieldMask = (int64_t(1) << kFieldBits) - 1;

__device__ __forceinline__ int64_t lower_bound_win(const int32_t *__restrict__ win, int64_t P, int64_t w) {
    int64_t a = 0, b = P;
    while (a < b) {
        const int64_t m = (a + b) >> 1;
        if (__ldg(win + m) < w) a = m + 1; else b = m;
    }
    return a;
}

__device__ __forceinline__ void part_rank(const int32_t *__restrict__ win, int64_t P, int64_t p,
                                          int64_t &rank, int64_t &np) {
    const int32_t w = __ldg(win + p);
    int64_t a = 0, b = p;
    while (a < b) {
        const int64_t m = (a + b) >> 1;
        if (__ldg(win + m) < w) a = m + 1; else b = m;
    }
    int64_t c = p + 1, d = P;
    while (c < d) {
        const int64_t m = (c + d) >> 1;
        if (__ldg(win + m) <= w) c = m + 1; else d = m;
    }
    rank = p - a;
    np = c - a;
}

__global__ void k_group_flags(const int32_t *__restrict__ win, int64_t P, int G,
                              int64_t *__restrict__ flags) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P) return;
    int64_t rank, np;
    part_rank(win, P, p, rank, np);
    const int64_t gs = rank % G == 0, multi = np > G;
    flags[p] = gs | ((gs & multi) << kFieldBits) | ((int64_t)(multi && rank == 0) << (2 * kFieldBits));
}

__global__ void k_group_scatter(const int32_t *__restrict__ win, int64_t P, int G,
                                const int64_t *__restrict__ scanned, int32_t *__restrict__ group_part,
                                int32_t *__restrict__ group_slot, int32_t *__restrict__ red_first,
                                int64_t *__restrict__ counts) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (P == 0) {
        if (p == 0) {
            group_part[0] = 0;
            red_first[0] = 0;
            counts[0] = counts[1] = counts[2] = 0;
        }
        return;
    }
    if (p >= P) return;
    int64_t rank, np;
    part_rank(win, P, p, rank, np);
    const bool gs = rank % G == 0, multi = np > G;
    const int64_t ex = scanned[p];
    const int64_t gi = ex & kFieldMask, si = (ex >> kFieldBits) & kFieldMask, ri = ex >> (2 * kFieldBits);
    if (gs) {
        group_part[gi] = (int32_t)p;
        group_slot[gi] = multi ? (int32_t)si : -1;
    }
    if (multi && rank == 0) red_first[ri] = (int32_t)gi;
    if (p == P - 1) {
        const int64_t ng = gi + gs, ns = si + (gs && multi), nr = ri + (multi && rank == 0);
        group_part[ng] = (int32_t)P;
        red_first[nr] = (int32_t)ng;
        counts[0] = ng;
        counts[1] = nr;
        counts[2] = ns;
    }
}

__global__ void k_empty_flags(const int32_t *__restrict__ win, int64_t P, int64_t n_windows,
                              int64_t *__restrict__ flags) {
    const int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= n_windows) return;
    const int64_t a = lower_bound_win(win, P, w);
    flags[w] = !(a < P && __ldg(win + a) == w);
}

__global__ void k_empty_scatter(const int32_t *__restrict__ win, int64_t P, int64_t n_windows,
                                const int64_t *__restrict__ scanned, int32_t *__restrict__ empty_win,
                                int64_t *__restrict__ counts) {
    const int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (n_windows == 0) {
        if (w == 0) counts[3] = 0;
        return;
    }
    if (w >= n_windows) return;
    const int64_t a = lower_bound_win(win, P, w);
    const bool empty = !(a < P && __ldg(win + a) == w);
    if (empty) empty_win[scanned[w]] = (int32_t)w;
    if (w == n_windows - 1) counts[3] = scanned[w] + empty;
}

// Outputs up to this size are zeroed whole before the SpMM kernel (one
// memset, a few microseconds); larger ones by k_zero_uncovered.
constexpr size_t kZeroAllBytes = 32ull << 20;

// Zeroes the rows of Y that no unsplit part stores (windows whose parts add
// with red.add, windows without parts, rows past the last window), before
// the SpMM kernel.  Thread per part, plus one thread for the end: the first
// part of each window zeroes the windows between the previous part's window
// and its own, and its own window when that window is split; the extra
// thread zeroes the windows after the last part's.  No searches: every
// thread reads at most two window ids and one flag, coalesced.  The warp
// zeroes each lane's rows together.
__global__ void k_zero_uncovered(const int32_t *__restrict__ win, const int32_t *__restrict__ atomic,
                                 int64_t n_parts, int W, float *__restrict__ Y, int64_t m_out,
                                 int64_t F, int64_t ldy) {
    const int lane = threadIdx.x & 31;
    const int64_t n_w = (m_out + W - 1) / W;
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int64_t g0 = 0, g1 = 0, own = -1;  // gap [g0, g1) and the own window to zero
    if (p < n_parts) {
        const int64_t w = __ldg(win + p);
        const int64_t prev = p > 0 ? (int64_t)__ldg(win + p - 1) : -1;
        if (prev != w) {
            g0 = prev + 1;
            g1 = w;
            if (__ldg(atomic + p) != 0) own = w;
        }
    } else if (p == n_parts) {
        g0 = n_parts > 0 ? (int64_t)__ldg(win + n_parts - 1) + 1 : 0;
        g1 = n_w;
    }
    g0 = g0 < 0 ? 0 : g0;
    g1 = g1 > n_w ? n_w : g1;
    if (own >= n_w) own = -1;
    unsigned m = __ballot_sync(0xffffffffu, g1 > g0 || own >= 0);
    while (m) {
        const int l = __ffs(m) - 1;
        m &= m - 1;
        const int64_t lg0 = __shfl_sync(0xffffffffu, g0, l), lg1 = __shfl_sync(0xffffffffu, g1, l);
        const int64_t lown = __shfl_sync(0xffffffffu, own, l);
        for (int pass = 0; pass < 2; ++pass) {
            const int64_t w0 = pass == 0 ? lg0 : lown, w1 = pass == 0 ? lg1 : lown + 1;
            if (w1 <= w0 || w0 < 0) continue;
            const int64_t r1 = w1 * W < m_out ? w1 * W : m_out;
            for (int64_t r = w0 * W; r < r1; ++r)
                for (int64_t f = lane; f < F; f += 32) Y[r * ldy + f] = 0.f;
        }
    }
}

template <typename K>
int occupancy_grid(K kernel, int smem, int64_t items) {
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kThreads, smem);
    if (per_sm < 1) per_sm = 1;
    int64_t want = (items + kWarps - 1) / kWarps;
    int64_t cap = (int64_t)sm_count() * per_sm;
    return (int)(want < cap ? (want > 0 ? want : 1) : cap);
}

template <typename K>
int prepare(K kernel, int smem) {
    // opt in to large dynamic shared memory once per kernel instantiation
    cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    return cuda_status(e, "cudaFuncSetAttribute");
}

template <typename T, int W, int FC, int WIDE, int S = kStages>
int launch16(const int32_t *rowptr, const int32_t *col, const void *val, const int32_t *win,
             const int32_t *atomic, int64_t n_parts, const void *X, int64_t n_x, int64_t F,
             int64_t ldx, float *Y, int64_t m_out, int64_t ldy, int32_t *err, cudaStream_t st) {
    using C = Cfg16<T, W, FC, WIDE, S>;
    const int n_chunks = (int)((F + FC - 1) / FC);
    const int64_t items = n_parts * n_chunks;
    if (items == 0) return ATT_OK;
    // 32-bit indices when every element offset stays below 2^31: X rows
    // (n_x * ldx), Y rows (m_out * ldy) and items (plus one grid stride of
    // overshoot); value offsets are below 2^31 by the format's own limit
    const int64_t lim = INT32_MAX - (1 << 22);
    const bool small = n_x * ldx < lim && m_out * ldy < lim && items < lim;
    auto run = [&](auto kernel) {
        static std::once_flag once;
        static int prep = ATT_OK;
        std::call_once(once, [&] { prep = prepare(kernel, C::SMEM); });
        if (prep != ATT_OK) return prep;
        const int grid = occupancy_grid(kernel, C::SMEM, items);
        kernel<<<grid, kThreads, C::SMEM, st>>>(rowptr, col, (const T *)val, win, atomic, n_parts,
                                                (const T *)X, n_x, F, ldx, Y, m_out, ldy, n_chunks,
                                                err);
        return launch_status("k_spmm16");
    };
    if (small && F % FC == 0) return run(k_spmm16<T, W, FC, WIDE, S, int32_t, true>);
    if (small) return run(k_spmm16<T, W, FC, WIDE, S, int32_t, false>);
    return run(k_spmm16<T, W, FC, WIDE, S, int64_t, false>);
}

template <typename T, int S>
int launch16_bulk(const int32_t *rowptr, const int32_t *col, const void *val, const int32_t *win,
                  const int32_t *atomic, int64_t n_parts, const void *X, int64_t n_x, int64_t F,
                  int64_t ldx, float *Y, int64_t m_out, int64_t ldy, int32_t *err,
                  cudaStream_t st) {
    constexpr int SMEM = kWarps * S * 16 * kBulkPitch;
    const int n_chunks = (int)((F + 63) / 64);
    const int64_t items = n_parts * n_chunks;
    if (items == 0) return ATT_OK;
    const int64_t lim = INT32_MAX - (1 << 22);
    const bool small = n_x * ldx < lim && m_out * ldy < lim && items < lim;
    auto run = [&](auto kernel) {
        static std::once_flag once;
        static int prep = ATT_OK;
        std::call_once(once, [&] { prep = prepare(kernel, SMEM); });
        if (prep != ATT_OK) return prep;
        const int grid = occupancy_grid(kernel, SMEM, items);
        kernel<<<grid, kThreads, SMEM, st>>>(rowptr, col, (const T *)val, win, atomic, n_parts,
                                             (const T *)X, n_x, F, ldx, Y, m_out, ldy, n_chunks, err);
        return launch_status("k_spmm16_bulk");
    };
    if (small) return run(k_spmm16_bulk<T, S, int32_t>);
    return run(k_spmm16_bulk<T, S, int64_t>);
}

template <int W, int FC, int WIDE, int S = kStages>
int launch_tf32(const int32_t *rowptr, const int32_t *col, const void *val, const int32_t *win,
                const int32_t *atomic, int64_t n_parts, const void *X, int64_t n_x, int64_t F,
                int64_t ldx, float *Y, int64_t m_out, int64_t ldy, int32_t *err, cudaStream_t st) {
    using C = CfgTF32<W, FC, WIDE, S>;
    auto kernel = k_spmm_tf32<W, FC, WIDE, S>;
    static std::once_flag once;
    static int prep = ATT_OK;
    std::call_once(once, [&] { prep = prepare(kernel, C::SMEM); });
    if (prep != ATT_OK) return prep;
    const int n_chunks = (int)((F + FC - 1) / FC);
    const int64_t items = n_parts * n_chunks;
    if (items == 0) return ATT_OK;
    const int grid = occupancy_grid(kernel, C::SMEM, items);
    kernel<<<grid, kThreads, C::SMEM, st>>>(rowptr, col, (const float *)val, win, atomic, n_parts,
                                            (const float *)X, n_x, F, ldx, Y, m_out, ldy, n_chunks,
                                            err);
    return launch_status("k_spmm_tf32");
}

PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                             &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
    });
    return fn;
}

template <typename T, int W, int FC, int WIDE, int S>
int launch16_tma(const int32_t *rowptr, const int32_t *col, const void *val, const int32_t *win,
                 const int32_t *atomic, int64_t n_parts, const void *X, int64_t n_x, int64_t F,
                 int64_t ldx, float *Y, int64_t m_out, int64_t ldy, int32_t *err, cudaStream_t st) {
    using C = CfgTma<W, FC, S>;
    auto kernel = k_spmm16_tma<T, W, FC, WIDE, S>;
    static std::once_flag once;
    static int prep = ATT_OK;
    std::call_once(once, [&] { prep = prepare(kernel, C::SMEM); });
    if (prep != ATT_OK) return prep;
    const int n_chunks = (int)((F + FC - 1) / FC);
    const int64_t items = n_parts * n_chunks;
    if (items == 0) return ATT_OK;
    CUtensorMap tm;
    const cuuint64_t gdim[2] = {(cuuint64_t)F, (cuuint64_t)n_x};
    const cuuint64_t gstride[1] = {(cuuint64_t)ldx * sizeof(T)};
    const cuuint32_t box[2] = {(cuuint32_t)kBox, 1};
    const cuuint32_t estr[2] = {1, 1};
    CUresult r = tensor_map_encoder()(
        &tm, sizeof(T) == 2 && std::is_same<T, __half>::value ? CU_TENSOR_MAP_DATA_TYPE_FLOAT16
                                                               : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16,
        2, const_cast<void *>(X), gdim, gstride, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
        CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    ATT_CHECK(r == CUDA_SUCCESS, ATT_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
    const int grid = occupancy_grid(kernel, C::SMEM, items);
    kernel<<<grid, kThreads, C::SMEM, st>>>(tm, rowptr, col, (const T *)val, win, atomic, n_parts,
                                            n_x, F, Y, m_out, ldy, n_chunks, err);
    return launch_status("k_spmm16_tma");
}

constexpr int kTmaStages = 5;

// Launch-shape options of att_spmm.  Each has a process-wide default
// (att_set_option, atomic) and a per-thread override (att_set_thread_option,
// -1 = follow the default), so a caller -- or the autotuner -- can pick the
// shape of its own calls without changing the shape of calls made by other
// threads.
//  * spmm_gather: row-gather mechanism of the 16-bit kernel, 0 = cp.async
//    (default), 1 = TMA tile::gather4, 2 = cp.async.bulk per row.
//  * spmm_stages / spmm_fc: ring depth of the 16-bit cp.async kernel (2, 3,
//    4) and features per work item for F > 64 (64 or 128).  Measured on the
//    2.45M-node graph (F = 128): throughput follows resident warps per SM,
//    not the depth of each warp's ring.
//  * spmm_fp8: 1 = A fragments dequantized in registers (k_spmm_fp8r, 128
//    features per item when F > 64), 0 = through an fp16 shared tile
//    (k_spmm_fp8).
//  * spmm_tf32: fp32-feature (3xTF32) kernel shape 0..3.
enum SpmmOpt { kOptGather = 0, kOptStages, kOptFc, kOptFp8, kOptTf32, kNumOpts };
const char *const kOptNames[kNumOpts] = {"spmm_gather", "spmm_stages", "spmm_fc", "spmm_fp8",
                                         "spmm_tf32"};
std::atomic<int> g_opt[kNumOpts] = {{0}, {3}, {64}, {1}, {0}};
thread_local int t_opt[kNumOpts] = {-1, -1, -1, -1, -1};

inline int opt(SpmmOpt i) {
    const int v = t_opt[i];
    return v >= 0 ? v : g_opt[i].load(std::memory_order_relaxed);
}

int opt_index(const char *key) {
    for (int i = 0; i < kNumOpts; ++i)
        if (strcmp(key, kOptNames[i]) == 0) return i;
    return -1;
}

bool opt_valid(int i, int v) {
    switch (i) {
        case kOptGather: return v >= 0 && v <= 2;
        case kOptStages: return v == 2 || v == 3 || v == 4;
        case kOptFc: return v == 64 || v == 128;
        case kOptFp8: return v == 0 || v == 1;
        case kOptTf32: return v >= 0 && v <= 3;
    }
    return false;
}

template <int W, int FC, int WIDE>
int launch_fp8(const int32_t *rowptr, const int32_t *col, const void *val, const int32_t *win,
               const int32_t *atomic, int64_t n_parts, const void *X, const float *xscale,
               int64_t n_x, int64_t F, int64_t ldx, float *Y, int64_t m_out, int64_t ldy,
               int32_t *err, cudaStream_t st) {
    using C = CfgF8<W, FC>;
    const int n_chunks = (int)((F + FC - 1) / FC);
    const int64_t items = n_parts * n_chunks;
    if (items == 0) return ATT_OK;
    const int64_t lim = INT32_MAX - (1 << 22);
    const bool small = n_x * ldx < lim && m_out * ldy < lim && items < lim;
    auto run = [&](auto kernel) {
        static std::once_flag once;
        static int prep = ATT_OK;
        std::call_once(once, [&] { prep = prepare(kernel, C::SMEM); });
        if (prep != ATT_OK) return prep;
        const int grid = occupancy_grid(kernel, C::SMEM, items);
        kernel<<<grid, kThreads, C::SMEM, st>>>(rowptr, col, (const __half *)val, win, atomic,
                                                n_parts, (const uint8_t *)X, xscale, n_x, F, ldx,
                                                Y, m_out, ldy, n_chunks, err);
        return launch_status("k_spmm_fp8");
    };
    if (small) return run(k_spmm_fp8<W, FC, WIDE, int32_t>);
    return run(k_spmm_fp8<W, FC, WIDE, int64_t>);
}

template <int W, int FC, int WIDE>
int launch_fp8r(const int32_t *rowptr, const int32_t *col, const void *val, const int32_t *win,
                const int32_t *atomic, int64_t n_parts, const void *X, const float *xscale,
                int64_t n_x, int64_t F, int64_t ldx, float *Y, int64_t m_out, int64_t ldy,
                int32_t *err, cudaStream_t st) {
    using C = CfgF8R<W, FC>;
    const int n_chunks = (int)((F + FC - 1) / FC);
    const int64_t items = n_parts * n_chunks;
    if (items == 0) return ATT_OK;
    const int64_t lim = INT32_MAX - (1 << 22);
    const bool small = n_x * ldx < lim && m_out * ldy < lim && items < lim;
    const int vec_out = (ldy % 2 == 0 && ((uintptr_t)Y & 7) == 0) ? 1 : 0;
    auto run = [&](auto kernel) {
        static std::once_flag once;
        static int prep = ATT_OK;
        std::call_once(once, [&] { prep = prepare(kernel, C::SMEM); });
        if (prep != ATT_OK) return prep;
        const int grid = occupancy_grid(kernel, C::SMEM, items);
        kernel<<<grid, kThreads, C::SMEM, st>>>(rowptr, col, (const __half *)val, win, atomic,
                                                n_parts, (const uint8_t *)X, xscale, n_x, F, ldx,
                                                Y, m_out, ldy, n_chunks, vec_out, err);
        return launch_status("k_spmm_fp8r");
    };
    if (small && F % FC == 0) return run(k_spmm_fp8r<W, FC, WIDE, int32_t, true>);
    if (small) return run(k_spmm_fp8r<W, FC, WIDE, int32_t, false>);
    return run(k_spmm_fp8r<W, FC, WIDE, int64_t, false>);
}

template <typename T, int W, int WIDE>
int dispatch_fc16(const int32_t *rowptr, const int32_t *col, const void *val, const int32_t *win,
                  const int32_t *atomic, int64_t n_parts, const void *X, int64_t n_x, int64_t F,
                  int64_t ldx, float *Y, int64_t m_out, int64_t ldy, int32_t *err,
                  cudaStream_t st) {
    // TMA row gathers for F >= 64 (the tensor map's 64-feature box fits); the
    // cp.async kernel for narrower features or an X without rows
    if (opt(kOptGather) == 1 && F >= 64 && n_x > 0 && n_x < INT32_MAX &&
        tensor_map_encoder() != nullptr) {
        if (F <= 64)
            return launch16_tma<T, W, 64, WIDE, kTmaStages>(rowptr, col, val, win, atomic, n_parts,
                                                            X, n_x, F, ldx, Y, m_out, ldy, err, st);
        return launch16_tma<T, W, 128, WIDE, kTmaStages>(rowptr, col, val, win, atomic, n_parts, X,
                                                         n_x, F, ldx, Y, m_out, ldy, err, st);
    }
    if (F <= 32)
        return launch16<T, W, 32, WIDE>(rowptr, col, val, win, atomic, n_parts, X, n_x, F, ldx, Y,
                                        m_out, ldy, err, st);
    if constexpr (W == 8 && WIDE == 8) {
        if (opt(kOptGather) == 2 && (F <= 64 || opt(kOptFc) == 64))
            return launch16_bulk<T, 3>(rowptr, col, val, win, atomic, n_parts, X, n_x, F, ldx, Y,
                                       m_out, ldy, err, st);
    }
#define ATT_L16S(FCv, Sv)                                                                       \
    return launch16<T, W, FCv, WIDE, Sv>(rowptr, col, val, win, atomic, n_parts, X, n_x, F, ldx, \
                                         Y, m_out, ldy, err, st)
    if (F <= 64 || opt(kOptFc) == 64) {
        if (opt(kOptStages) == 2) ATT_L16S(64, 2);
        if (opt(kOptStages) == 4) ATT_L16S(64, 4);
        ATT_L16S(64, 3);
    }
    if (opt(kOptStages) == 2) ATT_L16S(128, 2);
    if (opt(kOptStages) == 4) ATT_L16S(128, 4);
    ATT_L16S(128, 3);
#undef ATT_L16S
}

template <int W, int WIDE>
int dispatch_fc32(const int32_t *rowptr, const int32_t *col, const void *val, const int32_t *win,
                  const int32_t *atomic, int64_t n_parts, const void *X, int64_t n_x, int64_t F,
                  int64_t ldx, float *Y, int64_t m_out, int64_t ldy, int32_t *err,
                  cudaStream_t st) {
#define ATT_LTF(FCv, Sv)                                                                        \
    return launch_tf32<W, FCv, WIDE, Sv>(rowptr, col, val, win, atomic, n_parts, X, n_x, F, ldx, \
                                         Y, m_out, ldy, err, st)
    // shapes (features per item x ring depth): 0 = 64 x 4, 1 = 32 x 3,
    // 2 = 32 x 4, 3 = 64 x 2 (F <= 32 always takes 32-feature items)
    if (F <= 32 || opt(kOptTf32) == 1 || opt(kOptTf32) == 2) {
        if (opt(kOptTf32) == 1) ATT_LTF(32, 3);
        ATT_LTF(32, 4);
    }
    if (opt(kOptTf32) == 3) ATT_LTF(64, 2);
    ATT_LTF(64, 4);
#undef ATT_LTF
}

}  // namespace
}  // namespace att

using namespace att;

extern "C" int att_spmm(const int32_t *rowptr, const int32_t *col, const void *val, int val_dtype,
                        const int32_t *window_of_part, const int32_t *atomic, int64_t n_parts,
                        const void *X, int x_dtype, const float *x_scale, int64_t n_x_rows,
                        int64_t F, int64_t ldx, float *Y, int64_t m_out, int64_t ldy, int window,
                        int wide, int32_t *err_flag, void *stream) {
    clear_error();
    ATT_CHECK(n_parts >= 0 && m_out >= 0 && F >= 0 && n_x_rows >= 0, ATT_ERR_INVALID,
              "negative size");
    ATT_CHECK(window == 8 || window == 16, ATT_ERR_UNSUPPORTED, "window must be 8 or 16, got %d",
              window);
    ATT_CHECK(m_out == 0 || F == 0 || Y != nullptr, ATT_ERR_INVALID, "Y is null");
    ATT_CHECK(ldy >= F, ATT_ERR_INVALID, "ldy %lld < F %lld", (long long)ldy, (long long)F);
    ATT_CHECK(n_parts == 0 || (rowptr && col && val && window_of_part && atomic && X),
              ATT_ERR_INVALID, "null format or X pointer");
    cudaStream_t st = (cudaStream_t)stream;
    if (m_out == 0 || F == 0) return ATT_OK;
    int s = ATT_OK;
    if ((size_t)m_out * (size_t)ldy * sizeof(float) <= kZeroAllBytes) {
        // a small Y: zeroing all of it costs less than finding what to zero
        ATT_CUDA(cudaMemset2DAsync(Y, (size_t)ldy * sizeof(float), 0, (size_t)F * sizeof(float),
                                   (size_t)m_out, st),
                 "zero Y");
    } else {
        const int64_t threads = n_parts + 1;
        k_zero_uncovered<<<(unsigned)((threads + 255) / 256), 256, 0, st>>>(
            window_of_part, atomic, n_parts, window, Y, m_out, F, ldy);
        s = launch_status("k_zero_uncovered");
        if (s != ATT_OK) return s;
    }
    if (n_parts == 0) return ATT_OK;
    const bool is16 = (val_dtype == ATT_F16 && x_dtype == ATT_F16) ||
                      (val_dtype == ATT_BF16 && x_dtype == ATT_BF16);
    if (is16) {
        ATT_CHECK(wide == 8 || wide == 16, ATT_ERR_UNSUPPORTED,
                  "16-bit values need wide 8 or 16, got %d", wide);
        ATT_CHECK(F % 8 == 0 && ldx % 8 == 0 && ((uintptr_t)X & 15) == 0 && ((uintptr_t)val & 15) == 0,
                  ATT_ERR_UNSUPPORTED,
                  "16-bit SpMM needs F and ldx multiples of 8 and 16-byte aligned X and values");
        ATT_CHECK(ldx >= F, ATT_ERR_INVALID, "ldx < F");
#define ATT_SPMM16(T, Wv, WIDEv)                                                             \
    return dispatch_fc16<T, Wv, WIDEv>(rowptr, col, val, window_of_part, atomic, n_parts, X, \
                                       n_x_rows, F, ldx, Y, m_out, ldy, err_flag, st)
        if (val_dtype == ATT_F16) {
            if (window == 8 && wide == 8) ATT_SPMM16(__half, 8, 8);
            if (window == 8 && wide == 16) ATT_SPMM16(__half, 8, 16);
            if (window == 16 && wide == 8) ATT_SPMM16(__half, 16, 8);
            ATT_SPMM16(__half, 16, 16);
        } else {
            if (window == 8 && wide == 8) ATT_SPMM16(__nv_bfloat16, 8, 8);
            if (window == 8 && wide == 16) ATT_SPMM16(__nv_bfloat16, 8, 16);
            if (window == 16 && wide == 8) ATT_SPMM16(__nv_bfloat16, 16, 8);
            ATT_SPMM16(__nv_bfloat16, 16, 16);
        }
#undef ATT_SPMM16
    }
    if (val_dtype == ATT_F32 && x_dtype == ATT_F32) {
        ATT_CHECK(wide == 4 || wide == 8, ATT_ERR_UNSUPPORTED, "fp32 values need wide 4 or 8, got %d",
                  wide);
        ATT_CHECK(F % 4 == 0 && ldx % 4 == 0 && ((uintptr_t)X & 15) == 0 && ((uintptr_t)val & 15) == 0,
                  ATT_ERR_UNSUPPORTED,
                  "fp32 SpMM needs F and ldx multiples of 4 and 16-byte aligned X and values");
        ATT_CHECK(ldx >= F, ATT_ERR_INVALID, "ldx < F");
        if (window == 8 && wide == 4)
            return dispatch_fc32<8, 4>(rowptr, col, val, window_of_part, atomic, n_parts, X,
                                       n_x_rows, F, ldx, Y, m_out, ldy, err_flag, st);
        if (window == 8 && wide == 8)
            return dispatch_fc32<8, 8>(rowptr, col, val, window_of_part, atomic, n_parts, X,
                                       n_x_rows, F, ldx, Y, m_out, ldy, err_flag, st);
        if (window == 16 && wide == 4)
            return dispatch_fc32<16, 4>(rowptr, col, val, window_of_part, atomic, n_parts, X,
                                        n_x_rows, F, ldx, Y, m_out, ldy, err_flag, st);
        return dispatch_fc32<16, 8>(rowptr, col, val, window_of_part, atomic, n_parts, X, n_x_rows,
                                    F, ldx, Y, m_out, ldy, err_flag, st);
    }
    if (val_dtype == ATT_F16 && x_dtype == ATT_F8E4M3) {
        ATT_CHECK(x_scale != nullptr, ATT_ERR_INVALID, "fp8 features need per-row scales");
        ATT_CHECK(wide == 8 || wide == 16, ATT_ERR_UNSUPPORTED, "fp16 values need wide 8 or 16");
        ATT_CHECK(F % 16 == 0 && ldx % 16 == 0 && ((uintptr_t)X & 15) == 0 &&
                      ((uintptr_t)val & 15) == 0 && ldx >= F,
                  ATT_ERR_UNSUPPORTED,
                  "fp8 SpMM needs F and ldx multiples of 16 and 16-byte aligned X and values");
#define ATT_F8R(Wv, FCv, WIDEv)                                                                \
    return launch_fp8r<Wv, FCv, WIDEv>(rowptr, col, val, window_of_part, atomic, n_parts, X,   \
                                       x_scale, n_x_rows, F, ldx, Y, m_out, ldy, err_flag, st)
        if (opt(kOptFp8) == 1) {
            if (F > 64) {
                if (window == 8) { if (wide == 8) ATT_F8R(8, 128, 8); ATT_F8R(8, 128, 16); }
                if (wide == 8) ATT_F8R(16, 128, 8);
                ATT_F8R(16, 128, 16);
            }
            if (window == 8) { if (wide == 8) ATT_F8R(8, 64, 8); ATT_F8R(8, 64, 16); }
            if (wide == 8) ATT_F8R(16, 64, 8);
            ATT_F8R(16, 64, 16);
        }
#undef ATT_F8R
#define ATT_F8(Wv, FCv, WIDEv)                                                                \
    return launch_fp8<Wv, FCv, WIDEv>(rowptr, col, val, window_of_part, atomic, n_parts, X,   \
                                      x_scale, n_x_rows, F, ldx, Y, m_out, ldy, err_flag, st)
        // 64 features per work item: like the 16-bit kernel, throughput
        // follows resident warps per SM
        if (window == 8) { if (wide == 8) ATT_F8(8, 64, 8); ATT_F8(8, 64, 16); }
        if (wide == 8) ATT_F8(16, 64, 8);
        ATT_F8(16, 64, 16);
#undef ATT_F8
    }
    set_error("unsupported (val_dtype=%d, x_dtype=%d) combination", val_dtype, x_dtype);
    return ATT_ERR_UNSUPPORTED;
}

extern "C" int att_set_option(const char *key, int value) {
    clear_error();
    ATT_CHECK(key != nullptr, ATT_ERR_INVALID, "null option name");
    const int i = opt_index(key);
    ATT_CHECK(i >= 0, ATT_ERR_INVALID, "unknown option '%s'", key);
    ATT_CHECK(opt_valid(i, value), ATT_ERR_INVALID, "invalid value %d for option '%s'", value,
              key);
    g_opt[i].store(value, std::memory_order_relaxed);
    return ATT_OK;
}

extern "C" int att_set_thread_option(const char *key, int value) {
    clear_error();
    ATT_CHECK(key != nullptr, ATT_ERR_INVALID, "null option name");
    const int i = opt_index(key);
    ATT_CHECK(i >= 0, ATT_ERR_INVALID, "unknown option '%s'", key);
    ATT_CHECK(value == -1 || opt_valid(i, value), ATT_ERR_INVALID,
              "invalid value %d for option '%s'", value, key);
    t_opt[i] = value;
    return ATT_OK;
}

extern "C" int att_get_option(const char *key, int *value) {
    clear_error();
    ATT_CHECK(key != nullptr && value != nullptr, ATT_ERR_INVALID, "null argument");
    const int i = opt_index(key);
    ATT_CHECK(i >= 0, ATT_ERR_INVALID, "unknown option '%s'", key);
    *value = opt((SpmmOpt)i);
    return ATT_OK;
}

extern "C" size_t att_spmm_groups_scratch_bytes(int64_t n_parts, int64_t n_windows) {
    if (n_parts < 0) n_parts = 0;
    if (n_windows < 0) n_windows = 0;
    const int64_t m = n_parts > n_windows ? n_parts : n_windows;
    return align_up((size_t)n_parts * 8, 256) + align_up((size_t)n_windows * 8, 256) +
           scan64_tmp_bytes(m);
}

extern "C" int att_spmm_groups(const int32_t *window_of_part, int64_t n_parts, int64_t n_windows,
                               int group_parts, int32_t *group_part, int32_t *group_slot,
                               int32_t *red_first, int32_t *empty_win, int64_t *counts,
                               void *scratch, size_t scratch_bytes, void *stream) {
    clear_error();
    ATT_CHECK(n_parts >= 0 && n_parts < kFieldMask, ATT_ERR_UNSUPPORTED,
              "att_spmm_groups takes fewer than %lld parts", (long long)kFieldMask);
    ATT_CHECK(n_windows >= 0 && n_windows <= INT32_MAX, ATT_ERR_INVALID, "bad window count");
    ATT_CHECK(group_parts >= 1 && group_parts <= 1024, ATT_ERR_INVALID,
              "group_parts %d outside [1, 1024]", group_parts);
    ATT_CHECK(group_part && red_first && counts, ATT_ERR_INVALID, "null output");
    ATT_CHECK(n_parts == 0 || (window_of_part && group_slot), ATT_ERR_INVALID, "null input");
    ATT_CHECK(n_windows == 0 || empty_win, ATT_ERR_INVALID, "null empty-window output");
    ATT_CHECK(scratch && scratch_bytes >= att_spmm_groups_scratch_bytes(n_parts, n_windows),
              ATT_ERR_WORKSPACE, "scratch of %zu bytes, %zu needed", scratch_bytes,
              att_spmm_groups_scratch_bytes(n_parts, n_windows));
    cudaStream_t st = (cudaStream_t)stream;
    int64_t *pflags = (int64_t *)scratch;
    int64_t *wflags = (int64_t *)((char *)scratch + align_up((size_t)n_parts * 8, 256));
    int64_t *tmp = (int64_t *)((char *)wflags + align_up((size_t)n_windows * 8, 256));
    const unsigned pblocks = (unsigned)((n_parts + 255) / 256);
    const unsigned wblocks = (unsigned)((n_windows + 255) / 256);
    int s;
    if (n_parts > 0) {
        k_group_flags<<<pblocks, 256, 0, st>>>(window_of_part, n_parts, group_parts, pflags);
        if ((s = launch_status("k_group_flags")) != ATT_OK) return s;
        if ((s = scan64_exclusive(pflags, n_parts, tmp, st)) != ATT_OK) return s;
    }
    k_group_scatter<<<pblocks > 0 ? pblocks : 1, 256, 0, st>>>(window_of_part, n_parts, group_parts,
                                                               pflags, group_part, group_slot,
                                                               red_first, counts);
    if ((s = launch_status("k_group_scatter")) != ATT_OK) return s;
    if (n_windows > 0) {
        k_empty_flags<<<wblocks, 256, 0, st>>>(window_of_part, n_parts, n_windows, wflags);
        if ((s = launch_status("k_empty_flags")) != ATT_OK) return s;
        if ((s = scan64_exclusive(wflags, n_windows, tmp, st)) != ATT_OK) return s;
    }
    k_empty_scatter<<<wblocks > 0 ? wblocks : 1, 256, 0, st>>>(window_of_part, n_parts, n_windows,
                                                               wflags, empty_win, counts);
    return launch_status("k_empty_scatter");
}

extern "C" int att_host_device_pointer(const void *host, void **device) {
    clear_error();
    ATT_CHECK(host && device, ATT_ERR_INVALID, "null pointer");
    cudaPointerAttributes a;
    ATT_CUDA(cudaPointerGetAttributes(&a, host), "cudaPointerGetAttributes");
    ATT_CHECK(a.type == cudaMemoryTypeHost && a.devicePointer != nullptr, ATT_ERR_INVALID,
              "%p is not page-locked host memory mapped for the device", host);
    *device = a.devicePointer;
    return ATT_OK;
}

extern "C" size_t att_spmm_batched_grid(void) {
    using C = Cfg16<__half, 8, 64, 8, 3>;
    auto kernel = k_spmm16_batched<8, 64, 8, 3>;
    if (prepare(kernel, C::SMEM) != ATT_OK) return 0;
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kThreads, C::SMEM);
    return (size_t)sm_count() * (per_sm > 0 ? per_sm : 1);
}

extern "C" int att_spmm_batched(const att_spmm_job *jobs, int64_t *header, int64_t grid,
                                int window, int wide, int32_t *err_flag, void *stream) {
    clear_error();
    ATT_CHECK(window == 8 && wide == 8, ATT_ERR_UNSUPPORTED,
              "the batched SpMM takes the (8-row, 8-wide) fp16 format");
    ATT_CHECK(jobs && header && grid > 0, ATT_ERR_INVALID, "null table or empty grid");
    using C = Cfg16<__half, 8, 64, 8, 3>;
    auto kernel = k_spmm16_batched<8, 64, 8, 3>;
    static std::once_flag once;
    static int prep = ATT_OK;
    std::call_once(once, [&] { prep = prepare(kernel, C::SMEM); });
    if (prep != ATT_OK) return prep;
    cudaStream_t st = (cudaStream_t)stream;
    const unsigned side = (unsigned)(sm_count() * 8);
    k_zero_empty_batched<8><<<side, 256, 0, st>>>(jobs, header);
    int s = launch_status("k_zero_empty_batched");
    if (s != ATT_OK) return s;
    kernel<<<(unsigned)grid, kThreads, C::SMEM, st>>>(jobs, header, err_flag);
    s = launch_status("k_spmm16_batched");
    if (s != ATT_OK) return s;
    k_reduce_groups_batched<8><<<(unsigned)(sm_count() * 4), 256, 0, st>>>(jobs, header);
    return launch_status("k_reduce_groups_batched");
}
