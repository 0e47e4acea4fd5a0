/*
 * att_gb300.h -- C ABI of the GB300 (sm_103a) ATT sparse hot path.
 *
 * Every entry point takes plain device pointers, element counts and a CUDA
 * stream (passed as `void *`, a cudaStream_t; NULL = legacy default stream),
 * launches asynchronously on that stream and returns an att_status.  No entry
 * point allocates device memory: outputs and workspaces are the caller's.
 * Only the two-phase conversion's plan step synchronises the stream (it has
 * to return the output sizes to the host).
 *
 * Block format ("row-window block-condensed", the reference's layout):
 *   rows are grouped in windows of W rows; each window's distinct columns are
 *   listed in ascending order and padded with -1 to a multiple of `wide`;
 *   the columns of all windows are concatenated (col[n_cols]); the value of
 *   slot (window row r, condensed column c) sits at
 *       val[(c - c % wide) * W + r * wide + c % wide]
 *   (blocks of W x wide, row-major, one block after another).  A window with
 *   more than `part` blocks is split into parts; part p covers condensed
 *   columns [rowptr[2p], rowptr[2p+2]), of which [rowptr[2p], rowptr[2p+1])
 *   are real; window_of_part[p] is its window, atomic[p] = 1 if its window
 *   was split.  Parts are in ascending window order.
 *
 * The reference interfaces each function replaces are cited by file:line of
 * the reference project.
 */
#ifndef ATT_GB300_H
#define ATT_GB300_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define ATT_API __attribute__((visibility("default")))
#else
#define ATT_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
enum att_status {
    ATT_OK = 0,
    ATT_ERR_INVALID = 1,     /* bad argument (null pointer, size, dtype, alignment) */
    ATT_ERR_CUDA = 2,        /* a CUDA runtime call or launch failed */
    ATT_ERR_WORKSPACE = 3,   /* workspace smaller than the size query returned */
    ATT_ERR_UNSUPPORTED = 4, /* valid but not implemented combination */
    ATT_ERR_OVERFLOW = 5,    /* output would exceed int32 indexing */
    ATT_ERR_FORMAT = 6       /* device-side check found a malformed input */
};

/* ---- element types ----------------------------------------------------- */
enum att_dtype {
    ATT_F32 = 0,
    ATT_F16 = 1,
    ATT_BF16 = 2,
    ATT_F8E4M3 = 3,
    ATT_I32 = 4,
    ATT_NONE = -1
};

/* Tuning knobs (no counterpart in the reference).  att_set_option sets the
 * process-wide default of a knob; att_set_thread_option overrides it for the
 * calling host thread only (-1 returns the thread to the default), so a
 * caller can fix the launch shape of its own calls without changing other
 * threads' calls; att_get_option reads the value in effect on the calling
 * thread.
 *   "spmm_gather": 0 = 16-byte cp.async row gathers (default),
 *                  1 = TMA tile::gather4 row gathers (F >= 64),
 *                  2 = one cp.async.bulk per gathered row (8-row windows,
 *                      8-wide blocks, 64-feature chunks).
 *   "spmm_stages": ring depth of the 16-bit cp.async kernel (2, 3, 4).
 *   "spmm_fc":     features per work item for F > 64 (64, the default, or 128).
 *   "spmm_fp8":    FP8 feature kernel: 1 = dequantized in registers (default),
 *                  0 = dequantized through an fp16 shared-memory tile.
 *   "spmm_tf32":   fp32-feature (3xTF32) kernel, features per item x ring
 *                  depth: 0 = 64 x 4 (default), 1 = 32 x 3, 2 = 32 x 4, 3 = 64 x 2. */
ATT_API int att_set_option(const char *key, int value);
ATT_API int att_set_thread_option(const char *key, int value);
ATT_API int att_get_option(const char *key, int *value);

/* Human-readable name of a status. */
ATT_API const char *att_status_string(int status);
/* Message of the last failing call on this host thread ("" if none). */
ATT_API const char *att_last_error(void);
/* Library version, major*10000 + minor*100 + patch. */
ATT_API int att_version(void);

/* ======================================================================
 * Conversion: CSR -> row-window block-condensed format, on the GPU.
 * Replaces Block_sr_bcrs.blockProcess_fp16_balance / _tf32_balance
 * (gcn/Block_gcn/example.cpp:48-200, :203-348; pybind :353-357) and
 * ATT_Block[_v3].blockProcess_sddmm_balance_gnn[_trans]
 * (Block/include/example.h:4-6, called from
 * end2end_ori/gat_final/mgat_csr/mdataset_fp16.py:57-62) and the GPU
 * preprocessing ATT_Block_gpu.preprocess_gpu_fs
 * (end2end_overhead/gat_final/mgat_csr_ov/mdataset_fp16.py:53-58).
 * Output is bit-identical to the reference's CPU conversion.
 *
 * n_rows = rowptr length - 1; column ids must lie in [0, n_cols).
 * emit_empty = 1 reproduces the tf32 variant (an empty window emits a
 * (0,0) part), 0 the fp16 variant (empty windows emit nothing).
 * ====================================================================== */

/* Bytes of device workspace att_block_plan / att_block_fill need. */
ATT_API size_t att_block_workspace_bytes(int64_t n_rows, int64_t nnz, int64_t n_cols, int window);

/* Phase 1: per-window distinct columns.  Writes the number of parts and of
 * padded condensed columns to the host pointers; synchronises `stream`. */
ATT_API int att_block_plan(const int32_t *rowptr, const int32_t *col, int64_t n_rows, int64_t nnz,
                   int64_t n_cols, int window, int wide, int part, int emit_empty,
                   void *workspace, size_t workspace_bytes,
                   int64_t *n_parts_out, int64_t *n_condensed_out, void *stream);

/* Phase 1 without the synchronisation (no counterpart in the reference):
 * enqueues the plan and a copy of its 3-int64 summary to `summary` (pinned
 * host memory for an asynchronous copy).  Once `stream` has passed that copy,
 * att_block_plan_result() validates the summary (ATT_ERR_FORMAT for a bad
 * rowptr or column, ATT_ERR_OVERFLOW) and returns the two sizes.  The
 * workspace must stay untouched until att_block_fill has run. */
ATT_API int att_block_plan_async(const int32_t *rowptr, const int32_t *col, int64_t n_rows,
                   int64_t nnz, int64_t n_cols, int window, int wide, int part, int emit_empty,
                   void *workspace, size_t workspace_bytes, int64_t *summary, void *stream);
ATT_API int att_block_plan_result(const int64_t *summary, int64_t n_cols, int window,
                   int64_t *n_parts_out, int64_t *n_condensed_out);

/* Phase 2: write the format.  Output sizes: rowptr 2*n_parts+1, col
 * n_condensed, val / map / map_t n_condensed*window, window_of_part and atomic
 * n_parts.  Any of val, map, map_t may be NULL to skip it.
 *   deg (deg_dtype ATT_F16 or ATT_F32, length >= n_cols and >= n_rows) gives
 *   val = deg[row]*deg[col] computed in fp32 and rounded to val_dtype
 *   (ATT_F16, ATT_BF16 or ATT_F32); duplicate (row,col) entries overwrite.
 *   map[slot]   = the last CSR edge id landing in the slot, -1 if empty.
 *   map_t[slot] = the last CSR edge id of the mirrored edge (col,row), -1 if
 *                 absent; needs rows sorted by column (checked: status
 *                 ATT_ERR_FORMAT otherwise).
 *   edge_slot (may be NULL): for each CSR edge e, the slot index its value
 *   landed in (the compact per-edge form the GAT kernels consume).
 * Synchronises `stream` to read the device-side checks. */
ATT_API int att_block_fill(const int32_t *rowptr, const int32_t *col, int64_t n_rows, int64_t nnz,
                   int64_t n_cols, int window, int wide, int part, int emit_empty,
                   const void *deg, int deg_dtype, const void *workspace, size_t workspace_bytes,
                   int32_t *out_rowptr, int32_t *out_col, void *out_val, int val_dtype,
                   int32_t *out_map, int32_t *out_map_t, int32_t *out_edge_slot,
                   int32_t *out_window, int32_t *out_atomic, void *stream);

/* Phase 2 without the synchronisations (no counterpart in the reference):
 * the sizes come from att_block_plan_result of the same plan, and the
 * device-side checks go to `flags` (4 int32, pinned host memory for an
 * asynchronous copy).  Once `stream` has passed that copy,
 * att_block_fill_result(flags, map_t != NULL) returns what att_block_fill
 * would have returned.  For a scheduler that must not block (the serving
 * loop). */
ATT_API int att_block_fill_async(const int32_t *rowptr, const int32_t *col, int64_t n_rows,
                   int64_t nnz, int64_t n_cols, int window, int wide, int part, int emit_empty,
                   const void *deg, int deg_dtype, const void *workspace, size_t workspace_bytes,
                   int64_t n_parts, int64_t n_condensed, int32_t *out_rowptr, int32_t *out_col,
                   void *out_val, int val_dtype, int32_t *out_map, int32_t *out_map_t,
                   int32_t *out_edge_slot, int32_t *out_window, int32_t *out_atomic,
                   int32_t *flags, void *stream);
ATT_API int att_block_fill_result(const int32_t *flags, int with_map_t);

/* ----------------------------------------------------------------------
 * Allocation-free conversion.  No counterpart in the reference: it exists
 * for callers that cannot allocate device memory -- hosts that hand out
 * device memory only from their own arena or budget and forbid a library
 * from allocating, and latency-critical callers that cannot afford
 * cudaMalloc/cudaFree, which may synchronise the device.  It does what
 * att_block_plan + att_block_fill do, in one call, with the scratch taken
 * from a 64 MiB device array the library owns (att_block_convert_noalloc_max_scratch()
 * bytes) instead of a caller workspace; it calls no allocating routine.
 *   - Graphs whose att_block_workspace_bytes() exceeds that size are
 *     rejected with ATT_ERR_WORKSPACE.
 *   - Outputs are the caller's, as for att_block_fill; max_parts and
 *     max_condensed are their capacities (in parts and condensed columns).
 *     The sizes are written to n_parts_out / n_condensed_out; if they exceed
 *     the capacities the call returns ATT_ERR_WORKSPACE before writing.
 *   - The first call on a device looks up the array's device address and
 *     keeps it for the life of the process; the kept address does not
 *     survive cudaDeviceReset (do not call this after resetting a device).
 *   - The call blocks until its GPU work is done (it synchronises `stream`
 *     to read the sizes and again to read the device-side checks), so it
 *     cannot be used inside a stream capture, and calls made one after the
 *     other never overlap.  All calls share the array: calls from different
 *     host threads at the same time race on it -- the caller orders them.
 * ---------------------------------------------------------------------- */
ATT_API size_t att_block_convert_noalloc_max_scratch(void);
ATT_API int att_block_convert_noalloc(const int32_t *rowptr, const int32_t *col, int64_t n_rows,
                   int64_t nnz, int64_t n_cols, int window, int wide, int part, int emit_empty,
                   const void *deg, int deg_dtype,
                   int32_t *out_rowptr, int32_t *out_col, void *out_val, int val_dtype,
                   int32_t *out_map, int32_t *out_map_t, int32_t *out_edge_slot,
                   int32_t *out_window, int32_t *out_atomic,
                   int64_t max_parts, int64_t max_condensed,
                   int64_t *n_parts_out, int64_t *n_condensed_out, void *stream);

/* ======================================================================
 * Blocked SpMM:  Y[m_out, F] = A_blocks * X   (tensor cores, fp32 accumulate)
 * Replaces SpMM_sr_bcrs.forward_fp16_gnn / forward_tf32_gnn /
 * forward_fp16_gnn_acc / forward_tf32_gnn_acc (gcn/SpMM/src/benchmark.cpp:35-75,
 * :91-130, :259-296, :305-335; kernels gcn/SpMM/src/spmmKernel.cu:158-265,
 * :959-1075, :2066-2173, :2214-2330; launchers :1693-1765, :2175-2209,
 * :2332-2366).
 *
 *   val_dtype / x_dtype: (ATT_F16, ATT_F16), (ATT_BF16, ATT_BF16),
 *     (ATT_F32, ATT_F32) [3xTF32 split, fp32-level accuracy], or
 *     (ATT_F16, ATT_F8E4M3) with x_scale[n_x_rows] fp32 per-row scales
 *     (X_true[j] = x_scale[j] * X_e4m3[j]).
 *   X row j at X + j*ldx elements; Y row i at Y + i*ldy elements (fp32).
 *   Every row of Y in [0, m_out) is written (rows of windows without parts
 *   are zeroed), so Y needs no prior clearing.
 *   window: 8 or 16; wide: 8 or 16 for 16-bit values, 4 or 8 for fp32.
 *   err_flag (device int32, may be NULL): bit 1 set if a column id is
 *   outside [-1, n_x_rows) (such columns contribute nothing); bit 2 set if a
 *   part does not start and end on a `wide` block boundary (it is skipped).
 * ====================================================================== */
ATT_API int att_spmm(const int32_t *rowptr, const int32_t *col, const void *val, int val_dtype,
             const int32_t *window_of_part, const int32_t *atomic, int64_t n_parts,
             const void *X, int x_dtype, const float *x_scale, int64_t n_x_rows,
             int64_t F, int64_t ldx, float *Y, int64_t m_out, int64_t ldy,
             int window, int wide, int32_t *err_flag, void *stream);

/* ======================================================================
 * GAT operators on the block format with a slot -> edge map (the format
 * att_block_fill writes with `map` / `map_t`).  They replace the
 * ATT_SDDMM_v{1,3,4} and ATT_SpMM_v{1,3,4} extension ops, whose CUDA source
 * is absent from the reference; the meaning of each is pinned by the
 * reference's tests (benchmark-v3/sddmm-benchmark/test/*,
 * benchmark-v3/spmm-benchmark/test/*) and callers
 * (end2end_ori/gat_final/mgat_csr/mgat_conv.py:14-198,
 * end2end_head/gat_final/mgat_csr/mgat_conv.py:14-198,
 * end2end_acc/gat_final/mgat_csr/mgat_conv.py:16-232).
 * Edge-valued arrays are addressed base[h*stride_h + e*stride_e] and
 * node-valued arrays base[h*stride_h + node*stride_n], so [h,nnz] / [nnz,h]
 * and [h,M,F] / [M,h,F] layouts are views.  Edge ids are CSR positions.
 * ====================================================================== */

/* scores[h][m] = sum_f X[h][m][f] * a[h][f]  (fp32 accumulate).  Building
 * block of att_*_h_nnz / attv2_*_h_nnz (mgat_conv.py:21-30). */
ATT_API int att_node_scores(const void *X, int x_dtype, int64_t n_heads, int64_t n_nodes,
                   int64_t F, int64_t x_stride_h, int64_t x_stride_n, const void *a,
                   int a_dtype, int64_t a_stride_h, float *scores, int64_t s_stride_h,
                   void *stream);
/* s0[h][m] = X[h][m] . a0[h] and s1[h][m] = X[h][m] . a1[h] in one pass over
 * X (fp32 attention vectors a0 / a1 [h][F] with row stride a_stride_h).
 * No counterpart in the reference: the fused GAT layer's two node-score
 * vectors, the building block of att_*_h_nnz computed once per node instead
 * of per edge. */
ATT_API int att_node_scores_pair(const void *X, int x_dtype, int64_t n_heads, int64_t n_nodes,
                   int64_t F, int64_t x_stride_h, int64_t x_stride_n, const float *a0,
                   const float *a1, int64_t a_stride_h, float *s0, float *s1,
                   int64_t s_stride_h, void *stream);

/* For every slot with an edge e (row i = window*W + r, column j = col[c]):
 *   mode 0: out[h][e] = s0[h][i] + s1[h][j]   (att_*_h_nnz: X_i.a0 + X_j.a1;
 *           attv2_*_h_nnz: X0_i.a + X1_j.a; test_sddmm_tf32_att.py,
 *           test_sddmm_fp16_att_v2.py:70-77)
 *   mode 1: out[h][e] = g[h][i]               (sddmm_*_ones_h_nnz,
 *           test_sddmm_fp16_ones.py:62-68)
 * Edges no slot holds are not written. */
ATT_API int att_slot_edges(const int32_t *rowptr, const int32_t *col, const int32_t *map,
                   const int32_t *window_of_part, int64_t n_parts, int window, int wide,
                   int mode, const float *s0, const float *s1, int64_t s_stride_h,
                   const void *g, int g_dtype, int64_t g_stride_h, int64_t g_stride_n,
                   int64_t n_nodes, int64_t n_heads, void *out, int out_dtype,
                   int64_t out_stride_h, int64_t out_stride_e, void *stream);

/* Blocked SDDMM: out[h][e(i,j)] = A[h][i] . B[h][j] for every slot with an edge
 * (sddmm_*_h_nnz, test_sddmm_fp16.py:62-69; mgat_conv.py:109-117).  Tensor
 * cores: mma.sync m16n8k16 (dtype ATT_F16 / ATT_BF16, fp32 accumulate) or a
 * 3xTF32 m16n8k8 split (ATT_F32).  F <= 256 (<= 128 for fp32); wide 4/8/16;
 * 16-bit B rows need F and strides multiples of 8 (16-byte rows). */
ATT_API int att_sddmm(const int32_t *rowptr, const int32_t *col, const int32_t *map,
                   const int32_t *window_of_part, int64_t n_parts, int window, int wide,
                   const void *A, const void *B, int dtype, int64_t n_heads, int64_t F,
                   int64_t a_stride_h, int64_t a_stride_n, int64_t n_a,
                   int64_t b_stride_h, int64_t b_stride_n, int64_t n_b, void *out,
                   int out_dtype, int64_t out_stride_h, int64_t out_stride_e,
                   int32_t *err_flag, void *stream);

/* Dense block values from per-edge values: out[h][s] = vals[h][map[s']] or 0,
 * where s (block width out_wide) and s' (block width map_wide) name the same
 * (window row, condensed column).  With att_spmm this is spmm_*_h_m / _m_h
 * (test_spmm_h_m.py:45-66, test_spmm_m_h.py:47-80; mgat_conv.py:79-86,99-106). */
ATT_API int att_gather_slot_values(const int32_t *map, int64_t n_slots, int window,
                   int map_wide, int out_wide, const void *vals, int v_dtype,
                   int64_t v_stride_h, int64_t v_stride_e, int64_t n_heads,
                   void *out, int out_dtype, int64_t out_stride_h, void *stream);

/* Row sums of per-edge values through the map: out[h][i] = sum over slots of
 * row i of vals[h][map[s]] (spmm_*_{h_m,m_h}_rowsum, test_spmm_h_m_ones.py:45-68;
 * mgat_conv.py:126-132).  Every row < m_out is written (fp32). */
ATT_API int att_rowsum(const int32_t *rowptr, const int32_t *map,
                   const int32_t *window_of_part, const int32_t *atomic, int64_t n_parts,
                   int window, int wide, const void *vals, int v_dtype, int64_t v_stride_h,
                   int64_t v_stride_e, int64_t n_heads, float *out, int64_t out_stride_h,
                   int64_t out_stride_n, int64_t m_out, void *stream);

/* ======================================================================
 * Fused GAT attention layer (SDDMM -> LeakyReLU -> edge softmax -> SpMM in
 * one pass, no per-edge intermediates).  Replaces the reference's op chain of
 * end2end_ori/gat_final/mgat_csr/mgat_conv.py:173-198 (att_fp16_h_nnz,
 * leakyrelu, exp, spmm_fp16_h_m_rowsum, spmm_fp16_h_m, div).
 * ====================================================================== */

/* Occupancy bitmap of a block format: bit s set iff slot s holds an edge
 * (from att_block_fill's edge_slot).  mask has n_words = ceil(n_slots/32)
 * words and is cleared first. */
ATT_API int att_slot_mask(const int32_t *edge_slot, int64_t nnz, uint32_t *mask,
                   int64_t n_words, void *stream);

/* out[i][h*F + f] = sum_j softmax_j(LeakyReLU(e_ij)) X'[j][h*F + f] over the
 * edges (i, j) of row i, per head h, with
 *   mode 0: e_ij = X'_i . X'_j (SDDMM of X' X'^T masked to the edges)
 *   mode 1: e_ij = s0[h][i] + s1[h][j] (GAT's additive a0/a1 scores).
 * Row max and sum stay fp32.  Work items are chunks of consecutive parts of
 * one window: chunk c covers parts [chunk_begin[c], chunk_begin[c+1]);
 * chunk_slot[c] = -1 if the chunk covers its whole window, else its row in
 * `partial` ([n_slots][n_heads][8][F+2] fp32 scratch); multi_chunk_begin holds
 * (first, end) chunk pairs of the n_multi windows spread over several chunks.
 * row_max / row_sum ([n_heads][n_nodes], may be NULL) receive the softmax
 * statistics for the backward pass; when row_sum is given the aggregation
 * also runs with the probabilities split into a hi + lo pair of 16-bit
 * values, so the output is fp32-consistent with them (the backward relies on
 * dout . out matching its recomputed probabilities).  8-row windows, F in {32, 64, 128},
 * fp16 or bf16 X'.  Every row < n_nodes of out is written. */
ATT_API int att_gat_forward(const int32_t *rowptr, const int32_t *col, const uint32_t *slot_mask,
                   const int32_t *window_of_part, int64_t n_parts,
                   const int32_t *chunk_begin, const int32_t *chunk_slot, int64_t n_chunks,
                   const int32_t *multi_chunk_begin, int64_t n_multi, int window, int wide,
                   const void *Xp, int x_dtype, int64_t n_nodes, int64_t n_heads, int64_t F,
                   int64_t ldx, int mode, const float *s0, const float *s1, float slope,
                   float *out, int64_t ldo, float *row_max, float *row_sum, float *partial,
                   int32_t *err_flag, void *stream);

/* Backward of the additive GAT layer (mode 1 of att_gat_forward), fused: with
 * the forward's row max / sum and c[h][i] = dout_i . out_i,
 *   p_ij = exp(LeakyReLU(s0_i + s1_j) - m_i) / l_i,
 *   dz_ij = p_ij (dout_i . X'_j - c_i) LeakyReLU'(s0_i + s1_j),
 *   dXp[j] += p_ij dout_i  (SpMM adjoint),  ds1[j] += dz_ij,  ds0[i] += dz_ij,
 * in one pass over the block format of the TRANSPOSED graph (for a symmetric
 * graph, the forward format itself).  dXp, ds0, ds1 are accumulated
 * (red.add): zero them first.  dout_lo (may be NULL) is dout minus its
 * rounding to the 16-bit type: with it both products run as a hi + lo pair,
 * which keeps bf16 gradients at fp16-like accuracy.  Replaces the backward of
 * end2end_ori/gat_final/mgat_csr/mgat_conv.py:34-151 (two rowsum SpMMs, an
 * SDDMM, a broadcast and a transposed SpMM). */
ATT_API int att_gat_backward(const int32_t *rowptr_t, const int32_t *col_t,
                   const uint32_t *slot_mask_t, const int32_t *window_of_part_t,
                   int64_t n_parts_t, int window, int wide, const void *Xp, const void *dout,
                   const void *dout_lo, int x_dtype, int64_t n_nodes, int64_t n_heads, int64_t F, int64_t ldx,
                   int64_t ldd, const float *s0, const float *s1, const float *row_max,
                   const float *row_sum, const float *c, float slope, float *dXp, int64_t ldg,
                   float *ds0, float *ds1, int32_t *err_flag, void *stream);

/* Row softmax of per-edge logits over CSR rows, optionally after LeakyReLU:
 * out[h][e] = exp(x_e - m_r) / l_r with x = LeakyReLU(logits[h][e]) when
 * leaky != 0, m_r the row max and l_r = sum exp(x - m_r) (fp32; written to
 * row_max / row_sum [H][n_rows] when not NULL; -inf and 0 for rows without
 * edges).  out: fp32, fp16 or bf16, [H] rows of out_stride_h.  Replaces the
 * exp -> rowsum -> divide ops of the reference's GAT composition
 * (end2end_ori/gat_final/mgat_csr/mgat_conv.py:173-198), with the row max
 * subtracted so exp cannot overflow. */
ATT_API int att_edge_softmax(const int32_t *rowptr, int64_t n_rows, const float *logits,
                   int64_t logit_stride_h, int64_t n_heads, float slope, int leaky, void *out,
                   int out_dtype, int64_t out_stride_h, float *row_max, float *row_sum,
                   void *stream);

/* The elementwise ends of the fused GAT backward, one pass over [N, H*F]
 * each (no counterpart in the reference, whose backward does them as separate
 * torch ops between its extension calls:
 * end2end_ori/gat_final/mgat_csr/mgat_conv.py:34-151).
 *   att_gat_grad_prepare: c[h][n] = dout[n, hF:hF+F] . out[n, hF:hF+F] (fp32)
 *     and dout split into dout_hi = dtype(dout), dout_lo = dtype(dout - hi),
 *     the inputs att_gat_backward takes.
 *   att_gat_grad_finish: dX[n, hF+f] = dtype(dXp + ds0[h][n] a0[h][f] +
 *     ds1[h][n] a1[h][f]), and da0[h][f] += sum_n ds0[h][n] Xp[n, hF+f], da1
 *     likewise (fp32 atomics: zero da0 / da1 first).  dtype: fp16 or bf16. */
ATT_API int att_gat_grad_prepare(const float *dout, int64_t ldd, const float *out, int64_t ldo,
                   int64_t n_nodes, int64_t n_heads, int64_t F, void *dout_hi, void *dout_lo,
                   int dtype, int64_t ldh, float *c, void *stream);
ATT_API int att_gat_grad_finish(const float *dXp, int64_t ldg, const float *ds0, const float *ds1,
                   const float *a0, const float *a1, const void *Xp, int dtype, int64_t ldx,
                   int64_t n_nodes, int64_t n_heads, int64_t F, void *dX, int64_t ld_dx,
                   float *da0, float *da1, void *stream);

/* ======================================================================
 * Batched SpMM over many graphs in one launch (the serving loop's kernel; no
 * counterpart in the reference, which runs one graph per call).
 *
 * Work is cut into GROUPS: runs of at most group_parts consecutive parts of
 * one window (att_spmm_groups builds them).  A window covered by one group is stored
 * directly; a longer window's groups write partial sums to `partial` slots that
 * a second pass adds in group order.  No atomics: Y is bit-identical whatever
 * other jobs share the launch.
 * ====================================================================== */
typedef struct {
    const int32_t *rowptr, *col;            /* block format (8-row windows, 8-wide, fp16 values) */
    const void *val;
    const int32_t *window_of_part;
    int64_t n_parts;
    const int32_t *group_part;              /* [n_groups + 1]: first part of each group, then n_parts */
    const int32_t *group_slot;              /* [n_groups]: -1 = whole window, else partial slot */
    const int32_t *red_first;               /* [n_red + 1]: first group of each multi-group window */
    const int32_t *empty_win;               /* [n_empty]: output windows that own no part */
    float *partial;                         /* [n_slots, 8, F] fp32, 16-byte aligned (null if n_slots == 0) */
    int64_t n_groups, n_red, n_slots, n_empty;
    const void *X;                          /* fp16 [n_x, F], F and row stride ldx multiples of 8 */
    int64_t n_x, F, ldx;
    float *Y;                               /* fp32 [m_out, F], row stride ldy */
    int64_t m_out, ldy;
    int64_t item_begin;   /* exclusive prefix of work items (n_groups * ceil(F/64)) */
    int64_t empty_begin;  /* exclusive prefix of empty windows (n_empty) */
    int64_t red_begin;    /* exclusive prefix of multi-group windows (n_red) */
} att_spmm_job;

/* Groups of a block format for att_spmm_batched (device arrays; stream-ordered,
 * no host synchronisation).  Inputs: window_of_part [n_parts] (non-decreasing),
 * n_windows = output windows (ceil(m_out / 8)), group_parts in [1, 1024].
 * Outputs (device, caller-allocated): group_part and red_first n_parts + 1
 * entries, group_slot max(n_parts, 1), empty_win max(n_windows, 1); `counts`
 * (device int64[4]) receives {n_groups, n_red, n_slots, n_empty}.  `scratch`
 * holds att_spmm_groups_scratch_bytes(n_parts, n_windows) bytes. */
ATT_API size_t att_spmm_groups_scratch_bytes(int64_t n_parts, int64_t n_windows);
ATT_API int att_spmm_groups(const int32_t *window_of_part, int64_t n_parts, int64_t n_windows,
                  int group_parts, int32_t *group_part, int32_t *group_slot, int32_t *red_first,
                  int32_t *empty_win, int64_t *counts, void *scratch, size_t scratch_bytes,
                  void *stream);

/* Device address of page-locked (pinned) host memory, for kernels that write
 * results straight to the host (a Y of att_spmm_batched may live there: the
 * launch only writes Y).  ATT_ERR_INVALID if `host` is not mapped pinned memory. */
ATT_API int att_host_device_pointer(const void *host, void **device);

/* Grid size (persistent: SMs x resident CTAs) to launch att_spmm_batched with. */
ATT_API size_t att_spmm_batched_grid(void);

/* Y_j = A_j X_j for every job of the DEVICE table `jobs`; `header` (device,
 * int64[5]) holds {n_jobs >= 1, total work items, total empty windows, total
 * multi-group windows, scratch (the work-queue counter, reset by the launch)}.
 * The launch reads the job count and sizes from device memory, so a captured
 * CUDA graph can be replayed after the table and header are rewritten.  Every
 * row < m_out of every Y is written.  Offsets are 32-bit: each job needs
 * n_x * ldx, m_out * ldy and n_slots * 8 * F below 2^31 - 4096 and the total
 * work items below 2^31 - grid * 4; a job that does not fit is skipped.
 * err_flag (optional) gets bit 1 for a column id outside [0, n_x), bit 2 for
 * a part off the 8-column grid, bit 8 for a job or item count that does not
 * fit 32-bit offsets. */
ATT_API int att_spmm_batched(const att_spmm_job *jobs, int64_t *header, int64_t grid,
                   int window, int wide, int32_t *err_flag, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* ATT_GB300_H */
