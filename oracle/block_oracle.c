/*
 * oracle/block_oracle.c -- CPU restatement of the row-window block conversion.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker for the CUDA conversion
 * kernels; only tests, the smoke entry and the bench's CPU-baseline leg load
 * it.  The product path never calls it.
 *
 * It restates, in plain C and in its own code, the algorithm of the
 * reference's CPU conversion:
 *   - blockProcess_fp16_balance   gcn/Block_gcn/example.cpp:48-200
 *   - blockProcess_tf32_balance   gcn/Block_gcn/example.cpp:203-348
 *   - blockProcess_sddmm_balance_gnn[_trans] (declared Block/include/example.h:4-6;
 *     source absent from the reference tree) -- the same window/part layout
 *     with the value array replaced by the CSR edge id of each slot (-1 in
 *     padding), as consumed by benchmark-v3/sddmm-benchmark/include/output_tile.h:15-37,
 *     plus the edge id of the mirrored edge (j,i) for the transposed map.
 *
 * Per window i of `window` consecutive rows (only the first rows/window
 * windows; trailing rows are dropped, example.cpp:56-57):
 *   1. sorted, de-duplicated union of the rows' column ids     (example.cpp:66-67)
 *   2. padded with -1 to a multiple of `wide`                   (example.cpp:69-81)
 *   3. slot value at [block][row-in-window][col-in-block]
 *      = deg[row] * deg[col]; duplicates overwrite              (example.cpp:93-108)
 *      fp16: half(float(deg_r) * float(deg_c)), round-to-nearest-even
 *   4. blocks = pad/wide split into parts of <= part blocks; each part emits
 *      the pair (real columns, padding columns); `atomic` = 1 when the window
 *      is split                                                 (example.cpp:112-152)
 *      fp16 skips empty windows (example.cpp:113); tf32 emits a (0,0) part
 *      for them (example.cpp:267-273)  -> `emit_empty`
 *   5. concatenated in window order                              (example.cpp:166-175)
 *
 * Map outputs (GAT form): map[slot] = the largest CSR edge id that lands in
 * the slot (the last duplicate in CSR order), -1 in empty slots;
 * map_t[slot] = the last CSR edge id of (col,row) within row `col`, -1 if the
 * mirrored edge is absent.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
    int64_t n_parts;   /* number of parts */
    int64_t n_cols;    /* total padded condensed columns */
    int32_t *rowptr;   /* 2*n_parts+1 */
    int32_t *col;      /* n_cols */
    uint16_t *val16;   /* n_cols*window, fp16 bits (deg_kind 1) */
    float *val32;      /* n_cols*window (deg_kind 2) */
    int32_t *map;      /* n_cols*window (want_map) */
    int32_t *map_t;    /* n_cols*window (want_trans) */
    int32_t *window;   /* n_parts */
    int32_t *atomic;   /* n_parts */
} oracle_blocks;

/* ---- IEEE binary16 <-> binary32, round to nearest even ----------------- */
static float f16_to_f32(uint16_t h) {
    uint32_t sign = (uint32_t)(h & 0x8000) << 16;
    uint32_t e = (h >> 10) & 0x1f, m = h & 0x3ff, bits;
    if (e == 0) {
        if (m == 0) {
            bits = sign;
        } else { /* subnormal: normalise */
            int sh = 0;
            while (!(m & 0x400)) { m <<= 1; sh++; }
            m &= 0x3ff;
            bits = sign | ((uint32_t)(113 - sh) << 23) | (m << 13);
        }
    } else if (e == 31) {
        bits = sign | 0x7f800000u | (m << 13);
    } else {
        bits = sign | ((e + 112) << 23) | (m << 13);
    }
    float f;
    memcpy(&f, &bits, 4);
    return f;
}

static uint16_t f32_to_f16(float f) {
    uint32_t x;
    memcpy(&x, &f, 4);
    uint16_t sign = (uint16_t)((x >> 16) & 0x8000);
    int exp = (int)((x >> 23) & 0xff);
    uint32_t mant = x & 0x7fffff;
    if (exp == 0xff) return (uint16_t)(sign | 0x7c00 | (mant ? 0x200 : 0));
    int e = exp - 112; /* rebias 127 -> 15 */
    if (e >= 31) return (uint16_t)(sign | 0x7c00);
    if (e <= 0) {
        if (e < -10) return sign;
        uint32_t m24 = mant | 0x800000u;
        int shift = 14 - e; /* 14..24 */
        uint32_t hm = m24 >> shift;
        uint32_t rem = m24 & ((1u << shift) - 1u);
        uint32_t halfway = 1u << (shift - 1);
        if (rem > halfway || (rem == halfway && (hm & 1u))) hm++;
        return (uint16_t)(sign | hm);
    }
    uint32_t hm = mant >> 13, rem = mant & 0x1fff;
    uint16_t h = (uint16_t)(sign | ((uint32_t)e << 10) | hm);
    if (rem > 0x1000 || (rem == 0x1000 && (hm & 1u))) h++;
    return h;
}

uint16_t oracle_f32_to_f16(float f) { return f32_to_f16(f); }
float oracle_f16_to_f32(uint16_t h) { return f16_to_f32(h); }

static int cmp_i32(const void *a, const void *b) {
    int32_t x = *(const int32_t *)a, y = *(const int32_t *)b;
    return (x > y) - (x < y);
}

/* first index in sorted u[0..n) equal to key (key is known to be present) */
static int64_t find_sorted(const int32_t *u, int64_t n, int32_t key) {
    int64_t lo = 0, hi = n;
    while (lo < hi) {
        int64_t mid = (lo + hi) >> 1;
        if (u[mid] < key) lo = mid + 1; else hi = mid;
    }
    return lo;
}

void oracle_free(oracle_blocks *b) {
    if (!b) return;
    free(b->rowptr); free(b->col); free(b->val16); free(b->val32);
    free(b->map); free(b->map_t); free(b->window); free(b->atomic);
    memset(b, 0, sizeof(*b));
}

/*
 * deg_kind: 0 = no values, 1 = fp16 degrees (uint16 bits), 2 = fp32 degrees.
 * Returns 0 on success, -1 on bad arguments, -2 on allocation failure.
 */
int oracle_block_convert(const int32_t *rowptr, const int32_t *col, int64_t n_rows,
                         const void *deg, int deg_kind, int window, int wide,
                         int part, int emit_empty, int want_map, int want_trans,
                         oracle_blocks *out) {
    memset(out, 0, sizeof(*out));
    if (window <= 0 || wide <= 0 || part <= 0 || n_rows < 0) return -1;
    int64_t n_win = n_rows / window;

    /* pass 1: per-window unique counts -> sizes */
    int64_t *ucount = (int64_t *)calloc((size_t)(n_win + 1), sizeof(int64_t));
    int64_t max_e = 0;
    for (int64_t w = 0; w < n_win; ++w) {
        int64_t e = (int64_t)rowptr[(w + 1) * window] - rowptr[w * window];
        if (e > max_e) max_e = e;
    }
    int32_t *buf = (int32_t *)malloc((size_t)(max_e + 1) * sizeof(int32_t));
    if (!ucount || !buf) { free(ucount); free(buf); return -2; }
    int64_t total_cols = 0, total_parts = 0;
    for (int64_t w = 0; w < n_win; ++w) {
        int64_t b0 = rowptr[w * window], b1 = rowptr[(w + 1) * window];
        int64_t n = b1 - b0, u = 0;
        memcpy(buf, col + b0, (size_t)n * sizeof(int32_t));
        qsort(buf, (size_t)n, sizeof(int32_t), cmp_i32);
        for (int64_t k = 0; k < n; ++k)
            if (k == 0 || buf[k] != buf[k - 1]) u++;
        ucount[w] = u;
        int64_t pad = (u + wide - 1) / wide * wide;
        int64_t blocks = pad / wide;
        total_cols += pad;
        if (blocks == 0) total_parts += emit_empty ? 1 : 0;
        else total_parts += (blocks + part - 1) / part;
    }

    out->n_parts = total_parts;
    out->n_cols = total_cols;
    out->rowptr = (int32_t *)malloc((size_t)(2 * total_parts + 1) * sizeof(int32_t));
    out->col = (int32_t *)malloc((size_t)(total_cols + 1) * sizeof(int32_t));
    out->window = (int32_t *)malloc((size_t)(total_parts + 1) * sizeof(int32_t));
    out->atomic = (int32_t *)malloc((size_t)(total_parts + 1) * sizeof(int32_t));
    size_t nslot = (size_t)total_cols * (size_t)window + 1;
    if (deg_kind == 1) out->val16 = (uint16_t *)calloc(nslot, sizeof(uint16_t));
    if (deg_kind == 2) out->val32 = (float *)calloc(nslot, sizeof(float));
    if (want_map) out->map = (int32_t *)malloc(nslot * sizeof(int32_t));
    if (want_trans) out->map_t = (int32_t *)malloc(nslot * sizeof(int32_t));
    if (!out->rowptr || !out->col || !out->window || !out->atomic ||
        (deg_kind == 1 && !out->val16) || (deg_kind == 2 && !out->val32) ||
        (want_map && !out->map) || (want_trans && !out->map_t)) {
        free(ucount); free(buf); oracle_free(out); return -2;
    }
    if (want_map) for (size_t s = 0; s < nslot; ++s) out->map[s] = -1;
    if (want_trans) for (size_t s = 0; s < nslot; ++s) out->map_t[s] = -1;

    /* pass 2: fill */
    int64_t cbase = 0, pidx = 0;
    out->rowptr[0] = 0;
    for (int64_t w = 0; w < n_win; ++w) {
        int64_t b0 = rowptr[w * window], b1 = rowptr[(w + 1) * window];
        int64_t n = b1 - b0, u = 0;
        memcpy(buf, col + b0, (size_t)n * sizeof(int32_t));
        qsort(buf, (size_t)n, sizeof(int32_t), cmp_i32);
        for (int64_t k = 0; k < n; ++k)
            if (k == 0 || buf[k] != buf[k - 1]) buf[u++] = buf[k];
        int64_t pad = (u + wide - 1) / wide * wide;
        int64_t blocks = pad / wide;
        for (int64_t k = 0; k < pad; ++k) out->col[cbase + k] = k < u ? buf[k] : -1;

        for (int64_t r = 0; r < window; ++r) {
            int64_t row = w * window + r;
            for (int64_t e = rowptr[row]; e < rowptr[row + 1]; ++e) {
                int32_t c = col[e];
                int64_t ci = find_sorted(buf, u, c);
                int64_t slot = (cbase + (ci / wide) * wide) * window + r * wide + (ci % wide);
                if (deg_kind == 1) {
                    const uint16_t *d = (const uint16_t *)deg;
                    out->val16[slot] = f32_to_f16(f16_to_f32(d[row]) * f16_to_f32(d[c]));
                } else if (deg_kind == 2) {
                    const float *d = (const float *)deg;
                    out->val32[slot] = d[row] * d[c];
                }
                if (want_map) out->map[slot] = (int32_t)e; /* CSR order: last wins */
                if (want_trans) {
                    int32_t t = -1;
                    if (c >= 0 && c < n_rows)
                        for (int64_t f = rowptr[c]; f < rowptr[c + 1]; ++f)
                            if (col[f] == (int32_t)row) t = (int32_t)f;
                    out->map_t[slot] = t;
                }
            }
        }

        /* parts: pairs (real, padding) of the running column offset */
        int64_t padamt = pad - u;
        if (blocks == 0) {
            if (emit_empty) {
                out->rowptr[2 * pidx + 1] = (int32_t)cbase;
                out->rowptr[2 * pidx + 2] = (int32_t)cbase;
                out->window[pidx] = (int32_t)w;
                out->atomic[pidx] = 0;
                pidx++;
            }
        } else {
            int64_t nparts = (blocks + part - 1) / part;
            for (int64_t p = 0; p < nparts; ++p) {
                int64_t nb = blocks - p * part < part ? blocks - p * part : part;
                int64_t cols_p = nb * wide;
                int64_t pad_p = (p == nparts - 1) ? padamt : 0;
                int64_t start = cbase + p * part * wide;
                out->rowptr[2 * pidx + 1] = (int32_t)(start + cols_p - pad_p);
                out->rowptr[2 * pidx + 2] = (int32_t)(start + cols_p);
                out->window[pidx] = (int32_t)w;
                out->atomic[pidx] = nparts > 1 ? 1 : 0;
                pidx++;
            }
        }
        cbase += pad;
    }
    free(ucount);
    free(buf);
    return 0;
}
