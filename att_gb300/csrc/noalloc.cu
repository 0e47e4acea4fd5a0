// noalloc.cu -- the block conversion with its scratch in a fixed, library-owned
// device array, for callers that must not allocate device memory.
//
// Who needs this: hosts that own every byte of device memory through their
// own arena or budget (plugin hosts, serving loops that admit work against a
// fixed HBM budget) and forbid a library from allocating behind their back,
// and latency-critical callers that cannot afford cudaMalloc/cudaFree, which
// can synchronise the whole device.  att_block_plan/att_block_fill need a
// caller-allocated workspace; this entry point needs none.
//
// The scratch is one file-scope __device__ array of kStaticScratchBytes.  Every
// process that loads the library holds it on every GPU it touches, until exit.
// Host code cannot use the array's name as a device address (on the host it is
// only a stand-in symbol), so the address is looked up once per device with
// cudaGetSymbolAddress while that device is current, checked, cached, and then
// passed to the kernels.  The first call on a device performs this set-up.
// The cached address is not refreshed after cudaDeviceReset: a process that
// resets a device must not call this entry point afterwards.
//
// The call returns only when its GPU work is done (the plan synchronises the
// stream to read the sizes, the fill to read the device-side checks), so it
// cannot be captured into a CUDA graph and successive calls never overlap.
// All calls share the one array and it keeps the previous call's contents:
// everything the kernels read is cleared or rewritten by the call itself
// (flags, per-window counts and bitmaps are zeroed, merge flags cleared).
// Calls from two host threads at the same time race on the array; callers
// must order them.
#include "att_common.cuh"

#include <mutex>

namespace att {
namespace {

constexpr size_t kStaticScratchBytes = 64ull << 20;  // 64 MiB
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_block_scratch[kStaticScratchBytes];

std::mutex g_scratch_mutex;
void *g_scratch_ptr[kMaxDevices] = {nullptr};

// Device address of the scratch array for the current device (set up once).
int scratch_address(void **out) {
    int dev = 0;
    ATT_CUDA(cudaGetDevice(&dev), "cudaGetDevice");
    ATT_CHECK(dev >= 0 && dev < kMaxDevices, ATT_ERR_UNSUPPORTED, "device index %d >= %d", dev,
              kMaxDevices);
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (g_scratch_ptr[dev] == nullptr) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_block_scratch);
        if (e != cudaSuccess || p == nullptr) {
            set_error("cudaGetSymbolAddress of the static scratch failed: %s",
                      cudaGetErrorString(e));
            return ATT_ERR_CUDA;
        }
        g_scratch_ptr[dev] = p;
    }
    *out = g_scratch_ptr[dev];
    return ATT_OK;
}

}  // namespace
}  // namespace att

using namespace att;

extern "C" size_t att_block_convert_noalloc_max_scratch(void) { return kStaticScratchBytes; }

extern "C" int att_block_convert_noalloc(
    const int32_t *rowptr, const int32_t *col, int64_t n_rows, int64_t nnz, int64_t n_cols,
    int window, int wide, int part, int emit_empty, const void *deg, int deg_dtype,
    int32_t *out_rowptr, int32_t *out_col, void *out_val, int val_dtype, int32_t *out_map,
    int32_t *out_map_t, int32_t *out_edge_slot, int32_t *out_window, int32_t *out_atomic,
    int64_t max_parts, int64_t max_condensed, int64_t *n_parts_out, int64_t *n_condensed_out,
    void *stream) {
    clear_error();
    ATT_CHECK(window > 0 && n_rows >= 0 && nnz >= 0 && n_cols >= 0, ATT_ERR_INVALID,
              "invalid sizes or window");
    ATT_CHECK(n_parts_out && n_condensed_out, ATT_ERR_INVALID, "null size outputs");
    const size_t need = att_block_workspace_bytes(n_rows, nnz, n_cols, window);
    ATT_CHECK(need <= kStaticScratchBytes, ATT_ERR_WORKSPACE,
              "graph needs %zu bytes of scratch; the allocation-free conversion holds at most "
              "%zu (use att_block_plan/att_block_fill with a caller workspace)",
              need, kStaticScratchBytes);
    void *scratch = nullptr;
    int s = scratch_address(&scratch);
    if (s != ATT_OK) return s;
    int64_t n_parts = 0, n_cond = 0;
    s = att_block_plan(rowptr, col, n_rows, nnz, n_cols, window, wide, part, emit_empty, scratch,
                       kStaticScratchBytes, &n_parts, &n_cond, stream);
    if (s != ATT_OK) return s;
    *n_parts_out = n_parts;
    *n_condensed_out = n_cond;
    ATT_CHECK(n_parts <= max_parts && n_cond <= max_condensed, ATT_ERR_WORKSPACE,
              "outputs too small: need %lld parts and %lld condensed columns, have %lld and %lld",
              (long long)n_parts, (long long)n_cond, (long long)max_parts,
              (long long)max_condensed);
    return att_block_fill(rowptr, col, n_rows, nnz, n_cols, window, wide, part, emit_empty, deg,
                          deg_dtype, scratch, kStaticScratchBytes, out_rowptr, out_col, out_val,
                          val_dtype, out_map, out_map_t, out_edge_slot, out_window, out_atomic,
                          stream);
}
