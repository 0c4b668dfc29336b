// vx_build_dense_noalloc: dense-chunk construction that allocates no memory during the call.
//
// Who needs it: callers that cannot call cudaMalloc (or anything that does) while they run: code
// that records the call into a CUDA graph (allocation is not permitted during stream capture),
// frame loops and servers that fix their device memory up front and treat any allocation as a
// failure, and hosts whose device allocator belongs to another runtime. The regular entry points
// grow a device workspace on demand; this one stages the levels above the 32^3 blocks in a fixed
// array compiled into the library.
//
// Limits and sharing: the array holds VX_NOALLOC_SCRATCH_ENTRIES block-level entries (3 MiB of
// device memory that every GPU loading the library keeps until the process exits). A call needs
// n * (8^(d-5) + 8^(d-6) + ... + 8) entries for chunks of depth d > 5 (none for d <= 5); larger
// requests are rejected with VX_E_BUFFER before any work is queued. All calls share the one array:
// two calls whose device work overlaps (different streams or interners at the same time) race on
// it, so serialise them. The part of the array a call uses is cleared (cudaMemsetAsync) before its
// kernels run.
//
// Set-up: the array's device address is resolved with cudaGetSymbolAddress once per device, on the
// first call made with that device current; make that first call before any stream capture.
#include <mutex>
#include <string>

#include "../../include/voxelis_gb300.h"
#include "vx_launch.h"

namespace vxg {
bool interner_parts(vx_interner *it, DevInterner *dev, cudaStream_t *stream, int *num_sms, uint32_t *flags,
                    bool marks_trees);
void interner_set_error(vx_interner *it, const char *msg);
}  // namespace vxg

using namespace vxg;

namespace {

constexpr uint64_t kEntries = VX_NOALLOC_SCRATCH_ENTRIES;
// block-root ids (8 B) then their LOD values (4 B) for every staged level
static __device__ __align__(256) unsigned char g_noalloc_scratch[kEntries * 12];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
unsigned char *g_scratch_ptr[kMaxDevices] = {};

// Device address of the scratch array for the current device (resolved on first use).
cudaError_t scratch_for_current_device(unsigned char **out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_ptr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_scratch_ptr[dev] = static_cast<unsigned char *>(p);
    }
    *out = g_scratch_ptr[dev];
    return cudaSuccess;
}

}  // namespace

extern "C" int vx_build_dense_noalloc(vx_interner *it, uint32_t n, const vx_tree *trees_dev, const void *grids_dev,
                                      uint8_t *changed_dev, int max_depth) {
    DevInterner D;
    cudaStream_t s;
    int num_sms;
    uint32_t flags;
    if (!interner_parts(it, &D, &s, &num_sms, &flags, false)) return VX_E_INVALID_ARG;
    if (n && (!trees_dev || !grids_dev)) return VX_E_INVALID_ARG;
    const int limit = (flags & VX_PATCH_P2) ? 11 : 7;
    if (max_depth < 0 || max_depth >= limit) {
        interner_set_error(it, "Max depth exceeds allowed limit");
        return VX_E_DEPTH;
    }
    if (max_depth < 2) {
        interner_set_error(it, "batch apply needs max_depth >= 2 (usize underflow in the reference)");
        return VX_E_REF_PANIC;
    }
    if ((uintptr_t)grids_dev % 16) {
        interner_set_error(it, "grids must be 16-byte aligned");
        return VX_E_INVALID_ARG;
    }
    uint64_t need = 0;
    for (int k = max_depth - 5; k >= 1; --k) need += (uint64_t)n << (3 * k);
    if (need > kEntries) {
        interner_set_error(it, "request exceeds the fixed scratch of vx_build_dense_noalloc");
        return VX_E_BUFFER;
    }
    unsigned char *scratch = nullptr;
    cudaError_t e = scratch_for_current_device(&scratch);
    if (e != cudaSuccess) {
        interner_set_error(it, cudaGetErrorString(e));
        return VX_E_CUDA;
    }
    interner_parts(it, &D, &s, &num_sms, &flags, true);
    if (n == 0) return VX_OK;

    DenseArgs a{};
    a.grids = grids_dev;
    a.trees = trees_dev;
    a.n_chunks = n;
    a.depth = max_depth;
    a.bdepth = max_depth < 5 ? max_depth : 5;
    a.blocks_per_chunk = 1u << (3 * (max_depth - a.bdepth));
    a.changed = changed_dev;
    uint64_t *ids = reinterpret_cast<uint64_t *>(scratch);
    uint32_t *vals = reinterpret_cast<uint32_t *>(scratch + kEntries * 8);
    if (need) {
        if ((e = cudaMemsetAsync(ids, 0, need * 8, s)) != cudaSuccess ||
            (e = cudaMemsetAsync(vals, 0, need * 4, s)) != cudaSuccess) {
            interner_set_error(it, cudaGetErrorString(e));
            return VX_E_CUDA;
        }
    }
    a.block_roots = ids;
    a.block_vals = vals;
    e = launch_dense_blocks(D, a, num_sms, s);
    uint64_t *in_ids = ids;
    uint32_t *in_vals = vals;
    uint64_t off = (uint64_t)n << (3 * (max_depth - a.bdepth));
    for (int k = max_depth - 6; k >= 0 && e == cudaSuccess; --k) {
        const uint64_t np = (uint64_t)n << (3 * k);
        uint64_t *out_ids = k > 0 ? ids + off : nullptr;
        uint32_t *out_vals = k > 0 ? vals + off : nullptr;
        e = launch_fresh_level(D, in_ids, in_vals, out_ids, out_vals, np, k == 0, trees_dev, changed_dev, s);
        in_ids = out_ids;
        in_vals = out_vals;
        off += np;
    }
    if (e == cudaSuccess) e = launch_epoch_refcounts(D, num_sms, s);
    if (e != cudaSuccess) {
        interner_set_error(it, cudaGetErrorString(e));
        return VX_E_CUDA;
    }
    return VX_OK;
}
