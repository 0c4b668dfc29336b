// vx_build_dense_noalloc: dense-chunk construction that allocates no memory during the call.
//
// Who needs it: callers that cannot call cudaMalloc (or anything that does) while they run: code
// that records the call into a CUDA graph (allocation is not permitted during stream capture),
// frame loops and servers that fix their device memory up front and treat any allocation as a
// failure, and hosts whose device allocator belongs to another runtime. The regular entry points
// grow a device workspace on demand; this one stages the levels above the 32^3 blocks in a fixed
// array compiled into the library.
//
// Limits and sharing: the array holds VX_NOALLOC_SCRATCH_BYTES (3 MiB of device memory that every
// GPU loading the library keeps until the process exits). Chunks of depth 5-10 are reduced one CTA
// per 32^3 block (dense_cta32_kernel); for depth d >= 6 a call stages the node rows of the levels
// above those blocks and their arrival counts, 12 * n * (8 + 8^2 + ... + 8^(d-5)) bytes rounded up to
// 256 plus 4 * n * (1 + 8 + ... + 8^(d-6)) + 256 bytes (dense_octant_scratch_bytes, the layout the
// launch carves). Depths 2-5 stage nothing. Larger requests are rejected with VX_E_BUFFER before
// any work is queued. All calls share the one array: two calls whose device work
// overlaps (different streams or interners at the same time) race on it, so serialise them. The
// arrival counts a call uses are cleared (cudaMemsetAsync) before its kernel runs; every node row is
// written before it is read.
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

constexpr uint64_t kBytes = VX_NOALLOC_SCRATCH_BYTES;
// node rows (ids, LOD values) of the levels above the 32^3 blocks, then their arrival counts
static __device__ __align__(256) unsigned char g_noalloc_scratch[kBytes];

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
    const uint64_t need = max_depth >= 4 ? dense_octant_scratch_bytes(n, max_depth) : 0;
    if (need > kBytes) {
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
    if (max_depth >= 4) {
        e = launch_dense_octants(D, grids_dev, trees_dev, n, max_depth, changed_dev, scratch, num_sms, s);
    } else {
        DenseArgs a{};
        a.grids = grids_dev;
        a.trees = trees_dev;
        a.n_chunks = n;
        a.depth = max_depth;
        a.changed = changed_dev;
        e = launch_dense_blocks(D, a, num_sms, s);
    }
    if (e == cudaSuccess) e = launch_epoch_refcounts(D, num_sms, s);
    if (e != cudaSuccess) {
        interner_set_error(it, cudaGetErrorString(e));
        return VX_E_CUDA;
    }
    return VX_OK;
}
