// Host implementation of the C ABI declared in include/voxelis_gb300.h.
//
// Owns the device interner (vx_device.cuh), the device tree table (roots + depths), a growable
// device workspace for the batched paths, pinned staging for host<->device copies, and the host
// Batch buffers. Every entry point returns a status; device failures are sticky error bits that are
// read back at the synchronising calls.
#include <algorithm>
#include <atomic>
#include <cstring>
#include <functional>
#include <new>
#include <string>
#include <thread>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "../../include/voxelis_gb300.h"
#include "vx_launch.h"

using namespace vxg;

namespace vxg {
static std::atomic<uint64_t> g_launches{0};
void count_launches(uint64_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
}

// ---- host Batch<T> (core/batch.rs:39-240) ------------------------------------------------------
struct vx_batch {
    int depth = 0;
    int vbits = 8;
    uint32_t flags = 0;
    uint64_t groups = 0;
    std::vector<uint8_t> set, clear;
    std::vector<uint8_t> vals;  // groups * 8 voxels of vbits/8 bytes
    bool has_fill = false;
    uint32_t fill = 0;
    bool has_patches = false;
    // groups written since the last clear, in first-write order (the staging of an apply visits
    // only these); all_touched after a dense fill, which writes every group
    mutable std::vector<uint32_t> touched;
    mutable bool touched_sorted = true;
    bool all_touched = false;
};

namespace {

constexpr uint32_t kStickyMask = ERR_OOM | ERR_TABLE_FULL | ERR_TIMEOUT | ERR_INTERNAL | ERR_REF_UB;
constexpr uint8_t kUnused = TREE_UNUSED;

uint32_t morton_encode(int32_t x, int32_t y, int32_t z) {
    auto split = [](uint32_t v) {
        v &= 0x3FF;
        v = (v | (v << 16)) & 0x30000FF;
        v = (v | (v << 8)) & 0x300F00F;
        v = (v | (v << 4)) & 0x30C30C3;
        v = (v | (v << 2)) & 0x9249249;
        return v;
    };
    return split((uint32_t)x) | (split((uint32_t)y) << 1) | (split((uint32_t)z) << 2);
}

int depth_limit(uint32_t flags) { return (flags & VX_PATCH_P2) ? 11 : 7; }

// Records group gi as touched (first write since the last clear).
inline void batch_touch(vx_batch *b, uint64_t gi) {
    if (b->all_touched || (b->set[gi] | b->clear[gi])) return;
    if (!b->touched.empty() && b->touched.back() > gi) b->touched_sorted = false;
    b->touched.push_back((uint32_t)gi);
}

uint64_t batch_touched_count(const vx_batch *b) {
    if (!b->all_touched) return b->touched.size();
    uint64_t n = 0;
    for (uint64_t g = 0; g < b->groups; ++g) n += (b->set[g] | b->clear[g]) != 0;
    return n;
}

// Calls f(g) for every group with a set or clear bit, in ascending group order.
template <class F>
void batch_for_each_touched(const vx_batch *b, F f) {
    // a dense fill, or a touched list long enough that scanning the group arrays in order beats
    // sorting it
    if (b->all_touched || (!b->touched_sorted && b->touched.size() * 16 > b->groups)) {
        for (uint64_t g = 0; g < b->groups; ++g)
            if (b->set[g] | b->clear[g]) f(g);
        return;
    }
    if (!b->touched_sorted) {
        std::sort(b->touched.begin(), b->touched.end());
        b->touched_sorted = true;
    }
    // sparse groups: their mask and value bytes are fetched a few groups ahead of use
    const size_t m = b->touched.size(), vb = (size_t)b->vbits / 8;
    for (size_t k = 0; k < m; ++k) {
        if (k + 16 < m) {
            const uint64_t gp = b->touched[k + 16];
            __builtin_prefetch(b->set.data() + gp);
            __builtin_prefetch(b->clear.data() + gp);
            __builtin_prefetch(b->vals.data() + 8 * vb * gp);
        }
        f((uint64_t)b->touched[k]);
    }
}

struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
    cudaError_t reserve(size_t n) {
        if (n <= bytes) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
        size_t want = std::max(n, (size_t)1 << 20);
        cudaError_t e = cudaMalloc(&p, want);
        if (e == cudaSuccess) bytes = want;
        return e;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
};

// Pieces of a host-memory dense build (the copy of piece k+1 overlaps the build of piece k), as
// relative sizes. Only the last piece's build is left once the copies end, so it is the smallest;
// a piece's build is latency-bound, so small pieces build below the copy rate. Measured on the
// 4096-chunk dunes (e2e ms): {2,2,2,1} 0.787, equal quarters 0.796, {3,3,2} 0.799, equal thirds
// 0.804, {4,4,4,3,1} 0.822; 8 and 16 equal pieces were slower still.
#ifndef VX_PIECE_PLAN
#define VX_PIECE_PLAN 2
#endif
#if VX_PIECE_PLAN == 1
constexpr int kPieceWeights[] = {4, 4, 4, 3, 1};
#elif VX_PIECE_PLAN == 2
constexpr int kPieceWeights[] = {2, 2, 2, 1};
#elif VX_PIECE_PLAN == 3
constexpr int kPieceWeights[] = {1, 1, 1};
#elif VX_PIECE_PLAN == 4
constexpr int kPieceWeights[] = {3, 3, 2};
#else
constexpr int kPieceWeights[] = {1, 1, 1, 1};
#endif
constexpr int kCopyPieces = (int)(sizeof(kPieceWeights) / sizeof(kPieceWeights[0]));

struct HostBuf {
    void *p = nullptr;
    size_t bytes = 0;
    cudaError_t reserve(size_t n) {
        if (n <= bytes) return cudaSuccess;
        if (p) cudaFreeHost(p);
        p = nullptr;
        bytes = 0;
        size_t want = std::max(n + n / 4, (size_t)1 << 20);
        cudaError_t e = cudaHostAlloc(&p, want, cudaHostAllocDefault);
        if (e == cudaSuccess) bytes = want;
        return e;
    }
    void release() {
        if (p) cudaFreeHost(p);
        p = nullptr;
        bytes = 0;
    }
};

struct Carve {
    char *base;
    size_t off = 0;
    explicit Carve(void *b) : base((char *)b) {}
    template <class T>
    T *take(size_t n) {
        off = (off + 255) & ~(size_t)255;
        T *r = reinterpret_cast<T *>(base + off);
        off += n * sizeof(T);
        return r;
    }
    static size_t need(std::initializer_list<size_t> bytes) {
        size_t s = 0;
        for (size_t b : bytes) s = ((s + 255) & ~(size_t)255) + b;
        return s + 256;
    }
};

}  // namespace

struct vx_interner {
    int vbits = 8;
    uint32_t flags = 0;
    uint64_t capacity = 0;
    uint64_t node_size = 0;
    uint64_t table_slots = 0;
    DevInterner dev{};
    cudaStream_t stream = nullptr;
    cudaStream_t own_stream = nullptr;
    cudaStream_t copy_stream = nullptr;       // host-to-device copies that overlap device work
    cudaEvent_t copy_events[kCopyPieces] = {};
    int num_sms = 148;
    int apply_threads = 256;       // launch shape of the batched-apply kernels (autotuned)
    int apply_blocks_per_sm = 8;
    int apply_single = 1;          // 1: the whole apply as one cooperative launch; 0: a launch per phase
    // tree table
    uint32_t tree_cap = 0;
    std::vector<uint8_t> tree_depth, tree_used, tree_maybe_nonempty;
    std::vector<uint32_t> tree_stamp;  // duplicate detection within one call
    uint32_t stamp_epoch = 0;
    std::vector<uint32_t> free_trees;
    uint32_t tree_count = 0;
    bool all_trees_unknown = false;
    // device scratch
    DevBuf ws;
    DevBuf staging;  // host-memory arguments copied to the device
    HostBuf pinned;  // pinned host memory for staging batched applies
    uint32_t *frontier = nullptr;  // 2 * capacity u32 (the single-thread queue aliases it under P3)
    uint64_t *seq_queue = nullptr;
    uint64_t seq_queue_cap = 0;
    unsigned long long *d_live = nullptr;
    int *d_status = nullptr;
    unsigned long long *scan_status = nullptr;  // kScanStatusTiles look-back words, zero between scans
    // pinned staging
    DevCounters *h_ctr = nullptr;
    int *h_status = nullptr;
    unsigned long long *h_live = nullptr;
    std::string last_error;
    // instrumentation: event pairs recorded around the phases while profiling is on
    bool profile = false;
    std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> marks;
    std::vector<cudaEvent_t> event_pool;
};

namespace {

cudaEvent_t take_event(vx_interner *it) {
    if (!it->event_pool.empty()) {
        cudaEvent_t e = it->event_pool.back();
        it->event_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

// Records CUDA events around one phase on the interner's stream while profiling is enabled.
struct Phase {
    vx_interner *it;
    int id;
    cudaEvent_t a = nullptr, b = nullptr;
    Phase(vx_interner *i, int phase) : it(i), id(phase) {
        if (!it->profile) return;
        a = take_event(it);
        b = take_event(it);
        cudaEventRecord(a, it->stream);
    }
    ~Phase() {
        if (!a) return;
        cudaEventRecord(b, it->stream);
        it->marks.push_back({id, {a, b}});
    }
};

// Two back-to-back phases on the stream: `first` until next() is called, then `second` until the
// object dies (next() is the host callback launch_dense_split runs between its two kernel groups).
struct PhaseSwitch {
    vx_interner *it;
    int second;
    Phase *cur;
    PhaseSwitch(vx_interner *i, int first, int second_) : it(i), second(second_), cur(new Phase(i, first)) {}
    static void next(void *self) {
        PhaseSwitch *ps = static_cast<PhaseSwitch *>(self);
        delete ps->cur;
        ps->cur = new Phase(ps->it, ps->second);
    }
    ~PhaseSwitch() { delete cur; }
};

int set_err(vx_interner *it, int code, const std::string &msg) {
    if (it) it->last_error = msg;
    return code;
}

int cuda_fail(vx_interner *it, cudaError_t e, const char *where) {
    return set_err(it, VX_E_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

#define VX_CUDA(call)                                    \
    do {                                                 \
        cudaError_t _e = (call);                         \
        if (_e != cudaSuccess) return cuda_fail(it, _e, #call); \
    } while (0)

// Waits for the stream, reads the counters and converts device error bits into a status.
int sync_and_check(vx_interner *it) {
    VX_CUDA(cudaMemcpyAsync(it->h_ctr, it->dev.ctr, sizeof(DevCounters), cudaMemcpyDeviceToHost, it->stream));
    VX_CUDA(cudaStreamSynchronize(it->stream));
    const uint32_t err = it->h_ctr->error;
    if (!err) return VX_OK;
    const uint32_t keep = err & kStickyMask;  // OOB, INVALID and REF_PANIC leave the state usable
    if (keep != err) {
        VX_CUDA(cudaMemcpyAsync(&it->dev.ctr->error, &keep, sizeof(uint32_t), cudaMemcpyHostToDevice, it->stream));
        VX_CUDA(cudaStreamSynchronize(it->stream));
    }
    const uint32_t info = it->h_ctr->error_info;
    std::string where = " (site " + std::to_string(info) + ")";
    if (err & ERR_OOM) return set_err(it, VX_E_OOM, "Out of memory: node capacity exhausted" + where);
    if (err & ERR_TABLE_FULL) return set_err(it, VX_E_TABLE_FULL, "branch table probe limit reached" + where);
    if (err & ERR_TIMEOUT) return set_err(it, VX_E_TIMEOUT, "bounded device wait gave up" + where);
    if (err & ERR_INTERNAL) return set_err(it, VX_E_UNSUPPORTED, "internal consistency check failed" + where);
    if (err & ERR_REF_UB) return set_err(it, VX_E_REF_UB, "reference undefined behaviour (refcount underflow or release-queue overflow)" + where);
    if (err & ERR_REF_PANIC) return set_err(it, VX_E_REF_PANIC, "the reference panics on this input" + where);
    if (err & ERR_INVALID) return set_err(it, VX_E_INVALID_ARG, "unknown tree handle or depth mismatch" + where);
    if (err & ERR_OOB) return set_err(it, VX_E_OOB, "position out of bounds" + where);
    return set_err(it, VX_E_UNSUPPORTED, "unknown device error" + where);
}

cudaError_t grow_tree_table(vx_interner *it, uint32_t need) {
    if (need <= it->tree_cap) return cudaSuccess;
    uint32_t cap = std::max<uint32_t>(1024, it->tree_cap);
    while (cap < need) cap *= 2;
    uint64_t *roots = nullptr;
    uint8_t *depths = nullptr;
    cudaError_t e = cudaMalloc(&roots, cap * sizeof(uint64_t));
    if (e != cudaSuccess) return e;
    e = cudaMalloc(&depths, cap);
    if (e != cudaSuccess) {
        cudaFree(roots);
        return e;
    }
    cudaMemsetAsync(roots, 0, cap * sizeof(uint64_t), it->stream);
    cudaMemsetAsync(depths, kUnused, cap, it->stream);
    if (it->dev.roots) {
        cudaMemcpyAsync(roots, it->dev.roots, it->tree_cap * sizeof(uint64_t), cudaMemcpyDeviceToDevice, it->stream);
        cudaMemcpyAsync(depths, it->dev.depths, it->tree_cap, cudaMemcpyDeviceToDevice, it->stream);
        cudaStreamSynchronize(it->stream);
        cudaFree(it->dev.roots);
        cudaFree(it->dev.depths);
    }
    it->dev.roots = roots;
    it->dev.depths = depths;
    it->dev.tree_cap = cap;
    it->tree_cap = cap;
    it->tree_depth.resize(cap, kUnused);
    it->tree_used.resize(cap, 0);
    it->tree_maybe_nonempty.resize(cap, 0);
    return cudaSuccess;
}

bool tree_ok(vx_interner *it, vx_tree t) { return t < it->tree_count && it->tree_used[t]; }

bool value_fits(vx_interner *it, uint32_t v) { return it->vbits == 8 ? v <= 0xFFu : v <= 0xFFFFu; }

// Host-side tree helpers -------------------------------------------------------------------------
int read_root(vx_interner *it, vx_tree t, uint64_t *out) {
    VX_CUDA(cudaMemcpyAsync(out, it->dev.roots + t, sizeof(uint64_t), cudaMemcpyDeviceToHost, it->stream));
    VX_CUDA(cudaStreamSynchronize(it->stream));
    return VX_OK;
}

void maybe_rehash(vx_interner *it) {
    if (it->h_ctr->tombstones * 4 > it->table_slots) {
        launch_rehash(it->dev, it->table_slots, it->num_sms, it->stream);
        cudaStreamSynchronize(it->stream);
    }
}

// Snapshot of the node store for the verification helpers.
struct Snapshot {
    uint64_t n = 0;
    std::vector<uint64_t> ids, children;
    std::vector<uint32_t> values, refcount;
    std::vector<uint16_t> generation;
};

int take_snapshot(vx_interner *it, Snapshot &s) {
    int st = sync_and_check(it);
    if (st != VX_OK && st != VX_E_REF_PANIC && st != VX_E_OOB) return st;
    s.n = it->h_ctr->next_index;
    s.ids.resize(s.n);
    s.children.resize(s.n * 8);
    s.refcount.resize(s.n);
    s.generation.resize(s.n);
    s.values.resize(s.n);
    VX_CUDA(cudaMemcpy(s.ids.data(), it->dev.ids, s.n * 8, cudaMemcpyDeviceToHost));
    VX_CUDA(cudaMemcpy(s.children.data(), it->dev.children, s.n * 64, cudaMemcpyDeviceToHost));
    VX_CUDA(cudaMemcpy(s.refcount.data(), it->dev.refcount, s.n * 4, cudaMemcpyDeviceToHost));
    VX_CUDA(cudaMemcpy(s.generation.data(), it->dev.generation, s.n * 2, cudaMemcpyDeviceToHost));
    if (it->vbits == 8) {
        std::vector<uint8_t> v(s.n);
        VX_CUDA(cudaMemcpy(v.data(), it->dev.values, s.n, cudaMemcpyDeviceToHost));
        for (uint64_t i = 0; i < s.n; ++i) s.values[i] = v[i];
    } else {
        std::vector<uint16_t> v(s.n);
        VX_CUDA(cudaMemcpy(v.data(), it->dev.values, s.n * 2, cudaMemcpyDeviceToHost));
        for (uint64_t i = 0; i < s.n; ++i) s.values[i] = v[i];
    }
    return VX_OK;
}

int read_roots(vx_interner *it, uint32_t n, const vx_tree *trees, std::vector<uint64_t> &roots) {
    roots.resize(n);
    std::vector<uint64_t> all(it->tree_count);
    if (it->tree_count)
        VX_CUDA(cudaMemcpy(all.data(), it->dev.roots, it->tree_count * sizeof(uint64_t), cudaMemcpyDeviceToHost));
    for (uint32_t i = 0; i < n; ++i) {
        if (!tree_ok(it, trees[i])) return set_err(it, VX_E_INVALID_ARG, "unknown tree handle");
        roots[i] = all[trees[i]];
    }
    return VX_OK;
}

// ---- the batched apply ---------------------------------------------------------------------------
struct Item {
    vx_tree tree;
    const vx_batch *batch;
    uint32_t caller_index;
};

// Words of scan scratch an apply over Rp = R + 1 flags needs (block sums of the per-phase scans, or
// the per-CTA partial sums of the single-launch path).
size_t scan_words(vx_interner *it, size_t Rp) {
    return std::max(scan_tmp_words((uint32_t)Rp) * 4, apply_single_scan_words(it->num_sms));
}

// Device scratch of one batched apply over n items and R touched groups. With `own_inputs` the
// item and record input arrays are carved from the workspace too (host-staging path).
int carve_apply(vx_interner *it, uint32_t n, uint64_t R, bool own_inputs, ApplyArgs &a) {
    const size_t Rp = R + 1;
    const size_t in_items = own_inputs ? 1 : 0, in_recs = own_inputs ? 1 : 0;
    const size_t need = Carve::need({n * 4 * in_items, n, n * in_items, n * 4 * in_items, n * 8, n * 8, n * 8, n,
                                     n, R * 4 * in_recs, R * 4 * in_recs, R * in_recs, R * in_recs, R * 16 * in_recs,
                                     Rp * 4, Rp * 4, scan_words(it, Rp) * 4, R * 4, R * 4, R * 4,
                                     R * 4, R * 8, R * 8, R * 4, R * 4, Rp * 4, R * 8, R * 4, n * 8,
                                     (n + 1) * 4 * in_items});
    VX_CUDA(it->ws.reserve(need));
    Carve c(it->ws.p);
    a.mode = 0;
    a.n_items = n;
    a.n_records = (uint32_t)R;
    a.threads = it->apply_threads;
    a.blocks_per_sm = it->apply_blocks_per_sm;
    if (own_inputs) a.it_tree = c.take<uint32_t>(n);
    a.it_depth = c.take<uint8_t>(n);
    if (own_inputs) {
        a.it_flags = c.take<uint8_t>(n);
        a.it_fill = c.take<uint32_t>(n);
    }
    a.it_init = c.take<uint64_t>(n);
    a.it_old = c.take<uint64_t>(n);
    a.it_new = c.take<uint64_t>(n);
    a.it_panic = c.take<uint8_t>(n);
    a.it_changed = c.take<uint8_t>(n);
    if (own_inputs) {
        a.rec_item = c.take<uint32_t>(R);
        a.rec_group = c.take<uint32_t>(R);
        a.rec_set = c.take<uint8_t>(R);
        a.rec_clear = c.take<uint8_t>(R);
        a.rec_vals = c.take<uint16_t>(R * 8);
    }
    a.flags = c.take<uint32_t>(Rp);
    a.pos = c.take<uint32_t>(Rp);
    a.scan_tmp = c.take<uint32_t>(scan_words(it, Rp));
    a.scan_status = it->scan_status;
    a.e_item[0] = c.take<uint32_t>(R);
    a.e_item[1] = c.take<uint32_t>(R);
    a.e_path[0] = c.take<uint32_t>(R);
    a.e_path[1] = c.take<uint32_t>(R);
    a.e_id[0] = c.take<uint64_t>(R);
    a.e_id[1] = c.take<uint64_t>(R);
    a.e_val[0] = c.take<uint32_t>(R);
    a.e_val[1] = c.take<uint32_t>(R);
    a.p_start = c.take<uint32_t>(Rp);
    a.rec_id = c.take<uint64_t>(R);
    a.rec_val = c.take<uint32_t>(R);
    a.release_list = c.take<uint64_t>(n);
    if (own_inputs) a.it_first = c.take<uint32_t>((size_t)n + 1);
    return VX_OK;
}

// The set phase (its kernels count references as they create nodes and close the allocation epoch)
// and its release, then (P4) the clear pass with its own epoch and release. No host synchronisation.
int apply_sequence(vx_interner *it, ApplyArgs &a, bool clear_pass, bool check_depths = false) {
    cudaStream_t s = it->stream;
    // the roots that die are the first dying set, retired by the first release pass; a root heads a
    // subtree of height at most max_depth, whose leaves are retired by pass max_depth + 1
    const int rounds = a.max_depth > 0 && a.max_depth < 10 ? a.max_depth + 1 : 11;
    if (it->apply_single) {
        Phase ph(it, VX_PROF_APPLY);
        VX_CUDA(launch_apply_single(it->dev, a, check_depths, clear_pass, it->frontier, it->frontier + it->capacity,
                                    rounds, it->num_sms, s));
        return VX_OK;
    }
    if (check_depths) VX_CUDA(launch_item_depths(it->dev, a, s));
    for (int mode = 0; mode < (clear_pass ? 2 : 1); ++mode) {
        a.mode = mode;
        {
            Phase ph(it, VX_PROF_BOTTOM);
            VX_CUDA(launch_apply_bottom(it->dev, a, it->num_sms, s));
        }
        {
            Phase ph(it, VX_PROF_APPLY);
            VX_CUDA(launch_apply_levels(it->dev, a, it->num_sms, s));
        }
        {
            Phase ph(it, VX_PROF_RELEASE);
            VX_CUDA(launch_release(it->dev, a.release_list, it->frontier, it->frontier + it->capacity, it->capacity,
                                   rounds, it->num_sms, s));
        }
    }
    return VX_OK;
}

int run_apply(vx_interner *it, std::vector<Item> items, uint8_t *changed_out) {
    const uint32_t n = (uint32_t)items.size();
    if (n == 0) return VX_OK;
    std::stable_sort(items.begin(), items.end(),
                     [&](const Item &a, const Item &b) { return it->tree_depth[a.tree] > it->tree_depth[b.tree]; });
    int max_depth = 0;
    std::vector<uint64_t> off(n + 1, 0);  // first record of each item
    for (uint32_t i = 0; i < n; ++i) {
        const Item &x = items[i];
        max_depth = std::max(max_depth, (int)it->tree_depth[x.tree]);
        off[i + 1] = off[i] + (x.batch->has_patches ? batch_touched_count(x.batch) : 0);
    }
    const uint64_t R = off[n];
    for (auto &x : items)
        if (x.batch->has_patches && it->tree_depth[x.tree] < 2)
            return set_err(it, VX_E_REF_PANIC, "batch apply needs max_depth >= 2 (usize underflow in the reference)");
    if (R >= 0xFFFFFFF0ull) return set_err(it, VX_E_UNSUPPORTED, "too many touched groups in one call");

    // host staging in pinned memory: items, then the touched groups of every batch as records sorted
    // by (item, group). Several threads fill them in record groups; each group's records go to the
    // device (on the interner's stream) while the threads fill the next one. The record -> item index
    // is expanded on the device from the items' first records.
    VX_CUDA(it->pinned.reserve(Carve::need({n * 4, n * 4, n, n, (n + 1) * 4, R * 4, R, R, R * 16})));
    Carve hc(it->pinned.p);
    uint32_t *it_tree = hc.take<uint32_t>(n), *it_fill = hc.take<uint32_t>(n);
    uint8_t *it_depth = hc.take<uint8_t>(n), *it_flags = hc.take<uint8_t>(n);
    uint32_t *it_off = hc.take<uint32_t>(n + 1);
    uint32_t *rec_group = hc.take<uint32_t>(R);
    uint8_t *rec_set = hc.take<uint8_t>(R), *rec_clear = hc.take<uint8_t>(R);
    uint16_t *rec_vals = hc.take<uint16_t>(R * 8);
    for (uint32_t i = 0; i < n; ++i) {
        const vx_batch *b = items[i].batch;
        it_tree[i] = items[i].tree;
        it_depth[i] = it->tree_depth[items[i].tree];
        it_flags[i] = (b->has_fill ? 1 : 0) | (b->has_patches ? 2 : 0);
        it_fill[i] = b->fill;
    }
    for (uint32_t i = 0; i <= n; ++i) it_off[i] = (uint32_t)off[i];
    auto fill_items = [&](uint32_t i0, uint32_t i1) {
        bool cs = false;
        for (uint32_t i = i0; i < i1; ++i) {
            const vx_batch *b = items[i].batch;
            if (!b->has_patches) continue;
            uint64_t r = off[i];
            const bool wide = b->vbits != 8;
            batch_for_each_touched(b, [&](uint64_t g) {
                rec_group[r] = (uint32_t)g;
                rec_set[r] = b->set[g];
                rec_clear[r] = b->clear[g];
                cs |= b->clear[g] != 0;
                if (wide) {
                    std::memcpy(rec_vals + 8 * r, b->vals.data() + 16 * g, 16);
                } else {
                    for (int k = 0; k < 8; ++k) rec_vals[8 * r + k] = b->vals[8 * g + k];
                }
                ++r;
            });
        }
        return cs;
    };
    // first item whose records start at or after record r
    auto item_at = [&](uint64_t r) { return (uint32_t)(std::lower_bound(off.begin(), off.end() - 1, r) - off.begin()); };
    unsigned nt = std::thread::hardware_concurrency();
    nt = std::max(1u, std::min(nt, 16u));
#ifndef VX_STAGE_GROUPS
#define VX_STAGE_GROUPS 4
#endif
    const unsigned K = R >= (1u << 20) ? VX_STAGE_GROUPS : 1;  // record groups: the copy of one overlaps the fill of the next
    if (R < (1u << 16)) nt = 1;
    // small tasks (item ranges of about R / (16 nt) records) taken from a counter in group order, so a
    // thread the OS deschedules delays one task, not a fixed share of every group
    std::vector<uint32_t> task_lo, task_hi;
    std::vector<unsigned> task_group;
    std::vector<uint32_t> gb(K + 1, n);
    gb[0] = 0;
    for (unsigned c = 1; c < K; ++c) gb[c] = item_at(R * c / K);
    const unsigned per_group = std::max(1u, 16 * nt / K);
    for (unsigned c = 0; c < K; ++c) {
        const uint64_t r0 = off[gb[c]], r1 = off[gb[c + 1]];
        uint32_t lo = gb[c];
        for (unsigned k = 1; k <= per_group; ++k) {
            const uint32_t hi = k == per_group ? gb[c + 1] : std::min(gb[c + 1], item_at(r0 + (r1 - r0) * k / per_group));
            if (hi > lo) {
                task_lo.push_back(lo);
                task_hi.push_back(hi);
                task_group.push_back(c);
                lo = hi;
            }
        }
    }
    const uint32_t n_tasks = (uint32_t)task_lo.size();
    std::vector<std::atomic<unsigned>> left(K);
    for (auto &x : left) x.store(0);
    for (uint32_t t = 0; t < n_tasks; ++t) left[task_group[t]].fetch_add(1);
    std::atomic<uint32_t> next_task{0};
    std::vector<char> clears(nt, 0);
    auto run_tasks = [&](const std::function<void()> &after_task) {
        bool cs = false;
        for (;;) {
            const uint32_t t = next_task.fetch_add(1, std::memory_order_relaxed);
            if (t >= n_tasks) break;
            cs |= fill_items(task_lo[t], task_hi[t]);
            left[task_group[t]].fetch_sub(1, std::memory_order_release);
            if (after_task) after_task();
        }
        return cs;
    };

    ApplyArgs a{};
    int st0 = carve_apply(it, n, R, true, a);
    if (st0 != VX_OK) return st0;
    a.max_depth = max_depth;
    cudaStream_t s = it->stream;
    VX_CUDA(cudaMemcpyAsync((void *)a.it_tree, it_tree, n * 4, cudaMemcpyHostToDevice, s));
    VX_CUDA(cudaMemcpyAsync((void *)a.it_depth, it_depth, n, cudaMemcpyHostToDevice, s));
    VX_CUDA(cudaMemcpyAsync((void *)a.it_flags, it_flags, n, cudaMemcpyHostToDevice, s));
    VX_CUDA(cudaMemcpyAsync((void *)a.it_fill, it_fill, n * 4, cudaMemcpyHostToDevice, s));
    if (R) {
        VX_CUDA(cudaMemcpyAsync(a.it_first, it_off, (n + 1) * 4, cudaMemcpyHostToDevice, s));
        VX_CUDA(launch_expand_items(a.it_first, n, (uint32_t *)a.rec_item, s));
    }
    std::vector<std::thread> pool;
    for (unsigned t = 1; t < nt; ++t) pool.emplace_back([&, t] { clears[t] = run_tasks(nullptr); });
    // this thread fills tasks too, and queues each record group's copies once its tasks are done
    cudaError_t copy_err = cudaSuccess;
    unsigned copied = 0;
    auto copy_ready = [&] {
        while (copied < K && left[copied].load(std::memory_order_acquire) == 0) {
            const uint64_t r0 = off[gb[copied]], r1 = off[gb[copied + 1]];
            ++copied;
            if (r1 == r0 || copy_err != cudaSuccess) continue;
            const uint64_t m = r1 - r0;
            cudaError_t e = cudaMemcpyAsync((void *)(a.rec_group + r0), rec_group + r0, m * 4, cudaMemcpyHostToDevice, s);
            if (e == cudaSuccess) e = cudaMemcpyAsync((void *)(a.rec_set + r0), rec_set + r0, m, cudaMemcpyHostToDevice, s);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync((void *)(a.rec_clear + r0), rec_clear + r0, m, cudaMemcpyHostToDevice, s);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync((void *)(a.rec_vals + 8 * r0), rec_vals + 8 * r0, m * 16, cudaMemcpyHostToDevice, s);
            copy_err = e;
        }
    };
    clears[0] = run_tasks(copy_ready);
    while (copied < K) {
        copy_ready();
        if (copied < K) std::this_thread::yield();
    }
    for (auto &th : pool) th.join();
    if (copy_err != cudaSuccess) return cuda_fail(it, copy_err, "record copy");
    bool any_clear = false;
    for (char c : clears) any_clear |= c != 0;
    int st1 = apply_sequence(it, a, any_clear && (it->flags & VX_PATCH_P4));
    if (st1 != VX_OK) return st1;
    std::vector<uint8_t> ch(n);
    VX_CUDA(cudaMemcpyAsync(ch.data(), a.it_changed, n, cudaMemcpyDeviceToHost, s));
    int st = sync_and_check(it);
    for (uint32_t i = 0; i < n; ++i) {
        if (changed_out) changed_out[items[i].caller_index] = ch[i];
        if (ch[i]) it->tree_maybe_nonempty[items[i].tree] = 1;
    }
    if (st == VX_OK) maybe_rehash(it);
    return st;
}

// Batch filled from a dense [y][z][x] grid by just_set (batch.rs:145-172), in y, z, x order.
void batch_from_dense(vx_batch *b, const void *grid) {
    b->all_touched = true;  // every group is written
    b->touched.clear();
    b->touched_sorted = true;
    const int32_t n = 1 << b->depth;
    const int vb = b->vbits / 8;
    const uint8_t *g8 = static_cast<const uint8_t *>(grid);
    const uint16_t *g16 = static_cast<const uint16_t *>(grid);
    for (int32_t y = 0; y < n; ++y)
        for (int32_t z = 0; z < n; ++z)
            for (int32_t x = 0; x < n; ++x) {
                const size_t o = ((size_t)y * n + z) * n + x;
                const uint32_t v = vb == 1 ? g8[o] : g16[o];
                const uint32_t full = morton_encode(x, y, z);
                const uint64_t gi = full >> 3;
                const unsigned idx = full & 7;
                const uint8_t bit = (uint8_t)(1u << idx);
                if (v) {
                    b->set[gi] |= bit;
                    b->clear[gi] &= (uint8_t)~bit;
                } else {
                    b->set[gi] &= (uint8_t)~bit;
                    b->clear[gi] |= bit;
                }
                if (vb == 1)
                    b->vals[8 * gi + idx] = (uint8_t)v;
                else
                    reinterpret_cast<uint16_t *>(b->vals.data())[8 * gi + idx] = (uint16_t)v;
                b->has_patches = true;
            }
}

// Fused dense construction on EMPTY trees (vx_build.cu). All arguments in device memory.
int dense_fast(vx_interner *it, uint32_t n, const uint32_t *d_trees, const void *d_grids, uint8_t *d_changed,
               int depth) {
    cudaStream_t s = it->stream;
    if (depth >= 5) {  // quad kernel, then one pass per level
        const size_t sb = (dense_split_scratch_bytes(n, depth) + 255) & ~(size_t)255;
        VX_CUDA(it->ws.reserve(sb + dense_octant_memo_bytes(n, depth, it->vbits, it->dev.memo_shift)));
        PhaseSwitch ps(it, VX_PROF_DENSE, VX_PROF_LEVELS);
        // one piece: its creators count references (no in-degree pass over the allocation log)
        VX_CUDA(launch_dense_split(it->dev, d_grids, d_trees, n, depth, d_changed, it->ws.p, it->num_sms, s,
                                   static_cast<char *>(it->ws.p) + sb, true, 0, &PhaseSwitch::next, &ps, true));
    } else if (depth == 4) {  // one warp per chunk
        const size_t sb = (dense_octant_scratch_bytes(n, depth) + 255) & ~(size_t)255;
        VX_CUDA(it->ws.reserve(sb + dense_octant_memo_bytes(n, depth, it->vbits, it->dev.memo_shift)));
        Phase ph(it, VX_PROF_DENSE);
        VX_CUDA(launch_dense_octants(it->dev, d_grids, d_trees, n, depth, d_changed, it->ws.p, it->num_sms, s,
                                     static_cast<char *>(it->ws.p) + sb));
    } else {
        DenseArgs a{};
        a.grids = d_grids;
        a.trees = d_trees;
        a.n_chunks = n;
        a.depth = depth;
        a.changed = d_changed;
        Phase ph(it, VX_PROF_DENSE);
        VX_CUDA(launch_dense_blocks(it->dev, a, it->num_sms, s));
    }
    if (depth >= 5 && dense_split_counts_refs(it->dev)) return VX_OK;  // counted and closed by the build
    Phase ph(it, VX_PROF_REFCOUNT);
    VX_CUDA(launch_epoch_refcounts(it->dev, it->num_sms, s));
    return VX_OK;
}

}  // namespace

namespace vxg {
// The device view, stream and SM count of an interner, for entry points compiled in other
// translation units. When `marks_trees` is set, every tree of the interner counts as possibly
// non-empty afterwards (the caller names trees by device handles the host does not inspect).
bool interner_parts(vx_interner *it, DevInterner *dev, cudaStream_t *stream, int *num_sms, uint32_t *flags,
                    bool marks_trees) {
    if (!it) return false;
    *dev = it->dev;
    *stream = it->stream;
    *num_sms = it->num_sms;
    *flags = it->flags;
    if (marks_trees) it->all_trees_unknown = true;
    return true;
}
void interner_set_error(vx_interner *it, const char *msg) {
    if (it) it->last_error = msg;
}
// Releases (dec_ref_recursive) the ids in list_dev, as many as the release slot counts, in `rounds`
// breadth-first rounds, on the interner's stream.
int interner_release_list(vx_interner *it, uint64_t *list_dev, int rounds) {
    Phase ph(it, VX_PROF_RELEASE);
    VX_CUDA(launch_release(it->dev, list_dev, it->frontier, it->frontier + it->capacity, it->capacity, rounds,
                           it->num_sms, it->stream));
    return VX_OK;
}
}  // namespace vxg

extern "C" {

// ---- interner ---------------------------------------------------------------------------------
int vx_interner_create(uint64_t budget_bytes, int voxel_bits, uint32_t patch_flags, int table_log2,
                       vx_interner **out) {
    if (!out || (voxel_bits != 8 && voxel_bits != 16) || table_log2 < 0 || table_log2 > 34)
        return VX_E_INVALID_ARG;
    *out = nullptr;
    vx_interner *it = new (std::nothrow) vx_interner();
    if (!it) return VX_E_OOM;
    it->vbits = voxel_bits;
    it->flags = patch_flags;
    it->node_size = 4 + 2 + 64 + (uint64_t)voxel_bits / 8 + 8;  // interner/mod.rs:158-164
    const uint64_t cap = budget_bytes / it->node_size;
    if (cap == 0) {
        delete it;
        return VX_E_REF_PANIC;  // "Requested budget is too small" (interner/mod.rs:68)
    }
    if (cap > 0xFFFFFFF0ull) {
        delete it;
        return VX_E_INVALID_ARG;  // "Requested budget is too large" (interner/mod.rs:70-73)
    }
    it->capacity = cap;
    uint64_t slots = 1024;
    if (table_log2 > 0)
        slots = 1ull << table_log2;
    else
        while (slots < 2 * cap) slots <<= 1;
    it->table_slots = slots;
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&it->num_sms, cudaDevAttrMultiProcessorCount, dev);
    cudaError_t e = cudaStreamCreateWithFlags(&it->own_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete it;
        return VX_E_CUDA;
    }
    it->stream = it->own_stream;
    DevInterner &D = it->dev;
    D.capacity = (uint32_t)cap;
    D.vbits = voxel_bits;
    D.flags = patch_flags;
    D.table_mask = slots - 1;
    D.max_probes = (uint32_t)std::min<uint64_t>(slots, 1u << 16);
    D.round_limit = ROUND_LIMIT;
    D.spin_limit = SPIN_LIMIT;
    D.memo_shift = 2;
    const size_t vb = voxel_bits / 8;
    bool ok = true;
    auto alloc = [&](void **p, size_t bytes) {
        if (!ok) return;
        if (cudaMalloc(p, std::max<size_t>(bytes, 256)) != cudaSuccess) ok = false;
    };
    alloc((void **)&D.children, cap * 64);
    alloc(&D.values, cap * vb);
    alloc((void **)&D.refcount, cap * 4);
    alloc((void **)&D.generation, cap * 2);
    alloc((void **)&D.hash, cap * 8);
    alloc((void **)&D.ids, cap * 8);
    alloc((void **)&D.free_list, cap * 4);
    alloc((void **)&D.ctr, sizeof(DevCounters));
    alloc((void **)&D.table, slots * 8);
    alloc((void **)&D.leaf_table, ((size_t)1 << voxel_bits) * 8);
    alloc((void **)&it->frontier, 2 * cap * 4 + 64);
    alloc((void **)&it->d_live, 2 * sizeof(unsigned long long));
    alloc((void **)&it->d_status, sizeof(int) * 4);
    alloc((void **)&it->scan_status, (size_t)kScanStatusTiles * 8);
    if (ok && cudaMemset(it->scan_status, 0, (size_t)kScanStatusTiles * 8) != cudaSuccess) ok = false;
    if (patch_flags & VX_PATCH_P3) {
        it->seq_queue_cap = std::max<uint64_t>(cap + 1, 32768);
        alloc((void **)&it->seq_queue, it->seq_queue_cap * 8);
    } else {
        it->seq_queue_cap = 32768;  // PREALLOCATED_STACK_SIZE (interner/consts.rs:15)
        alloc((void **)&it->seq_queue, it->seq_queue_cap * 8);
    }
    if (ok && cudaMallocHost((void **)&it->h_ctr, sizeof(DevCounters)) != cudaSuccess) ok = false;
    if (ok && cudaMallocHost((void **)&it->h_status, sizeof(int) * 4) != cudaSuccess) ok = false;
    if (ok && cudaMallocHost((void **)&it->h_live, 2 * sizeof(unsigned long long)) != cudaSuccess) ok = false;
    if (!ok || grow_tree_table(it, 1024) != cudaSuccess) {
        vx_interner_destroy(it);
        return VX_E_OOM;
    }
    cudaStream_t s = it->stream;
    cudaMemsetAsync(D.children, 0, cap * 64, s);
    cudaMemsetAsync(D.values, 0, cap * vb, s);
    cudaMemsetAsync(D.refcount, 0, cap * 4, s);
    cudaMemsetAsync(D.generation, 0, cap * 2, s);
    cudaMemsetAsync(D.hash, 0, cap * 8, s);
    cudaMemsetAsync(D.ids, 0, cap * 8, s);
    cudaMemsetAsync(D.table, 0xFF, slots * 8, s);
    cudaMemsetAsync(D.leaf_table, 0, ((size_t)1 << voxel_bits) * 8, s);
    DevCounters c0{};
    c0.next_index = 1;  // slot 0 is the EMPTY branch (interner/mod.rs:80-97)
    *it->h_ctr = c0;
    cudaMemcpyAsync(D.ctr, it->h_ctr, sizeof(DevCounters), cudaMemcpyHostToDevice, s);
    e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        vx_interner_destroy(it);
        return VX_E_CUDA;
    }
    *out = it;
    return VX_OK;
}

int vx_interner_destroy(vx_interner *it) {
    if (!it) return VX_E_INVALID_ARG;
    if (it->stream) cudaStreamSynchronize(it->stream);
    DevInterner &D = it->dev;
    void *ptrs[] = {D.children, D.values, D.refcount, D.generation, D.hash, D.ids, D.free_list, D.ctr, D.table,
                    D.leaf_table, D.roots, D.depths, it->frontier, it->seq_queue, it->d_live, it->d_status,
                    it->scan_status};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    it->ws.release();
    it->staging.release();
    it->pinned.release();
    if (it->h_ctr) cudaFreeHost(it->h_ctr);
    if (it->h_status) cudaFreeHost(it->h_status);
    if (it->h_live) cudaFreeHost(it->h_live);
    for (auto &m : it->marks) {
        cudaEventDestroy(m.second.first);
        cudaEventDestroy(m.second.second);
    }
    for (cudaEvent_t e : it->event_pool) cudaEventDestroy(e);
    for (cudaEvent_t e : it->copy_events)
        if (e) cudaEventDestroy(e);
    if (it->copy_stream) cudaStreamDestroy(it->copy_stream);
    if (it->own_stream) cudaStreamDestroy(it->own_stream);
    delete it;
    return VX_OK;
}

int vx_profile_enable(vx_interner *it, int on) {
    if (!it) return VX_E_INVALID_ARG;
    it->profile = on != 0;
    return VX_OK;
}

int vx_profile_collect(vx_interner *it, double *ms, uint64_t *count) {
    if (!it) return VX_E_INVALID_ARG;
    VX_CUDA(cudaStreamSynchronize(it->stream));
    for (int k = 0; k < VX_PROF_N; ++k) {
        if (ms) ms[k] = 0.0;
        if (count) count[k] = 0;
    }
    for (auto &m : it->marks) {
        float t = 0.f;
        cudaEventElapsedTime(&t, m.second.first, m.second.second);
        if (ms) ms[m.first] += t;
        if (count) count[m.first] += 1;
        it->event_pool.push_back(m.second.first);
        it->event_pool.push_back(m.second.second);
    }
    it->marks.clear();
    return VX_OK;
}

uint64_t vx_kernel_launches(void) { return vxg::g_launches.load(); }

int vx_interner_reset(vx_interner *it) {
    if (!it) return VX_E_INVALID_ARG;
    cudaStream_t s = it->stream;
    VX_CUDA(cudaStreamSynchronize(s));
    VX_CUDA(cudaMemsetAsync(it->dev.table, 0xFF, it->table_slots * 8, s));
    VX_CUDA(cudaMemsetAsync(it->dev.leaf_table, 0, ((size_t)1 << it->vbits) * 8, s));
    VX_CUDA(cudaMemsetAsync(it->dev.roots, 0, (size_t)it->tree_cap * 8, s));
    VX_CUDA(cudaMemsetAsync(it->dev.ids, 0, it->capacity * 8, s));
    VX_CUDA(cudaMemsetAsync(it->dev.refcount, 0, it->capacity * 4, s));
    // the rest of the node records as vx_interner_create leaves them: recycled slots carry bumped
    // generations (which become part of new BlockIds) and old records
    VX_CUDA(cudaMemsetAsync(it->dev.generation, 0, it->capacity * 2, s));
    VX_CUDA(cudaMemsetAsync(it->dev.children, 0, it->capacity * 64, s));
    VX_CUDA(cudaMemsetAsync(it->dev.values, 0, it->capacity * (it->vbits / 8), s));
    VX_CUDA(cudaMemsetAsync(it->dev.hash, 0, it->capacity * 8, s));
    DevCounters c0{};
    c0.next_index = 1;
    *it->h_ctr = c0;
    VX_CUDA(cudaMemcpyAsync(it->dev.ctr, it->h_ctr, sizeof(DevCounters), cudaMemcpyHostToDevice, s));
    VX_CUDA(cudaStreamSynchronize(s));
    std::fill(it->tree_maybe_nonempty.begin(), it->tree_maybe_nonempty.end(), 0);
    it->all_trees_unknown = false;
    return VX_OK;
}

int vx_interner_set_limits(vx_interner *it, uint32_t max_probes, uint32_t round_limit, uint32_t spin_limit) {
    if (!it || max_probes == 0) return VX_E_INVALID_ARG;
    VX_CUDA(cudaStreamSynchronize(it->stream));  // kernels already queued keep the limits they were given
    it->dev.max_probes = (uint32_t)std::min<uint64_t>(max_probes, it->table_slots);
    it->dev.round_limit = round_limit;
    it->dev.spin_limit = spin_limit;
    return VX_OK;
}

int vx_interner_get_limits(vx_interner *it, uint32_t *max_probes, uint32_t *round_limit, uint32_t *spin_limit) {
    if (!it || !max_probes || !round_limit || !spin_limit) return VX_E_INVALID_ARG;
    *max_probes = it->dev.max_probes;
    *round_limit = it->dev.round_limit;
    *spin_limit = it->dev.spin_limit;
    return VX_OK;
}

int vx_interner_set_stream(vx_interner *it, void *cuda_stream) {
    if (!it) return VX_E_INVALID_ARG;
    VX_CUDA(cudaStreamSynchronize(it->stream));
    it->stream = cuda_stream ? (cudaStream_t)cuda_stream : it->own_stream;
    return VX_OK;
}

int vx_interner_sync(vx_interner *it) {
    if (!it) return VX_E_INVALID_ARG;
    return sync_and_check(it);
}

int vx_interner_maintain(vx_interner *it) {
    if (!it) return VX_E_INVALID_ARG;
    int st = sync_and_check(it);
    if (st == VX_OK) maybe_rehash(it);
    return st;
}

int vx_interner_stats_get(vx_interner *it, vx_interner_stats *out) {
    if (!it || !out) return VX_E_INVALID_ARG;
    VX_CUDA(launch_count_live(it->dev, it->d_live, it->num_sms, it->stream));
    VX_CUDA(cudaMemcpyAsync(it->h_live, it->d_live, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, it->stream));
    int st = sync_and_check(it);
    *out = vx_interner_stats{};
    out->capacity = it->capacity;
    out->node_size = it->node_size;
    out->next_index = it->h_ctr->next_index;
    out->free_count = it->h_ctr->free_count;
    out->alive_nodes = out->next_index - out->free_count;
    out->branch_patterns = it->h_live[0] + 1;  // the EMPTY branch is a pattern in the reference
    out->leaf_patterns = it->h_live[1];
    out->table_slots = it->table_slots;
    out->table_tombstones = it->h_ctr->tombstones;
    out->error_flags = it->h_ctr->error;
    out->nodes_created = it->h_ctr->created;
    return st == VX_E_OOB || st == VX_E_REF_PANIC ? VX_OK : st;
}

const char *vx_last_error(vx_interner *it) { return it ? it->last_error.c_str() : "null interner"; }

int vx_get_ref(vx_interner *it, uint64_t block_id, uint32_t *out) {
    if (!it || !out) return VX_E_INVALID_ARG;
    const uint32_t idx = id_index(block_id);
    if (idx >= it->capacity) return VX_E_INVALID_ARG;
    uint16_t gen = 0;
    VX_CUDA(cudaMemcpyAsync(&gen, it->dev.generation + idx, 2, cudaMemcpyDeviceToHost, it->stream));
    VX_CUDA(cudaMemcpyAsync(out, it->dev.refcount + idx, 4, cudaMemcpyDeviceToHost, it->stream));
    VX_CUDA(cudaStreamSynchronize(it->stream));
    if (gen != id_generation(block_id)) return set_err(it, VX_E_INVALID_ARG, "stale block id");
    return VX_OK;
}

int vx_get_value(vx_interner *it, uint64_t block_id, uint32_t *out) {
    if (!it || !out) return VX_E_INVALID_ARG;
    const uint32_t idx = id_index(block_id);
    if (idx >= it->capacity) return VX_E_INVALID_ARG;
    uint16_t gen = 0;
    uint16_t v = 0;
    VX_CUDA(cudaMemcpyAsync(&gen, it->dev.generation + idx, 2, cudaMemcpyDeviceToHost, it->stream));
    VX_CUDA(cudaMemcpyAsync(&v, (char *)it->dev.values + idx * (it->vbits / 8), it->vbits / 8,
                            cudaMemcpyDeviceToHost, it->stream));
    VX_CUDA(cudaStreamSynchronize(it->stream));
    if (gen != id_generation(block_id)) return set_err(it, VX_E_INVALID_ARG, "stale block id");
    *out = it->vbits == 8 ? (v & 0xFF) : v;
    return VX_OK;
}

// ---- trees -----------------------------------------------------------------------------------
int vx_trees_create(vx_interner *it, uint32_t n, const uint8_t *depths, vx_tree *out) {
    if (!it || (!out && n)) return VX_E_INVALID_ARG;
    for (uint32_t i = 0; i < n; ++i)
        if ((int)depths[i] >= depth_limit(it->flags))
            return set_err(it, VX_E_DEPTH, "Max depth exceeds allowed limit");
    std::vector<vx_tree> slots(n);
    uint32_t fresh_needed = 0;
    size_t reuse = std::min<size_t>(n, it->free_trees.size());
    fresh_needed = n - (uint32_t)reuse;
    VX_CUDA(grow_tree_table(it, it->tree_count + fresh_needed));
    for (uint32_t i = 0; i < n; ++i) {
        vx_tree t;
        if (i < reuse) {
            t = it->free_trees.back();
            it->free_trees.pop_back();
        } else {
            t = it->tree_count++;
        }
        slots[i] = t;
        it->tree_used[t] = 1;
        it->tree_depth[t] = depths[i];
        it->tree_maybe_nonempty[t] = 0;
    }
    // upload the depth and EMPTY root of every new handle
    uint32_t lo = 0xFFFFFFFFu, hi = 0;
    for (vx_tree t : slots) {
        lo = std::min(lo, t);
        hi = std::max(hi, t);
    }
    if (n) {
        std::vector<uint64_t> roots(hi - lo + 1);
        VX_CUDA(cudaMemcpyAsync(roots.data(), it->dev.roots + lo, roots.size() * 8, cudaMemcpyDeviceToHost, it->stream));
        VX_CUDA(cudaStreamSynchronize(it->stream));
        for (vx_tree t : slots) roots[t - lo] = 0;
        VX_CUDA(cudaMemcpyAsync(it->dev.roots + lo, roots.data(), roots.size() * 8, cudaMemcpyHostToDevice, it->stream));
        VX_CUDA(cudaMemcpyAsync(it->dev.depths + lo, it->tree_depth.data() + lo, hi - lo + 1, cudaMemcpyHostToDevice,
                                it->stream));
        VX_CUDA(cudaStreamSynchronize(it->stream));
    }
    for (uint32_t i = 0; i < n; ++i) out[i] = slots[i];
    return VX_OK;
}

int vx_tree_create(vx_interner *it, int max_depth, vx_tree *out) {
    if (!it || !out) return VX_E_INVALID_ARG;
    if (max_depth < 0 || max_depth >= depth_limit(it->flags))
        return set_err(it, VX_E_DEPTH, "Max depth exceeds allowed limit");
    uint8_t d = (uint8_t)max_depth;
    return vx_trees_create(it, 1, &d, out);
}

int vx_tree_fill(vx_interner *it, vx_tree tree, uint32_t value) {
    if (!it || !tree_ok(it, tree) || !value_fits(it, value)) return VX_E_INVALID_ARG;
    VX_CUDA(launch_tree_fill(it->dev, tree, value, it->seq_queue, it->seq_queue_cap, it->d_status, it->stream));
    VX_CUDA(cudaMemcpyAsync(it->h_status, it->d_status, sizeof(int), cudaMemcpyDeviceToHost, it->stream));
    int st = sync_and_check(it);
    it->tree_maybe_nonempty[tree] = value != 0;
    if (st == VX_OK) maybe_rehash(it);
    return st;
}

int vx_tree_clear(vx_interner *it, vx_tree tree) { return vx_tree_fill(it, tree, 0); }

int vx_tree_destroy(vx_interner *it, vx_tree tree) {
    if (!it || !tree_ok(it, tree)) return VX_E_INVALID_ARG;
    int st = vx_tree_clear(it, tree);
    it->tree_used[tree] = 0;
    it->tree_depth[tree] = kUnused;
    const uint8_t u = kUnused;
    cudaMemcpyAsync(it->dev.depths + tree, &u, 1, cudaMemcpyHostToDevice, it->stream);
    cudaStreamSynchronize(it->stream);
    it->free_trees.push_back(tree);
    return st;
}

int vx_tree_root(vx_interner *it, vx_tree tree, uint64_t *out_root) {
    if (!it || !out_root || !tree_ok(it, tree)) return VX_E_INVALID_ARG;
    return read_root(it, tree, out_root);
}

int vx_tree_max_depth(vx_interner *it, vx_tree tree, int *out) {
    if (!it || !out || !tree_ok(it, tree)) return VX_E_INVALID_ARG;
    *out = it->tree_depth[tree];
    return VX_OK;
}

int vx_tree_set(vx_interner *it, vx_tree tree, int32_t x, int32_t y, int32_t z, uint32_t value, int *changed) {
    if (!it || !tree_ok(it, tree) || !value_fits(it, value)) return VX_E_INVALID_ARG;
    const int32_t side = 1 << it->tree_depth[tree];
    if (x < 0 || y < 0 || z < 0 || x >= side || y >= side || z >= side)
        return set_err(it, VX_E_OOB, "position out of bounds");
    VX_CUDA(launch_tree_set(it->dev, tree, x, y, z, value, it->seq_queue, it->seq_queue_cap, it->d_status, it->stream));
    VX_CUDA(cudaMemcpyAsync(it->h_status, it->d_status, sizeof(int), cudaMemcpyDeviceToHost, it->stream));
    int st = sync_and_check(it);
    if (changed) *changed = *it->h_status == 1;
    if (*it->h_status == 1) it->tree_maybe_nonempty[tree] = 1;
    if (st == VX_OK) maybe_rehash(it);
    return st;
}

int vx_tree_get(vx_interner *it, vx_tree tree, int32_t x, int32_t y, int32_t z, int *found, uint32_t *value) {
    if (!it || !found || !value || !tree_ok(it, tree)) return VX_E_INVALID_ARG;
    const int32_t side = 1 << it->tree_depth[tree];
    if (x < 0 || y < 0 || z < 0 || x >= side || y >= side || z >= side)
        return set_err(it, VX_E_OOB, "position out of bounds");
    int32_t xyz[3] = {x, y, z};
    uint8_t f = 0;
    uint16_t v = 0;
    int st = vx_get_many(it, 1, &tree, xyz, &f, &v, VX_MEM_HOST);
    *found = f;
    *value = f ? (it->vbits == 8 ? (v & 0xFF) : v) : 0;
    return st;
}

// ---- batches ---------------------------------------------------------------------------------
int vx_batch_create(int max_depth, int voxel_bits, uint32_t patch_flags, vx_batch **out) {
    if (!out || (voxel_bits != 8 && voxel_bits != 16)) return VX_E_INVALID_ARG;
    if (max_depth < 0 || max_depth >= depth_limit(patch_flags)) return VX_E_DEPTH;
    vx_batch *b = new (std::nothrow) vx_batch();
    if (!b) return VX_E_OOM;
    b->depth = max_depth;
    b->vbits = voxel_bits;
    b->flags = patch_flags;
    const int lower = max_depth > 0 ? max_depth - 1 : 0;
    b->groups = 1ull << (3 * lower);
    try {
        b->set.assign(b->groups, 0);
        b->clear.assign(b->groups, 0);
        b->vals.assign(b->groups * 8 * (voxel_bits / 8), 0);
    } catch (const std::bad_alloc &) {
        delete b;
        return VX_E_OOM;
    }
    *out = b;
    return VX_OK;
}

int vx_batch_destroy(vx_batch *b) {
    delete b;
    return VX_OK;
}

int vx_batch_set(vx_batch *b, int32_t x, int32_t y, int32_t z, uint32_t value) {
    if (!b) return VX_E_INVALID_ARG;
    if (value > (b->vbits == 8 ? 0xFFu : 0xFFFFu)) return VX_E_INVALID_ARG;
    const int32_t n = 1 << b->depth;
    if (x < 0 || y < 0 || z < 0 || x >= n || y >= n || z >= n) return VX_E_OOB;
    const uint32_t full = morton_encode(x, y, z);
    const uint64_t gi = full >> 3;
    const unsigned idx = full & 7;
    const uint8_t bit = (uint8_t)(1u << idx);
    batch_touch(b, gi);
    if (value) {
        b->set[gi] |= bit;
        b->clear[gi] &= (uint8_t)~bit;
    } else {
        b->set[gi] &= (uint8_t)~bit;
        b->clear[gi] |= bit;
    }
    if (b->vbits == 8)
        b->vals[8 * gi + idx] = (uint8_t)value;
    else
        reinterpret_cast<uint16_t *>(b->vals.data())[8 * gi + idx] = (uint16_t)value;
    b->has_patches = true;
    return VX_OK;
}

int vx_batch_set_many(vx_batch *b, uint64_t n, const int32_t *xyz, const uint32_t *values) {
    if (!b || (n && (!xyz || !values))) return VX_E_INVALID_ARG;
    for (uint64_t i = 0; i < n; ++i) {
        const int st = vx_batch_set(b, xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], values[i]);
        if (st != VX_OK) return st;
    }
    return VX_OK;
}

int vx_batch_clear(vx_batch *b) {
    if (!b) return VX_E_INVALID_ARG;
    if (b->all_touched) {
        std::fill(b->set.begin(), b->set.end(), 0);
        std::fill(b->clear.begin(), b->clear.end(), 0);
        std::fill(b->vals.begin(), b->vals.end(), 0);
    } else {
        const size_t vb = b->vbits / 8;
        for (uint32_t g : b->touched) {
            b->set[g] = 0;
            b->clear[g] = 0;
            std::memset(b->vals.data() + (size_t)g * 8 * vb, 0, 8 * vb);
        }
    }
    b->touched.clear();
    b->touched_sorted = true;
    b->all_touched = false;
    b->has_fill = false;
    b->fill = 0;
    b->has_patches = false;
    return VX_OK;
}

int vx_batch_fill(vx_batch *b, uint32_t value) {
    if (!b || value > (b->vbits == 8 ? 0xFFu : 0xFFFFu)) return VX_E_INVALID_ARG;
    vx_batch_clear(b);
    b->has_fill = true;
    b->fill = value;
    return VX_OK;
}

int vx_batch_set_dense(vx_batch *b, const void *grid) {
    if (!b || !grid) return VX_E_INVALID_ARG;
    batch_from_dense(b, grid);
    return VX_OK;
}

int vx_batch_size(const vx_batch *b, uint64_t *out) {
    if (!b || !out) return VX_E_INVALID_ARG;
    *out = batch_touched_count(b);
    return VX_OK;
}

int vx_batch_has_patches(const vx_batch *b, int *out) {
    if (!b || !out) return VX_E_INVALID_ARG;
    *out = b->has_patches ? 1 : 0;
    return VX_OK;
}

// ---- the hot path -----------------------------------------------------------------------------
int vx_apply_batches(vx_interner *it, uint32_t n, const vx_tree *trees, const vx_batch *const *batches,
                     uint8_t *changed) {
    if (!it || (n && (!trees || !batches))) return VX_E_INVALID_ARG;
    std::vector<Item> items(n);
    std::unordered_set<vx_tree> seen;
    for (uint32_t i = 0; i < n; ++i) {
        if (!tree_ok(it, trees[i]) || !batches[i]) return set_err(it, VX_E_INVALID_ARG, "unknown tree or batch");
        if (batches[i]->vbits != it->vbits) return set_err(it, VX_E_INVALID_ARG, "batch voxel width differs");
        if (batches[i]->depth != it->tree_depth[trees[i]])
            return set_err(it, VX_E_REF_PANIC, "batch depth differs from the tree depth");
        if (!seen.insert(trees[i]).second) return set_err(it, VX_E_INVALID_ARG, "a tree appears twice in one call");
        items[i] = Item{trees[i], batches[i], i};
    }
    return run_apply(it, std::move(items), changed);
}

int vx_apply_batch(vx_interner *it, vx_tree tree, const vx_batch *batch, int *changed) {
    uint8_t c = 0;
    int st = vx_apply_batches(it, 1, &tree, &batch, &c);
    if (changed) *changed = c;
    return st;
}

int vx_apply_groups_async(vx_interner *it, uint32_t n_items, const vx_tree *trees_dev, const uint8_t *item_flags_dev,
                          const uint32_t *fill_dev, uint32_t n_records, const uint32_t *rec_item_dev,
                          const uint32_t *rec_group_dev, const uint8_t *rec_set_dev, const uint8_t *rec_clear_dev,
                          const uint16_t *rec_values_dev, uint8_t *changed_dev, int max_depth) {
    if (!it || (n_items && (!trees_dev || !item_flags_dev || !fill_dev)) ||
        (n_records && (!rec_item_dev || !rec_group_dev || !rec_set_dev || !rec_clear_dev || !rec_values_dev)))
        return VX_E_INVALID_ARG;
    if (max_depth < 2 || max_depth >= depth_limit(it->flags)) return set_err(it, VX_E_DEPTH, "unsupported max_depth");
    it->all_trees_unknown = true;
    if (n_items == 0) return VX_OK;
    ApplyArgs a{};
    int st = carve_apply(it, n_items, n_records, false, a);
    if (st != VX_OK) return st;
    a.it_tree = trees_dev;
    a.it_flags = item_flags_dev;
    a.it_fill = fill_dev;
    a.rec_item = rec_item_dev;
    a.rec_group = rec_group_dev;
    a.rec_set = rec_set_dev;
    a.rec_clear = rec_clear_dev;
    a.rec_vals = rec_values_dev;
    a.max_depth = max_depth;
    st = apply_sequence(it, a, (it->flags & VX_PATCH_P4) != 0, true);
    if (st != VX_OK) return st;
    if (changed_dev) VX_CUDA(cudaMemcpyAsync(changed_dev, a.it_changed, n_items, cudaMemcpyDeviceToDevice, it->stream));
    return VX_OK;
}

int vx_trees_set_many(vx_interner *it, uint64_t n, const vx_tree *trees, const int32_t *xyz, const uint32_t *values,
                      uint8_t *changed) {
    if (!it || (n && (!trees || !xyz || !values))) return VX_E_INVALID_ARG;
    if (n == 0) return VX_OK;
    if (n >= 0xFFFFFFFFull) return set_err(it, VX_E_UNSUPPORTED, "2^32 calls or more in one call");
    int dmax = 0;
    for (uint64_t k = 0; k < n; ++k) {  // every call is checked before any runs
        const vx_tree t = trees[k];
        if (!tree_ok(it, t) || !value_fits(it, values[k])) return set_err(it, VX_E_INVALID_ARG, "bad tree or value");
        const int32_t side = 1 << it->tree_depth[t];
        const int32_t x = xyz[3 * k], y = xyz[3 * k + 1], z = xyz[3 * k + 2];
        if (x < 0 || y < 0 || z < 0 || x >= side || y >= side || z >= side)
            return set_err(it, VX_E_OOB, "position out of bounds");
        dmax = std::max(dmax, (int)it->tree_depth[t]);
    }
    int st = sync_and_check(it);  // also gives the allocation state before the calls
    if (st != VX_OK) return st;
    const unsigned long long fc0 = it->h_ctr->free_count, ni0 = it->h_ctr->next_index;
    // the calls grouped by tree, in call order within a tree
    std::vector<uint32_t> order(n);
    for (uint64_t k = 0; k < n; ++k) order[k] = (uint32_t)k;
    std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return trees[a] < trees[b]; });
    std::vector<uint32_t> group_tree, begin;
    std::vector<int32_t> sx(3 * n);
    std::vector<uint32_t> sv(n);
    for (uint64_t k = 0; k < n; ++k) {
        const uint32_t o = order[k];
        if (k == 0 || trees[o] != trees[order[k - 1]]) {
            group_tree.push_back(trees[o]);
            begin.push_back((uint32_t)k);
        }
        for (int a = 0; a < 3; ++a) sx[3 * k + a] = xyz[3 * (size_t)o + a];
        sv[k] = values[o];
    }
    begin.push_back((uint32_t)n);
    const size_t G = group_tree.size();
    const size_t list_cap = G + (size_t)n * (dmax + 1) + 16;  // old roots + every node the calls can create
    VX_CUDA(it->ws.reserve(Carve::need({G * 4, (G + 1) * 4, n * 12, n * 4, n * 4, n, G * 8, list_cap * 8})));
    Carve c(it->ws.p);
    uint32_t *d_group = c.take<uint32_t>(G);
    uint32_t *d_begin = c.take<uint32_t>(G + 1);
    int32_t *d_xyz = c.take<int32_t>(3 * n);
    uint32_t *d_vals = c.take<uint32_t>(n);
    uint32_t *d_order = c.take<uint32_t>(n);
    uint8_t *d_changed = c.take<uint8_t>(n);
    uint64_t *d_roots = c.take<uint64_t>(G);
    uint64_t *d_list = c.take<uint64_t>(list_cap);
    cudaStream_t s = it->stream;
    VX_CUDA(cudaMemcpyAsync(d_group, group_tree.data(), G * 4, cudaMemcpyHostToDevice, s));
    VX_CUDA(cudaMemcpyAsync(d_begin, begin.data(), (G + 1) * 4, cudaMemcpyHostToDevice, s));
    VX_CUDA(cudaMemcpyAsync(d_xyz, sx.data(), n * 12, cudaMemcpyHostToDevice, s));
    VX_CUDA(cudaMemcpyAsync(d_vals, sv.data(), n * 4, cudaMemcpyHostToDevice, s));
    VX_CUDA(cudaMemcpyAsync(d_order, order.data(), n * 4, cudaMemcpyHostToDevice, s));
    SetCalls calls{(uint32_t)G, d_group, d_begin, d_xyz, d_vals, d_order, d_changed, d_roots};
    {
        Phase ph(it, VX_PROF_APPLY);
        VX_CUDA(launch_trees_set(it->dev, calls, d_list, fc0, ni0, it->frontier, it->frontier + it->capacity, dmax,
                                 it->num_sms, s));
    }
    std::vector<uint8_t> ch(n);
    VX_CUDA(cudaMemcpyAsync(ch.data(), d_changed, n, cudaMemcpyDeviceToHost, s));
    st = sync_and_check(it);
    if (st != VX_OK) return st;
    for (uint64_t k = 0; k < n; ++k) {
        if (changed) changed[k] = ch[k];
        if (ch[k]) it->tree_maybe_nonempty[trees[k]] = 1;
    }
    maybe_rehash(it);
    return VX_OK;
}

int vx_tune_set(vx_interner *it, int apply_threads, int apply_blocks_per_sm) {
    if (!it || apply_threads < 32 || apply_threads > 512 || apply_threads % 32 || apply_blocks_per_sm < 1 ||
        apply_blocks_per_sm > 64)
        return VX_E_INVALID_ARG;
    it->apply_threads = apply_threads;
    it->apply_blocks_per_sm = apply_blocks_per_sm;
    return VX_OK;
}

int vx_tune_get(vx_interner *it, int *apply_threads, int *apply_blocks_per_sm) {
    if (!it || !apply_threads || !apply_blocks_per_sm) return VX_E_INVALID_ARG;
    *apply_threads = it->apply_threads;
    *apply_blocks_per_sm = it->apply_blocks_per_sm;
    return VX_OK;
}

int vx_tune_set_dense(vx_interner *it, int memo_shift) {
    if (!it || memo_shift < 0 || memo_shift > 8) return VX_E_INVALID_ARG;
    VX_CUDA(cudaStreamSynchronize(it->stream));  // queued builds keep the geometry they were given
    it->dev.memo_shift = (uint32_t)memo_shift;
    return VX_OK;
}

int vx_tune_get_dense(vx_interner *it, int *memo_shift) {
    if (!it || !memo_shift) return VX_E_INVALID_ARG;
    *memo_shift = (int)it->dev.memo_shift;
    return VX_OK;
}

int vx_tune_set_launch(vx_interner *it, int single_launch) {
    if (!it || (single_launch != 0 && single_launch != 1)) return VX_E_INVALID_ARG;
    it->apply_single = single_launch;
    return VX_OK;
}

int vx_tune_get_launch(vx_interner *it, int *single_launch) {
    if (!it || !single_launch) return VX_E_INVALID_ARG;
    *single_launch = it->apply_single;
    return VX_OK;
}

int vx_build_dense_async(vx_interner *it, uint32_t n, const vx_tree *trees_dev, const void *grids_dev,
                         uint8_t *changed_dev, int max_depth) {
    if (!it || (n && (!trees_dev || !grids_dev))) return VX_E_INVALID_ARG;
    if (max_depth < 0 || max_depth >= depth_limit(it->flags)) return set_err(it, VX_E_DEPTH, "Max depth exceeds allowed limit");
    if (max_depth < 2) return set_err(it, VX_E_REF_PANIC, "batch apply needs max_depth >= 2 (usize underflow in the reference)");
    if ((uintptr_t)grids_dev % 16) return set_err(it, VX_E_INVALID_ARG, "grids must be 16-byte aligned");
    // the trees are named by device handles the host does not inspect: every tree counts as
    // possibly non-empty until the next reset.
    it->all_trees_unknown = true;
    if (n == 0) return VX_OK;
    return dense_fast(it, n, trees_dev, grids_dev, changed_dev, max_depth);
}

int vx_build_dense(vx_interner *it, uint32_t n, const vx_tree *trees, const void *grids, uint8_t *changed,
                   vx_mem mem) {
    if (!it || (n && (!trees || !grids))) return VX_E_INVALID_ARG;
    if (n == 0) return VX_OK;
    std::vector<vx_tree> htrees(n);
    if (mem == VX_MEM_DEVICE) {
        VX_CUDA(cudaMemcpyAsync(htrees.data(), trees, n * sizeof(vx_tree), cudaMemcpyDeviceToHost, it->stream));
        VX_CUDA(cudaStreamSynchronize(it->stream));
    } else {
        std::copy(trees, trees + n, htrees.begin());
    }
    // duplicate check with a per-interner stamp per tree slot (no allocation per call)
    if (it->tree_stamp.size() < it->tree_depth.size()) it->tree_stamp.assign(it->tree_depth.size(), 0);
    if (++it->stamp_epoch == 0) {
        std::fill(it->tree_stamp.begin(), it->tree_stamp.end(), 0u);
        it->stamp_epoch = 1;
    }
    int d = -1;
    bool fresh = !it->all_trees_unknown;
    for (vx_tree t : htrees) {
        if (!tree_ok(it, t)) return set_err(it, VX_E_INVALID_ARG, "unknown tree handle");
        if (it->tree_stamp[t] == it->stamp_epoch) return set_err(it, VX_E_INVALID_ARG, "a tree appears twice in one call");
        it->tree_stamp[t] = it->stamp_epoch;
        if (d >= 0 && it->tree_depth[t] != d) return set_err(it, VX_E_INVALID_ARG, "trees of one call share a depth");
        d = it->tree_depth[t];
        fresh = fresh && !it->tree_maybe_nonempty[t];
    }
    if (d < 2) return set_err(it, VX_E_REF_PANIC, "batch apply needs max_depth >= 2 (usize underflow in the reference)");
    const size_t vb = it->vbits / 8;
    const size_t per = ((size_t)1 << (3 * d)) * vb;
    if (!fresh) {
        // general path: Batch per grid, then the batched apply
        std::vector<uint8_t> hgrids;
        const uint8_t *g = static_cast<const uint8_t *>(grids);
        if (mem == VX_MEM_DEVICE) {
            hgrids.resize(per * n);
            VX_CUDA(cudaMemcpy(hgrids.data(), grids, per * n, cudaMemcpyDeviceToHost));
            g = hgrids.data();
        }
        std::vector<vx_batch *> bs(n, nullptr);
        int st = VX_OK;
        for (uint32_t i = 0; i < n && st == VX_OK; ++i) {
            st = vx_batch_create(d, it->vbits, it->flags, &bs[i]);
            if (st == VX_OK) batch_from_dense(bs[i], g + per * i);
        }
        std::vector<uint8_t> ch(n);
        if (st == VX_OK) st = vx_apply_batches(it, n, htrees.data(), bs.data(), ch.data());
        for (auto *b : bs) vx_batch_destroy(b);
        if (changed) {
            if (mem == VX_MEM_DEVICE)
                cudaMemcpy(changed, ch.data(), n, cudaMemcpyHostToDevice);
            else
                std::copy(ch.begin(), ch.end(), changed);
        }
        return st;
    }
    if (mem == VX_MEM_HOST && d >= 4 && n >= 2 * kCopyPieces) {
        // pipelined: the grids go over in kCopyPieces pieces on a copy stream; piece k is built on
        // the interner's stream as soon as its copy lands, while piece k+1 is still in flight
        if (!it->copy_stream) {
            VX_CUDA(cudaStreamCreateWithFlags(&it->copy_stream, cudaStreamNonBlocking));
            for (auto &e : it->copy_events) VX_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        }
        VX_CUDA(it->staging.reserve(Carve::need({n * 4, per * n, n})));
        Carve c(it->staging.p);
        uint32_t *dt = c.take<uint32_t>(n);
        uint8_t *dg = c.take<uint8_t>(per * n);
        uint8_t *dc = c.take<uint8_t>(n);
        const bool split = d >= 5;
        const size_t sb = ((split ? dense_split_scratch_bytes(n, d) : dense_octant_scratch_bytes(n, d)) + 255) &
                          ~(size_t)255;
        VX_CUDA(it->ws.reserve(sb + dense_octant_memo_bytes(n, d, it->vbits, it->dev.memo_shift)));
        char *memo = static_cast<char *>(it->ws.p) + sb;
        cudaStream_t s = it->stream;
        {
            Phase ph(it, VX_PROF_COPY);
            VX_CUDA(cudaMemcpyAsync(dt, htrees.data(), n * 4, cudaMemcpyHostToDevice, s));
            VX_CUDA(cudaMemsetAsync(dc, 0, n, s));
            // the copy stream must not overwrite grids a previous call's kernels still read
            VX_CUDA(cudaEventRecord(it->copy_events[0], s));
            VX_CUDA(cudaStreamWaitEvent(it->copy_stream, it->copy_events[0], 0));
        }
        int weight_total = 0;
        for (int w : kPieceWeights) weight_total += w;
        bool first = true;  // the first piece clears the quad memo the later ones share
        for (int k = 0, acc = 0; k < kCopyPieces; ++k) {
            const uint32_t c0 = (uint32_t)((uint64_t)n * acc / weight_total);
            acc += kPieceWeights[k];
            const uint32_t c1 = (uint32_t)((uint64_t)n * acc / weight_total);
            if (c0 >= c1) continue;
            VX_CUDA(cudaMemcpyAsync(dg + per * c0, static_cast<const uint8_t *>(grids) + per * c0, per * (c1 - c0),
                                    cudaMemcpyHostToDevice, it->copy_stream));
            VX_CUDA(cudaEventRecord(it->copy_events[k], it->copy_stream));
            VX_CUDA(cudaStreamWaitEvent(s, it->copy_events[k], 0));
            if (split) {
                PhaseSwitch ps(it, VX_PROF_DENSE, VX_PROF_LEVELS);
                VX_CUDA(launch_dense_split(it->dev, dg + per * c0, dt + c0, c1 - c0, d, dc + c0, it->ws.p, it->num_sms,
                                           s, memo, first, n, &PhaseSwitch::next, &ps));
            } else {
                Phase ph(it, VX_PROF_DENSE);
                VX_CUDA(launch_dense_octants(it->dev, dg + per * c0, dt + c0, c1 - c0, d, dc + c0, it->ws.p,
                                             it->num_sms, s, memo, first, n));
            }
            first = false;
        }
        {  // pieces count by one in-degree pass: counting in each piece's kernels measured slower here
            Phase ph(it, VX_PROF_REFCOUNT);
            VX_CUDA(launch_epoch_refcounts(it->dev, it->num_sms, s));
        }
        if (changed) {
            Phase ph(it, VX_PROF_COPY);
            VX_CUDA(cudaMemcpyAsync(changed, dc, n, cudaMemcpyDeviceToHost, s));
        }
        const int st = sync_and_check(it);
        for (vx_tree t : htrees) it->tree_maybe_nonempty[t] = 1;
        return st;
    }
    const uint32_t *d_trees;
    const void *d_grids;
    uint8_t *d_changed;
    if (mem == VX_MEM_HOST) {
        VX_CUDA(it->staging.reserve(Carve::need({n * 4, per * n, n})));
        Carve c(it->staging.p);
        uint32_t *dt = c.take<uint32_t>(n);
        uint8_t *dg = c.take<uint8_t>(per * n);
        uint8_t *dc = c.take<uint8_t>(n);
        Phase ph(it, VX_PROF_COPY);
        VX_CUDA(cudaMemcpyAsync(dt, htrees.data(), n * 4, cudaMemcpyHostToDevice, it->stream));
        VX_CUDA(cudaMemcpyAsync(dg, grids, per * n, cudaMemcpyHostToDevice, it->stream));
        VX_CUDA(cudaMemsetAsync(dc, 0, n, it->stream));
        d_trees = dt;
        d_grids = dg;
        d_changed = dc;
    } else {
        if ((uintptr_t)grids % 16) return set_err(it, VX_E_INVALID_ARG, "grids must be 16-byte aligned");
        d_trees = trees;
        d_grids = grids;
        d_changed = changed;
    }
    int st = dense_fast(it, n, d_trees, d_grids, d_changed, d);
    if (st != VX_OK) return st;
    if (mem == VX_MEM_HOST && changed) {
        Phase ph(it, VX_PROF_COPY);
        VX_CUDA(cudaMemcpyAsync(changed, d_changed, n, cudaMemcpyDeviceToHost, it->stream));
    }
    st = sync_and_check(it);
    for (vx_tree t : htrees) it->tree_maybe_nonempty[t] = 1;
    return st;
}

int vx_get_many_async(vx_interner *it, uint64_t n, const vx_tree *trees_dev, const int32_t *xyz_dev,
                      uint8_t *found_dev, void *values_dev) {
    if (!it || (n && (!trees_dev || !xyz_dev || !found_dev || !values_dev))) return VX_E_INVALID_ARG;
    Phase ph(it, VX_PROF_GET);
    VX_CUDA(launch_get_many(it->dev, n, trees_dev, xyz_dev, found_dev, values_dev, it->num_sms, it->stream));
    return VX_OK;
}

int vx_get_many(vx_interner *it, uint64_t n, const vx_tree *trees, const int32_t *xyz, uint8_t *found, void *values,
                vx_mem mem) {
    if (!it || (n && (!trees || !xyz || !found || !values))) return VX_E_INVALID_ARG;
    if (n == 0) return VX_OK;
    if (mem == VX_MEM_DEVICE) {
        {
            Phase ph(it, VX_PROF_GET);
            VX_CUDA(launch_get_many(it->dev, n, trees, xyz, found, values, it->num_sms, it->stream));
        }
        return sync_and_check(it);
    }
    const size_t vb = it->vbits / 8;
    VX_CUDA(it->staging.reserve(Carve::need({n * 4, n * 12, n, n * vb})));
    Carve c(it->staging.p);
    uint32_t *dt = c.take<uint32_t>(n);
    int32_t *dx = c.take<int32_t>(n * 3);
    uint8_t *df = c.take<uint8_t>(n);
    uint8_t *dv = c.take<uint8_t>(n * vb);
    {
        Phase ph(it, VX_PROF_COPY);
        VX_CUDA(cudaMemcpyAsync(dt, trees, n * 4, cudaMemcpyHostToDevice, it->stream));
        VX_CUDA(cudaMemcpyAsync(dx, xyz, n * 12, cudaMemcpyHostToDevice, it->stream));
    }
    {
        Phase ph(it, VX_PROF_GET);
        VX_CUDA(launch_get_many(it->dev, n, dt, dx, df, dv, it->num_sms, it->stream));
    }
    {
        Phase ph(it, VX_PROF_COPY);
        VX_CUDA(cudaMemcpyAsync(found, df, n, cudaMemcpyDeviceToHost, it->stream));
        VX_CUDA(cudaMemcpyAsync(values, dv, n * vb, cudaMemcpyDeviceToHost, it->stream));
    }
    return sync_and_check(it);
}

// ---- verification helpers ----------------------------------------------------------------------
int vx_export_canonical(vx_interner *it, uint32_t n_trees, const vx_tree *trees, vx_canonical *out,
                        uint64_t *n_nodes) {
    if (!it || !n_nodes || (n_trees && !trees)) return VX_E_INVALID_ARG;
    Snapshot s;
    int st = take_snapshot(it, s);
    if (st != VX_OK) return st;
    std::vector<uint64_t> roots;
    st = read_roots(it, n_trees, trees, roots);
    if (st != VX_OK) return st;
    std::vector<int32_t> ids(s.n, -1);  // node index -> canonical id
    std::vector<uint64_t> order, stack;
    std::vector<int32_t> croots(n_trees, -1);
    for (uint32_t t = 0; t < n_trees; ++t) {
        const uint64_t r = roots[t];
        if (r == 0) continue;
        stack.push_back(r);
        while (!stack.empty()) {
            const uint64_t nd = stack.back();
            stack.pop_back();
            const uint32_t idx = id_index(nd);
            if (idx >= s.n) return set_err(it, VX_E_REF_UB, "child index outside the node store");
            if (ids[idx] >= 0) continue;
            ids[idx] = (int32_t)order.size();
            order.push_back(nd);
            if (id_is_branch(nd))
                for (int k = 7; k >= 0; --k)
                    if (s.children[8ull * idx + k]) stack.push_back(s.children[8ull * idx + k]);
        }
        croots[t] = ids[id_index(r)];
    }
    *n_nodes = order.size();
    if (!out) return VX_OK;
    if (out->capacity < order.size()) return VX_E_BUFFER;
    for (size_t k = 0; k < order.size(); ++k) {
        const uint64_t nd = order[k];
        const uint32_t idx = id_index(nd);
        const bool leaf = id_is_leaf(nd);
        out->kind[k] = leaf ? 1 : 0;
        out->types[k] = leaf ? 0 : (uint8_t)id_types(nd);
        out->mask[k] = leaf ? 0 : (uint8_t)id_mask(nd);
        out->value[k] = s.values[idx];
        out->refcount[k] = s.refcount[idx];
        for (int j = 0; j < 8; ++j) {
            int32_t c = -1;
            if (!leaf) {
                const uint64_t cid = s.children[8ull * idx + j];
                if (cid) c = ids[id_index(cid)];
            }
            out->children[k * 8 + j] = c;
        }
    }
    if (out->roots)
        for (uint32_t t = 0; t < n_trees; ++t) out->roots[t] = croots[t];
    return VX_OK;
}

int vx_validate(vx_interner *it, uint32_t n_trees, const vx_tree *trees) {
    if (!it || (n_trees && !trees)) return VX_E_INVALID_ARG;
    Snapshot s;
    int st = take_snapshot(it, s);
    if (st != VX_OK) return st;
    std::vector<uint64_t> roots;
    st = read_roots(it, n_trees, trees, roots);
    if (st != VX_OK) return st;
    std::vector<uint8_t> seen(s.n, 0);
    std::vector<uint64_t> stack;
    for (uint64_t r : roots) {
        if (r == 0) continue;
        stack.push_back(r);
        while (!stack.empty()) {
            const uint64_t nd = stack.back();
            stack.pop_back();
            const uint32_t idx = id_index(nd);
            if (idx >= s.n) return set_err(it, VX_E_REF_UB, "child index outside the node store");
            if (s.generation[idx] != id_generation(nd) || s.ids[idx] != nd)
                return set_err(it, VX_E_REF_UB, "dangling child: generation mismatch");
            if (s.refcount[idx] == 0) return set_err(it, VX_E_REF_UB, "reachable node with zero refcount");
            if (seen[idx]) continue;
            seen[idx] = 1;
            if (id_is_branch(nd))
                for (int k = 0; k < 8; ++k)
                    if (s.children[8ull * idx + k]) stack.push_back(s.children[8ull * idx + k]);
        }
    }
    return VX_OK;
}

int vx_trees_to_dense_async(vx_interner *it, uint32_t n, const vx_tree *trees_dev, int depth, void *out_dev) {
    if (!it || depth < 1 || depth > 10 || (n && (!trees_dev || !out_dev))) return VX_E_INVALID_ARG;
    if (reinterpret_cast<uintptr_t>(out_dev) % 16) return set_err(it, VX_E_INVALID_ARG, "out_dev must be 16-byte aligned");
    if (n == 0) return VX_OK;
    const int lc = depth < 5 ? depth : 5;
    const uint64_t cubes = (uint64_t)n << (3 * (depth - lc));
    Phase ph(it, VX_PROF_GET);
    VX_CUDA(launch_to_dense(it->dev, trees_dev, depth, 0, cubes, out_dev, it->num_sms, it->stream));
    return VX_OK;
}

int vx_trees_to_dense(vx_interner *it, uint32_t n, const vx_tree *trees, void *out, vx_mem mem) {
    if (!it || (n && (!trees || !out))) return VX_E_INVALID_ARG;
    if (n == 0) return VX_OK;
    const int d = tree_ok(it, trees[0]) ? (int)it->tree_depth[trees[0]] : -1;
    for (uint32_t k = 0; k < n; ++k)
        if (!tree_ok(it, trees[k]) || it->tree_depth[trees[k]] != d) return VX_E_INVALID_ARG;
    if (d < 1) return VX_E_INVALID_ARG;
    const size_t vb = it->vbits / 8;
    const int lc = d < 5 ? d : 5;
    const uint64_t K = 1ull << (d - lc), S = 1ull << d;
    const uint64_t slab_bytes = (S * S << lc) * vb;  // one cy-slab: K^2 cubes
    const uint64_t n_slabs = (uint64_t)n * K;
    if (mem == VX_MEM_DEVICE) {
        if (reinterpret_cast<uintptr_t>(out) % 16) return set_err(it, VX_E_INVALID_ARG, "out must be 16-byte aligned");
        VX_CUDA(it->staging.reserve(Carve::need({(size_t)n * 4})));
        uint32_t *dt = static_cast<uint32_t *>(it->staging.p);
        VX_CUDA(cudaMemcpyAsync(dt, trees, (size_t)n * 4, cudaMemcpyHostToDevice, it->stream));
        {
            Phase ph(it, VX_PROF_GET);
            VX_CUDA(launch_to_dense(it->dev, dt, d, 0, n_slabs * K * K, out, it->num_sms, it->stream));
        }
        return sync_and_check(it);
    }
    // host output: whole cy-slabs through a device buffer of at most ~256 MiB per piece
    const uint64_t piece_slabs = std::max<uint64_t>(1, ((uint64_t)256 << 20) / slab_bytes);
    const uint64_t piece = std::min(piece_slabs, n_slabs);
    VX_CUDA(it->staging.reserve(Carve::need({(size_t)n * 4, (size_t)(piece * slab_bytes)})));
    Carve c(it->staging.p);
    uint32_t *dt = c.take<uint32_t>(n);
    uint8_t *dg = c.take<uint8_t>(piece * slab_bytes);
    VX_CUDA(cudaMemcpyAsync(dt, trees, (size_t)n * 4, cudaMemcpyHostToDevice, it->stream));
    for (uint64_t s0 = 0; s0 < n_slabs; s0 += piece) {
        const uint64_t ns = std::min(piece, n_slabs - s0);
        {
            Phase ph(it, VX_PROF_GET);
            VX_CUDA(launch_to_dense(it->dev, dt, d, s0 * K * K, ns * K * K, dg, it->num_sms, it->stream));
        }
        {
            Phase ph(it, VX_PROF_COPY);
            VX_CUDA(cudaMemcpyAsync(static_cast<uint8_t *>(out) + s0 * slab_bytes, dg, ns * slab_bytes,
                                    cudaMemcpyDeviceToHost, it->stream));
        }
    }
    return sync_and_check(it);
}

int vx_occupancy_masks(vx_interner *it, uint32_t n_trees, const vx_tree *trees, const uint32_t *offsets,
                       uint64_t *global, uint64_t *active, uint32_t max_materials, uint32_t *n_materials,
                       uint32_t *material_ids, uint64_t *material_counts, uint64_t *material_masks) {
    if (!it || !n_trees || !trees || !offsets || !global || !active || !n_materials ||
        (max_materials && (!material_ids || !material_counts || !material_masks)))
        return VX_E_INVALID_ARG;
    const int d = tree_ok(it, trees[0]) ? (int)it->tree_depth[trees[0]] : -1;
    if (d < 1 || d > 6) return set_err(it, VX_E_INVALID_ARG, "occupancy masks need trees of MaxDepth 1..6");
    const uint32_t S = 1u << d;
    for (uint32_t k = 0; k < n_trees; ++k) {
        if (!tree_ok(it, trees[k]) || it->tree_depth[trees[k]] != d)
            return set_err(it, VX_E_INVALID_ARG, "trees of one builder share a MaxDepth");
        for (int a = 0; a < 3; ++a)
            if (offsets[3 * k + a] > 64 - S) return set_err(it, VX_E_OOB, "tree outside the 64^3 builder");
    }
    const size_t vb = it->vbits / 8;
    const uint32_t n_values = 1u << it->vbits;
    const size_t per = (size_t)S * S * S * vb;
    const size_t plane = 3 * 4096;
    VX_CUDA(it->staging.reserve(Carve::need({(size_t)n_trees * 4, (size_t)n_trees * 12, per * n_trees,
                                             (size_t)n_values * 8, (size_t)n_values * 4, (size_t)n_values * 4,
                                             (size_t)n_values * 8, 64, plane * 8, 64,
                                             (size_t)max_materials * plane * 8})));
    Carve c(it->staging.p);
    uint32_t *dt = c.take<uint32_t>(n_trees);
    uint32_t *doff = c.take<uint32_t>((size_t)n_trees * 3);
    uint8_t *dg = c.take<uint8_t>(per * n_trees);
    unsigned long long *counts = c.take<unsigned long long>(n_values);
    uint32_t *slot = c.take<uint32_t>(n_values);
    uint32_t *ids = c.take<uint32_t>(n_values);
    unsigned long long *mcounts = c.take<unsigned long long>(n_values);
    uint32_t *nm = c.take<uint32_t>(16);
    unsigned long long *dglobal = c.take<unsigned long long>(plane);
    unsigned long long *dactive = c.take<unsigned long long>(8);
    unsigned long long *dmat = c.take<unsigned long long>((size_t)max_materials * plane);
    cudaStream_t s = it->stream;
    VX_CUDA(cudaMemcpyAsync(dt, trees, (size_t)n_trees * 4, cudaMemcpyHostToDevice, s));
    VX_CUDA(cudaMemcpyAsync(doff, offsets, (size_t)n_trees * 12, cudaMemcpyHostToDevice, s));
    VX_CUDA(cudaMemsetAsync(counts, 0, (size_t)n_values * 8, s));
    VX_CUDA(cudaMemsetAsync(dglobal, 0, plane * 8, s));
    if (max_materials) VX_CUDA(cudaMemsetAsync(dmat, 0, (size_t)max_materials * plane * 8, s));
    {
        Phase ph(it, VX_PROF_GET);
        const int lc = d < 5 ? d : 5;
        VX_CUDA(launch_to_dense(it->dev, dt, d, 0, (uint64_t)n_trees << (3 * (d - lc)), dg, it->num_sms, s));
        VX_CUDA(launch_occupancy(it->dev, dg, n_trees, d, doff, counts, slot, ids, mcounts, nm, max_materials,
                                 dglobal, dmat, dactive, it->num_sms, s));
    }
    uint32_t n_mat = 0;
    VX_CUDA(cudaMemcpyAsync(&n_mat, nm, 4, cudaMemcpyDeviceToHost, s));
    VX_CUDA(cudaMemcpyAsync(global, dglobal, plane * 8, cudaMemcpyDeviceToHost, s));
    VX_CUDA(cudaMemcpyAsync(active, dactive, 48, cudaMemcpyDeviceToHost, s));
    int st = sync_and_check(it);
    if (st != VX_OK) return st;
    *n_materials = n_mat;
    const uint32_t k = std::min(n_mat, max_materials);
    if (k) {
        VX_CUDA(cudaMemcpyAsync(material_ids, ids, (size_t)k * 4, cudaMemcpyDeviceToHost, s));
        VX_CUDA(cudaMemcpyAsync(material_counts, mcounts, (size_t)k * 8, cudaMemcpyDeviceToHost, s));
        VX_CUDA(cudaMemcpyAsync(material_masks, dmat, (size_t)k * plane * 8, cudaMemcpyDeviceToHost, s));
        st = sync_and_check(it);
        if (st != VX_OK) return st;
    }
    return n_mat > max_materials ? set_err(it, VX_E_BUFFER, "more materials than max_materials") : VX_OK;
}

int vx_occupancy_masks_async(vx_interner *it, uint32_t n_builders, uint32_t n_trees, const vx_tree *trees_dev,
                             const uint32_t *builder_of_dev, const uint32_t *offsets_dev, int max_depth,
                             uint32_t max_materials, uint64_t *global_dev, uint64_t *active_dev,
                             uint32_t *n_materials_dev, uint32_t *material_ids_dev, uint64_t *material_counts_dev,
                             uint64_t *material_masks_dev) {
    if (!it || !n_builders || !n_trees || !trees_dev || !builder_of_dev || !offsets_dev || !global_dev || !active_dev ||
        !n_materials_dev || (max_materials && (!material_ids_dev || !material_counts_dev || !material_masks_dev)))
        return VX_E_INVALID_ARG;
    if (it->vbits != 8) return set_err(it, VX_E_UNSUPPORTED, "the batched occupancy masks take 8-bit voxels");
    if (max_depth < 1 || max_depth > 6) return set_err(it, VX_E_INVALID_ARG, "occupancy masks need MaxDepth 1..6");
    const size_t per = (size_t)1 << (3 * max_depth);
    const size_t plane = 3 * 4096;
    VX_CUDA(it->ws.reserve(Carve::need({per * n_trees, (size_t)n_builders * 256 * 4, (size_t)n_builders * 256 * 4})));
    Carve c(it->ws.p);
    uint8_t *dg = c.take<uint8_t>(per * n_trees);
    unsigned int *counts = c.take<unsigned int>((size_t)n_builders * 256);
    uint32_t *slot = c.take<uint32_t>((size_t)n_builders * 256);
    cudaStream_t s = it->stream;
    VX_CUDA(cudaMemsetAsync(counts, 0, (size_t)n_builders * 256 * 4, s));
    VX_CUDA(cudaMemsetAsync(global_dev, 0, (size_t)n_builders * plane * 8, s));
    if (max_materials) VX_CUDA(cudaMemsetAsync(material_masks_dev, 0, (size_t)n_builders * max_materials * plane * 8, s));
    Phase ph(it, VX_PROF_GET);
    const int lc = max_depth < 5 ? max_depth : 5;
    VX_CUDA(launch_to_dense(it->dev, trees_dev, max_depth, 0, (uint64_t)n_trees << (3 * (max_depth - lc)), dg,
                            it->num_sms, s));
    VX_CUDA(launch_occupancy_many(it->dev, dg, n_trees, max_depth, builder_of_dev, offsets_dev, n_builders, counts,
                                  slot, max_materials, material_ids_dev,
                                  reinterpret_cast<unsigned long long *>(material_counts_dev), n_materials_dev,
                                  reinterpret_cast<unsigned long long *>(global_dev),
                                  reinterpret_cast<unsigned long long *>(material_masks_dev),
                                  reinterpret_cast<unsigned long long *>(active_dev), it->num_sms, s));
    return VX_OK;
}

int vx_serialize_model(vx_interner *it, uint32_t n_chunks, const vx_tree *trees, const int32_t *positions,
                       uint8_t *out, uint64_t capacity, uint64_t *size) {
    if (!it || !size || (n_chunks && (!trees || !positions))) return VX_E_INVALID_ARG;
    for (uint32_t k = 0; k < n_chunks; ++k)
        if (!tree_ok(it, trees[k])) return set_err(it, VX_E_INVALID_ARG, "unknown tree handle");
    const size_t words = serialize_scratch_words(it->dev);
    const size_t tmpw = scan_tmp_words(it->capacity) * 4;  // the recursive scan's block sums
    VX_CUDA(it->ws.reserve(Carve::need({words * 4, tmpw * 4, (size_t)n_chunks * 4 + 4, (size_t)n_chunks * 12 + 4, 64})));
    Carve c(it->ws.p);
    uint32_t *w = c.take<uint32_t>(words);
    uint32_t *tmp = c.take<uint32_t>(tmpw);
    uint32_t *dt = c.take<uint32_t>((size_t)n_chunks + 1);
    int32_t *dp = c.take<int32_t>((size_t)n_chunks * 3 + 1);
    unsigned long long *dtotal = c.take<unsigned long long>(2);
    cudaStream_t s = it->stream;
    if (n_chunks) {
        VX_CUDA(cudaMemcpyAsync(dt, trees, (size_t)n_chunks * 4, cudaMemcpyHostToDevice, s));
        VX_CUDA(cudaMemcpyAsync(dp, positions, (size_t)n_chunks * 12, cudaMemcpyHostToDevice, s));
    }
    unsigned long long total = 0;
    {
        Phase ph(it, VX_PROF_GET);
        VX_CUDA(launch_serialize_plan(it->dev, w, tmp, n_chunks, dt, dtotal, it->num_sms, s));
    }
    VX_CUDA(cudaMemcpyAsync(&total, dtotal, 8, cudaMemcpyDeviceToHost, s));
    int st = sync_and_check(it);
    if (st != VX_OK) return st;
    *size = total;
    if (!out) return VX_OK;
    if (capacity < total) return set_err(it, VX_E_BUFFER, "output buffer smaller than the serialised model");
    VX_CUDA(it->staging.reserve(total + 256));
    uint8_t *dout = static_cast<uint8_t *>(it->staging.p);
    {
        Phase ph(it, VX_PROF_GET);
        VX_CUDA(launch_serialize_write(it->dev, w, n_chunks, dt, dp, dout, dtotal, it->num_sms, s));
    }
    VX_CUDA(cudaMemcpyAsync(out, dout, total, cudaMemcpyDeviceToHost, s));
    return sync_and_check(it);
}

// VoxModel::deserialize (world/voxmodel.rs:284-408) into an interner without nodes: the stream is
// parsed on the device (launch_vtm_parse); the host reads back the three counts, creates the chunk
// trees and launches the placement of the nodes, refcounts and roots (launch_vtm_place).
int vx_deserialize_model(vx_interner *it, const uint8_t *data, uint64_t n_bytes, int max_depth, uint32_t max_chunks,
                         vx_tree *out_trees, int32_t *out_positions, uint32_t *out_n_chunks) {
    if (!it || !out_n_chunks || (n_bytes && !data)) return VX_E_INVALID_ARG;
    *out_n_chunks = 0;
    if (max_depth < 0 || max_depth >= depth_limit(it->flags))
        return set_err(it, VX_E_DEPTH, "Max depth exceeds allowed limit");
    if (n_bytes < 4) return set_err(it, VX_E_REF_PANIC, "stream too short for its leaf count");
    if (n_bytes >= 0xFFFFFFFFull) return set_err(it, VX_E_UNSUPPORTED, "streams of 4 GiB or more");
    int st = sync_and_check(it);
    if (st != VX_OK) return st;
    const unsigned long long ni = it->h_ctr->next_index, fc = it->h_ctr->free_count;
    const VtmScratchSizes z = vtm_scratch_sizes(n_bytes);
    const uint64_t chunk_room = std::min<uint64_t>(max_chunks, z.chunk_cap);  // a chunk record takes 25+ bytes
    VX_CUDA(it->staging.reserve(n_bytes + 64));
    VX_CUDA(it->ws.reserve(Carve::need({sizeof(VtmSections), z.table_words * 8, z.entry_words * 8, z.leaf_cap * 4,
                                        z.branch_cap * 4, z.chunk_cap * 4, chunk_room * 4 + 4, chunk_room * 12 + 4})));
    Carve c(it->ws.p);
    VtmSections *sec = c.take<VtmSections>(1);
    uint64_t *tables = c.take<uint64_t>(z.table_words);
    uint64_t *entries = c.take<uint64_t>(z.entry_words);
    uint32_t *leaf_off = c.take<uint32_t>(z.leaf_cap);
    uint32_t *branch_off = c.take<uint32_t>(z.branch_cap);
    uint32_t *chunk_off = c.take<uint32_t>(z.chunk_cap);
    uint32_t *d_trees = c.take<uint32_t>(chunk_room + 1);
    int32_t *d_pos = c.take<int32_t>(chunk_room * 3 + 1);
    uint8_t *bytes = static_cast<uint8_t *>(it->staging.p);
    cudaStream_t s = it->stream;
    VtmSections h{};
    h.start[0] = 4;
    h.count[0] = ((uint32_t)data[0] << 24) | ((uint32_t)data[1] << 16) | ((uint32_t)data[2] << 8) | data[3];
    h.start[1] = h.start[2] = h.start[3] = ~0ull;
    VX_CUDA(cudaMemcpyAsync(bytes, data, n_bytes, cudaMemcpyHostToDevice, s));
    VX_CUDA(cudaMemcpyAsync(sec, &h, sizeof(h), cudaMemcpyHostToDevice, s));
    {
        Phase ph(it, VX_PROF_GET);
        VX_CUDA(launch_vtm_parse(it->dev, bytes, n_bytes, sec, tables, entries, leaf_off, branch_off, chunk_off,
                                 it->num_sms, s));
    }
    VX_CUDA(cudaMemcpyAsync(&h, sec, sizeof(h), cudaMemcpyDeviceToHost, s));
    st = sync_and_check(it);
    if (st != VX_OK) return st;
    for (int k = 0; k < 3; ++k)
        if (!h.done[k]) return set_err(it, VX_E_REF_PANIC, "stream ends inside section " + std::to_string(k));
    const uint64_t nodes = h.count[0] + h.count[1], C = h.count[2];
    // deserialize_leaf / preallocate_branch_id assert that each id is the next index allocated
    // (interner/mod.rs:930-968): with nodes in the stream the interner must hold none yet
    if (nodes && (ni != 1 || fc != 0))
        return set_err(it, VX_E_REF_PANIC, "deserialize needs an interner without nodes (Invalid block id)");
    if (nodes + 1 > it->capacity) return set_err(it, VX_E_OOM, "Out of memory: node capacity exhausted");
    *out_n_chunks = (uint32_t)C;
    if (C > max_chunks) return set_err(it, VX_E_BUFFER, "more chunks in the stream than max_chunks");
    if (C && (!out_trees || !out_positions)) return VX_E_INVALID_ARG;
    std::vector<uint8_t> depths(C, (uint8_t)max_depth);
    st = vx_trees_create(it, (uint32_t)C, depths.data(), out_trees);
    if (st != VX_OK) return st;
    if (C) VX_CUDA(cudaMemcpyAsync(d_trees, out_trees, C * 4, cudaMemcpyHostToDevice, s));
    {
        Phase ph(it, VX_PROF_GET);
        VX_CUDA(launch_vtm_place(it->dev, bytes, sec, nodes, h.count[1] + C, leaf_off, branch_off, chunk_off, d_trees,
                                 d_pos, it->num_sms, s));
    }
    if (C) VX_CUDA(cudaMemcpyAsync(out_positions, d_pos, C * 12, cudaMemcpyDeviceToHost, s));
    for (uint64_t k = 0; k < C; ++k) it->tree_maybe_nonempty[out_trees[k]] = 1;
    return sync_and_check(it);
}

int vx_tree_to_dense(vx_interner *it, vx_tree tree, void *out_grid) {
    return vx_trees_to_dense(it, 1, &tree, out_grid, VX_MEM_HOST);
}

}  // extern "C"
