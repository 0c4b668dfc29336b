// Batched VoxTree::apply_batch over many trees sharing one interner, level-synchronous on the GPU.
//
// Restates set_batch_at_depth_iterative (spatial/voxtree.rs:724-1118) for n trees at once:
//   prep     Phase 0 fill (voxtree.rs:742-758): the fill leaf replaces the old root as the
//            starting node; without patches it is the new root.
//   bottom   Phase 1 (voxtree.rs:770-897), one thread per touched bottom group: descend the old
//            tree to depth d-1, collapse a full uniform group to a leaf, otherwise merge the set
//            voxels into the existing children (or into 8 copies of an ancestor leaf) and
//            hash-cons the branch. Groups that change nothing drop out, as in the reference.
//   levels   Phase 2 (voxtree.rs:905-1106), one step per level for all trees together: entries
//            are kept sorted by (tree, path), so the siblings of one parent form a run; run heads
//            are found by comparing sibling prefixes (PATH_MASKS), numbered by a prefix scan,
//            and each parent gathers its run, clones the untouched children of the old parent or
//            replicates an ancestor leaf, collapses 8 equal leaves, and hash-conses the result.
//   finish   apply_batch (voxtree.rs:303-328): commit the new root, queue the old root for
//            release, report assert_ne!(new_root, old_root) as a reference panic.
// Clear pass (P4). The reference ignores Batch clear bits (voxtree.rs:779). With P4 they are
// honoured as VoxTree::set(pos, 0) for every cleared voxel after the set phase (remove_at_depth,
// voxtree.rs:542-706). Those removals commute, so the same level-synchronous machinery applies them
// in one pass (mode 1): a touched group drops its cleared children (or splits an ancestor leaf into
// 8 copies minus the cleared ones), a parent takes the new children over the old node's children
// (or over 8 copies of an ancestor leaf), clears their types bits, drops children that became
// EMPTY from its mask, and becomes EMPTY itself when its mask empties. Nothing collapses. The
// removal path is refcount-exact, so no correction applies.
// Trees are processed deepest first, so the trees whose root is produced at a step are the tail
// of that step's list and the next list is a prefix of the parents.
//
// Refcounts. After the build every count is the in-degree from newly created nodes plus tree roots,
// plus the corrections below. The lane that creates a branch adds its children's references right
// away, from the key it still holds in registers (no re-read of the node): branch children by a
// global reduction, leaf children into a per-CTA table indexed by leaf value that the CTA flushes
// once (leaves are the hot spots: a few values are named by most bottom groups). The last CTA of
// the root-commit kernel closes the allocation epoch. The corrections reproduce where the
// reference's increments differ from the references its nodes hold:
//   Q5 (voxtree.rs:835-839, 846-868): an ancestor leaf is charged 8 - |set| references, but only
//      8 - |modified| slots keep it: + (|modified| - |set|), or + (8 - |set|) when nothing changed.
//   Q6 (voxtree.rs:1062-1072): a collapse with c cloned children gives back min(c, 7) instead of
//      7 - c references: + (7 - 2c).
//   Q7 (voxtree.rs:742-758): the fill leaf's Phase-0 reference is never released when the batch
//      also has patches: + 1.
#include "vx_launch.h"

namespace vxg {
namespace {

constexpr int kThreads = 256;
// minimum resident CTAs of 512 threads the branch-creating kernels are compiled for (2: at most 64
// registers a thread)
#ifndef VX_APPLY_MIN_BLOCKS
#define VX_APPLY_MIN_BLOCKS 2
#endif
constexpr int kScanPer = 8;
constexpr int kScanBlock = kThreads * kScanPer;

__device__ __forceinline__ void add_ref_delta(const DevInterner &I, uint64_t id, int delta) {
    if (delta != 0 && id != EMPTY_ID) atomicAdd(I.refcount + id_index(id), (unsigned)delta);
}

// Per-CTA counts of leaf-child references (dynamic shared memory, leaf_refs_smem bytes). 8-bit
// voxels: one counter per value. 16-bit voxels: kLeafSlots counters direct-mapped by value with the
// owning value as a tag; a value whose slot another value owns goes straight to a global reduction.
constexpr uint32_t kLeafSlots = 4096;
struct LeafRefs {
    uint32_t *cnt;
    uint32_t *tag;  // value + 1 owning the slot, 0 = free (16-bit voxels only)
    uint32_t slots;
    bool direct;
};

__device__ __forceinline__ LeafRefs leaf_refs_init(const DevInterner &I) {
    extern __shared__ uint32_t leaf_smem[];
    LeafRefs L;
    L.direct = I.vbits == 8;
    L.slots = L.direct ? 256u : kLeafSlots;
    L.cnt = leaf_smem;
    L.tag = leaf_smem + L.slots;
    for (uint32_t k = threadIdx.x; k < (L.direct ? L.slots : 2 * L.slots); k += blockDim.x) leaf_smem[k] = 0;
    __syncthreads();
    return L;
}

__device__ __forceinline__ void leaf_ref_add(const DevInterner &I, const LeafRefs &L, uint64_t leaf, uint32_t value,
                                             uint32_t n) {
    if (L.direct) {
        atomicAdd(L.cnt + value, n);
        return;
    }
    const uint32_t s = value & (kLeafSlots - 1u), key = value + 1u;
    uint32_t t = L.tag[s];
    if (t == 0) {
        t = atomicCAS(L.tag + s, 0u, key);
        if (t == 0) t = key;
    }
    if (t == key)
        atomicAdd(L.cnt + s, n);
    else
        atomicAdd(I.refcount + id_index(leaf), n);
}

// One reference per child slot of a node this lane just created (equal children summed first).
__device__ __forceinline__ void add_child_refs(const DevInterner &I, const LeafRefs &L, const uint64_t c[8],
                                               const uint32_t cv[8]) {
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        if (c[k] == EMPTY_ID) continue;
        bool seen = false;
        uint32_t n = 1;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            if (j < k && c[j] == c[k]) seen = true;
            if (j > k && c[j] == c[k]) ++n;
        }
        if (seen) continue;
        if (id_is_leaf(c[k]))
            leaf_ref_add(I, L, c[k], cv[k], n);
        else
            atomicAdd(I.refcount + id_index(c[k]), n);
    }
}

// Adds the CTA's leaf counts to the leaves' global counts (every thread of the CTA calls it).
__device__ __forceinline__ void leaf_refs_flush(const DevInterner &I, const LeafRefs &L) {
    __syncthreads();
    for (uint32_t s = threadIdx.x; s < L.slots; s += blockDim.x) {
        const uint32_t n = L.cnt[s];
        if (n == 0) continue;
        const uint32_t v = L.direct ? s : L.tag[s] - 1u;
        const uint64_t lid = I.leaf_table[v];
        if (lid > LEAF_BUSY)
            atomicAdd(I.refcount + id_index(lid), n);
        else
            set_error(I, ERR_INTERNAL, 47);
    }
}

__device__ __forceinline__ void prep_item(const DevInterner &I, const ApplyArgs &a, int mode, uint32_t i) {
    const uint32_t t = a.it_tree[i];
    const uint64_t old = I.roots[t];
    const uint8_t f = a.it_flags[i];
    uint64_t init = old;
    a.it_old[i] = old;
    if (mode == 1) {  // the clear pass starts from the root the set phase left
        a.it_init[i] = old;
        a.it_new[i] = INVALID_ID;
        return;
    }
    a.it_panic[i] = 0;
    if (f & 1) {
        bool created;
        const uint64_t fill = intern_leaf(I, a.it_fill[i], &created);
        init = fill;
        if (f & 2) add_ref_delta(I, fill, 1);  // Q7
    }
    a.it_init[i] = init;
    a.it_new[i] = (f & 2) ? INVALID_ID : init;
}

__global__ void prep_items_kernel(DevInterner I, ApplyArgs a) {
    pdl_wait();
    pdl_release();
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < a.n_items) prep_item(I, a, a.mode, i);
}

// Phase 1 for records cta_base + threadIdx.x, + stride, ... (a CTA-uniform loop: whole warps take
// part in the warp-cooperative interning).
__device__ __forceinline__ void bottom_range(const DevInterner &I, const ApplyArgs &a, int mode, const LeafRefs &L,
                                             uint64_t cta_base, uint64_t stride) {
    for (uint64_t base = cta_base; base < a.n_records; base += stride) {
        const uint64_t r = base + threadIdx.x;
        bool active = r < a.n_records;
        uint32_t i = 0, set = 0, changed = 0;
        int d = 0;
        uint64_t cur = EMPTY_ID, anc = EMPTY_ID, out = EMPTY_ID;
        uint32_t v[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        uint64_t c[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        uint32_t cv[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        uint32_t types = 0, mask = 0, lod = 0;
        bool want_branch = false;
        if (active) {
            i = a.rec_item[r];
            d = a.it_depth[i];
            set = mode ? a.rec_clear[r] : a.rec_set[r];
            if (set == 0 || a.it_panic[i]) active = false;
        }
        bool uniform = false;
        if (active) {
            const uint32_t path = a.rec_group[r] << 3;
#pragma unroll
            for (int k = 0; k < 8; ++k) v[k] = a.rec_vals[8 * r + k];
            // descend to depth d-1 (voxtree.rs:792-822)
            cur = a.it_init[i];
            for (int cd = 0; cd < d - 1; ++cd) {
                if (id_is_branch(cur)) {
                    const uint32_t idx = (path >> (3 * (d - cd - 1))) & 7u;
                    cur = I.children[8ull * id_index(cur) + idx];
                } else {
                    anc = cur;
                    cur = EMPTY_ID;
                }
                if (cur == EMPTY_ID) break;
            }
            uniform = set == 0xFF;
#pragma unroll
            for (int k = 1; k < 8; ++k) uniform = uniform && v[k] == v[0];
            if (cur != EMPTY_ID && id_is_leaf(cur)) {
                if ((I.flags & 1u) || mode == 1) {  // P1 (removals always split a leaf)
                    anc = cur;
                    cur = EMPTY_ID;
                } else if (!uniform) {  // the reference panics in BlockId::types()
                    a.it_panic[i] = 1;
                    set_error(I, ERR_REF_PANIC, 40);
                    active = false;
                }
            }
        }
        if (active && mode == 1) {  // remove_at_depth_branch / _leaf at depth d-1
            uint32_t modified = 0;
            if (cur != EMPTY_ID) {
                const uint64_t *src = I.children + 8ull * id_index(cur);
#pragma unroll
                for (int k = 0; k < 8; ++k) {
                    c[k] = src[k];
                    cv[k] = c[k] ? node_value(I, id_index(c[k])) : 0;
                }
                types = id_types(cur);
                mask = id_mask(cur);
                modified = set & mask;
            } else if (anc != EMPTY_ID) {
                const uint32_t av = node_value(I, id_index(anc));
#pragma unroll
                for (int k = 0; k < 8; ++k) {
                    c[k] = anc;
                    cv[k] = av;
                }
                types = mask = 0xFF;
                modified = set;
            }
            if (modified) {
#pragma unroll
                for (int k = 0; k < 8; ++k)
                    if ((modified >> k) & 1) {
                        c[k] = EMPTY_ID;
                        cv[k] = 0;
                    }
                types &= ~modified;
                mask &= ~modified;
                changed = 1;
                if (mask) {
                    want_branch = true;
                    lod = calc_average8(cv);
                }
            }
        } else if (active && uniform) {  // voxtree.rs:826, 887-896
            bool created;
            out = intern_leaf(I, v[0], &created);
            lod = v[0];
            changed = 1;
        } else if (active) {  // voxtree.rs:829-883
            if (cur != EMPTY_ID) {
                const uint64_t *src = I.children + 8ull * id_index(cur);
#pragma unroll
                for (int k = 0; k < 8; ++k) {
                    c[k] = src[k];
                    cv[k] = c[k] ? node_value(I, id_index(c[k])) : 0;
                }
                types = id_types(cur);
                mask = id_mask(cur);
            } else if (anc != EMPTY_ID) {
                const uint32_t av = node_value(I, id_index(anc));
#pragma unroll
                for (int k = 0; k < 8; ++k) {
                    c[k] = anc;
                    cv[k] = av;
                }
                types = mask = 0xFF;
            }
            // the set voxels whose value differs from the existing leaf become new leaves: their
            // leaf-table slots are read together (one round trip for all of them); only a leaf not
            // created yet takes the claiming path
            uint32_t modified = 0;
#pragma unroll
            for (int k = 0; k < 8; ++k)
                if (((set >> k) & 1) && !(c[k] != EMPTY_ID && cv[k] == v[k])) modified |= 1u << k;
#pragma unroll
            for (int k = 0; k < 8; ++k)
                if ((modified >> k) & 1) c[k] = ld_cg(I.leaf_table + v[k]);
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                if (!((modified >> k) & 1)) continue;
                if (c[k] <= LEAF_BUSY) {
                    bool created;
                    c[k] = intern_leaf(I, v[k], &created);
                }
                cv[k] = v[k];
            }
            types |= modified;
            mask |= modified;
            if (anc != EMPTY_ID && cur == EMPTY_ID) {  // Q5
                const int ds = __popc(set), dm = __popc(modified);
                add_ref_delta(I, anc, modified ? dm - ds : 8 - ds);
            }
            if (modified) {
                want_branch = true;
                lod = calc_average8(cv);
                changed = 1;
            }
        }
        bool created;
        const uint64_t id = warp_intern_branch_inl(I, want_branch, c, types, mask, lod, &created);
        if (created) add_child_refs(I, L, c, cv);
        if (want_branch) out = id;
        if (r < a.n_records) {
            a.flags[r] = changed;
            a.rec_id[r] = out;
            a.rec_val[r] = lod;
        }
    }
}

__global__ void __launch_bounds__(512, VX_APPLY_MIN_BLOCKS) bottom_kernel(DevInterner I, ApplyArgs a) {
    pdl_wait();
    pdl_release();
    const LeafRefs L = leaf_refs_init(I);
    bottom_range(I, a, a.mode, L, (uint64_t)blockIdx.x * blockDim.x, (uint64_t)gridDim.x * blockDim.x);
    leaf_refs_flush(I, L);
}

// Exclusive scan of n flags: per-block scan, scan of block sums, add-back. pos[n] = total.
__global__ void __launch_bounds__(kThreads) scan_blocks_kernel(const uint32_t *in, uint32_t *out, uint32_t *sums,
                                                              uint32_t n) {
    pdl_wait();
    pdl_release();
    __shared__ uint32_t warp_tot[kThreads / 32];
    const uint32_t base = blockIdx.x * kScanBlock + threadIdx.x * kScanPer;
    uint32_t x[kScanPer];
    uint32_t local = 0;
#pragma unroll
    for (int k = 0; k < kScanPer; ++k) {
        x[k] = (base + k < n) ? in[base + k] : 0u;
        local += x[k];
    }
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    uint32_t incl = local;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if (lane >= (unsigned)o) incl += y;
    }
    if (lane == 31) warp_tot[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < kThreads / 32 ? warp_tot[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xFFFFFFFFu, w, o);
            if (lane >= (unsigned)o) w += y;
        }
        if (lane < kThreads / 32) warp_tot[lane] = w;
    }
    __syncthreads();
    uint32_t run = incl - local + (warp ? warp_tot[warp - 1] : 0);
#pragma unroll
    for (int k = 0; k < kScanPer; ++k) {
        if (base + k < n) out[base + k] = run;
        run += x[k];
    }
    if (threadIdx.x == kThreads - 1) sums[blockIdx.x] = warp_tot[kThreads / 32 - 1];
}

// Variants reading the element count from device memory (entries of a level pass); blocks past the
// count only record an empty block sum.
__global__ void __launch_bounds__(kThreads) scan_blocks_dev_kernel(const uint32_t *in, uint32_t *out, uint32_t *sums,
                                                                  const unsigned long long *n_dev) {
    pdl_wait();
    pdl_release();
    const uint32_t n = (uint32_t)*n_dev;
    if (blockIdx.x * kScanBlock >= n) {
        if (threadIdx.x == 0) sums[blockIdx.x] = 0;
        return;
    }
    __shared__ uint32_t warp_tot[kThreads / 32];
    const uint32_t base = blockIdx.x * kScanBlock + threadIdx.x * kScanPer;
    uint32_t x[kScanPer];
    uint32_t local = 0;
#pragma unroll
    for (int k = 0; k < kScanPer; ++k) {
        x[k] = (base + k < n) ? in[base + k] : 0u;
        local += x[k];
    }
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    uint32_t incl = local;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if (lane >= (unsigned)o) incl += y;
    }
    if (lane == 31) warp_tot[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < kThreads / 32 ? warp_tot[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xFFFFFFFFu, w, o);
            if (lane >= (unsigned)o) w += y;
        }
        if (lane < kThreads / 32) warp_tot[lane] = w;
    }
    __syncthreads();
    uint32_t run = incl - local + (warp ? warp_tot[warp - 1] : 0);
#pragma unroll
    for (int k = 0; k < kScanPer; ++k) {
        if (base + k < n) out[base + k] = run;
        run += x[k];
    }
    if (threadIdx.x == kThreads - 1) sums[blockIdx.x] = warp_tot[kThreads / 32 - 1];
}

// One-pass exclusive scan of the first n = *n_dev flags (decoupled look-back): out[i] = sum of
// in[0..i), out[n] = the total. CTAs take tiles of kScanBlock elements in launch order from a ticket
// counter, publish their tile sum (state 1) at once and their inclusive prefix (state 2) as soon as
// they know it; a tile's prefix is found by walking back over earlier tiles' status words until one
// holds an inclusive prefix. A CTA only waits on tiles whose tickets were taken earlier, by CTAs
// that are therefore running or done, and the walk is bounded (ERR_TIMEOUT). Every scan starts with
// all status words at state 0: the last CTA to finish (all look-back walks are over by then) clears
// the words this scan used, so the state lives on the device alone and a scan replayed from a CUDA
// graph behaves as one launched directly. The CTA with the last ticket resets the ticket counter.
__global__ void __launch_bounds__(kThreads) scan_onepass_dev_kernel(DevInterner I, const uint32_t *in, uint32_t *out,
                                                                   unsigned long long *status,
                                                                   const unsigned long long *n_dev) {
    pdl_wait();
    pdl_release();
    __shared__ uint32_t tile_s, prefix_s;
    __shared__ uint32_t warp_tot[kThreads / 32];
    unsigned long long *ticket = &I.ctr->scratch[SC_SCAN_TICKET];
    if (threadIdx.x == 0) {
        tile_s = (uint32_t)atomicAdd(ticket, 1ull);
        if (tile_s == gridDim.x - 1) *ticket = 0;  // every ticket is taken: ready for the next scan
    }
    __syncthreads();
    const uint32_t tile = tile_s;
    const uint32_t n = (uint32_t)*n_dev;
    const uint32_t base = tile * kScanBlock + threadIdx.x * kScanPer;
    uint32_t x[kScanPer];
    uint32_t local = 0;
#pragma unroll
    for (int k = 0; k < kScanPer; ++k) {
        x[k] = (base + k < n) ? in[base + k] : 0u;
        local += x[k];
    }
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    uint32_t incl = local;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if (lane >= (unsigned)o) incl += y;
    }
    if (lane == 31) warp_tot[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < kThreads / 32 ? warp_tot[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xFFFFFFFFu, w, o);
            if (lane >= (unsigned)o) w += y;
        }
        if (lane < kThreads / 32) warp_tot[lane] = w;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const uint32_t agg = warp_tot[kThreads / 32 - 1];
        uint32_t excl = 0;
        if (tile > 0) {
            st_release_u64(status + tile, (1ull << 32) | agg);
            uint32_t j = tile - 1;
            for (uint32_t spin = 0;; ++spin) {
                if (spin >= I.spin_limit) {
                    set_error(I, ERR_TIMEOUT, 40);
                    break;
                }
                const unsigned long long w = ld_acquire(reinterpret_cast<const uint64_t *>(status + j));
                const unsigned long long state = (w >> 32) & 3ull;
                if (state == 0) continue;  // tile j has not published yet
                excl += (uint32_t)w;
                if (state == 2ull || j == 0) break;  // an inclusive prefix ends the walk
                --j;
            }
        }
        st_release_u64(status + tile, (2ull << 32) | (excl + agg));
        prefix_s = excl;
    }
    __syncthreads();
    uint32_t run = prefix_s + incl - local + (warp ? warp_tot[warp - 1] : 0);
#pragma unroll
    for (int k = 0; k < kScanPer; ++k) {
        if (base + k < n) out[base + k] = run;
        run += x[k];
        if (base + k + 1 == n) out[n] = run;  // the total after the last element
    }
    if (n == 0 && tile == 0 && threadIdx.x == 0) out[0] = 0;
    if (grid_last_cta(&I.ctr->scratch[SC_SCAN_DONE]))  // no walk reads a status word any more
        for (uint32_t t = 0; t < gridDim.x; ++t) status[t] = 0;
}

__global__ void scan_add_dev_kernel(uint32_t *out, const uint32_t *sums, const unsigned long long *n_dev) {
    pdl_wait();
    pdl_release();
    const uint32_t n = (uint32_t)*n_dev;
    const uint32_t b = blockIdx.x;
    if (b == 0 || b * kScanBlock >= n) return;
    const uint32_t add = sums[b];
    const uint32_t base = b * kScanBlock;
    for (uint32_t k = threadIdx.x; k < kScanBlock; k += blockDim.x)
        if (base + k < n) out[base + k] += add;
}

__global__ void scan_total_dev_kernel(const uint32_t *in, uint32_t *out, const unsigned long long *n_dev) {
    pdl_wait();
    pdl_release();
    const uint32_t n = (uint32_t)*n_dev;
    out[n] = n ? out[n - 1] + in[n - 1] : 0u;
}

__global__ void scan_add_kernel(uint32_t *out, const uint32_t *sums, uint32_t n) {
    pdl_wait();
    pdl_release();
    const uint32_t b = blockIdx.x;
    if (b == 0) return;
    const uint32_t add = sums[b];
    const uint32_t base = b * kScanBlock;
    for (uint32_t k = threadIdx.x; k < kScanBlock; k += blockDim.x)
        if (base + k < n) out[base + k] += add;
}

__global__ void scan_total_kernel(const uint32_t *in, uint32_t *out, uint32_t n) {
    pdl_wait();
    pdl_release();
    out[n] = n ? out[n - 1] + in[n - 1] : 0u;
}

__device__ __forceinline__ void scatter_record(const ApplyArgs &a, uint32_t r) {
    if (!a.flags[r]) return;
    const uint32_t e = a.pos[r];
    a.e_item[0][e] = a.rec_item[r];
    a.e_path[0][e] = a.rec_group[r] << 3;
    a.e_id[0][e] = a.rec_id[r];
    a.e_val[0][e] = a.rec_val[r];
}

__global__ void scatter_bottom_kernel(DevInterner I, ApplyArgs a) {
    pdl_wait();
    pdl_release();
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r == 0) I.ctr->scratch[SC_ENTRIES] = a.pos[a.n_records];
    if (r < a.n_records) scatter_record(a, r);
}

__device__ __forceinline__ uint32_t parent_key_path(uint32_t path, int d, int t) {
    return t == 1 ? 0u : (path & path_mask(d, t - 2));
}

// Run heads of a level step: entry j starts a sibling run unless entry j-1 has the same parent.
__device__ __forceinline__ void head_flag(const ApplyArgs &a, int step, int buf, uint32_t j) {
    const uint32_t i = a.e_item[buf][j];
    const int d = a.it_depth[i];
    const int t = d - step;
    uint32_t head = 1;
    if (j > 0) {
        const uint32_t ip = a.e_item[buf][j - 1];
        if (ip == i && parent_key_path(a.e_path[buf][j - 1], d, t) == parent_key_path(a.e_path[buf][j], d, t))
            head = 0;
    }
    a.flags[j] = head;
}

__global__ void heads_kernel(DevInterner I, ApplyArgs a, int step, int buf) {
    pdl_wait();
    pdl_release();
    const uint32_t count = (uint32_t)I.ctr->scratch[SC_ENTRIES];
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < count; j += gridDim.x * blockDim.x)
        head_flag(a, step, buf, j);
}

// After the scan of the head flags: the number of parents and where each one's run starts.
__device__ __forceinline__ void starts_head(const DevInterner &I, const ApplyArgs &a, uint32_t count) {
    const uint32_t np = a.pos[count];
    a.p_start[np] = count;
    I.ctr->scratch[SC_PARENTS] = np;
    I.ctr->scratch[SC_ROOTS] = 0;
}

__global__ void starts_kernel(DevInterner I, ApplyArgs a) {
    pdl_wait();
    pdl_release();
    const uint32_t count = (uint32_t)I.ctr->scratch[SC_ENTRIES];
    if (blockIdx.x == 0 && threadIdx.x == 0) starts_head(I, a, count);
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < count; j += gridDim.x * blockDim.x)
        if (a.flags[j]) a.p_start[a.pos[j]] = j;
}

// Entries of the next level pass: the parents just reduced that are not tree roots.
__device__ __forceinline__ void next_count(const DevInterner &I) {
    I.ctr->scratch[SC_ENTRIES] = I.ctr->scratch[SC_PARENTS] - I.ctr->scratch[SC_ROOTS];
}

// Phase 2 for one level: parents cta_base + threadIdx.x, + stride, ... of the n_par run heads
// (a CTA-uniform loop, as in bottom_range).
__device__ __forceinline__ void parents_range(const DevInterner &I, const ApplyArgs &a, int mode, const LeafRefs &L,
                                              int step, int buf, uint32_t n_par, uint64_t cta_base, uint64_t stride) {
    const int nb = buf ^ 1;
    for (uint64_t base = cta_base; base < n_par; base += stride) {
        const uint64_t p = base + threadIdx.x;
        const bool in = p < n_par;
        uint64_t c[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        uint32_t cv[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        uint32_t types = 0, mask = 0, lod = 0;
        uint32_t i = 0, path0 = 0;
        int d = 0, t = 0;
        bool want_branch = false;
        uint64_t out = EMPTY_ID;
        uint32_t out_val = 0;
        if (in) {
            const uint32_t b = a.p_start[p], e = a.p_start[p + 1];
            i = a.e_item[buf][b];
            d = a.it_depth[i];
            t = d - step;
            path0 = a.e_path[buf][b];
            // the old node at the parent's place (voxtree.rs:934-952)
            uint64_t eq = a.it_init[i], leaf = EMPTY_ID;
            for (int cd = 0; cd + 1 < t; ++cd) {
                if (id_is_leaf(eq)) {
                    leaf = eq;
                    eq = EMPTY_ID;
                    break;
                }
                const uint32_t idx = (path0 >> (3 * (d - cd - 1))) & 7u;
                eq = I.children[8ull * id_index(eq) + idx];
                if (eq == EMPTY_ID) break;
            }
            if (id_is_leaf(eq)) {
                leaf = eq;
                eq = EMPTY_ID;
            }
            // gather the run of new children (voxtree.rs:959-1000); slots by select, so that the
            // arrays stay in registers
            for (uint32_t j = b; j < e; ++j) {
                const uint32_t ti = (a.e_path[buf][j] >> (3 * (d - t))) & 7u;
                const uint64_t id = a.e_id[buf][j];
                const uint32_t ev = a.e_val[buf][j];
#pragma unroll
                for (int k = 0; k < 8; ++k)
                    if ((uint32_t)k == ti) {
                        c[k] = id;
                        cv[k] = ev;
                    }
                types |= (id_is_leaf(id) ? 1u : 0u) << ti;
                mask |= 1u << ti;
            }
            if (mode == 1) {  // remove_at_depth_branch / _leaf one level up (voxtree.rs:559-706)
                const uint32_t ch = mask;
                uint64_t nc[8];
                uint32_t nv[8];
#pragma unroll
                for (int k = 0; k < 8; ++k) {
                    nc[k] = c[k];
                    nv[k] = cv[k];
                }
                if (eq != EMPTY_ID) {
                    const uint64_t *src = I.children + 8ull * id_index(eq);
#pragma unroll
                    for (int k = 0; k < 8; ++k) {
                        c[k] = src[k];
                        cv[k] = c[k] ? node_value(I, id_index(c[k])) : 0;
                    }
                    types = id_types(eq) & ~ch;
                    mask = id_mask(eq);
                } else if (leaf != EMPTY_ID) {
                    const uint32_t lv = node_value(I, id_index(leaf));
#pragma unroll
                    for (int k = 0; k < 8; ++k) {
                        c[k] = leaf;
                        cv[k] = lv;
                    }
                    types = 0xFFu & ~ch;
                    mask = 0xFF;
                } else {
                    set_error(I, ERR_INTERNAL, 45);
                    types = 0;
                    mask = 0;
                }
#pragma unroll
                for (int k = 0; k < 8; ++k)
                    if ((ch >> k) & 1) {
                        c[k] = nc[k];
                        cv[k] = nv[k];
                        if (nc[k] == EMPTY_ID)
                            mask &= ~(1u << k);
                        else
                            mask |= 1u << k;
                    }
                if (mask) {
                    want_branch = true;
                    lod = calc_average8(cv);
                } else {
                    out = EMPTY_ID;
                    out_val = 0;
                }
            } else {
                const uint32_t existing_mask = eq != EMPTY_ID ? id_mask(eq) : 0u;
                const uint32_t inv = (~mask) & 0xFFu;
                const uint32_t cloned = existing_mask & inv;
                if (mask != 0xFF) {
                    if (cloned) {  // voxtree.rs:1017-1031
                        const uint64_t *src = I.children + 8ull * id_index(eq);
    #pragma unroll
                        for (int k = 0; k < 8; ++k) {
                            if (!((cloned >> k) & 1)) continue;
                            c[k] = src[k];
                            cv[k] = c[k] ? node_value(I, id_index(c[k])) : 0;
                            types |= (id_is_leaf(c[k]) ? 1u : 0u) << k;
                            mask |= 1u << k;
                        }
                    } else if (leaf != EMPTY_ID) {  // voxtree.rs:1032-1047
                        const uint32_t lv = node_value(I, id_index(leaf));
    #pragma unroll
                        for (int k = 0; k < 8; ++k)
                            if ((inv >> k) & 1) {
                                c[k] = leaf;
                                cv[k] = lv;
                            }
                        types |= inv;
                        mask |= inv;
                    }
                }
                bool same = types == 0xFF;
    #pragma unroll
                for (int k = 1; k < 8; ++k) same = same && c[k] == c[0];
                if (same) {  // voxtree.rs:1062-1075
                    out = c[0];
                    out_val = cv[0];
                    if (cloned) add_ref_delta(I, c[0], 7 - 2 * __popc(cloned));  // Q6
                } else {
                    want_branch = true;
                    lod = calc_average8(cv);
                }
            }
            }
        bool created;
        const uint64_t id = warp_intern_branch_inl(I, want_branch, c, types, mask, lod, &created);
        if (created) add_child_refs(I, L, c, cv);
        if (!in) continue;
        if (want_branch) {
            out = id;
            out_val = lod;
        }
        if (t == 1) {
            a.it_new[i] = out;
            atomicAdd(&I.ctr->scratch[SC_ROOTS], 1ull);
        } else {
            a.e_item[nb][p] = i;
            a.e_path[nb][p] = path0 & path_mask(d, t - 2);
            a.e_id[nb][p] = out;
            a.e_val[nb][p] = out_val;
        }
    }
}

__global__ void __launch_bounds__(512, VX_APPLY_MIN_BLOCKS) parents_kernel(DevInterner I, ApplyArgs a, int step, int buf) {
    pdl_wait();
    pdl_release();
    const LeafRefs L = leaf_refs_init(I);
    parents_range(I, a, a.mode, L, step, buf, (uint32_t)I.ctr->scratch[SC_PARENTS],
                  (uint64_t)blockIdx.x * blockDim.x, (uint64_t)gridDim.x * blockDim.x);
    leaf_refs_flush(I, L);
    if (grid_last_cta(&I.ctr->scratch[SC_DONE])) next_count(I);  // entries of the next step
}



__device__ __forceinline__ void finish_item(const DevInterner &I, const ApplyArgs &a, int mode, uint32_t i) {
    if (mode == 1) {
        const uint64_t nw = a.it_new[i], old = a.it_old[i];
        if (nw == INVALID_ID) return;
        if (nw != EMPTY_ID) atomicAdd(I.refcount + id_index(nw), 1u);
        if (old != EMPTY_ID) {
            const unsigned long long e = atomicAdd(&I.ctr->scratch[SC_RELEASE], 1ull);
            a.release_list[e] = old;
        }
        I.roots[a.it_tree[i]] = nw;
        a.it_changed[i] = 1;
        return;
    }
    a.it_changed[i] = 0;
    if (a.it_panic[i]) return;
    const uint64_t nw = a.it_new[i], old = a.it_old[i];
    if (nw == INVALID_ID) return;
    const uint8_t f = a.it_flags[i];
    if ((f & 3) && nw != EMPTY_ID) atomicAdd(I.refcount + id_index(nw), 1u);  // the tree's root reference
    if (old != EMPTY_ID) {
        if (nw == old && !(I.flags & (1u << 4))) {  // assert_ne!(new_root_id, self.root_id) (voxtree.rs:311)
            set_error(I, ERR_REF_PANIC, 41);
            return;
        }
        const unsigned long long e = atomicAdd(&I.ctr->scratch[SC_RELEASE], 1ull);
        a.release_list[e] = old;
    }
    I.roots[a.it_tree[i]] = nw;
    a.it_changed[i] = 1;
}

// Commits every item's root, then (last CTA) closes the allocation epoch: every node of this apply
// pass has been created and has added its children's references by now.
__global__ void finish_items_kernel(DevInterner I, ApplyArgs a) {
    pdl_wait();
    pdl_release();
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < a.n_items) finish_item(I, a, a.mode, i);
    if (grid_last_cta(&I.ctr->scratch[SC_DONE])) epoch_finalize_body(I);
}

__global__ void zero_counter_kernel(DevInterner I, int slot) { pdl_wait(); pdl_release(); I.ctr->scratch[slot] = 0; }

__device__ __forceinline__ void item_depth(const DevInterner &I, const ApplyArgs &a, uint32_t i) {
    const uint32_t t = a.it_tree[i];
    const int d = t < I.tree_cap ? I.depths[t] : TREE_UNUSED;
    int prev = 0xFF;
    if (i > 0) {
        const uint32_t tp = a.it_tree[i - 1];
        prev = tp < I.tree_cap ? I.depths[tp] : TREE_UNUSED;
    }
    if (d == TREE_UNUSED || d > a.max_depth || d < 2 || (i > 0 && d > prev)) {
        set_error(I, ERR_INVALID, 46);
        const_cast<uint8_t *>(a.it_depth)[i] = 2;
        return;
    }
    const_cast<uint8_t *>(a.it_depth)[i] = (uint8_t)d;
}

__global__ void item_depths_kernel(DevInterner I, ApplyArgs a) {
    pdl_wait();
    pdl_release();
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < a.n_items) item_depth(I, a, i);
}

// ---- the whole apply in one cooperative launch -------------------------------------------------------
// Exclusive scan of one value per thread across the CTA (blockDim.x a multiple of 32, at most 1024);
// *total receives the CTA's sum. Every thread of the CTA calls it.
__device__ __forceinline__ uint32_t cta_exclusive_scan(uint32_t x, uint32_t *total) {
    __shared__ uint32_t wsum[32];
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    uint32_t incl = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if (lane >= (unsigned)o) incl += y;
    }
    if (lane == 31) wsum[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < nw ? wsum[lane] : 0u;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, w, o);
            if (lane >= (unsigned)o) w += y;
        }
        if (lane < nw) wsum[lane] = w;
    }
    __syncthreads();
    const uint32_t excl = incl - x + (warp ? wsum[warp - 1] : 0u);
    *total = wsum[nw - 1];
    __syncthreads();  // wsum is reused by the next call
    return excl;
}

// Exclusive scan of in[0..n) into out (out[n] = the total) by the whole cooperative grid: each CTA
// sums a contiguous range, the sums meet at a grid barrier, then each CTA scans its range from the
// sum of the ranges before it. Ends with a grid barrier (out is read across CTAs afterwards).
__device__ __forceinline__ bool grid_exclusive_scan(const DevInterner &I, const uint32_t *in, uint32_t *out,
                                                    uint32_t n, uint32_t *partials) {
    const uint32_t per = (n + gridDim.x - 1) / gridDim.x;
    const uint32_t lo = min(n, blockIdx.x * per), hi = min(n, lo + per);
    uint32_t s = 0, tot;
    for (uint32_t k = lo + threadIdx.x; k < hi; k += blockDim.x) s += in[k];
    cta_exclusive_scan(s, &tot);
    if (threadIdx.x == 0) partials[blockIdx.x] = tot;
    if (!grid_sync(I)) return false;
    uint32_t before = 0;
    for (uint32_t b = threadIdx.x; b < blockIdx.x; b += blockDim.x) before += partials[b];
    cta_exclusive_scan(before, &tot);
    uint32_t carry = tot;
    for (uint32_t base = lo; base < hi; base += blockDim.x) {
        const uint32_t k = base + threadIdx.x;
        const uint32_t x = k < hi ? in[k] : 0u;
        const uint32_t e = cta_exclusive_scan(x, &tot);
        if (k < hi) out[k] = carry + e;
        carry += tot;
    }
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) out[n] = carry;
    return grid_sync(I);
}

// The set phase (mode 0) and, when `clear_pass`, the clear pass (mode 1) with their releases: the
// launch sequence of launch_apply_bottom / launch_apply_levels / launch_release in one kernel whose
// phases are separated by grid barriers. Counts stay in device memory and are read by every CTA
// after the barrier that follows their last write.
__global__ void __launch_bounds__(512, VX_APPLY_MIN_BLOCKS) apply_single_kernel(const DevInterner I, const ApplyArgs a,
                                                                                   int check_depths, int clear_pass,
                                                                                   uint32_t *frontier_a,
                                                                                   uint32_t *frontier_b, int rounds) {
    const uint64_t cta_base = (uint64_t)blockIdx.x * blockDim.x, stride = (uint64_t)gridDim.x * blockDim.x;
    const uint64_t gt = cta_base + threadIdx.x;
    const bool t0 = gt == 0;
    DevCounters *ctr = I.ctr;
    if (check_depths) {
        for (uint64_t i = gt; i < a.n_items; i += stride) item_depth(I, a, (uint32_t)i);
        if (!grid_sync(I)) return;
    }
    for (int mode = 0; mode <= clear_pass; ++mode) {
        const LeafRefs L = leaf_refs_init(I);
        for (uint64_t i = gt; i < a.n_items; i += stride) prep_item(I, a, mode, (uint32_t)i);
        if (!grid_sync(I)) return;
        // Phase 1, then the changed groups become the first level's entries
        bottom_range(I, a, mode, L, cta_base, stride);
        if (!grid_sync(I)) return;
        if (!grid_exclusive_scan(I, a.flags, a.pos, a.n_records, a.scan_tmp)) return;
        for (uint64_t r = gt; r < a.n_records; r += stride) scatter_record(a, (uint32_t)r);
        uint32_t count = a.pos[a.n_records];
        if (!grid_sync(I)) return;
        // Phase 2, one level step at a time
        int buf = 0;
        for (int step = 1; step <= a.max_depth - 1; ++step) {
            for (uint64_t j = gt; j < count; j += stride) head_flag(a, step, buf, (uint32_t)j);
            if (!grid_sync(I)) return;
            if (!grid_exclusive_scan(I, a.flags, a.pos, count, a.scan_tmp)) return;
            const uint32_t np = a.pos[count];
            if (t0) {
                a.p_start[np] = count;
                ctr->scratch[SC_ROOTS] = 0;
            }
            for (uint64_t j = gt; j < count; j += stride)
                if (a.flags[j]) a.p_start[a.pos[j]] = (uint32_t)j;
            if (!grid_sync(I)) return;
            parents_range(I, a, mode, L, step, buf, np, cta_base, stride);
            if (!grid_sync(I)) return;
            count = np - (uint32_t)ctr->scratch[SC_ROOTS];  // parents that are not tree roots
            buf ^= 1;
        }
        // roots, the epoch, the release of the replaced roots
        if (t0) ctr->scratch[SC_RELEASE] = 0;
        if (!grid_sync(I)) return;
        for (uint64_t i = gt; i < a.n_items; i += stride) finish_item(I, a, mode, (uint32_t)i);
        leaf_refs_flush(I, L);
        if (t0) {
            ctr->rel_count[0] = 0;
            ctr->rel_count[1] = 0;
        }
        if (!grid_sync(I)) return;
        if (t0) epoch_finalize_body(I);
        release_roots_range(I, a.release_list, frontier_a, &ctr->rel_count[0], cta_base, stride);
        if (!grid_sync(I)) return;
        // round r reads set r % 3 and writes set (r + 1) % 3; set (r + 2) % 3 was read by round r - 1
        // and is written by round r + 1, so it is cleared now
        uint32_t *fr[2] = {frontier_a, frontier_b};
        for (int r = 0; r < rounds; ++r) {
            if (t0) ctr->rel_count[(r + 2) % 3] = 0;
            release_round_range(I, fr[r & 1], fr[(r + 1) & 1], &ctr->rel_count[r % 3], &ctr->rel_count[(r + 1) % 3],
                                cta_base, stride);
            if (!grid_sync(I)) return;
        }
    }
}

}  // namespace

size_t scan_tmp_words(uint32_t n) { return (size_t)(n + kScanBlock - 1) / kScanBlock + 32; }

// Dynamic shared memory of the kernels that create branches (their LeafRefs table).
static size_t leaf_refs_smem(const DevInterner &I) { return I.vbits == 8 ? 256 * 4 : 2 * kLeafSlots * 4; }

// Scan of the first *n_dev of n_max flags (count in device memory): one launch with the look-back
// status words for up to kScanStatusTiles tiles (a serving wave's records: 4 fewer launches per
// level), else block sums, their scan and an add (large batches: the single-thread look-back walk
// measured 12% slower than the three launches on 45 M edits).
static cudaError_t launch_scan_dev(const DevInterner &I, const uint32_t *flags, uint32_t *pos, uint32_t *tmp,
                                   uint32_t n_max, const unsigned long long *n_dev, unsigned long long *status,
                                   cudaStream_t s) {
    const uint32_t nb = (n_max + kScanBlock - 1) / kScanBlock;
    if (nb == 0) return cudaSuccess;
    if (status && nb <= kScanStatusTiles) {
        count_launches(1);
        (void)launch_pdl(scan_onepass_dev_kernel, dim3(nb), dim3(kThreads), 0, s, I, flags, pos, status, n_dev);
        return cudaGetLastError();
    }
    count_launches(1);
    (void)launch_pdl(scan_blocks_dev_kernel, dim3(nb), dim3(kThreads), 0, s, flags, pos, tmp, n_dev);
    if (nb > 1) {
        uint32_t *tmp2 = tmp + nb;
        cudaError_t e = launch_scan(tmp, tmp2, tmp2 + nb + 1 + 32, nb, s);
        if (e != cudaSuccess) return e;
        count_launches(1);
        (void)launch_pdl(scan_add_dev_kernel, dim3(nb), dim3(kThreads), 0, s, pos, tmp2, n_dev);
    }
    count_launches(1);
    (void)launch_pdl(scan_total_dev_kernel, dim3(1), dim3(1), 0, s, flags, pos, n_dev);
    return cudaGetLastError();
}

cudaError_t launch_scan(const uint32_t *flags, uint32_t *pos, uint32_t *tmp, uint32_t n, cudaStream_t s) {
    const uint32_t nb = (n + kScanBlock - 1) / kScanBlock;
    if (nb == 0) {
        count_launches(1);
        (void)launch_pdl(scan_total_kernel, dim3(1), dim3(1), 0, s, flags, pos, 0);
        return cudaGetLastError();
    }
    count_launches(1);
    (void)launch_pdl(scan_blocks_kernel, dim3(nb), dim3(kThreads), 0, s, flags, pos, tmp, n);
    if (nb > 1) {
        uint32_t *tmp2 = tmp + nb;  // scan of the block sums (recursive)
        cudaError_t e = launch_scan(tmp, tmp2, tmp2 + nb + 1 + 32, nb, s);
        if (e != cudaSuccess) return e;
        count_launches(1);
        (void)launch_pdl(scan_add_kernel, dim3(nb), dim3(kThreads), 0, s, pos, tmp2, n);
    }
    count_launches(1);
    (void)launch_pdl(scan_total_kernel, dim3(1), dim3(1), 0, s, flags, pos, n);
    return cudaGetLastError();
}

cudaError_t launch_item_depths(const DevInterner &I, const ApplyArgs &a, cudaStream_t s) {
    if (a.n_items == 0) return cudaSuccess;
    count_launches(1);
    (void)launch_pdl(item_depths_kernel, dim3((a.n_items + kThreads - 1) / kThreads), dim3(kThreads), 0, s, I, a);
    return cudaGetLastError();
}

cudaError_t launch_apply_bottom(const DevInterner &I, const ApplyArgs &a, int num_sms, cudaStream_t s) {
    const unsigned ib = (a.n_items + kThreads - 1) / kThreads;
    count_launches(1);
    (void)launch_pdl(prep_items_kernel, dim3(ib), dim3(kThreads), 0, s, I, a);
    const uint32_t R = a.n_records;
    if (R) {
        const int bt = a.threads > 0 ? a.threads : kThreads;
        const unsigned cap = (unsigned)num_sms * (unsigned)(a.blocks_per_sm > 0 ? a.blocks_per_sm : 8);
        const unsigned need = (R + bt - 1) / bt;
        const unsigned g = need < cap ? need : cap;
        count_launches(1);
        (void)launch_pdl(bottom_kernel, dim3(g), dim3(bt), leaf_refs_smem(I), s, I, a);
    }
    return cudaGetLastError();
}

cudaError_t launch_apply_levels(const DevInterner &I, const ApplyArgs &a, int num_sms, cudaStream_t s) {
    const unsigned ib = (a.n_items + kThreads - 1) / kThreads;
    const uint32_t R = a.n_records;
    const unsigned rb = (R + kThreads - 1) / kThreads;
    if (R) {
        const int bt = a.threads > 0 ? a.threads : kThreads;
        const unsigned cap = (unsigned)num_sms * (unsigned)(a.blocks_per_sm > 0 ? a.blocks_per_sm : 8);
        const unsigned need = (R + bt - 1) / bt;
        const unsigned g = need < cap ? need : cap;
        cudaError_t e = launch_scan(a.flags, a.pos, a.scan_tmp, R, s);
        if (e != cudaSuccess) return e;
        count_launches(1);
        (void)launch_pdl(scatter_bottom_kernel, dim3(rb), dim3(kThreads), 0, s, I, a);
        int buf = 0;
        const unsigned sb = rb < (unsigned)num_sms * 16 ? rb : (unsigned)num_sms * 16;
        for (int step = 1; step <= a.max_depth - 1; ++step) {
            count_launches(1);
            (void)launch_pdl(heads_kernel, dim3(sb), dim3(kThreads), 0, s, I, a, step, buf);
            e = launch_scan_dev(I, a.flags, a.pos, a.scan_tmp, R, &I.ctr->scratch[SC_ENTRIES], a.scan_status, s);
            if (e != cudaSuccess) return e;
            count_launches(1);
            (void)launch_pdl(starts_kernel, dim3(sb), dim3(kThreads), 0, s, I, a);
            count_launches(1);
            (void)launch_pdl(parents_kernel, dim3(g), dim3(bt), leaf_refs_smem(I), s, I, a, step, buf);  // its last CTA sets the next entry count
            buf ^= 1;
        }
    }
    count_launches(1);
    (void)launch_pdl(zero_counter_kernel, dim3(1), dim3(1), 0, s, I, SC_RELEASE);
    count_launches(1);
    (void)launch_pdl(finish_items_kernel, dim3(ib), dim3(kThreads), 0, s, I, a);  // its last CTA closes the epoch
    return cudaGetLastError();
}

namespace {
// rec_item[r] = i for every record r of item i (records of item i: [first[i], first[i+1])), one CTA
// per item with coalesced stores.
__global__ void __launch_bounds__(kThreads) expand_items_kernel(const uint32_t *first, uint32_t n,
                                                               uint32_t *rec_item) {
    for (uint32_t i = blockIdx.x; i < n; i += gridDim.x) {
        const uint32_t r1 = first[i + 1];
        for (uint32_t r = first[i] + threadIdx.x; r < r1; r += blockDim.x) rec_item[r] = i;
    }
}
}  // namespace

cudaError_t launch_expand_items(const uint32_t *first, uint32_t n, uint32_t *rec_item, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    count_launches(1);
    expand_items_kernel<<<n < 65535u ? n : 65535u, kThreads, 0, s>>>(first, n, rec_item);
    return cudaGetLastError();
}

size_t apply_single_scan_words(int num_sms) { return (size_t)num_sms * 32 + 64; }

// The whole apply sequence in one cooperative launch: as many CTAs as can be resident at once (the
// grid barrier needs every CTA running).
cudaError_t launch_apply_single(const DevInterner &I, const ApplyArgs &a, bool check_depths, bool clear_pass,
                                uint32_t *frontier_a, uint32_t *frontier_b, int rounds, int num_sms, cudaStream_t s) {
    const int bt = a.threads > 0 ? a.threads : kThreads;
    const size_t smem = leaf_refs_smem(I);
    static int per_sm_cache[2][17] = {};  // [vbits == 16][threads / 32]
    int &per_sm = per_sm_cache[I.vbits == 16][bt / 32];
    if (per_sm == 0) {
        cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, apply_single_kernel, bt, smem);
        if (e != cudaSuccess) return e;
        if (per_sm < 1) return cudaErrorInvalidConfiguration;
    }
    int want = a.blocks_per_sm > 0 ? a.blocks_per_sm : per_sm;
    if (want > per_sm) want = per_sm;
    if ((size_t)num_sms * want > apply_single_scan_words(num_sms) - 64) want = 32;  // partials of the grid scan
    // a small apply (a serving wave) runs on as few CTAs as its records fill, no fewer than a quarter
    // of the SMs: every grid barrier costs one arrival per CTA
    uint64_t grid = (uint64_t)num_sms * want;
    const uint64_t fill = ((uint64_t)(a.n_records > a.n_items ? a.n_records : a.n_items) + bt - 1) / bt;
    const uint64_t floor_ctas = (uint64_t)(num_sms + 3) / 4;
    if (fill < grid) grid = fill > floor_ctas ? fill : floor_ctas;
    DevInterner Ic = I;
    ApplyArgs ac = a;
    int cd = check_depths ? 1 : 0, cp = clear_pass ? 1 : 0;
    void *args[] = {&Ic, &ac, &cd, &cp, &frontier_a, &frontier_b, &rounds};
    count_launches(1);
    return cudaLaunchCooperativeKernel(reinterpret_cast<const void *>(apply_single_kernel), dim3((unsigned)grid), dim3(bt), args,
                                       smem, s);
}

cudaError_t launch_apply(const DevInterner &I, const ApplyArgs &a, int num_sms, cudaStream_t s) {
    cudaError_t e = launch_apply_bottom(I, a, num_sms, s);
    if (e != cudaSuccess) return e;
    return launch_apply_levels(I, a, num_sms, s);
}

}  // namespace vxg
