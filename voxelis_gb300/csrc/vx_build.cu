// Dense-chunk construction on EMPTY trees, and the refcount epoch shared by all batch paths.
//
// Reference behaviour restated here: a Batch filled by just_set from every voxel of a dense grid and
// applied to an EMPTY tree (core/batch.rs:145-172, spatial/voxtree.rs:724-1118). On an EMPTY tree
// the batch algorithm reduces to:
//   bottom group (depth d-1, 8 voxels): all zero -> not touched (no path); all 8 set and equal ->
//     leaf(v) (voxtree.rs:826, 887-896); otherwise branch(children = leaf(v) or EMPTY, types = mask =
//     set bits) (voxtree.rs:840-883);
//   every level above: a parent exists iff one of its children was touched; children that were not
//     touched stay EMPTY; 8 equal leaf children collapse into that leaf (voxtree.rs:1050-1075);
//     otherwise branch(children, types = leaf bits, mask = present bits) (voxtree.rs:1052-1061).
//   The root is the level-0 result; an all-zero grid leaves the tree unchanged (voxtree.rs:905-911).
//
// GB300 mapping, by chunk depth:
//   5-10 (launch_dense_split): dense_quads16_kernel streams every 16^3 octant through a per-warp
//     shared tile (4-D TMA tensor copies completing on an mbarrier; octants after a warp's first one
//     come from a device-wide counter) and settles every quad (4^3 voxels): uniform quads directly,
//     the others through a device-wide quad memo, where a miss claims a record;
//     dense_memo_compute_kernel then computes each claimed record (a distinct quad of the build)
//     once, 8 lanes per quad; one pass per level above the quads resolves them and reduces parents
//     (fresh_level_kernel, fresh_top_kernel for the three top levels).
//   4: dense_octants_kernel, a warp per chunk-sized octant with all levels in the warp.
//   2-3: dense_blocks_kernel, a CTA per chunk staged by one cp.async.bulk copy.
//   vx_build_dense_noalloc: dense_cta32_kernel, a CTA per 32^3 block with block-level scratch only.
// Only hash-consing touches global memory besides the grids. Warps deduplicate identical keys with
// __match_any_sync before probing the branch table, and inserts are warp-cooperative
// (vx_device.cuh). Grids are persistent: a multiple of the SM count.
//
// Refcounts follow from the reference's accounting (interner/mod.rs:712-829): a hash-cons hit gives
// back the references its children were pre-charged with, so after a build every node's count equals
// the number of child slots of newly created nodes that name it, plus one per tree root. The split
// path of 8-bit interners adds it as it creates nodes (the creating lane counts the new node's
// children; leaf children into per-CTA value counters) and its last kernel closes the epoch; the
// other builds compute the sum once per epoch over the allocation log (launch_epoch_refcounts).
#include <cuda.h>
#include <mutex>
#include <type_traits>
#include <cudaTypedefs.h>

#include "vx_launch.h"

namespace vxg {
namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ uint32_t compact3(uint32_t x) {
    x &= 0x09249249u;
    x = (x ^ (x >> 2)) & 0x030C30C3u;
    x = (x ^ (x >> 4)) & 0x0300F00Fu;
    x = (x ^ (x >> 8)) & 0xFF0000FFu;
    x = (x ^ (x >> 16)) & 0x000003FFu;
    return x;
}

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ void bulk_copy_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}

// Fills the CTA's 8-bit leaf cache from the leaf table (one coalesced 2 KB read): leaves already
// interned (every value a build has met so far) are found in shared memory from the first lookup,
// instead of one dependent global read per value and CTA. Leaves cannot be released during a build.
// All threads of the CTA call it; a barrier follows before the first lookup.
__device__ __forceinline__ void leaf_cache_warm(const DevInterner &I, uint64_t *leaf_cache, unsigned tid) {
    for (unsigned k = tid; k < 256; k += blockDim.x) {
        const uint64_t s = ld_volatile(I.leaf_table + k);
        leaf_cache[k] = s > LEAF_BUSY ? s : 0ull;
    }
}

// Leaf id of value v (v != 0): a per-CTA shared cache for 8-bit voxels, the global table otherwise.
template <class T>
__device__ __forceinline__ uint64_t leaf_of(const DevInterner &I, uint64_t *leaf_cache, uint32_t v) {
    if (sizeof(T) == 1) {
        uint64_t id = leaf_cache[v];
        if (id) return id;
        bool created;
        id = intern_leaf(I, v, &created);
        if (id != EMPTY_ID) leaf_cache[v] = id;
        return id;
    }
    uint64_t id = ld_volatile(I.leaf_table + v);
    if (id > LEAF_BUSY) return id;
    bool created;
    return intern_leaf(I, v, &created);
}

// leaf_of for 8-bit voxels with one global lookup per CTA and value: the first lane to miss the CTA's
// cache claims the value in `claim` and finds or creates the leaf; the others wait (bounded) on the
// shared cache, so a leaf that every warp of the grid needs at once is awaited in shared memory, not
// by thousands of lanes re-reading one leaf-table word. A claimer that fails marks the value (2) and
// the waiters go to the table themselves.
#ifndef VX_LEAF_CLAIM
#define VX_LEAF_CLAIM 1
#endif
__device__ __forceinline__ uint64_t leaf_of_claimed(const DevInterner &I, uint64_t *leaf_cache, uint32_t *claim,
                                                    uint32_t v) {
    uint64_t id = *(volatile uint64_t *)(leaf_cache + v);
    if (id) return id;
    bool created;
    if (atomicCAS(claim + v, 0u, 1u) == 0u) {
        id = intern_leaf(I, v, &created);
        if (id != EMPTY_ID)
            *(volatile uint64_t *)(leaf_cache + v) = id;
        else
            *(volatile uint32_t *)(claim + v) = 2u;
        return id;
    }
    for (uint32_t spin = 0; spin < (1u << 16); ++spin) {
        id = *(volatile uint64_t *)(leaf_cache + v);
        if (id) return id;
        if (*(volatile uint32_t *)(claim + v) == 2u) break;
        __nanosleep(32);
    }
    return intern_leaf(I, v, &created);
}

template <class T>
__global__ void __launch_bounds__(kThreads) dense_blocks_kernel(DevInterner I, DenseArgs a) {
    extern __shared__ __align__(128) unsigned char smem[];
    const int B = a.depth;
    const int S = 1 << B;
    const uint32_t V = 1u << (3 * B);
    const uint32_t G = V >> 3;
    const uint32_t n_nodes = (V - 1) / 7;  // 1 + 8 + ... + 8^(B-1)
    T *vox = reinterpret_cast<T *>(smem);
    const size_t vox_bytes = ((size_t)V * sizeof(T) + 127) & ~(size_t)127;
    uint64_t *lvl = reinterpret_cast<uint64_t *>(smem + vox_bytes);
    uint32_t *lval = reinterpret_cast<uint32_t *>(lvl + n_nodes);
    uint64_t *leaf_cache = reinterpret_cast<uint64_t *>(lval + ((n_nodes + 1) & ~1u));
    uint64_t *bar = leaf_cache + 256;

    const unsigned tid = threadIdx.x, lane = tid & 31u;
    if (sizeof(T) == 1)
        leaf_cache_warm(I, leaf_cache, tid);
    if (tid == 0) {
        mbar_init(bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();

    uint32_t phase = 0;
    for (uint32_t chunk = blockIdx.x; chunk < a.n_chunks; chunk += gridDim.x) {
        {
            // tree handles may come from device memory: check them before any write
            const uint32_t tree = a.trees[chunk];
            const bool bad = tree >= I.tree_cap || I.depths[tree] != a.depth || I.roots[tree] != EMPTY_ID;
            if (__syncthreads_or(bad)) {
                if (tid == 0) set_error(I, ERR_INVALID, 21);
                continue;
            }
        }
        const T *grid = reinterpret_cast<const T *>(a.grids) + (size_t)chunk * V;

        // ---- stage the chunk into shared memory (V * sizeof(T) >= 64 bytes: a multiple of 16) ---
        if (tid == 0) {
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            mbar_expect_tx(bar, V * (uint32_t)sizeof(T));
            bulk_copy_g2s(vox, grid, V * (uint32_t)sizeof(T), bar);
        }
        bool ok = false;
        for (uint32_t spin = 0; spin < SPIN_LIMIT; ++spin)
            if ((ok = mbar_try_wait(bar, phase))) break;
        if (__syncthreads_or(!ok)) {  // every thread leaves together; the copy is drained first
            if (tid == 0) set_error(I, ERR_TIMEOUT, 20);
            for (uint32_t spin = 0; spin < SPIN_LIMIT && !mbar_try_wait(bar, phase); ++spin) {
            }
            return;
        }
        phase ^= 1u;

        // ---- bottom groups (depth d-1) ------------------------------------------------------
        uint64_t *bottom = lvl + (G - 1) / 7;
        uint32_t *bottom_val = lval + (G - 1) / 7;
        for (uint32_t g0 = 0; g0 < G; g0 += blockDim.x) {
            const uint32_t g = g0 + tid;
            const bool in = g < G;
            uint32_t v[8] = {0, 0, 0, 0, 0, 0, 0, 0};
            uint64_t klo = 0, khi = 0;
            if (in) {
                const uint32_t gx = compact3(g), gy = compact3(g >> 1), gz = compact3(g >> 2);
                const uint32_t base = ((2 * gy) * S + 2 * gz) * S + 2 * gx;
                const uint32_t off[4] = {base, base + (uint32_t)(S * S), base + (uint32_t)S,
                                         base + (uint32_t)(S * S + S)};
                if (sizeof(T) == 1) {
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        uint32_t w = *reinterpret_cast<const uint16_t *>(vox + off[q]);
                        v[2 * q] = w & 0xFF;
                        v[2 * q + 1] = w >> 8;
                        klo |= (uint64_t)w << (16 * q);
                    }
                } else {
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        uint32_t w = *reinterpret_cast<const uint32_t *>(vox + off[q]);
                        v[2 * q] = w & 0xFFFF;
                        v[2 * q + 1] = w >> 16;
                        if (q < 2)
                            klo |= (uint64_t)w << (32 * q);
                        else
                            khi |= (uint64_t)w << (32 * (q - 2));
                    }
                }
            }
            uint32_t set = 0;
#pragma unroll
            for (int k = 0; k < 8; ++k) set |= (v[k] != 0 ? 1u : 0u) << k;
            bool uniform = set == 0xFF;
#pragma unroll
            for (int k = 1; k < 8; ++k) uniform = uniform && v[k] == v[0];
            const bool is_branch = in && set != 0 && !uniform;

            // warp dedup of identical groups (the 8 values are the whole key of a bottom branch)
            const unsigned bm = __ballot_sync(0xFFFFFFFFu, is_branch);
            const uint64_t mk_lo = is_branch ? klo : ~(uint64_t)lane;
            unsigned grp = __match_any_sync(0xFFFFFFFFu, mk_lo);
            if (sizeof(T) == 2) grp &= __match_any_sync(0xFFFFFFFFu, is_branch ? khi : ~(uint64_t)lane);
            grp &= bm;
            const int leader = is_branch ? __ffs(grp) - 1 : (int)lane;
            const bool lead = is_branch && leader == (int)lane;

            uint64_t c[8];
            uint32_t lod = 0;
            if (lead) {
#pragma unroll
                for (int k = 0; k < 8; ++k) c[k] = v[k] ? leaf_of<T>(I, leaf_cache, v[k]) : EMPTY_ID;
                lod = calc_average8(v);
            } else {
#pragma unroll
                for (int k = 0; k < 8; ++k) c[k] = 0;
            }
            bool created;
            uint64_t id = warp_intern_branch(I, lead, c, set, set, lod, &created);
            id = __shfl_sync(0xFFFFFFFFu, id, leader);
            lod = __shfl_sync(0xFFFFFFFFu, lod, leader);
            if (in) {
                uint64_t out;
                uint32_t val;
                if (set == 0) {
                    out = EMPTY_ID;
                    val = 0;
                } else if (uniform) {
                    out = leaf_of<T>(I, leaf_cache, v[0]);
                    val = v[0];
                } else {
                    out = id;
                    val = lod;
                }
                bottom[g] = out;
                bottom_val[g] = val;
            }
        }
        __syncthreads();

        // ---- levels above, inside the block ----------------------------------------------------
        for (int l = B - 2; l >= 0; --l) {
            const uint32_t P = 1u << (3 * l);
            uint64_t *cur = lvl + (P - 1) / 7;
            uint32_t *cur_val = lval + (P - 1) / 7;
            const uint64_t *below = lvl + (8 * P - 1) / 7;
            const uint32_t *below_val = lval + (8 * P - 1) / 7;
            for (uint32_t p0 = 0; p0 < P; p0 += blockDim.x) {
                const uint32_t p = p0 + tid;
                const bool in = p < P;
                uint64_t c[8];
                uint32_t cv[8];
                uint32_t types = 0, mask = 0;
#pragma unroll
                for (int k = 0; k < 8; ++k) {
                    c[k] = in ? below[8 * p + k] : 0;
                    cv[k] = in ? below_val[8 * p + k] : 0;
                    mask |= (c[k] != 0 ? 1u : 0u) << k;
                    types |= (id_is_leaf(c[k]) ? 1u : 0u) << k;
                }
                bool same = types == 0xFF;
#pragma unroll
                for (int k = 1; k < 8; ++k) same = same && c[k] == c[0];
                const bool is_branch = in && mask != 0 && !same;
                const uint32_t lod = is_branch ? calc_average8(cv) : 0;
                bool created;
                uint64_t id = warp_intern_branch(I, is_branch, c, types, mask, lod, &created);
                if (in) {
                    if (mask == 0) {
                        cur[p] = EMPTY_ID;
                        cur_val[p] = 0;
                    } else if (same) {
                        cur[p] = c[0];
                        cur_val[p] = cv[0];
                    } else {
                        cur[p] = id;
                        cur_val[p] = lod;
                    }
                }
            }
            __syncthreads();
        }

        // ---- chunk root ----------------------------------------------------------------------
        if (tid == 0) {
            const uint64_t root = lvl[0];
            const uint32_t tree = a.trees[chunk];
            if (root != EMPTY_ID) {
                I.roots[tree] = root;
                atomicAdd(I.refcount + id_index(root), 1u);
            }
            if (a.changed) a.changed[chunk] = root != EMPTY_ID;
        }
        __syncthreads();
    }
}

// ---- CTA-wide caches of the dense-build kernels ------------------------------------------------
//
// Bottom-group keys (the 8 packed voxel values of a 2^3 group) are looked up first in a CTA-wide
// shared cache of the branches this CTA already interned, with their LOD values; only misses go to
// the global branch table, deduplicated within the warp.

#ifndef VX_KEY_CACHE
#define VX_KEY_CACHE 256
#endif
#ifndef VX_OCT_TILES
#define VX_OCT_TILES 1
#endif
constexpr int kKeyCache = VX_KEY_CACHE;  // entries of the shared bottom-key cache (power of two)
constexpr int kOctTiles = VX_OCT_TILES;  // tile buffers per warp in the octant kernel (1 or 2)

struct KeyCache {
    uint64_t *k0, *k1, *id;
    uint32_t *val;  // LOD value of each entry, or null when the caller does not cache it
};

__device__ __forceinline__ uint32_t kc_slot(uint64_t lo, uint64_t hi) {
    return (uint32_t)(fmix64(lo ^ (hi * 0x9E3779B97F4A7C15ull)) >> 40) & (kKeyCache - 1);
}

// Branch id cached for (lo, hi), or 0 (and its LOD value in *lod when cached). An entry is
// published by writing its id (>= 2) last.
__device__ __forceinline__ uint64_t kc_lookup(const KeyCache &C, uint64_t lo, uint64_t hi, uint32_t *lod = nullptr) {
    uint32_t h = kc_slot(lo, hi);
#pragma unroll 1
    for (int p = 0; p < 8; ++p) {
        const uint64_t id = *(volatile uint64_t *)(C.id + h);
        if (id == 0) return 0;
        if (id > 1 && *(volatile uint64_t *)(C.k0 + h) == lo && *(volatile uint64_t *)(C.k1 + h) == hi) {
            if (lod) *lod = *(volatile uint32_t *)(C.val + h);
            return id;
        }
        h = (h + 1) & (kKeyCache - 1);
    }
    return 0;
}

__device__ __forceinline__ void kc_insert(const KeyCache &C, uint64_t lo, uint64_t hi, uint64_t id, uint32_t lod = 0) {
    uint32_t h = kc_slot(lo, hi);
#pragma unroll 1
    for (int p = 0; p < 8; ++p) {
        if (atomicCAS((unsigned long long *)(C.id + h), 0ull, 1ull) == 0ull) {
            C.k0[h] = lo;
            C.k1[h] = hi;
            if (C.val) C.val[h] = lod;
            __threadfence_block();
            *(volatile uint64_t *)(C.id + h) = id;
            return;
        }
        h = (h + 1) & (kKeyCache - 1);
    }
}

// One reference per child slot of branch `id`, which the calling lane just created (equal children
// summed first): leaves of 8-bit interners into the CTA's per-value counters when leaf_cnt is given
// (added to the leaves by leaf_cnt_flush), everything else by fire-and-forget atomics. The children
// are read back from the record just written rather than kept live in registers across the insert.
__device__ __forceinline__ void count_created(const DevInterner &I, uint32_t *leaf_cnt, uint64_t id) {
    uint64_t c[8];
    const ulonglong2 *src = reinterpret_cast<const ulonglong2 *>(I.children + 8ull * id_index(id));
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const ulonglong2 w = src[k];
        c[2 * k] = w.x;
        c[2 * k + 1] = w.y;
    }
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
        if (leaf_cnt && id_is_leaf(c[k]))
            atomicAdd(leaf_cnt + (node_value(I, id_index(c[k])) & 0xFFu), n);
        else
            atomicAdd(I.refcount + id_index(c[k]), n);
    }
}

// The same from children and values still held in registers (no read-back of the record).
__device__ __forceinline__ void count_created_regs(const DevInterner &I, uint32_t *leaf_cnt, const uint64_t c[8],
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
        if (leaf_cnt && id_is_leaf(c[k]))
            atomicAdd(leaf_cnt + (cv[k] & 0xFFu), n);
        else
            atomicAdd(I.refcount + id_index(c[k]), n);
    }
}

// A created bottom group of an 8-bit interner: its children are the leaves of its nonzero voxel
// values, so the per-value counters take them straight from the values.
__device__ __forceinline__ void count_group_leaves(uint32_t *leaf_cnt, const uint32_t v[8]) {
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        if (v[k] == 0) continue;
        bool seen = false;
        uint32_t n = 1;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            if (j < k && v[j] == v[k]) seen = true;
            if (j > k && v[j] == v[k]) ++n;
        }
        if (!seen) atomicAdd(leaf_cnt + (v[k] & 0xFFu), n);
    }
}

// Adds a CTA's per-value leaf counts to the leaves (every thread of the CTA calls it).
__device__ __forceinline__ void leaf_cnt_flush(const DevInterner &I, uint32_t *leaf_cnt) {
    __syncthreads();
    for (unsigned v = threadIdx.x; v < 256; v += blockDim.x) {
        const uint32_t n = leaf_cnt[v];
        if (n == 0) continue;
        const uint64_t lid = I.leaf_table[v];
        if (lid > LEAF_BUSY)
            atomicAdd(I.refcount + id_index(lid), n);
        else
            set_error(I, ERR_INTERNAL, 31);
    }
}

__device__ __forceinline__ void leaf_cnt_clear(uint32_t *leaf_cnt) {
    for (unsigned v = threadIdx.x; v < 256; v += blockDim.x) leaf_cnt[v] = 0;
}

// One parent from 8 children held by the calling lane: EMPTY, a collapsed leaf, or an interned
// branch (warp-cooperative; every lane of the warp calls it). created (optional): whether this lane
// created the branch, for callers that count references.
__device__ __forceinline__ void reduce_parent(const DevInterner &I, bool active, const uint64_t c[8],
                                              const uint32_t cv[8], uint64_t &out, uint32_t &out_val,
                                              bool *created_out = nullptr) {
    uint32_t types = 0, mask = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        mask |= (c[k] != 0 ? 1u : 0u) << k;
        types |= (id_is_leaf(c[k]) ? 1u : 0u) << k;
    }
    bool same = types == 0xFF;
#pragma unroll
    for (int k = 1; k < 8; ++k) same = same && c[k] == c[0];
    const bool is_branch = active && mask != 0 && !same;
    const uint32_t lod = is_branch ? calc_average8(cv) : 0;
    bool created;
    const uint64_t id = warp_intern_branch(I, is_branch, c, types, mask, lod, &created);
    if (created_out) *created_out = created;
    if (mask == 0) {
        out = EMPTY_ID;
        out_val = 0;
    } else if (same) {
        out = c[0];
        out_val = cv[0];
    } else {
        out = id;
        out_val = lod;
    }
}

// ---- 16^3 octants, one warp each, TMA tensor copies, last-arriver reduction above ------------
//
// Each warp streams its own octants: lane 0 issues a 4-D tiled TMA copy (box 16 x 16 x 16 of the
// [chunk][y][z][x] grid tensor) of the next octant into the warp's second tile while the warp reduces
// the current one, so loads overlap work and no warp ever waits for another at a CTA barrier. An
// octant root is stored in its level's scratch row; the warp that brings the 8th sibling of a parent
// (an atomic arrival count per parent) reads the siblings and reduces the parent, up to the chunk
// root. The only CTA-wide structures are the shared bottom-key cache and the 8-bit leaf cache.

struct OctArgs {
    const uint32_t *trees;
    uint32_t n_chunks;
    int depth;
    uint8_t *changed;
    uint64_t *ids;   // octant and higher level nodes: level k (1 .. depth-4) at lvl_off[k]
    uint32_t *vals;
    uint32_t *cnt;   // arrival counts of levels 0 .. depth-5 at cnt_off[k]
    uint64_t lvl_off[12];
    uint64_t cnt_off[12];
    const void *grids;               // the chunks' dense grids (for plain bulk copies)
    // quad memo (optional: slots == nullptr disables it)
    unsigned long long *memo_slots;  // tag:32 | (record + 1):32, 0 = empty
    unsigned int *memo_count;        // records handed out
    unsigned char *memo_recs;        // record r: 16 row words, then id (8 B) and LOD value (4 B)
    uint32_t memo_mask;              // slots - 1
    uint32_t memo_cap;               // records
    unsigned long long *work;        // octants handed out beyond the first one per warp (nullptr: fixed stride)
    unsigned int *live_count;        // records whose claim won its slot (nullptr: no list)
    uint32_t *live;                  // their indices, in claim order (memo_cap entries)
    int count_refs;                  // creators count their children's references (no epoch pass)
};

constexpr int kOctWarps = 8;

// ---- CTA-wide cache of parents by their 8 child ids ----------------------------------------------
//
// Parents above the quads are looked up in a small shared cache keyed by their 8 child ids before the
// global branch table; every entry also holds the node's LOD value, so a hit skips calc_average.

#ifndef VX_NODE_CACHE
#define VX_NODE_CACHE 64
#endif
constexpr int kNodeCache = VX_NODE_CACHE;  // entries (power of two)

struct NodeCache {
    uint64_t *key;   // [kNodeCache][8]
    uint64_t *id;    // 0 free, 1 being written, else a branch id
    uint32_t *meta;  // kind << 31 | LOD value (kind 0: quad voxels, 1: child ids)
};

__device__ __forceinline__ uint32_t nc_slot(const uint64_t k[8], uint32_t kind) {
    uint32_t h = kind ? 0x2545F491u : 0x9E3779B9u;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        h = h * 0x01000193u + (uint32_t)k[i];
        h = h * 0x01000193u + (uint32_t)(k[i] >> 32);
    }
    h ^= h >> 16;
    h *= 0x85EBCA6Bu;
    h ^= h >> 13;
    return h & (kNodeCache - 1);
}

__device__ __forceinline__ uint64_t nc_lookup(const NodeCache &N, const uint64_t k[8], uint32_t kind,
                                              uint32_t &lod) {
    uint32_t h = nc_slot(k, kind);
#pragma unroll 1
    for (int p = 0; p < 4; ++p) {
        const uint64_t id = *(volatile uint64_t *)(N.id + h);
        if (id == 0) return 0;
        if (id > 1) {
            const uint32_t m = *(volatile uint32_t *)(N.meta + h);
            bool eq = (m >> 31) == kind;
            const volatile ulonglong2 *e = reinterpret_cast<const volatile ulonglong2 *>(N.key + 8 * h);
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const uint64_t a = e[i].x, b = e[i].y;
                eq = eq && a == k[2 * i] && b == k[2 * i + 1];
            }
            if (eq) {
                lod = m & 0x7FFFFFFFu;
                return id;
            }
        }
        h = (h + 1) & (kNodeCache - 1);
    }
    return 0;
}

__device__ __forceinline__ void nc_insert(const NodeCache &N, const uint64_t k[8], uint32_t kind, uint64_t id,
                                          uint32_t lod) {
    uint32_t h = nc_slot(k, kind);
#pragma unroll 1
    for (int p = 0; p < 4; ++p) {
        if (atomicCAS((unsigned long long *)(N.id + h), 0ull, 1ull) == 0ull) {
            ulonglong2 *e = reinterpret_cast<ulonglong2 *>(N.key + 8 * h);
#pragma unroll
            for (int i = 0; i < 4; ++i) e[i] = make_ulonglong2(k[2 * i], k[2 * i + 1]);
            N.meta[h] = (kind << 31) | lod;
            __threadfence_block();
            *(volatile uint64_t *)(N.id + h) = id;
            return;
        }
        h = (h + 1) & (kNodeCache - 1);
    }
}

// reduce_parent with the parent looked up first in the node cache by its 8 child ids.
__device__ __forceinline__ void reduce_parent_cached(const DevInterner &I, const NodeCache &N, bool active,
                                                     const uint64_t c[8], const uint32_t cv[8], uint64_t &out,
                                                     uint32_t &out_val) {
    uint32_t types = 0, mask = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        mask |= (c[k] != 0 ? 1u : 0u) << k;
        types |= (id_is_leaf(c[k]) ? 1u : 0u) << k;
    }
    bool same = types == 0xFF;
#pragma unroll
    for (int k = 1; k < 8; ++k) same = same && c[k] == c[0];
    const bool is_branch = active && mask != 0 && !same;
    uint32_t lod = 0;
    uint64_t id = is_branch ? nc_lookup(N, c, 1u, lod) : 0ull;
    const bool need = is_branch && id == 0;
    if (__any_sync(0xFFFFFFFFu, need)) {
        if (need) lod = calc_average8(cv);
        bool created;
        const uint64_t nid = warp_intern_branch_inl(I, need, c, types, mask, lod, &created);
        if (need) {
            id = nid;
            if (nid != EMPTY_ID) nc_insert(N, c, 1u, nid, lod);
        }
    }
    if (mask == 0) {
        out = EMPTY_ID;
        out_val = 0;
    } else if (same) {
        out = c[0];
        out_val = cv[0];
    } else {
        out = id;
        out_val = lod;
    }
}

// Nonzero-voxel mask of 8 voxels packed as in quad_groups (voxel j in bits [j*w, (j+1)*w) of lo:hi).
template <class T>
__device__ __forceinline__ uint32_t set_mask8(uint64_t lo, uint64_t hi) {
    if (sizeof(T) == 1) {
        const uint32_t a = __vcmpne4((uint32_t)lo, 0u) & 0x01010101u, b = __vcmpne4((uint32_t)(lo >> 32), 0u) & 0x01010101u;
        return ((a * 0x01020408u) >> 24) | (((b * 0x01020408u) >> 24) << 4);
    } else {
        auto nz2 = [](uint32_t x) {
            const uint32_t m = __vcmpne2(x, 0u) & 0x00010001u;
            return (m | (m >> 15)) & 3u;
        };
        return nz2((uint32_t)lo) | (nz2((uint32_t)(lo >> 32)) << 2) | (nz2((uint32_t)hi) << 4) |
               (nz2((uint32_t)(hi >> 32)) << 6);
    }
}

template <class T>
__device__ __forceinline__ void unpack8(uint64_t lo, uint64_t hi, uint32_t v[8]) {
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        if (sizeof(T) == 1)
            v[j] = (uint32_t)(lo >> (8 * j)) & 0xFFu;
        else
            v[j] = (uint32_t)((j < 4 ? lo : hi) >> (16 * (j & 3))) & 0xFFFFu;
    }
}

// ---- octant reduction with a device-wide quad memo ---------------------------------------------
//
// Terrain repeats: the 4096-chunk dune workload has 508k non-uniform quads (4^3 voxels) but only
// 4,468 distinct ones. A quad's node is a pure function of its voxels, so a call-wide memo in global
// memory (open addressing, 64-bit slots tag:32 | record+1, records = the quad's 16 row words, its node
// id and LOD value, published by a CAS after the record is written and fenced) replaces the 8-group
// reduction and the level-3 intern of every repeated quad by one slot load and one record load. Each
// lane keeps its two quads' probes in flight together. Misses take the bottom-group path
// (quad_groups) and insert the result; the memo only ever holds nodes created or found in this
// call (no release runs during a build), and inserts stop when its records run out.

template <class T>
struct QuadWord {
    using type = typename std::conditional<sizeof(T) == 1, uint32_t, uint64_t>::type;
};

// Row r = yy * 4 + zz of the quad at qbase in a tile of side S ([y][z][x], S voxels per row).
template <class T, int S>
__device__ __forceinline__ const typename QuadWord<T>::type *quad_row(const T *qbase, int r) {
    return reinterpret_cast<const typename QuadWord<T>::type *>(qbase + ((r >> 2) * S + (r & 3)) * S);
}

template <class T, int S = 16>
__device__ __forceinline__ void quad_rows(const T *qbase, typename QuadWord<T>::type w[16]) {
#pragma unroll
    for (int r = 0; r < 16; ++r) w[r] = *quad_row<T, S>(qbase, r);
}

// Bytes of one memo record: 16 row words of 4 voxels, then id (8 B) and LOD value, padded to whole
// 128-byte lines, so a record never shares a cache line with another.
__host__ __device__ constexpr size_t memo_stride(size_t voxel_bytes) {
    return ((16 * 4 * voxel_bytes + 16) + 127) & ~(size_t)127;
}

// A memo slot goes from 0 to its final value once and never changes again.
__device__ __forceinline__ uint64_t memo_slot_load(const unsigned long long *slots, uint32_t slot) {
    return ld_probe(reinterpret_cast<const uint64_t *>(slots) + slot);
}

// Record r's address; the record's content is 16 row words of 4 voxels.
template <class T>
__device__ __forceinline__ unsigned char *memo_rec(const OctArgs &a, uint32_t r) {
    return a.memo_recs + (size_t)r * memo_stride(sizeof(T));
}

template <class T, int S = 16>
__device__ __forceinline__ bool memo_match(const OctArgs &a, uint32_t r, const T *qbase, uint64_t &id, uint32_t &lod) {
    using W = typename QuadWord<T>::type;
    const unsigned char *rec = memo_rec<T>(a, r);
    const uint4 *rv = reinterpret_cast<const uint4 *>(rec);
    bool eq = true;
#pragma unroll
    for (int k = 0; k < 4 * (int)sizeof(T); ++k) {
        const uint4 x = __ldcg(rv + k);  // a published record never changes
        if (sizeof(T) == 1) {
            eq = eq && x.x == (uint32_t)*quad_row<T, S>(qbase, 4 * k) && x.y == (uint32_t)*quad_row<T, S>(qbase, 4 * k + 1) &&
                 x.z == (uint32_t)*quad_row<T, S>(qbase, 4 * k + 2) && x.w == (uint32_t)*quad_row<T, S>(qbase, 4 * k + 3);
        } else {
            const W a0 = *quad_row<T, S>(qbase, 2 * k), a1 = *quad_row<T, S>(qbase, 2 * k + 1);
            eq = eq && ((uint64_t)x.x | ((uint64_t)x.y << 32)) == (uint64_t)a0 &&
                 ((uint64_t)x.z | ((uint64_t)x.w << 32)) == (uint64_t)a1;
        }
    }
    if (!eq) return false;
    const uint4 tail = __ldcg(reinterpret_cast<const uint4 *>(rec + 16 * 4 * sizeof(T)));
    id = (uint64_t)tail.x | ((uint64_t)tail.y << 32);
    lod = tail.z;
    return true;
}

template <class T, int S = 16>
__device__ __forceinline__ void memo_insert(const OctArgs &a, uint32_t h1, uint32_t h2, const T *qbase, uint64_t id,
                                            uint32_t lod) {
    using W = typename QuadWord<T>::type;
    const uint32_t r = atomicAdd(a.memo_count, 1u);
    if (r >= a.memo_cap) return;
    unsigned char *rec = memo_rec<T>(a, r);
    W *dst = reinterpret_cast<W *>(rec);
#pragma unroll
    for (int k = 0; k < 16; ++k) dst[k] = *quad_row<T, S>(qbase, k);
    *reinterpret_cast<uint4 *>(rec + 16 * 4 * sizeof(T)) = make_uint4((uint32_t)id, (uint32_t)(id >> 32), lod, 0u);
    uint32_t slot = h1 & a.memo_mask;
    const unsigned long long v = ((unsigned long long)h2 << 32) | (r + 1u);
#pragma unroll 1
    for (int p = 0; p < 4; ++p) {  // the CAS publishes the record (release)
        if (atom_cas_acq_rel(a.memo_slots + slot, 0ull, v) == 0ull) return;
        slot = (slot + 1) & a.memo_mask;
    }
}

#ifndef VX_QUAD_DEFER
#define VX_QUAD_DEFER 1  // memo misses claim a pending record computed by a later kernel (else inline)
#endif
// q_vals marker of a quad whose node is still being computed: its q_ids entry is the memo record.
constexpr uint32_t kQuadPending = 0xFFFFFFFFu;
// Record tail id of a claimed record that lost its slot to an identical quad (never computed).
constexpr uint64_t kRecordDead = 1ull;

// Claims record r for a quad that missed the memo: the record gets the quad's rows and a pending
// tail (id 0), then is published by a release CAS into the first free slot from h1. A CAS that meets
// an identical quad published meanwhile follows that record instead (r is marked dead). Without a
// free slot within 4 steps r stays pending and reachable only from this quad. id / val receive the
// record to resolve (val = kQuadPending) or, for a record already computed, its node. Returns whether
// r must be computed (false: r is dead).
template <class T, int S>
__device__ __forceinline__ bool memo_claim(const OctArgs &a, uint32_t h1, uint32_t h2, const T *qbase, uint32_t r,
                                           uint64_t &id, uint32_t &val) {
    using W = typename QuadWord<T>::type;
    unsigned char *rec = memo_rec<T>(a, r);
    W *dst = reinterpret_cast<W *>(rec);
#pragma unroll
    for (int k = 0; k < 16; ++k) dst[k] = *quad_row<T, S>(qbase, k);
    uint4 *tail = reinterpret_cast<uint4 *>(rec + 16 * 4 * sizeof(T));
    *tail = make_uint4(0u, 0u, 0u, 0u);
    id = r;
    val = kQuadPending;
    uint32_t slot = h1 & a.memo_mask;
    const unsigned long long v = ((unsigned long long)h2 << 32) | (r + 1u);
#pragma unroll 1
    for (int p = 0; p < 4; ++p) {
        // release: the record is visible with the slot; acquire: so is a record published meanwhile
        const unsigned long long prev = atom_cas_acq_rel(a.memo_slots + slot, 0ull, v);
        if (prev == 0ull) return true;
        if ((uint32_t)(prev >> 32) == h2) {
            uint64_t oid;
            uint32_t olod;
            if (memo_match<T, S>(a, (uint32_t)prev - 1u, qbase, oid, olod)) {
                tail->x = (uint32_t)kRecordDead;
                if (oid == 0) {
                    id = (uint32_t)prev - 1u;
                } else {
                    id = oid;
                    val = olod;
                }
                return false;
            }
        }
        slot = (slot + 1) & a.memo_mask;
    }
    return true;  // no free slot within the probe limit: the record still names this quad and is computed
}

// The 8 bottom groups of one quad (4^3 voxels at qbase in a tile of side S) reduced as Phase 1 and
// Phase 2 do, then the quad's own node, which a non-uniform quad always is a branch. Warp-collective:
// every lane calls it; lanes with active == false only take part in the ballots.
template <class T, int S>
__device__ __forceinline__ void quad_groups(const DevInterner &I, const KeyCache &C, uint64_t *leaf_cache,
                                            const T *qbase, bool active, uint64_t &qid, uint32_t &qval,
                                            bool count = false) {
    const unsigned lane = threadIdx.x & 31u;
    const bool wide = sizeof(T) == 2;
    uint64_t c3[8];
    uint32_t cv3[8];
#pragma unroll 1
    for (int k = 0; k < 8; ++k) {
        const uint32_t gx = k & 1, gy = (k >> 1) & 1, gz = k >> 2;
        const T *g = qbase + ((2 * gy) * S + 2 * gz) * S + 2 * gx;
        uint64_t lo = 0, hi = 0;
        if (sizeof(T) == 1) {
            const uint32_t p0 = *reinterpret_cast<const uint16_t *>(g);
            const uint32_t p1 = *reinterpret_cast<const uint16_t *>(g + S * S);
            const uint32_t p2 = *reinterpret_cast<const uint16_t *>(g + S);
            const uint32_t p3 = *reinterpret_cast<const uint16_t *>(g + S * S + S);
            lo = (uint64_t)(p0 | (p1 << 16)) | ((uint64_t)(p2 | (p3 << 16)) << 32);
        } else {
            lo = (uint64_t)*reinterpret_cast<const uint32_t *>(g) |
                 ((uint64_t)*reinterpret_cast<const uint32_t *>(g + S * S) << 32);
            hi = (uint64_t)*reinterpret_cast<const uint32_t *>(g + S) |
                 ((uint64_t)*reinterpret_cast<const uint32_t *>(g + S * S + S) << 32);
        }
        const uint32_t set = set_mask8<T>(lo, hi);
        const uint32_t gv0 = (uint32_t)lo & (sizeof(T) == 1 ? 0xFFu : 0xFFFFu);
        const bool guni = sizeof(T) == 1 ? lo == (uint64_t)gv0 * 0x0101010101010101ull
                                         : (lo == hi && lo == (uint64_t)gv0 * 0x0001000100010001ull);
        const bool is_branch = active && set != 0 && !(guni && set == 0xFFu);
        uint32_t lod = 0;
        uint64_t id = is_branch ? kc_lookup(C, lo, hi, &lod) : 0ull;
        const bool need = is_branch && id == 0;
        const unsigned bm = __ballot_sync(0xFFFFFFFFu, need);
        if (bm) {
            uint32_t v[8];
            unpack8<T>(lo, hi, v);
            if (need) lod = calc_average8(v);
            unsigned grp = __match_any_sync(0xFFFFFFFFu, need ? lo : ~(uint64_t)lane);
            if (wide) grp &= __match_any_sync(0xFFFFFFFFu, need ? hi : ~(uint64_t)lane);
            grp &= bm;
            const int leader = need ? __ffs(grp) - 1 : (int)lane;
            const bool lead = need && leader == (int)lane;
            uint64_t c[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) c[j] = (lead && v[j]) ? leaf_of<T>(I, leaf_cache, v[j]) : 0ull;
            bool created;
            uint64_t nid = warp_intern_branch(I, lead, c, set, set, lod, &created);
            if (count && created) count_created(I, nullptr, nid);
            nid = __shfl_sync(0xFFFFFFFFu, nid, leader);
            if (lead && nid != EMPTY_ID) kc_insert(C, lo, hi, nid, lod);
            if (need) id = nid;
        }
        if (set == 0) {
            c3[k] = EMPTY_ID;
            cv3[k] = 0;
        } else if (!is_branch) {
            c3[k] = active ? leaf_of<T>(I, leaf_cache, gv0) : 0ull;
            cv3[k] = gv0;
        } else {
            c3[k] = id;
            cv3[k] = lod;
        }
    }
    bool qc = false;
    reduce_parent(I, active, c3, cv3, qid, qval, &qc);
    if (count && qc) count_created(I, nullptr, qid);
}

template <class T>
__device__ __forceinline__ void reduce_tile16(const DevInterner &I, const OctArgs &a, const T *tile,
                                                 const KeyCache &C, const NodeCache &N, uint64_t *leaf_cache,
                                                 uint64_t &oct_id, uint32_t &oct_val) {
    using W = typename QuadWord<T>::type;
    const unsigned lane = threadIdx.x & 31u;
    const bool memo = a.memo_slots != nullptr;
    const T *qb[2];
    bool uni[2];
    uint32_t h1[2], h2[2];
    uint64_t qid[2];
    uint32_t qval[2];
#pragma unroll
    for (int q = 0; q < 2; ++q) {
        const uint32_t p = lane + 32 * q;
        const uint32_t qx = compact3(p), qy = compact3(p >> 1), qz = compact3(p >> 2);
        qb[q] = tile + ((4 * qy) * 16 + 4 * qz) * 16 + 4 * qx;
        W w[16];
        quad_rows<T>(qb[q], w);
        const uint32_t v0 = (uint32_t)(w[0] & (sizeof(T) == 1 ? 0xFFu : 0xFFFFu));
        const W splat = sizeof(T) == 1 ? (W)(v0 * 0x01010101u) : (W)((uint64_t)v0 * 0x0001000100010001ull);
        bool u = true;
        uint32_t x = 0x9E3779B9u, y = 0x7F4A7C15u;
#pragma unroll
        for (int r = 0; r < 16; ++r) {
            u = u && w[r] == splat;
            x = x * 0x01000193u + (uint32_t)w[r];
            y = (y ^ (uint32_t)w[r]) * 0x85EBCA6Bu;
            if (sizeof(T) == 2) {
                x = x * 0x01000193u + (uint32_t)((uint64_t)w[r] >> 32);
                y = (y ^ (uint32_t)((uint64_t)w[r] >> 32)) * 0x85EBCA6Bu;
            }
        }
        x ^= x >> 15;
        x *= 0x2C1B3C6Du;
        x ^= x >> 12;
        y ^= y >> 16;
        uni[q] = u;
        h1[q] = x;
        h2[q] = y;
        qid[q] = 0;
        qval[q] = v0;
        if (u) qid[q] = v0 ? leaf_of<T>(I, leaf_cache, v0) : EMPTY_ID;
    }
    // memo probes, both quads in flight
    bool look[2];
    uint32_t slot[2];
    unsigned long long sv[2];
#pragma unroll
    for (int q = 0; q < 2; ++q) {
        look[q] = memo && !uni[q];
        slot[q] = h1[q] & a.memo_mask;
        sv[q] = look[q] ? memo_slot_load(a.memo_slots, slot[q]) : 0ull;
    }
#pragma unroll 1
    for (int step = 0; step < 4 && (look[0] || look[1]); ++step) {
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            if (!look[q]) continue;
            if (sv[q] == 0ull) {
                look[q] = false;  // empty slot: not in the memo
            } else if ((uint32_t)(sv[q] >> 32) == h2[q] &&
                       memo_match<T>(a, (uint32_t)sv[q] - 1u, qb[q], qid[q], qval[q])) {
                look[q] = false;
            } else if (step == 3) {
                look[q] = false;
            } else {
                slot[q] = (slot[q] + 1) & a.memo_mask;
                sv[q] = memo_slot_load(a.memo_slots, slot[q]);
            }
        }
    }
    uint64_t l3[2];
    uint32_t l3v[2];
#pragma unroll 1
    for (int q = 0; q < 2; ++q) {
        const bool active = !uni[q] && qid[q] == 0;
        if (__any_sync(0xFFFFFFFFu, active)) {
            uint64_t pid;
            uint32_t pval;
            quad_groups<T, 16>(I, C, leaf_cache, qb[q], active, pid, pval);
            if (active) {
                qid[q] = pid;
                qval[q] = pval;
                if (memo && pid != EMPTY_ID) memo_insert<T>(a, h1[q], h2[q], qb[q], pid, pval);
            }
        }
        l3[q] = qid[q];
        l3v[q] = qval[q];
    }
    // level 2: lane q < 8 takes quads 8q .. 8q+7 (pass q >> 2)
    uint64_t c2[8];
    uint32_t cv2[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const int src = (8 * lane + j) & 31;
        const uint64_t a0 = __shfl_sync(0xFFFFFFFFu, l3[0], src), a1 = __shfl_sync(0xFFFFFFFFu, l3[1], src);
        const uint32_t b0 = __shfl_sync(0xFFFFFFFFu, l3v[0], src), b1 = __shfl_sync(0xFFFFFFFFu, l3v[1], src);
        c2[j] = lane < 8 ? (lane < 4 ? a0 : a1) : 0ull;
        cv2[j] = lane < 4 ? b0 : b1;
    }
    uint64_t l2;
    uint32_t l2v;
    reduce_parent_cached(I, N, lane < 8, c2, cv2, l2, l2v);
    uint64_t c1[8];
    uint32_t cv1[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        c1[j] = __shfl_sync(0xFFFFFFFFu, l2, j);
        cv1[j] = __shfl_sync(0xFFFFFFFFu, l2v, j);
    }
    uint64_t l1;
    uint32_t l1v;
    reduce_parent_cached(I, N, lane == 0, c1, cv1, l1, l1v);
    oct_id = __shfl_sync(0xFFFFFFFFu, l1, 0);
    oct_val = __shfl_sync(0xFFFFFFFFu, l1v, 0);
}

__device__ __forceinline__ void tma_load_octant(void *dst, const CUtensorMap *tmap, int x, int z, int y, int c,
                                                uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, "
        "%5}], [%6];" ::"r"(smem_addr(dst)),
        "l"(tmap), "r"(x), "r"(z), "r"(y), "r"(c), "r"(smem_addr(bar))
        : "memory");
}

#ifdef VX_OCT_MAXNREG
#define VX_OCT_BOUNDS __maxnreg__(VX_OCT_MAXNREG)
#else
#define VX_OCT_BOUNDS __launch_bounds__(kThreads)
#endif
template <class T>
__global__ void VX_OCT_BOUNDS dense_octants_kernel(DevInterner I, OctArgs a,
                                                                 const __grid_constant__ CUtensorMap tmap) {
    extern __shared__ __align__(128) unsigned char smem[];
    constexpr uint32_t TILE = 4096 * sizeof(T);
    const unsigned tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    T *tiles = reinterpret_cast<T *>(smem + warp * kOctTiles * TILE);
    uint64_t *kc = reinterpret_cast<uint64_t *>(smem + kOctWarps * kOctTiles * TILE);
    uint64_t *leaf_cache = kc + 3 * kKeyCache;
    uint64_t *bars = leaf_cache + 256 + warp * 2;
    uint64_t *nc = leaf_cache + 256 + 2 * kOctWarps;
    uint32_t *u32s = reinterpret_cast<uint32_t *>(nc + 9 * kNodeCache);
    KeyCache C{kc, kc + kKeyCache, kc + 2 * kKeyCache, u32s};
    NodeCache N{nc, nc + 8 * kNodeCache, u32s + kKeyCache};

    for (unsigned k = tid; k < kKeyCache; k += blockDim.x) C.id[k] = 0;
    for (unsigned k = tid; k < kNodeCache; k += blockDim.x) N.id[k] = 0;
    if (sizeof(T) == 1)
        leaf_cache_warm(I, leaf_cache, tid);
    if (lane == 0) {
        mbar_init(bars, 1);
        mbar_init(bars + 1, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();

    const int d = a.depth;
    const int ob = 3 * (d - 4);  // octant-index bits inside a chunk
    const uint64_t n_oct = (uint64_t)a.n_chunks << ob;
    const uint64_t total = (uint64_t)gridDim.x * kOctWarps;
    uint64_t o = (uint64_t)blockIdx.x * kOctWarps + warp;
    auto issue = [&](uint64_t oo, int buf) {
        const uint32_t c = (uint32_t)(oo >> ob);
        const uint32_t q = (uint32_t)(oo & ((1ull << ob) - 1));
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        mbar_expect_tx(bars + buf, TILE);
        tma_load_octant(tiles + buf * 4096, &tmap, (int)(compact3(q) * 16), (int)(compact3(q >> 2) * 16),
                        (int)(compact3(q >> 1) * 16), (int)c, bars + buf);
    };
    uint32_t ph0 = 0, ph1 = 0;
    int buf = 0;
    if (o < n_oct && lane == 0) issue(o, 0);
    for (; o < n_oct; o += total) {
        const uint64_t nx = o + total;
        if (kOctTiles == 2 && nx < n_oct && lane == 0) issue(nx, buf ^ 1);
        uint32_t &ph = buf ? ph1 : ph0;
        bool ok = false;
        for (uint32_t spin = 0; spin < SPIN_LIMIT; ++spin)
            if ((ok = mbar_try_wait(bars + buf, ph))) break;
        if (__any_sync(0xFFFFFFFFu, !ok)) {  // give up: drain this warp's copies, report, leave
            if (lane == 0) set_error(I, ERR_TIMEOUT, 25);
            for (int b = 0; b < kOctTiles; ++b)
                for (uint32_t spin = 0; spin < SPIN_LIMIT && !mbar_try_wait(bars + b, b ? ph1 : ph0); ++spin) {
                }
            return;
        }
        ph ^= 1u;
        const uint32_t c = (uint32_t)(o >> ob);
        uint64_t q = o & ((1ull << ob) - 1);
        const uint32_t tree = a.trees[c];
        const bool bad = tree >= I.tree_cap || I.depths[tree] != d || I.roots[tree] != EMPTY_ID;
        if (bad) {
            if (lane == 0) set_error(I, ERR_INVALID, 26);
            if (kOctTiles == 1 && nx < n_oct && lane == 0) issue(nx, 0);
            if (kOctTiles == 2) buf ^= 1;
            continue;
        }
        uint64_t node;
        uint32_t val;
        reduce_tile16<T>(I, a, tiles + buf * 4096, C, N, leaf_cache, node, val);
        __syncwarp();
        if (kOctTiles == 1 && nx < n_oct && lane == 0) issue(nx, 0);  // single buffer: load after use
        // climb while this warp brings the last child of a parent
        for (int k = d - 4;; --k) {
            if (k == 0) {
                if (lane == 0) {
                    if (node != EMPTY_ID) {
                        I.roots[tree] = node;
                        atomicAdd(I.refcount + id_index(node), 1u);
                    }
                    if (a.changed) a.changed[c] = node != EMPTY_ID;
                }
                break;
            }
            const uint64_t gi = a.lvl_off[k] + ((uint64_t)c << (3 * k)) + q;
            if (lane == 0) {
                a.ids[gi] = node;
                a.vals[gi] = val;
            }
            __threadfence();
            uint32_t arrived = 0;
            if (lane == 0)
                arrived = atomicAdd(a.cnt + a.cnt_off[k - 1] + ((uint64_t)c << (3 * (k - 1))) + (q >> 3), 1u);
            arrived = __shfl_sync(0xFFFFFFFFu, arrived, 0);
            if (arrived != 7) break;
            __threadfence();
            const uint64_t sb = a.lvl_off[k] + ((uint64_t)c << (3 * k)) + (q & ~7ull);
            const uint64_t sid = lane < 8 ? ld_cg(a.ids + sb + lane) : 0ull;
            const uint32_t sval = lane < 8 ? __ldcg(a.vals + sb + lane) : 0u;
            uint64_t ch[8];
            uint32_t cv[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                ch[j] = __shfl_sync(0xFFFFFFFFu, sid, j);
                cv[j] = __shfl_sync(0xFFFFFFFFu, sval, j);
            }
            reduce_parent_cached(I, N, lane == 0, ch, cv, node, val);
            node = __shfl_sync(0xFFFFFFFFu, node, 0);
            val = __shfl_sync(0xFFFFFFFFu, val, 0);
            q >>= 3;
        }
        if (kOctTiles == 2) buf ^= 1;
    }
}

// ---- 32^3 blocks, one CTA each, level-synchronous phases -------------------------------------------
//
// For chunk depths >= 5. A CTA takes 32^3 blocks in turn (4-D TMA tensor copy of the block into one
// shared tile, mbarrier completion, bounded wait). Phase 1: each of the 256 threads takes two of the
// block's 512 quads (4^3), tests uniformity on row words, and probes the device-wide quad memo, so
// all 512 probes of the block are in flight together; memo misses run the bottom-group path
// (quad_groups) warp by warp and are inserted. Quad results go to shared memory in Morton order and
// the tile is released: the next block's copy starts while the upper levels run. Phase 2: 64 threads
// reduce the 8^3 nodes; phase 3: warp 0 reduces the 8 16^3 nodes and the block root (shared cache of
// parents by child ids first, then the global table), and climbs above the block with per-parent
// arrival counters like the octant kernel.
#ifndef VX_DENSE_CTA32
#define VX_DENSE_CTA32 1
#endif
constexpr int kCtaThreads = 256;

template <class T>
struct Cta32Smem {
    static constexpr size_t tile = 32768 * sizeof(T);
    static constexpr size_t qid = tile;                            // 512 u64: quad nodes, Morton order
    static constexpr size_t kc = qid + 512 * 8;                    // 3 * kKeyCache u64
    static constexpr size_t leaf = kc + 3 * (size_t)kKeyCache * 8;  // 256 u64
    static constexpr size_t nc = leaf + 256 * 8;                    // 9 * kNodeCache u64
    static constexpr size_t bar = nc + 9 * (size_t)kNodeCache * 8;  // 2 u64
    static constexpr size_t lid = bar + 16;                         // 72 u64: level-2 nodes, then level 1
    static constexpr size_t qval = lid + 72 * 8;                    // 512 u32
    static constexpr size_t lval = qval + 512 * 4;                  // 72 u32
    static constexpr size_t kcval = lval + 72 * 4;                  // kKeyCache u32
    static constexpr size_t ncmeta = kcval + (size_t)kKeyCache * 4;  // kNodeCache u32
    static constexpr size_t total = ncmeta + (size_t)kNodeCache * 4;
};

__device__ __forceinline__ uint32_t spread3b(uint32_t v) { return (v & 1u) | ((v & 2u) << 2) | ((v & 4u) << 4); }

__device__ __forceinline__ void tma_load_block32(void *dst, const CUtensorMap *tmap, int x, int z, int y, int c,
                                                 uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, "
        "%5}], [%6];" ::"r"(smem_addr(dst)),
        "l"(tmap), "r"(x), "r"(z), "r"(y), "r"(c), "r"(smem_addr(bar))
        : "memory");
}

template <class T>
__global__ void __launch_bounds__(kCtaThreads) dense_cta32_kernel(DevInterner I, OctArgs a,
                                                                 const __grid_constant__ CUtensorMap tmap) {
    using L = Cta32Smem<T>;
    using W = typename QuadWord<T>::type;
    extern __shared__ __align__(128) unsigned char smem[];
    const unsigned tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    T *tile = reinterpret_cast<T *>(smem);
    uint64_t *qid_s = reinterpret_cast<uint64_t *>(smem + L::qid);
    uint64_t *kc = reinterpret_cast<uint64_t *>(smem + L::kc);
    uint64_t *leaf_cache = reinterpret_cast<uint64_t *>(smem + L::leaf);
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem + L::bar);
    uint64_t *lid = reinterpret_cast<uint64_t *>(smem + L::lid);
    uint32_t *qval_s = reinterpret_cast<uint32_t *>(smem + L::qval);
    uint32_t *lval = reinterpret_cast<uint32_t *>(smem + L::lval);
    KeyCache C{kc, kc + kKeyCache, kc + 2 * kKeyCache, reinterpret_cast<uint32_t *>(smem + L::kcval)};
    uint64_t *nc = reinterpret_cast<uint64_t *>(smem + L::nc);
    NodeCache N{nc, nc + 8 * kNodeCache, reinterpret_cast<uint32_t *>(smem + L::ncmeta)};
    for (unsigned k = tid; k < kKeyCache; k += blockDim.x) C.id[k] = 0;
    for (unsigned k = tid; k < kNodeCache; k += blockDim.x) N.id[k] = 0;
    if (sizeof(T) == 1)
        leaf_cache_warm(I, leaf_cache, tid);
    if (tid == 0) {
        mbar_init(bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();

    const int d = a.depth;
    const int bb = 3 * (d - 5);  // block-index bits inside a chunk
    const uint64_t n_blk = (uint64_t)a.n_chunks << bb;
    const bool memo = a.memo_slots != nullptr;
    auto issue = [&](uint64_t b) {
        const uint32_t c = (uint32_t)(b >> bb);
        const uint32_t q = (uint32_t)(b & ((1ull << bb) - 1));
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        mbar_expect_tx(bar, (uint32_t)L::tile);
        tma_load_block32(tile, &tmap, (int)(compact3(q) * 32), (int)(compact3(q >> 2) * 32),
                         (int)(compact3(q >> 1) * 32), (int)c, bar);
    };
    uint32_t phase = 0;
    uint64_t blk = blockIdx.x;
    if (tid == 0 && blk < n_blk) issue(blk);
    for (; blk < n_blk; blk += gridDim.x) {
        const uint64_t nxt = blk + gridDim.x;
        bool ok = false;
        for (uint32_t spin = 0; spin < SPIN_LIMIT; ++spin)
            if ((ok = mbar_try_wait(bar, phase))) break;
        if (__syncthreads_or(!ok)) {  // give up together; drain the copy first
            if (tid == 0) set_error(I, ERR_TIMEOUT, 27);
            for (uint32_t spin = 0; spin < SPIN_LIMIT && !mbar_try_wait(bar, phase); ++spin) {
            }
            return;
        }
        phase ^= 1u;
        const uint32_t c = (uint32_t)(blk >> bb);
        uint64_t q = blk & ((1ull << bb) - 1);
        const uint32_t tree = a.trees[c];
        if (tree >= I.tree_cap || I.depths[tree] != d || I.roots[tree] != EMPTY_ID) {  // the same answer in every thread
            if (tid == 0) {
                set_error(I, ERR_INVALID, 28);
                if (nxt < n_blk) issue(nxt);
            }
            __syncthreads();
            continue;
        }

        // ---- phase 1: quads (qx = lane & 7, qz = lane >> 3 (+4), qy = warp) ----
        const T *qb[2];
        uint32_t qm[2], h1[2], h2[2];
        bool uni[2];
        uint64_t qidv[2];
        uint32_t qvalv[2];
#pragma unroll
        for (int p = 0; p < 2; ++p) {
            const uint32_t qx = lane & 7u, qz = (lane >> 3) + 4u * p, qy = warp;
            qm[p] = spread3b(qx) | (spread3b(qy) << 1) | (spread3b(qz) << 2);
            qb[p] = tile + ((4 * qy) * 32 + 4 * qz) * 32 + 4 * qx;
            W w[16];
            quad_rows<T, 32>(qb[p], w);
            const uint32_t v0 = (uint32_t)(w[0] & (sizeof(T) == 1 ? 0xFFu : 0xFFFFu));
            const W splat = sizeof(T) == 1 ? (W)(v0 * 0x01010101u) : (W)((uint64_t)v0 * 0x0001000100010001ull);
            bool u = true;
            uint32_t x = 0x9E3779B9u, y = 0x7F4A7C15u;
#pragma unroll
            for (int r = 0; r < 16; ++r) {
                u = u && w[r] == splat;
                x = x * 0x01000193u + (uint32_t)w[r];
                y = (y ^ (uint32_t)w[r]) * 0x85EBCA6Bu;
                if (sizeof(T) == 2) {
                    x = x * 0x01000193u + (uint32_t)((uint64_t)w[r] >> 32);
                    y = (y ^ (uint32_t)((uint64_t)w[r] >> 32)) * 0x85EBCA6Bu;
                }
            }
            x ^= x >> 15;
            x *= 0x2C1B3C6Du;
            x ^= x >> 12;
            y ^= y >> 16;
            uni[p] = u;
            h1[p] = x;
            h2[p] = y;
            qidv[p] = 0;
            qvalv[p] = v0;
            if (u) qidv[p] = v0 ? leaf_of<T>(I, leaf_cache, v0) : EMPTY_ID;
        }
        {  // memo probes, both quads in flight
            bool look[2];
            uint32_t slot[2];
            unsigned long long sv[2];
#pragma unroll
            for (int p = 0; p < 2; ++p) {
                look[p] = memo && !uni[p];
                slot[p] = h1[p] & a.memo_mask;
                sv[p] = look[p] ? memo_slot_load(a.memo_slots, slot[p]) : 0ull;
            }
#pragma unroll 1
            for (int step = 0; step < 4 && (look[0] || look[1]); ++step) {
#pragma unroll
                for (int p = 0; p < 2; ++p) {
                    if (!look[p]) continue;
                    if (sv[p] == 0ull) {
                        look[p] = false;
                    } else if ((uint32_t)(sv[p] >> 32) == h2[p] &&
                               memo_match<T, 32>(a, (uint32_t)sv[p] - 1u, qb[p], qidv[p], qvalv[p])) {
                        look[p] = false;
                    } else if (step == 3) {
                        look[p] = false;
                    } else {
                        slot[p] = (slot[p] + 1) & a.memo_mask;
                        sv[p] = memo_slot_load(a.memo_slots, slot[p]);
                    }
                }
            }
        }
#pragma unroll 1
        for (int p = 0; p < 2; ++p) {
            const bool active = !uni[p] && qidv[p] == 0;
            if (__any_sync(0xFFFFFFFFu, active)) {
                uint64_t pid;
                uint32_t pval;
                quad_groups<T, 32>(I, C, leaf_cache, qb[p], active, pid, pval);
                if (active) {
                    qidv[p] = pid;
                    qvalv[p] = pval;
                    if (memo && pid != EMPTY_ID) memo_insert<T, 32>(a, h1[p], h2[p], qb[p], pid, pval);
                }
            }
            qid_s[qm[p]] = qidv[p];
            qval_s[qm[p]] = qvalv[p];
        }
        __syncthreads();
        if (tid == 0 && nxt < n_blk) issue(nxt);  // the tile is free: the next block's copy overlaps phases 2-3

        // ---- phase 2: the 64 nodes of 8^3 voxels ----
        if (warp < 2) {
            uint64_t ch[8];
            uint32_t cv[8];
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                ch[k] = qid_s[8 * tid + k];
                cv[k] = qval_s[8 * tid + k];
            }
            uint64_t o;
            uint32_t ov;
            reduce_parent_cached(I, N, true, ch, cv, o, ov);
            lid[tid] = o;
            lval[tid] = ov;
        }
        __syncthreads();
        // ---- phase 3 (warp 0): the 8 nodes of 16^3 voxels, the block root, then the climb ----
        if (warp == 0) {
            uint64_t ch[8];
            uint32_t cv[8];
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                ch[k] = lane < 8 ? lid[8 * lane + k] : 0ull;
                cv[k] = lane < 8 ? lval[8 * lane + k] : 0u;
            }
            uint64_t o1;
            uint32_t v1;
            reduce_parent_cached(I, N, lane < 8, ch, cv, o1, v1);
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                ch[k] = __shfl_sync(0xFFFFFFFFu, o1, k);
                cv[k] = __shfl_sync(0xFFFFFFFFu, v1, k);
            }
            uint64_t node;
            uint32_t val;
            reduce_parent_cached(I, N, lane == 0, ch, cv, node, val);
            node = __shfl_sync(0xFFFFFFFFu, node, 0);
            val = __shfl_sync(0xFFFFFFFFu, val, 0);
            for (int k = d - 5;; --k) {
                if (k == 0) {
                    if (lane == 0) {
                        if (node != EMPTY_ID) {
                            I.roots[tree] = node;
                            atomicAdd(I.refcount + id_index(node), 1u);
                        }
                        if (a.changed) a.changed[c] = node != EMPTY_ID;
                    }
                    break;
                }
                const uint64_t gi = a.lvl_off[k] + ((uint64_t)c << (3 * k)) + q;
                if (lane == 0) {
                    a.ids[gi] = node;
                    a.vals[gi] = val;
                }
                __threadfence();
                uint32_t arrived = 0;
                if (lane == 0)
                    arrived = atomicAdd(a.cnt + a.cnt_off[k - 1] + ((uint64_t)c << (3 * (k - 1))) + (q >> 3), 1u);
                arrived = __shfl_sync(0xFFFFFFFFu, arrived, 0);
                if (arrived != 7) break;
                __threadfence();
                const uint64_t sb = a.lvl_off[k] + ((uint64_t)c << (3 * k)) + (q & ~7ull);
                const uint64_t sid = lane < 8 ? ld_cg(a.ids + sb + lane) : 0ull;
                const uint32_t sval = lane < 8 ? __ldcg(a.vals + sb + lane) : 0u;
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    ch[j] = __shfl_sync(0xFFFFFFFFu, sid, j);
                    cv[j] = __shfl_sync(0xFFFFFFFFu, sval, j);
                }
                reduce_parent_cached(I, N, lane == 0, ch, cv, node, val);
                node = __shfl_sync(0xFFFFFFFFu, node, 0);
                val = __shfl_sync(0xFFFFFFFFu, val, 0);
                q >>= 3;
            }
        }
        __syncthreads();  // shared quad and level arrays are reused by the next block
    }
}

// ---- quads of 16^3 octants, then one pass per level above them ------------------------------------
//
// The upper levels of a chunk are a chain of dependent probes (8^3 nodes, then 16^3, then the root),
// which leaves most of a CTA idle when one CTA walks it per block. Here the quad kernel only reduces
// quads (uniformity on row words, the device-wide quad memo, the bottom-group path on misses) and
// writes them to global memory in per-chunk Morton order; every level above is then one
// fresh_level_kernel pass over all chunks, one parent per thread, so the probes of a whole level are
// in flight together.
#ifndef VX_QUAD_DEDUP
#define VX_QUAD_DEDUP 1  // identical quads of a warp are looked up once
#endif
#ifndef VX_LEVEL_DEDUP
#define VX_LEVEL_DEDUP 1  // identical parents of a warp probe the table once
#endif

template <class T, int S>
__device__ __forceinline__ bool rows_equal(const T *a, const T *b) {
    bool eq = true;
#pragma unroll
    for (int r = 0; r < 16; ++r) eq = eq && *quad_row<T, S>(a, r) == *quad_row<T, S>(b, r);
    return eq;
}

// The 64 quads of the 16^3 octant at `tile` ([y][z][x]) reduced by one warp, two per lane: uniformity
// on row words, the quad memo, the bottom-group path on misses; results to oid/oval in Morton order.
template <class T>
__device__ __forceinline__ void quads_of_tile(const DevInterner &I, const OctArgs &a, const T *tile,
                                              const KeyCache &C, uint64_t *leaf_cache, uint64_t *oid,
                                              uint32_t *oval) {
    constexpr int S = 16;
    using W = typename QuadWord<T>::type;
    const unsigned lane = threadIdx.x & 31u;
    const bool memo = a.memo_slots != nullptr;
    const T *qb[2];
    uint32_t qm[2], h1[2], h2[2];
    bool uni[2];
    uint64_t qidv[2];
    uint32_t qvalv[2];
#pragma unroll
    for (int p = 0; p < 2; ++p) {
        const uint32_t q = lane + 32u * p, qx = compact3(q), qy = compact3(q >> 1), qz = compact3(q >> 2);
        qm[p] = q;
        qb[p] = tile + ((4 * qy) * 16 + 4 * qz) * 16 + 4 * qx;
        W w[16];
        quad_rows<T, S>(qb[p], w);
        const uint32_t v0 = (uint32_t)(w[0] & (sizeof(T) == 1 ? 0xFFu : 0xFFFFu));
        const W splat = sizeof(T) == 1 ? (W)(v0 * 0x01010101u) : (W)((uint64_t)v0 * 0x0001000100010001ull);
        bool u = true;
        uint32_t x = 0x9E3779B9u, y = 0x7F4A7C15u;
#pragma unroll
        for (int r = 0; r < 16; ++r) {
            u = u && w[r] == splat;
            x = x * 0x01000193u + (uint32_t)w[r];
            y = (y ^ (uint32_t)w[r]) * 0x85EBCA6Bu;
            if (sizeof(T) == 2) {
                x = x * 0x01000193u + (uint32_t)((uint64_t)w[r] >> 32);
                y = (y ^ (uint32_t)((uint64_t)w[r] >> 32)) * 0x85EBCA6Bu;
            }
        }
        x ^= x >> 15;
        x *= 0x2C1B3C6Du;
        x ^= x >> 12;
        y ^= y >> 16;
        uni[p] = u;
        h1[p] = x;
        h2[p] = y;
        qidv[p] = 0;
        qvalv[p] = v0;
        if (u) qidv[p] = v0 ? leaf_of<T>(I, leaf_cache, v0) : EMPTY_ID;
    }
    // identical quads of the warp: only the lowest lane of each set looks them up
    int leader[2];
    bool follow[2];
#pragma unroll
    for (int p = 0; p < 2; ++p) {
        const uint64_t hk = (uni[p] || !VX_QUAD_DEDUP) ? (~0ull - lane) : (((uint64_t)h2[p] << 32) | h1[p]);
        const unsigned peers = __match_any_sync(0xFFFFFFFFu, hk);
        leader[p] = __ffs(peers) - 1;
        const T *lq = reinterpret_cast<const T *>(
            __shfl_sync(0xFFFFFFFFu, reinterpret_cast<unsigned long long>(qb[p]), leader[p]));
        follow[p] = !uni[p] && leader[p] != (int)lane && rows_equal<T, S>(qb[p], lq);
    }
    // have[p]: the quad's result is known (uniform, a memo hit, or a pending record of this build)
    bool have[2] = {uni[0], uni[1]};
    {  // memo probes, both quads in flight
        bool look[2];
        uint32_t slot[2];
        unsigned long long sv[2];
#pragma unroll
        for (int p = 0; p < 2; ++p) {
            look[p] = memo && !uni[p] && !follow[p];
            slot[p] = h1[p] & a.memo_mask;
            sv[p] = look[p] ? memo_slot_load(a.memo_slots, slot[p]) : 0ull;
        }
#pragma unroll 1
        for (int step = 0; step < 4 && (look[0] || look[1]); ++step) {
#pragma unroll
            for (int p = 0; p < 2; ++p) {
                if (!look[p]) continue;
                if (sv[p] == 0ull) {
                    look[p] = false;
                } else if ((uint32_t)(sv[p] >> 32) == h2[p] &&
                           memo_match<T, S>(a, (uint32_t)sv[p] - 1u, qb[p], qidv[p], qvalv[p])) {
                    look[p] = false;
                    have[p] = true;
                    if (qidv[p] == 0) {  // pending: computed after this kernel by dense_memo_compute_kernel
                        qidv[p] = (uint32_t)sv[p] - 1u;
                        qvalv[p] = kQuadPending;
                    }
                } else if (step == 3) {
                    look[p] = false;
                } else {
                    slot[p] = (slot[p] + 1) & a.memo_mask;
                    sv[p] = memo_slot_load(a.memo_slots, slot[p]);
                }
            }
        }
    }
    if (memo && VX_QUAD_DEFER) {  // misses claim a pending record: one record range per warp
        const bool cl0 = !uni[0] && !follow[0] && !have[0], cl1 = !uni[1] && !follow[1] && !have[1];
        const unsigned b0 = __ballot_sync(0xFFFFFFFFu, cl0), b1 = __ballot_sync(0xFFFFFFFFu, cl1);
        if (b0 | b1) {
            uint32_t base = 0;
            if (lane == 0) base = atomicAdd(a.memo_count, (unsigned)(__popc(b0) + __popc(b1)));
            base = __shfl_sync(0xFFFFFFFFu, base, 0);
            const unsigned lt = (1u << lane) - 1u;
            const uint32_t r0 = base + __popc(b0 & lt), r1 = base + __popc(b0) + __popc(b1 & lt);
            bool live[2] = {false, false};
#pragma unroll
            for (int p = 0; p < 2; ++p) {
                const bool cl = p ? cl1 : cl0;
                const uint32_t r = p ? r1 : r0;
                if (cl && r < a.memo_cap) {
                    live[p] = memo_claim<T, S>(a, h1[p], h2[p], qb[p], r, qidv[p], qvalv[p]);
                    have[p] = true;
                }
            }
            if (a.live) {  // the records to compute, listed once per warp (dead claims stay off the list)
                const unsigned l0 = __ballot_sync(0xFFFFFFFFu, live[0]), l1 = __ballot_sync(0xFFFFFFFFu, live[1]);
                if (l0 | l1) {
                    uint32_t lb = 0;
                    if (lane == 0) lb = atomicAdd(a.live_count, (unsigned)(__popc(l0) + __popc(l1)));
                    lb = __shfl_sync(0xFFFFFFFFu, lb, 0);
                    if (live[0]) a.live[lb + __popc(l0 & lt)] = r0;
                    if (live[1]) a.live[lb + __popc(l0) + __popc(l1 & lt)] = r1;
                }
            }
        }
    }
#pragma unroll 1
    for (int p = 0; p < 2; ++p) {
        // computed here only without a memo, with deferral off, or once the memo's records run out
        const bool active = !uni[p] && !follow[p] && !have[p];
        if (__any_sync(0xFFFFFFFFu, active)) {
            uint64_t pid;
            uint32_t pval;
            quad_groups<T, S>(I, C, leaf_cache, qb[p], active, pid, pval, a.count_refs != 0);
            if (active) {
                qidv[p] = pid;
                qvalv[p] = pval;
                if (memo && !VX_QUAD_DEFER && pid != EMPTY_ID) memo_insert<T, S>(a, h1[p], h2[p], qb[p], pid, pval);
            }
        }
        const uint64_t lid = __shfl_sync(0xFFFFFFFFu, qidv[p], leader[p]);
        const uint32_t lval = __shfl_sync(0xFFFFFFFFu, qvalv[p], leader[p]);
        if (follow[p]) {
            qidv[p] = lid;
            qvalv[p] = lval;
        }
        oid[qm[p]] = qidv[p];
        oval[qm[p]] = qvalv[p];
    }
}

// ---- quads of 16^3 octants, one warp each, with no coupling between warps ----------------------------
// Each warp streams its own octants through its own tile(s) (4-D TMA box of 16^3; the copy of the next
// octant is issued as soon as a tile has been reduced), so a warp slowed by memo misses holds back
// nobody.
#ifndef VX_Q16_TILES
#define VX_Q16_TILES 1  // 1: more resident warps beat prefetching within a warp (measured)
#endif
#ifndef VX_Q16_DYNAMIC
#define VX_Q16_DYNAMIC 1  // octants after each warp's first one come from a device-wide counter
#endif
#ifndef VX_Q16_MINB
#define VX_Q16_MINB 4  // resident CTAs per SM the register allocation must allow
#endif
constexpr int kQ16Warps = 8;

template <class T>
struct Q16Smem {
    static constexpr size_t tile = 4096 * sizeof(T);
    static constexpr size_t kc = (size_t)kQ16Warps * VX_Q16_TILES * tile;  // 3 * kKeyCache u64
    static constexpr size_t leaf = kc + 3 * (size_t)kKeyCache * 8;        // 256 u64
    static constexpr size_t bars = leaf + 256 * 8;                         // VX_Q16_TILES per warp
    static constexpr size_t kcval = bars + (size_t)kQ16Warps * VX_Q16_TILES * 8;
    static constexpr size_t total = kcval + (size_t)kKeyCache * 4;
};

template <class T>
__global__ void __launch_bounds__(kQ16Warps * 32, VX_Q16_MINB) dense_quads16_kernel(DevInterner I, OctArgs a, uint64_t *q_ids,
                                                                       uint32_t *q_vals,
                                                                       const __grid_constant__ CUtensorMap tmap) {
    pdl_release();  // the record kernel may launch early: it waits for this grid before it starts
    using L = Q16Smem<T>;
    constexpr int NT = VX_Q16_TILES;
    extern __shared__ __align__(128) unsigned char smem[];
    const unsigned tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    uint64_t *kc = reinterpret_cast<uint64_t *>(smem + L::kc);
    uint64_t *leaf_cache = reinterpret_cast<uint64_t *>(smem + L::leaf);
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + L::bars) + warp * NT;
    T *tiles = reinterpret_cast<T *>(smem + (size_t)warp * NT * L::tile);
    KeyCache C{kc, kc + kKeyCache, kc + 2 * kKeyCache, reinterpret_cast<uint32_t *>(smem + L::kcval)};
    for (unsigned k = tid; k < kKeyCache; k += blockDim.x) C.id[k] = 0;
    if (sizeof(T) == 1)
        leaf_cache_warm(I, leaf_cache, tid);
    if (lane == 0) {
        for (int b = 0; b < NT; ++b) mbar_init(bars + b, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();

    const int d = a.depth;
    const int ob = 3 * (d - 4);
    const uint64_t n_oct = (uint64_t)a.n_chunks << ob;
    const uint64_t per_chunk = 1ull << (3 * (d - 2));
    const uint64_t total = (uint64_t)gridDim.x * kQ16Warps;
    const uint64_t gw = (uint64_t)blockIdx.x * kQ16Warps + warp;
    auto issue = [&](uint64_t o, int b) {
        const uint32_t c = (uint32_t)(o >> ob);
        const uint32_t q = (uint32_t)(o & ((1ull << ob) - 1));
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        mbar_expect_tx(bars + b, (uint32_t)L::tile);
        tma_load_octant(tiles + (size_t)b * 4096, &tmap, (int)(compact3(q) * 16), (int)(compact3(q >> 2) * 16),
                        (int)(compact3(q >> 1) * 16), (int)c, bars + b);
    };
    // Octants in the order this warp claimed them; fifo[0] is in tile j % NT. The first NT are fixed
    // (gw + b * total); later ones come from a device-wide counter: octant cost varies by an order of
    // magnitude (uniform air or rock against dune surface), and a fixed stride would give a warp the
    // same octant position in each of its chunks. Claims only grow, so once fifo[0] is past the end
    // every later one is too and no copy is left in flight.
    const bool dyn = VX_Q16_DYNAMIC && a.work != nullptr;
    uint64_t fifo[NT];
#pragma unroll
    for (int b = 0; b < NT; ++b) {
        fifo[b] = gw + b * total;
        if (lane == 0 && fifo[b] < n_oct) issue(fifo[b], b);
    }
    for (uint32_t j = 0; fifo[0] < n_oct; ++j) {
        const uint64_t o = fifo[0];
        const int b = (int)(j % NT);
        const uint32_t c = (uint32_t)(o >> ob);
        const uint64_t q = o & ((1ull << ob) - 1);
        // the tree check's two dependent loads go out before the wait, beside the tile's copy
        const uint32_t tree = a.trees[c];
        const bool tree_ok = tree < I.tree_cap && I.depths[tree] == d && I.roots[tree] == EMPTY_ID;
        bool ok = false;
        for (uint32_t spin = 0; spin < SPIN_LIMIT; ++spin)
            if ((ok = mbar_try_wait(bars + b, (j / NT) & 1u))) break;
        if (!__all_sync(0xFFFFFFFFu, ok)) {  // give up: wait (bounded) for this warp's copies, then leave
            if (lane == 0) set_error(I, ERR_TIMEOUT, 33);
#pragma unroll
            for (int k = 0; k < NT; ++k)
                if (fifo[k] < n_oct)
                    for (uint32_t spin = 0;
                         spin < SPIN_LIMIT && !mbar_try_wait(bars + (j + k) % NT, ((j + k) / NT) & 1u); ++spin) {
                    }
            return;
        }
        // the next octant is claimed now and its number read after this one is done, so the
        // atomic's round trip overlaps this octant's work
        unsigned long long claim = 0;
        if (dyn && lane == 0) claim = atomicAdd(a.work, 1ull);
        uint64_t *oid = q_ids + (uint64_t)c * per_chunk + (q << 6);
        uint32_t *oval = q_vals + (uint64_t)c * per_chunk + (q << 6);
        if (tree_ok) {
            quads_of_tile<T>(I, a, tiles + (size_t)b * 4096, C, leaf_cache, oid, oval);
        } else {
            if (lane == 0) set_error(I, ERR_INVALID, 34);
            for (unsigned k = lane; k < 64; k += 32) {
                oid[k] = EMPTY_ID;
                oval[k] = 0;
            }
        }
        __syncwarp();
        const uint64_t nx = dyn ? (uint64_t)NT * total + __shfl_sync(0xFFFFFFFFu, claim, 0) : o + (uint64_t)NT * total;
#pragma unroll
        for (int k = 0; k + 1 < NT; ++k) fifo[k] = fifo[k + 1];
        fifo[NT - 1] = nx;
        if (lane == 0 && nx < n_oct) issue(nx, b);
    }
}

#ifndef VX_LIVE_LIST
#define VX_LIVE_LIST 1  // claims that need computing are listed, so the record kernel skips dead claims
#endif

// ---- pending memo records, computed once each ------------------------------------------------------
//
// Every record on the live list (claims that won their memo slot, or found none) is a distinct quad
// of this build; dead claims, about nine in ten on a cold memo, are not walked. Without the list every
// handed-out record is checked. A warp takes 4 records at a time, 8 lanes each: lane 8m + k reduces
// bottom group k of the m-th record from the record's row words (the groups, keys and interning of
// quad_groups), then lane 8m reduces the quad node and writes the record's tail. Group keys go
// through the CTA's key cache.
template <class T>
__global__ void __launch_bounds__(kQ16Warps * 32) dense_memo_compute_kernel(DevInterner I, OctArgs a) {
    pdl_wait();
    pdl_release();
    extern __shared__ __align__(128) unsigned char smem[];
    const unsigned tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    uint64_t *kc = reinterpret_cast<uint64_t *>(smem);
    uint64_t *leaf_cache = kc + 3 * kKeyCache;
    KeyCache C{kc, kc + kKeyCache, kc + 2 * kKeyCache, reinterpret_cast<uint32_t *>(leaf_cache + 256)};
    for (unsigned k = tid; k < kKeyCache; k += blockDim.x) C.id[k] = 0;
    if (sizeof(T) == 1)
        leaf_cache_warm(I, leaf_cache, tid);
    __shared__ uint32_t leaf_cnt_s[256];
    __shared__ uint32_t leaf_claim[256];
    if (sizeof(T) == 1)
        for (unsigned k = tid; k < 256; k += blockDim.x) leaf_claim[k] = 0;
    const bool count = sizeof(T) == 1 && a.count_refs != 0;  // 8-bit interners only
    uint32_t *leaf_cnt = count ? leaf_cnt_s : nullptr;
    if (leaf_cnt) leaf_cnt_clear(leaf_cnt);
    __syncthreads();
    using W = typename QuadWord<T>::type;
    const bool wide = sizeof(T) == 2;
    const uint32_t cnt = *(volatile unsigned int *)(a.live ? a.live_count : a.memo_count);
    const uint32_t n = cnt < a.memo_cap ? cnt : a.memo_cap;
    const uint32_t m = lane >> 3;
    const int k = (int)(lane & 7u);
    const uint32_t gx = k & 1, gy = (k >> 1) & 1, gz = k >> 2;
    const uint64_t stride = (uint64_t)gridDim.x * kQ16Warps * 4;
    for (uint64_t base = ((uint64_t)blockIdx.x * kQ16Warps + warp) * 4; base < n; base += stride) {
        const uint64_t r = base + m;
        unsigned char *rec = r < n ? memo_rec<T>(a, a.live ? a.live[r] : (uint32_t)r) : nullptr;
        uint4 *tail = rec ? reinterpret_cast<uint4 *>(rec + 16 * 4 * sizeof(T)) : nullptr;
        const bool act = rec && tail->x == 0u && tail->y == 0u;
        uint64_t lo = 0, hi = 0;
        if (act) {  // bottom group k: rows y*4 + z of 4 voxels along x
            const W *w = reinterpret_cast<const W *>(rec);
            const W r00 = w[(2 * gy) * 4 + 2 * gz], r10 = w[(2 * gy + 1) * 4 + 2 * gz];
            const W r01 = w[(2 * gy) * 4 + 2 * gz + 1], r11 = w[(2 * gy + 1) * 4 + 2 * gz + 1];
            if (sizeof(T) == 1) {
                const uint32_t sh = 16 * gx;
                const uint64_t p0 = ((uint32_t)r00 >> sh) & 0xFFFFu, p1 = ((uint32_t)r10 >> sh) & 0xFFFFu;
                const uint64_t p2 = ((uint32_t)r01 >> sh) & 0xFFFFu, p3 = ((uint32_t)r11 >> sh) & 0xFFFFu;
                lo = p0 | (p1 << 16) | (p2 << 32) | (p3 << 48);
            } else {
                const uint32_t sh = 32 * gx;
                lo = (((uint64_t)r00 >> sh) & 0xFFFFFFFFull) | ((((uint64_t)r10 >> sh) & 0xFFFFFFFFull) << 32);
                hi = (((uint64_t)r01 >> sh) & 0xFFFFFFFFull) | ((((uint64_t)r11 >> sh) & 0xFFFFFFFFull) << 32);
            }
        }
        const uint32_t set = set_mask8<T>(lo, hi);
        const uint32_t gv0 = (uint32_t)lo & (sizeof(T) == 1 ? 0xFFu : 0xFFFFu);
        const bool guni = sizeof(T) == 1 ? lo == (uint64_t)gv0 * 0x0101010101010101ull
                                         : (lo == hi && lo == (uint64_t)gv0 * 0x0001000100010001ull);
        const bool is_branch = act && set != 0 && !(guni && set == 0xFFu);
        uint32_t lod = 0;
        uint64_t id = is_branch ? kc_lookup(C, lo, hi, &lod) : 0ull;
        const bool need = is_branch && id == 0;
        const unsigned bm = __ballot_sync(0xFFFFFFFFu, need);
        if (bm) {
            uint32_t v[8];
            unpack8<T>(lo, hi, v);
            if (need) lod = calc_average8(v);
            unsigned grp = __match_any_sync(0xFFFFFFFFu, need ? lo : ~(uint64_t)lane);
            if (wide) grp &= __match_any_sync(0xFFFFFFFFu, need ? hi : ~(uint64_t)lane);
            grp &= bm;
            const int leader = need ? __ffs(grp) - 1 : (int)lane;
            const bool lead = need && leader == (int)lane;
            uint64_t c[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const bool want = lead && v[j] != 0;
                if (sizeof(T) == 1 && VX_LEAF_CLAIM) {  // one lookup per warp and value
                    const unsigned peers = __match_any_sync(0xFFFFFFFFu, want ? v[j] : 0x100u + lane);
                    const int ldr = __ffs(peers) - 1;
                    uint64_t lid = 0;
                    if (want && ldr == (int)lane) lid = leaf_of_claimed(I, leaf_cache, leaf_claim, v[j]);
                    lid = __shfl_sync(0xFFFFFFFFu, lid, ldr);
                    c[j] = want ? lid : 0ull;
                } else {
                    c[j] = want ? leaf_of<T>(I, leaf_cache, v[j]) : 0ull;
                }
            }
            bool created;
            uint64_t nid = warp_intern_branch(I, lead, c, set, set, lod, &created);
            if (count && created) {
                if (leaf_cnt)
                    count_group_leaves(leaf_cnt, v);
                else
                    count_created(I, nullptr, nid);
            }
            nid = __shfl_sync(0xFFFFFFFFu, nid, leader);
            if (lead && nid != EMPTY_ID) kc_insert(C, lo, hi, nid, lod);
            if (need) id = nid;
        }
        const bool gleaf = act && set != 0 && !is_branch;  // a uniform group: its leaf
        uint64_t glid = 0;
        if (sizeof(T) == 1 && VX_LEAF_CLAIM) {  // one lookup per warp and value
            const unsigned peers = __match_any_sync(0xFFFFFFFFu, gleaf ? gv0 : 0x100u + lane);
            const int ldr = __ffs(peers) - 1;
            if (gleaf && ldr == (int)lane) glid = leaf_of_claimed(I, leaf_cache, leaf_claim, gv0);
            glid = __shfl_sync(0xFFFFFFFFu, glid, ldr);
        } else if (gleaf) {
            glid = leaf_of<T>(I, leaf_cache, gv0);
        }
        uint64_t gid;
        uint32_t gval;
        if (set == 0) {
            gid = EMPTY_ID;
            gval = 0;
        } else if (!is_branch) {
            gid = act ? glid : 0ull;
            gval = gv0;
        } else {
            gid = id;
            gval = lod;
        }
        uint64_t c3[8];
        uint32_t cv3[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            c3[j] = __shfl_sync(0xFFFFFFFFu, gid, (lane & ~7u) + j);
            cv3[j] = __shfl_sync(0xFFFFFFFFu, gval, (lane & ~7u) + j);
        }
        uint64_t qid;
        uint32_t qval;
        bool qc = false;
        reduce_parent(I, act && k == 0, c3, cv3, qid, qval, &qc);
        if (count && qc) count_created_regs(I, leaf_cnt, c3, cv3);
        if (act && k == 0) *tail = make_uint4((uint32_t)qid, (uint32_t)(qid >> 32), qval, 0u);
    }
    if (leaf_cnt) leaf_cnt_flush(I, leaf_cnt);
}

// One parent per lane from its 8 children: EMPTY, a collapsed leaf, or the interned branch.
// Identical parents of the warp (common in repetitive terrain) probe the table once. Warp-collective:
// every lane calls it; lanes with in == false only take part.
__device__ __forceinline__ void reduce_parent_dedup(const DevInterner &I, bool in, const uint64_t c[8],
                                                    const uint32_t cv[8], uint64_t &out, uint32_t &val,
                                                    bool *created_out = nullptr) {
    uint32_t types = 0, mask = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        mask |= (c[k] != 0 ? 1u : 0u) << k;
        types |= (id_is_leaf(c[k]) ? 1u : 0u) << k;
    }
    bool same = types == 0xFF;
#pragma unroll
    for (int k = 1; k < 8; ++k) same = same && c[k] == c[0];
    const bool is_branch = in && mask != 0 && !same;
    const uint64_t h = is_branch ? branch_fingerprint(c, (types << 8) | mask) : 0ull;
    const unsigned peers =
        __match_any_sync(0xFFFFFFFFu, (is_branch && VX_LEVEL_DEDUP) ? h : (~0ull - (threadIdx.x & 31u)));
    const int leader = __ffs(peers) - 1;
    bool same_key = true;
#pragma unroll
    for (int k = 0; k < 8; ++k) {  // every lane takes part in each shuffle
        const uint64_t lk = __shfl_sync(0xFFFFFFFFu, c[k], leader);
        same_key = same_key && lk == c[k];
    }
    const bool follow = is_branch && leader != (int)(threadIdx.x & 31u) && same_key;
    const bool probe = is_branch && !follow;
    const uint32_t lod = probe ? calc_average8(cv) : 0;
    bool created;
    uint64_t id = warp_intern_branch_inl(I, probe, c, types, mask, lod, &created, h);
    if (created_out) *created_out = created;
    const uint64_t lead_id = __shfl_sync(0xFFFFFFFFu, id, leader);
    const uint32_t lead_lod = __shfl_sync(0xFFFFFFFFu, lod, leader);
    if (follow) id = lead_id;
    out = mask == 0 ? EMPTY_ID : (same ? c[0] : id);
    val = mask == 0 ? 0 : (same ? cv[0] : (follow ? lead_lod : lod));
}

__device__ __forceinline__ void commit_root(const DevInterner &I, const uint32_t *trees, uint8_t *changed, uint64_t p,
                                            uint64_t out) {
    const uint32_t tree = trees[p];
    if (tree >= I.tree_cap) {
        set_error(I, ERR_INVALID, 22);
        return;
    }
    if (out != EMPTY_ID) {
        I.roots[tree] = out;
        atomicAdd(I.refcount + id_index(out), 1u);
    }
    if (changed) changed[p] = out != EMPTY_ID;
}

// Memo records that quads still pending in q_ids / q_vals name (recs == nullptr: nothing pending).
struct PendingView {
    const unsigned char *recs;
    uint32_t stride;    // bytes per record
    uint32_t tail_off;  // offset of the (id, LOD value) tail in a record
};

__device__ __forceinline__ void resolve_pending(const PendingView &P, uint64_t &id, uint32_t &val) {
    if (P.recs && val == kQuadPending) {
        const uint4 t = __ldcg(reinterpret_cast<const uint4 *>(P.recs + (size_t)id * P.stride + P.tail_off));
        id = (uint64_t)t.x | ((uint64_t)t.y << 32);
        val = t.z;
    }
}

__global__ void __launch_bounds__(kThreads, 4) fresh_level_kernel(DevInterner I, const uint64_t *in_ids,
                                                               const uint32_t *in_vals, uint64_t *out_ids,
                                                               uint32_t *out_vals, uint64_t n_parents, int is_root,
                                                               const uint32_t *trees, uint8_t *changed,
                                                               PendingView P, int count_refs) {
    pdl_wait();
    pdl_release();
    __shared__ uint32_t leaf_cnt_s[256];
    const bool count = count_refs != 0;
    uint32_t *leaf_cnt = (count && I.vbits == 8) ? leaf_cnt_s : nullptr;
    if (leaf_cnt) {
        leaf_cnt_clear(leaf_cnt);
        __syncthreads();
    }
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t base = (uint64_t)blockIdx.x * blockDim.x; base < n_parents; base += stride) {
        const uint64_t p = base + threadIdx.x;
        const bool in = p < n_parents;
        uint64_t c[8];
        uint32_t cv[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            c[k] = in ? in_ids[8 * p + k] : 0;
            cv[k] = in ? in_vals[8 * p + k] : 0;
            resolve_pending(P, c[k], cv[k]);
        }
        uint64_t out;
        uint32_t val;
        bool created = false;
        reduce_parent_dedup(I, in, c, cv, out, val, &created);
        if (!in) continue;
        if (is_root) {
            commit_root(I, trees, changed, p, out);
        } else {
            out_ids[p] = out;
            out_vals[p] = val;
        }
        if (count && created) count_created(I, leaf_cnt, out);
    }
    if (leaf_cnt) leaf_cnt_flush(I, leaf_cnt);
}

#ifndef VX_TOP_COMPACT
#define VX_TOP_COMPACT 1  // fresh_top_kernel packs the depth-2 parents that need an insert into one round
#endif

// The three top levels (depths 2, 1 and 0: 64 + 8 + 1 nodes a chunk) with one warp per chunk and
// no CTA barrier: lanes reduce the chunk's 64 depth-2 parents in two passes, lanes 0-7 its 8 depth-1
// parents from those (shuffles), lane 0 the root. 8 chunks per CTA; a 4096-chunk build is one wave
// of warps at 64 registers (a CTA per 4 chunks with the levels split by CTA barriers needed 1.7
// waves and idled 7 of its 8 warps at the barriers: 0.054 against 0.050 ms).
// 4 resident CTAs per SM: the 4096-chunk build's 512 CTAs then run in a single wave on 152 SMs
__global__ void __launch_bounds__(kThreads, 4) fresh_top_kernel(DevInterner I, const uint64_t *in_ids,
                                                                  const uint32_t *in_vals, uint32_t n_chunks,
                                                                  const uint32_t *trees, uint8_t *changed,
                                                                  PendingView P, int count_refs) {
    pdl_wait();
    pdl_release();
    __shared__ uint32_t leaf_cnt_s[256];
#if VX_TOP_COMPACT
    __shared__ uint64_t top_ch[kThreads * 8];  // per warp: 32 packed depth-2 parents x 8 children
    __shared__ uint32_t top_cv[kThreads * 8];
    __shared__ uint64_t top_rid[kThreads * 2];  // per warp: the chunk's 64 depth-2 results
    __shared__ uint32_t top_rval[kThreads * 2];
    __shared__ uint8_t top_par[kThreads];       // per warp: the parent of each packed slot
#endif
    const bool count = count_refs != 0;
    uint32_t *leaf_cnt = (count && I.vbits == 8) ? leaf_cnt_s : nullptr;
    if (leaf_cnt) {
        leaf_cnt_clear(leaf_cnt);
        __syncthreads();
    }
    const unsigned lane = threadIdx.x & 31u;
    const uint64_t c = (uint64_t)blockIdx.x * (kThreads / 32) + (threadIdx.x >> 5);
    if (c < n_chunks) {  // the whole warp
#if VX_TOP_COMPACT
        // depth 2: parent lane + 32 r of the chunk. Parents that are EMPTY or collapse to a leaf are
        // settled at once; the others (the surface layer, usually at most 32 of the 64) are packed
        // into the warp's shared slots and interned in one round instead of one per half. Results go
        // to the warp's shared row of 64, where the depth-1 lanes read them.
        const unsigned wslot = threadIdx.x >> 5;
        uint64_t *sch = top_ch + wslot * 32 * 8;
        uint32_t *scv = top_cv + wslot * 32 * 8;
        uint64_t *rid = top_rid + wslot * 64;
        uint32_t *rval = top_rval + wslot * 64;
        uint8_t *spar = top_par + wslot * 32;
        unsigned nneed = 0;
        bool over = false;  // this lane's second-half parent did not get a slot
#pragma unroll 1
        for (int r = 0; r < 2; ++r) {
            const uint64_t p = c * 64 + lane + 32u * r;
            uint64_t ch[8];
            uint32_t cv[8];
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                ch[k] = in_ids[8 * p + k];
                cv[k] = in_vals[8 * p + k];
                resolve_pending(P, ch[k], cv[k]);
            }
            uint32_t mask = 0;
            bool same = true;
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                mask |= (ch[k] != 0 ? 1u : 0u) << k;
                same = same && id_is_leaf(ch[k]) && ch[k] == ch[0];
            }
            const bool need = mask != 0 && !same;
            const unsigned b = __ballot_sync(0xFFFFFFFFu, need);
            const unsigned slot = nneed + __popc(b & ((1u << lane) - 1u));
            nneed += __popc(b);
            if (need && slot < 32) {
#pragma unroll
                for (int k = 0; k < 8; ++k) {
                    sch[slot * 8 + k] = ch[k];
                    scv[slot * 8 + k] = cv[k];
                }
                spar[slot] = (uint8_t)(lane + 32u * r);
            }
            over = over || (need && slot >= 32);
            rid[lane + 32u * r] = mask == 0 ? EMPTY_ID : ch[0];
            rval[lane + 32u * r] = mask == 0 ? 0u : cv[0];
        }
        __syncwarp();
        {
            const bool in = lane < nneed;
            uint64_t ch[8];
            uint32_t cv[8];
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                ch[k] = in ? sch[lane * 8 + k] : 0ull;
                cv[k] = in ? scv[lane * 8 + k] : 0u;
            }
            uint64_t out;
            uint32_t val;
            bool created = false;
            reduce_parent_dedup(I, in, ch, cv, out, val, &created);
            if (count && created) count_created(I, leaf_cnt, out);
            if (in) {
                const unsigned q = spar[lane];
                rid[q] = out;
                rval[q] = val;
            }
        }
        if (__any_sync(0xFFFFFFFFu, over)) {  // second-half parents past the 32 slots: one more round
            const uint64_t p = c * 64 + lane + 32u;
            uint64_t ch[8];
            uint32_t cv[8];
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                ch[k] = over ? in_ids[8 * p + k] : 0ull;
                cv[k] = over ? in_vals[8 * p + k] : 0u;
                resolve_pending(P, ch[k], cv[k]);
            }
            uint64_t out;
            uint32_t val;
            bool created = false;
            reduce_parent_dedup(I, over, ch, cv, out, val, &created);
            if (count && created) count_created(I, leaf_cnt, out);
            if (over) {
                rid[lane + 32u] = out;
                rval[lane + 32u] = val;
            }
        }
        __syncwarp();
        // depth 1: lane q < 8 takes depth-2 nodes 8q .. 8q+7
        uint64_t ch[8];
        uint32_t cv[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const unsigned src = (8 * lane + k) & 63u;
            ch[k] = rid[src];
            cv[k] = rval[src];
        }
#else
        uint64_t d2[2];
        uint32_t v2[2];
#pragma unroll
        for (int r = 0; r < 2; ++r) {  // depth 2: parent lane + 32 r of the chunk
            const uint64_t p = c * 64 + lane + 32u * r;
            uint64_t ch[8];
            uint32_t cv[8];
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                ch[k] = in_ids[8 * p + k];
                cv[k] = in_vals[8 * p + k];
                resolve_pending(P, ch[k], cv[k]);
            }
            bool created = false;
            reduce_parent_dedup(I, true, ch, cv, d2[r], v2[r], &created);
            if (count && created) count_created(I, leaf_cnt, d2[r]);
        }
        // depth 1: lane q < 8 takes depth-2 nodes 8q .. 8q+7 (pass q >> 2)
        uint64_t ch[8];
        uint32_t cv[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const int src = (8 * lane + k) & 31;
            const uint64_t a0 = __shfl_sync(0xFFFFFFFFu, d2[0], src), a1 = __shfl_sync(0xFFFFFFFFu, d2[1], src);
            const uint32_t b0 = __shfl_sync(0xFFFFFFFFu, v2[0], src), b1 = __shfl_sync(0xFFFFFFFFu, v2[1], src);
            ch[k] = lane < 4 ? a0 : a1;
            cv[k] = lane < 4 ? b0 : b1;
        }
#endif
        uint64_t d1;
        uint32_t v1;
        bool created = false;
        reduce_parent_dedup(I, lane < 8, ch, cv, d1, v1, &created);
        if (count && created) count_created(I, leaf_cnt, d1);
#pragma unroll
        for (int k = 0; k < 8; ++k) {  // the root from lanes 0-7
            ch[k] = __shfl_sync(0xFFFFFFFFu, d1, k);
            cv[k] = __shfl_sync(0xFFFFFFFFu, v1, k);
        }
        uint64_t root;
        uint32_t rv;
        reduce_parent_dedup(I, lane == 0, ch, cv, root, rv, &created);
        if (lane == 0) commit_root(I, trees, changed, c, root);
        if (count && created) count_created(I, leaf_cnt, root);
    }
    if (leaf_cnt) leaf_cnt_flush(I, leaf_cnt);
    // counting builds: the last CTA closes the epoch (every creation of the build is done by then)
    if (count && grid_last_cta(&I.ctr->scratch[SC_REF_DONE])) epoch_finalize_body(I);
}

// Adds one reference per child slot of every node created in this epoch. Leaf references are the hot spots of the in-degree count (a few leaf values are named by most
// bottom groups), so they are summed per CTA before touching global memory: 8-bit leaves in a
// 256-entry array indexed by value, wider leaves in an open-addressed shared table keyed by node
// index (entries that find no slot within kLeafProbe steps go straight to global atomics).
constexpr int kLeafTab = 4096;
#ifndef VX_REF_FOLD
#define VX_REF_FOLD 1  // the refcount kernel's last CTA closes the epoch (else a separate launch)
#endif
constexpr int kLeafProbe = 16;

__device__ __forceinline__ void leaf_tab_add(uint32_t *tab_key, uint32_t *tab_cnt, const DevInterner &I,
                                             uint32_t idx, uint32_t cnt) {
    const uint32_t key = idx + 1;
    uint32_t h = (key * 0x9E3779B1u) >> 20;  // 12 bits: kLeafTab entries
#pragma unroll 1
    for (int p = 0; p < kLeafProbe; ++p) {
        uint32_t k = tab_key[h];
        if (k == 0) k = atomicCAS(tab_key + h, 0u, key), k = k ? k : key;
        if (k == key) {
            atomicAdd(tab_cnt + h, cnt);
            return;
        }
        h = (h + 1) & (kLeafTab - 1);
    }
    atomicAdd(I.refcount + idx, cnt);
}

__global__ void __launch_bounds__(kThreads) epoch_refcount_kernel(DevInterner I) {
    pdl_wait();
    // 8-bit leaves: 256 counters; wider leaves: the kLeafTab-entry table (dynamic shared memory, so
    // the 8-bit case keeps its occupancy)
    extern __shared__ uint32_t ref_smem[];
    uint32_t *leaf_cnt = ref_smem;
    uint32_t *tab_key = ref_smem, *tab_cnt = ref_smem + kLeafTab;
    const bool small = I.vbits == 8;
    if (small)
        for (unsigned k = threadIdx.x; k < 256; k += blockDim.x) leaf_cnt[k] = 0;
    else
        for (unsigned k = threadIdx.x; k < kLeafTab; k += blockDim.x) tab_key[k] = 0, tab_cnt[k] = 0;
    __syncthreads();
    const unsigned long long n = I.ctr->alloc_count;
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    for (unsigned long long t = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += stride) {
        const uint32_t idx = node_for_ticket(I, t);
        if (idx == NO_NODE) continue;
        const uint64_t id = I.ids[idx];
        if (id == 0 || id_is_leaf(id)) continue;
        uint64_t c[8];
        const ulonglong2 *src = reinterpret_cast<const ulonglong2 *>(I.children + 8ull * idx);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            ulonglong2 w = src[k];
            c[2 * k] = w.x;
            c[2 * k + 1] = w.y;
        }
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            if (c[k] == 0) continue;
            bool seen = false;
            uint32_t cnt = 1;
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                if (j < k && c[j] == c[k]) seen = true;
                if (j > k && c[j] == c[k]) ++cnt;
            }
            if (seen) continue;
            if (id_is_leaf(c[k])) {
                if (small)
                    atomicAdd(&leaf_cnt[node_value(I, id_index(c[k]))], cnt);
                else
                    leaf_tab_add(tab_key, tab_cnt, I, id_index(c[k]), cnt);
            } else {
                atomicAdd(I.refcount + id_index(c[k]), cnt);
            }
        }
    }
    __syncthreads();
    if (small) {
        for (unsigned v = threadIdx.x; v < 256; v += blockDim.x)
            if (leaf_cnt[v]) {
                const uint64_t lid = I.leaf_table[v];
                if (lid > LEAF_BUSY)
                    atomicAdd(I.refcount + id_index(lid), leaf_cnt[v]);
                else
                    set_error(I, ERR_INTERNAL, 30);
            }
    } else {
        for (unsigned k = threadIdx.x; k < kLeafTab; k += blockDim.x)
            if (tab_key[k] && tab_cnt[k]) atomicAdd(I.refcount + tab_key[k] - 1, tab_cnt[k]);
    }
    if (VX_REF_FOLD) {  // the last CTA to finish closes the epoch (no separate launch)
        __shared__ unsigned int last_cta;
        __syncthreads();
        if (threadIdx.x == 0) {
            __threadfence();
            last_cta = atomicAdd(&I.ctr->scratch[SC_REF_DONE], 1ull) == gridDim.x - 1;
        }
        __syncthreads();
        if (last_cta && threadIdx.x == 0) {
            __threadfence();
            epoch_finalize_body(I);
            I.ctr->scratch[SC_REF_DONE] = 0;
        }
    }
}


__global__ void epoch_finalize_kernel(DevInterner I) { epoch_finalize_body(I); }

}  // namespace

// Opts `kernel` in to `smem` bytes of dynamic shared memory and returns its resident CTAs per SM,
// cached per (kernel, threads, smem): both calls cost host time on every launch otherwise. The
// opt-in is a property of the kernel, so it only ever rises (a kernel launched with several sizes,
// such as the dense-block kernel at depths 2 and 3, keeps the largest size it was opted in to).
static int prepare_kernel(const void *kernel, int threads, size_t smem, cudaError_t *err) {
    struct Entry {
        const void *k;
        int threads;
        size_t smem;
        int per_sm;
    };
    struct OptIn {
        const void *k;
        size_t smem;
    };
    static Entry cache[64];
    static OptIn opted[32];
    static int used = 0, n_opted = 0;
    static std::mutex mu;
    std::lock_guard<std::mutex> lock(mu);
    for (int i = 0; i < used; ++i)
        if (cache[i].k == kernel && cache[i].threads == threads && cache[i].smem == smem) return cache[i].per_sm;
    int o = 0;
    while (o < n_opted && opted[o].k != kernel) ++o;
    if (o == n_opted || opted[o].smem < smem) {
        *err = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (*err != cudaSuccess) return 0;
        if (o == n_opted && n_opted < 32) ++n_opted;
        if (o < 32) opted[o] = OptIn{kernel, smem};
    }
    int per_sm = 1;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem);
    if (per_sm < 1) per_sm = 1;
    if (used < 64) cache[used++] = Entry{kernel, threads, smem, per_sm};
    return per_sm;
}

size_t dense_smem_bytes(int depth, int vbytes) {
    const size_t V = (size_t)1 << (3 * depth);
    const size_t n_nodes = (V - 1) / 7;
    const size_t vox = (V * vbytes + 127) & ~(size_t)127;
    return vox + n_nodes * 8 + ((n_nodes + 1) & ~(size_t)1) * 4 + 256 * 8 + 16;
}

template <class K>
static cudaError_t launch_persistent(K kernel, const DevInterner &I, const DenseArgs &a, size_t smem, int num_sms,
                                    cudaStream_t s) {
    const uint64_t total = a.n_chunks;
    cudaError_t e = cudaSuccess;
    const int per_sm = prepare_kernel(reinterpret_cast<const void *>(kernel), kThreads, smem, &e);
    if (e != cudaSuccess) return e;
    uint64_t grid = (uint64_t)num_sms * per_sm;
    if (grid > total) grid = total;
    count_launches(1);
    kernel<<<(unsigned)grid, kThreads, smem, s>>>(I, a);
    return cudaGetLastError();
}


cudaError_t launch_dense_blocks(const DevInterner &I, const DenseArgs &a, int num_sms, cudaStream_t s) {
    if (a.n_chunks == 0) return cudaSuccess;
    if (a.depth < 2 || a.depth > 3) return cudaErrorInvalidValue;
    const size_t smem = dense_smem_bytes(a.depth, I.vbits / 8);
    if (I.vbits == 8) return launch_persistent(dense_blocks_kernel<uint8_t>, I, a, smem, num_sms, s);
    return launch_persistent(dense_blocks_kernel<uint16_t>, I, a, smem, num_sms, s);
}

// log2 of the side of the unit that one CTA (32^3 blocks, depths 5-10) or one warp (16^3 octants,
// depth 4) of launch_dense_octants reduces; the scratch holds the levels above that unit.
static int dense_octant_unit(int depth) { return (VX_DENSE_CTA32 && depth >= 5) ? 5 : 4; }

// Scratch of launch_dense_octants, laid out as it carves it: node ids (8 B) and LOD values (4 B) of
// every level above the unit, then (from a 256-byte boundary) the arrival counts of every level
// above the unit's parents.
size_t dense_octant_scratch_bytes(uint64_t n_chunks, int depth) {
    const int unit = dense_octant_unit(depth);
    size_t ids = 0, cnts = 0;
    for (int k = 1; k <= depth - unit; ++k) ids += (size_t)n_chunks << (3 * k);
    for (int k = 0; k <= depth - unit - 1; ++k) cnts += (size_t)n_chunks << (3 * k);
    return ((ids * 12 + 255) & ~(size_t)255) + cnts * 4 + 256;
}

static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }
    return fn;
}

// Quad memo geometry for a call: slots = a power of two near the call's quads >> shift (a quarter by
// default; 1 Ki to 2 Mi), records = half the slots.
static void memo_geometry(uint64_t n_chunks, int depth, uint32_t shift, uint64_t *slots, uint64_t *recs) {
    const uint64_t quads = n_chunks << (3 * (depth - 2));
    uint64_t sl = 1024;
    while (sl < (quads >> shift) && sl < (1ull << 21)) sl <<= 1;
    *slots = sl;
    *recs = sl / 2;
}

size_t dense_octant_memo_bytes(uint64_t n_chunks, int depth, int vbits, uint32_t memo_shift) {
    if (depth < 4) return 0;
    uint64_t sl, rc;
    memo_geometry(n_chunks, depth, memo_shift, &sl, &rc);
    const size_t stride = memo_stride((size_t)(vbits / 8));
    return sl * 8 + 256 + rc * stride + rc * 4 + 256;
}

cudaError_t launch_dense_octants(const DevInterner &I, const void *grids, const uint32_t *trees, uint32_t n_chunks,
                                 int depth, uint8_t *changed, void *scratch, int num_sms, cudaStream_t s,
                                 void *memo, bool clear_memo, uint64_t memo_chunks) {
    if (n_chunks == 0) return cudaSuccess;
    if (depth < 4 || depth > 10) return cudaErrorInvalidValue;
    const int unit = dense_octant_unit(depth);
    const bool cta32 = unit == 5;
    OctArgs a{};
    a.trees = trees;
    a.n_chunks = n_chunks;
    a.depth = depth;
    a.changed = changed;
    size_t ids = 0, cnts = 0;
    for (int k = 1; k <= depth - unit; ++k) {
        a.lvl_off[k] = ids;
        ids += (size_t)n_chunks << (3 * k);
    }
    for (int k = 0; k <= depth - unit - 1; ++k) {
        a.cnt_off[k] = cnts;
        cnts += (size_t)n_chunks << (3 * k);
    }
    if (memo) {
        uint64_t sl, rc;
        memo_geometry(memo_chunks ? memo_chunks : n_chunks, depth, I.memo_shift, &sl, &rc);
        char *m = static_cast<char *>(memo);
        a.memo_slots = reinterpret_cast<unsigned long long *>(m);
        a.memo_count = reinterpret_cast<unsigned int *>(m + sl * 8);
        a.memo_recs = reinterpret_cast<unsigned char *>(m + sl * 8 + 256);
        a.memo_mask = (uint32_t)(sl - 1);
        a.memo_cap = (uint32_t)rc;
        if (clear_memo) {
            cudaError_t e = cudaMemsetAsync(m, 0, sl * 8 + 256, s);
            if (e != cudaSuccess) return e;
        }
    }
    char *base = static_cast<char *>(scratch);
    a.ids = reinterpret_cast<uint64_t *>(base);
    a.vals = reinterpret_cast<uint32_t *>(base + ids * 8);
    a.cnt = reinterpret_cast<uint32_t *>(base + ((ids * 12 + 255) & ~(size_t)255));
    if (cnts) {
        cudaError_t e = cudaMemsetAsync(a.cnt, 0, cnts * 4, s);
        if (e != cudaSuccess) return e;
    }
    PFN_cuTensorMapEncodeTiled_v12000 encode = tensor_map_encoder();
    if (!encode) return cudaErrorNotSupported;
    const uint64_t side = 1ull << depth;
    const uint32_t es = (uint32_t)(I.vbits / 8);
    CUtensorMap tmap;
    cuuint64_t dims[4] = {side, side, side, n_chunks};
    cuuint64_t strides[3] = {side * es, side * side * es, side * side * side * es};
    const cuuint32_t bs = cta32 ? 32 : 16;
    cuuint32_t box[4] = {bs, bs, bs, 1};
    cuuint32_t estr[4] = {1, 1, 1, 1};
    CUresult r = encode(&tmap, es == 1 ? CU_TENSOR_MAP_DATA_TYPE_UINT8 : CU_TENSOR_MAP_DATA_TYPE_UINT16, 4,
                        const_cast<void *>(grids), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                        CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return cudaErrorInvalidValue;
    const size_t smem = (size_t)kOctWarps * kOctTiles * 4096 * es +
                        (3 * kKeyCache + 256 + 2 * kOctWarps + 9 * kNodeCache) * 8 + (kKeyCache + kNodeCache) * 4 + 64;
    const uint64_t n_oct = (uint64_t)n_chunks << (3 * (depth - 4));
    auto launch = [&](auto kernel) -> cudaError_t {
        cudaError_t e = cudaSuccess;
        const int per_sm = prepare_kernel(reinterpret_cast<const void *>(kernel), kThreads, smem, &e);
        if (e != cudaSuccess) return e;
        uint64_t grid = (uint64_t)num_sms * per_sm;
        const uint64_t need = (n_oct + kOctWarps - 1) / kOctWarps;
        if (grid > need) grid = need;
        count_launches(1);
        kernel<<<(unsigned)grid, kThreads, smem, s>>>(I, a, tmap);
        return cudaGetLastError();
    };
    if (cta32) {
        auto launch32 = [&](auto kernel, size_t smem32) -> cudaError_t {
            cudaError_t e = cudaSuccess;
            const int per_sm = prepare_kernel(reinterpret_cast<const void *>(kernel), kCtaThreads, smem32, &e);
            if (e != cudaSuccess) return e;
            uint64_t grid = (uint64_t)num_sms * per_sm;
            const uint64_t need = (uint64_t)n_chunks << (3 * (depth - 5));
            if (grid > need) grid = need;
            count_launches(1);
            kernel<<<(unsigned)grid, kCtaThreads, smem32, s>>>(I, a, tmap);
            return cudaGetLastError();
        };
        if (es == 1) return launch32(dense_cta32_kernel<uint8_t>, Cta32Smem<uint8_t>::total);
        return launch32(dense_cta32_kernel<uint16_t>, Cta32Smem<uint16_t>::total);
    }
    if (es == 1) return launch(dense_octants_kernel<uint8_t>);
    return launch(dense_octants_kernel<uint16_t>);
}

size_t dense_split_scratch_bytes(uint64_t n_chunks, int depth) {
    if (depth < 5) return 0;
    size_t nodes = 0;  // quads and every level above them except the roots
    for (int k = 1; k <= depth - 2; ++k) nodes += (size_t)n_chunks << (3 * k);
    return nodes * 12 + 512;
}

static cudaError_t launch_fresh_level(const DevInterner &I, const uint64_t *in_ids, const uint32_t *in_vals,
                                      uint64_t *out_ids, uint32_t *out_vals, uint64_t n_parents, bool is_root,
                                      const uint32_t *trees, uint8_t *changed, cudaStream_t s, PendingView P,
                                      int count_refs);

// The split path's creators add their children's references as they create nodes (8-bit interners,
// whose leaf references sum in 256 per-CTA counters); the epoch then needs only closing, not the
// in-degree pass over the allocation log. A creator's child id comes from the child's own creation
// (shuffle, shared key cache, table) after the child creator's release store, which is issued only
// once the child's zeroed count is visible, so no count lands before that zero.
#ifndef VX_SPLIT_REFS
#define VX_SPLIT_REFS 1
#endif
bool dense_split_counts_refs(const DevInterner &I) { return VX_SPLIT_REFS && I.vbits == 8; }

cudaError_t launch_dense_split(const DevInterner &I, const void *grids, const uint32_t *trees, uint32_t n_chunks,
                               int depth, uint8_t *changed, void *scratch, int num_sms, cudaStream_t s, void *memo,
                               bool clear_memo, uint64_t memo_chunks, void (*levels_begin)(void *),
                               void *levels_ctx, bool count_refs) {
    if (n_chunks == 0) return cudaSuccess;
    if (depth < 5 || depth > 10) return cudaErrorInvalidValue;
    OctArgs a{};
    a.trees = trees;
    a.n_chunks = n_chunks;
    a.depth = depth;
    a.changed = changed;
    a.grids = grids;
    a.count_refs = (count_refs && dense_split_counts_refs(I)) ? 1 : 0;
    if (memo) {
        uint64_t sl, rc;
        memo_geometry(memo_chunks ? memo_chunks : n_chunks, depth, I.memo_shift, &sl, &rc);
        char *m = static_cast<char *>(memo);
        a.memo_slots = reinterpret_cast<unsigned long long *>(m);
        a.memo_count = reinterpret_cast<unsigned int *>(m + sl * 8);
        a.memo_recs = reinterpret_cast<unsigned char *>(m + sl * 8 + 256);
        a.memo_mask = (uint32_t)(sl - 1);
        a.memo_cap = (uint32_t)rc;
        a.work = reinterpret_cast<unsigned long long *>(m + sl * 8 + 128);  // in the header the clear zeroes
        if (VX_LIVE_LIST) {  // the list count sits in the header too; the list after the records
            a.live_count = reinterpret_cast<unsigned int *>(m + sl * 8 + 64);
            a.live = reinterpret_cast<uint32_t *>(m + sl * 8 + 256 + rc * memo_stride(I.vbits / 8));
        }
        cudaError_t e = clear_memo ? cudaMemsetAsync(m, 0, sl * 8 + 256, s) : cudaMemsetAsync(a.work, 0, 8, s);
        if (e != cudaSuccess) return e;
    }
    // level k (k = 1 .. depth-2, quads at k = depth-2) holds n_chunks * 8^k nodes
    size_t off[12] = {0}, total = 0;
    for (int k = depth - 2; k >= 1; --k) {
        off[k] = total;
        total += (size_t)n_chunks << (3 * k);
    }
    uint64_t *ids = static_cast<uint64_t *>(scratch);
    uint32_t *vals = reinterpret_cast<uint32_t *>(static_cast<char *>(scratch) + total * 8);
    PFN_cuTensorMapEncodeTiled_v12000 encode = tensor_map_encoder();
    if (!encode) return cudaErrorNotSupported;
    const uint64_t side = 1ull << depth;
    const uint32_t es = (uint32_t)(I.vbits / 8);
    CUtensorMap tmap;
    cuuint64_t dims[4] = {side, side, side, n_chunks};
    cuuint64_t strides[3] = {side * es, side * side * es, side * side * side * es};
    cuuint32_t box[4] = {16, 16, 16, 1};
    cuuint32_t estr[4] = {1, 1, 1, 1};
    CUresult r = encode(&tmap, es == 1 ? CU_TENSOR_MAP_DATA_TYPE_UINT8 : CU_TENSOR_MAP_DATA_TYPE_UINT16, 4,
                        const_cast<void *>(grids), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                        CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return cudaErrorInvalidValue;
    uint64_t *q_ids = ids + off[depth - 2];
    uint32_t *q_vals = vals + off[depth - 2];
    auto launch16 = [&](auto kernel, size_t smem) -> cudaError_t {
        cudaError_t e2 = cudaSuccess;
        const int per_sm = prepare_kernel(reinterpret_cast<const void *>(kernel), kQ16Warps * 32, smem, &e2);
        if (e2 != cudaSuccess) return e2;
        uint64_t grid = (uint64_t)num_sms * per_sm;
        const uint64_t need = (((uint64_t)n_chunks << (3 * (depth - 4))) + kQ16Warps - 1) / kQ16Warps;
        if (grid > need) grid = need;
        count_launches(1);
        kernel<<<(unsigned)grid, kQ16Warps * 32, smem, s>>>(I, a, q_ids, q_vals, tmap);
        return cudaGetLastError();
    };
    cudaError_t e = es == 1 ? launch16(dense_quads16_kernel<uint8_t>, Q16Smem<uint8_t>::total)
                            : launch16(dense_quads16_kernel<uint16_t>, Q16Smem<uint16_t>::total);
    if (e != cudaSuccess) return e;
    PendingView P{nullptr, 0, 0};
    if (memo && VX_QUAD_DEFER) {  // the quads that claimed records, one computation per distinct quad
        const size_t smemc = (3 * (size_t)kKeyCache + 256) * 8 + (size_t)kKeyCache * 4;
        auto launchc = [&](auto kernel) -> cudaError_t {
            cudaError_t e2 = cudaSuccess;
            const int per_sm = prepare_kernel(reinterpret_cast<const void *>(kernel), kQ16Warps * 32, smemc, &e2);
            if (e2 != cudaSuccess) return e2;
            count_launches(1);
            return launch_pdl(kernel, dim3((unsigned)(num_sms * per_sm)), dim3(kQ16Warps * 32), smemc, s, I, a);
        };
        e = es == 1 ? launchc(dense_memo_compute_kernel<uint8_t>) : launchc(dense_memo_compute_kernel<uint16_t>);
        if (e != cudaSuccess) return e;
        P = PendingView{a.memo_recs, (uint32_t)memo_stride(es), (uint32_t)(16 * 4 * es)};
    }
    if (levels_begin) (*levels_begin)(levels_ctx);
    for (int k = depth - 3; k >= 3; --k) {  // the first pass reads the quads
        const uint64_t np = (uint64_t)n_chunks << (3 * k);
        e = launch_fresh_level(I, ids + off[k + 1], vals + off[k + 1], ids + off[k], vals + off[k], np, false, trees,
                               changed, s, k == depth - 3 ? P : PendingView{nullptr, 0, 0}, a.count_refs);
        if (e != cudaSuccess) return e;
    }
    // depths 2, 1 and 0 in one launch
    count_launches(1);
    const unsigned wb = (unsigned)((n_chunks + kThreads / 32 - 1) / (kThreads / 32));
    return launch_pdl(fresh_top_kernel, dim3(wb), dim3(kThreads), 0, s, I, (const uint64_t *)(ids + off[3]),
                      (const uint32_t *)(vals + off[3]), n_chunks, trees, changed,
                      depth == 5 ? P : PendingView{nullptr, 0, 0}, a.count_refs);
}

// One level of fresh parents: n_parents = n_chunks * 8^k; children pending in P are resolved first.
static cudaError_t launch_fresh_level(const DevInterner &I, const uint64_t *in_ids, const uint32_t *in_vals,
                                      uint64_t *out_ids, uint32_t *out_vals, uint64_t n_parents, bool is_root,
                                      const uint32_t *trees, uint8_t *changed, cudaStream_t s, PendingView P,
                                      int count_refs) {
    if (n_parents == 0) return cudaSuccess;
    uint64_t blocks = (n_parents + kThreads - 1) / kThreads;
    if (blocks > 65535) blocks = 65535;
    count_launches(1);
    return launch_pdl(fresh_level_kernel, dim3((unsigned)blocks), dim3(kThreads), 0, s, I, in_ids, in_vals, out_ids,
                      out_vals, n_parents, is_root ? 1 : 0, trees, changed, P, count_refs);
}

cudaError_t launch_epoch_refcounts(const DevInterner &I, int num_sms, cudaStream_t s) {
    const size_t smem = I.vbits == 8 ? 256 * 4 : (size_t)2 * kLeafTab * 4;
    count_launches(1);
    cudaError_t e = launch_pdl(epoch_refcount_kernel, dim3(num_sms * 16), dim3(kThreads), smem, s, I);
    if (e != cudaSuccess || VX_REF_FOLD) return e;
    return launch_epoch_finalize(I, s);
}

cudaError_t launch_epoch_finalize(const DevInterner &I, cudaStream_t s) {
    count_launches(1);
    epoch_finalize_kernel<<<1, 1, 0, s>>>(I);
    return cudaGetLastError();
}

}  // namespace vxg
