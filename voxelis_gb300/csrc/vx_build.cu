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
// GB300 mapping: one CTA owns a 32^3 block (or the whole chunk when it is smaller). The block is
// brought into shared memory by one cp.async.bulk copy (TMA bulk engine) completing on an mbarrier,
// then the CTA reduces it level by level entirely in shared memory; only hash-consing touches global
// memory. Warps deduplicate identical 8-voxel groups with __match_any_sync before probing the
// branch table, and inserts are warp-cooperative (vx_device.cuh). Grids are persistent: a multiple
// of the SM count, each CTA striding over blocks.
//
// Refcounts follow from the reference's accounting (interner/mod.rs:712-829): a hash-cons hit gives
// back the references its children were pre-charged with, so after a build every node's count equals
// the number of child slots of newly created nodes that name it, plus one per tree root. That sum is
// computed once per epoch over the allocation log (launch_epoch_refcounts) instead of per lookup.
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

// Leaf id of value v (v != 0): a per-CTA shared cache for 8-bit voxels, the global table otherwise.
template <class T>
__device__ __forceinline__ uint64_t leaf_of(const DevInterner &I, uint64_t *leaf_cache, uint32_t v) {
    if (sizeof(T) == 1) {
        uint64_t id = leaf_cache[v];
        if (id) return id;
        bool created;
        id = intern_leaf(I, v, &created);
        if (id != INVALID_ID) leaf_cache[v] = id;
        return id;
    }
    uint64_t id = ld_volatile(I.leaf_table + v);
    if (id > LEAF_BUSY) return id;
    bool created;
    return intern_leaf(I, v, &created);
}

template <class T>
__global__ void __launch_bounds__(kThreads) dense_blocks_kernel(DevInterner I, DenseArgs a) {
    extern __shared__ __align__(128) unsigned char smem[];
    const int B = a.bdepth;
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
        for (unsigned k = tid; k < 256; k += blockDim.x) leaf_cache[k] = 0;
    if (tid == 0) {
        mbar_init(bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();

    const uint64_t total_blocks = (uint64_t)a.n_chunks * a.blocks_per_chunk;
    const int side = 1 << a.depth;
    uint32_t phase = 0;
    for (uint64_t blk = blockIdx.x; blk < total_blocks; blk += gridDim.x) {
        const uint32_t chunk = (uint32_t)(blk / a.blocks_per_chunk);
        const uint32_t m = (uint32_t)(blk % a.blocks_per_chunk);
        {
            // tree handles may come from device memory: check them before any write
            const uint32_t tree = a.trees[chunk];
            const bool bad = tree >= I.tree_cap || I.depths[tree] != a.depth;
            if (__syncthreads_or(bad)) {
                if (tid == 0) set_error(I, ERR_INVALID, 21);
                continue;
            }
        }
        const T *grid = reinterpret_cast<const T *>(a.grids) + (size_t)chunk * side * side * side;

        // ---- stage the block into shared memory ------------------------------------------------
        if (a.depth == B) {
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
        } else {
            const uint32_t bx = compact3(m), by = compact3(m >> 1), bz = compact3(m >> 2);
            const int rows = S * S;
            const int vec_per_row = S * (int)sizeof(T) / 16;
            for (int r = tid; r < rows * vec_per_row; r += blockDim.x) {
                const int row = r / vec_per_row, v = r % vec_per_row;
                const int y = row / S, z = row % S;
                const T *src = grid + ((size_t)(by * S + y) * side + (bz * S + z)) * side + bx * S;
                reinterpret_cast<uint4 *>(vox + (size_t)row * S)[v] = __ldcs(reinterpret_cast<const uint4 *>(src) + v);
            }
            __syncthreads();
        }

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

        // ---- block result -------------------------------------------------------------------
        if (tid == 0) {
            const uint64_t root = lvl[0];
            if (a.depth == B) {
                const uint32_t tree = a.trees[chunk];
                if (root != EMPTY_ID) {
                    I.roots[tree] = root;
                    atomicAdd(I.refcount + id_index(root), 1u);
                }
                if (a.changed) a.changed[chunk] = root != EMPTY_ID;
            } else {
                a.block_roots[blk] = root;
                a.block_vals[blk] = lval[0];
            }
        }
        __syncthreads();
    }
}

__global__ void __launch_bounds__(kThreads) fresh_level_kernel(DevInterner I, const uint64_t *in_ids,
                                                               const uint32_t *in_vals, uint64_t *out_ids,
                                                               uint32_t *out_vals, uint64_t n_parents, int is_root,
                                                               const uint32_t *trees, uint8_t *changed) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t base = (uint64_t)blockIdx.x * blockDim.x; base < n_parents; base += stride) {
        const uint64_t p = base + threadIdx.x;
        const bool in = p < n_parents;
        uint64_t c[8];
        uint32_t cv[8];
        uint32_t types = 0, mask = 0;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            c[k] = in ? in_ids[8 * p + k] : 0;
            cv[k] = in ? in_vals[8 * p + k] : 0;
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
        if (!in) continue;
        uint64_t out = mask == 0 ? EMPTY_ID : (same ? c[0] : id);
        uint32_t val = mask == 0 ? 0 : (same ? cv[0] : lod);
        if (is_root) {
            const uint32_t tree = trees[p];
            if (tree >= I.tree_cap) {
                set_error(I, ERR_INVALID, 22);
                continue;
            }
            if (out != EMPTY_ID) {
                I.roots[tree] = out;
                atomicAdd(I.refcount + id_index(out), 1u);
            }
            if (changed) changed[p] = out != EMPTY_ID;
        } else {
            out_ids[p] = out;
            out_vals[p] = val;
        }
    }
}

// Adds one reference per child slot of every node created in this epoch. Leaf children of 8-bit
// interners are first summed per value in shared memory (a handful of leaves is named by most
// bottom branches).
__global__ void __launch_bounds__(kThreads) epoch_refcount_kernel(DevInterner I) {
    __shared__ uint32_t leaf_cnt[256];
    const bool small = I.vbits == 8;
    if (small)
        for (unsigned k = threadIdx.x; k < 256; k += blockDim.x) leaf_cnt[k] = 0;
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
            if (small && id_is_leaf(c[k]))
                atomicAdd(&leaf_cnt[node_value(I, id_index(c[k]))], cnt);
            else
                atomicAdd(I.refcount + id_index(c[k]), cnt);
        }
    }
    __syncthreads();
    if (small)
        for (unsigned v = threadIdx.x; v < 256; v += blockDim.x)
            if (leaf_cnt[v]) {
                const uint64_t lid = I.leaf_table[v];
                if (lid > LEAF_BUSY)
                    atomicAdd(I.refcount + id_index(lid), leaf_cnt[v]);
                else
                    set_error(I, ERR_INTERNAL, 30);
            }
}

__global__ void epoch_finalize_kernel(DevInterner I) {
    DevCounters *c = I.ctr;
    const unsigned long long alloc = c->alloc_count, fc = c->free_count;
    const unsigned long long used_free = alloc < fc ? alloc : fc;
    c->free_count = fc - used_free;
    unsigned long long ni = c->next_index + (alloc - used_free);
    if (ni > I.capacity) ni = I.capacity;
    c->next_index = ni;
    c->alloc_count = 0;
}

}  // namespace

size_t dense_smem_bytes(int bdepth, int vbytes) {
    const size_t V = (size_t)1 << (3 * bdepth);
    const size_t n_nodes = (V - 1) / 7;
    const size_t vox = (V * vbytes + 127) & ~(size_t)127;
    return vox + n_nodes * 8 + ((n_nodes + 1) & ~(size_t)1) * 4 + 256 * 8 + 16;
}

cudaError_t launch_dense_blocks(const DevInterner &I, const DenseArgs &a, int num_sms, cudaStream_t s) {
    const size_t smem = dense_smem_bytes(a.bdepth, I.vbits / 8);
    const uint64_t total = (uint64_t)a.n_chunks * a.blocks_per_chunk;
    if (total == 0) return cudaSuccess;
    int per_sm = 1;
    cudaError_t e;
    if (I.vbits == 8) {
        e = cudaFuncSetAttribute(dense_blocks_kernel<uint8_t>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, dense_blocks_kernel<uint8_t>, kThreads, smem);
    } else {
        e = cudaFuncSetAttribute(dense_blocks_kernel<uint16_t>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, dense_blocks_kernel<uint16_t>, kThreads, smem);
    }
    if (per_sm < 1) per_sm = 1;
    uint64_t grid = (uint64_t)num_sms * per_sm;
    if (grid > total) grid = total;
    count_launches(1);
    if (I.vbits == 8)
        dense_blocks_kernel<uint8_t><<<(unsigned)grid, kThreads, smem, s>>>(I, a);
    else
        dense_blocks_kernel<uint16_t><<<(unsigned)grid, kThreads, smem, s>>>(I, a);
    return cudaGetLastError();
}

cudaError_t launch_fresh_level(const DevInterner &I, const uint64_t *in_ids, const uint32_t *in_vals,
                               uint64_t *out_ids, uint32_t *out_vals, uint64_t n_parents, bool is_root,
                               const uint32_t *trees, uint8_t *changed, cudaStream_t s) {
    if (n_parents == 0) return cudaSuccess;
    uint64_t blocks = (n_parents + kThreads - 1) / kThreads;
    if (blocks > 65535) blocks = 65535;
    count_launches(1);
    fresh_level_kernel<<<(unsigned)blocks, kThreads, 0, s>>>(I, in_ids, in_vals, out_ids, out_vals, n_parents,
                                                             is_root ? 1 : 0, trees, changed);
    return cudaGetLastError();
}

cudaError_t launch_epoch_refcounts(const DevInterner &I, int num_sms, cudaStream_t s) {
    count_launches(1);
    epoch_refcount_kernel<<<num_sms * 2, kThreads, 0, s>>>(I);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    return launch_epoch_finalize(I, s);
}

cudaError_t launch_epoch_finalize(const DevInterner &I, cudaStream_t s) {
    count_launches(1);
    epoch_finalize_kernel<<<1, 1, 0, s>>>(I);
    return cudaGetLastError();
}

}  // namespace vxg
