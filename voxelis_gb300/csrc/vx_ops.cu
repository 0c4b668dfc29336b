// Batched reads, releases, single-voxel edits and table maintenance.
//
//   get_many      VoxTree::get -> get_at_depth (voxtree.rs:145-159, utils/common.rs:122-156), one
//                 thread per query descending at most d levels through the L2-resident node array.
//   release       dec_ref_recursive (interner/mod.rs:419-534) for many roots at once, breadth
//                 first: a round decrements the children of the nodes that died in the previous
//                 round; a child whose count reaches zero dies in the next round. Dead nodes leave
//                 their table, are cleared, get a new generation and go on the free list
//                 (recycle, interner/mod.rs:566-625).
//   set / fill    VoxTree::set (voxtree.rs:163-260, 393-706) and fill/clear (voxtree.rs:264-292)
//                 run by a single thread with the reference's own refcount order (hit: give back
//                 the children's references, interner/mod.rs:767-772), its LIFO free list and its
//                 32768-entry release queue (P3 lifts the limit).
//   rehash        rebuilds the branch table from the live nodes once tombstones accumulate.
#include "vx_launch.h"

namespace vxg {
namespace {

constexpr int kThreads = 256;

template <class T>
__global__ void __launch_bounds__(kThreads) get_kernel(DevInterner I, uint64_t n, const uint32_t *trees,
                                                      const int32_t *xyz, uint8_t *found, T *values) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    bool oob = false, bad = false;
    for (uint64_t q = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += stride) {
        const uint32_t t = __ldg(trees + q);
        const int d = t < I.tree_cap ? I.depths[t] : TREE_UNUSED;
        const int32_t x = __ldg(xyz + 3 * q), y = __ldg(xyz + 3 * q + 1), z = __ldg(xyz + 3 * q + 2);
        uint32_t val = 0;
        uint8_t f = 0;
        if (d == TREE_UNUSED) {
            bad = true;
        } else if (x < 0 || y < 0 || z < 0 || x >= (1 << d) || y >= (1 << d) || z >= (1 << d)) {
            oob = true;
        } else {
            uint64_t node = I.roots[t];
            int depth = 0;
            while (node != EMPTY_ID) {
                if (depth >= d) {
                    const uint32_t v = node_value(I, id_index(node));
                    if (v != 0) {
                        val = v;
                        f = 1;
                    }
                    break;
                }
                if (id_is_branch(node)) {
                    const int shift = d - depth - 1;
                    const uint32_t ci = ((x >> shift) & 1) | (((y >> shift) & 1) << 1) | (((z >> shift) & 1) << 2);
                    node = __ldg(reinterpret_cast<const unsigned long long *>(I.children) + 8ull * id_index(node) + ci);
                    ++depth;
                } else {
                    val = node_value(I, id_index(node));
                    f = 1;
                    break;
                }
            }
        }
        found[q] = f;
        values[q] = (T)val;
    }
    if (oob) set_error(I, ERR_OOB, 50);
    if (bad) set_error(I, ERR_INVALID, 51);
}

// ---- release (bodies in vx_device.cuh, shared with the single-launch apply) ------------------------
__global__ void __launch_bounds__(kThreads) release_roots_kernel(DevInterner I, const uint64_t *list,
                                                                uint32_t *out) {
    pdl_wait();
    pdl_release();
    release_roots_range(I, list, out, &I.ctr->scratch[SC_REL_OUT], (uint64_t)blockIdx.x * blockDim.x,
                        (uint64_t)gridDim.x * blockDim.x);
    if (grid_last_cta(&I.ctr->scratch[SC_DONE])) release_advance(I);
}

__global__ void __launch_bounds__(kThreads) release_round_kernel(DevInterner I, const uint32_t *in, uint32_t *out) {
    pdl_wait();
    pdl_release();
    release_round_range(I, in, out, &I.ctr->scratch[SC_REL_IN], &I.ctr->scratch[SC_REL_OUT],
                        (uint64_t)blockIdx.x * blockDim.x, (uint64_t)gridDim.x * blockDim.x);
    if (grid_last_cta(&I.ctr->scratch[SC_DONE])) release_advance(I);
}

__global__ void release_advance_kernel(DevInterner I) { pdl_wait(); pdl_release(); release_advance(I); }

// ---- single-thread reference-order operations ---------------------------------------------------
struct Seq {
    DevInterner I;
    uint64_t *queue;
    uint64_t queue_cap;
    bool ok;
};

__device__ uint32_t seq_alloc(Seq &S) {
    DevCounters *c = S.I.ctr;
    if (c->free_count > 0) {
        c->free_count -= 1;
        c->created += 1;
        return S.I.free_list[c->free_count];
    }
    if (c->next_index >= S.I.capacity) {
        set_error(S.I, ERR_OOM, 70);
        S.ok = false;
        return NO_NODE;
    }
    c->created += 1;
    return (uint32_t)(c->next_index++);
}

__device__ void seq_recycle(Seq &S, uint32_t idx) {
    const bool branch = id_is_branch(S.I.ids[idx]);
    recycle_node(S.I, idx, S.I.ctr->free_count);
    S.I.ctr->free_count += 1;
    if (branch) S.I.ctr->tombstones += 1;
}

__device__ bool seq_valid(Seq &S, uint64_t id) {
    const uint32_t i = id_index(id);
    return i < S.I.capacity && S.I.generation[i] == id_generation(id);
}

__device__ void seq_dec(Seq &S, uint64_t id) {  // dec_ref (interner/mod.rs:260-296)
    const uint32_t i = id_index(id);
    if (S.I.refcount[i] == 0) {
        set_error(S.I, ERR_REF_UB, 71);
        S.ok = false;
        return;
    }
    S.I.refcount[i] -= 1;
    if (S.I.refcount[i] == 0) seq_recycle(S, i);
}

// get_or_create_leaf (interner/mod.rs:627-710)
__device__ uint64_t seq_leaf(Seq &S, uint32_t v) {
    const uint64_t s = S.I.leaf_table[v];
    if (s > LEAF_BUSY) {
        S.I.refcount[id_index(s)] += 1;
        return s;
    }
    const uint32_t idx = seq_alloc(S);
    if (idx == NO_NODE) return INVALID_ID;
    const uint64_t id = make_leaf_id(idx, S.I.generation[idx]);
    set_node_value(S.I, idx, v);
    S.I.hash[idx] = 0;
    S.I.ids[idx] = id;
    S.I.refcount[idx] = 1;
    S.I.leaf_table[v] = id;
    return id;
}

// get_or_create_branch (interner/mod.rs:712-829)
__device__ uint64_t seq_branch(Seq &S, const uint64_t c[8], uint32_t types, uint32_t mask) {
    const DevInterner &I = S.I;
    const uint64_t h = branch_fingerprint(c, (types << 8) | mask);
    const uint32_t tag = slot_tag(h);
    uint64_t pos = h & I.table_mask;
    for (uint32_t p = 0; p <= I.max_probes; ++p, pos = (pos + 1) & I.table_mask) {
        const uint64_t s = I.table[pos];
        if (s == SLOT_EMPTY) {
            const uint32_t idx = seq_alloc(S);
            if (idx == NO_NODE) return INVALID_ID;
            uint32_t cv[8];
            for (int k = 0; k < 8; ++k) cv[k] = node_value(I, id_index(c[k]));
            const uint64_t id = write_branch(I, idx, c, types, mask, h, calc_average8(cv));
            I.refcount[idx] = 1;
            I.table[pos] = make_slot(tag, idx);
            return id;
        }
        if ((uint32_t)(s >> 32) == tag && s != SLOT_TOMB && key_equal(I, (uint32_t)s, c, types, mask)) {
            const uint64_t existing = I.ids[(uint32_t)s];
            for (int k = 0; k < 8; ++k)
                if (c[k] != EMPTY_ID) seq_dec(S, c[k]);
            I.refcount[(uint32_t)s] += 1;
            return existing;
        }
    }
    set_error(I, ERR_TABLE_FULL, 72);
    S.ok = false;
    return INVALID_ID;
}

// dec_ref_recursive (interner/mod.rs:419-534) with its fixed queue (grown under P3).
__device__ void seq_release(Seq &S, uint64_t root) {
    const DevInterner &I = S.I;
    uint64_t r = 0, w = 1;
    S.queue[0] = root;
    while (r < w && S.ok) {
        const uint64_t cur = S.queue[r++];
        const uint32_t ci = id_index(cur);
        if (I.refcount[ci] == 0) {
            set_error(I, ERR_REF_UB, 73);
            S.ok = false;
            return;
        }
        I.refcount[ci] -= 1;
        if (I.refcount[ci] != 0) continue;
        for (int k = 0; k < 8; ++k) {
            const uint64_t child = I.children[8ull * ci + k];
            if (child == EMPTY_ID) continue;
            const uint32_t k2 = id_index(child);
            if (I.refcount[k2] > 1) {
                I.refcount[k2] -= 1;
            } else {
                if (w >= S.queue_cap) {
                    set_error(I, ERR_REF_UB, 74);  // release queue overflow (interner/mod.rs:509-513)
                    S.ok = false;
                    return;
                }
                S.queue[w++] = child;
            }
        }
        seq_recycle(S, ci);
    }
}

__device__ __forceinline__ uint32_t cidx(int32_t x, int32_t y, int32_t z, int cur, int max) {
    const int sh = max - cur - 1;
    return ((x >> sh) & 1) | (((y >> sh) & 1) << 1) | (((z >> sh) & 1) << 2);
}

// set_at_depth_iterative (voxtree.rs:393-540)
__device__ uint64_t seq_set(Seq &S, uint64_t root, int32_t x, int32_t y, int32_t z, int d, uint32_t voxel) {
    const DevInterner &I = S.I;
    uint64_t st_node[11], st_leaf[11];
    uint32_t st_idx[11];
    uint64_t cur = root, leaf = EMPTY_ID;
    int depth = 0;
    while (depth < d) {
        const uint32_t index = cidx(x, y, z, depth, d);
        if (id_is_branch(cur)) {
            st_node[depth] = cur;
            st_leaf[depth] = leaf;
            st_idx[depth] = index;
            cur = I.children[8ull * id_index(cur) + index];
        } else {
            if (node_value(I, id_index(cur)) == voxel) return INVALID_ID;
            leaf = cur;
            cur = EMPTY_ID;
            st_node[depth] = cur;
            st_leaf[depth] = leaf;
            st_idx[depth] = index;
        }
        ++depth;
    }
    if (id_is_leaf(cur) && node_value(I, id_index(cur)) == voxel) return INVALID_ID;
    cur = seq_leaf(S, voxel);
    while (depth > 0 && S.ok) {
        --depth;
        const uint64_t pn = st_node[depth], pl = st_leaf[depth];
        const uint32_t pi = st_idx[depth];
        if (pn != EMPTY_ID) {
            const uint32_t types = id_types(pn) | ((id_is_leaf(cur) ? 1u : 0u) << pi);
            uint64_t br[8];
            for (int k = 0; k < 8; ++k) br[k] = I.children[8ull * id_index(pn) + k];
            br[pi] = cur;
            bool same = types == 0xFF;
            for (int k = 0; k < 8; ++k) same = same && br[k] == cur;
            if (!same) {
                const uint32_t mask = id_mask(pn) | (1u << pi);
                for (int k = 0; k < 8; ++k)
                    if (k != (int)pi && br[k] != EMPTY_ID) I.refcount[id_index(br[k])] += 1;
                cur = seq_branch(S, br, types, mask);
            }
        } else if (pl == EMPTY_ID) {
            uint64_t ch[8] = {0, 0, 0, 0, 0, 0, 0, 0};
            ch[pi] = cur;
            cur = seq_branch(S, ch, (id_is_leaf(cur) ? 1u : 0u) << pi, 1u << pi);
        } else {
            uint64_t ch[8];
            for (int k = 0; k < 8; ++k) ch[k] = pl;
            I.refcount[id_index(pl)] += 7;
            ch[pi] = cur;
            const uint32_t types = ((~(1u << pi)) | ((id_is_leaf(cur) ? 1u : 0u) << pi)) & 0xFFu;
            cur = seq_branch(S, ch, types, 0xFF);
        }
    }
    return cur;
}

// remove_at_depth / _branch / _leaf (voxtree.rs:542-706), unrolled into a descent and an ascent.
__device__ uint64_t seq_remove(Seq &S, uint64_t root, int32_t x, int32_t y, int32_t z, int d) {
    const DevInterner &I = S.I;
    uint64_t frames[11];
    int depth = 0;
    uint64_t node = root;
    uint64_t result;
    while (true) {
        if (!seq_valid(S, node)) {
            set_error(I, ERR_REF_PANIC, 75);
            S.ok = false;
            return INVALID_ID;
        }
        if (id_is_branch(node)) {
            if (!(depth < d)) {
                set_error(I, ERR_REF_PANIC, 76);  // "Branch node at max depth"
                S.ok = false;
                return INVALID_ID;
            }
            const uint32_t index = cidx(x, y, z, depth, d);
            if (!((id_mask(node) >> index) & 1)) return INVALID_ID;
            frames[depth] = node;
            node = I.children[8ull * id_index(node) + index];
            ++depth;
            continue;
        }
        // remove_at_depth_leaf from `depth` down to d, built bottom-up
        result = EMPTY_ID;
        for (int k = d - 1; k >= depth && S.ok; --k) {
            const uint32_t index = cidx(x, y, z, k, d);
            uint64_t ch[8];
            for (int j = 0; j < 8; ++j) ch[j] = node;
            ch[index] = result;
            const bool lf = id_is_leaf(result), em = result == EMPTY_ID;
            const uint32_t types = ((~(1u << index)) | ((lf ? 1u : 0u) << index)) & 0xFFu;
            const uint32_t mask = ((~(1u << index)) | ((!em ? 1u : 0u) << index)) & 0xFFu;
            I.refcount[id_index(node)] += 7;
            result = seq_branch(S, ch, types, mask);
        }
        break;
    }
    // ascend through the branch frames (remove_at_depth_branch)
    while (depth > 0 && S.ok) {
        --depth;
        const uint64_t pn = frames[depth];
        const uint32_t index = cidx(x, y, z, depth, d);
        const bool empty = result == EMPTY_ID;
        const uint32_t mask = empty ? (id_mask(pn) & ~(1u << index)) : id_mask(pn);
        if (mask == 0) {
            result = EMPTY_ID;
            continue;
        }
        if (!id_is_branch(result)) {
            set_error(I, ERR_REF_PANIC, 77);  // "Removing voxel should never produce a leaf node"
            S.ok = false;
            return INVALID_ID;
        }
        const uint32_t types = id_types(pn) & ~(1u << index);
        uint64_t br[8];
        for (int k = 0; k < 8; ++k) br[k] = I.children[8ull * id_index(pn) + k];
        br[index] = result;
        for (int k = 0; k < 8; ++k)
            if (k != (int)index && br[k] != EMPTY_ID) I.refcount[id_index(br[k])] += 1;
        result = seq_branch(S, br, types, mask);
    }
    return result;
}

// VoxTree::set (voxtree.rs:163-260). status: 0 unchanged, 1 changed, -1 error.
__global__ void tree_set_kernel(DevInterner I, uint32_t tree, int32_t x, int32_t y, int32_t z, uint32_t v,
                                uint64_t *queue, uint64_t queue_cap, int *status) {
    Seq S{I, queue, queue_cap, true};
    const uint64_t root = I.roots[tree];
    const int d = I.depths[tree];
    *status = 0;
    if (root == EMPTY_ID && v == 0) return;
    const uint64_t nw = v != 0 ? seq_set(S, root, x, y, z, d, v) : seq_remove(S, root, x, y, z, d);
    if (!S.ok) {
        *status = -1;
        return;
    }
    if (nw == INVALID_ID) return;
    if (root != EMPTY_ID) {
        if (nw == root) {
            set_error(I, ERR_REF_PANIC, 78);
            *status = -1;
            return;
        }
        seq_release(S, root);
        if (!S.ok) {
            *status = -1;
            return;
        }
    }
    I.roots[tree] = nw;
    *status = 1;
}

// ---- many VoxTree::set calls at once (vx_trees_set_many) ------------------------------------------
// The calls of one tree run in call order, one warp per tree and trees in parallel. Each call is the
// reference's set_at_depth_iterative / remove_at_depth (voxtree.rs:393-706) on the tree's current
// root, so every node it creates, including the stale types bits of the set path (the old parent's
// types ORed with the new child's leaf bit, voxtree.rs:513-514), is the node the reference creates.
// All 32 lanes run the same sequence on the same values (loads of one address are one transaction);
// lane 0 interns, through the concurrent leaf and branch inserts, and broadcasts. Refcounts are not
// touched during the calls and nothing is released: every node stays valid until the call ends, and
// a call that finds a node made by an earlier call gets the same node the reference would recreate.
// Afterwards the epoch refcount kernel counts one reference per child slot of every created node,
// the trees take their final roots (+1) and release their first ones, and created nodes that ended
// unreferenced (the intermediate roots and paths) are released, which leaves the refcounts the
// reference's per-call inc/dec bookkeeping gives.
struct WSeq {
    const DevInterner &I;
    bool ok;
};

__device__ __forceinline__ uint64_t wchild(const DevInterner &I, uint64_t id, uint32_t k) {
    return __ldcg((const unsigned long long *)(I.children + 8ull * id_index(id) + k));
}

__device__ uint64_t wleaf(WSeq &S, uint32_t v) {
    uint64_t id = EMPTY_ID;
    if ((threadIdx.x & 31u) == 0) {
        bool created;
        id = intern_leaf(S.I, v, &created);
    }
    id = __shfl_sync(0xFFFFFFFFu, id, 0);
    if (id == EMPTY_ID) S.ok = false;
    return id;
}

__device__ uint64_t wbranch(WSeq &S, const uint64_t c[8], uint32_t types, uint32_t mask) {
    uint32_t cv[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) cv[k] = c[k] ? node_value_cg(S.I, id_index(c[k])) : 0u;
    bool created;
    uint64_t id = warp_intern_branch(S.I, (threadIdx.x & 31u) == 0, c, types & 0xFFu, mask & 0xFFu,
                                     calc_average8(cv), &created);
    id = __shfl_sync(0xFFFFFFFFu, id, 0);
    if (id == EMPTY_ID) S.ok = false;
    return id;
}

// set_at_depth_iterative (voxtree.rs:393-540)
__device__ uint64_t wset(WSeq &S, uint64_t root, int32_t x, int32_t y, int32_t z, int d, uint32_t voxel) {
    const DevInterner &I = S.I;
    uint64_t st_node[11], st_leaf[11];
    uint32_t st_idx[11];
    uint64_t cur = root, leaf = EMPTY_ID;
    int depth = 0;
    while (depth < d) {
        const uint32_t index = cidx(x, y, z, depth, d);
        if (id_is_branch(cur)) {
            st_node[depth] = cur;
            st_leaf[depth] = leaf;
            cur = wchild(I, cur, index);
        } else {
            if (node_value_cg(I, id_index(cur)) == voxel) return INVALID_ID;
            leaf = cur;
            cur = EMPTY_ID;
            st_node[depth] = cur;
            st_leaf[depth] = leaf;
        }
        st_idx[depth] = index;
        ++depth;
    }
    if (id_is_leaf(cur) && node_value_cg(I, id_index(cur)) == voxel) return INVALID_ID;
    cur = wleaf(S, voxel);
    while (depth > 0 && S.ok) {
        --depth;
        const uint64_t pn = st_node[depth], pl = st_leaf[depth];
        const uint32_t pi = st_idx[depth];
        const uint32_t lbit = (id_is_leaf(cur) ? 1u : 0u) << pi;
        uint64_t br[8];
        if (pn != EMPTY_ID) {
            const uint32_t types = id_types(pn) | lbit;
            for (int k = 0; k < 8; ++k) br[k] = wchild(I, pn, k);
            br[pi] = cur;
            bool same = types == 0xFF;
            for (int k = 0; k < 8; ++k) same = same && br[k] == cur;
            if (!same) cur = wbranch(S, br, types, id_mask(pn) | (1u << pi));
        } else if (pl == EMPTY_ID) {
            for (int k = 0; k < 8; ++k) br[k] = EMPTY_ID;
            br[pi] = cur;
            cur = wbranch(S, br, lbit, 1u << pi);
        } else {
            for (int k = 0; k < 8; ++k) br[k] = pl;
            br[pi] = cur;
            cur = wbranch(S, br, ~(1u << pi) | lbit, 0xFFu);
        }
    }
    return cur;
}

// remove_at_depth / _branch / _leaf (voxtree.rs:542-706)
__device__ uint64_t wremove(WSeq &S, uint64_t root, int32_t x, int32_t y, int32_t z, int d) {
    const DevInterner &I = S.I;
    uint64_t frames[11];
    int depth = 0;
    uint64_t node = root, result = EMPTY_ID;
    while (id_is_branch(node)) {
        if (depth >= d) {
            set_error(I, ERR_REF_PANIC, 80);  // "Branch node at max depth"
            S.ok = false;
            return INVALID_ID;
        }
        const uint32_t index = cidx(x, y, z, depth, d);
        if (!((id_mask(node) >> index) & 1u)) return INVALID_ID;
        frames[depth] = node;
        node = wchild(I, node, index);
        ++depth;
    }
    for (int k = d - 1; k >= depth && S.ok; --k) {  // remove_at_depth_leaf, built bottom-up
        const uint32_t index = cidx(x, y, z, k, d);
        uint64_t ch[8];
        for (int j = 0; j < 8; ++j) ch[j] = node;
        ch[index] = result;
        const uint32_t types = ~(1u << index) | ((id_is_leaf(result) ? 1u : 0u) << index);
        const uint32_t mask = ~(1u << index) | ((result != EMPTY_ID ? 1u : 0u) << index);
        result = wbranch(S, ch, types, mask);
    }
    while (depth > 0 && S.ok) {  // remove_at_depth_branch on the way up
        --depth;
        const uint64_t pn = frames[depth];
        const uint32_t index = cidx(x, y, z, depth, d);
        const uint32_t mask = result == EMPTY_ID ? (id_mask(pn) & ~(1u << index)) : id_mask(pn);
        if (mask == 0) {
            result = EMPTY_ID;
            continue;
        }
        if (!id_is_branch(result)) {
            set_error(I, ERR_REF_PANIC, 81);  // "Removing voxel should never produce a leaf node"
            S.ok = false;
            return INVALID_ID;
        }
        uint64_t br[8];
        for (int k = 0; k < 8; ++k) br[k] = wchild(I, pn, k);
        br[index] = result;
        result = wbranch(S, br, id_types(pn) & ~(1u << index), mask);
    }
    return result;
}

// One warp per tree group g: calls [begin[g], begin[g+1]) in call order.
__global__ void __launch_bounds__(kThreads) trees_set_kernel(DevInterner I, const SetCalls c) {
    if (blockIdx.x == 0 && threadIdx.x == 0) I.ctr->scratch[SC_RELEASE] = 0;
    const uint32_t warps = gridDim.x * (blockDim.x / 32);
    for (uint32_t g = (blockIdx.x * blockDim.x + threadIdx.x) / 32; g < c.n_groups; g += warps) {
        const uint32_t tree = c.group_tree[g];
        const int d = I.depths[tree];
        uint64_t root = I.roots[tree];
        WSeq S{I, true};
        for (uint32_t k = c.begin[g]; k < c.begin[g + 1] && S.ok; ++k) {
            const int32_t x = c.xyz[3 * k], y = c.xyz[3 * k + 1], z = c.xyz[3 * k + 2];
            const uint32_t v = c.values[k];
            uint8_t changed = 0;
            if (root != EMPTY_ID || v != 0) {
                const uint64_t nw = v != 0 ? wset(S, root, x, y, z, d, v) : wremove(S, root, x, y, z, d);
                if (!S.ok) break;
                if (nw != INVALID_ID) {
                    if (root != EMPTY_ID && nw == root) {  // assert_ne!(new_root_id, self.root_id)
                        set_error(I, ERR_REF_PANIC, 82);
                        break;
                    }
                    root = nw;
                    changed = 1;
                }
            }
            if ((threadIdx.x & 31u) == 0 && c.changed) c.changed[c.order[k]] = changed;
        }
        if ((threadIdx.x & 31u) == 0) c.new_root[g] = root;
    }
}

// The trees take their final roots (one reference each) and list their first roots for release.
__global__ void __launch_bounds__(kThreads) trees_set_roots_kernel(DevInterner I, const SetCalls c, uint64_t *list) {
    for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < c.n_groups; g += gridDim.x * blockDim.x) {
        const uint32_t tree = c.group_tree[g];
        const uint64_t old = I.roots[tree], nw = c.new_root[g];
        if (nw == old) continue;
        I.roots[tree] = nw;
        if (nw != EMPTY_ID) atomicAdd(I.refcount + id_index(nw), 1u);
        if (old != EMPTY_ID) list[atomicAdd(&I.ctr->scratch[SC_RELEASE], 1ull)] = old;
    }
}

// Created nodes left without a reference are listed for release with a count of one. The created
// slots are free_list[free_count .. fc0) and [ni0, next_index) once the epoch is closed.
__global__ void __launch_bounds__(kThreads) trees_set_garbage_kernel(DevInterner I, unsigned long long fc0,
                                                                    unsigned long long ni0, uint64_t *list) {
    const unsigned long long fc = I.ctr->free_count, ni = I.ctr->next_index;
    const unsigned long long n_free = fc0 - fc, n = n_free + (ni - ni0);
    for (unsigned long long t = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; t < n;
         t += (unsigned long long)gridDim.x * blockDim.x) {
        const uint32_t idx = t < n_free ? I.free_list[fc + t] : (uint32_t)(ni0 + (t - n_free));
        const uint64_t id = I.ids[idx];
        if (id == EMPTY_ID || I.refcount[idx] != 0) continue;
        I.refcount[idx] = 1;
        list[atomicAdd(&I.ctr->scratch[SC_RELEASE], 1ull)] = id;
    }
}

// VoxTree::fill / clear (voxtree.rs:264-292). status: 1 if the tree was dirtied.
__global__ void tree_fill_kernel(DevInterner I, uint32_t tree, uint32_t v, uint64_t *queue, uint64_t queue_cap,
                                 int *status) {
    Seq S{I, queue, queue_cap, true};
    const uint64_t root = I.roots[tree];
    *status = 0;
    if (root != EMPTY_ID) {
        seq_release(S, root);
        if (!S.ok) {
            *status = -1;
            return;
        }
        I.roots[tree] = EMPTY_ID;
        *status = 1;
    }
    if (v != 0) {
        const uint64_t leaf = seq_leaf(S, v);
        if (!S.ok) {
            *status = -1;
            return;
        }
        I.roots[tree] = leaf;
        *status = 1;
    }
}

// ---- maintenance -------------------------------------------------------------------------------
__global__ void rehash_kernel(DevInterner I) {
    const unsigned long long n = I.ctr->next_index;
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    for (unsigned long long idx = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x + 1; idx < n;
         idx += stride) {
        const uint64_t id = I.ids[idx];
        if (id == 0 || id_is_leaf(id)) continue;
        const uint64_t h = I.hash[idx];
        uint64_t pos = h & I.table_mask;
        const uint64_t slot = make_slot(slot_tag(h), (uint32_t)idx);
        bool placed = false;
        for (uint32_t p = 0; p <= I.max_probes; ++p, pos = (pos + 1) & I.table_mask)
            if (atomicCAS((unsigned long long *)(I.table + pos), SLOT_EMPTY, slot) == SLOT_EMPTY) {
                placed = true;
                break;
            }
        if (!placed) set_error(I, ERR_TABLE_FULL, 80);
    }
}

__global__ void rehash_done_kernel(DevInterner I) { I.ctr->tombstones = 0; }

__global__ void count_live_kernel(DevInterner I, unsigned long long *out2) {
    const unsigned long long n = I.ctr->next_index;
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    unsigned long long br = 0, lf = 0;
    for (unsigned long long idx = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x + 1; idx < n;
         idx += stride) {
        const uint64_t id = I.ids[idx];
        if (id == 0) continue;
        if (id_is_leaf(id))
            ++lf;
        else
            ++br;
    }
    for (int o = 16; o > 0; o >>= 1) {
        br += __shfl_down_sync(0xFFFFFFFFu, br, o);
        lf += __shfl_down_sync(0xFFFFFFFFu, lf, o);
    }
    if ((threadIdx.x & 31) == 0) {
        if (br) atomicAdd(out2, br);
        if (lf) atomicAdd(out2 + 1, lf);
    }
}


// ---- to_vec: DAG -> dense grid (utils/common.rs:158-246) ----------------------------------------
// One CTA per cube of side C = 2^lc (lc = min(d, 5)) of one tree; cubes are ordered (tree, cy, cz,
// cx), so a run of whole cy-slabs is one contiguous range of the output. Thread 0 descends from the
// root to the cube's root (d - lc levels); EMPTY or a leaf met on the way, or as the cube root, makes
// the cube uniform (EMPTY children are never visited by to_vec, leaving the default; a leaf fills
// its whole sub-cube). Otherwise the cube's subtree is expanded level by level in shared memory,
// 8^k ids at level k in Morton order, a leaf or EMPTY replicating into its 8 children; the last
// level resolves each voxel to the value of the node covering it (a leaf's value, or the value of a
// node at depth d, as to_vec's else-branch does) and the CTA writes the cube row by row with 16-byte
// stores.
constexpr int kDenseOutThreads = 256;

__device__ __forceinline__ uint32_t morton_compact3(uint32_t m) {
    m &= 0x09249249u;
    m = (m ^ (m >> 2)) & 0x030C30C3u;
    m = (m ^ (m >> 4)) & 0x0300F00Fu;
    m = (m ^ (m >> 8)) & 0x030000FFu;
    m = (m ^ (m >> 16)) & 0x000003FFu;
    return m;
}

template <class T>
__device__ __forceinline__ uint4 replicate16(uint32_t v) {
    uint32_t w = sizeof(T) == 1 ? (v & 0xFFu) * 0x01010101u : (v & 0xFFFFu) * 0x00010001u;
    return make_uint4(w, w, w, w);
}

template <class T>
__global__ void __launch_bounds__(kDenseOutThreads) to_dense_kernel(DevInterner I, const uint32_t *trees, int d,
                                                                     int lc, uint64_t cube_begin, uint64_t n_cubes,
                                                                     T *out) {
    extern __shared__ __align__(16) unsigned char smem[];
    const uint32_t C = 1u << lc;
    const uint32_t K = 1u << (d - lc);          // cubes per axis
    const uint64_t K2 = (uint64_t)K * K, K3 = K2 * K;
    const uint64_t S = 1ull << d;
    const uint64_t slab_elems = (uint64_t)C * S * S;
    const uint32_t tile_elems = C * C * C;
    T *tile = reinterpret_cast<T *>(smem);
    uint64_t *lv_big = reinterpret_cast<uint64_t *>(smem + ((tile_elems * sizeof(T) + 15) & ~15u));
    uint64_t *lv_small = lv_big + (lc >= 1 ? (1u << (3 * (lc - 1))) : 1u);
    __shared__ uint64_t cube_root;
    __shared__ int uniform;  // 1: whole cube = cube_val
    __shared__ uint32_t cube_val;
    const uint64_t first_slab = cube_begin / K2;
    bool bad = false;
    for (uint64_t c = cube_begin + blockIdx.x; c < cube_begin + n_cubes; c += gridDim.x) {
        const uint64_t t_idx = c / K3;
        const uint32_t within = (uint32_t)(c % K3);
        const uint32_t cx = within % K, cz = (within / K) % K, cy = within / (K * K);
        if (threadIdx.x == 0) {
            const uint32_t t = __ldg(trees + t_idx);
            const int td = t < I.tree_cap ? I.depths[t] : TREE_UNUSED;
            uint64_t node = EMPTY_ID;
            int un = 1;
            uint32_t val = 0;
            if (td != d) {
                bad = true;
            } else {
                node = I.roots[t];
                const int L0 = d - lc;
                for (int depth = 0; depth < L0 && node != EMPTY_ID && id_is_branch(node); ++depth) {
                    const int sh = L0 - depth - 1;
                    const uint32_t ci = ((cx >> sh) & 1) | (((cy >> sh) & 1) << 1) | (((cz >> sh) & 1) << 2);
                    node = I.children[8ull * id_index(node) + ci];
                }
                if (node == EMPTY_ID) {
                    val = 0;
                } else if (!id_is_branch(node)) {
                    val = node_value(I, id_index(node));
                } else {
                    un = 0;
                }
            }
            cube_root = node;
            uniform = un;
            cube_val = val;
        }
        __syncthreads();
        T *dst = out + (c / K2 - first_slab) * slab_elems;  // the cube's cy-slab
        const uint64_t cube_off = (uint64_t)cz * C * S + (uint64_t)cx * C;
        if (!uniform) {
            // level-by-level expansion: level 0 is the cube root; ping-pong between the two id buffers
            // so that level lc-1 (the parents of the voxels) lands in lv_big
            uint64_t *cur = ((lc - 1) & 1) ? lv_small : lv_big;
            if (threadIdx.x == 0) cur[0] = cube_root;
            __syncthreads();
            for (int k = 0; k + 1 < lc; ++k) {
                uint64_t *nxt = (cur == lv_big) ? lv_small : lv_big;
                const uint32_t m = 1u << (3 * (k + 1));
                for (uint32_t j = threadIdx.x; j < m; j += blockDim.x) {
                    const uint64_t p = cur[j >> 3];
                    uint64_t ch = p;
                    if (p != EMPTY_ID && id_is_branch(p)) ch = I.children[8ull * id_index(p) + (j & 7)];
                    nxt[j] = ch;
                }
                __syncthreads();
                cur = nxt;
            }
            const uint32_t m = 1u << (3 * (lc - 1));
            for (uint32_t j = threadIdx.x; j < m; j += blockDim.x) {
                const uint64_t p = cur[j];
                uint32_t v8[8];
                if (p == EMPTY_ID) {
#pragma unroll
                    for (int k = 0; k < 8; ++k) v8[k] = 0;
                } else if (!id_is_branch(p)) {
                    const uint32_t v = node_value(I, id_index(p));
#pragma unroll
                    for (int k = 0; k < 8; ++k) v8[k] = v;
                } else {
                    const ulonglong2 *src = reinterpret_cast<const ulonglong2 *>(I.children + 8ull * id_index(p));
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        const ulonglong2 w = src[k];
                        v8[2 * k] = w.x ? node_value(I, id_index(w.x)) : 0u;
                        v8[2 * k + 1] = w.y ? node_value(I, id_index(w.y)) : 0u;
                    }
                }
                const uint32_t bx = morton_compact3(j), by = morton_compact3(j >> 1), bz = morton_compact3(j >> 2);
#pragma unroll
                for (int k = 0; k < 8; ++k) {
                    const uint32_t x = 2 * bx + (k & 1), y = 2 * by + ((k >> 1) & 1), z = 2 * bz + (k >> 2);
                    tile[(y * C + z) * C + x] = (T)v8[k];
                }
            }
            __syncthreads();
        }
        // store the cube: rows of C elements along x
        const uint32_t row_bytes = C * (uint32_t)sizeof(T);
        if (row_bytes % 16 == 0) {
            const uint32_t vec_per_row = row_bytes / 16, rows = C * C;
            const uint4 fillv = replicate16<T>(cube_val);
            for (uint32_t q = threadIdx.x; q < rows * vec_per_row; q += blockDim.x) {
                const uint32_t r = q / vec_per_row, v = q % vec_per_row;
                const uint32_t y = r / C, z = r % C;
                uint4 w = uniform ? fillv : reinterpret_cast<const uint4 *>(tile + (size_t)r * C)[v];
                T *row = dst + cube_off + (uint64_t)y * S * S + (uint64_t)z * S;
                reinterpret_cast<uint4 *>(row)[v] = w;
            }
        } else {
            for (uint32_t q = threadIdx.x; q < tile_elems; q += blockDim.x) {
                const uint32_t y = q / (C * C), z = (q / C) % C, x = q % C;
                dst[cube_off + (uint64_t)y * S * S + (uint64_t)z * S + x] = uniform ? (T)cube_val : tile[q];
            }
        }
        __syncthreads();
    }
    if (bad) set_error(I, ERR_INVALID, 52);
}
}  // namespace


// ---- occupancy masks for greedy meshing (utils/mesh.rs:418-597) ----------------------------------
// From the trees' dense grids ([tree][y][z][x], side 2^d <= 64): voxel counts per value, the sorted
// list of present values, then the bits of every non-default voxel in the 64^3 builder's three
// planes (YZ [y][z] -> x bits, XZ [z][x] -> y bits, XY [y][x] -> z bits), globally and per material.
// OR-ing voxel bits equals fill_masks_for_region's region fills (each region is a cube of voxels).
constexpr uint32_t kOccAll = 3 * 64 * 64;

template <class T>
__global__ void __launch_bounds__(kThreads) occupancy_hist_kernel(const T *grids, uint64_t n_vox,
                                                                   unsigned long long *counts) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    const unsigned lane = threadIdx.x & 31u;
    for (uint64_t base = (uint64_t)blockIdx.x * blockDim.x; base < n_vox; base += stride) {
        const uint64_t i = base + threadIdx.x;
        const uint32_t v = i < n_vox ? (uint32_t)grids[i] : 0u;
        const unsigned peers = __match_any_sync(0xFFFFFFFFu, v);
        if (v != 0 && lane == (unsigned)(__ffs(peers) - 1)) atomicAdd(counts + v, (unsigned long long)__popc(peers));
    }
}

// One CTA: slot[v] = rank of v among the present values (ascending), or ~0u.
__global__ void __launch_bounds__(1024) occupancy_index_kernel(const unsigned long long *counts, uint32_t n_values,
                                                               uint32_t *slot, uint32_t *ids,
                                                               unsigned long long *mcounts, uint32_t *n_out) {
    __shared__ uint32_t part[1024];
    const uint32_t per = (n_values + blockDim.x - 1) / blockDim.x;
    const uint32_t v0 = threadIdx.x * per;
    uint32_t c = 0;
    for (uint32_t v = v0; v < v0 + per && v < n_values; ++v) c += (v != 0 && counts[v] != 0) ? 1u : 0u;
    part[threadIdx.x] = c;
    __syncthreads();
    for (uint32_t off = 1; off < blockDim.x; off <<= 1) {  // inclusive scan (Hillis-Steele)
        const uint32_t y = threadIdx.x >= off ? part[threadIdx.x - off] : 0u;
        __syncthreads();
        part[threadIdx.x] += y;
        __syncthreads();
    }
    uint32_t r = part[threadIdx.x] - c;
    for (uint32_t v = v0; v < v0 + per && v < n_values; ++v) {
        if (v != 0 && counts[v] != 0) {
            slot[v] = r;
            ids[r] = v;
            mcounts[r] = counts[v];
            ++r;
        } else {
            slot[v] = ~0u;
        }
    }
    if (threadIdx.x == blockDim.x - 1) *n_out = part[threadIdx.x];
}

// Batched form for 8-bit voxels: tree t belongs to builder builder_of[t]; per-builder value counts
// (256 bins), ranks, planes and masks, indexed by builder.
__global__ void __launch_bounds__(kThreads) occupancy_hist_many_kernel(const uint8_t *grids, uint32_t n_trees, int d,
                                                                        const uint32_t *builder_of, uint32_t n_builders,
                                                                        unsigned int *counts) {
    const uint64_t per_tree = 1ull << (3 * d);
    const uint64_t n_vox = per_tree * n_trees;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    const unsigned lane = threadIdx.x & 31u;
    for (uint64_t base = (uint64_t)blockIdx.x * blockDim.x; base < n_vox; base += stride) {
        const uint64_t i = base + threadIdx.x;
        const bool in = i < n_vox;
        const uint32_t v = in ? grids[i] : 0u;
        const uint32_t b = (in && v) ? builder_of[(uint32_t)(i / per_tree)] : 0u;
        const bool on = in && v && b < n_builders;
        const uint32_t key = on ? b * 256u + v : 0xFFFFFFFFu - lane;
        const unsigned peers = __match_any_sync(0xFFFFFFFFu, key);
        if (on && lane == (unsigned)(__ffs(peers) - 1)) atomicAdd(counts + key, (unsigned)__popc(peers));
    }
}

// One warp per builder: ranks of the present values 1..255 (ascending).
__global__ void occupancy_index_many_kernel(const unsigned int *counts, uint32_t n_builders, uint32_t *slot,
                                            uint32_t max_mat, uint32_t *ids, unsigned long long *mcounts,
                                            uint32_t *n_mat) {
    const uint32_t b = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
    const unsigned lane = threadIdx.x & 31u;
    if (b >= n_builders) return;
    uint32_t r = 0;
    for (uint32_t v0 = 0; v0 < 256; v0 += 32) {
        const uint32_t v = v0 + lane;
        const unsigned c = counts[b * 256 + v];
        const bool present = v != 0 && c != 0;
        const unsigned bal = __ballot_sync(0xFFFFFFFFu, present);
        const uint32_t k = r + __popc(bal & ((1u << lane) - 1u));
        slot[b * 256 + v] = present ? k : ~0u;
        if (present && k < max_mat) {
            ids[(size_t)b * max_mat + k] = v;
            mcounts[(size_t)b * max_mat + k] = c;
        }
        r += __popc(bal);
    }
    if (lane == 0) n_mat[b] = r;
}

// Column form of the mask kernels: one thread per line of a tree's grid (a row along x, a column
// along y or along z; orientation o = 0, 1, 2 for the YZ, XZ and XY planes), which builds the line's
// occupancy bits in registers and ORs them into the builder's plane word with one atomic; the same for
// each material present on the line (up to kLineMats tracked in registers, else every material of the
// builder in turn).
constexpr int kLineMats = 6;

template <class T>
__global__ void __launch_bounds__(kThreads) occupancy_lines_kernel(DevInterner I, const T *grids, uint32_t n_trees,
                                                                    int d, const uint32_t *builder_of,
                                                                    uint32_t n_builders, const uint32_t *offsets,
                                                                    const uint32_t *slot, uint32_t slot_stride,
                                                                    const uint32_t *n_mat, uint32_t mat_cap,
                                                                    unsigned long long *global,
                                                                    unsigned long long *per_mat) {
    const uint32_t S = 1u << d;
    const uint64_t lines_per_tree = 3ull * S * S;
    const uint64_t n_lines = lines_per_tree * n_trees;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    bool bad = false;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_lines; i += stride) {
        const uint32_t t = (uint32_t)(i / lines_per_tree), w = (uint32_t)(i % lines_per_tree);
        const uint32_t o = w / (S * S), ab = w % (S * S), a = ab / S, bb = ab % S;
        const uint32_t b = builder_of ? builder_of[t] : 0u;
        const uint32_t ox = offsets[3 * t], oy = offsets[3 * t + 1], oz = offsets[3 * t + 2];
        if (b >= n_builders || ox + S > 64 || oy + S > 64 || oz + S > 64) {
            bad = true;
            continue;
        }
        const T *g = grids + (uint64_t)t * S * S * S;
        // line origin and step in the [y][z][x] grid, target word and the line's bit offset
        uint64_t base, step;
        uint32_t word, shift;
        if (o == 0) {  // YZ[y][z] <- x bits: a = y, bb = z
            base = ((uint64_t)a * S + bb) * S;
            step = 1;
            word = 0 * 4096 + (oy + a) * 64 + (oz + bb);
            shift = ox;
        } else if (o == 1) {  // XZ[z][x] <- y bits: a = z, bb = x
            base = (uint64_t)a * S + bb;
            step = (uint64_t)S * S;
            word = 1 * 4096 + (oz + a) * 64 + (ox + bb);
            shift = oy;
        } else {  // XY[y][x] <- z bits: a = y, bb = x
            base = (uint64_t)a * S * S + bb;
            step = S;
            word = 2 * 4096 + (oy + a) * 64 + (ox + bb);
            shift = oz;
        }
        uint64_t occ = 0;
        uint32_t mv[kLineMats];
        uint64_t mm[kLineMats];
        int nm = 0;
        bool overflow = false;
        for (uint32_t k = 0; k < S; ++k) {
            const uint32_t v = g[base + k * step];
            if (!v) continue;
            occ |= 1ull << k;
            int j = 0;
            while (j < nm && mv[j] != v) ++j;
            if (j == nm) {
                if (nm < kLineMats) {
                    mv[nm] = v;
                    mm[nm] = 0;
                    ++nm;
                } else {
                    overflow = true;
                    continue;
                }
            }
            mm[j] |= 1ull << k;
        }
        if (!occ) continue;
        unsigned long long *gb = global + (size_t)b * kOccAll;
        atomicOr(gb + word, (unsigned long long)(occ << shift));
        if (!overflow) {
            for (int j = 0; j < nm; ++j) {
                const uint32_t m = slot[(size_t)b * slot_stride + mv[j]];
                if (m < mat_cap) atomicOr(per_mat + ((size_t)b * mat_cap + m) * kOccAll + word, (unsigned long long)(mm[j] << shift));
            }
        } else {  // more materials on this line than tracked: one pass per material of the builder
            const uint32_t nmb = n_mat[b] < mat_cap ? n_mat[b] : mat_cap;
            for (uint32_t m = 0; m < nmb; ++m) {
                uint64_t bits = 0;
                for (uint32_t k = 0; k < S; ++k) {
                    const uint32_t v = g[base + k * step];
                    if (v && slot[(size_t)b * slot_stride + v] == m) bits |= 1ull << k;
                }
                if (bits) atomicOr(per_mat + ((size_t)b * mat_cap + m) * kOccAll + word, (unsigned long long)(bits << shift));
            }
        }
    }
    if (bad) set_error(I, ERR_OOB, 54);
}

// active[0..5] (mesh.rs:453-463): the occupied y, z, z, x, y, x coordinates.
__global__ void __launch_bounds__(kThreads) occupancy_active_kernel(const unsigned long long *global,
                                                                    unsigned long long *active) {
    global += (size_t)blockIdx.x * kOccAll;  // one CTA per builder
    active += (size_t)blockIdx.x * 6;
    __shared__ unsigned long long acc[3];
    if (threadIdx.x < 3) acc[threadIdx.x] = 0;
    __syncthreads();
    unsigned long long xs = 0, ys = 0, zs = 0;
    for (uint32_t k = threadIdx.x; k < 4096; k += blockDim.x) {
        xs |= global[k];         // YZ words hold x bits
        ys |= global[4096 + k];  // XZ words hold y bits
        zs |= global[8192 + k];  // XY words hold z bits
    }
    atomicOr(&acc[0], xs);
    atomicOr(&acc[1], ys);
    atomicOr(&acc[2], zs);
    __syncthreads();
    if (threadIdx.x == 0) {
        active[0] = acc[1];  // YZ rows: y
        active[1] = acc[2];  // YZ cols: z
        active[2] = acc[2];  // XZ rows: z
        active[3] = acc[0];  // XZ cols: x
        active[4] = acc[1];  // XY rows: y
        active[5] = acc[0];  // XY cols: x
    }
}

// ---- model serialisation (VoxModel::serialize, world/voxmodel.rs:177-282; serialize_chunk,
// world/voxchunk.rs:382-405) ------------------------------------------------------------------------
// Live leaves and live branches other than EMPTY are renumbered in slot-index order (leaves 1..L,
// then branches L+1..), each record's byte length is computed in parallel, exclusive scans place
// the records, and every node writes its own record: varint(new id) then the value (leaves), or
// varint(new id), mask, varint(new id) of each non-empty child and the LOD value (branches); values
// big-endian. Chunk records: "VoxTreeChunk", position (3 x i32 BE), varint(new id of the root).
__device__ __forceinline__ uint32_t varint_len(uint32_t v) {
    uint32_t n = 1;
    while (v >= 0x80u) {
        v >>= 7;
        ++n;
    }
    return n;
}

__device__ __forceinline__ uint8_t *put_varint(uint8_t *p, uint32_t v) {
    while (v >= 0x80u) {
        *p++ = (uint8_t)((v & 0x7Fu) | 0x80u);
        v >>= 7;
    }
    *p++ = (uint8_t)v;
    return p;
}

__device__ __forceinline__ uint8_t *put_value_be(uint8_t *p, uint32_t v, int vb) {
    if (vb == 2) *p++ = (uint8_t)(v >> 8);
    *p++ = (uint8_t)v;
    return p;
}

__global__ void ser_classify_kernel(DevInterner I, uint32_t *leaf_flag, uint32_t *branch_flag) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < I.capacity; i += gridDim.x * blockDim.x) {
        const uint64_t id = I.ids[i];
        leaf_flag[i] = (id != 0 && id_is_leaf(id)) ? 1u : 0u;
        branch_flag[i] = (id != 0 && !id_is_leaf(id) && i != 0) ? 1u : 0u;
    }
}

__global__ void ser_newid_kernel(DevInterner I, const uint32_t *leaf_flag, const uint32_t *leaf_rank,
                                 const uint32_t *branch_flag, const uint32_t *branch_rank, uint32_t *new_id) {
    const uint32_t L = leaf_rank[I.capacity];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < I.capacity; i += gridDim.x * blockDim.x)
        new_id[i] = leaf_flag[i] ? leaf_rank[i] + 1 : (branch_flag[i] ? L + 1 + branch_rank[i] : 0u);
}

__global__ void ser_size_kernel(DevInterner I, const uint32_t *leaf_flag, const uint32_t *branch_flag,
                                const uint32_t *new_id, uint32_t *leaf_size, uint32_t *branch_size) {
    const int vb = I.vbits / 8;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < I.capacity; i += gridDim.x * blockDim.x) {
        uint32_t ls = 0, bs = 0;
        if (leaf_flag[i]) ls = varint_len(new_id[i]) + vb;
        if (branch_flag[i]) {
            bs = varint_len(new_id[i]) + 1 + vb;
            const uint64_t *c = I.children + 8ull * i;
#pragma unroll
            for (int k = 0; k < 8; ++k)
                if (c[k] != EMPTY_ID) bs += varint_len(new_id[id_index(c[k])]);
        }
        leaf_size[i] = ls;
        branch_size[i] = bs;
    }
}

// out = [u32 L][leaf records][u32 B][branch records][u32 n_chunks][chunk records]
__global__ void ser_write_kernel(DevInterner I, const uint32_t *leaf_flag, const uint32_t *leaf_off,
                                 const uint32_t *branch_flag, const uint32_t *branch_off, const uint32_t *new_id,
                                 uint8_t *out) {
    const int vb = I.vbits / 8;
    const uint64_t leaf_base = 4, branch_base = 8 + (uint64_t)leaf_off[I.capacity];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < I.capacity; i += gridDim.x * blockDim.x) {
        if (leaf_flag[i]) {
            uint8_t *p = out + leaf_base + leaf_off[i];
            p = put_varint(p, new_id[i]);
            put_value_be(p, node_value(I, i), vb);
        } else if (branch_flag[i]) {
            uint8_t *p = out + branch_base + branch_off[i];
            const uint64_t id = I.ids[i];
            p = put_varint(p, new_id[i]);
            *p++ = (uint8_t)id_mask(id);
            const uint64_t *c = I.children + 8ull * i;
#pragma unroll
            for (int k = 0; k < 8; ++k)
                if (c[k] != EMPTY_ID) p = put_varint(p, new_id[id_index(c[k])]);
            put_value_be(p, node_value(I, i), vb);
        }
    }
}

__device__ __forceinline__ void put_u32_be(uint8_t *p, uint32_t v) {
    p[0] = (uint8_t)(v >> 24);
    p[1] = (uint8_t)(v >> 16);
    p[2] = (uint8_t)(v >> 8);
    p[3] = (uint8_t)v;
}

// One thread: the three counts, then the chunk records in the caller's order.
__global__ void ser_tail_kernel(DevInterner I, const uint32_t *leaf_rank, const uint32_t *branch_rank,
                                const uint32_t *leaf_off, const uint32_t *branch_off, const uint32_t *new_id,
                                uint32_t n_chunks, const uint32_t *trees, const int32_t *pos, uint8_t *out,
                                unsigned long long *total) {
    const uint32_t L = leaf_rank[I.capacity], B = branch_rank[I.capacity];
    put_u32_be(out, L);
    const uint64_t bh = 4 + (uint64_t)leaf_off[I.capacity];
    put_u32_be(out + bh, B);  // branch_patterns without EMPTY (the reference writes its size - 1)
    uint64_t o = bh + 4 + branch_off[I.capacity];
    put_u32_be(out + o, n_chunks);
    o += 4;
    const char magic[12] = {'V', 'o', 'x', 'T', 'r', 'e', 'e', 'C', 'h', 'u', 'n', 'k'};
    for (uint32_t k = 0; k < n_chunks; ++k) {
        for (int j = 0; j < 12; ++j) out[o + j] = (uint8_t)magic[j];
        o += 12;
        for (int a = 0; a < 3; ++a) put_u32_be(out + o + 4 * a, (uint32_t)pos[3 * k + a]);
        o += 12;
        const uint32_t t = trees[k];
        const uint64_t root = t < I.tree_cap ? I.roots[t] : EMPTY_ID;
        o = (uint64_t)(put_varint(out + o, new_id[id_index(root)]) - out);
    }
    *total = o;
}

size_t to_dense_smem_bytes(int d, int vbits) {
    const int lc = d < 5 ? d : 5;
    const size_t tile = ((size_t)1 << (3 * lc)) * (vbits / 8);
    const size_t big = lc >= 1 ? ((size_t)1 << (3 * (lc - 1))) : 1;
    const size_t small = lc >= 2 ? ((size_t)1 << (3 * (lc - 2))) : 1;
    return ((tile + 15) & ~(size_t)15) + 8 * (big + small);
}

cudaError_t launch_to_dense(const DevInterner &I, const uint32_t *trees, int d, uint64_t cube_begin,
                            uint64_t n_cubes, void *out, int num_sms, cudaStream_t s) {
    if (n_cubes == 0) return cudaSuccess;
    const int lc = d < 5 ? d : 5;
    const size_t smem = to_dense_smem_bytes(d, I.vbits);
    uint64_t blocks = n_cubes;
    const uint64_t cap = (uint64_t)num_sms * 8;
    if (blocks > cap) blocks = cap;
    count_launches(1);
    if (I.vbits == 8) {
        cudaFuncSetAttribute(to_dense_kernel<uint8_t>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        to_dense_kernel<uint8_t><<<(unsigned)blocks, kDenseOutThreads, smem, s>>>(I, trees, d, lc, cube_begin,
                                                                                  n_cubes, (uint8_t *)out);
    } else {
        cudaFuncSetAttribute(to_dense_kernel<uint16_t>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        to_dense_kernel<uint16_t><<<(unsigned)blocks, kDenseOutThreads, smem, s>>>(I, trees, d, lc, cube_begin,
                                                                                   n_cubes, (uint16_t *)out);
    }
    return cudaGetLastError();
}

cudaError_t launch_occupancy(const DevInterner &I, const void *grids, uint32_t n_trees, int d, const uint32_t *offsets,
                             unsigned long long *counts, uint32_t *slot, uint32_t *ids, unsigned long long *mcounts,
                             uint32_t *n_mat, uint32_t mat_cap, unsigned long long *global, unsigned long long *per_mat,
                             unsigned long long *active, int num_sms, cudaStream_t s) {
    const uint64_t n_vox = ((uint64_t)n_trees) << (3 * d);
    uint64_t blocks = (n_vox + kThreads - 1) / kThreads;
    if (blocks > (uint64_t)num_sms * 16) blocks = (uint64_t)num_sms * 16;
    const uint32_t n_values = 1u << I.vbits;
    count_launches(4);
    if (I.vbits == 8)
        occupancy_hist_kernel<uint8_t><<<(unsigned)blocks, kThreads, 0, s>>>((const uint8_t *)grids, n_vox, counts);
    else
        occupancy_hist_kernel<uint16_t><<<(unsigned)blocks, kThreads, 0, s>>>((const uint16_t *)grids, n_vox, counts);
    occupancy_index_kernel<<<1, 1024, 0, s>>>(counts, n_values, slot, ids, mcounts, n_mat);
    uint64_t lblocks = ((3ull * n_trees << (2 * d)) + kThreads - 1) / kThreads;
    if (lblocks > (uint64_t)num_sms * 16) lblocks = (uint64_t)num_sms * 16;
    if (I.vbits == 8)
        occupancy_lines_kernel<uint8_t><<<(unsigned)lblocks, kThreads, 0, s>>>(
            I, (const uint8_t *)grids, n_trees, d, nullptr, 1, offsets, slot, 0, n_mat, mat_cap, global, per_mat);
    else
        occupancy_lines_kernel<uint16_t><<<(unsigned)lblocks, kThreads, 0, s>>>(
            I, (const uint16_t *)grids, n_trees, d, nullptr, 1, offsets, slot, 0, n_mat, mat_cap, global, per_mat);
    occupancy_active_kernel<<<1, kThreads, 0, s>>>(global, active);
    return cudaGetLastError();
}

// Scratch of the serialisation: nine arrays of capacity + 1 u32.
size_t serialize_scratch_words(const DevInterner &I) { return 9 * ((size_t)I.capacity + 1) + 64; }

namespace {
struct SerBufs {
    uint32_t *leaf_flag, *branch_flag, *leaf_rank, *branch_rank, *new_id, *leaf_size, *branch_size, *leaf_off,
        *branch_off;
    SerBufs(uint32_t *w, uint32_t n) {
        uint32_t **all[9] = {&leaf_flag, &branch_flag, &leaf_rank, &branch_rank, &new_id,
                             &leaf_size, &branch_size, &leaf_off, &branch_off};
        for (int k = 0; k < 9; ++k) *all[k] = w + (size_t)k * (n + 1);
    }
};

__global__ void ser_total_kernel(DevInterner I, SerBufs b, uint32_t n_chunks, const uint32_t *trees,
                                 unsigned long long *total) {
    unsigned long long t = 12ull + b.leaf_off[I.capacity] + b.branch_off[I.capacity];
    for (uint32_t k = 0; k < n_chunks; ++k) {
        const uint32_t tr = trees[k];
        const uint64_t root = tr < I.tree_cap ? I.roots[tr] : EMPTY_ID;
        t += 24 + varint_len(b.new_id[id_index(root)]);
    }
    *total = t;
}
}  // namespace

cudaError_t launch_serialize_plan(const DevInterner &I, uint32_t *w, uint32_t *tmp_scan, uint32_t n_chunks,
                                  const uint32_t *trees, unsigned long long *total, int num_sms, cudaStream_t s) {
    const uint32_t n = I.capacity;
    SerBufs b(w, n);
    const unsigned g = (unsigned)num_sms * 8;
    count_launches(1);
    ser_classify_kernel<<<g, kThreads, 0, s>>>(I, b.leaf_flag, b.branch_flag);
    cudaError_t e = launch_scan(b.leaf_flag, b.leaf_rank, tmp_scan, n, s);
    if (e == cudaSuccess) e = launch_scan(b.branch_flag, b.branch_rank, tmp_scan, n, s);
    if (e != cudaSuccess) return e;
    count_launches(2);
    ser_newid_kernel<<<g, kThreads, 0, s>>>(I, b.leaf_flag, b.leaf_rank, b.branch_flag, b.branch_rank, b.new_id);
    ser_size_kernel<<<g, kThreads, 0, s>>>(I, b.leaf_flag, b.branch_flag, b.new_id, b.leaf_size, b.branch_size);
    e = launch_scan(b.leaf_size, b.leaf_off, tmp_scan, n, s);
    if (e == cudaSuccess) e = launch_scan(b.branch_size, b.branch_off, tmp_scan, n, s);
    if (e != cudaSuccess) return e;
    count_launches(1);
    ser_total_kernel<<<1, 1, 0, s>>>(I, b, n_chunks, trees, total);
    return cudaGetLastError();
}

cudaError_t launch_serialize_write(const DevInterner &I, uint32_t *w, uint32_t n_chunks, const uint32_t *trees,
                                   const int32_t *pos, uint8_t *out, unsigned long long *total, int num_sms,
                                   cudaStream_t s) {
    SerBufs b(w, I.capacity);
    const unsigned g = (unsigned)num_sms * 8;
    count_launches(2);
    ser_write_kernel<<<g, kThreads, 0, s>>>(I, b.leaf_flag, b.leaf_off, b.branch_flag, b.branch_off, b.new_id, out);
    ser_tail_kernel<<<1, 1, 0, s>>>(I, b.leaf_rank, b.branch_rank, b.leaf_off, b.branch_off, b.new_id, n_chunks, trees,
                                    pos, out, total);
    return cudaGetLastError();
}

cudaError_t launch_occupancy_many(const DevInterner &I, const uint8_t *grids, uint32_t n_trees, int d,
                                  const uint32_t *builder_of, const uint32_t *offsets, uint32_t n_builders,
                                  unsigned int *counts, uint32_t *slot, uint32_t max_mat, uint32_t *ids,
                                  unsigned long long *mcounts, uint32_t *n_mat, unsigned long long *global,
                                  unsigned long long *per_mat, unsigned long long *active, int num_sms, cudaStream_t s) {
    const uint64_t n_vox = ((uint64_t)n_trees) << (3 * d);
    uint64_t blocks = (n_vox + kThreads - 1) / kThreads;
    if (blocks > (uint64_t)num_sms * 16) blocks = (uint64_t)num_sms * 16;
    count_launches(4);
    occupancy_hist_many_kernel<<<(unsigned)blocks, kThreads, 0, s>>>(grids, n_trees, d, builder_of, n_builders, counts);
    occupancy_index_many_kernel<<<(n_builders + 7) / 8, 256, 0, s>>>(counts, n_builders, slot, max_mat, ids, mcounts,
                                                                     n_mat);
    uint64_t lblocks = ((3ull * n_trees << (2 * d)) + kThreads - 1) / kThreads;
    if (lblocks > (uint64_t)num_sms * 16) lblocks = (uint64_t)num_sms * 16;
    occupancy_lines_kernel<uint8_t><<<(unsigned)lblocks, kThreads, 0, s>>>(I, grids, n_trees, d, builder_of, n_builders,
                                                                          offsets, slot, 256, n_mat, max_mat, global,
                                                                          per_mat);
    occupancy_active_kernel<<<n_builders, kThreads, 0, s>>>(global, active);
    return cudaGetLastError();
}

cudaError_t launch_get_many(const DevInterner &I, uint64_t n, const uint32_t *trees, const int32_t *xyz,
                            uint8_t *found, void *values, int num_sms, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    uint64_t blocks = (n + kThreads - 1) / kThreads;
    const uint64_t cap = (uint64_t)num_sms * 16;
    if (blocks > cap) blocks = cap;
    count_launches(1);
    if (I.vbits == 8)
        get_kernel<uint8_t><<<(unsigned)blocks, kThreads, 0, s>>>(I, n, trees, xyz, found, (uint8_t *)values);
    else
        get_kernel<uint16_t><<<(unsigned)blocks, kThreads, 0, s>>>(I, n, trees, xyz, found, (uint16_t *)values);
    return cudaGetLastError();
}

cudaError_t launch_release(const DevInterner &I, uint64_t *list, uint32_t *frontier_a, uint32_t *frontier_b,
                           uint64_t frontier_cap, int rounds, int num_sms, cudaStream_t s) {
    (void)frontier_cap;
    const unsigned g = (unsigned)num_sms * 4;
    count_launches(1);
    (void)launch_pdl(release_advance_kernel, dim3(1), dim3(1), 0, s, I);  // clears the output count
    count_launches(1);
    (void)launch_pdl(release_roots_kernel, dim3(g), dim3(kThreads), 0, s, I, list, frontier_a);
    uint32_t *in = frontier_a, *out = frontier_b;
    for (int r = 0; r < rounds; ++r) {  // each kernel's last CTA advances the dying set
        count_launches(1);
        (void)launch_pdl(release_round_kernel, dim3(g), dim3(kThreads), 0, s, I, in, out);
        uint32_t *t = in;
        in = out;
        out = t;
    }
    return cudaGetLastError();
}

cudaError_t launch_tree_set(const DevInterner &I, uint32_t tree, int32_t x, int32_t y, int32_t z, uint32_t v,
                            uint64_t *queue, uint64_t queue_cap, int *status_out, cudaStream_t s) {
    count_launches(1);
    tree_set_kernel<<<1, 1, 0, s>>>(I, tree, x, y, z, v, queue, queue_cap, status_out);
    return cudaGetLastError();
}

cudaError_t launch_trees_set(const DevInterner &I, const SetCalls &c, uint64_t *list, unsigned long long fc0,
                             unsigned long long ni0, uint32_t *frontier_a, uint32_t *frontier_b, int max_depth,
                             int num_sms, cudaStream_t s) {
    const unsigned per_block = kThreads / 32;
    unsigned g = (c.n_groups + per_block - 1) / per_block;
    if (g > (unsigned)num_sms * 8) g = (unsigned)num_sms * 8;
    if (g == 0) g = 1;
    count_launches(1);
    trees_set_kernel<<<g, kThreads, 0, s>>>(I, c);
    cudaError_t e = launch_epoch_refcounts(I, num_sms, s);
    if (e != cudaSuccess) return e;
    unsigned gr = (c.n_groups + kThreads - 1) / kThreads;
    count_launches(2);
    trees_set_roots_kernel<<<gr ? gr : 1, kThreads, 0, s>>>(I, c, list);
    trees_set_garbage_kernel<<<(unsigned)num_sms * 4, kThreads, 0, s>>>(I, fc0, ni0, list);
    return launch_release(I, list, frontier_a, frontier_b, 0, max_depth + 2, num_sms, s);
}

cudaError_t launch_tree_fill(const DevInterner &I, uint32_t tree, uint32_t v, uint64_t *queue,
                             uint64_t queue_cap, int *status_out, cudaStream_t s) {
    count_launches(1);
    tree_fill_kernel<<<1, 1, 0, s>>>(I, tree, v, queue, queue_cap, status_out);
    return cudaGetLastError();
}

cudaError_t launch_rehash(const DevInterner &I, uint64_t table_slots, int num_sms, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(I.table, 0xFF, table_slots * sizeof(uint64_t), s);
    if (e != cudaSuccess) return e;
    count_launches(1);
    rehash_kernel<<<num_sms * 4, kThreads, 0, s>>>(I);
    count_launches(1);
    rehash_done_kernel<<<1, 1, 0, s>>>(I);
    return cudaGetLastError();
}

cudaError_t launch_count_live(const DevInterner &I, unsigned long long *out2, int num_sms, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(out2, 0, 2 * sizeof(unsigned long long), s);
    if (e != cudaSuccess) return e;
    count_launches(1);
    count_live_kernel<<<num_sms * 4, kThreads, 0, s>>>(I, out2);
    return cudaGetLastError();
}

}  // namespace vxg
