// Device-side data structures and primitives of the GB300 interner.
//
// The interner (the reference's VoxInterner<T>, interner/mod.rs:25-40) lives in HBM as SoA arrays
// of `capacity` node records (capacity = budget / node_size, interner/mod.rs:49-53, 158-164):
//   children[8*i]  u64 BlockIds of the 8 children (zero for leaves)      64 B
//   values[i]      u8 / u16 voxel value (leaf) or LOD value (branch)      1-2 B
//   refcount[i]    u32                                                     4 B
//   generation[i]  u16, bumped when the slot is recycled                  2 B
//   hash[i]        u64 key fingerprint (branches)                          8 B
//   ids[i]         u64 live BlockId of the slot, 0 while free            (+8 B, outside the budget)
// Hash-consing tables (outside the budget, like the reference's HashMaps):
//   table[]        open-addressed branch table of 64-bit slots: tag (32 bits of the key
//                  fingerprint) | node index. Inserts claim a slot with atomicCAS and publish the
//                  index after writing the node; lookups compare the full key (types, mask and the
//                  8 child ids), so equal keys always dedup and unequal keys never alias.
//   leaf_table[v]  direct-mapped leaf ids, one slot per voxel value (0 = none, 1 = being created).
// Allocation pops the LIFO free list first, then bumps next_index (interner/macros.rs:1-41).
// Every spin-wait is bounded; failures set sticky error bits that the host turns into statuses.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace vxg {

constexpr uint64_t EMPTY_ID = 0ull;
constexpr uint64_t INVALID_ID = ~0ull;
constexpr uint16_t MAX_GENERATION = 0x7FFE;
constexpr uint32_t NO_NODE = 0xFFFFFFFFu;

// table slot encoding
constexpr uint64_t SLOT_EMPTY = ~0ull;
constexpr uint64_t SLOT_TOMB = 0xFFFFFFFEFFFFFFFEull;
constexpr uint32_t IDX_BUSY = 0xFFFFFFFFu;
constexpr uint64_t LEAF_BUSY = 1ull;

// sticky error bits (mapped to VX_E_* by the host)
enum : uint32_t {
    ERR_OOM = 1u << 0,
    ERR_TABLE_FULL = 1u << 1,
    ERR_TIMEOUT = 1u << 2,
    ERR_REF_PANIC = 1u << 3,
    ERR_REF_UB = 1u << 4,
    ERR_OOB = 1u << 5,
    ERR_INTERNAL = 1u << 6,
    ERR_INVALID = 1u << 7,
};

constexpr uint8_t TREE_UNUSED = 0xFF;  // depth marker of a free tree slot

// Bounds of every wait. The copy waits of the dense kernels (TMA tiles, and the drain of a warp's
// own copies after giving up) always use SPIN_LIMIT; the waits on other threads (leaf creation, grid
// barriers, scan look-back) use the interner's spin_limit and the warp-intern loop its round_limit,
// both settable per interner (vx_interner_set_limits) and SPIN_LIMIT / ROUND_LIMIT by default.
constexpr uint32_t SPIN_LIMIT = 1u << 22;   // bounded waits (~tens of ms with nanosleep)
constexpr uint32_t ROUND_LIMIT = 1u << 20;  // bounded warp-intern rounds

struct DevCounters {
    unsigned long long next_index;   // bump pointer
    unsigned long long free_count;   // free-list length
    unsigned long long alloc_count;  // allocations in the current epoch
    unsigned long long tombstones;   // deleted branch-table slots
    unsigned int error;              // sticky ERR_* bits
    unsigned int error_info;         // first error detail
    unsigned long long scratch[10];  // per-launch counters used by the kernels
    unsigned long long created;      // nodes allocated since the interner was created or reset
    unsigned long long bar_count;    // grid barrier of single-launch kernels: CTAs arrived
    unsigned long long bar_gen;      //   and the barrier's generation
    unsigned long long rel_count[3]; // dying-set sizes of single-launch release rounds (rotating)
};

struct DevInterner {
    uint64_t *children;
    void *values;
    uint32_t *refcount;
    uint16_t *generation;
    uint64_t *hash;
    uint64_t *ids;
    uint32_t *free_list;
    DevCounters *ctr;
    uint64_t *table;
    uint64_t table_mask;
    uint64_t *leaf_table;
    uint64_t *roots;
    uint8_t *depths;
    uint32_t tree_cap;
    uint32_t capacity;
    int vbits;
    uint32_t flags;
    uint32_t max_probes;   // branch-table probes before ERR_TABLE_FULL
    uint32_t round_limit;  // warp-intern rounds before ERR_TIMEOUT
    uint32_t spin_limit;   // iterations of a wait on another thread before ERR_TIMEOUT
    uint32_t memo_shift;   // dense builds: quad-memo slots ~ the call's quads >> memo_shift (tunable)
};

// ---- BlockId (core/block_id.rs:19-418) -------------------------------------------------------
__host__ __device__ __forceinline__ bool id_is_leaf(uint64_t id) { return (id >> 63) != 0; }
__host__ __device__ __forceinline__ bool id_is_branch(uint64_t id) { return (id >> 63) == 0; }
__host__ __device__ __forceinline__ uint32_t id_index(uint64_t id) { return (uint32_t)id; }
__host__ __device__ __forceinline__ uint32_t id_generation(uint64_t id) { return (uint32_t)((id >> 32) & 0x7FFF); }
__host__ __device__ __forceinline__ uint32_t id_types(uint64_t id) { return (uint32_t)((id >> 55) & 0xFF); }
__host__ __device__ __forceinline__ uint32_t id_mask(uint64_t id) { return (uint32_t)((id >> 47) & 0xFF); }
__host__ __device__ __forceinline__ uint64_t make_leaf_id(uint32_t index, uint32_t gen) {
    return (1ull << 63) | ((uint64_t)(gen & 0x7FFF) << 32) | index;
}
__host__ __device__ __forceinline__ uint64_t make_branch_id(uint32_t index, uint32_t gen, uint32_t types,
                                                            uint32_t mask) {
    return ((uint64_t)(types & 0xFF) << 55) | ((uint64_t)(mask & 0xFF) << 47) |
           ((uint64_t)(gen & 0x7FFF) << 32) | index;
}

// Sibling-prefix mask PATH_MASKS[d][k] (voxtree.rs:41-105), closed form.
__host__ __device__ __forceinline__ uint32_t path_mask(int d, int k) {
    if (d <= 0 || k > d - 1) return 0;
    return ((1u << (3 * (k + 1))) - 1u) << (3 * (d - 1 - k));
}

// ---- memory helpers --------------------------------------------------------------------------
__device__ __forceinline__ uint64_t ld_volatile(const uint64_t *p) { return *(const volatile uint64_t *)p; }
// Acquire load of a table slot: the node record published before the slot is visible after it.
__device__ __forceinline__ uint64_t ld_acquire(const uint64_t *p) {
    uint64_t v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ uint64_t ld_cg(const uint64_t *p) { return __ldcg((const unsigned long long *)p); }
// Load of a hash-table slot while probing. Publishers write the node record, fence, then store the
// slot; everything a prober reads after a slot (record words) is read from L2 (ld.global.cg) at an
// address computed from the slot value. VX_PROBE_ACQUIRE=1 makes the slot load an acquire instead.
#ifndef VX_PROBE_ACQUIRE
#define VX_PROBE_ACQUIRE 1
#endif
__device__ __forceinline__ uint64_t ld_probe(const uint64_t *p) {
    uint64_t v;
#if VX_PROBE_ACQUIRE
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
#else
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
#endif
    return v;
}

__device__ __forceinline__ void st_release_u64(unsigned long long *p, unsigned long long v) {
    asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// Publication with release semantics: every store of this thread before it is visible to a thread
// that reads the new value with acquire semantics (ld_probe). Cheaper than a full fence before a
// plain atomic, which also orders loads and waits for sequential consistency.
__device__ __forceinline__ unsigned long long atom_exch_release(unsigned long long *p, unsigned long long v) {
    unsigned long long old;
    asm volatile("atom.release.gpu.global.exch.b64 %0, [%1], %2;" : "=l"(old) : "l"(p), "l"(v) : "memory");
    return old;
}
// Publication of a slot this thread owns (claimed in a busy state that no other thread writes): a
// release store waits for this thread's earlier writes like the exchange, but not for a reply.
#ifndef VX_PUB_STORE
#define VX_PUB_STORE 1
#endif
__device__ __forceinline__ void publish_release(unsigned long long *p, unsigned long long v) {
    if (VX_PUB_STORE)
        st_release_u64(p, v);
    else
        atom_exch_release(p, v);
}
// Compare-and-swap that publishes this thread's earlier stores (release) and, whatever its outcome,
// makes the stores published with the value it read visible to this thread (acquire).
__device__ __forceinline__ unsigned long long atom_cas_acq_rel(unsigned long long *p, unsigned long long cmp,
                                                               unsigned long long v) {
    unsigned long long old;
    asm volatile("atom.acq_rel.gpu.global.cas.b64 %0, [%1], %2, %3;" : "=l"(old) : "l"(p), "l"(cmp), "l"(v) : "memory");
    return old;
}

// Counts the calling CTA as done on *done and returns true in thread 0 of the last CTA of the grid to
// finish (every other CTA's writes are visible to it), after resetting *done for the next kernel.
// All threads of the CTA must call it. Lets a kernel's last CTA do the one-thread follow-up work that
// would otherwise be a separate launch.
__device__ __forceinline__ bool grid_last_cta(unsigned long long *done) {
    __shared__ unsigned int is_last;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        is_last = atomicAdd(done, 1ull) == gridDim.x - 1;
    }
    __syncthreads();
    if (threadIdx.x != 0 || !is_last) return false;
    __threadfence();
    *done = 0;
    return true;
}

// Programmatic dependent launch: a kernel launched with the programmatic-serialization attribute may
// start while its predecessor on the stream still runs; pdl_wait() blocks until the predecessor has
// completed and its writes are visible (a no-op for a normal launch), and pdl_release() lets the next
// kernel of the stream launch early. A kernel calls pdl_wait() before its first access to memory the
// predecessor writes.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_release() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

__device__ __forceinline__ void set_error(const DevInterner &I, uint32_t bit, uint32_t info = 0) {
    unsigned int old = atomicOr(&I.ctr->error, bit);
    if (old == 0) atomicExch(&I.ctr->error_info, info);
}

__device__ __forceinline__ uint32_t node_value(const DevInterner &I, uint32_t idx) {
    return I.vbits == 8 ? (uint32_t)((const uint8_t *)I.values)[idx] : (uint32_t)((const uint16_t *)I.values)[idx];
}
__device__ __forceinline__ uint32_t node_value_cg(const DevInterner &I, uint32_t idx) {
    if (I.vbits == 8) return (uint32_t)__ldcg((const unsigned char *)I.values + idx);
    return (uint32_t)__ldcg((const unsigned short *)I.values + idx);
}
__device__ __forceinline__ void set_node_value(const DevInterner &I, uint32_t idx, uint32_t v) {
    if (I.vbits == 8)
        ((uint8_t *)I.values)[idx] = (uint8_t)v;
    else
        ((uint16_t *)I.values)[idx] = (uint16_t)v;
}

// ---- key fingerprint -------------------------------------------------------------------------
__device__ __forceinline__ uint64_t fmix64(uint64_t k) {
    k ^= k >> 33;
    k *= 0xff51afd7ed558ccdull;
    k ^= k >> 33;
    k *= 0xc4ceb9fe1a85ec53ull;
    k ^= k >> 33;
    return k;
}
__device__ __forceinline__ uint64_t branch_fingerprint(const uint64_t c[8], uint32_t tm) {
    uint64_t h = 0x9E3779B97F4A7C15ull ^ ((uint64_t)tm << 17);
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        h ^= c[i] * 0x87C37B91114253D5ull;
        h = ((h << 31) | (h >> 33)) * 0x4CF5AD432745937Full;
    }
    return fmix64(h);
}
__device__ __forceinline__ uint32_t slot_tag(uint64_t h) {
    uint32_t t = (uint32_t)(h >> 32);
    return t >= 0xFFFFFFFEu ? 0xFFFFFFFDu : t;
}
__device__ __forceinline__ uint64_t make_slot(uint32_t tag, uint32_t idx) { return ((uint64_t)tag << 32) | idx; }

// calc_average (core/voxel.rs:96-141): the mode of the 8 values. Distinct values are visited in
// first-seen order; a later value replaces the current best when it is more frequent, or equally
// frequent while the best is the default value and it is not. Fully unrolled on registers.
__device__ __forceinline__ uint32_t calc_average8(const uint32_t v[8]) {
    uint32_t best = v[0];
    uint32_t best_cnt = 0;
#pragma unroll
    for (int j = 0; j < 8; ++j) best_cnt += v[j] == v[0] ? 1u : 0u;
#pragma unroll
    for (int k = 1; k < 8; ++k) {
        bool first = true;
#pragma unroll
        for (int j = 0; j < k; ++j) first = first && v[j] != v[k];
        uint32_t cnt = 0;
#pragma unroll
        for (int j = 0; j < 8; ++j) cnt += v[j] == v[k] ? 1u : 0u;
        if (first && (cnt > best_cnt || (cnt == best_cnt && best == 0 && v[k] != 0))) {
            best = v[k];
            best_cnt = cnt;
        }
    }
    return best;
}

// ---- allocation --------------------------------------------------------------------------------
// The t-th allocation of an epoch takes free_list[free_count-1-t] while the free list lasts, then
// next_index + (t - free_count). free_count and next_index only change between epochs.
__device__ __forceinline__ uint32_t node_for_ticket(const DevInterner &I, unsigned long long t,
                                                    unsigned long long fc, unsigned long long ni) {
    unsigned long long idx = (t < fc) ? (unsigned long long)I.free_list[fc - 1 - t] : ni + (t - fc);
    return idx < I.capacity ? (uint32_t)idx : NO_NODE;
}
__device__ __forceinline__ uint32_t node_for_ticket(const DevInterner &I, unsigned long long t) {
    return node_for_ticket(I, t, I.ctr->free_count, I.ctr->next_index);
}

// Closes the epoch (one thread, after every allocation of the epoch): the free-list entries and
// fresh indices its tickets took become allocated.
__device__ __forceinline__ void epoch_finalize_body(const DevInterner &I) {
    DevCounters *c = I.ctr;
    const unsigned long long alloc = c->alloc_count, fc = c->free_count;
    const unsigned long long used_free = alloc < fc ? alloc : fc;
    c->free_count = fc - used_free;
    unsigned long long ni = c->next_index + (alloc - used_free);
    if (ni > I.capacity) ni = I.capacity;
    c->created += used_free + (ni - c->next_index);
    c->next_index = ni;
    c->alloc_count = 0;
}

// Slots past next_index have never held a node since the interner was created or reset (the bump
// allocator hands each out once, recycling only bumps the generation of slots handed out before,
// and creation, reset and model loading zero the generations), so their generation is 0: a ticket
// past the free list needs no dependent load of it.
#ifndef VX_FRESH_GEN
#define VX_FRESH_GEN 1
#endif
__device__ __forceinline__ uint32_t slot_generation(const DevInterner &I, uint32_t idx, bool bumped) {
    return (VX_FRESH_GEN && bumped) ? 0u : (uint32_t)I.generation[idx];
}

// Writes a new branch record (children, LOD value, fingerprint, live id); rc starts at 0. bumped: idx
// came from past the free list (generation 0).
__device__ __forceinline__ uint64_t write_branch(const DevInterner &I, uint32_t idx, const uint64_t c[8],
                                                 uint32_t types, uint32_t mask, uint64_t h, uint32_t lod,
                                                 bool bumped = false) {
    uint32_t gen = slot_generation(I, idx, bumped);
    uint64_t id = make_branch_id(idx, gen, types, mask);
    ulonglong2 *dst = reinterpret_cast<ulonglong2 *>(I.children + 8ull * idx);
    dst[0] = make_ulonglong2(c[0], c[1]);
    dst[1] = make_ulonglong2(c[2], c[3]);
    dst[2] = make_ulonglong2(c[4], c[5]);
    dst[3] = make_ulonglong2(c[6], c[7]);
    set_node_value(I, idx, lod);
    I.hash[idx] = h;
    I.refcount[idx] = 0;
    I.ids[idx] = id;
    return id;
}

// The id and the children of node idx are loaded together (one round trip); *id_out gets the id.
__device__ __forceinline__ bool key_equal(const DevInterner &I, uint32_t idx, const uint64_t c[8], uint32_t types,
                                          uint32_t mask, uint64_t *id_out = nullptr) {
    const ulonglong2 *src = reinterpret_cast<const ulonglong2 *>(I.children + 8ull * idx);
    const uint64_t id = ld_cg(I.ids + idx);
    ulonglong2 w[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) w[k] = __ldcg(src + k);
    if (id == 0 || id_is_leaf(id) || id_types(id) != types || id_mask(id) != mask) return false;
#pragma unroll
    for (int k = 0; k < 4; ++k)
        if (w[k].x != c[2 * k] || w[k].y != c[2 * k + 1]) return false;
    if (id_out) *id_out = id;
    return true;
}

// Warp-cooperative find-or-insert of branch keys. Every lane of the warp must call it (converged);
// lanes with active == false only take part in the ballots. Each round every unfinished lane makes
// one non-blocking probe step; lanes that claimed an empty slot receive node indices from a single
// warp-aggregated ticket range, write their node and publish it. A lane that meets a slot still being
// written retries it next round, so no lane ever waits inside a divergent branch.
// Returns the BlockId; *created tells whether this lane inserted the node. On failure (probe limit,
// round limit, out of nodes: a sticky error bit is set) the lane gets EMPTY_ID, which every consumer
// handles without dereferencing it, so a failed call leaves wrong but memory-safe results until
// vx_interner_reset.
#ifndef VX_INTERN_INLINE
#define VX_INTERN_INLINE __noinline__
#endif
__device__ __forceinline__ uint64_t warp_intern_branch_inl(const DevInterner &I, bool active, const uint64_t c[8],
                                                           uint32_t types, uint32_t mask, uint32_t lod, bool *created,
                                                           uint64_t h_in = 0) {
    const unsigned lane = threadIdx.x & 31u;
    const uint32_t tm = (types << 8) | mask;
    uint64_t h = 0;
    uint32_t tag = 0;
    uint64_t pos = 0;
    uint32_t probes = 0;
    bool done = !active;
    uint64_t result = EMPTY_ID;
    *created = false;
    // constant during an epoch: loaded beside the first probe instead of after a ticket is taken
    const unsigned long long fc = I.ctr->free_count, ni = I.ctr->next_index;
    if (active) {
        h = h_in ? h_in : branch_fingerprint(c, tm);
        tag = slot_tag(h);
        pos = h & I.table_mask;
    }
    for (uint32_t round = 0;; ++round) {
        bool claimed = false;
        bool waiting = false;
        if (!done) {
            uint64_t s = ld_probe(I.table + pos);
            if (s == SLOT_EMPTY) {
                uint64_t prev = atomicCAS((unsigned long long *)(I.table + pos), SLOT_EMPTY, make_slot(tag, IDX_BUSY));
                if (prev == SLOT_EMPTY)
                    claimed = true;
                else
                    s = prev;
            }
            if (!claimed) {
                if ((uint32_t)(s >> 32) == tag && s != SLOT_TOMB) {
                    uint32_t idx = (uint32_t)s;
                    if (idx == IDX_BUSY) {
                        waiting = true;  // retry the same slot next round
                    } else {
                        if (key_equal(I, idx, c, types, mask, &result)) {
                            done = true;
                        } else {
                            pos = (pos + 1) & I.table_mask;
                            ++probes;
                        }
                    }
                } else {
                    pos = (pos + 1) & I.table_mask;
                    ++probes;
                }
                if (!done && probes > I.max_probes) {
                    set_error(I, ERR_TABLE_FULL, 1);
                    done = true;
                }
            }
        }
        const unsigned cm = __ballot_sync(0xFFFFFFFFu, claimed);
        if (cm) {
            unsigned long long base = 0;
            const int leader = __ffs(cm) - 1;
            if ((int)lane == leader) base = atomicAdd(&I.ctr->alloc_count, (unsigned long long)__popc(cm));
            base = __shfl_sync(0xFFFFFFFFu, base, leader);
            if (claimed) {
                const unsigned rank = __popc(cm & ((1u << lane) - 1u));
                const uint32_t idx = node_for_ticket(I, base + rank, fc, ni);
                if (idx == NO_NODE) {
                    set_error(I, ERR_OOM, 1);
                    atomicExch((unsigned long long *)(I.table + pos), SLOT_TOMB);
                } else {
                    result = write_branch(I, idx, c, types, mask, h, lod, base + rank >= fc);
                    publish_release((unsigned long long *)(I.table + pos), make_slot(tag, idx));
                    *created = true;
                }
                done = true;
            }
        }
        if (!__any_sync(0xFFFFFFFFu, !done)) break;
        if (round >= I.round_limit) {
            if (!done) {
                set_error(I, ERR_TIMEOUT, 2);
                done = true;
            }
            break;
        }
        if (waiting) __nanosleep(32);
    }
    return result;
}

// The same, out of line (for call sites on rare paths, to keep kernels small).
static __device__ VX_INTERN_INLINE uint64_t warp_intern_branch(const DevInterner &I, bool active, const uint64_t c[8],
                                                       uint32_t types, uint32_t mask, uint32_t lod, bool *created,
                                                       uint64_t h_in = 0) {
    return warp_intern_branch_inl(I, active, c, types, mask, lod, created, h_in);
}

// Find-or-create of the leaf for value v (v != 0) through the direct-mapped leaf table.
// *created tells whether this call allocated the leaf (its refcount starts at 0). On failure (out of
// nodes, wait limit: sticky error bit set) it returns EMPTY_ID, like warp_intern_branch.
__device__ __forceinline__ uint64_t intern_leaf(const DevInterner &I, uint32_t v, bool *created) {
    *created = false;
    unsigned long long *slot = (unsigned long long *)(I.leaf_table + v);
    uint64_t s = ld_volatile(I.leaf_table + v);
    if (s > LEAF_BUSY) return s;
    // constant during an epoch: loaded before the claim instead of after the ticket
    const unsigned long long fc = I.ctr->free_count, ni = I.ctr->next_index;
    for (uint32_t spin = 0; spin < I.spin_limit; ++spin) {
        if (s == 0) {  // free (or its creator ran out of memory and backed off): claim it
            const uint64_t prev = atomicCAS(slot, 0ull, LEAF_BUSY);
            if (prev == 0) {
                const unsigned long long t = atomicAdd(&I.ctr->alloc_count, 1ull);
                const uint32_t idx = node_for_ticket(I, t, fc, ni);
                if (idx == NO_NODE) {
                    set_error(I, ERR_OOM, 2);
                    atomicExch(slot, 0ull);
                    return EMPTY_ID;
                }
                const uint64_t id = make_leaf_id(idx, slot_generation(I, idx, t >= fc));
                set_node_value(I, idx, v);
                I.hash[idx] = 0;
                I.refcount[idx] = 0;
                I.ids[idx] = id;
                publish_release(slot, id);
                *created = true;
                return id;
            }
            if (prev > LEAF_BUSY) return prev;
        }
        __nanosleep(64);  // being created by another thread
        s = ld_volatile(I.leaf_table + v);
        if (s > LEAF_BUSY) return s;
    }
    set_error(I, ERR_TIMEOUT, 3);
    return EMPTY_ID;
}

// Removes a dead node from its table, clears the record, bumps the generation and pushes the slot
// on the free list (recycle, interner/mod.rs:566-625). `free_pos` is the free-list position.
__device__ __forceinline__ void recycle_node(const DevInterner &I, uint32_t idx, unsigned long long free_pos) {
    uint64_t id = I.ids[idx];
    if (id_is_leaf(id)) {
        uint32_t v = node_value(I, idx);
        atomicCAS((unsigned long long *)(I.leaf_table + v), id, 0ull);
    } else {
        uint64_t h = I.hash[idx];
        uint32_t tag = slot_tag(h);
        uint64_t pos = h & I.table_mask;
        bool removed = false;
        for (uint32_t p = 0; p <= I.max_probes; ++p) {
            uint64_t s = ld_volatile(I.table + pos);
            if (s == SLOT_EMPTY) break;
            if (s == make_slot(tag, idx)) {
                atomicExch((unsigned long long *)(I.table + pos), SLOT_TOMB);
                removed = true;
                break;
            }
            pos = (pos + 1) & I.table_mask;
        }
        if (!removed) set_error(I, ERR_INTERNAL, 10);
        ulonglong2 *dst = reinterpret_cast<ulonglong2 *>(I.children + 8ull * idx);
        dst[0] = dst[1] = dst[2] = dst[3] = make_ulonglong2(0ull, 0ull);
    }
    set_node_value(I, idx, 0);
    I.hash[idx] = 0;
    I.refcount[idx] = 0;
    I.ids[idx] = 0;
    uint32_t g = (uint32_t)I.generation[idx] + 1u;
    if (g >= MAX_GENERATION) g = 0;
    I.generation[idx] = (uint16_t)g;
    I.free_list[free_pos] = idx;
}

// ---- grid barrier of single-launch (cooperative) kernels -------------------------------------------
// Every CTA of the grid must call it (all CTAs are resident: cooperative launch). Thread 0 arrives
// with a fence and waits, bounded, for the generation to move; the last to arrive resets the count
// and moves the generation with release semantics. Writes before the barrier are visible to every
// thread of the grid after it. Returns false if the wait gave up (ERR_TIMEOUT recorded).
__device__ __forceinline__ bool grid_sync(const DevInterner &I) {
    __shared__ int ok_s;
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = 1;
        const unsigned long long gen = ld_acquire(reinterpret_cast<const uint64_t *>(&I.ctr->bar_gen));
        __threadfence();
        if (atomicAdd(&I.ctr->bar_count, 1ull) == gridDim.x - 1) {
            I.ctr->bar_count = 0;
            st_release_u64(&I.ctr->bar_gen, gen + 1);
        } else {
            uint32_t spin = 0;
            while (ld_acquire(reinterpret_cast<const uint64_t *>(&I.ctr->bar_gen)) == gen) {
                // a CTA that gave up at an earlier barrier never arrives: stop waiting at once
                const bool gave_up = (spin & 1023u) == 1023u &&
                                     (*reinterpret_cast<volatile unsigned int *>(&I.ctr->error) & ERR_TIMEOUT);
                if (++spin >= I.spin_limit || gave_up) {
                    set_error(I, ERR_TIMEOUT, 49);
                    ok = 0;
                    break;
                }
                __nanosleep(32);
            }
        }
        __threadfence();
        ok_s = ok;
    }
    __syncthreads();
    return ok_s != 0;
}

// ---- release (dec_ref_recursive, interner/mod.rs:419-534, breadth first) ------------------------
// Counter slots of the release rounds in DevCounters::scratch (the batched-apply launcher's table
// lists every slot).
constexpr int kScRelease = 3, kScRelIn = 4, kScRelOut = 5;

// The dying set just produced becomes the input of the next round.
__device__ __forceinline__ void release_advance(const DevInterner &I) {
    I.ctr->scratch[kScRelIn] = I.ctr->scratch[kScRelOut];
    I.ctr->scratch[kScRelOut] = 0;
}

__device__ __forceinline__ void push_dying(uint32_t *list, unsigned long long *count, bool push, uint32_t idx) {
    const unsigned m = __ballot_sync(0xFFFFFFFFu, push);
    if (!m) return;
    const unsigned lane = threadIdx.x & 31u;
    unsigned long long base = 0;
    const int leader = __ffs(m) - 1;
    if ((int)lane == leader) base = atomicAdd(count, (unsigned long long)__popc(m));
    base = __shfl_sync(0xFFFFFFFFu, base, leader);
    if (push) list[base + __popc(m & ((1u << lane) - 1u))] = idx;
}

// Decrements each listed root (count at scratch[kScRelease]); roots whose count reaches zero become
// the first dying set. Entry cta_base + threadIdx.x, then + stride, ...: the loop is uniform across
// the CTA, so the warp votes inside see whole warps.
__device__ __forceinline__ void release_roots_range(const DevInterner &I, const uint64_t *list, uint32_t *out,
                                                    unsigned long long *n_out, uint64_t cta_base, uint64_t stride) {
    const uint64_t n = I.ctr->scratch[kScRelease];
    for (uint64_t base = cta_base; base < n; base += stride) {
        const uint64_t j = base + threadIdx.x;
        bool dies = false;
        uint32_t idx = 0;
        if (j < n) {
            const uint64_t id = list[j];
            if (id != EMPTY_ID) {
                idx = id_index(id);
                const unsigned old = atomicSub(I.refcount + idx, 1u);
                if (old == 0) {
                    atomicAdd(I.refcount + idx, 1u);
                    set_error(I, ERR_REF_UB, 60);
                } else {
                    dies = old == 1;
                }
            }
        }
        push_dying(out, n_out, dies, idx);
    }
}

// Retires the *n_in dying nodes of `in`: their children lose one reference each (children reaching
// zero are the next dying set, appended to `out` and counted in *n_out) and the nodes are recycled.
__device__ __forceinline__ void release_round_range(const DevInterner &I, const uint32_t *in, uint32_t *out,
                                                    const unsigned long long *n_in, unsigned long long *n_out,
                                                    uint64_t cta_base, uint64_t stride) {
    const uint64_t n = *n_in;
    const unsigned lane = threadIdx.x & 31u;
    for (uint64_t base = cta_base; base < n; base += stride) {
        const uint64_t j = base + threadIdx.x;
        const bool in_range = j < n;
        const uint32_t idx = in_range ? in[j] : 0u;
        const uint64_t id = in_range ? I.ids[idx] : 0ull;
        const bool branch = in_range && id != 0 && id_is_branch(id);
        for (int k = 0; k < 8; ++k) {
            bool dies = false;
            uint32_t cidx = 0;
            if (branch) {
                const uint64_t c = I.children[8ull * idx + k];
                if (c != EMPTY_ID) {
                    cidx = id_index(c);
                    const unsigned old = atomicSub(I.refcount + cidx, 1u);
                    if (old == 0) {
                        atomicAdd(I.refcount + cidx, 1u);
                        set_error(I, ERR_REF_UB, 61);
                    } else {
                        dies = old == 1;
                    }
                }
            }
            push_dying(out, n_out, dies, cidx);
        }
        const bool rec = in_range && id != 0;
        if (in_range && id == 0) set_error(I, ERR_INTERNAL, 62);
        const unsigned m = __ballot_sync(0xFFFFFFFFu, rec);
        unsigned long long fbase = 0;
        if (m) {
            const int leader = __ffs(m) - 1;
            if ((int)lane == leader) fbase = atomicAdd(&I.ctr->free_count, (unsigned long long)__popc(m));
            fbase = __shfl_sync(0xFFFFFFFFu, fbase, leader);
        }
        const unsigned tomb = __ballot_sync(0xFFFFFFFFu, rec && branch);
        if (lane == 0 && tomb) atomicAdd(&I.ctr->tombstones, (unsigned long long)__popc(tomb));
        if (rec) recycle_node(I, idx, fbase + __popc(m & ((1u << lane) - 1u)));
    }
}

}  // namespace vxg
