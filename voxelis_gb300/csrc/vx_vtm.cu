// Model deserialisation on the device: VoxModel::deserialize (world/voxmodel.rs:284-408) with
// VoxInterner::deserialize_leaf / preallocate_branch_id / deserialize_branch (interner/mod.rs:930-993)
// and deserialize_chunk (world/voxchunk.rs:408-440), for a payload in the layout VoxModel::serialize
// writes:
//   u32 L | L leaf records  varint(id) value
//   u32 B | B branch records varint(id) u8 mask, varint(child id) per set mask bit, LOD value
//   u32 C | C chunk records  "VoxTreeChunk" i32 x y z, varint(root id)
// (u32 / i32 / values big-endian; varints as io/varint.rs:47-69: 7 bits a byte, low group first, at
// most 5 bytes). Into an interner that holds no node yet, record ids are the slots the nodes land on
// (the reference asserts each id equals the next index allocated): leaves 1..L, branches L+1..L+B.
//
// Parsing. Record boundaries depend on every byte before them, so a section is parsed speculatively
// in segments of S bytes: for each segment and each entry offset o < 64 (more than the longest record,
// 48 bytes) one lane parses the section's records from segment start + o while they start inside the
// segment, giving table T0[seg][o] = records << 8 | exit offset into the next segment (or dead, when
// a record fails to parse). Tables of 32 consecutive segments compose into T1, those of 32 T1 into T2
// (S is chosen so that a section has at most 32^3 segments). One CTA then walks T2 from entry 0 and
// walks down, giving every segment its true entry offset and the number of records before it; one
// thread per segment re-parses its records from there, validates each against the reference's
// assertions, records its offset by rank, and the thread that parses the section's last record reads
// the next section's header. Sections run one after another (each start is the previous one's end).
//
// Placement. With L, B and C known the host creates C trees; then one kernel writes every leaf and
// the BlockId of every branch (types = which children are leaves), and a second writes the branch
// records (children, LOD value, fingerprint), inserts them into the branch table, adds one reference
// per child slot naming a node (inc_all_child_refs, interner/mod.rs:328-356) and one per chunk root
// (set_root_id, voxtree.rs:135-141: the EMPTY slot too), all with warp-aggregated atomics.
#include "vx_launch.h"

namespace vxg {

namespace {

constexpr int kThreads = 256;
constexpr int kEntries = 64;  // entry offsets per segment
constexpr int kFan = 32;      // tables composed per table of the level above
constexpr uint64_t kDead = ~0ull;

// decode_varint_u32_from_reader (io/varint.rs:47-69): bits past 32 of a fifth byte are dropped, a
// continuation bit on the fifth byte fails. Returns the bytes used, 0 on failure.
__device__ __forceinline__ int vtm_varint(const uint8_t *b, uint64_t p, uint64_t n, uint32_t *v) {
    uint32_t r = 0;
#pragma unroll
    for (int k = 0; k < 5; ++k) {
        if (p + k >= n) return 0;
        const uint32_t c = b[p + k];
        r |= (c & 0x7Fu) << (7 * k);
        if (c < 0x80u) {
            *v = r;
            return k + 1;
        }
    }
    return 0;
}

__device__ __forceinline__ uint32_t vtm_be32(const uint8_t *b, uint64_t p) {
    return ((uint32_t)b[p] << 24) | ((uint32_t)b[p + 1] << 16) | ((uint32_t)b[p + 2] << 8) | (uint32_t)b[p + 3];
}

__device__ __forceinline__ uint32_t vtm_value(const uint8_t *b, uint64_t p, int vb) {
    return vb == 2 ? ((uint32_t)b[p] << 8) | (uint32_t)b[p + 1] : (uint32_t)b[p];
}

// Length of the record of section `kind` (0 leaf, 1 branch, 2 chunk) that starts at p, 0 when it
// does not parse or runs past the end of the stream.
__device__ __forceinline__ uint32_t vtm_record_len(int kind, const uint8_t *b, uint64_t p, uint64_t n, int vb) {
    uint32_t v;
    if (kind == 2) {
        const int l = vtm_varint(b, p + 24, n, &v);
        return l ? 24u + (uint32_t)l : 0u;
    }
    const int l = vtm_varint(b, p, n, &v);
    if (!l) return 0;
    uint64_t q = p + (uint64_t)l;
    if (kind == 1) {
        if (q >= n) return 0;
        const uint32_t mask = b[q++];
        for (int k = 0; k < 8; ++k) {
            if (!((mask >> k) & 1u)) continue;
            const int m = vtm_varint(b, q, n, &v);
            if (!m) return 0;
            q += (uint64_t)m;
        }
    }
    if (q + (uint64_t)vb > n) return 0;
    return (uint32_t)(q + (uint64_t)vb - p);
}

// The checks the reference makes while reading a record (as panics): leaf ids 1..L in order and a
// non-default value (deserialize_leaf's debug assertion); branch ids L+1..L+B in order, a non-empty
// mask, child ids naming a node or 0 (EMPTY, which the reference's branch map holds); the chunk magic
// and a root id naming a node or EMPTY.
__device__ __forceinline__ bool vtm_record_ok(int kind, const uint8_t *b, uint64_t p, uint64_t rank, uint64_t L,
                                              uint64_t B, int vb) {
    uint32_t v = 0;
    if (kind == 2) {
        const char magic[12] = {'V', 'o', 'x', 'T', 'r', 'e', 'e', 'C', 'h', 'u', 'n', 'k'};
        for (int j = 0; j < 12; ++j)
            if (b[p + j] != (uint8_t)magic[j]) return false;
        vtm_varint(b, p + 24, ~0ull, &v);
        return (uint64_t)v <= L + B;
    }
    const int l = vtm_varint(b, p, ~0ull, &v);
    if (kind == 0) return (uint64_t)v == rank + 1 && vtm_value(b, p + l, vb) != 0;
    if ((uint64_t)v != L + 1 + rank) return false;
    uint64_t q = p + (uint64_t)l;
    const uint32_t mask = b[q++];
    if (mask == 0) return false;
    for (int k = 0; k < 8; ++k) {
        if (!((mask >> k) & 1u)) continue;
        q += (uint64_t)vtm_varint(b, q, ~0ull, &v);
        if ((uint64_t)v > L + B) return false;
    }
    return true;
}

struct Geometry {
    uint64_t start;  // first byte of the section
    uint32_t n0;     // segments
    uint32_t n1, n2;  // tables of the two composed levels
};

__device__ __forceinline__ Geometry vtm_geometry(const VtmSections *sec, int kind, uint64_t n, uint32_t S) {
    Geometry g;
    g.start = sec->start[kind];
    const uint64_t len = g.start < n ? n - g.start : 0;
    g.n0 = (uint32_t)((len + S - 1) / S);
    g.n1 = (g.n0 + kFan - 1) / kFan;
    g.n2 = (g.n1 + kFan - 1) / kFan;
    return g;
}

// Applies one table to a packed state (records before << 8 | entry offset).
__device__ __forceinline__ uint64_t vtm_step(uint64_t e, const uint64_t *T) {
    if (e == kDead) return kDead;
    const uint64_t t = T[e & 0xFFu];
    if (t == kDead) return kDead;
    return (((e >> 8) + (t >> 8)) << 8) | (t & 0xFFu);
}

__global__ void __launch_bounds__(kThreads) vtm_table_kernel(const uint8_t *b, uint64_t n, const VtmSections *sec,
                                                             int kind, int vb, uint32_t S, uint64_t *T0) {
    if (sec->count[kind] == 0) return;
    const Geometry g = vtm_geometry(sec, kind, n, S);
    const unsigned lane = threadIdx.x & 31u;
    const uint32_t warps = gridDim.x * (blockDim.x / 32);
    for (uint32_t seg = (blockIdx.x * blockDim.x + threadIdx.x) / 32; seg < g.n0; seg += warps) {
        const uint64_t s0 = g.start + (uint64_t)seg * S;
        const uint64_t end = s0 + S < n ? s0 + S : n;
        for (int h = 0; h < kEntries / 32; ++h) {
            const uint32_t o = lane + 32u * h;
            uint64_t pos = s0 + o, cnt = 0;
            bool ok = true;
            while (pos < end) {
                const uint32_t l = vtm_record_len(kind, b, pos, n, vb);
                if (!l) {
                    ok = false;
                    break;
                }
                pos += l;
                ++cnt;
            }
            T0[(uint64_t)seg * kEntries + o] = ok ? (cnt << 8) | (pos - end) : kDead;
        }
    }
}

// U[g][o] = the kFan child tables of group g applied in turn from entry o (one warp per group).
__global__ void __launch_bounds__(kThreads) vtm_compose_kernel(uint64_t n, const VtmSections *sec, int kind, uint32_t S,
                                                               int level, const uint64_t *T, uint64_t *U) {
    if (sec->count[kind] == 0) return;
    const Geometry geo = vtm_geometry(sec, kind, n, S);
    const uint32_t n_child = level == 1 ? geo.n0 : geo.n1, n_group = level == 1 ? geo.n1 : geo.n2;
    const unsigned lane = threadIdx.x & 31u;
    const uint32_t warps = gridDim.x * (blockDim.x / 32);
    for (uint32_t g = (blockIdx.x * blockDim.x + threadIdx.x) / 32; g < n_group; g += warps) {
        for (int h = 0; h < kEntries / 32; ++h) {
            const uint32_t o = lane + 32u * h;
            uint64_t e = o;
            for (uint32_t j = 0; j < (uint32_t)kFan && (uint64_t)g * kFan + j < n_child; ++j)
                e = vtm_step(e, T + ((uint64_t)g * kFan + j) * kEntries);
            U[(uint64_t)g * kEntries + o] = e;
        }
    }
}

// One CTA of 1024 threads: the true entry state of every T2 group, T1 group and segment.
__global__ void __launch_bounds__(1024) vtm_down_kernel(uint64_t n, const VtmSections *sec, int kind, uint32_t S,
                                                        const uint64_t *T0, const uint64_t *T1, const uint64_t *T2,
                                                        uint64_t *E0, uint64_t *E1, uint64_t *E2) {
    if (sec->count[kind] == 0) return;
    const Geometry g = vtm_geometry(sec, kind, n, S);
    if (threadIdx.x == 0) {
        uint64_t e = 0;
        for (uint32_t k = 0; k < g.n2; ++k) {
            E2[k] = e;
            e = vtm_step(e, T2 + (uint64_t)k * kEntries);
        }
    }
    __syncthreads();
    if (threadIdx.x < g.n2) {
        uint64_t e = E2[threadIdx.x];
        for (uint32_t j = 0; j < (uint32_t)kFan && threadIdx.x * kFan + j < g.n1; ++j) {
            E1[threadIdx.x * kFan + j] = e;
            e = vtm_step(e, T1 + ((uint64_t)threadIdx.x * kFan + j) * kEntries);
        }
    }
    __syncthreads();
    for (uint32_t h = threadIdx.x; h < g.n1; h += blockDim.x) {
        uint64_t e = E1[h];
        for (uint32_t j = 0; j < (uint32_t)kFan && (uint64_t)h * kFan + j < g.n0; ++j) {
            E0[(uint64_t)h * kFan + j] = e;
            e = vtm_step(e, T0 + ((uint64_t)h * kFan + j) * kEntries);
        }
    }
}

// The section ends at `end`: the next section's header (its record count) follows.
__device__ void vtm_close(const DevInterner &I, const uint8_t *b, uint64_t n, VtmSections *sec, int kind,
                          uint64_t end) {
    if (kind < 2) {
        if (end + 4 > n) {
            set_error(I, ERR_REF_PANIC, 40 + kind);  // read_u32 of the next count fails
            return;
        }
        sec->count[kind + 1] = vtm_be32(b, end);
        sec->start[kind + 1] = end + 4;
    } else {
        sec->start[3] = end;
    }
    sec->done[kind] = 1;
}

__global__ void __launch_bounds__(kThreads) vtm_emit_kernel(DevInterner I, const uint8_t *b, uint64_t n,
                                                            VtmSections *sec, int kind, int vb, uint32_t S,
                                                            const uint64_t *E0, uint32_t *off, uint64_t cap) {
    const uint64_t count = sec->count[kind];
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (sec->start[kind] > n) return;  // an earlier section failed (its error bit is set)
    if (count == 0) {
        if (t == 0) vtm_close(I, b, n, sec, kind, sec->start[kind]);
        return;
    }
    const Geometry g = vtm_geometry(sec, kind, n, S);
    if (g.n0 == 0) {
        if (t == 0) set_error(I, ERR_REF_PANIC, 43 + kind);  // records announced past the end
        return;
    }
    if (t >= g.n0) return;
    const uint64_t e = E0[t];
    if (e == kDead) return;
    uint64_t rank = e >> 8;
    if (rank >= count) return;
    const uint64_t L = sec->count[0], B = kind >= 1 ? sec->count[1] : 0;
    uint64_t pos = g.start + (uint64_t)t * S + (e & 0xFFu);
    const uint64_t end = g.start + (uint64_t)(t + 1) * S < n ? g.start + (uint64_t)(t + 1) * S : n;
    while (pos < end) {
        const uint32_t len = vtm_record_len(kind, b, pos, n, vb);
        if (!len || rank >= cap) {
            set_error(I, ERR_REF_PANIC, 46 + kind);  // truncated record
            return;
        }
        if (!vtm_record_ok(kind, b, pos, rank, L, B, vb)) {
            set_error(I, ERR_REF_PANIC, 49 + kind);
            return;
        }
        off[rank] = (uint32_t)pos;
        pos += len;
        if (++rank == count) {
            vtm_close(I, b, n, sec, kind, pos);
            return;
        }
    }
}

// Leaves at slots 1..L (value, leaf table) and the BlockId of every branch at L+1..L+B.
__global__ void __launch_bounds__(kThreads) vtm_nodes_kernel(DevInterner I, const uint8_t *b, const VtmSections *sec,
                                                             const uint32_t *leaf_off, const uint32_t *branch_off,
                                                             int vb) {
    const uint64_t L = sec->count[0], B = sec->count[1];
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < L + B; i += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t v = 0;
        const uint32_t idx = (uint32_t)(i + 1);
        uint64_t id;
        if (i < L) {
            const uint64_t p = leaf_off[i];
            const int l = vtm_varint(b, p, ~0ull, &v);
            const uint32_t value = vtm_value(b, p + l, vb);
            id = make_leaf_id(idx, 0);
            set_node_value(I, idx, value);
            I.hash[idx] = 0;
            // the later of two equal leaves is the one the table finds (the reference's map insert)
            atomicMax((unsigned long long *)(I.leaf_table + value), (unsigned long long)id);
        } else {
            uint64_t q = branch_off[i - L];
            q += (uint64_t)vtm_varint(b, q, ~0ull, &v);
            const uint32_t mask = b[q++];
            uint32_t types = 0;
            for (int k = 0; k < 8; ++k) {
                if (!((mask >> k) & 1u)) continue;
                q += (uint64_t)vtm_varint(b, q, ~0ull, &v);
                if (v >= 1 && (uint64_t)v <= L) types |= 1u << k;
            }
            id = make_branch_id(idx, 0, types, mask);
        }
        I.generation[idx] = 0;
        I.refcount[idx] = 0;
        I.ids[idx] = id;
    }
}

// Insert of a deserialised branch into the branch table. Keys of one stream are distinct unless the
// stream holds a pattern twice; then the first insert stays findable (the reference keeps one of the
// two in its map as well).
__device__ void vtm_insert(const DevInterner &I, uint32_t idx, const uint64_t c[8], uint32_t types, uint32_t mask,
                           uint64_t h) {
    const uint32_t tag = slot_tag(h);
    uint64_t pos = h & I.table_mask;
    for (uint32_t probes = 0; probes <= I.max_probes; ++probes) {
        uint64_t s = ld_probe(I.table + pos);
        if (s == SLOT_EMPTY) {
            const unsigned long long prev =
                atom_cas_acq_rel((unsigned long long *)(I.table + pos), SLOT_EMPTY, make_slot(tag, idx));
            if (prev == SLOT_EMPTY) return;
            s = prev;
        }
        if ((uint32_t)(s >> 32) == tag && s != SLOT_TOMB && (uint32_t)s != IDX_BUSY &&
            key_equal(I, (uint32_t)s, c, types, mask))
            return;
        pos = (pos + 1) & I.table_mask;
    }
    set_error(I, ERR_TABLE_FULL, 52);
}

// Branch records (children, LOD, fingerprint, table insert, child references) and chunk roots.
__global__ void __launch_bounds__(kThreads) vtm_links_kernel(DevInterner I, const uint8_t *b, const VtmSections *sec,
                                                             const uint32_t *branch_off, const uint32_t *chunk_off,
                                                             const uint32_t *trees, int32_t *positions, int vb) {
    const uint64_t L = sec->count[0], B = sec->count[1], C = sec->count[2];
    const unsigned lane = threadIdx.x & 31u;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t base = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) & ~31ull; base < B + C; base += stride) {
        const uint64_t k = base + lane;
        uint32_t ref[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) ref[j] = NO_NODE;
        uint64_t c[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        uint32_t types = 0, mask = 0, idx = 0;
        uint64_t h = 0;
        if (k < B) {
            idx = (uint32_t)(L + 1 + k);
            uint32_t v = 0;
            uint64_t q = branch_off[k];
            q += (uint64_t)vtm_varint(b, q, ~0ull, &v);
            mask = b[q++];
            for (int j = 0; j < 8; ++j) {
                if (!((mask >> j) & 1u)) continue;
                q += (uint64_t)vtm_varint(b, q, ~0ull, &v);
                if (v == 0) continue;  // EMPTY under a set mask bit, as the reference's branch map gives
                if ((uint64_t)v <= L) {
                    c[j] = make_leaf_id(v, 0);
                    types |= 1u << j;
                } else {
                    c[j] = I.ids[v];
                }
                ref[j] = v;
            }
            const uint32_t lod = vtm_value(b, q, vb);
            ulonglong2 *dst = reinterpret_cast<ulonglong2 *>(I.children + 8ull * idx);
#pragma unroll
            for (int j = 0; j < 4; ++j) dst[j] = make_ulonglong2(c[2 * j], c[2 * j + 1]);
            set_node_value(I, idx, lod);
            h = branch_fingerprint(c, (types << 8) | mask);
            I.hash[idx] = h;
        } else if (k < B + C) {
            const uint64_t j = k - B;
            const uint64_t p = chunk_off[j];
            for (int a = 0; a < 3; ++a) positions[3 * j + a] = (int32_t)vtm_be32(b, p + 12 + 4 * a);
            uint32_t r = 0;
            vtm_varint(b, p + 24, ~0ull, &r);
            const uint64_t root = r == 0 ? EMPTY_ID : ((uint64_t)r <= L ? make_leaf_id(r, 0) : I.ids[r]);
            I.roots[trees[j]] = root;
            ref[0] = r;  // set_root_id counts EMPTY too
        }
        // one atomic per distinct target within the warp, per child slot
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const unsigned peers = __match_any_sync(0xFFFFFFFFu, ref[j]);
            if (ref[j] != NO_NODE && (int)lane == __ffs(peers) - 1) atomicAdd(I.refcount + ref[j], (unsigned)__popc(peers));
        }
        if (k < B) vtm_insert(I, idx, c, types, mask, h);
    }
}

__global__ void vtm_finish_kernel(DevInterner I, const VtmSections *sec) {
    const unsigned long long nodes = sec->count[0] + sec->count[1];
    I.ctr->next_index = 1 + nodes;
    I.ctr->created += nodes;
}

}  // namespace

uint32_t vtm_segment_bytes(uint64_t n) {
    uint64_t s = (n + 32767) / 32768;  // at most 32^3 segments a section
    s = (s + 63) & ~63ull;
    return (uint32_t)(s < 256 ? 256 : s);
}

VtmScratchSizes vtm_scratch_sizes(uint64_t n) {
    const uint32_t S = vtm_segment_bytes(n);
    VtmScratchSizes z;
    z.seg_bytes = S;
    z.n0 = (n + S - 1) / S + 1;
    z.n1 = (z.n0 + kFan - 1) / kFan + 1;
    z.n2 = (z.n1 + kFan - 1) / kFan + 1;
    z.table_words = (z.n0 + z.n1 + z.n2) * kEntries;
    z.entry_words = z.n0 + z.n1 + z.n2;
    z.leaf_cap = n / 2 + 1;     // a leaf record holds at least 2 bytes
    z.branch_cap = n / 3 + 1;   // a branch record at least 3
    z.chunk_cap = n / 25 + 1;   // a chunk record at least 25
    return z;
}

cudaError_t launch_vtm_parse(const DevInterner &I, const uint8_t *bytes, uint64_t n, VtmSections *sec,
                             uint64_t *tables, uint64_t *entries, uint32_t *leaf_off, uint32_t *branch_off,
                             uint32_t *chunk_off, int num_sms, cudaStream_t s) {
    const VtmScratchSizes z = vtm_scratch_sizes(n);
    const int vb = I.vbits / 8;
    uint64_t *T0 = tables, *T1 = T0 + z.n0 * kEntries, *T2 = T1 + z.n1 * kEntries;
    uint64_t *E0 = entries, *E1 = E0 + z.n0, *E2 = E1 + z.n1;
    uint32_t *offs[3] = {leaf_off, branch_off, chunk_off};
    const uint64_t caps[3] = {z.leaf_cap, z.branch_cap, z.chunk_cap};
    auto blocks_for = [&](uint64_t items, int per_block) {
        uint64_t g = (items + per_block - 1) / per_block;
        const uint64_t cap = (uint64_t)num_sms * 16;
        return (unsigned)(g < 1 ? 1 : (g > cap ? cap : g));
    };
    for (int kind = 0; kind < 3; ++kind) {
        count_launches(5);
        vtm_table_kernel<<<blocks_for(z.n0, kThreads / 32), kThreads, 0, s>>>(bytes, n, sec, kind, vb, z.seg_bytes, T0);
        vtm_compose_kernel<<<blocks_for(z.n1, kThreads / 32), kThreads, 0, s>>>(n, sec, kind, z.seg_bytes, 1, T0, T1);
        vtm_compose_kernel<<<blocks_for(z.n2, kThreads / 32), kThreads, 0, s>>>(n, sec, kind, z.seg_bytes, 2, T1, T2);
        vtm_down_kernel<<<1, 1024, 0, s>>>(n, sec, kind, z.seg_bytes, T0, T1, T2, E0, E1, E2);
        vtm_emit_kernel<<<(unsigned)((z.n0 + kThreads - 1) / kThreads), kThreads, 0, s>>>(
            I, bytes, n, sec, kind, vb, z.seg_bytes, E0, offs[kind], caps[kind]);
    }
    return cudaGetLastError();
}

cudaError_t launch_vtm_place(const DevInterner &I, const uint8_t *bytes, const VtmSections *sec, uint64_t n_nodes,
                             uint64_t n_links, const uint32_t *leaf_off, const uint32_t *branch_off,
                             const uint32_t *chunk_off, const uint32_t *trees, int32_t *positions, int num_sms,
                             cudaStream_t s) {
    const int vb = I.vbits / 8;
    auto blocks_for = [&](uint64_t items) {
        uint64_t g = (items + kThreads - 1) / kThreads;
        const uint64_t cap = (uint64_t)num_sms * 8;
        return (unsigned)(g < 1 ? 1 : (g > cap ? cap : g));
    };
    count_launches(3);
    vtm_nodes_kernel<<<blocks_for(n_nodes), kThreads, 0, s>>>(I, bytes, sec, leaf_off, branch_off, vb);
    vtm_links_kernel<<<blocks_for(n_links), kThreads, 0, s>>>(I, bytes, sec, branch_off, chunk_off, trees, positions,
                                                              vb);
    vtm_finish_kernel<<<1, 1, 0, s>>>(I, sec);
    return cudaGetLastError();
}

}  // namespace vxg
