// World-level helpers for the serving loop: a grid of equal-depth chunks addressed by world voxel
// coordinates. Not part of the reference's API; they stage the same Batch contents the reference's
// callers build by hand (Batch::just_set per voxel, core/batch.rs:145-172) and read a world with
// VoxTree::get per chunk (voxtree.rs:145-159).
//
//   vx_stage_spheres    sphere brushes (center, radius, value) applied in order as just_set calls
//                       into one Batch per touched chunk, emitted as compacted touched groups
//                       sorted by (chunk, group) — the input of vx_apply_groups_async.
//   vx_world_get_async  batched get at world coordinates: chunk lookup in the device world table,
//                       then the per-tree descent of get_at_depth (utils/common.rs:122-156).
#include <algorithm>
#include <cstring>
#include <vector>

#include "../../include/voxelis_gb300.h"
#include "vx_launch.h"

using namespace vxg;

namespace vxg {
bool interner_parts(vx_interner *it, DevInterner *dev, cudaStream_t *stream, int *num_sms, uint32_t *flags,
                    bool marks_trees);
void interner_set_error(vx_interner *it, const char *msg);
}  // namespace vxg

namespace {

uint32_t morton3(uint32_t x, uint32_t y, uint32_t z) {
    auto split = [](uint32_t v) {
        v &= 0x3FF;
        v = (v | (v << 16)) & 0x30000FF;
        v = (v | (v << 8)) & 0x300F00F;
        v = (v | (v << 4)) & 0x30C30C3;
        v = (v | (v << 2)) & 0x9249249;
        return v;
    };
    return split(x) | (split(y) << 1) | (split(z) << 2);
}

struct GroupRec {
    uint64_t key;  // chunk << 32 | group
    uint8_t set, clear;
    uint16_t vals[8];
};

// Open-addressing map key -> record slot, grown at load 1/2.
struct RecMap {
    std::vector<uint64_t> keys;
    std::vector<uint32_t> slot;
    std::vector<GroupRec> recs;
    uint64_t mask = 0;
    void init(size_t cap) {
        size_t n = 1024;
        while (n < 2 * cap) n <<= 1;
        keys.assign(n, ~0ull);
        slot.assign(n, 0);
        mask = n - 1;
        recs.clear();
    }
    GroupRec &at(uint64_t key) {
        if ((recs.size() + 1) * 2 > keys.size()) grow();
        uint64_t h = (key * 0x9E3779B97F4A7C15ull) >> 20;
        for (;;) {
            const uint64_t i = h & mask;
            if (keys[i] == key) return recs[slot[i]];
            if (keys[i] == ~0ull) {
                keys[i] = key;
                slot[i] = (uint32_t)recs.size();
                GroupRec r{};
                r.key = key;
                recs.push_back(r);
                return recs.back();
            }
            ++h;
        }
    }
    void grow() {
        std::vector<GroupRec> old;
        old.swap(recs);
        init(old.size() * 2 + 16);
        for (auto &r : old) {
            GroupRec &n = at(r.key);
            n = r;
        }
    }
};

// Gets at world coordinates. With old_roots, a chunk whose edit_rank is cut or more (and not
// kNoRank) is read at the root held for it before the wave's apply (see vx_world_hold_async).
constexpr uint32_t kNoRank = 0xFFFFFFFFu;

template <class T>
__global__ void world_get_kernel(DevInterner I, vx_world W, uint64_t n, const int32_t *xyz, uint8_t *found,
                                 T *values, const uint64_t *old_roots, const uint32_t *edit_rank, uint32_t cut) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    const int d = W.chunk_depth;
    const int32_t side = 1 << d;
    bool oob = false;
    for (uint64_t q = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += stride) {
        const int32_t x = __ldg(xyz + 3 * q), y = __ldg(xyz + 3 * q + 1), z = __ldg(xyz + 3 * q + 2);
        uint32_t val = 0;
        uint8_t f = 0;
        if (x < 0 || y < 0 || z < 0 || x >= W.nx * side || y >= W.ny * side || z >= W.nz * side) {
            oob = true;
        } else {
            const uint32_t chunk = ((uint32_t)(y >> d) * W.nz + (uint32_t)(z >> d)) * W.nx + (uint32_t)(x >> d);
            const uint32_t t = __ldg(W.trees_dev + chunk);
            const int32_t lx = x & (side - 1), ly = y & (side - 1), lz = z & (side - 1);
            uint64_t node = t < I.tree_cap ? I.roots[t] : EMPTY_ID;
            if (old_roots) {
                const uint32_t r = __ldg(edit_rank + chunk);
                if (r != kNoRank && r >= cut) node = __ldg(reinterpret_cast<const unsigned long long *>(old_roots) + chunk);
            }
            int depth = 0;
            while (node != EMPTY_ID) {
                if (depth >= d) {
                    const uint32_t v = node_value(I, id_index(node));
                    if (v) {
                        val = v;
                        f = 1;
                    }
                    break;
                }
                if (id_is_branch(node)) {
                    const int sh = d - depth - 1;
                    const uint32_t ci = ((lx >> sh) & 1) | (((ly >> sh) & 1) << 1) | (((lz >> sh) & 1) << 2);
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
    if (oob) set_error(I, ERR_OOB, 90);
}

// Holds the current root of each listed chunk for the gets of a wave that must not see the wave's
// edits: one more reference on it (VoxInterner::inc_ref, interner/mod.rs:235-260), its id in
// held[k] and old_roots[chunk], the rank of the wave's edit of that chunk in edit_rank[chunk].
__global__ void world_hold_kernel(DevInterner I, vx_world W, uint32_t n, const uint32_t *chunks, const uint32_t *ranks,
                                  uint64_t *held, uint64_t *old_roots, uint32_t *edit_rank) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const uint32_t c = chunks[k];
    if (c >= (uint32_t)(W.nx * W.ny * W.nz)) {
        set_error(I, ERR_OOB, 91);
        held[k] = EMPTY_ID;
        return;
    }
    const uint32_t t = W.trees_dev[c];
    const uint64_t root = t < I.tree_cap ? I.roots[t] : EMPTY_ID;
    held[k] = root;
    old_roots[c] = root;
    edit_rank[c] = ranks[k];
    if (root != EMPTY_ID) atomicAdd(I.refcount + id_index(root), 1u);
}

// Ends the holds: the listed chunks read their current roots again, and the held ids become the
// list of the release that follows (count in the release slot).
__global__ void world_unhold_kernel(DevInterner I, vx_world W, uint32_t n, const uint32_t *chunks, uint32_t *edit_rank) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k == 0) I.ctr->scratch[SC_RELEASE] = n;
    if (k < n && chunks[k] < (uint32_t)(W.nx * W.ny * W.nz)) edit_rank[chunks[k]] = kNoRank;
}

}  // namespace

extern "C" int vx_stage_spheres(int chunk_depth, int32_t nx, int32_t ny, int32_t nz, uint32_t n,
                                const int32_t *centers, const int32_t *radii, const uint32_t *values,
                                uint64_t cap_items, uint32_t *item_chunks, uint64_t cap_records, uint32_t *rec_item,
                                uint32_t *rec_group, uint8_t *rec_set, uint8_t *rec_clear, uint16_t *rec_vals,
                                uint64_t *n_items, uint64_t *n_records) {
    if (chunk_depth < 1 || chunk_depth > 10 || nx <= 0 || ny <= 0 || nz <= 0 || !n_items || !n_records ||
        (n && (!centers || !radii || !values)))
        return VX_E_INVALID_ARG;
    const int32_t side = 1 << chunk_depth;
    const int32_t WX = nx * side, WY = ny * side, WZ = nz * side;
    RecMap map;
    map.init(4096);
    for (uint32_t s = 0; s < n; ++s) {
        const int32_t cx = centers[3 * s], cy = centers[3 * s + 1], cz = centers[3 * s + 2], r = radii[s];
        const uint32_t v = values[s];
        if (r < 0 || v > 0xFFFF) return VX_E_INVALID_ARG;
        const int32_t x0 = std::max(0, cx - r) & ~1, x1 = std::min(WX - 1, cx + r);
        const int32_t y0 = std::max(0, cy - r) & ~1, y1 = std::min(WY - 1, cy + r);
        const int32_t z0 = std::max(0, cz - r) & ~1, z1 = std::min(WZ - 1, cz + r);
        const int64_t r2 = (int64_t)r * r;
        for (int32_t gy = y0; gy <= y1; gy += 2)
            for (int32_t gz = z0; gz <= z1; gz += 2)
                for (int32_t gx = x0; gx <= x1; gx += 2) {
                    GroupRec *rec = nullptr;
                    for (int k = 0; k < 8; ++k) {
                        const int32_t x = gx + (k & 1), y = gy + ((k >> 1) & 1), z = gz + (k >> 2);
                        if (x > x1 || y > y1 || z > z1 || x < std::max(0, cx - r) || y < std::max(0, cy - r) ||
                            z < std::max(0, cz - r))
                            continue;
                        const int64_t dx = x - cx, dy = y - cy, dz = z - cz;
                        if (dx * dx + dy * dy + dz * dz > r2) continue;
                        if (!rec) {
                            const uint32_t chunk = ((uint32_t)(y >> chunk_depth) * nz + (uint32_t)(z >> chunk_depth)) * nx +
                                                   (uint32_t)(x >> chunk_depth);
                            const uint32_t lx = x & (side - 1), ly = y & (side - 1), lz = z & (side - 1);
                            const uint32_t group = morton3(lx, ly, lz) >> 3;
                            rec = &map.at(((uint64_t)chunk << 32) | group);
                        }
                        // just_set (batch.rs:145-172): last write wins, a zero value records a clear
                        const uint8_t bit = (uint8_t)(1u << k);
                        if (v) {
                            rec->set |= bit;
                            rec->clear &= (uint8_t)~bit;
                        } else {
                            rec->set &= (uint8_t)~bit;
                            rec->clear |= bit;
                        }
                        rec->vals[k] = (uint16_t)v;
                    }
                }
    }
    std::vector<uint32_t> order(map.recs.size());
    for (uint32_t i = 0; i < order.size(); ++i) order[i] = i;
    std::sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return map.recs[a].key < map.recs[b].key; });
    uint64_t items = 0;
    uint64_t last_chunk = ~0ull;
    for (uint32_t i : order) {
        const uint64_t ch = map.recs[i].key >> 32;
        if (ch != last_chunk) {
            ++items;
            last_chunk = ch;
        }
    }
    *n_items = items;
    *n_records = order.size();
    if (items > cap_items || order.size() > cap_records) return VX_E_BUFFER;
    if (!order.empty() && (!item_chunks || !rec_item || !rec_group || !rec_set || !rec_clear || !rec_vals))
        return VX_E_INVALID_ARG;
    int64_t item = -1;
    last_chunk = ~0ull;
    for (uint64_t j = 0; j < order.size(); ++j) {
        const GroupRec &g = map.recs[order[j]];
        const uint64_t ch = g.key >> 32;
        if (ch != last_chunk) {
            ++item;
            item_chunks[item] = (uint32_t)ch;
            last_chunk = ch;
        }
        rec_item[j] = (uint32_t)item;
        rec_group[j] = (uint32_t)(g.key & 0xFFFFFFFFu);
        rec_set[j] = g.set;
        rec_clear[j] = g.clear;
        std::memcpy(rec_vals + 8 * j, g.vals, 16);
    }
    return VX_OK;
}

extern "C" int vx_world_get_async(vx_interner *it, const vx_world *world, uint64_t n, const int32_t *world_xyz_dev,
                                  uint8_t *found_dev, void *values_dev) {
    DevInterner D;
    cudaStream_t s;
    int num_sms;
    uint32_t flags;
    if (!interner_parts(it, &D, &s, &num_sms, &flags, false) || !world) return VX_E_INVALID_ARG;
    if (n == 0) return VX_OK;
    if (!world->trees_dev || !world_xyz_dev || !found_dev || !values_dev || world->chunk_depth < 0 ||
        world->chunk_depth > 10)
        return VX_E_INVALID_ARG;
    uint64_t blocks = (n + 255) / 256;
    if (blocks > (uint64_t)num_sms * 16) blocks = (uint64_t)num_sms * 16;
    count_launches(1);
    if (D.vbits == 8)
        world_get_kernel<uint8_t><<<(unsigned)blocks, 256, 0, s>>>(D, *world, n, world_xyz_dev, found_dev,
                                                                   (uint8_t *)values_dev, nullptr, nullptr, 0);
    else
        world_get_kernel<uint16_t><<<(unsigned)blocks, 256, 0, s>>>(D, *world, n, world_xyz_dev, found_dev,
                                                                    (uint16_t *)values_dev, nullptr, nullptr, 0);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        interner_set_error(it, cudaGetErrorString(e));
        return VX_E_CUDA;
    }
    return VX_OK;
}

extern "C" int vx_world_hold_async(vx_interner *it, const vx_world *world, uint32_t n, const uint32_t *chunks_dev,
                                   const uint32_t *ranks_dev, uint64_t *held_dev, uint64_t *old_roots_dev,
                                   uint32_t *edit_rank_dev) {
    DevInterner D;
    cudaStream_t s;
    int num_sms;
    uint32_t flags;
    if (!interner_parts(it, &D, &s, &num_sms, &flags, false) || !world) return VX_E_INVALID_ARG;
    if (n == 0) return VX_OK;
    if (!world->trees_dev || !chunks_dev || !ranks_dev || !held_dev || !old_roots_dev || !edit_rank_dev)
        return VX_E_INVALID_ARG;
    count_launches(1);
    world_hold_kernel<<<(n + 255) / 256, 256, 0, s>>>(D, *world, n, chunks_dev, ranks_dev, held_dev, old_roots_dev,
                                                      edit_rank_dev);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        interner_set_error(it, cudaGetErrorString(e));
        return VX_E_CUDA;
    }
    return VX_OK;
}

extern "C" int vx_world_get_at_async(vx_interner *it, const vx_world *world, uint64_t n, const int32_t *world_xyz_dev,
                                     uint8_t *found_dev, void *values_dev, const uint64_t *old_roots_dev,
                                     const uint32_t *edit_rank_dev, uint32_t cut) {
    DevInterner D;
    cudaStream_t s;
    int num_sms;
    uint32_t flags;
    if (!interner_parts(it, &D, &s, &num_sms, &flags, false) || !world) return VX_E_INVALID_ARG;
    if (n == 0) return VX_OK;
    if (!world->trees_dev || !world_xyz_dev || !found_dev || !values_dev || !old_roots_dev || !edit_rank_dev ||
        world->chunk_depth < 0 || world->chunk_depth > 10)
        return VX_E_INVALID_ARG;
    uint64_t blocks = (n + 255) / 256;
    if (blocks > (uint64_t)num_sms * 16) blocks = (uint64_t)num_sms * 16;
    count_launches(1);
    if (D.vbits == 8)
        world_get_kernel<uint8_t><<<(unsigned)blocks, 256, 0, s>>>(D, *world, n, world_xyz_dev, found_dev,
                                                                   (uint8_t *)values_dev, old_roots_dev, edit_rank_dev,
                                                                   cut);
    else
        world_get_kernel<uint16_t><<<(unsigned)blocks, 256, 0, s>>>(D, *world, n, world_xyz_dev, found_dev,
                                                                    (uint16_t *)values_dev, old_roots_dev,
                                                                    edit_rank_dev, cut);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        interner_set_error(it, cudaGetErrorString(e));
        return VX_E_CUDA;
    }
    return VX_OK;
}

namespace vxg {
int interner_release_list(vx_interner *it, uint64_t *list_dev, int rounds);
}

extern "C" int vx_world_release_async(vx_interner *it, const vx_world *world, uint32_t n, const uint32_t *chunks_dev,
                                      uint64_t *held_dev, uint32_t *edit_rank_dev) {
    DevInterner D;
    cudaStream_t s;
    int num_sms;
    uint32_t flags;
    if (!interner_parts(it, &D, &s, &num_sms, &flags, false) || !world) return VX_E_INVALID_ARG;
    if (n == 0) return VX_OK;
    if (!world->trees_dev || !chunks_dev || !held_dev || !edit_rank_dev || world->chunk_depth < 0 ||
        world->chunk_depth > 10)
        return VX_E_INVALID_ARG;
    count_launches(1);
    world_unhold_kernel<<<(n + 255) / 256, 256, 0, s>>>(D, *world, n, chunks_dev, edit_rank_dev);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        interner_set_error(it, cudaGetErrorString(e));
        return VX_E_CUDA;
    }
    // dec_ref_recursive of every held root: a held root the apply replaced dies here
    return interner_release_list(it, held_dev, world->chunk_depth + 1);
}

// n host -> device copies on the interner's stream, one cudaMemcpyAsync each (serving loops stage a
// wave's arrays with one call instead of one runtime call per array from Python).
extern "C" int vx_copy_to_device_async(vx_interner *it, uint32_t n, void *const *dst_dev, const void *const *src_host,
                                       const uint64_t *bytes) {
    DevInterner D;
    cudaStream_t s;
    int num_sms;
    uint32_t flags;
    if (!interner_parts(it, &D, &s, &num_sms, &flags, false)) return VX_E_INVALID_ARG;
    if (n && (!dst_dev || !src_host || !bytes)) return VX_E_INVALID_ARG;
    for (uint32_t k = 0; k < n; ++k) {
        if (!bytes[k]) continue;
        const cudaError_t e = cudaMemcpyAsync(dst_dev[k], src_host[k], bytes[k], cudaMemcpyHostToDevice, s);
        if (e != cudaSuccess) {
            interner_set_error(it, cudaGetErrorString(e));
            return VX_E_CUDA;
        }
    }
    return VX_OK;
}
