// C ABI over the CPU restatement in vx_oracle.hpp — TEST INFRASTRUCTURE ONLY (the oracle).
//
// The entry points mirror include/voxelis_gb300.h one for one with a `vxo_` prefix, so that a test
// can drive the oracle and the GPU library through the same calls and compare the results.
// Reference panics become VX_E_REF_PANIC / VX_E_OOM / VX_E_OOB, reference undefined behaviour
// becomes VX_E_REF_UB; the message is available from vxo_last_error.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <memory>
#include <thread>
#include <unordered_map>

#include "../include/voxelis_gb300.h"
#include "vx_oracle.hpp"

namespace {

struct OBatchBase {
    virtual ~OBatchBase() = default;
    int bits = 8;
    uint32_t flags = 0;
};
template <class T>
struct OBatch : OBatchBase {
    vxo::Batch<T> b;
    OBatch(int depth, uint32_t f) : b(depth, f) {
        bits = 8 * (int)sizeof(T);
        flags = f;
    }
};

struct OInternerBase {
    virtual ~OInternerBase() = default;
    int bits = 8;
    uint32_t flags = 0;
    std::string last_error;
};

template <class T>
struct OInterner : OInternerBase {
    vxo::Interner<T> it;
    std::vector<std::unique_ptr<vxo::Tree<T>>> trees;
    std::vector<uint32_t> free_slots;
    OInterner(size_t budget, uint32_t f) : it(budget, f) {
        bits = 8 * (int)sizeof(T);
        flags = f;
    }
    vxo::Tree<T> *tree(uint32_t t) {
        if (t >= trees.size() || !trees[t]) throw std::invalid_argument("unknown tree handle");
        return trees[t].get();
    }
};

int fail(OInternerBase *o, int code, const char *msg) {
    if (o) o->last_error = msg;
    return code;
}

template <class F>
int guard(OInternerBase *o, F f) {
    try {
        return f();
    } catch (const vxo::RefOOM &e) {
        return fail(o, VX_E_OOM, e.what());
    } catch (const vxo::RefOOB &e) {
        return fail(o, VX_E_OOB, e.what());
    } catch (const vxo::RefUB &e) {
        return fail(o, VX_E_REF_UB, e.what());
    } catch (const vxo::RefPanic &e) {
        std::string m = e.what();
        return fail(o, m.find("Max depth") != std::string::npos ? VX_E_DEPTH : VX_E_REF_PANIC, e.what());
    } catch (const std::invalid_argument &e) {
        return fail(o, VX_E_INVALID_ARG, e.what());
    } catch (const std::bad_alloc &) {
        return fail(o, VX_E_OOM, "host allocation failed");
    } catch (const std::exception &e) {
        return fail(o, VX_E_REF_PANIC, e.what());
    }
}

// Dispatch on the voxel width of an interner.
template <class F>
int with_interner(void *h, F f) {
    auto *base = static_cast<OInternerBase *>(h);
    if (!base) return VX_E_INVALID_ARG;
    return guard(base, [&]() -> int {
        if (base->bits == 8) return f(*static_cast<OInterner<uint8_t> *>(base));
        return f(*static_cast<OInterner<uint16_t> *>(base));
    });
}

template <class T>
bool fits(uint32_t v) {
    return v <= (uint32_t)(T)~T(0);
}

// Canonical pre-order export (the format is documented at vx_canonical in voxelis_gb300.h).
template <class T>
int export_canonical(OInterner<T> &o, uint32_t n_trees, const uint32_t *trees, vx_canonical *out,
                     uint64_t *n_nodes) {
    auto &it = o.it;
    std::unordered_map<uint32_t, int32_t> ids;
    std::vector<uint64_t> order;
    std::vector<int32_t> roots(n_trees, -1);
    std::vector<uint64_t> stack;
    for (uint32_t t = 0; t < n_trees; ++t) {
        uint64_t r = o.tree(trees[t])->root();
        if (vxo::bid::is_empty(r)) continue;
        stack.push_back(r);
        while (!stack.empty()) {
            uint64_t n = stack.back();
            stack.pop_back();
            uint32_t idx = vxo::bid::index(n);
            if (ids.count(idx)) continue;
            ids[idx] = (int32_t)order.size();
            order.push_back(n);
            if (vxo::bid::is_branch(n)) {
                const auto &ch = it.get_children(n);
                for (int s = 7; s >= 0; --s)
                    if (!vxo::bid::is_empty(ch[s])) stack.push_back(ch[s]);
            }
        }
        roots[t] = ids[vxo::bid::index(r)];
    }
    *n_nodes = order.size();
    if (!out) return VX_OK;
    if (out->capacity < order.size()) return VX_E_BUFFER;
    for (size_t k = 0; k < order.size(); ++k) {
        uint64_t n = order[k];
        bool leaf = vxo::bid::is_leaf(n);
        out->kind[k] = leaf ? 1 : 0;
        out->types[k] = leaf ? 0 : (uint8_t)((n >> 55) & 0xFF);
        out->mask[k] = leaf ? 0 : (uint8_t)((n >> 47) & 0xFF);
        out->value[k] = (uint32_t)it.get_value(n);
        out->refcount[k] = it.slot_refcount(vxo::bid::index(n));
        for (int s = 0; s < 8; ++s) {
            int32_t c = -1;
            if (!leaf) {
                uint64_t cid = it.get_children(n)[s];
                if (!vxo::bid::is_empty(cid)) c = ids[vxo::bid::index(cid)];
            }
            out->children[k * 8 + s] = c;
        }
    }
    if (out->roots)
        for (uint32_t t = 0; t < n_trees; ++t) out->roots[t] = roots[t];
    return VX_OK;
}

template <class F>
int with_batch(void *h, F f) {
    auto *base = static_cast<OBatchBase *>(h);
    if (!base) return VX_E_INVALID_ARG;
    try {
        if (base->bits == 8) return f(static_cast<OBatch<uint8_t> *>(base)->b);
        return f(static_cast<OBatch<uint16_t> *>(base)->b);
    } catch (const vxo::RefOOB &) {
        return VX_E_OOB;
    } catch (const std::exception &) {
        return VX_E_REF_PANIC;
    }
}

}  // namespace

// Big-endian reader of a serialised model (the reference reads through byteorder / BufReader).
namespace {
struct Reader {
    const uint8_t *b;
    uint64_t n, p = 0;
    void need(uint64_t k) const {
        if (p + k > n) throw vxo::RefPanic("unexpected end of the stream");
    }
    uint8_t u8() {
        need(1);
        return b[p++];
    }
    uint32_t u32() {
        need(4);
        uint32_t v = ((uint32_t)b[p] << 24) | ((uint32_t)b[p + 1] << 16) | ((uint32_t)b[p + 2] << 8) | b[p + 3];
        p += 4;
        return v;
    }
    // decode_varint_u32_from_reader (io/varint.rs:47-69)
    uint32_t varint() {
        uint32_t r = 0;
        for (int shift = 0;; shift += 7) {
            const uint8_t c = u8();
            r |= (uint32_t)(c & 0x7F) << shift;
            if (c < 0x80) return r;
            if (shift + 7 >= 32) throw vxo::RefPanic("varint longer than 5 bytes");
        }
    }
    template <class T>
    T value() {
        uint32_t v = 0;
        for (size_t k = 0; k < sizeof(T); ++k) v = (v << 8) | u8();
        return (T)v;
    }
};
}  // namespace

extern "C" {

int vxo_interner_create(uint64_t budget, int bits, uint32_t flags, int table_log2, void **out) {
    (void)table_log2;
    if (!out || (bits != 8 && bits != 16)) return VX_E_INVALID_ARG;
    try {
        if (bits == 8)
            *out = new OInterner<uint8_t>(budget, flags);
        else
            *out = new OInterner<uint16_t>(budget, flags);
    } catch (const vxo::RefPanic &) {
        return VX_E_REF_PANIC;
    } catch (const std::bad_alloc &) {
        return VX_E_OOM;
    }
    return VX_OK;
}

int vxo_interner_destroy(void *h) {
    delete static_cast<OInternerBase *>(h);
    return VX_OK;
}

const char *vxo_last_error(void *h) {
    auto *o = static_cast<OInternerBase *>(h);
    return o ? o->last_error.c_str() : "null interner";
}

int vxo_interner_stats_get(void *h, vx_interner_stats *s) {
    return with_interner(h, [&](auto &o) {
        *s = vx_interner_stats{};
        s->capacity = o.it.capacity();
        s->node_size = o.it.node_size();
        s->next_index = o.it.next_index();
        s->free_count = o.it.free_count();
        s->alive_nodes = s->next_index - s->free_count;
        s->branch_patterns = o.it.branch_patterns();
        s->leaf_patterns = o.it.leaf_patterns();
        s->nodes_created = o.it.created();
        return VX_OK;
    });
}

int vxo_collisions(void *h, uint64_t *out) {
    return with_interner(h, [&](auto &o) {
        *out = o.it.collisions;
        return VX_OK;
    });
}

int vxo_get_ref(void *h, uint64_t id, uint32_t *out) {
    return with_interner(h, [&](auto &o) {
        if (!o.it.is_valid_block_id(id)) return VX_E_INVALID_ARG;
        *out = o.it.get_ref(id);
        return VX_OK;
    });
}

int vxo_get_value(void *h, uint64_t id, uint32_t *out) {
    return with_interner(h, [&](auto &o) {
        if (!o.it.is_valid_block_id(id)) return VX_E_INVALID_ARG;
        *out = (uint32_t)o.it.get_value(id);
        return VX_OK;
    });
}

int vxo_tree_create(void *h, int depth, uint32_t *out) {
    return with_interner(h, [&](auto &o) {
        using TreeT = std::remove_reference_t<decltype(*o.trees[0])>;
        auto t = std::make_unique<TreeT>(depth, o.flags);
        uint32_t slot;
        if (!o.free_slots.empty()) {
            slot = o.free_slots.back();
            o.free_slots.pop_back();
            o.trees[slot] = std::move(t);
        } else {
            slot = (uint32_t)o.trees.size();
            o.trees.push_back(std::move(t));
        }
        *out = slot;
        return VX_OK;
    });
}

int vxo_tree_destroy(void *h, uint32_t tree) {
    return with_interner(h, [&](auto &o) {
        o.tree(tree)->clear(o.it);
        o.trees[tree].reset();
        o.free_slots.push_back(tree);
        return VX_OK;
    });
}

int vxo_tree_root(void *h, uint32_t tree, uint64_t *out) {
    return with_interner(h, [&](auto &o) {
        *out = o.tree(tree)->root();
        return VX_OK;
    });
}

int vxo_tree_max_depth(void *h, uint32_t tree, int *out) {
    return with_interner(h, [&](auto &o) {
        *out = o.tree(tree)->max_depth();
        return VX_OK;
    });
}

int vxo_tree_get(void *h, uint32_t tree, int32_t x, int32_t y, int32_t z, int *found, uint32_t *value) {
    return with_interner(h, [&](auto &o) {
        using T = std::decay_t<decltype(o.it.get_value(0))>;
        T v{};
        bool f = o.tree(tree)->get(o.it, x, y, z, &v);
        *found = f ? 1 : 0;
        *value = f ? (uint32_t)v : 0u;
        return VX_OK;
    });
}

int vxo_tree_set(void *h, uint32_t tree, int32_t x, int32_t y, int32_t z, uint32_t value, int *changed) {
    return with_interner(h, [&](auto &o) {
        using T = std::decay_t<decltype(o.it.get_value(0))>;
        if (!fits<T>(value)) return VX_E_INVALID_ARG;
        bool c = o.tree(tree)->set(o.it, x, y, z, (T)value);
        if (changed) *changed = c ? 1 : 0;
        return VX_OK;
    });
}

int vxo_tree_fill(void *h, uint32_t tree, uint32_t value) {
    return with_interner(h, [&](auto &o) {
        using T = std::decay_t<decltype(o.it.get_value(0))>;
        if (!fits<T>(value)) return VX_E_INVALID_ARG;
        o.tree(tree)->fill(o.it, (T)value);
        return VX_OK;
    });
}

int vxo_tree_clear(void *h, uint32_t tree) {
    return with_interner(h, [&](auto &o) {
        o.tree(tree)->clear(o.it);
        return VX_OK;
    });
}

// ---- batches --------------------------------------------------------------------------------
int vxo_batch_create(int depth, int bits, uint32_t flags, void **out) {
    if (!out || (bits != 8 && bits != 16)) return VX_E_INVALID_ARG;
    try {
        if (bits == 8)
            *out = new OBatch<uint8_t>(depth, flags);
        else
            *out = new OBatch<uint16_t>(depth, flags);
    } catch (const vxo::RefPanic &) {
        return VX_E_DEPTH;
    } catch (const std::bad_alloc &) {
        return VX_E_OOM;
    }
    return VX_OK;
}

int vxo_batch_destroy(void *b) {
    delete static_cast<OBatchBase *>(b);
    return VX_OK;
}

int vxo_batch_set(void *b, int32_t x, int32_t y, int32_t z, uint32_t value) {
    return with_batch(b, [&](auto &bb) {
        using T = std::decay_t<decltype(bb.fill_value())>;
        if (!fits<T>(value)) return VX_E_INVALID_ARG;
        bb.just_set(x, y, z, (T)value);
        return VX_OK;
    });
}

int vxo_batch_set_many(void *b, uint64_t n, const int32_t *xyz, const uint32_t *values) {
    return with_batch(b, [&](auto &bb) {
        using T = std::decay_t<decltype(bb.fill_value())>;
        for (uint64_t i = 0; i < n; ++i) {
            if (!fits<T>(values[i])) return VX_E_INVALID_ARG;
            bb.just_set(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], (T)values[i]);
        }
        return VX_OK;
    });
}

int vxo_batch_fill(void *b, uint32_t value) {
    return with_batch(b, [&](auto &bb) {
        using T = std::decay_t<decltype(bb.fill_value())>;
        if (!fits<T>(value)) return VX_E_INVALID_ARG;
        bb.just_fill((T)value);
        return VX_OK;
    });
}

int vxo_batch_clear(void *b) {
    return with_batch(b, [&](auto &bb) {
        bb.just_clear();
        return VX_OK;
    });
}

// just_set over a dense [y][z][x] grid, in the reference's y, z, x loop order.
int vxo_batch_set_dense(void *b, const void *grid) {
    return with_batch(b, [&](auto &bb) {
        using T = std::decay_t<decltype(bb.fill_value())>;
        const T *g = static_cast<const T *>(grid);
        const int32_t n = 1 << bb.max_depth();
        for (int32_t y = 0; y < n; ++y)
            for (int32_t z = 0; z < n; ++z)
                for (int32_t x = 0; x < n; ++x) bb.just_set(x, y, z, g[((size_t)y * n + z) * n + x]);
        return VX_OK;
    });
}

int vxo_batch_size(void *b, uint64_t *out) {
    return with_batch(b, [&](auto &bb) {
        *out = bb.size();
        return VX_OK;
    });
}

int vxo_batch_has_patches(void *b, int *out) {
    return with_batch(b, [&](auto &bb) {
        *out = bb.has_patches() ? 1 : 0;
        return VX_OK;
    });
}

// ---- the path -------------------------------------------------------------------------------
int vxo_apply_batch(void *h, uint32_t tree, void *batch, int *changed) {
    auto *bb = static_cast<OBatchBase *>(batch);
    auto *ib = static_cast<OInternerBase *>(h);
    if (!bb || !ib || bb->bits != ib->bits) return VX_E_INVALID_ARG;
    return with_interner(h, [&](auto &o) {
        using T = std::decay_t<decltype(o.it.get_value(0))>;
        auto &b = static_cast<OBatch<T> *>(bb)->b;
        bool c = o.tree(tree)->apply_batch(o.it, b);
        if (changed) *changed = c ? 1 : 0;
        return VX_OK;
    });
}

int vxo_apply_batches(void *h, uint32_t n, const uint32_t *trees, void *const *batches, uint8_t *changed) {
    for (uint32_t i = 0; i < n; ++i) {
        int c = 0;
        int st = vxo_apply_batch(h, trees[i], batches[i], &c);
        if (st != VX_OK) return st;
        if (changed) changed[i] = (uint8_t)c;
    }
    return VX_OK;
}

// Dense-chunk construction as the reference does it: a Batch filled by just_set from the grid,
// then apply_batch, one chunk after another into the shared interner (voxelis-voxelize
// src/lib.rs:357-361 applies its per-chunk batches the same way).
int vxo_build_dense(void *h, uint32_t n, const uint32_t *trees, const void *grids, uint8_t *changed, int mem) {
    if (mem != VX_MEM_HOST) return VX_E_INVALID_ARG;
    return with_interner(h, [&](auto &o) {
        using T = std::decay_t<decltype(o.it.get_value(0))>;
        if (n == 0) return VX_OK;
        const int d = o.tree(trees[0])->max_depth();
        const size_t per = (size_t)1 << (3 * d);
        vxo::Batch<T> b(d, o.flags);
        const T *g = static_cast<const T *>(grids);
        const int32_t side = 1 << d;
        for (uint32_t i = 0; i < n; ++i) {
            auto *t = o.tree(trees[i]);
            if (t->max_depth() != d) return VX_E_INVALID_ARG;
            b.just_clear();
            const T *grid = g + per * i;
            for (int32_t y = 0; y < side; ++y)
                for (int32_t z = 0; z < side; ++z)
                    for (int32_t x = 0; x < side; ++x)
                        b.just_set(x, y, z, grid[((size_t)y * side + z) * side + x]);
            bool c = t->apply_batch(o.it, b);
            if (changed) changed[i] = c ? 1 : 0;
        }
        return VX_OK;
    });
}

int vxo_get_many(void *h, uint64_t n, const uint32_t *trees, const int32_t *xyz, uint8_t *found, void *values, int mem) {
    if (mem != VX_MEM_HOST) return VX_E_INVALID_ARG;
    return with_interner(h, [&](auto &o) {
        using T = std::decay_t<decltype(o.it.get_value(0))>;
        T *vals = static_cast<T *>(values);
        int status = VX_OK;
        for (uint64_t q = 0; q < n; ++q) {
            T v{};
            bool f = false;
            try {
                f = o.tree(trees[q])->get(o.it, xyz[3 * q], xyz[3 * q + 1], xyz[3 * q + 2], &v);
            } catch (const vxo::RefOOB &) {
                status = VX_E_OOB;
            }
            found[q] = f ? 1 : 0;
            vals[q] = f ? v : T(0);
        }
        return status;
    });
}

int vxo_export_canonical(void *h, uint32_t n_trees, const uint32_t *trees, vx_canonical *out, uint64_t *n_nodes) {
    return with_interner(h, [&](auto &o) { return export_canonical(o, n_trees, trees, out, n_nodes); });
}

int vxo_tree_to_dense(void *h, uint32_t tree, void *out) {
    return with_interner(h, [&](auto &o) {
        using T = std::decay_t<decltype(o.it.get_value(0))>;
        o.tree(tree)->to_vec(o.it, static_cast<T *>(out));
        return VX_OK;
    });
}

int vxo_occupancy_masks(void *h, uint32_t n_trees, const uint32_t *trees, const uint32_t *offsets, uint64_t *global,
                        uint64_t *active, uint32_t max_materials, uint32_t *n_materials, uint32_t *material_ids,
                        uint64_t *material_counts, uint64_t *material_masks) {
    return with_interner(h, [&](auto &o) {
        if (!n_trees || !trees || !offsets || !global || !active || !n_materials) return VX_E_INVALID_ARG;
        vxo::Occupancy b;
        for (uint32_t k = 0; k < n_trees; ++k) {
            auto *t = o.tree(trees[k]);
            const uint32_t side = 1u << t->max_depth();
            for (int a = 0; a < 3; ++a)
                if (offsets[3 * k + a] + side > 64) return fail(&o, VX_E_OOB, "tree outside the 64^3 builder");
            t->occupancy_masks(o.it, b, offsets[3 * k], offsets[3 * k + 1], offsets[3 * k + 2]);
        }
        std::copy(b.global.begin(), b.global.end(), global);
        std::copy(b.active, b.active + 6, active);
        *n_materials = (uint32_t)b.materials.size();
        uint32_t k = 0;
        for (auto &kv : b.materials) {
            if (k >= max_materials) break;
            material_ids[k] = kv.first;
            material_counts[k] = kv.second;
            const auto &pm = b.per_material[kv.first];
            std::copy(pm.begin(), pm.end(), material_masks + (size_t)k * vxo::Occupancy::kAll);
            ++k;
        }
        return b.materials.size() > max_materials ? fail(&o, VX_E_BUFFER, "more materials than max_materials")
                                                  : VX_OK;
    });
}

// VoxModel::serialize (world/voxmodel.rs:177-282) with serialize_chunk (world/voxchunk.rs:382-405)
// for the given chunks, in the given order; varints as io/varint.rs:5-30.
static void put_varint(std::vector<uint8_t> &o, uint32_t v) {
    while (v >= 0x80) {
        o.push_back((uint8_t)((v & 0x7F) | 0x80));
        v >>= 7;
    }
    o.push_back((uint8_t)v);
}
static void put_u32(std::vector<uint8_t> &o, uint32_t v) {
    for (int s = 24; s >= 0; s -= 8) o.push_back((uint8_t)(v >> s));
}

int vxo_serialize_model(void *h, uint32_t n_chunks, const uint32_t *trees, const int32_t *positions, uint8_t *out,
                        uint64_t capacity, uint64_t *size) {
    return with_interner(h, [&](auto &o) {
        using T = std::decay_t<decltype(o.it.get_value(0))>;
        if (!size || (n_chunks && (!trees || !positions))) return VX_E_INVALID_ARG;
        std::vector<uint64_t> leaves, branches;
        o.it.for_each_pattern(1, [&](uint64_t id) { leaves.push_back(id); });
        o.it.for_each_pattern(0, [&](uint64_t id) { branches.push_back(id); });
        auto by_index = [](uint64_t a, uint64_t b) { return vxo::bid::index(a) < vxo::bid::index(b); };
        std::sort(leaves.begin(), leaves.end(), by_index);
        std::sort(branches.begin(), branches.end(), by_index);
        std::unordered_map<uint32_t, uint32_t> id_map;
        id_map[0] = 0;
        uint32_t next = 1;
        for (uint64_t id : leaves) id_map[vxo::bid::index(id)] = next++;
        for (uint64_t id : branches)
            if (vxo::bid::index(id) != 0) id_map[vxo::bid::index(id)] = next++;
        std::vector<uint8_t> b;
        auto put_value = [&](T v) {
            for (int s = 8 * ((int)sizeof(T) - 1); s >= 0; s -= 8) b.push_back((uint8_t)((uint32_t)v >> s));
        };
        put_u32(b, (uint32_t)leaves.size());
        for (uint64_t id : leaves) {
            put_varint(b, id_map.at(vxo::bid::index(id)));
            put_value(o.it.get_value(id));
        }
        put_u32(b, (uint32_t)branches.size() - 1);
        for (uint64_t id : branches) {
            if (vxo::bid::index(id) == 0) continue;
            put_varint(b, id_map.at(vxo::bid::index(id)));
            b.push_back((uint8_t)vxo::bid::mask(id));
            for (uint64_t c : o.it.get_children(id))
                if (!vxo::bid::is_empty(c)) put_varint(b, id_map.at(vxo::bid::index(c)));
            put_value(o.it.get_value(id));
        }
        put_u32(b, n_chunks);
        static const char magic[12] = {'V', 'o', 'x', 'T', 'r', 'e', 'e', 'C', 'h', 'u', 'n', 'k'};
        for (uint32_t k = 0; k < n_chunks; ++k) {
            b.insert(b.end(), magic, magic + 12);
            for (int a = 0; a < 3; ++a) put_u32(b, (uint32_t)positions[3 * k + a]);
            put_varint(b, id_map.at(vxo::bid::index(o.tree(trees[k])->root())));
        }
        *size = b.size();
        if (!out) return VX_OK;
        if (capacity < b.size()) return fail(&o, VX_E_BUFFER, "output buffer smaller than the serialised model");
        std::copy(b.begin(), b.end(), out);
        return VX_OK;
    });
}

// VoxModel::deserialize (world/voxmodel.rs:284-408) and deserialize_chunk (world/voxchunk.rs:408-440):
// reads records in stream order with the reference's checks (every read past the end is an unwrap
// panic). Before anything is interned, one read-only walk of the same layout finds the chunk count,
// so that VX_E_BUFFER leaves the interner unchanged, as the C ABI promises.

int vxo_deserialize_model(void *h, const uint8_t *data, uint64_t n_bytes, int max_depth, uint32_t max_chunks,
                          uint32_t *out_trees, int32_t *out_positions, uint32_t *out_n_chunks) {
    return with_interner(h, [&](auto &o) {
        using T = std::decay_t<decltype(o.it.get_value(0))>;
        using TreeT = std::remove_reference_t<decltype(*o.trees[0])>;
        if (!out_n_chunks || (n_bytes && !data)) return VX_E_INVALID_ARG;
        *out_n_chunks = 0;
        TreeT probe(max_depth, o.flags);  // MaxDepth::new (max_depth.rs:77-83)
        (void)probe;
        {  // the layout walk
            Reader r{data, n_bytes};
            for (uint32_t k = 0, L = r.u32(); k < L; ++k) {
                r.varint();
                r.template value<T>();
            }
            for (uint32_t k = 0, B = r.u32(); k < B; ++k) {
                r.varint();
                const uint8_t mask = r.u8();
                for (int j = 0; j < 8; ++j)
                    if (mask >> j & 1) r.varint();
                r.template value<T>();
            }
            const uint32_t C = r.u32();
            *out_n_chunks = C;
            if (C > max_chunks) return fail(&o, VX_E_BUFFER, "more chunks in the stream than max_chunks");
            if (C && (!out_trees || !out_positions)) return VX_E_INVALID_ARG;
        }
        Reader r{data, n_bytes};
        const uint32_t L = r.u32();
        std::unordered_map<uint32_t, uint64_t> leaf_patterns;
        for (uint32_t k = 0; k < L; ++k) {
            const uint32_t id = r.varint();
            const T value = r.template value<T>();
            leaf_patterns[id] = o.it.deserialize_leaf(id, value);
        }
        struct Pattern {
            uint64_t id;
            uint32_t children[8];
            T lod;
        };
        const uint32_t B = r.u32();
        std::unordered_map<uint32_t, Pattern> branch_patterns;
        branch_patterns[0] = Pattern{vxo::bid::EMPTY, {}, T(0)};
        std::vector<uint32_t> order;
        for (uint32_t k = 0; k < B; ++k) {
            const uint32_t id = r.varint();
            if (id == 0) throw vxo::RefPanic("assert_ne!(id, 0)");
            const uint8_t mask = r.u8();
            uint8_t types = 0;
            Pattern p{0, {}, T(0)};
            for (int j = 0; j < 8; ++j) {
                if (!(mask >> j & 1)) continue;
                p.children[j] = r.varint();
                if (leaf_patterns.count(p.children[j])) types |= (uint8_t)(1u << j);
            }
            p.lod = r.template value<T>();
            p.id = o.it.preallocate_branch_id(id, types, mask);
            branch_patterns[id] = p;
            order.push_back(id);
            if (mask == 0) throw vxo::RefPanic("assert_ne!(mask, 0)");
        }
        for (uint32_t id : order) {  // the reference walks its map; the result does not depend on the order
            const Pattern &p = branch_patterns.at(id);
            const uint8_t types = (uint8_t)vxo::bid::types(p.id), mask = (uint8_t)vxo::bid::mask(p.id);
            vxo::Children c{};
            for (int j = 0; j < 8; ++j) {
                if (!(mask >> j & 1)) continue;
                auto leaf = leaf_patterns.find(p.children[j]);
                if (types >> j & 1) {
                    c[j] = leaf->second;
                } else {
                    auto br = branch_patterns.find(p.children[j]);
                    if (br == branch_patterns.end()) throw vxo::RefPanic("child id names no pattern");
                    c[j] = br->second.id;
                }
            }
            o.it.deserialize_branch(p.id, c, types, mask, p.lod);
        }
        const uint32_t C = r.u32();
        static const char magic[12] = {'V', 'o', 'x', 'T', 'r', 'e', 'e', 'C', 'h', 'u', 'n', 'k'};
        for (uint32_t k = 0; k < C; ++k) {
            for (int j = 0; j < 12; ++j)
                if (r.u8() != (uint8_t)magic[j]) throw vxo::RefPanic("assert_eq!(magic, VTC_MAGIC)");
            for (int a = 0; a < 3; ++a) out_positions[3 * k + a] = (int32_t)r.u32();
            const uint32_t root = r.varint();
            uint64_t block;
            auto br = branch_patterns.find(root);
            if (br != branch_patterns.end()) {
                block = br->second.id;
            } else {
                auto leaf = leaf_patterns.find(root);
                if (leaf == leaf_patterns.end()) throw vxo::RefPanic("root id names no pattern");
                block = leaf->second;
            }
            uint32_t slot;
            if (int st = vxo_tree_create(&o, max_depth, &slot)) return st;
            o.tree(slot)->set_root_id(o.it, block);
            out_trees[k] = slot;
        }
        return VX_OK;
    });
}

// The UB fence: every child reachable from the trees has a matching generation and a positive
// refcount.
int vxo_validate(void *h, uint32_t n, const uint32_t *trees) {
    return with_interner(h, [&](auto &o) {
        std::vector<uint64_t> stack;
        std::unordered_map<uint32_t, bool> seen;
        for (uint32_t t = 0; t < n; ++t) {
            uint64_t r = o.tree(trees[t])->root();
            if (vxo::bid::is_empty(r)) continue;
            stack.push_back(r);
            while (!stack.empty()) {
                uint64_t id = stack.back();
                stack.pop_back();
                uint32_t i = vxo::bid::index(id);
                if (i >= o.it.capacity()) return fail(&o, VX_E_REF_UB, "child index outside the pool");
                if (o.it.slot_generation(i) != vxo::bid::generation(id))
                    return fail(&o, VX_E_REF_UB, "dangling child: generation mismatch");
                if (o.it.slot_refcount(i) == 0) return fail(&o, VX_E_REF_UB, "reachable node with zero refcount");
                if (seen[i]) continue;
                seen[i] = true;
                if (vxo::bid::is_branch(id))
                    for (uint64_t c : o.it.get_children(id))
                        if (!vxo::bid::is_empty(c)) stack.push_back(c);
            }
        }
        return VX_OK;
    });
}

// Wall-clock helper for the CPU baseline: builds n dense chunks and returns the elapsed seconds.
int vxo_time_build_dense(void *h, uint32_t n, const uint32_t *trees, const void *grids, double *seconds) {
    auto t0 = std::chrono::steady_clock::now();
    int st = vxo_build_dense(h, n, trees, grids, nullptr, VX_MEM_HOST);
    auto t1 = std::chrono::steady_clock::now();
    *seconds = std::chrono::duration<double>(t1 - t0).count();
    return st;
}

// The reference's many-chunks pattern on all host threads (voxelis-voxelize src/lib.rs:284-361):
// per-chunk Batches are filled in parallel, then applied one after another to the shared interner
// (apply_batch needs &mut VoxInterner). Returns the seconds of both phases.
int vxo_build_dense_mt(void *h, uint32_t n, const uint32_t *trees, const void *grids, int threads,
                       double *fill_seconds, double *apply_seconds) {
    return with_interner(h, [&](auto &o) {
        using T = std::decay_t<decltype(o.it.get_value(0))>;
        if (n == 0) return VX_OK;
        const int d = o.tree(trees[0])->max_depth();
        const size_t per = (size_t)1 << (3 * d);
        const int32_t side = 1 << d;
        const T *g = static_cast<const T *>(grids);
        std::vector<std::unique_ptr<vxo::Batch<T>>> batches(n);
        auto t0 = std::chrono::steady_clock::now();
        std::atomic<uint32_t> next{0};
        std::atomic<int> failed{0};
        auto worker = [&]() {
            for (;;) {
                uint32_t i = next.fetch_add(1);
                if (i >= n) break;
                try {
                    auto b = std::make_unique<vxo::Batch<T>>(d, o.flags);
                    const T *grid = g + per * i;
                    for (int32_t y = 0; y < side; ++y)
                        for (int32_t z = 0; z < side; ++z)
                            for (int32_t x = 0; x < side; ++x)
                                b->just_set(x, y, z, grid[((size_t)y * side + z) * side + x]);
                    batches[i] = std::move(b);
                } catch (...) {
                    failed = 1;
                }
            }
        };
        std::vector<std::thread> pool;
        for (int k = 0; k < std::max(1, threads); ++k) pool.emplace_back(worker);
        for (auto &t : pool) t.join();
        if (failed) return VX_E_REF_PANIC;
        auto t1 = std::chrono::steady_clock::now();
        for (uint32_t i = 0; i < n; ++i) o.tree(trees[i])->apply_batch(o.it, *batches[i]);
        auto t2 = std::chrono::steady_clock::now();
        *fill_seconds = std::chrono::duration<double>(t1 - t0).count();
        *apply_seconds = std::chrono::duration<double>(t2 - t1).count();
        return VX_OK;
    });
}

}  // extern "C"
