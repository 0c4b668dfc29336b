// CPU restatement of voxelis' batched SVO-DAG edit-and-intern path — TEST INFRASTRUCTURE ONLY.
//
// This is the oracle: a line-by-line C++ restatement of the reference's Rust code for the path
// (the reference is Rust and no Rust toolchain exists here, so it cannot be compiled or linked).
// Only the tests, the smoke check and bench.py's CPU-baseline leg may use it, as the checker or as
// the timed CPU baseline. The GPU library never calls it.
//
// Each function cites the reference file:line it restates (paths relative to the voxelis repo).
// Parity pins: the reference's own unit tests for this path (voxtree.rs:1128-2202,
// block_id.rs:475-609, max_depth.rs:157-230) are re-run against this restatement by
// tests/test_oracle_pins.py, together with known answers derived by reading the code.
//
// Behaviour notes
//   * Reference panics (assert!, BlockId::types() on a leaf, out of memory) throw RefPanic /
//     RefOOM. Reference undefined behaviour in release builds (refcount underflow, release
//     stack overflow, dangling children) throws RefUB. The C ABI maps both to status codes.
//   * Hash values are rustc-hash 2.1.1 FxHasher (Cargo.lock:4456-4457) restated from its published
//     algorithm; dedup is by the 64-bit hash as in the reference (interner/mod.rs:636, 728). With
//     check_keys on, a hash hit whose stored key differs is counted as a collision (the reference
//     would alias the two nodes; debug builds assert at interner/mod.rs:744-765).
//   * Patches P1..P4 (behaviour switches, default off) are defined in include/voxelis_gb300.h.
#pragma once

#include <array>
#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <string>
#include <map>
#include <vector>

namespace vxo {

struct RefPanic : std::runtime_error {
    using std::runtime_error::runtime_error;
};
struct RefOOM : std::runtime_error {
    using std::runtime_error::runtime_error;
};
struct RefUB : std::runtime_error {
    using std::runtime_error::runtime_error;
};
struct RefOOB : std::runtime_error {
    using std::runtime_error::runtime_error;
};

enum : uint32_t { P1 = 1u << 0, P2 = 1u << 1, P3 = 1u << 2, P4 = 1u << 3, P5 = 1u << 4 };

using Children = std::array<uint64_t, 8>;

// ---- BlockId (core/block_id.rs:19-418) ----------------------------------------------------------
namespace bid {
constexpr uint64_t INVALID = ~0ull;  // block_id.rs:120
constexpr uint64_t EMPTY = 0ull;     // block_id.rs:123
constexpr uint16_t MAX_GENERATION = 0x7FFE;

// new_extended (block_id.rs:216-226)
inline uint64_t make(uint32_t index, uint16_t generation, uint8_t types, uint8_t mask, bool leaf) {
    if (generation > MAX_GENERATION) throw RefPanic("Generation overflow");
    return ((uint64_t)leaf << 63) | ((uint64_t)types << 55) | ((uint64_t)mask << 47) |
           ((uint64_t)(generation & 0x7FFF) << 32) | (uint64_t)index;
}
inline uint64_t new_leaf(uint32_t index, uint16_t generation) {
    return make(index, generation, 0, 0, true);
}
inline uint64_t new_branch(uint32_t index, uint16_t generation, uint8_t types, uint8_t mask) {
    return make(index, generation, types, mask, false);
}
inline uint32_t index(uint64_t id) { return (uint32_t)(id & 0xFFFFFFFFull); }
inline uint16_t generation(uint64_t id) { return (uint16_t)((id >> 32) & 0x7FFF); }
inline bool is_leaf(uint64_t id) { return (id >> 63) == 1; }
inline bool is_branch(uint64_t id) { return (id >> 63) == 0; }
inline bool is_empty(uint64_t id) { return id == 0; }
// types()/mask()/has_child() assert is_branch (block_id.rs:273-276, 294-297, 316-321)
inline uint8_t types(uint64_t id) {
    if (!is_branch(id)) throw RefPanic("Cannot get types from a leaf node");
    return (uint8_t)((id >> 55) & 0xFF);
}
inline uint8_t mask(uint64_t id) {
    if (!is_branch(id)) throw RefPanic("Cannot get mask from a leaf node");
    return (uint8_t)((id >> 47) & 0xFF);
}
inline bool has_child(uint64_t id, unsigned child) {
    if (!is_branch(id)) throw RefPanic("Cannot check child on a leaf node");
    if (child >= 8) throw RefPanic("Child index out of bounds (0-7)");
    return ((mask(id) >> child) & 1) != 0;
}
}  // namespace bid

// ---- depth caps (interner/consts.rs:5, core/max_depth.rs:77-83) ---------------------------------
constexpr int MAX_ALLOWED_DEPTH = 7;
constexpr int MAX_PATCHED_DEPTH = 11;  // P2: depths 0..10 (u32 Morton paths, common.rs:25-31)
constexpr size_t PREALLOCATED_STACK_SIZE = 32768;  // consts.rs:15

inline int depth_limit(uint32_t flags) { return (flags & P2) ? MAX_PATCHED_DEPTH : MAX_ALLOWED_DEPTH; }

// PATH_MASKS[max_depth][k] (voxtree.rs:41-105) in closed form; equal to the table for depths
// 0..6 and extended to 10 under P2.
inline uint32_t path_mask(int max_depth, int k) {
    if (max_depth <= 0 || k > max_depth - 1) return 0;
    return ((1u << (3 * (k + 1))) - 1u) << (3 * (max_depth - 1 - k));
}

// encode_child_index_path (utils/common.rs:24-55): x at bits 3n, y at 3n+1, z at 3n+2.
inline uint32_t encode_child_index_path(int32_t px, int32_t py, int32_t pz) {
    const uint32_t M10 = 0x3FF, M1 = 0x30000FF, M2 = 0x300F00F, M3 = 0x30C30C3, M4 = 0x9249249;
    auto split = [&](uint32_t v) {
        v &= M10;
        v = (v | (v << 16)) & M1;
        v = (v | (v << 8)) & M2;
        v = (v | (v << 4)) & M3;
        v = (v | (v << 2)) & M4;
        return v;
    };
    return split((uint32_t)px) | (split((uint32_t)py) << 1) | (split((uint32_t)pz) << 2);
}

// child_index_macro_2 (utils/common.rs:104-111)
inline unsigned child_index(int32_t x, int32_t y, int32_t z, int current, int max) {
    int shift = max - current - 1;
    return (((uint32_t)x >> shift) & 1) | ((((uint32_t)y >> shift) & 1) << 1) |
           ((((uint32_t)z >> shift) & 1) << 2);
}

// ---- rustc-hash 2.1.1 FxHasher, 64-bit (restated from its published algorithm) ------------------
struct FxHasher {
    static constexpr uint64_t K = 0xf1357aea2e62a9c5ull;
    uint64_t hash = 0;
    void add(uint64_t i) { hash = (hash + i) * K; }
    void write_u8(uint8_t v) { add(v); }
    void write_u16(uint16_t v) { add(v); }
    void write_u64(uint64_t v) { add(v); }
    uint64_t finish() const { return (hash << 26) | (hash >> 38); }
};

template <class T>
inline void hash_value(FxHasher &h, T v) {
    if (sizeof(T) == 1)
        h.write_u8((uint8_t)v);
    else
        h.write_u16((uint16_t)v);
}

// compute_empty_branch_hash (interner/hash.rs:41-52)
inline uint64_t compute_empty_branch_hash() {
    FxHasher h;
    h.write_u8(1);  // NODE_TYPE_BRANCH
    for (int i = 0; i < 8; ++i) h.write_u8(0);  // CHILD_ABSENT
    return h.finish();
}
// compute_leaf_hash_for_value (interner/hash.rs:54-64)
template <class T>
inline uint64_t compute_leaf_hash(T value) {
    FxHasher h;
    h.write_u8(0);  // NODE_TYPE_LEAF
    hash_value(h, value);
    return h.finish();
}
// compute_branch_hash_for_children (interner/hash.rs:66-81)
inline uint64_t compute_branch_hash(const Children &c, uint8_t types, uint8_t mask) {
    FxHasher h;
    h.write_u8(1);
    h.write_u16((uint16_t)(((uint16_t)types << 8) | mask));
    for (uint64_t id : c) h.write_u64(id);
    return h.finish();
}

// calc_average (core/voxel.rs:96-141): the mode of the 8 child values, ties broken toward a
// non-default value, first-seen order otherwise.
template <class T>
inline T calc_average(const T *children, int n) {
    T values[8] = {};
    int counts[8] = {};
    int unique = 0;
    for (int k = 0; k < n; ++k) {
        T c = children[k];
        int i = 0;
        while (i < unique) {
            if (values[i] == c) {
                counts[i] += 1;
                break;
            }
            ++i;
        }
        if (i == unique) {
            values[unique] = c;
            counts[unique] = 1;
            unique += 1;
        }
    }
    if (unique == 0) return T(0);
    const T def = T(0);
    int max_i = 0, max_cnt = counts[0];
    for (int i = 1; i < unique; ++i) {
        int cnt = counts[i];
        bool is_default_i = values[i] == def;
        bool is_default_max = values[max_i] == def;
        if (cnt > max_cnt || (cnt == max_cnt && is_default_max && !is_default_i)) {
            max_cnt = cnt;
            max_i = i;
        }
    }
    return values[max_i];
}

// ---- the patterns map: HashMap<u64, BlockId> with an identity hasher (interner/hash.rs:15-39) --
// Open addressing with linear probing and backward-shift deletion, grown at load 1/2.
class FlatMap {
   public:
    explicit FlatMap(size_t initial = 16384) { init(pow2(initial * 2)); }
    const uint64_t *find(uint64_t key) const {
        size_t i = slot(key);
        while (used_[i]) {
            if (keys_[i] == key) return &vals_[i];
            i = (i + 1) & mask_;
        }
        return nullptr;
    }
    void insert(uint64_t key, uint64_t val) {
        if ((count_ + 1) * 2 > keys_.size()) grow();
        size_t i = slot(key);
        while (used_[i]) {
            if (keys_[i] == key) {
                vals_[i] = val;
                return;
            }
            i = (i + 1) & mask_;
        }
        used_[i] = 1;
        keys_[i] = key;
        vals_[i] = val;
        ++count_;
    }
    bool erase(uint64_t key) {
        size_t i = slot(key);
        while (used_[i]) {
            if (keys_[i] == key) break;
            i = (i + 1) & mask_;
        }
        if (!used_[i]) return false;
        size_t j = i;
        for (;;) {
            j = (j + 1) & mask_;
            if (!used_[j]) break;
            size_t k = slot(keys_[j]);
            // move j back to i if k is cyclically outside (i, j]
            bool move = (i <= j) ? (k <= i || k > j) : (k <= i && k > j);
            if (move) {
                keys_[i] = keys_[j];
                vals_[i] = vals_[j];
                i = j;
            }
        }
        used_[i] = 0;
        --count_;
        return true;
    }
    size_t size() const { return count_; }
    template <class F>
    void for_each(F f) const {
        for (size_t i = 0; i < keys_.size(); ++i)
            if (used_[i]) f(keys_[i], vals_[i]);
    }

   private:
    static size_t pow2(size_t n) {
        size_t p = 16;
        while (p < n) p <<= 1;
        return p;
    }
    void init(size_t n) {
        keys_.assign(n, 0);
        vals_.assign(n, 0);
        used_.assign(n, 0);
        mask_ = n - 1;
        shift_ = 64;
        for (size_t t = n; t > 1; t >>= 1) --shift_;
        count_ = 0;
    }
    size_t slot(uint64_t key) const { return (size_t)((key * 0x9E3779B97F4A7C15ull) >> shift_) & mask_; }
    void grow() {
        std::vector<uint64_t> k, v;
        std::vector<uint8_t> u;
        k.swap(keys_);
        v.swap(vals_);
        u.swap(used_);
        init(k.size() * 2);
        for (size_t i = 0; i < k.size(); ++i)
            if (u[i]) insert(k[i], v[i]);
    }
    std::vector<uint64_t> keys_, vals_;
    std::vector<uint8_t> used_;
    size_t mask_ = 0, count_ = 0;
    int shift_ = 64;
};

// ---- VoxInterner<T> (interner/mod.rs:25-1166) ---------------------------------------------------
template <class T>
class Interner {
   public:
    static constexpr size_t INITIAL_CAPACITY = 16384;  // mod.rs:43
    static constexpr size_t node_size() { return 4 + 2 + 64 + sizeof(T) + 8; }  // mod.rs:158-164

    // with_memory_budget (mod.rs:45-156)
    Interner(size_t requested_budget, uint32_t flags)
        : patterns_{FlatMap(INITIAL_CAPACITY), FlatMap(INITIAL_CAPACITY)}, flags_(flags) {
        size_t nodes_capacity = requested_budget / node_size();
        if (nodes_capacity == 0) throw RefPanic("Requested budget is too small");
        if (nodes_capacity > 0xFFFFFFFFull) throw RefPanic("Requested budget is too large");
        capacity_ = nodes_capacity;
        ref_counts_.assign(capacity_, 0);
        generations_.assign(capacity_, 0);
        children_.assign(capacity_, Children{});
        values_.assign(capacity_, T(0));
        hashes_.assign(capacity_, 0);
        empty_branch_hash_ = compute_empty_branch_hash();
        empty_branch_id_ = bid::new_branch(0, 0, 0, 0);
        hashes_[0] = empty_branch_hash_;
        patterns_[0].insert(empty_branch_hash_, empty_branch_id_);
        stack_.assign(PREALLOCATED_STACK_SIZE, 0);
        next_index_ = 1;
    }

    uint32_t flags() const { return flags_; }
    size_t capacity() const { return capacity_; }
    uint32_t next_index() const { return next_index_; }
    size_t free_count() const { return free_indices_.size(); }
    // The ids of the interned patterns: kind 0 branches (including EMPTY), 1 leaves (mod.rs:1031-1038).
    template <class F>
    void for_each_pattern(int kind, F f) const {
        patterns_[kind].for_each([&](uint64_t, uint64_t id) { f(id); });
    }
    size_t branch_patterns() const { return patterns_[0].size(); }
    size_t leaf_patterns() const { return patterns_[1].size(); }
    uint64_t collisions = 0;  // hash hits whose stored key differs (reference would alias)
    bool check_keys = true;

    // is_valid_block_id, release variant (mod.rs:1003-1008)
    bool is_valid_block_id(uint64_t id) const {
        uint32_t i = bid::index(id);
        return i < capacity_ && generations_[i] == bid::generation(id);
    }
    void require_valid(uint64_t id) const {
        if (!is_valid_block_id(id)) throw RefUB("stale or invalid block id");
    }
    const T &get_value(uint64_t id) const { return values_[checked(id)]; }  // mod.rs:166-176
    const Children &get_children(uint64_t id) const { return children_[checked(id)]; }  // :178-203
    uint64_t get_child_id(uint64_t id, unsigned i) const { return children_[checked(id)][i]; }  // :205-220
    uint32_t get_ref(uint64_t id) const { return ref_counts_[checked(id)]; }  // :222-233
    uint16_t slot_generation(uint32_t index) const { return generations_[index]; }
    uint32_t slot_refcount(uint32_t index) const { return ref_counts_[index]; }

    // inc_ref (mod.rs:235-258)
    void inc_ref(uint64_t id) { ref_counts_[checked(id)] += 1; }
    // inc_ref_by (mod.rs:359-385)
    void inc_ref_by(uint64_t id, uint32_t count) { ref_counts_[checked(id)] += count; }

    // dec_ref (mod.rs:260-296). A decrement of a zero count wraps in a release build of the
    // reference; here it is reported as undefined behaviour.
    bool dec_ref(uint64_t id) {
        uint32_t i = checked(id);
        if (ref_counts_[i] == 0) throw RefUB("refcount underflow in dec_ref");
        ref_counts_[i] -= 1;
        if (ref_counts_[i] == 0) {
            patterns_[bid::is_leaf(id) ? 1 : 0].erase(hashes_[i]);
            recycle(id);
            return true;
        }
        return false;
    }
    // dec_ref_by (mod.rs:387-417)
    void dec_ref_by(uint64_t id, uint32_t count) {
        uint32_t i = checked(id);
        if (ref_counts_[i] < count) throw RefUB("refcount underflow in dec_ref_by");
        ref_counts_[i] -= count;
        if (ref_counts_[i] == 0) {
            patterns_[bid::is_leaf(id) ? 1 : 0].erase(hashes_[i]);
            recycle(id);
        }
    }
    // inc_child_refs (mod.rs:298-326): every non-empty child except slot `skip`
    void inc_child_refs(const Children &c, unsigned skip) {
        for (unsigned i = 0; i < 8; ++i) {
            if (i == skip) continue;
            if (!bid::is_empty(c[i])) inc_ref(c[i]);
        }
    }
    // dec_child_refs (mod.rs:536-564)
    void dec_child_refs(const Children &c) {
        for (uint64_t id : c)
            if (!bid::is_empty(id)) dec_ref(id);
    }

    // dec_ref_recursive (mod.rs:419-534): breadth-first release over a preallocated queue of
    // 32768 entries; a child whose count is above one is decremented in place, a child at one
    // is queued. Overflowing the queue is undefined behaviour in the reference (the overflow
    // check is debug-only); P3 grows the queue instead.
    void dec_ref_recursive(uint64_t id) {
        checked(id);
        size_t read_idx = 0, write_idx = 1;
        stack_[0] = id;
        while (read_idx < write_idx) {
            uint64_t current = stack_[read_idx++];
            uint32_t ci = checked(current);
            if (ref_counts_[ci] == 0) throw RefUB("refcount underflow in dec_ref_recursive");
            ref_counts_[ci] -= 1;
            if (ref_counts_[ci] == 0) {
                const Children ch = children_[ci];
                for (uint64_t child : ch) {
                    if (bid::is_empty(child)) continue;
                    uint32_t k = checked(child);
                    if (ref_counts_[k] > 1) {
                        ref_counts_[k] -= 1;
                    } else {
                        if (write_idx >= stack_.size()) {
                            if (flags_ & P3)
                                stack_.resize(stack_.size() * 2);
                            else
                                throw RefUB("dec_ref_recursive queue overflow (32768 entries)");
                        }
                        stack_[write_idx++] = child;
                    }
                }
                patterns_[bid::is_leaf(current) ? 1 : 0].erase(hashes_[ci]);
                recycle(current);
            }
        }
    }

    // recycle (mod.rs:566-625)
    void recycle(uint64_t id) {
        if (id == empty_branch_id_) throw RefPanic("Cannot recycle empty branch");
        uint32_t i = bid::index(id);
        values_[i] = T(0);
        children_[i] = Children{};
        hashes_[i] = 0;
        ref_counts_[i] = 0;
        uint16_t g = (uint16_t)(generations_[i] + 1);
        if (g >= bid::MAX_GENERATION) g = 0;
        generations_[i] = g;
        free_indices_.push_back(i);
    }

    // get_next_index_macro! (interner/macros.rs:1-41): LIFO free list, then bump, else panic.
    uint32_t get_next_index() {
        if (!free_indices_.empty()) {
            uint32_t i = free_indices_.back();
            free_indices_.pop_back();
            ++created_;
            return i;
        }
        if (next_index_ < capacity_) {
            ++created_;
            return next_index_++;
        }
        throw RefOOM("Out of memory");
    }
    // allocations so far (instrumentation; the reference keeps no such count)
    uint64_t created() const { return created_; }

    // get_or_create_leaf (mod.rs:627-710)
    uint64_t get_or_create_leaf(T value) {
        uint64_t hash = compute_leaf_hash(value);
        if (const uint64_t *hit = patterns_[1].find(hash)) {
            uint64_t existing = *hit;
            if (!is_valid_block_id(existing)) throw RefPanic("Expired node in patterns");
            inc_ref(existing);
            if (check_keys && values_[bid::index(existing)] != value) ++collisions;
            return existing;
        }
        uint32_t index = get_next_index();
        uint16_t generation = generations_[index];
        uint64_t id = bid::new_leaf(index, generation);
        patterns_[1].insert(hash, id);
        values_[index] = value;
        hashes_[index] = hash;
        inc_ref(id);
        return id;
    }

    // get_or_create_branch (mod.rs:712-829). Contract (mod.rs:712-715): every non-empty child
    // already carries one reference for its slot; a hit gives them back.
    uint64_t get_or_create_branch(const Children &c, uint8_t types, uint8_t mask) {
        uint64_t hash = compute_branch_hash(c, types, mask);
        if (const uint64_t *hit = patterns_[0].find(hash)) {
            uint64_t existing = *hit;
            if (check_keys && (bid::types(existing) != types || bid::mask(existing) != mask ||
                               children_[bid::index(existing)] != c))
                ++collisions;
            dec_child_refs(c);
            inc_ref(existing);
            return existing;
        }
        uint32_t index = get_next_index();
        uint16_t generation = generations_[index];
        uint64_t id = bid::new_branch(index, generation, types, mask);
        patterns_[0].insert(hash, id);
        T vals[8];
        for (int i = 0; i < 8; ++i) vals[i] = values_[bid::index(c[i])];
        children_[index] = c;
        values_[index] = calc_average(vals, 8);
        hashes_[index] = hash;
        inc_ref(id);
        return id;
    }

    // preallocate_branch_id (mod.rs:930-941): the record's index must be the next one allocated, on
    // a slot never recycled.
    uint64_t preallocate_branch_id(uint32_t index, uint8_t types, uint8_t mask) {
        if (get_next_index() != index) throw RefPanic("Invalid block id");
        if (generations_[index] != 0) throw RefPanic("Invalid generation");
        return bid::new_branch(index, 0, types, mask);
    }
    // deserialize_leaf (mod.rs:943-968); the default-value check is the reference's debug assertion.
    uint64_t deserialize_leaf(uint32_t index, T value) {
        if (value == T(0)) throw RefPanic("Leaf value should not be default");
        const uint64_t hash = compute_leaf_hash(value);
        if (get_next_index() != index) throw RefPanic("Invalid block id");
        if (generations_[index] != 0) throw RefPanic("Invalid generation");
        const uint64_t id = bid::new_leaf(index, 0);
        values_[index] = value;
        hashes_[index] = hash;
        patterns_[1].insert(hash, id);
        return id;
    }
    // deserialize_branch (mod.rs:970-993), with inc_all_child_refs (mod.rs:328-356).
    void deserialize_branch(uint64_t id, const Children &c, uint8_t types, uint8_t mask, T average) {
        const uint64_t hash = compute_branch_hash(c, types, mask);
        const uint32_t i = bid::index(id);
        children_[i] = c;
        values_[i] = average;
        hashes_[i] = hash;
        patterns_[0].insert(hash, id);
        inc_child_refs(c, 8);
    }

   private:
    uint32_t checked(uint64_t id) const {
        uint32_t i = bid::index(id);
        if (i >= capacity_) throw RefUB("block index outside the pool");
        return i;
    }

    FlatMap patterns_[2];  // [0] branch, [1] leaf (consts.rs:11-12)
    std::vector<uint32_t> free_indices_;
    uint32_t next_index_ = 1;
    std::vector<uint32_t> ref_counts_;
    std::vector<uint16_t> generations_;
    std::vector<Children> children_;
    std::vector<T> values_;
    std::vector<uint64_t> hashes_;
    size_t capacity_ = 0;
    uint64_t created_ = 0;
    uint64_t empty_branch_id_ = 0, empty_branch_hash_ = 0;
    std::vector<uint64_t> stack_;
    uint32_t flags_ = 0;
};

// ---- Batch<T> (core/batch.rs:39-240) -------------------------------------------------------------
template <class T>
class Batch {
   public:
    // Batch::new (batch.rs:63-81)
    Batch(int max_depth, uint32_t flags) : max_depth_(max_depth) {
        if (max_depth < 0 || max_depth >= depth_limit(flags)) throw RefPanic("Max depth exceeds allowed limit");
        int lower = max_depth > 0 ? max_depth - 1 : 0;
        size_t size = (size_t)1 << (3 * lower);
        set_.assign(size, 0);
        clear_.assign(size, 0);
        values_.assign(size * 8, T(0));
    }
    int max_depth() const { return max_depth_; }
    size_t groups() const { return set_.size(); }
    const uint8_t *set_masks() const { return set_.data(); }
    const uint8_t *clear_masks() const { return clear_.data(); }
    const T *values() const { return values_.data(); }  // [group][8]
    bool has_fill() const { return has_fill_; }
    T fill_value() const { return fill_; }
    bool has_patches() const { return has_patches_; }

    // Batch::size (batch.rs:115-123)
    size_t size() const {
        size_t n = 0;
        for (size_t g = 0; g < set_.size(); ++g) n += (set_[g] | clear_[g]) != 0;
        return n;
    }
    // Batch::just_set (batch.rs:145-172). Positions are bounds-checked (debug_assert at :146-148;
    // in release an out-of-range group index panics on the Vec index).
    bool just_set(int32_t x, int32_t y, int32_t z, T voxel) {
        int32_t n = 1 << max_depth_;
        if (x < 0 || y < 0 || z < 0 || x >= n || y >= n || z >= n) throw RefOOB("position out of bounds");
        uint32_t full = encode_child_index_path(x, y, z);
        size_t gi = full >> 3;
        unsigned idx = full & 7;
        uint8_t bit = (uint8_t)(1u << idx);
        if (voxel != T(0)) {
            set_[gi] |= bit;
            clear_[gi] &= (uint8_t)~bit;
        } else {
            set_[gi] &= (uint8_t)~bit;
            clear_[gi] |= bit;
        }
        values_[gi * 8 + idx] = voxel;
        has_patches_ = true;
        return true;
    }
    // Batch::just_fill (batch.rs:178-184)
    void just_fill(T value) {
        just_clear();
        has_fill_ = true;
        fill_ = value;
    }
    // Batch::just_clear (batch.rs:187-195)
    void just_clear() {
        std::fill(set_.begin(), set_.end(), 0);
        std::fill(clear_.begin(), clear_.end(), 0);
        std::fill(values_.begin(), values_.end(), T(0));
        has_fill_ = false;
        fill_ = T(0);
        has_patches_ = false;
    }

   private:
    int max_depth_;
    std::vector<uint8_t> set_, clear_;
    std::vector<T> values_;
    bool has_fill_ = false;
    T fill_ = T(0);
    bool has_patches_ = false;
};

// ---- get_at_depth (utils/common.rs:122-156) ------------------------------------------------------
// Returns true and writes *out when the voxel is non-empty.
template <class T>
inline bool get_at_depth(const Interner<T> &it, uint64_t node, int32_t x, int32_t y, int32_t z,
                         int current, int max, T *out) {
    const T def = T(0);
    int depth = current;
    while (!bid::is_empty(node)) {
        if (depth >= max) {
            T v = it.get_value(node);
            if (v != def) {
                *out = v;
                return true;
            }
            return false;
        }
        if (bid::is_branch(node)) {
            node = it.get_child_id(node, child_index(x, y, z, depth, max));
            depth += 1;
        } else {
            *out = it.get_value(node);
            return true;
        }
    }
    return false;
}

// ---- VoxTree<T> (spatial/voxtree.rs:108-1118) ----------------------------------------------------
// OccupancyDataBuilder (utils/mesh.rs:181-193) and fill_masks_for_region (mesh.rs:418-511): a 64^3
// space, three planes of 64 x 64 u64 words (YZ: [y][z] -> x bits, XZ: [z][x] -> y bits, XY: [y][x]
// -> z bits), global and per material, six active row/column masks and voxel counts per material.
struct Occupancy {
    static constexpr uint32_t kAxis = 64, kPlane = 64 * 64, kAll = 3 * 64 * 64;
    static constexpr uint32_t kYZ = 0, kXZ = kPlane, kXY = 2 * kPlane;
    std::vector<uint64_t> global = std::vector<uint64_t>(kAll, 0);
    uint64_t active[6] = {0, 0, 0, 0, 0, 0};
    std::map<uint32_t, std::vector<uint64_t>> per_material;
    std::map<uint32_t, uint64_t> materials;

    void fill_region(uint32_t sx, uint32_t sy, uint32_t sz, uint32_t side, uint32_t material) {
        materials[material] += (uint64_t)side * side * side;
        if (side != kAxis) {
            auto &pm = per_material[material];
            if (pm.empty()) pm.assign(kAll, 0);
            const uint64_t run = (1ull << side) - 1;
            const uint64_t xm = run << sx, ym = run << sy, zm = run << sz;
            active[0] |= ym;
            active[1] |= zm;
            active[2] |= zm;
            active[3] |= xm;
            active[4] |= ym;
            active[5] |= xm;
            for (uint32_t i = 0; i < side; ++i) {
                const uint32_t z = sz + i, y = sy + i;
                const uint32_t by = kXZ + z * kAxis + sx, bz = kXY + y * kAxis + sx, bx = kYZ + y * kAxis + sz;
                for (uint32_t j = 0; j < side; ++j) {
                    global[by + j] |= ym;
                    pm[by + j] |= ym;
                    global[bz + j] |= zm;
                    pm[bz + j] |= zm;
                    global[bx + j] |= xm;
                    pm[bx + j] |= xm;
                }
            }
        } else {
            per_material[material].assign(kAll, ~0ull);
            std::fill(global.begin(), global.end(), ~0ull);
            for (auto &a : active) a = ~0ull;
        }
    }
};

template <class T>
class Tree {
   public:
    // VoxTree::new (voxtree.rs:116-127); MaxDepth::new asserts the cap (max_depth.rs:77-83).
    Tree(int max_depth, uint32_t flags) : max_depth_(max_depth) {
        if (max_depth < 0 || max_depth >= depth_limit(flags)) throw RefPanic("Max depth exceeds allowed limit");
    }
    int max_depth() const { return max_depth_; }
    uint64_t root() const { return root_; }
    bool dirty() const { return dirty_; }
    void clear_dirty() { dirty_ = false; }
    bool is_empty() const { return bid::is_empty(root_); }
    bool is_leaf() const { return bid::is_leaf(root_); }

    void check_bounds(int32_t x, int32_t y, int32_t z) const {
        int32_t n = 1 << max_depth_;
        if (x < 0 || y < 0 || z < 0 || x >= n || y >= n || z >= n) throw RefOOB("position out of bounds");
    }

    // VoxOpsRead::get (voxtree.rs:145-159)
    bool get(const Interner<T> &it, int32_t x, int32_t y, int32_t z, T *out) const {
        check_bounds(x, y, z);
        return get_at_depth(it, root_, x, y, z, 0, max_depth_, out);
    }

    // VoxOpsWrite::set (voxtree.rs:163-260)
    bool set(Interner<T> &it, int32_t x, int32_t y, int32_t z, T voxel) {
        check_bounds(x, y, z);
        uint64_t new_root;
        if (!bid::is_empty(root_) || voxel != T(0))
            new_root = set_at_root(it, root_, x, y, z, max_depth_, voxel);
        else
            return false;
        if (new_root != bid::INVALID) {
            if (!bid::is_empty(root_)) {
                if (new_root == root_) throw RefPanic("assert_ne!(new_root_id, self.root_id)");
                it.dec_ref_recursive(root_);
            }
            if (!it.is_valid_block_id(new_root)) throw RefPanic("Invalid new root id");
            root_ = new_root;
            dirty_ = true;
            return true;
        }
        return false;
    }

    // VoxOpsBulkWrite::fill (voxtree.rs:264-277)
    void fill(Interner<T> &it, T value) {
        if (value != T(0)) {
            if (!bid::is_empty(root_)) it.dec_ref_recursive(root_);
            root_ = it.get_or_create_leaf(value);
            dirty_ = true;
        } else {
            clear(it);
        }
    }
    // VoxOpsBulkWrite::clear (voxtree.rs:279-292)
    void clear(Interner<T> &it) {
        if (!bid::is_empty(root_)) {
            it.dec_ref_recursive(root_);
            root_ = bid::EMPTY;
            dirty_ = true;
        }
    }

    // VoxOpsBatch::apply_batch (voxtree.rs:303-328). Under P4 every cleared voxel is then removed
    // with VoxTree::set(pos, 0), in ascending Morton order.
    bool apply_batch(Interner<T> &it, const Batch<T> &batch) {
        if (batch.max_depth() != max_depth_) throw RefPanic("batch depth differs from the tree depth");
        uint64_t new_root = set_batch_at_root(it, root_, max_depth_, batch);
        bool changed = false;
        if (new_root != bid::INVALID) {
            if (!bid::is_empty(root_)) {
                if (new_root == root_ && !(it.flags() & P5)) throw RefPanic("assert_ne!(new_root_id, self.root_id)");
                it.dec_ref_recursive(root_);
            }
            if (!it.is_valid_block_id(new_root)) throw RefPanic("Invalid new root id");
            root_ = new_root;
            dirty_ = true;
            changed = true;
        }
        if (it.flags() & P4) {
            const uint8_t *cm = batch.clear_masks();
            const int d = max_depth_;
            for (size_t g = 0; g < batch.groups(); ++g) {
                if (!cm[g]) continue;
                for (unsigned s = 0; s < 8; ++s) {
                    if (!((cm[g] >> s) & 1)) continue;
                    int32_t x, y, z;
                    decode_path((uint32_t)((g << 3) | s), d, &x, &y, &z);
                    changed |= set(it, x, y, z, T(0));
                }
            }
        }
        return changed;
    }

    // to_vec (utils/common.rs:158-246): dense [y][z][x] grid.
    void to_vec(const Interner<T> &it, T *data) const {
        const int md = max_depth_;
        const size_t n = (size_t)1 << md;
        const size_t size = n * n * n;
        if (!bid::is_branch(root_)) {
            T v = it.get_value(root_);
            for (size_t i = 0; i < size; ++i) data[i] = v;
            return;
        }
        for (size_t i = 0; i < size; ++i) data[i] = T(0);
        if (bid::is_empty(root_)) return;
        struct E {
            uint64_t id;
            int32_t x, y, z;
            int depth;
        };
        std::vector<E> stack;
        stack.push_back({root_, 0, 0, 0, 0});
        while (!stack.empty()) {
            E e = stack.back();
            stack.pop_back();
            if (bid::is_branch(e.id) && e.depth < md) {
                int32_t half = 1 << (md - e.depth - 1);
                const Children &ch = it.get_children(e.id);
                for (int i = 7; i >= 0; --i) {
                    uint64_t c = ch[i];
                    if (bid::is_empty(c)) continue;
                    stack.push_back({c, e.x + (i & 1) * half, e.y + ((i >> 1) & 1) * half,
                                     e.z + ((i >> 2) & 1) * half, e.depth + 1});
                }
            } else {
                T v = it.get_value(e.id);
                if (v == T(0)) continue;
                size_t side = (size_t)1 << (md - e.depth);
                for (size_t yy = e.y; yy < e.y + side; ++yy)
                    for (size_t zz = e.z; zz < e.z + side; ++zz) {
                        T *row = data + yy * n * n + zz * n + e.x;
                        for (size_t xx = 0; xx < side; ++xx) row[xx] = v;
                    }
            }
        }
    }

    // generate_occupancy_masks (utils/mesh.rs:515-597): the same traversal as to_vec, each
    // non-default leaf region passed to fill_masks_for_region at `offset` inside the 64^3 builder.
    template <class B>
    void occupancy_masks(const Interner<T> &it, B &builder, uint32_t ox, uint32_t oy, uint32_t oz) const {
        if (bid::is_empty(root_)) return;
        const uint32_t md = (uint32_t)max_depth_;
        if (!bid::is_branch(root_)) {
            T v = it.get_value(root_);
            if (v != T(0)) builder.fill_region(ox, oy, oz, 1u << md, (uint32_t)v);
            return;
        }
        struct E {
            uint64_t id;
            uint32_t x, y, z, depth;
        };
        std::vector<E> stack;
        stack.push_back({root_, 0, 0, 0, 0});
        while (!stack.empty()) {
            E e = stack.back();
            stack.pop_back();
            if (bid::is_branch(e.id) && e.depth < md) {
                const uint32_t half = 1u << (md - e.depth - 1);
                const Children &ch = it.get_children(e.id);
                for (int i = 7; i >= 0; --i) {
                    uint64_t c = ch[i];
                    if (bid::is_empty(c)) continue;
                    stack.push_back({c, e.x + (i & 1) * half, e.y + ((i >> 1) & 1) * half,
                                     e.z + ((i >> 2) & 1) * half, e.depth + 1});
                }
            } else {
                T v = it.get_value(e.id);
                if (v == T(0)) continue;
                builder.fill_region(ox + e.x, oy + e.y, oz + e.z, 1u << (md - e.depth), (uint32_t)v);
            }
        }
    }

    // The tree holds one reference to its root (set_root_id, voxtree.rs:136-142).
    void set_root_raw(uint64_t r) { root_ = r; }
    // set_root_id (voxtree.rs:135-141): counts a reference on the new root, EMPTY included.
    void set_root_id(Interner<T> &it, uint64_t r) {
        root_ = r;
        it.inc_ref(r);
    }

    static void decode_path(uint32_t path, int d, int32_t *x, int32_t *y, int32_t *z) {
        int32_t px = 0, py = 0, pz = 0;
        for (int b = 0; b < d; ++b) {
            px |= ((path >> (3 * b)) & 1) << b;
            py |= ((path >> (3 * b + 1)) & 1) << b;
            pz |= ((path >> (3 * b + 2)) & 1) << b;
        }
        *x = px;
        *y = py;
        *z = pz;
    }

   private:
    // set_at_root (voxtree.rs:372-391)
    static uint64_t set_at_root(Interner<T> &it, uint64_t node, int32_t x, int32_t y, int32_t z,
                                int max_depth, T voxel) {
        if (node == bid::INVALID) throw RefPanic("assert!(node_id != INVALID)");
        if (voxel != T(0)) return set_at_depth_iterative(it, node, x, y, z, 0, max_depth, voxel);
        return remove_at_depth(it, node, x, y, z, 0, max_depth);
    }

    // set_at_depth_iterative (voxtree.rs:393-540)
    static uint64_t set_at_depth_iterative(Interner<T> &it, uint64_t initial_node, int32_t x,
                                           int32_t y, int32_t z, int initial_depth, int max_depth,
                                           T voxel) {
        struct Frame {
            uint64_t node, leaf;
            uint8_t index;
        };
        Frame stack[MAX_PATCHED_DEPTH];
        uint64_t current = initial_node;
        int depth = initial_depth;
        uint64_t leaf_node = bid::EMPTY;
        // Phase 1: descend and build the chain (:421-459)
        while (depth < max_depth) {
            unsigned index = child_index(x, y, z, depth, max_depth);
            if (bid::is_branch(current)) {
                stack[depth] = {current, leaf_node, (uint8_t)index};
                current = it.get_child_id(current, index);
            } else {
                if (it.get_value(current) == voxel) return bid::INVALID;  // nothing changed
                leaf_node = current;
                current = bid::EMPTY;
                stack[depth] = {current, leaf_node, (uint8_t)index};
            }
            depth += 1;
        }
        // Phase 2: the leaf (:461-482)
        if (bid::is_leaf(current) && it.get_value(current) == voxel) return bid::INVALID;
        current = it.get_or_create_leaf(voxel);
        // Phase 3: propagate upwards (:484-532)
        while (depth > initial_depth) {
            depth -= 1;
            Frame f = stack[depth];
            if (!bid::is_empty(f.node)) {
                uint8_t types = (uint8_t)(bid::types(f.node) | ((bid::is_leaf(current) ? 1u : 0u) << f.index));
                Children branch = it.get_children(f.node);
                branch[f.index] = current;
                bool all_same = types == 0xFF;
                if (all_same)
                    for (uint64_t c : branch) all_same = all_same && c == current;
                if (!all_same) {
                    uint8_t mask = (uint8_t)(bid::mask(f.node) | (1u << f.index));
                    it.inc_child_refs(branch, f.index);
                    current = it.get_or_create_branch(branch, types, mask);
                }
            } else if (bid::is_empty(f.leaf)) {
                Children ch{};
                ch[f.index] = current;
                uint8_t types = (uint8_t)((bid::is_leaf(current) ? 1u : 0u) << f.index);
                uint8_t mask = (uint8_t)(1u << f.index);
                current = it.get_or_create_branch(ch, types, mask);
            } else {
                Children ch;
                ch.fill(f.leaf);
                it.inc_ref_by(f.leaf, 7);
                ch[f.index] = current;
                uint8_t types = (uint8_t)(~(1u << f.index) | ((bid::is_leaf(current) ? 1u : 0u) << f.index));
                current = it.get_or_create_branch(ch, types, 0xFF);
            }
        }
        return current;
    }

    // remove_at_depth (voxtree.rs:542-557)
    static uint64_t remove_at_depth(Interner<T> &it, uint64_t node, int32_t x, int32_t y, int32_t z,
                                    int current, int max) {
        if (node == bid::INVALID) throw RefPanic("assert!(node_id != INVALID)");
        if (bid::is_branch(node)) return remove_at_depth_branch(it, node, x, y, z, current, max);
        return remove_at_depth_leaf(it, node, x, y, z, current, max);
    }

    // remove_at_depth_branch (voxtree.rs:559-652)
    static uint64_t remove_at_depth_branch(Interner<T> &it, uint64_t node, int32_t x, int32_t y,
                                           int32_t z, int current, int max) {
        if (!it.is_valid_block_id(node)) throw RefPanic("assert!(is_valid_block_id)");
        if (!(current < max)) throw RefPanic("Branch node at max depth");
        unsigned index = child_index(x, y, z, current, max);
        if (!bid::has_child(node, index)) return bid::INVALID;
        Children branch = it.get_children(node);
        uint64_t child = branch[index];
        uint64_t new_child = remove_at_depth(it, child, x, y, z, current + 1, max);
        if (new_child == bid::INVALID) return bid::INVALID;
        if (!it.is_valid_block_id(new_child)) throw RefPanic("assert!(is_valid_block_id(new_child))");
        bool empty = bid::is_empty(new_child);
        uint8_t mask = empty ? (uint8_t)(bid::mask(node) & ~(1u << index)) : bid::mask(node);
        if (mask == 0) return bid::EMPTY;
        if (!bid::is_branch(new_child)) throw RefPanic("Removing voxel should never produce a leaf node");
        uint8_t types = (uint8_t)(bid::types(node) & ~(1u << index));
        branch[index] = new_child;
        it.inc_child_refs(branch, index);
        return it.get_or_create_branch(branch, types, mask);
    }

    // remove_at_depth_leaf (voxtree.rs:654-706)
    static uint64_t remove_at_depth_leaf(Interner<T> &it, uint64_t node, int32_t x, int32_t y,
                                         int32_t z, int current, int max) {
        if (!it.is_valid_block_id(node)) throw RefPanic("assert!(is_valid_block_id)");
        if (current == max) return bid::EMPTY;
        uint64_t new_node = remove_at_depth_leaf(it, node, x, y, z, current + 1, max);
        if (!it.is_valid_block_id(new_node)) throw RefPanic("assert!(is_valid_block_id(new_node))");
        unsigned index = child_index(x, y, z, current, max);
        Children ch;
        ch.fill(node);
        ch[index] = new_node;
        bool leaf = bid::is_leaf(new_node), empty = bid::is_empty(new_node);
        uint8_t types = (uint8_t)(~(1u << index) | ((leaf ? 1u : 0u) << index));
        uint8_t mask = (uint8_t)(~(1u << index) | ((!empty ? 1u : 0u) << index));
        it.inc_ref_by(node, 7);
        return it.get_or_create_branch(ch, types, mask);
    }

    // set_batch_at_root (voxtree.rs:708-722)
    static uint64_t set_batch_at_root(Interner<T> &it, uint64_t node, int max_depth, const Batch<T> &b) {
        if (node == bid::INVALID) throw RefPanic("assert!(node_id != INVALID)");
        return set_batch_at_depth_iterative(it, node, 0, max_depth, b);
    }

    // set_batch_at_depth_iterative (voxtree.rs:724-1118)
    static uint64_t set_batch_at_depth_iterative(Interner<T> &it, uint64_t initial_node,
                                                 int initial_depth_, int max_depth_i, const Batch<T> &batch) {
        // Phase 0: fill (:742-758)
        if (batch.has_fill()) initial_node = it.get_or_create_leaf(batch.fill_value());
        if (!batch.has_patches()) return initial_node;

        const size_t max_depth = (size_t)max_depth_i;
        const size_t initial_depth = (size_t)initial_depth_;
        // max_depth 0 and 1 underflow `max_depth - 1` / `target_depth - 1` in the reference (usize
        // arithmetic at :792 and :913); they are reported as reference panics here.
        if (max_depth < 2) throw RefPanic("batch apply needs max_depth >= 2 (usize underflow in the reference)");

        // Phase 1: bottom groups (:770-897)
        const size_t data_len = batch.groups();
        std::vector<uint64_t> current_level(data_len, bid::INVALID), next_level(data_len, bid::INVALID);
        std::vector<size_t> paths, next_paths;
        paths.reserve(data_len);
        next_paths.reserve(data_len);
        const uint8_t *set_masks = batch.set_masks();
        const T *all_values = batch.values();

        for (size_t path_index = 0; path_index < data_len; ++path_index) {
            const uint8_t set_mask = set_masks[path_index];
            if (set_mask == 0) continue;
            const size_t path = path_index << 3;
            uint64_t current = initial_node;
            uint64_t leaf_node = bid::EMPTY;
            for (size_t d = initial_depth; d < max_depth - 1; ++d) {
                if (bid::is_branch(current)) {
                    size_t index = (path >> ((max_depth - d - 1) * 3)) & 7;
                    current = it.get_child_id(current, (unsigned)index);
                } else {
                    leaf_node = current;
                    current = bid::EMPTY;
                }
                if (bid::is_empty(current)) break;
            }
            // P1: a leaf met exactly at depth max-1 is an ancestor leaf (the reference panics in
            // BlockId::types() below, block_id.rs:273-276).
            if ((it.flags() & P1) && !bid::is_empty(current) && bid::is_leaf(current)) {
                leaf_node = current;
                current = bid::EMPTY;
            }
            const T *values = all_values + path_index * 8;
            bool all_same = set_mask == 0xFF;
            if (all_same)
                for (int i = 1; i < 8; ++i) all_same = all_same && values[i] == values[0];

            if (!all_same) {
                Children children{};
                uint8_t types = 0, mask = 0;
                if (!bid::is_empty(current)) {
                    children = it.get_children(current);
                    types = bid::types(current);
                    mask = bid::mask(current);
                } else if (bid::is_leaf(leaf_node)) {
                    unsigned data = (unsigned)__builtin_popcount(set_mask);
                    it.inc_ref_by(leaf_node, 8 - data);
                    children.fill(leaf_node);
                    types = 0xFF;
                    mask = 0xFF;
                }
                uint8_t modified = 0;
                uint8_t bits = set_mask;
                while (bits) {
                    unsigned idx = (unsigned)__builtin_ctz(bits);
                    bits &= (uint8_t)~(1u << idx);
                    const T value = values[idx];
                    if (!bid::is_empty(children[idx]) && it.get_value(children[idx]) == value) continue;
                    children[idx] = it.get_or_create_leaf(value);
                    types |= (uint8_t)(1u << idx);
                    mask |= (uint8_t)(1u << idx);
                    modified |= (uint8_t)(1u << idx);
                }
                if (modified == 0) continue;
                if (bid::is_empty(leaf_node)) {
                    uint8_t nm = (uint8_t)~modified;
                    while (nm) {
                        unsigned idx = (unsigned)__builtin_ctz(nm);
                        nm &= (uint8_t)~(1u << idx);
                        if (!bid::is_empty(children[idx])) it.inc_ref_by(children[idx], 1);
                    }
                }
                uint64_t branch = it.get_or_create_branch(children, types, mask);
                current_level[path_index] = branch;
                paths.push_back(path);
            } else {
                T first = values[__builtin_ctz(set_mask)];
                current_level[path_index] = it.get_or_create_leaf(first);
                paths.push_back(path);
            }
        }

        // Phase 2: integrate upwards (:899-1106)
        if (paths.empty()) return bid::INVALID;
        size_t target_depth = max_depth - 1;
        while (!paths.empty()) {
            size_t path = paths.back();
            paths.pop_back();
            size_t path_mask_depth = target_depth > 1 ? target_depth - 2 : 0;
            size_t pmask = (size_t)path_mask((int)max_depth, (int)path_mask_depth);

            uint64_t equivalent = initial_node;
            uint64_t leaf_id = bid::EMPTY;
            for (size_t d = 0; d + 1 < target_depth; ++d) {  // 0..(target_depth - 1)
                if (bid::is_leaf(equivalent)) {
                    leaf_id = equivalent;
                    equivalent = bid::EMPTY;
                    break;
                } else {
                    size_t index = (path >> ((max_depth - d - 1) * 3)) & 7;
                    equivalent = it.get_child_id(equivalent, (unsigned)index);
                }
                if (bid::is_empty(equivalent)) break;
            }
            if (bid::is_leaf(equivalent)) {
                leaf_id = equivalent;
                equivalent = bid::EMPTY;
            }

            Children children{};
            uint8_t types = 0, mask = 0;
            bool has_next_sibling = true;
            while (has_next_sibling) {
                size_t target_index = (path >> ((max_depth - target_depth) * 3)) & 7;
                if (target_depth == 1)
                    has_next_sibling = !paths.empty();
                else if (!paths.empty())
                    has_next_sibling = (path & pmask) == (paths.back() & pmask);
                else
                    has_next_sibling = false;
                size_t cpi = path >> 3;
                uint64_t id = current_level[cpi];
                children[target_index] = id;
                current_level[cpi] = bid::INVALID;
                types |= (uint8_t)((bid::is_leaf(id) ? 1u : 0u) << target_index);
                mask |= (uint8_t)(1u << target_index);
                if (has_next_sibling && !paths.empty()) {
                    path = paths.back();
                    paths.pop_back();
                }
            }

            const uint8_t existing_mask = bid::mask(equivalent);
            const uint8_t inv_mask = (uint8_t)~mask;
            const uint8_t cloned = (uint8_t)(existing_mask & inv_mask);
            if (mask != 0xFF) {
                if (cloned != 0) {
                    const Children &existing = it.get_children(equivalent);
                    uint8_t bits = cloned;
                    while (bits) {
                        unsigned idx = (unsigned)__builtin_ctz(bits);
                        bits &= (uint8_t)~(1u << idx);
                        children[idx] = existing[idx];
                        types |= (uint8_t)((bid::is_leaf(children[idx]) ? 1u : 0u) << idx);
                        mask |= (uint8_t)(1u << idx);
                    }
                } else if (!bid::is_empty(leaf_id)) {
                    unsigned n = (unsigned)__builtin_popcount(inv_mask);
                    types |= inv_mask;
                    mask |= inv_mask;
                    uint8_t bits = inv_mask;
                    while (bits) {
                        unsigned idx = (unsigned)__builtin_ctz(bits);
                        children[idx] = leaf_id;
                        bits &= (uint8_t)~(1u << idx);
                    }
                    it.inc_ref_by(leaf_id, n);
                }
            }
            bool all_same = types == 0xFF;
            if (all_same)
                for (uint64_t c : children) all_same = all_same && c == children[0];
            uint64_t new_node;
            if (!all_same) {
                uint8_t bits = cloned;
                while (bits) {
                    unsigned idx = (unsigned)__builtin_ctz(bits);
                    bits &= (uint8_t)~(1u << idx);
                    it.inc_ref(children[idx]);
                }
                new_node = it.get_or_create_branch(children, types, mask);
            } else {
                unsigned dec = cloned != 0 ? std::min(7u, (unsigned)__builtin_popcount(cloned)) : 7u;
                it.dec_ref_by(children[0], dec);
                new_node = children[0];
            }
            size_t np = path & pmask;
            next_paths.push_back(np);
            next_level[np >> 3] = new_node;
            if (paths.empty()) {
                std::swap(current_level, next_level);
                std::swap(paths, next_paths);
                next_paths.clear();
                target_depth -= 1;
                if (target_depth == 0) break;
            }
        }
        return current_level[paths[0] >> 3];
    }

    int max_depth_;
    uint64_t root_ = bid::EMPTY;
    bool dirty_ = false;
};

}  // namespace vxo
