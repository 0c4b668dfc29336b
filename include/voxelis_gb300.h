/*
 * voxelis_gb300 — C ABI of the GB300-native SVO-DAG edit-and-intern path.
 *
 * This header is the drop-in boundary for voxelis' batched edit path. Each entry point names
 * the reference interface it replaces (paths are relative to the voxelis repository):
 *
 *   VoxInterner::<T>::with_memory_budget   voxelis/src/interner/mod.rs:45-164
 *   VoxTree::new / get / set / fill / clear voxelis/src/spatial/voxtree.rs:116-292
 *   VoxTree::apply_batch                    voxelis/src/spatial/voxtree.rs:303-328
 *   Batch::new / just_set / just_fill / just_clear / size / has_patches
 *                                           voxelis/src/core/batch.rs:63-195
 *   VoxInterner::get_ref                    voxelis/src/interner/mod.rs:222-233
 *   collect_stats / to_vec (verification)   voxelis/src/utils/common.rs:158-333
 *
 * Conventions
 *   - Every function returns an int status (VX_OK or a VX_E_* code). Reference panics map to
 *     status codes; nothing unwinds or aborts across this boundary.
 *   - The interner's node store, hash-consing tables, reference counts and generations live in
 *     device memory (HBM). Trees are small integer handles whose root ids also live on the device.
 *   - Voxel values cross the boundary as uint32_t and must fit the interner's voxel width
 *     (8 or 16 bits). Value 0 is the empty voxel (T::default()).
 *   - Functions taking a `vx_mem` argument read/write either host memory (VX_MEM_HOST; copies are
 *     done inside the call) or device memory (VX_MEM_DEVICE; pointers must be device pointers).
 *   - All device work is ordered on the interner's stream (vx_interner_set_stream). Calls that
 *     return results in host memory synchronise that stream before returning; the *_async calls
 *     do not, and their status is reported by the next vx_interner_sync.
 *   - One writer at a time per interner, as in the reference (&mut VoxInterner).
 */
#ifndef VOXELIS_GB300_H
#define VOXELIS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------------------------ */
#define VX_OK 0
#define VX_E_INVALID_ARG 1  /* null/unknown handle, bad voxel width, bad flag                    */
#define VX_E_OOB 2          /* position outside the tree (voxtree.rs:146-148 assert!)            */
#define VX_E_OOM 3          /* node capacity exhausted (interner/macros.rs:38 panic!)            */
#define VX_E_DEPTH 4        /* depth cap (core/max_depth.rs:77-83) or unsupported depth          */
#define VX_E_TABLE_FULL 5   /* device hash table probe limit reached                             */
#define VX_E_TIMEOUT 6      /* a bounded device spin-wait gave up; the context stays usable      */
#define VX_E_CUDA 7         /* CUDA runtime error                                                */
#define VX_E_REF_PANIC 8    /* the reference panics on this input (assert!, BlockId::types())   */
#define VX_E_REF_UB 9       /* the reference hits undefined behaviour (refcount underflow,
                               release-stack overflow, dangling child)                          */
#define VX_E_BUFFER 10      /* caller buffer too small; the required size is reported            */
#define VX_E_UNSUPPORTED 11 /* valid request outside this build's supported set                 */

/* ---- reference patches (behaviour switches, all OFF by default) --------------------------- */
/* P1: a leaf met exactly at depth max-1 during the batch descent is treated as an ancestor leaf
 *     instead of panicking in BlockId::types() (voxtree.rs:792-834, block_id.rs:273-276).      */
#define VX_PATCH_P1 (1u << 0)
/* P2: depths up to 10 with the closed-form sibling masks (voxtree.rs:41-105 covers 0..6).     */
#define VX_PATCH_P2 (1u << 1)
/* P3: growable release queue instead of the fixed 32768 entries (interner/mod.rs:99, 431-513). */
#define VX_PATCH_P3 (1u << 2)
/* P4: batch clear bits are honoured, as VoxTree::set(pos, 0) applied to every cleared voxel
 *     after the set phase (voxtree.rs:563-705); without it they are ignored (voxtree.rs:779).  */
#define VX_PATCH_P4 (1u << 3)
/* P5: apply_batch's assert_ne!(new_root, old_root) (voxtree.rs:311) is skipped: a batch that
 *     rebuilds the identical root releases the old root as usual, which leaves every count as it
 *     was (the reference panics instead, e.g. when a batch re-sets full uniform groups).         */
#define VX_PATCH_P5 (1u << 4)

/* ---- memory locations --------------------------------------------------------------------- */
typedef enum { VX_MEM_HOST = 0, VX_MEM_DEVICE = 1 } vx_mem;

/* ---- special block ids (core/block_id.rs:120-123) ----------------------------------------- */
#define VX_BLOCK_EMPTY 0ull
#define VX_BLOCK_INVALID 0xFFFFFFFFFFFFFFFFull

typedef struct vx_interner vx_interner; /* opaque: device-resident VoxInterner<T>          */
typedef struct vx_batch vx_batch;       /* opaque: host staging buffer mirroring Batch<T>   */
typedef uint32_t vx_tree;               /* tree handle, scoped to one interner              */

typedef struct {
    uint64_t capacity;        /* nodes_capacity = budget / node_size (interner/mod.rs:49-53)      */
    uint64_t node_size;       /* 4 + 2 + 64 + sizeof(T) + 8 bytes (interner/mod.rs:158-164)       */
    uint64_t next_index;      /* bump pointer (interner/macros.rs:19-35)                          */
    uint64_t free_count;      /* length of the LIFO free list (interner/mod.rs:608)               */
    uint64_t alive_nodes;     /* next_index - free_count (includes the EMPTY branch at index 0)   */
    uint64_t branch_patterns; /* live entries in the branch table                                 */
    uint64_t leaf_patterns;   /* live entries in the leaf table                                   */
    uint64_t table_slots;     /* device branch table size (slots), 0 for the oracle               */
    uint64_t table_tombstones;/* deleted slots awaiting a rehash                                  */
    uint64_t error_flags;     /* sticky device error bits (see vx_interner_sync)                  */
    uint64_t nodes_created;   /* node allocations (interner misses) since creation or reset       */
} vx_interner_stats;

/* Canonical depth-first export: nodes renumbered in pre-order over the given trees (children
 * visited in slot order 0..7, EMPTY children skipped), so that two interners holding the same
 * DAG produce byte-identical arrays whatever their allocation order. */
typedef struct {
    uint8_t *kind;      /* [n_nodes] 1 = leaf, 0 = branch                                   */
    uint8_t *types;     /* [n_nodes] BlockId types bits (0 for leaves)                      */
    uint8_t *mask;      /* [n_nodes] BlockId mask bits (0 for leaves)                       */
    uint32_t *value;    /* [n_nodes] leaf value, or the branch LOD value (voxel.rs:96-141)  */
    uint32_t *refcount; /* [n_nodes]                                                        */
    int32_t *children;  /* [n_nodes * 8] canonical child ids, -1 for EMPTY                  */
    int32_t *roots;     /* [n_trees] canonical root id, -1 for an EMPTY tree                */
    uint64_t capacity;  /* number of node entries the arrays above can hold                 */
} vx_canonical;

/* ---- interner ----------------------------------------------------------------------------- */
/* VoxInterner::<T>::with_memory_budget(budget) (interner/mod.rs:45). voxel_bits is 8 or 16.
 * patch_flags is a VX_PATCH_* mask. table_log2 = 0 sizes the device branch table
 * automatically (2 x capacity slots, rounded up to a power of two). */
int vx_interner_create(uint64_t budget_bytes, int voxel_bits, uint32_t patch_flags,
                       int table_log2, vx_interner **out);
int vx_interner_destroy(vx_interner *it);
/* Bounds of the device's waits for this interner (no counterpart in the reference, whose waits
 * cannot fail): max_probes branch-table probes per insert before VX_E_TABLE_FULL (at most the table's
 * slots; 1..65536 by default), round_limit rounds of the warp-cooperative insert loop and spin_limit
 * iterations of a wait on another thread (a leaf being created, a grid barrier, a scan's look-back)
 * before VX_E_TIMEOUT. Later calls use the new values; every wait ends, and the context stays usable
 * (vx_interner_reset clears the sticky status). Defaults: 2^20 rounds, 2^22 spins. */
int vx_interner_set_limits(vx_interner *it, uint32_t max_probes, uint32_t round_limit, uint32_t spin_limit);
int vx_interner_get_limits(vx_interner *it, uint32_t *max_probes, uint32_t *round_limit, uint32_t *spin_limit);
/* Orders all later work of this interner on `cuda_stream` (a cudaStream_t; NULL = the
 * interner's own stream). */
int vx_interner_set_stream(vx_interner *it, void *cuda_stream);
/* Waits for the interner's stream and returns the first sticky device error as a status. */
int vx_interner_sync(vx_interner *it);
int vx_interner_stats_get(vx_interner *it, vx_interner_stats *out);
/* VoxInterner::get_ref (interner/mod.rs:222-233); VX_E_INVALID_ARG for a stale id. */
int vx_get_ref(vx_interner *it, uint64_t block_id, uint32_t *out);
/* Copies of the value stored for a node (leaf value or branch LOD value). */
int vx_get_value(vx_interner *it, uint64_t block_id, uint32_t *out);
/* Human-readable text of the last error reported by this interner (never NULL). */
const char *vx_last_error(vx_interner *it);

/* ---- trees (VoxTree, voxtree.rs:108-142) -------------------------------------------------- */
int vx_tree_create(vx_interner *it, int max_depth, vx_tree *out);
/* Creates n trees at once; depths[i] per tree. */
int vx_trees_create(vx_interner *it, uint32_t n, const uint8_t *depths, vx_tree *out);
/* Releases the tree's root (dec_ref_recursive) and frees the handle. The reference has no Drop
 * on VoxTree; this is VoxTree::clear followed by forgetting the tree. */
int vx_tree_destroy(vx_interner *it, vx_tree tree);
int vx_tree_root(vx_interner *it, vx_tree tree, uint64_t *out_root);
int vx_tree_max_depth(vx_interner *it, vx_tree tree, int *out);
/* VoxOpsRead::get (voxtree.rs:145-159). *found = 0 for an empty voxel. */
int vx_tree_get(vx_interner *it, vx_tree tree, int32_t x, int32_t y, int32_t z, int *found,
                uint32_t *value);
/* VoxOpsWrite::set (voxtree.rs:163-260): single-voxel set; value 0 removes the voxel. */
int vx_tree_set(vx_interner *it, vx_tree tree, int32_t x, int32_t y, int32_t z,
                uint32_t value, int *changed);
/* VoxOpsBulkWrite::fill / clear (voxtree.rs:264-292). */
int vx_tree_fill(vx_interner *it, vx_tree tree, uint32_t value);
int vx_tree_clear(vx_interner *it, vx_tree tree);

/* ---- batches (Batch<T>, core/batch.rs) ----------------------------------------------------- */
/* Batch::new(MaxDepth) (batch.rs:63-81); the depth cap follows patch_flags (P2) like the
 * interner's. */
int vx_batch_create(int max_depth, int voxel_bits, uint32_t patch_flags, vx_batch **out);
int vx_batch_destroy(vx_batch *b);
/* Batch::just_set (batch.rs:145-172): last write to a voxel wins; value 0 records a clear. */
int vx_batch_set(vx_batch *b, int32_t x, int32_t y, int32_t z, uint32_t value);
/* Batch::just_fill (batch.rs:178-184). */
int vx_batch_fill(vx_batch *b, uint32_t value);
/* Batch::just_clear (batch.rs:187-195). */
int vx_batch_clear(vx_batch *b);
/* Batch::just_set for n voxels in order (xyz[3i..3i+2], values[i]); stops at the first invalid
 * position or value and reports it. */
int vx_batch_set_many(vx_batch *b, uint64_t n, const int32_t *xyz, const uint32_t *values);
/* just_set over every voxel of a dense grid laid out [y][z][x] (utils/common.rs:229-230),
 * elements of the batch's voxel width. */
int vx_batch_set_dense(vx_batch *b, const void *grid);
/* Batch::size (batch.rs:115-123) and Batch::has_patches (batch.rs:126-132). */
int vx_batch_size(const vx_batch *b, uint64_t *out);
int vx_batch_has_patches(const vx_batch *b, int *out);

/* ---- the hot path ---------------------------------------------------------------------- */
/* VoxOpsBatch::apply_batch (voxtree.rs:303-328). *changed mirrors its bool result. */
int vx_apply_batch(vx_interner *it, vx_tree tree, const vx_batch *batch, int *changed);
/* n independent apply_batch calls on distinct trees sharing the interner, in one batched device
 * pass; the result equals applying them one after the other in index order. */
int vx_apply_batches(vx_interner *it, uint32_t n, const vx_tree *trees,
                     const vx_batch *const *batches, uint8_t *changed);
/* Dense-chunk construction: for each i, a Batch filled by just_set from grids[i] (a dense
 * [y][z][x] grid of 2^(3*max_depth) voxels of the interner's width, grids packed back to back)
 * applied to trees[i]. All trees must share one max_depth. `changed` (n bytes) may be NULL.
 * trees/grids/changed live in `mem`. */
int vx_build_dense(vx_interner *it, uint32_t n, const vx_tree *trees, const void *grids,
                   uint8_t *changed, vx_mem mem);
/* Asynchronous form of vx_build_dense for trees that are EMPTY (freshly created, cleared or after
 * vx_interner_reset), all arguments in device memory and every tree of depth max_depth. Both are
 * checked on the device before a chunk is built: a tree of another depth, or one whose root is not
 * EMPTY, is left untouched, its changed flag is 0 and VX_E_INVALID_ARG is reported at the next sync
 * (merging into an existing tree is vx_apply_groups_async's job). No host synchronisation, so the
 * call can be captured in a CUDA graph. */
int vx_build_dense_async(vx_interner *it, uint32_t n, const vx_tree *trees_dev,
                         const void *grids_dev, uint8_t *changed_dev, int max_depth);
/* Batched to_vec (utils/common.rs:158-246): out receives n dense [y][z][x] grids of side 2^d, one
 * per tree, back to back; every tree must have the same depth d. With VX_MEM_DEVICE `out` is device
 * memory (16-byte aligned); with VX_MEM_HOST the grids are produced in pieces of whole 32-row slabs
 * and copied out. HBM-write-bound: one CTA per 32^3 cube expands the cube's subtree in shared memory. */
int vx_trees_to_dense(vx_interner *it, uint32_t n, const vx_tree *trees, void *out, vx_mem mem);
/* Asynchronous form, all arguments in device memory, trees checked on the device (a tree whose
 * depth is not `depth` reports VX_E_INVALID_ARG at the next sync and leaves its grid zero). */
int vx_trees_to_dense_async(vx_interner *it, uint32_t n, const vx_tree *trees_dev, int depth, void *out_dev);
/* Batched VoxOpsRead::get: query i reads tree trees[i] at xyz[3i..3i+2]. found[i] = 0/1,
 * values[i] has the interner's voxel width (uint8_t or uint16_t elements). Out-of-bounds
 * positions report VX_E_OOB (and found = 0). */
int vx_get_many(vx_interner *it, uint64_t n, const vx_tree *trees, const int32_t *xyz,
                uint8_t *found, void *values, vx_mem mem);
int vx_get_many_async(vx_interner *it, uint64_t n, const vx_tree *trees_dev,
                      const int32_t *xyz_dev, uint8_t *found_dev, void *values_dev);

/* Batched apply_batch over compacted touched groups already in device memory (the Batch's non-empty
 * (set, clear) groups, core/batch.rs:39-45). Items: trees_dev[i] with item_flags_dev[i] (bit0: the
 * batch has a fill, bit1: it has patches) and fill_dev[i]; items must be ordered deepest tree first
 * and name distinct trees. Records r: rec_item_dev[r] (item index), rec_group_dev[r] (bottom-group
 * Morton index, path >> 3), set/clear masks and 8 values (16-bit elements), ordered by (item, group).
 * changed_dev (n_items bytes) may be NULL. Equivalent to vx_apply_batches; no host synchronisation. */
int vx_apply_groups_async(vx_interner *it, uint32_t n_items, const vx_tree *trees_dev,
                          const uint8_t *item_flags_dev, const uint32_t *fill_dev, uint32_t n_records,
                          const uint32_t *rec_item_dev, const uint32_t *rec_group_dev,
                          const uint8_t *rec_set_dev, const uint8_t *rec_clear_dev,
                          const uint16_t *rec_values_dev, uint8_t *changed_dev, int max_depth);
/* Batched VoxOpsWrite::set (voxtree.rs:163-260 with set_at_depth_iterative and remove_at_depth,
 * voxtree.rs:373-705): the same result as calling vx_tree_set(trees[k], xyz[3k..3k+2], values[k])
 * for k = 0 .. n-1 in order (value 0 removes the voxel; the DAG, reference counts and live nodes are
 * those of the one-by-one calls), in one device pass: the calls of one tree run in order, one warp
 * per tree, trees in parallel; refcounts are settled and the replaced nodes released at the end, so
 * the calls need up to depth + 1 free nodes each until then (VX_E_OOM otherwise). changed[k] (may be
 * NULL) mirrors call k's bool result. Every position is checked first (VX_E_OOB, nothing applied). */
int vx_trees_set_many(vx_interner *it, uint64_t n, const vx_tree *trees, const int32_t *xyz,
                      const uint32_t *values, uint8_t *changed);
/* Launch shape of the batched-apply kernels (threads per block, blocks per SM); chosen by the
 * autotuner in voxelis_gb300/tune.py. */
int vx_tune_set(vx_interner *it, int apply_threads, int apply_blocks_per_sm);
int vx_tune_get(vx_interner *it, int *apply_threads, int *apply_blocks_per_sm);
/* How a batched apply is launched (no counterpart in the reference; autotuned): 1 (the default) runs
 * the whole apply, its level passes and the release of the replaced roots as one cooperative launch
 * whose phases meet at grid barriers (blocks per SM capped by what can be resident); 0 launches one
 * kernel per phase. Results are identical. */
int vx_tune_set_launch(vx_interner *it, int single_launch);
int vx_tune_get_launch(vx_interner *it, int *single_launch);
/* Geometry of the dense builds' quad memo (no counterpart in the reference; autotuned): about the
 * call's quads >> memo_shift slots (0..8, default 2), half as many records. Results are identical;
 * the branch table's load factor is chosen at vx_interner_create (table_log2). */
int vx_tune_set_dense(vx_interner *it, int memo_shift);
int vx_tune_get_dense(vx_interner *it, int *memo_shift);

/* ---- world helpers for serving (no counterpart in the reference) ---------------------------- */
/* A grid of nx x ny x nz chunks of depth chunk_depth; the chunk holding world voxel (x, y, z) is
 * ((y >> d) * nz + (z >> d)) * nx + (x >> d), whose tree handle is trees_dev[chunk] (device memory). */
typedef struct {
    int32_t nx, ny, nz;
    int32_t chunk_depth;
    const vx_tree *trees_dev;
} vx_world;
/* Sphere brushes (integer voxels with |p - center|^2 <= radius^2, clipped to the world) applied in
 * order as Batch::just_set calls (core/batch.rs:145-172) into one Batch per touched chunk, emitted as
 * compacted touched groups sorted by (chunk, group): item_chunks[i] is the chunk of item i, and the
 * record arrays are those of vx_apply_groups_async. Host memory. VX_E_BUFFER reports the sizes. */
int vx_stage_spheres(int chunk_depth, int32_t nx, int32_t ny, int32_t nz, uint32_t n, const int32_t *centers,
                     const int32_t *radii, const uint32_t *values, uint64_t cap_items, uint32_t *item_chunks,
                     uint64_t cap_records, uint32_t *rec_item, uint32_t *rec_group, uint8_t *rec_set,
                     uint8_t *rec_clear, uint16_t *rec_vals, uint64_t *n_items, uint64_t *n_records);
/* n host -> device copies (dst_dev[k] <- src_host[k], bytes[k]) on the interner's stream, one
 * cudaMemcpyAsync each: a serving loop stages a wave's arrays with one call. No reference
 * counterpart (host plumbing of the serving loop). */
int vx_copy_to_device_async(vx_interner *it, uint32_t n, void *const *dst_dev, const void *const *src_host,
                            const uint64_t *bytes);
/* Batched VoxOpsRead::get at world coordinates (world_xyz_dev[3i..3i+2]) over a vx_world. */
int vx_world_get_async(vx_interner *it, const vx_world *world, uint64_t n, const int32_t *world_xyz_dev,
                       uint8_t *found_dev, void *values_dev);

/* Snapshot reads for serving waves that mix edits and gets (no counterpart in the reference; built
 * on VoxInterner::inc_ref and dec_ref_recursive, interner/mod.rs:235-260 and 419-534). Before a wave's
 * apply, vx_world_hold_async takes one more reference on the current root of each of the n listed
 * chunks (their ids go to held_dev[k] and old_roots_dev[chunk]) and records ranks_dev[k], the
 * position of the wave's edit of that chunk, in edit_rank_dev[chunk]. old_roots_dev and
 * edit_rank_dev are world-sized device arrays of the caller; edit_rank_dev starts as 0xFFFFFFFF for
 * every chunk. vx_world_get_at_async is vx_world_get_async except that a chunk whose edit rank is
 * `cut` or more is read at its held root: a get issued with cut = the number of the wave's edits
 * that precede it sees exactly those edits. After the wave's gets, vx_world_release_async resets
 * the ranks of the listed chunks to 0xFFFFFFFF and releases the held roots (a root the apply
 * replaced is freed then). */
int vx_world_hold_async(vx_interner *it, const vx_world *world, uint32_t n, const uint32_t *chunks_dev,
                        const uint32_t *ranks_dev, uint64_t *held_dev, uint64_t *old_roots_dev, uint32_t *edit_rank_dev);
int vx_world_get_at_async(vx_interner *it, const vx_world *world, uint64_t n, const int32_t *world_xyz_dev,
                          uint8_t *found_dev, void *values_dev, const uint64_t *old_roots_dev,
                          const uint32_t *edit_rank_dev, uint32_t cut);
int vx_world_release_async(vx_interner *it, const vx_world *world, uint32_t n, const uint32_t *chunks_dev,
                           uint64_t *held_dev, uint32_t *edit_rank_dev);

/* Occupancy masks for greedy meshing (generate_occupancy_masks + fill_masks_for_region,
 * utils/mesh.rs:418-597; OccupancyDataBuilder, mesh.rs:181-193): the non-default voxels of n_trees
 * trees of one MaxDepth d (1..6) placed into one 64^3 builder, tree k at voxel offset
 * offsets[3k..3k+2] (x, y, z), each within 0..64-2^d. Host outputs:
 *   global[3 * 4096]  planes YZ ([y][z] -> bits of x), XZ ([z][x] -> bits of y), XY ([y][x] -> bits of z)
 *   active[6]         occupied y, z (YZ rows/cols), z, x (XZ), y, x (XY)
 *   n_materials       distinct material ids (voxel values) present
 *   material_ids[k], material_counts[k] (voxels), material_masks[k][3 * 4096] for k < max_materials,
 *                     in ascending material order (the builder's HashMaps, ordered)
 * VX_E_BUFFER (with *n_materials set) when more materials are present than max_materials. */
int vx_occupancy_masks(vx_interner *it, uint32_t n_trees, const vx_tree *trees, const uint32_t *offsets,
                       uint64_t *global, uint64_t *active, uint32_t max_materials, uint32_t *n_materials,
                       uint32_t *material_ids, uint64_t *material_counts, uint64_t *material_masks);

/* Batched, asynchronous form of vx_occupancy_masks for 8-bit voxels, all arguments in device
 * memory: tree t goes to builder builder_of[t] at offsets[3t..3t+2]; every tree has MaxDepth
 * max_depth. Outputs are indexed by builder b: global[b][3 * 4096], active[b][6], n_materials[b],
 * material_ids[b][max_materials], material_counts[b][max_materials],
 * material_masks[b][max_materials][3 * 4096] (materials beyond max_materials are counted in
 * n_materials[b] but not stored). A tree outside its builder or a builder index >= n_builders
 * reports VX_E_OOB at the next sync. */
int vx_occupancy_masks_async(vx_interner *it, uint32_t n_builders, uint32_t n_trees, const vx_tree *trees_dev,
                             const uint32_t *builder_of_dev, const uint32_t *offsets_dev, int max_depth,
                             uint32_t max_materials, uint64_t *global_dev, uint64_t *active_dev,
                             uint32_t *n_materials_dev, uint32_t *material_ids_dev, uint64_t *material_counts_dev,
                             uint64_t *material_masks_dev);

/* Model serialisation (VoxModel::serialize, world/voxmodel.rs:177-282, with serialize_chunk,
 * world/voxchunk.rs:382-405, for each chunk): the interner's live leaves and branches renumbered in
 * slot-index order (leaves 1..L, then branches), written as
 *   u32 L, L x (varint id, value), u32 B, B x (varint id, u8 mask, varint child ids, LOD value),
 *   u32 n_chunks, n_chunks x ("VoxTreeChunk", i32 x, y, z, varint root id)
 * (u32/i32/values big-endian, varints LEB128), chunk k = trees[k] at positions[3k..3k+2] in the given
 * order. This is the payload of a VTM file; the file header, MD5 and zstd stage of
 * export_model_to_vtm (io/export.rs:90-151) are not included. With out == NULL only *size is set;
 * VX_E_BUFFER when capacity < *size. */
int vx_serialize_model(vx_interner *it, uint32_t n_chunks, const vx_tree *trees, const int32_t *positions,
                       uint8_t *out, uint64_t capacity, uint64_t *size);

/* Model deserialisation (VoxModel::deserialize, world/voxmodel.rs:284-408, with deserialize_leaf /
 * preallocate_branch_id / deserialize_branch, interner/mod.rs:930-993, and deserialize_chunk,
 * world/voxchunk.rs:408-440) of the payload vx_serialize_model writes, parsed on the device. Record ids
 * are slots: leaf k lands on slot k, branch L+k on slot L+k, with generation 0. Refcounts are the
 * reference's: one per child slot naming a node (inc_all_child_refs), plus one per chunk root
 * (set_root_id; an EMPTY root counts on the EMPTY slot). Both hash tables hold every pattern. One
 * tree of depth max_depth is created per chunk record, in stream order: out_trees[k] at
 * out_positions[3k..3k+2] (x, y, z); repeated positions give one tree each.
 * VX_E_REF_PANIC where the reference panics: a stream that ends early, an id out of sequence or
 * naming no node, a branch with an empty mask, a zero-valued leaf (a debug assertion there), the
 * wrong chunk magic, or records while the interner already holds nodes (its ids must be the next
 * indices allocated). The interner is left unchanged then. VX_E_OOM when L + B nodes exceed the
 * capacity. VX_E_BUFFER when the stream holds more than max_chunks chunks; *out_n_chunks is set and
 * nothing is created. Host memory; streams below 4 GiB. */
int vx_deserialize_model(vx_interner *it, const uint8_t *data, uint64_t n_bytes, int max_depth, uint32_t max_chunks,
                         vx_tree *out_trees, int32_t *out_positions, uint32_t *out_n_chunks);

/* ---- verification helpers (not on the timed path) ---------------------------------------- */
/* Canonical DFS export of the DAG reachable from `trees` (see vx_canonical). On VX_E_BUFFER
 * *n_nodes holds the required capacity. */
int vx_export_canonical(vx_interner *it, uint32_t n_trees, const vx_tree *trees,
                        vx_canonical *out, uint64_t *n_nodes);
/* to_vec (utils/common.rs:158-246): dense [y][z][x] grid of the tree, voxel-width elements
 * (computed on the device, copied to out_grid in host memory). */
int vx_tree_to_dense(vx_interner *it, vx_tree tree, void *out_grid);
/* Checks every child reachable from the given trees: generation matches its slot and the
 * refcount is positive. VX_E_REF_UB when a dangling child is found. */
int vx_validate(vx_interner *it, uint32_t n_trees, const vx_tree *trees);

/* ---- instrumentation and maintenance (no counterpart in the reference) ------------------- */
/* Phases timed with CUDA events on the interner's stream while profiling is enabled. */
#define VX_PROF_DENSE 0    /* fused dense-chunk kernel (blocks of up to 32^3 voxels)          */
#define VX_PROF_LEVELS 1   /* fresh levels above 32^3 blocks (depth > 5)                       */
#define VX_PROF_REFCOUNT 2 /* end-of-epoch refcount pass and allocator update                  */
#define VX_PROF_APPLY 3    /* batched apply: level passes and root commit                      */
#define VX_PROF_RELEASE 4  /* breadth-first release of replaced roots                          */
#define VX_PROF_GET 5      /* batched gets                                                     */
#define VX_PROF_COPY 6     /* host<->device copies made inside an entry point                  */
#define VX_PROF_BOTTOM 7   /* batched apply: the bottom-group kernel alone (part of APPLY's work) */
#define VX_PROF_N 8
int vx_profile_enable(vx_interner *it, int on);
/* Waits for the stream and returns, per phase, the summed milliseconds and the number of timed
 * intervals since the last collect; then starts a new collection. */
int vx_profile_collect(vx_interner *it, double *ms, uint64_t *count);
/* Number of kernels this library has launched in this process. */
uint64_t vx_kernel_launches(void);
/* Dense-chunk construction that allocates no memory (no counterpart in the reference).
 * Same arguments and result as vx_build_dense_async, for callers that cannot allocate device memory
 * during the call: code recorded into a CUDA graph (allocation is not allowed during stream
 * capture), frame loops and servers that fix their memory up front, hosts whose allocator belongs
 * to another runtime. The levels above the 32^3 blocks (depth d >= 6) are staged in a fixed device
 * array of VX_NOALLOC_SCRATCH_BYTES compiled into the library (held by every GPU until exit): a call
 * needs 12 n (8 + ... + 8^(d-5)) + 4 n (1 + ... + 8^(d-6)) bytes, rounded up to 256, plus 256 (about
 * 100 bytes a chunk at depth 6, so some 31,000 chunks; depths 2-5 need no staging), and larger
 * requests return VX_E_BUFFER without queuing work. All calls share the array: calls whose device
 * work overlaps race, so serialise them. The first call on a device resolves the array's address
 * and must come before any stream capture. */
#define VX_NOALLOC_SCRATCH_BYTES (3u << 20)
int vx_build_dense_noalloc(vx_interner *it, uint32_t n, const vx_tree *trees_dev,
                           const void *grids_dev, uint8_t *changed_dev, int max_depth);
/* Waits for the stream, reports the sticky status, and rebuilds the branch table when deleted slots
 * exceed a quarter of it (the synchronous entry points do this themselves). */
int vx_interner_maintain(vx_interner *it);
/* Returns the interner to its freshly created state (no nodes, empty tables, every slot's
 * generation back to 0); tree handles stay valid and their roots become EMPTY. Same result as
 * destroying it and creating a new interner with the same budget, without reallocating device
 * memory. */
int vx_interner_reset(vx_interner *it);

#ifdef __cplusplus
}
#endif
#endif /* VOXELIS_GB300_H */
