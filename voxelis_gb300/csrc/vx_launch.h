// Host-side launchers of the device kernels (one declaration per kernel family).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "vx_device.cuh"

namespace vxg {

#ifndef VX_PDL
#define VX_PDL 1  // kernels after the first of a sequence launch early (programmatic dependent launch)
#endif
// Launches `kernel` with programmatic stream serialization: it may start while the previous kernel of
// the stream finishes and waits for it in pdl_wait().
template <typename... KArgs, typename... Args>
inline cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                              Args... args) {
    if (!VX_PDL) {
        kernel<<<grid, block, smem, s>>>(args...);
        return cudaGetLastError();
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

// Process-wide count of kernels launched by this library (reported by vx_kernel_launches).
void count_launches(uint64_t n);

// ---- dense-chunk construction on EMPTY trees (vx_build.cu) -----------------------------------
struct DenseArgs {
    const void *grids;           // n_chunks * side^3 voxels, [y][z][x] per chunk
    const uint32_t *trees;       // tree handle per chunk
    uint32_t n_chunks;
    int depth;                   // chunk depth d (2..3)
    uint8_t *changed;            // [n_chunks] or null
};
// Builds whole chunks of depth 2 or 3, one CTA per chunk (staged in shared memory by one bulk copy).
cudaError_t launch_dense_blocks(const DevInterner &I, const DenseArgs &a, int num_sms, cudaStream_t s);

// Fused dense construction for chunk depths 4..10: a warp per 16^3 octant at depth 4, a CTA per
// 32^3 block at depths 5-10 (TMA tensor copies); levels above those units are reduced by the
// last-arriving warp or CTA of each parent. `scratch` must hold dense_octant_scratch_bytes(n, depth)
// bytes (the layout the launch carves); its arrival counts are cleared inside.
// `memo` (optional, dense_octant_memo_bytes) holds the quad memo; it is cleared inside unless
// clear_memo is false (later pieces of one build share the memo of the first: no release runs in
// between, so every node it names is still alive). memo_chunks (0: n_chunks) sizes the memo and must
// be the same for every piece that shares it.
size_t dense_octant_scratch_bytes(uint64_t n_chunks, int depth);
size_t dense_octant_memo_bytes(uint64_t n_chunks, int depth, int vbits, uint32_t memo_shift);
cudaError_t launch_dense_octants(const DevInterner &I, const void *grids, const uint32_t *trees, uint32_t n_chunks,
                                 int depth, uint8_t *changed, void *scratch, int num_sms, cudaStream_t s,
                                 void *memo = nullptr, bool clear_memo = true, uint64_t memo_chunks = 0);
// Dense construction for chunk depths 5..10 in passes: a quad kernel over 32^3 blocks, then one
// fresh_level pass per level above the quads. `scratch` must hold dense_split_scratch_bytes.
// levels_begin(levels_ctx), when given, runs on the host between the quad launch and the level
// launches (the profiler marks its phases there).
size_t dense_split_scratch_bytes(uint64_t n_chunks, int depth);
cudaError_t launch_dense_split(const DevInterner &I, const void *grids, const uint32_t *trees, uint32_t n_chunks,
                               int depth, uint8_t *changed, void *scratch, int num_sms, cudaStream_t s, void *memo,
                               bool clear_memo = true, uint64_t memo_chunks = 0,
                               void (*levels_begin)(void *) = nullptr, void *levels_ctx = nullptr,
                               bool count_refs = false);
// In-degree refcounts of the nodes created in the current epoch, then closes the epoch.
cudaError_t launch_epoch_refcounts(const DevInterner &I, int num_sms, cudaStream_t s);
// Whether launch_dense_split, asked to (count_refs), counts references as it creates nodes and closes
// the epoch itself; otherwise the caller runs launch_epoch_refcounts after it.
bool dense_split_counts_refs(const DevInterner &I);
cudaError_t launch_epoch_finalize(const DevInterner &I, cudaStream_t s);

// rec_item[r] = i for the records [first[i], first[i+1]) of every item i < n (device memory).
cudaError_t launch_expand_items(const uint32_t *first, uint32_t n, uint32_t *rec_item, cudaStream_t s);


// ---- general batch apply (vx_apply.cu) ---------------------------------------------------------
struct ApplyArgs {
    int mode;                    // 0: set phase (set_batch_at_depth_iterative); 1: clear pass (P4)
    int threads;                 // launch shape of the bottom/parents kernels
    int blocks_per_sm;
    uint32_t n_items;
    uint32_t n_records;
    int max_depth;
    // items (ordered by depth, deepest first)
    const uint32_t *it_tree;
    const uint8_t *it_depth;
    const uint8_t *it_flags;     // bit0 has_fill, bit1 has_patches
    const uint32_t *it_fill;
    uint64_t *it_init;           // scratch
    uint64_t *it_old;
    uint64_t *it_new;
    uint8_t *it_panic;
    uint8_t *it_changed;         // result
    // records sorted by (item, group)
    const uint32_t *rec_item;
    const uint32_t *rec_group;
    const uint8_t *rec_set;
    const uint8_t *rec_clear;
    const uint16_t *rec_vals;    // [n_records * 8]
    // scratch
    uint32_t *flags;             // [n_records + 1]
    uint32_t *pos;               // [n_records + 1]
    uint32_t *scan_tmp;          // block sums
    unsigned long long *scan_status;  // [kScanStatusTiles] look-back words of one-pass scans (all 0 between scans)
    uint32_t *e_item[2];
    uint32_t *e_path[2];
    uint64_t *e_id[2];
    uint32_t *e_val[2];
    uint32_t *p_start;           // [n_records + 1]
    uint32_t *it_first;           // [n_items + 1] first record of each item (host staging of an apply)
    uint64_t *rec_id;
    uint32_t *rec_val;
    uint64_t *release_list;      // [n_items]
};
cudaError_t launch_apply(const DevInterner &I, const ApplyArgs &a, int num_sms, cudaStream_t s);
// The same sequence (with the item depth check when check_depths, the clear pass when clear_pass and
// the release of the replaced roots in `rounds` rounds) as one cooperative launch: every CTA
// resident, phases separated by grid barriers. a.scan_tmp must hold apply_single_scan_words words.
cudaError_t launch_apply_single(const DevInterner &I, const ApplyArgs &a, bool check_depths, bool clear_pass,
                                uint32_t *frontier_a, uint32_t *frontier_b, int rounds, int num_sms, cudaStream_t s);
size_t apply_single_scan_words(int num_sms);
// The same sequence in two parts: items + bottom groups, then the level passes and the commit.
cudaError_t launch_apply_bottom(const DevInterner &I, const ApplyArgs &a, int num_sms, cudaStream_t s);
cudaError_t launch_apply_levels(const DevInterner &I, const ApplyArgs &a, int num_sms, cudaStream_t s);
// Fills it_depth from the tree table and checks the deepest-first order (device-resident inputs).
cudaError_t launch_item_depths(const DevInterner &I, const ApplyArgs &a, cudaStream_t s);
// Counter slots used by launch_apply (DevCounters::scratch indices).
enum : int {
    SC_ENTRIES = 0, SC_PARENTS = 1, SC_ROOTS = 2, SC_RELEASE = 3, SC_REL_IN = 4, SC_REL_OUT = 5, SC_REF_DONE = 6,
    SC_DONE = 7, SC_SCAN_TICKET = 8, SC_SCAN_DONE = 9
};
static_assert(SC_RELEASE == kScRelease && SC_REL_IN == kScRelIn && SC_REL_OUT == kScRelOut,
              "release slots shared with vx_device.cuh");
// Tiles of a one-pass device scan with a status word each (ApplyArgs::scan_status, zero between
// scans: the scan's last CTA clears them); larger scans take the three-launch path.
constexpr uint32_t kScanStatusTiles = 64;

// Inclusive-to-exclusive scan of n u32 flags (n from the host) into pos; pos[n] = total.
cudaError_t launch_scan(const uint32_t *flags, uint32_t *pos, uint32_t *tmp, uint32_t n, cudaStream_t s);
// Block sums of one scan level; `tmp` must hold 4 x scan_tmp_words(n) words for the recursion.
size_t scan_tmp_words(uint32_t n);

// ---- reads, releases, single-voxel operations, maintenance (vx_ops.cu) -------------------------
cudaError_t launch_get_many(const DevInterner &I, uint64_t n, const uint32_t *trees, const int32_t *xyz,
                            uint8_t *found, void *values, int num_sms, cudaStream_t s);
// to_vec over trees of depth d into [y][z][x] grids: cubes [cube_begin, cube_begin + n_cubes) of side
// min(32, 2^d), ordered (tree, cy, cz, cx); cube_begin must start a cy-slab and `out` points at that
// slab's first element.
size_t to_dense_smem_bytes(int d, int vbits);
cudaError_t launch_to_dense(const DevInterner &I, const uint32_t *trees, int d, uint64_t cube_begin,
                            uint64_t n_cubes, void *out, int num_sms, cudaStream_t s);
// Occupancy masks of n_trees dense grids of side 2^d placed at offsets (x, y, z) of a 64^3 builder:
// counts[2^bits] and global/per_mat/active must be zero on entry; slot/ids/mcounts/n_mat are written.
cudaError_t launch_occupancy(const DevInterner &I, const void *grids, uint32_t n_trees, int d, const uint32_t *offsets,
                             unsigned long long *counts, uint32_t *slot, uint32_t *ids, unsigned long long *mcounts,
                             uint32_t *n_mat, uint32_t mat_cap, unsigned long long *global, unsigned long long *per_mat,
                             unsigned long long *active, int num_sms, cudaStream_t s);
// Batched occupancy masks, 8-bit voxels: tree t goes to builder builder_of[t]; counts (256 per
// builder), global, per_mat must be zero on entry.
cudaError_t launch_occupancy_many(const DevInterner &I, const uint8_t *grids, uint32_t n_trees, int d,
                                  const uint32_t *builder_of, const uint32_t *offsets, uint32_t n_builders,
                                  unsigned int *counts, uint32_t *slot, uint32_t max_mat, uint32_t *ids,
                                  unsigned long long *mcounts, uint32_t *n_mat, unsigned long long *global,
                                  unsigned long long *per_mat, unsigned long long *active, int num_sms, cudaStream_t s);
// Model serialisation: plan (renumbering, record sizes, offsets, total bytes into *total), then
// write (records, counts and chunk records into `out`, which holds *total bytes). `w` holds
// serialize_scratch_words(I) u32 and is shared by both steps.
size_t serialize_scratch_words(const DevInterner &I);
cudaError_t launch_serialize_plan(const DevInterner &I, uint32_t *w, uint32_t *tmp_scan, uint32_t n_chunks,
                                  const uint32_t *trees, unsigned long long *total, int num_sms, cudaStream_t s);
cudaError_t launch_serialize_write(const DevInterner &I, uint32_t *w, uint32_t n_chunks, const uint32_t *trees,
                                   const int32_t *pos, uint8_t *out, unsigned long long *total, int num_sms,
                                   cudaStream_t s);

// ---- model deserialisation (vx_vtm.cu) -------------------------------------------------------
// Section state of one parse, in device memory: sections 0 leaves, 1 branches, 2 chunks. The host
// sets start[0] = 4 and count[0] = the leaf count, start[1..3] = ~0 (unknown), the other counts and
// done[] = 0; each section's last record sets the next section's start and count and done[kind].
struct VtmSections {
    unsigned long long start[4];  // first byte of section k's records; start[3] = end of the chunks
    unsigned long long count[3];  // records announced by section k's header
    unsigned long long done[3];   // 1 once section k's last record was found
};
struct VtmScratchSizes {
    uint32_t seg_bytes;
    uint64_t n0, n1, n2;                     // tables per level (upper bounds)
    uint64_t table_words, entry_words;       // u64 words of the tables and the entry states
    uint64_t leaf_cap, branch_cap, chunk_cap;  // u32 record offsets per section (upper bounds)
};
uint32_t vtm_segment_bytes(uint64_t n_bytes);
VtmScratchSizes vtm_scratch_sizes(uint64_t n_bytes);
// Parses the three sections of `bytes` (device memory, n_bytes < 2^32): record offsets by rank into
// leaf_off / branch_off / chunk_off, counts into sec. A stream the reference panics on sets
// ERR_REF_PANIC and leaves done[] of the failing section 0.
cudaError_t launch_vtm_parse(const DevInterner &I, const uint8_t *bytes, uint64_t n_bytes, VtmSections *sec,
                             uint64_t *tables, uint64_t *entries, uint32_t *leaf_off, uint32_t *branch_off,
                             uint32_t *chunk_off, int num_sms, cudaStream_t s);
// Writes the parsed nodes into an interner that holds none (slots 1..L+B), the branch table, the
// refcounts and the roots of trees[k] (k < C), with the chunk positions into positions[3k..3k+2].
cudaError_t launch_vtm_place(const DevInterner &I, const uint8_t *bytes, const VtmSections *sec, uint64_t n_nodes,
                             uint64_t n_links, const uint32_t *leaf_off, const uint32_t *branch_off,
                             const uint32_t *chunk_off, const uint32_t *trees, int32_t *positions, int num_sms,
                             cudaStream_t s);
// Releases the roots listed in `list` (count at ctr->scratch[SC_RELEASE]) with `rounds`
// breadth-first rounds, using two frontier buffers of `frontier_cap` entries.
cudaError_t launch_release(const DevInterner &I, uint64_t *list, uint32_t *frontier_a, uint32_t *frontier_b,
                           uint64_t frontier_cap, int rounds, int num_sms, cudaStream_t s);
// Single-voxel VoxTree::set / fill / clear executed by one thread with the reference's own
// refcount order; the result status word is written to *status_out.
cudaError_t launch_tree_set(const DevInterner &I, uint32_t tree, int32_t x, int32_t y, int32_t z, uint32_t v,
                            uint64_t *queue, uint64_t queue_cap, int *status_out, cudaStream_t s);
// Many VoxTree::set calls (vx_trees_set_many): group g = the calls of tree group_tree[g], at
// [begin[g], begin[g+1]) of xyz / values in call order; order[k] = the call's index for changed[].
struct SetCalls {
    uint32_t n_groups;
    const uint32_t *group_tree;
    const uint32_t *begin;
    const int32_t *xyz;
    const uint32_t *values;
    const uint32_t *order;
    uint8_t *changed;    // per call, may be null
    uint64_t *new_root;  // per group (scratch)
};
// Runs the calls (one warp per tree), counts the created nodes' references, moves the roots and
// releases the first roots and the created nodes left unreferenced. fc0 / ni0: the interner's
// free_count and next_index before the call; `list` holds n_groups + every node the calls can create.
cudaError_t launch_trees_set(const DevInterner &I, const SetCalls &c, uint64_t *list, unsigned long long fc0,
                             unsigned long long ni0, uint32_t *frontier_a, uint32_t *frontier_b, int max_depth,
                             int num_sms, cudaStream_t s);
cudaError_t launch_tree_fill(const DevInterner &I, uint32_t tree, uint32_t v, uint64_t *queue,
                             uint64_t queue_cap, int *status_out, cudaStream_t s);
cudaError_t launch_rehash(const DevInterner &I, uint64_t table_slots, int num_sms, cudaStream_t s);
cudaError_t launch_count_live(const DevInterner &I, unsigned long long *out2, int num_sms, cudaStream_t s);

}  // namespace vxg
