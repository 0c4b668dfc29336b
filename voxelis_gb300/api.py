"""Host-side mirror of voxelis' VoxInterner / VoxTree / Batch API over the C ABI.

The classes keep the reference's names, argument meaning and results so that code written against
voxelis reads the same here:

    interner = VoxInterner.with_memory_budget(256 << 20)           # interner/mod.rs:45
    tree = VoxTree(5)                                               # voxtree.rs:116 (MaxDepth 5)
    batch = tree.create_batch()                                     # voxtree.rs:296
    batch.set(interner, (x, y, z), 3)                               # batch.rs:206-208
    tree.apply_batch(interner, batch)   -> bool                     # voxtree.rs:303-328
    tree.get(interner, (x, y, z))       -> value or None            # voxtree.rs:145-159

Errors: the reference panics where these raise `ReferencePanic` (bounds, depth cap, out of
memory, assert!) and has undefined behaviour where these raise `ReferenceUB`.

All classes run on the GPU library by default; `lib=` selects another library exposing the same
C ABI.
"""
import ctypes as C

import numpy as np

from . import _abi
from ._abi import VX_MEM_DEVICE, VX_MEM_HOST


def _pos(p):
    x, y, z = (int(v) for v in p)
    return x, y, z


def _np_ptr(a):
    return C.c_void_p(a.ctypes.data) if a is not None else None


def export_canonical(lib, handle, tree_handles):
    """Canonical DFS export (vx_export_canonical) of the DAG reachable from the trees with the given
    handles of the interner `handle` in library `lib`: a dict of numpy arrays (kind, types, mask,
    value, refcount, children [n, 8], roots). Two interners holding the same DAG give equal arrays
    whatever their allocation order."""
    handles = np.ascontiguousarray(tree_handles, dtype=np.uint32)
    n_nodes = C.c_uint64()
    lib.call("export_canonical", handle, len(handles), _np_ptr(handles), None, C.byref(n_nodes), handle=handle)
    n = n_nodes.value
    arrays = {
        "kind": np.zeros(n, np.uint8), "types": np.zeros(n, np.uint8),
        "mask": np.zeros(n, np.uint8), "value": np.zeros(n, np.uint32),
        "refcount": np.zeros(n, np.uint32), "children": np.zeros((n, 8), np.int32),
        "roots": np.zeros(len(handles), np.int32),
    }
    c = _abi.vx_canonical()
    for k in ("kind", "types", "mask"):
        setattr(c, k, arrays[k].ctypes.data_as(C.POINTER(C.c_uint8)))
    for k in ("value", "refcount"):
        setattr(c, k, arrays[k].ctypes.data_as(C.POINTER(C.c_uint32)))
    for k in ("children", "roots"):
        setattr(c, k, arrays[k].ctypes.data_as(C.POINTER(C.c_int32)))
    c.capacity = n
    lib.call("export_canonical", handle, len(handles), _np_ptr(handles), C.byref(c), C.byref(n_nodes), handle=handle)
    return arrays


def level_counts(canon):
    """collect_stats (utils/common.rs:302-333) over a canonical export: the number of nodes at each
    depth counted with tree multiplicity (a DAG node reached by k paths counts k times). Returns a
    list, index = depth below the roots."""
    n = len(canon["kind"])
    children = np.asarray(canon["children"]).reshape(n, 8)
    roots = np.asarray(canon["roots"])
    # multiplicity of every node at the current depth (dense over node ids; exact in float64 below
    # 2^53 paths)
    mult = np.bincount(roots[roots >= 0], minlength=n).astype(np.float64)
    out = []
    while True:
        nodes = np.flatnonzero(mult)
        if not len(nodes):
            return out
        out.append(int(mult[nodes].sum()))
        ch = children[nodes]                      # [m, 8], -1 for EMPTY (and every leaf slot)
        keep = ch >= 0
        mult = np.bincount(ch[keep], weights=np.repeat(mult[nodes], keep.sum(axis=1)), minlength=n)


def same_dag(a, b):
    """True when two canonical exports are identical in every array."""
    return a.keys() == b.keys() and all(np.array_equal(a[k], b[k]) for k in a)


class VoxInterner:
    """VoxInterner<T> (interner/mod.rs:25-40): the hash-consed node store, resident on the device."""

    def __init__(self, budget_bytes, voxel_bits=8, patches=0, table_log2=0, lib=None):
        self.lib = lib if lib is not None else _abi.gpu_lib()
        self.voxel_bits = int(voxel_bits)
        self.patches = int(patches)
        self.dtype = np.uint8 if self.voxel_bits == 8 else np.uint16
        h = C.c_void_p()
        st = self.lib.status("interner_create", C.c_uint64(int(budget_bytes)), self.voxel_bits,
                             self.patches, int(table_log2), C.byref(h))
        if st != _abi.VX_OK:
            raise _abi.error_for(st, "interner_create")
        self.handle = h

    @classmethod
    def with_memory_budget(cls, budget_bytes, voxel_bits=8, patches=0, lib=None):
        """VoxInterner::<T>::with_memory_budget (interner/mod.rs:45)."""
        return cls(budget_bytes, voxel_bits=voxel_bits, patches=patches, lib=lib)

    def close(self):
        if self.handle:
            self.lib.status("interner_destroy", self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _call(self, name, *args):
        return self.lib.call(name, self.handle, *args, handle=self.handle)

    def get_ref(self, block_id):
        """VoxInterner::get_ref (interner/mod.rs:222-233)."""
        out = C.c_uint32()
        self._call("get_ref", C.c_uint64(int(block_id)), C.byref(out))
        return out.value

    def get_value(self, block_id):
        out = C.c_uint32()
        self._call("get_value", C.c_uint64(int(block_id)), C.byref(out))
        return out.value

    def stats(self):
        s = _abi.vx_interner_stats()
        self._call("interner_stats_get", C.byref(s))
        return {name: getattr(s, name) for name, _ in s._fields_}

    def capacity(self):
        return self.stats()["capacity"]

    def sync(self):
        if self.lib.has("interner_sync"):
            self._call("interner_sync")

    def set_stream(self, cuda_stream_handle):
        """Orders this interner's device work on a caller stream (a cudaStream_t as int)."""
        self._call("interner_set_stream", C.c_void_p(int(cuda_stream_handle) or None))

    # ---- batched entry points ---------------------------------------------------------------
    def build_dense(self, trees, grids, mem=VX_MEM_HOST, changed=True):
        """Dense-chunk construction for many trees of one depth (see vx_build_dense)."""
        n = len(trees)
        handles = np.ascontiguousarray([t._bind(self) for t in trees], dtype=np.uint32)
        g = np.ascontiguousarray(grids, dtype=self.dtype)
        out = np.zeros(n, dtype=np.uint8) if changed else None
        self._call("build_dense", n, _np_ptr(handles), _np_ptr(g), _np_ptr(out), mem)
        for t, c in zip(trees, (out if out is not None else [1] * n)):
            if c:
                t._dirty = True
        return out

    def get_many(self, trees, xyz):
        """Batched VoxOpsRead::get; returns (found[bool], values)."""
        tr = np.ascontiguousarray(trees, dtype=np.uint32)
        p = np.ascontiguousarray(xyz, dtype=np.int32).reshape(-1, 3)
        n = p.shape[0]
        found = np.zeros(n, dtype=np.uint8)
        vals = np.zeros(n, dtype=self.dtype)
        self._call("get_many", C.c_uint64(n), _np_ptr(tr), _np_ptr(p), _np_ptr(found), _np_ptr(vals),
                   VX_MEM_HOST)
        return found.astype(bool), vals

    def to_vec_many(self, trees):
        """Batched to_vec over trees of one depth: an (n, S, S, S) [y][z][x] array. Uses the GPU
        library's vx_trees_to_dense; on the oracle it is to_vec per tree."""
        if not trees:
            return np.zeros((0, 0, 0, 0), dtype=self.dtype)
        if not self.lib.has("trees_to_dense"):
            return np.stack([t.to_vec(self) for t in trees])
        n = 1 << trees[0].max_depth_value
        handles = np.ascontiguousarray([t._bind(self) for t in trees], dtype=np.uint32)
        out = np.zeros((len(trees), n, n, n), dtype=self.dtype)
        self._call("trees_to_dense", len(trees), _np_ptr(handles), _np_ptr(out), VX_MEM_HOST)
        return out

    def occupancy_masks(self, trees, offsets, max_materials=256):
        """generate_occupancy_masks into one 64^3 builder (utils/mesh.rs:418-597): tree k at voxel
        offset offsets[k] = (x, y, z). Returns dict(global=[3, 64, 64] u64 planes YZ/XZ/XY,
        active=[6] u64, materials={id: (count, [3, 64, 64] u64 masks)})."""
        handles = np.ascontiguousarray([t._bind(self) for t in trees], dtype=np.uint32)
        offs = np.ascontiguousarray(offsets, dtype=np.uint32).reshape(-1, 3)
        glob = np.zeros(3 * 4096, np.uint64)
        active = np.zeros(6, np.uint64)
        n_mat = C.c_uint32()
        ids = np.zeros(max_materials, np.uint32)
        counts = np.zeros(max_materials, np.uint64)
        masks = np.zeros((max_materials, 3 * 4096), np.uint64)
        self._call("occupancy_masks", len(trees), _np_ptr(handles), _np_ptr(offs), _np_ptr(glob), _np_ptr(active),
                   max_materials, C.byref(n_mat), _np_ptr(ids), _np_ptr(counts), _np_ptr(masks))
        k = n_mat.value
        mats = {int(ids[i]): (int(counts[i]), masks[i].reshape(3, 64, 64)) for i in range(k)}
        return {"global": glob.reshape(3, 64, 64), "active": active, "materials": mats}

    def serialize_model(self, trees, positions):
        """VoxModel::serialize payload (world/voxmodel.rs:177-282) for chunks trees[k] at positions[k]."""
        handles = np.ascontiguousarray([t._bind(self) for t in trees], dtype=np.uint32)
        pos = np.ascontiguousarray(positions, dtype=np.int32).reshape(-1, 3)
        size = C.c_uint64()
        self._call("serialize_model", len(trees), _np_ptr(handles), _np_ptr(pos), None, C.c_uint64(0), C.byref(size))
        out = np.zeros(size.value, np.uint8)
        self._call("serialize_model", len(trees), _np_ptr(handles), _np_ptr(pos), _np_ptr(out),
                   C.c_uint64(size.value), C.byref(size))
        return out.tobytes()

    def deserialize_model(self, data, max_depth):
        """VoxModel::deserialize (world/voxmodel.rs:284-408) of a payload into this interner, which
        must hold no nodes yet: returns (trees, positions), one VoxTree of MaxDepth max_depth per chunk
        record in stream order and an int32 [C, 3] array of their positions."""
        buf = np.frombuffer(bytes(data), np.uint8)
        n = C.c_uint32()
        st = self.lib.status("deserialize_model", self.handle, _np_ptr(buf), C.c_uint64(len(buf)), int(max_depth), 0,
                             None, None, C.byref(n))
        if st not in (_abi.VX_OK, _abi.VX_E_BUFFER):
            raise _abi.error_for(st, self.lib.last_error(self.handle))
        handles = np.zeros(max(1, n.value), np.uint32)
        pos = np.zeros((max(1, n.value), 3), np.int32)
        if st == _abi.VX_E_BUFFER:
            self._call("deserialize_model", _np_ptr(buf), C.c_uint64(len(buf)), int(max_depth), n.value,
                       _np_ptr(handles), _np_ptr(pos), C.byref(n))
        trees = []
        for h in handles[:n.value]:
            t = VoxTree(max_depth)
            t.interner, t.tree, t._dirty = self, int(h), True
            trees.append(t)
        return trees, pos[:n.value].copy()

    def apply_batches(self, trees, batches):
        """n apply_batch calls in one batched device pass; returns the changed flags."""
        n = len(trees)
        handles = np.ascontiguousarray([t._bind(self) for t in trees], dtype=np.uint32)
        ptrs = (C.c_void_p * n)(*[b.handle.value for b in batches])
        out = np.zeros(n, dtype=np.uint8)
        self._call("apply_batches", n, _np_ptr(handles), C.cast(ptrs, C.c_void_p), _np_ptr(out))
        for t, c in zip(trees, out):
            if c:
                t._dirty = True
        return out.astype(bool)

    def set_many(self, trees, xyz, values):
        """VoxOpsWrite::set (voxtree.rs:163-260) for call k = (trees[k], xyz[k], values[k]) in order,
        in one batched device pass (vx_trees_set_many); returns each call's bool result."""
        handles = np.ascontiguousarray([t._bind(self) for t in trees], dtype=np.uint32)
        p = np.ascontiguousarray(xyz, dtype=np.int32).reshape(-1, 3)
        v = np.ascontiguousarray(values, dtype=np.uint32).reshape(-1)
        out = np.zeros(len(v), dtype=np.uint8)
        self._call("trees_set_many", C.c_uint64(len(v)), _np_ptr(handles), _np_ptr(p), _np_ptr(v), _np_ptr(out))
        for t, c in zip(trees, out):
            if c:
                t._dirty = True
        return out.astype(bool)

    def export_canonical(self, trees):
        """Canonical DFS export of the DAG reachable from `trees` (see vx_canonical)."""
        handles = np.ascontiguousarray([t._bind(self) for t in trees], dtype=np.uint32)
        return export_canonical(self.lib, self.handle, handles)

    def validate(self, trees):
        handles = np.ascontiguousarray([t._bind(self) for t in trees], dtype=np.uint32)
        self._call("validate", len(trees), _np_ptr(handles))


class Batch:
    """Batch<T> (core/batch.rs:39-240): per-group set/clear masks and values, plus a fill."""

    def __init__(self, max_depth, voxel_bits=8, patches=0, lib=None):
        self.lib = lib if lib is not None else _abi.gpu_lib()
        self.max_depth_value = int(max_depth)
        self.voxel_bits = int(voxel_bits)
        h = C.c_void_p()
        st = self.lib.status("batch_create", self.max_depth_value, self.voxel_bits, int(patches), C.byref(h))
        if st != _abi.VX_OK:
            raise _abi.error_for(st, "batch_create")
        self.handle = h

    def close(self):
        if self.handle:
            self.lib.status("batch_destroy", self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _call(self, name, *args):
        st = self.lib.status(name, self.handle, *args)
        if st != _abi.VX_OK:
            raise _abi.error_for(st, name)

    def just_set(self, position, voxel):
        """Batch::just_set (batch.rs:145-172)."""
        self._call("batch_set", *_pos(position), int(voxel))
        return True

    def set_many(self, xyz, values):
        """just_set for every (position, value) pair in order (last write wins per voxel)."""
        p = np.ascontiguousarray(xyz, dtype=np.int32).reshape(-1, 3)
        v = np.ascontiguousarray(values, dtype=np.uint32).reshape(-1)
        assert p.shape[0] == v.shape[0]
        self._call("batch_set_many", C.c_uint64(p.shape[0]), _np_ptr(p), _np_ptr(v))

    def set(self, interner, position, voxel):
        """VoxOpsWrite for Batch (batch.rs:206-208)."""
        return self.just_set(position, voxel)

    def just_fill(self, value):
        self._call("batch_fill", int(value))

    def fill(self, interner, value):
        self.just_fill(value)

    def just_clear(self):
        self._call("batch_clear")

    def clear(self, interner):
        self.just_clear()

    def set_dense(self, grid):
        """just_set for every voxel of a dense [y][z][x] grid."""
        g = np.ascontiguousarray(grid, dtype=np.uint8 if self.voxel_bits == 8 else np.uint16)
        n = 1 << self.max_depth_value
        assert g.size == n * n * n
        self._call("batch_set_dense", _np_ptr(g))

    def size(self):
        out = C.c_uint64()
        self._call("batch_size", C.byref(out))
        return out.value

    def has_patches(self):
        out = C.c_int()
        self._call("batch_has_patches", C.byref(out))
        return bool(out.value)

    def max_depth(self, lod=0):
        return max(0, self.max_depth_value - int(lod))

    def voxels_per_axis(self, lod=0):
        return 1 << self.max_depth(lod)


class VoxTree:
    """VoxTree<T> (spatial/voxtree.rs:108-1118). The root lives in the interner's device tree table;
    the tree binds to an interner on its first operation, as a VoxTree is only ever used with one."""

    def __init__(self, max_depth):
        self.max_depth_value = int(max_depth)
        self.interner = None
        self.tree = None
        self._dirty = False

    def _bind(self, interner):
        if self.interner is None:
            out = C.c_uint32()
            interner._call("tree_create", self.max_depth_value, C.byref(out))
            self.interner = interner
            self.tree = out.value
        elif self.interner is not interner:
            raise ValueError("a VoxTree is used with one interner")
        return self.tree

    # VoxOpsConfig (voxtree.rs:331-341)
    def max_depth(self, lod=0):
        return max(0, self.max_depth_value - int(lod))

    def voxels_per_axis(self, lod=0):
        return 1 << self.max_depth(lod)

    def get_root_id(self):
        if self.interner is None:
            return _abi.VX_BLOCK_EMPTY
        out = C.c_uint64()
        self.interner._call("tree_root", self.tree, C.byref(out))
        return out.value

    # VoxOpsState (voxtree.rs:343-353)
    def is_empty(self):
        return self.get_root_id() == 0

    def is_leaf(self):
        return (self.get_root_id() >> 63) == 1

    # VoxOpsDirty (voxtree.rs:355-370)
    def is_dirty(self):
        return self._dirty

    def mark_dirty(self):
        self._dirty = True

    def clear_dirty(self):
        self._dirty = False

    def get(self, interner, position):
        """VoxOpsRead::get (voxtree.rs:145-159): the voxel value, or None when empty."""
        t = self._bind(interner)
        found = C.c_int()
        val = C.c_uint32()
        interner._call("tree_get", t, *_pos(position), C.byref(found), C.byref(val))
        return val.value if found.value else None

    def set(self, interner, position, voxel):
        """VoxOpsWrite::set (voxtree.rs:163-260)."""
        t = self._bind(interner)
        changed = C.c_int()
        interner._call("tree_set", t, *_pos(position), int(voxel), C.byref(changed))
        if changed.value:
            self._dirty = True
        return bool(changed.value)

    def fill(self, interner, value):
        """VoxOpsBulkWrite::fill (voxtree.rs:264-277)."""
        t = self._bind(interner)
        before = self.get_root_id()
        interner._call("tree_fill", t, int(value))
        if value != 0 or before != 0:
            self._dirty = True

    def clear(self, interner):
        """VoxOpsBulkWrite::clear (voxtree.rs:279-292)."""
        t = self._bind(interner)
        if self.get_root_id() != 0:
            self._dirty = True
        interner._call("tree_clear", t)

    def create_batch(self, interner=None):
        """VoxOpsBatch::create_batch (voxtree.rs:296-301)."""
        lib = interner.lib if interner is not None else (self.interner.lib if self.interner else None)
        bits = interner.voxel_bits if interner is not None else (self.interner.voxel_bits if self.interner else 8)
        patches = interner.patches if interner is not None else (self.interner.patches if self.interner else 0)
        return Batch(self.max_depth_value, voxel_bits=bits, patches=patches, lib=lib)

    def apply_batch(self, interner, batch):
        """VoxOpsBatch::apply_batch (voxtree.rs:303-328)."""
        t = self._bind(interner)
        changed = C.c_int()
        interner._call("apply_batch", t, batch.handle, C.byref(changed))
        if changed.value:
            self._dirty = True
        return bool(changed.value)

    def to_vec(self, interner):
        """to_vec (utils/common.rs:158-246): dense [y][z][x] numpy grid."""
        t = self._bind(interner)
        n = 1 << self.max_depth_value
        out = np.zeros((n, n, n), dtype=interner.dtype)
        interner._call("tree_to_dense", t, _np_ptr(out))
        return out
