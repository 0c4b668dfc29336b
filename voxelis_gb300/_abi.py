"""ctypes binding of the voxelis_gb300 C ABI (include/voxelis_gb300.h).

`NativeLib(path, prefix)` binds every entry point of the header. The GPU library exports them with
the `vx_` prefix. Any other library exporting the same entry points under another prefix can be
bound the same way (the test-suite uses this to drive a CPU restatement through identical calls).
"""
import ctypes as C
import os

# ---- status codes (voxelis_gb300.h) ------------------------------------------------------------
VX_OK = 0
VX_E_INVALID_ARG = 1
VX_E_OOB = 2
VX_E_OOM = 3
VX_E_DEPTH = 4
VX_E_TABLE_FULL = 5
VX_E_TIMEOUT = 6
VX_E_CUDA = 7
VX_E_REF_PANIC = 8
VX_E_REF_UB = 9
VX_E_BUFFER = 10
VX_E_UNSUPPORTED = 11

STATUS_NAMES = {
    VX_OK: "VX_OK", VX_E_INVALID_ARG: "VX_E_INVALID_ARG", VX_E_OOB: "VX_E_OOB",
    VX_E_OOM: "VX_E_OOM", VX_E_DEPTH: "VX_E_DEPTH", VX_E_TABLE_FULL: "VX_E_TABLE_FULL",
    VX_E_TIMEOUT: "VX_E_TIMEOUT", VX_E_CUDA: "VX_E_CUDA", VX_E_REF_PANIC: "VX_E_REF_PANIC",
    VX_E_REF_UB: "VX_E_REF_UB", VX_E_BUFFER: "VX_E_BUFFER", VX_E_UNSUPPORTED: "VX_E_UNSUPPORTED",
}

VX_PATCH_P1 = 1 << 0
VX_PATCH_P2 = 1 << 1
VX_PATCH_P3 = 1 << 2
VX_PATCH_P4 = 1 << 3
VX_PATCH_P5 = 1 << 4

VX_MEM_HOST = 0
VX_MEM_DEVICE = 1

VX_PROF_NAMES = ["dense", "levels", "refcount", "apply_levels", "release", "get", "copy", "apply_bottom"]
VX_PROF_N = 8

VX_BLOCK_EMPTY = 0
VX_BLOCK_INVALID = 0xFFFFFFFFFFFFFFFF


class VoxelisError(RuntimeError):
    """A non-OK status returned by the C ABI."""

    def __init__(self, status, message=""):
        self.status = status
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")


class ReferencePanic(VoxelisError):
    """The reference implementation panics on this input (assert!, OOM, depth cap, bounds)."""


class ReferenceUB(VoxelisError):
    """The reference implementation hits undefined behaviour on this input."""


def error_for(status, message=""):
    if status in (VX_E_REF_PANIC, VX_E_OOM, VX_E_DEPTH, VX_E_OOB):
        return ReferencePanic(status, message)
    if status == VX_E_REF_UB:
        return ReferenceUB(status, message)
    return VoxelisError(status, message)


class vx_interner_stats(C.Structure):
    _fields_ = [(n, C.c_uint64) for n in (
        "capacity", "node_size", "next_index", "free_count", "alive_nodes", "branch_patterns",
        "leaf_patterns", "table_slots", "table_tombstones", "error_flags", "nodes_created")]


class vx_world(C.Structure):
    _fields_ = [("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32), ("chunk_depth", C.c_int32),
                ("trees_dev", C.c_void_p)]


class vx_canonical(C.Structure):
    _fields_ = [
        ("kind", C.POINTER(C.c_uint8)),
        ("types", C.POINTER(C.c_uint8)),
        ("mask", C.POINTER(C.c_uint8)),
        ("value", C.POINTER(C.c_uint32)),
        ("refcount", C.POINTER(C.c_uint32)),
        ("children", C.POINTER(C.c_int32)),
        ("roots", C.POINTER(C.c_int32)),
        ("capacity", C.c_uint64),
    ]


_P = C.c_void_p
_I = C.c_int
_U32 = C.c_uint32
_U64 = C.c_uint64
_I32 = C.c_int32
_PI = C.POINTER(C.c_int)
_PU32 = C.POINTER(C.c_uint32)
_PU64 = C.POINTER(C.c_uint64)

# name -> argument types (every function returns int, except last_error)
SIGNATURES = {
    "interner_create": [_U64, _I, _U32, _I, C.POINTER(_P)],
    "interner_destroy": [_P],
    "interner_stats_get": [_P, C.POINTER(vx_interner_stats)],
    "get_ref": [_P, _U64, _PU32],
    "get_value": [_P, _U64, _PU32],
    "tree_create": [_P, _I, _PU32],
    "tree_destroy": [_P, _U32],
    "tree_root": [_P, _U32, _PU64],
    "tree_max_depth": [_P, _U32, _PI],
    "tree_get": [_P, _U32, _I32, _I32, _I32, _PI, _PU32],
    "tree_set": [_P, _U32, _I32, _I32, _I32, _U32, _PI],
    "tree_fill": [_P, _U32, _U32],
    "tree_clear": [_P, _U32],
    "batch_create": [_I, _I, _U32, C.POINTER(_P)],
    "batch_destroy": [_P],
    "batch_set": [_P, _I32, _I32, _I32, _U32],
    "batch_fill": [_P, _U32],
    "batch_clear": [_P],
    "batch_set_dense": [_P, _P],
    "batch_set_many": [_P, _U64, _P, _P],
    "batch_size": [_P, _PU64],
    "batch_has_patches": [_P, _PI],
    "apply_batch": [_P, _U32, _P, _PI],
    "apply_batches": [_P, _U32, _P, _P, _P],
    "build_dense": [_P, _U32, _P, _P, _P, _I],
    "get_many": [_P, _U64, _P, _P, _P, _P, _I],
    "export_canonical": [_P, _U32, _P, C.POINTER(vx_canonical), _PU64],
    "tree_to_dense": [_P, _U32, _P],
    "validate": [_P, _U32, _P],
    "occupancy_masks": [_P, _U32, _P, _P, _P, _P, _U32, _P, _P, _P, _P],
    "serialize_model": [_P, _U32, _P, _P, _P, _U64, _PU64],
    "deserialize_model": [_P, _P, _U64, _I, _U32, _P, _P, C.POINTER(C.c_uint32)],
}

# entry points only the GPU library has
GPU_SIGNATURES = {
    "profile_enable": [_P, _I],
    "profile_collect": [_P, C.POINTER(C.c_double), _PU64],
    "interner_reset": [_P],
    "interner_maintain": [_P],
    "interner_set_stream": [_P, _P],
    "interner_set_limits": [_P, _U32, _U32, _U32],
    "interner_get_limits": [_P, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)],
    "interner_sync": [_P],
    "trees_create": [_P, _U32, _P, _P],
    "build_dense_async": [_P, _U32, _P, _P, _P, _I],
    "get_many_async": [_P, _U64, _P, _P, _P, _P],
    "apply_groups_async": [_P, _U32, _P, _P, _P, _U32, _P, _P, _P, _P, _P, _P, _I],
    "tune_set": [_P, _I, _I],
    "trees_set_many": [_P, _U64, _P, _P, _P, _P],
    "world_get_async": [_P, _P, _U64, _P, _P, _P],
    "world_hold_async": [_P, _P, _U32, _P, _P, _P, _P, _P],
    "world_get_at_async": [_P, _P, _U64, _P, _P, _P, _P, _P, _U32],
    "world_release_async": [_P, _P, _U32, _P, _P, _P],
    "copy_to_device_async": [_P, _U32, _P, _P, _P],
    "tune_get": [_P, _PI, _PI],
    "tune_set_launch": [_P, _I],
    "tune_get_launch": [_P, _PI],
    "tune_set_dense": [_P, _I],
    "tune_get_dense": [_P, _PI],
    "trees_to_dense": [_P, _U32, _P, _P, _I],
    "trees_to_dense_async": [_P, _U32, _P, _I, _P],
    "occupancy_masks_async": [_P, _U32, _U32, _P, _P, _P, _I, _U32, _P, _P, _P, _P, _P, _P],
}


class NativeLib:
    """One loaded library exposing the C ABI under `prefix`."""

    def __init__(self, path, prefix, extra=None):
        self.path = os.path.abspath(path)
        self.prefix = prefix
        self.lib = C.CDLL(self.path)
        self._fns = {}
        sigs = dict(SIGNATURES)
        if extra:
            sigs.update(extra)
        for name, argtypes in sigs.items():
            f = getattr(self.lib, prefix + name)
            f.argtypes = argtypes
            f.restype = C.c_int
            self._fns[name] = f
        if hasattr(self.lib, prefix + "kernel_launches"):
            kl = getattr(self.lib, prefix + "kernel_launches")
            kl.argtypes = []
            kl.restype = C.c_uint64
            self.kernel_launches = kl
        le = getattr(self.lib, prefix + "last_error")
        le.argtypes = [_P]
        le.restype = C.c_char_p
        self._last_error = le

    def has(self, name):
        return name in self._fns

    def raw(self, name):
        return self._fns[name]

    def last_error(self, handle):
        msg = self._last_error(handle)
        return msg.decode() if msg else ""

    def call(self, name, *args, handle=None):
        """Calls `prefix+name`; raises the matching VoxelisError on a non-OK status."""
        st = self._fns[name](*args)
        if st != VX_OK:
            raise error_for(st, self.last_error(handle) if handle else "")
        return st

    def status(self, name, *args):
        """Calls `prefix+name` and returns the raw status."""
        return self._fns[name](*args)


_GPU_LIB = None


def gpu_lib():
    """The in-tree GPU library (voxelis_gb300/_build/libvoxelis_gb300.so). Raises if it was not built."""
    global _GPU_LIB
    if _GPU_LIB is None:
        here = os.path.dirname(os.path.abspath(__file__))
        path = os.path.join(here, "_build", "libvoxelis_gb300.so")
        if not os.path.exists(path):
            raise RuntimeError(
                "voxelis_gb300 CUDA library is not built (%s); run __graft_entry__.build()" % path)
        _GPU_LIB = NativeLib(path, "vx_", extra=GPU_SIGNATURES)
    return _GPU_LIB
