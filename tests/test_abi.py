"""The C ABI boundary without a GPU: the CUDA library loads and exports every entry point that
include/voxelis_gb300.h declares, and the oracle exports the same core entry points under its prefix.
No device work is done here."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "voxelis_gb300.h")


def declared():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:int|uint64_t|const char \*)\s*(vx_\w+)\s*\(", text, re.M)))


@pytest.fixture(scope="module")
def gpu_library_path():
    from voxelis_gb300 import build

    try:
        return build.build()
    except RuntimeError as e:  # nvcc missing would be an environment problem, not a test failure
        pytest.skip(str(e))


def test_header_declares_the_boundary():
    names = declared()
    for must in ("vx_interner_create", "vx_tree_create", "vx_apply_batch", "vx_apply_batches", "vx_tree_get",
                 "vx_get_many", "vx_build_dense", "vx_batch_set", "vx_get_ref", "vx_export_canonical"):
        assert must in names
    assert len(names) >= 35


def test_library_exports_every_declared_symbol(gpu_library_path):
    lib = C.CDLL(gpu_library_path)
    missing = [n for n in declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_oracle_exports_the_core_boundary(oracle_lib):
    from voxelis_gb300._abi import SIGNATURES

    for name in SIGNATURES:
        assert hasattr(oracle_lib.lib, "vxo_" + name)


def test_python_binding_matches_the_library(gpu_library_path):
    from voxelis_gb300._abi import GPU_SIGNATURES, SIGNATURES, NativeLib

    lib = NativeLib(gpu_library_path, "vx_", extra=GPU_SIGNATURES)
    assert set(SIGNATURES) | set(GPU_SIGNATURES) <= {n[3:] for n in declared()}
    assert lib.kernel_launches() >= 0


def test_library_has_no_oracle_dependency(gpu_library_path):
    """The product library must not link or embed the oracle."""
    data = open(gpu_library_path, "rb").read()
    assert b"vxo_" not in data
    assert b"vx_oracle" not in data


def test_rust_binding_declares_every_entry_point():
    """INTEGRATION.md's extern block (what a Rust crate would bind) covers the whole header."""
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    block = text[text.index("```rust"):]
    block = block[:block.index("\n```\n")]
    bound = set(re.findall(r"pub fn (vx_\w+)\s*\(", block))
    missing = [n for n in declared() if n not in bound]
    assert not missing, missing
