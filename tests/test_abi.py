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


def _tool(name):
    import shutil

    exe = shutil.which(name)
    if not exe:
        pytest.skip("%s not installed" % name)
    return exe


def test_library_has_no_oracle_dependency(gpu_library_path):
    """The product library neither links the oracle nor defines any of its symbols: checked on the
    host ELF's dynamic section (needed libraries) and dynamic symbol table only."""
    import subprocess

    needed = subprocess.run([_tool("readelf"), "-d", gpu_library_path], capture_output=True, text=True, check=True)
    libs = re.findall(r"\(NEEDED\)\s+Shared library: \[([^\]]+)\]", needed.stdout)
    assert libs, needed.stdout
    assert not [n for n in libs if "oracle" in n], libs
    syms = subprocess.run([_tool("nm"), "-D", "--defined-only", gpu_library_path], capture_output=True, text=True,
                          check=True)
    names = [ln.split()[-1] for ln in syms.stdout.splitlines() if ln.strip()]
    assert "vx_apply_batches" in names
    assert not [n for n in names if n.startswith("vxo_") or "oracle" in n]


# ---- header prototypes against the Rust extern block ------------------------------------------
_RUST_BASE = {"vx_interner": "VxInterner", "vx_batch": "VxBatch", "vx_tree": "VxTree", "vx_mem": "VxMem",
              "vx_interner_stats": "VxInternerStats", "vx_canonical": "VxCanonical", "vx_world": "VxWorld",
              "void": "c_void", "char": "c_char", "int": "i32", "int32_t": "i32", "uint32_t": "u32",
              "uint64_t": "u64", "uint16_t": "u16", "uint8_t": "u8", "double": "f64", "size_t": "usize"}


def _rust_of_c(decl, named=True):
    """Rust spelling of a C parameter (or return) type: `const T *const *p` -> `*const *const T`."""
    toks = re.findall(r"\*|\w+", decl)
    if named:
        toks = toks[:-1]  # the parameter name
    base_const = toks[0] == "const"
    if base_const:
        toks = toks[1:]
    base, rest = toks[0], toks[1:]
    quals = []  # const-ness of each pointer, innermost first
    for t in rest:
        if t == "*":
            quals.append(False)
        elif t == "const" and quals:
            quals[-1] = True
    out = _RUST_BASE[base]
    for i, _ in enumerate(quals):
        pointee_const = base_const if i == 0 else quals[i - 1]
        out = ("*const " if pointee_const else "*mut ") + out
    return out


def _header_prototypes():
    text = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    protos = {}
    for m in re.finditer(r"^\s*(int|uint64_t|const char \*)\s*(vx_\w+)\s*\(([^)]*)\)\s*;", text, re.M):
        ret, name, params = m.group(1), m.group(2), m.group(3).strip()
        args = [] if params in ("", "void") else [_rust_of_c(p.strip()) for p in params.split(",")]
        protos[name] = (args, _rust_of_c(ret, named=False))
    return protos


def _rust_prototypes():
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    block = text[text.index("```rust"):]
    block = block[:block.index("\n```\n")]
    protos = {}
    for m in re.finditer(r"pub fn (vx_\w+)\s*\(([^)]*)\)\s*(?:->\s*([^;]+))?;", block):
        params = [p.strip() for p in m.group(2).split(",") if p.strip()]
        args = [" ".join(p.split(":", 1)[1].split()) for p in params]
        protos[m.group(1)] = (args, " ".join((m.group(3) or "()").split()))
    return protos


def test_rust_binding_declares_every_entry_point():
    """INTEGRATION.md's extern block (what a Rust crate would bind) covers the whole header, and each
    entry point there has the header's parameter count, parameter types and return type."""
    header, rust = _header_prototypes(), _rust_prototypes()
    assert set(header) == set(declared())
    missing = [n for n in header if n not in rust]
    assert not missing, missing
    for name, (args, ret) in header.items():
        r_args, r_ret = rust[name]
        assert len(r_args) == len(args), (name, args, r_args)
        assert r_args == args, (name, args, r_args)
        assert r_ret == ret, (name, ret, r_ret)
