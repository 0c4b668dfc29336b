"""Build recipe of the in-tree CUDA library voxelis_gb300/_build/libvoxelis_gb300.so (sm_103a).

Each translation unit is compiled in parallel with nvcc for exactly one target
(-gencode arch=compute_103a,code=sm_103a), then linked into one shared library exporting the C ABI
of include/voxelis_gb300.h. The build is incremental: unchanged objects are reused.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libvoxelis_gb300.so")
SOURCES = ["vx_build.cu", "vx_apply.cu", "vx_ops.cu", "vx_capi.cu", "vx_noalloc.cu", "vx_world.cu", "vx_vtm.cu"]
HEADERS = ["vx_device.cuh", "vx_launch.h"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]


def nvcc():
    exe = shutil.which("nvcc")
    if exe:
        return exe
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found")


def _deps():
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(ROOT, "include", "voxelis_gb300.h")]
    return max(os.path.getmtime(h) for h in hdrs)


def _compile(src, extra):
    obj = os.path.join(OUT_DIR, src.replace(".cu", ".o"))
    srcp = os.path.join(CSRC, src)
    if os.path.exists(obj) and os.path.getmtime(obj) > max(os.path.getmtime(srcp), _deps()):
        return obj
    cmd = [nvcc(), "-c", srcp, "-o", obj] + ARCH + FLAGS + extra
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, r.stdout, r.stderr))
    return obj


def build(force=False, verbose=False, extra=None):
    """Compiles and links the library if needed; returns its path."""
    extra = list(extra or [])
    os.makedirs(OUT_DIR, exist_ok=True)
    if force:
        for f in os.listdir(OUT_DIR):
            if f.endswith(".o"):
                os.remove(os.path.join(OUT_DIR, f))
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), SOURCES))
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        cmd = [nvcc(), "-shared", "-o", LIB] + objs + ARCH + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
    if verbose:
        print(LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True,
          extra=["-Xptxas", "-v"] if "--ptxas" in sys.argv else None)
