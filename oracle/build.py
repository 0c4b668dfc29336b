"""Build recipe for the CPU oracle (test infrastructure only).

Compiles the C++ restatement of the reference path (vx_oracle.hpp + vx_oracle_capi.cpp) into
oracle/_build/libvx_oracle.so with the host compiler. The reference itself is Rust and cannot be
compiled in this environment, so there is no oracle/_ref build.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libvx_oracle.so")
SOURCES = [os.path.join(HERE, "vx_oracle_capi.cpp")]
HEADERS = [os.path.join(HERE, "vx_oracle.hpp"), os.path.join(HERE, "..", "include", "voxelis_gb300.h")]


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(p) > t for p in SOURCES + HEADERS)


def build(force=False):
    """Compile the oracle library if it is missing or older than its sources; returns its path."""
    if not force and not _stale():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    cmd = [os.environ.get("CXX", "g++"), "-O3", "-std=c++17", "-shared", "-fPIC",
           "-fno-strict-aliasing", "-o", LIB] + SOURCES
    subprocess.run(cmd, check=True)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
