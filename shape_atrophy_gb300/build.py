"""Build the CUDA library libshape_atrophy_gb300.so for sm_103a (in-tree).

Plain nvcc, one -gencode (compute_103a -> sm_103a), translation units
compiled in parallel, output in shape_atrophy_gb300/_build/.  No torch,
no cmake.  Used by __graft_entry__.build() on every host.  A library is
reused only when a key file written beside it names this host's machine
architecture, this nvcc's version and the same flags, and no source is
newer: a binary built on another host (x86_64 vs aarch64) or by another
toolkit is rebuilt, whatever its modification time.
"""
from __future__ import annotations

import glob
import os
import platform
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libshape_atrophy_gb300.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
         "--expt-relaxed-constexpr", "-I", INCLUDE]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.sep not in c or os.path.exists(c)):
            return c
    return "nvcc"


def sources():
    return sorted(glob.glob(os.path.join(SRC, "*.cu")))


KEY = os.path.join(OUT, "build_key.txt")


def build_key(extra=()) -> str:
    """Host architecture, nvcc version and flags the library is built with."""
    try:
        ver = subprocess.run([nvcc(), "--version"], capture_output=True, text=True).stdout.strip().splitlines()
        ver = ver[-1] if ver else "unknown"
    except OSError:
        ver = "unknown"
    return "\n".join([platform.machine(), ver, " ".join(ARCH + FLAGS + list(extra))]) + "\n"


def up_to_date(extra=()) -> bool:
    if not os.path.exists(LIB) or not os.path.exists(KEY):
        return False
    with open(KEY) as f:
        if f.read() != build_key(extra):
            return False
    t = os.path.getmtime(LIB)
    deps = sources() + glob.glob(os.path.join(SRC, "*.cuh")) + glob.glob(os.path.join(INCLUDE, "*.h"))
    return all(os.path.getmtime(d) <= t for d in deps)


def build(force: bool = False, verbose: bool = False, extra=()) -> str:
    if not force and up_to_date(extra):
        return LIB
    os.makedirs(OUT, exist_ok=True)
    objs = []
    cmds = []
    for src in sources():
        obj = os.path.join(OUT, os.path.basename(src)[:-3] + ".o")
        objs.append(obj)
        cmds.append([nvcc()] + ARCH + FLAGS + list(extra) + ["-c", src, "-o", obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if verbose or r.returncode != 0:
            sys.stderr.write(r.stdout + r.stderr)
        return r.returncode

    with ThreadPoolExecutor(max(1, min(len(cmds), os.cpu_count() or 4))) as ex:
        rcs = list(ex.map(run, cmds))
    if any(rcs):
        raise RuntimeError("nvcc failed; see the messages above")
    tmp = LIB + ".tmp"
    link = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
    if run(link) != 0:
        raise RuntimeError("link failed")
    os.replace(tmp, LIB)
    with open(KEY, "w") as f:
        f.write(build_key(extra))
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
