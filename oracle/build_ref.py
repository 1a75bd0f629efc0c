"""Compile the reference's own CUDA sources for the CPU (checker only).

TEST INFRASTRUCTURE ONLY.  This recipe reads the reference tree (the
directory SA_REFERENCE_ROOT names or, when that is unset, a checkout named
``reference`` beside this repository's root, recognised by its
CUDA/compile.m), takes the four MEX
source lists from its CUDA/compile.m (parsed as text, the build script is
not run), and builds each list with g++ into oracle/_ref/:

    libref_deformation_2D_frame.so     libref_computeObjfcn_2D_frame.so
    libref_deformation_3D_frame.so     libref_computeObjfcn_3D_frame.so

The only change made to the sources is mechanical and happens in a
temporary directory outside the repository: each kernel launch
``k <<<grid, block>>> (args);`` becomes a call of the emulated launcher
(oracle/ref_shim/cuda_emu.h).  Headers are used in place.  CUDA runtime,
cuBLAS, cuSOLVER and MEX calls resolve to oracle/ref_shim/emu_runtime.cpp.
The reference's own mexFunction gateways are compiled unchanged and are
what oracle/ref.py calls.

Nothing here travels to or runs on the GPU host; tests use the libraries
only through the committed golden vectors (tests/golden/) and, in this
container, directly when they exist.
"""
from __future__ import annotations

import os
import re
import shutil
import subprocess
import sys
import tempfile
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
SHIM = os.path.join(HERE, "ref_shim")


def reference_root() -> str:
    """The reference checkout, or "" when none is found (then nothing here is built)."""
    env = os.environ.get("SA_REFERENCE_ROOT")
    if env:
        return env
    beside = os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")
    return beside if os.path.isfile(os.path.join(beside, "CUDA", "compile.m")) else ""


def parse_compile_m(path: str):
    """[(output, dimflag, [files])] from the mexcuda calls of compile.m."""
    text = open(path).read()
    targets = []
    for m in re.finditer(r"files\s*=\s*\.\.\.\s*\{(.*?)\};(.*?)mexcuda\((.*?)\);", text, re.S):
        files = re.findall(r"'([^']+\.cu)'", m.group(1))
        args = m.group(3)
        dim = re.search(r"'-D(DIM[23])'", args).group(1)
        out = re.search(r"'-output',\s*'([^']+)'", args).group(1)
        targets.append((out, dim, files))
    return targets


def _match_paren(s: str, i: int) -> int:
    depth = 0
    for j in range(i, len(s)):
        if s[j] == "(":
            depth += 1
        elif s[j] == ")":
            depth -= 1
            if depth == 0:
                return j
    raise ValueError("unbalanced launch")


def _split_top(s: str):
    parts, depth, cur = [], 0, ""
    for ch in s:
        if ch in "([{":
            depth += 1
        elif ch in ")]}":
            depth -= 1
        if ch == "," and depth == 0:
            parts.append(cur)
            cur = ""
        else:
            cur += ch
    parts.append(cur)
    return [p.strip() for p in parts]


def rewrite_launches(src: str, barrier_kernels: set) -> str:
    out, pos = [], 0
    pat = re.compile(r"(\w+)\s*<<<(.*?)>>>\s*\(", re.S)
    while True:
        m = pat.search(src, pos)
        if not m:
            out.append(src[pos:])
            break
        name, cfg = m.group(1), m.group(2)
        lp = m.end() - 1
        rp = _match_paren(src, lp)
        args = src[lp + 1:rp]
        grid, block = _split_top(cfg)[:2]
        sync = "true" if name in barrier_kernels else "false"
        out.append(src[pos:m.start()])
        out.append(f"sa_emu_launch(dim3({grid}), dim3({block}), [&]() {{ {name}({args}); }}, {sync})")
        pos = rp + 1
    return "".join(out)


def barrier_kernels(src: str) -> set:
    names = set()
    chunks = re.split(r"__global__\s+void\s+", src)
    for ch in chunks[1:]:
        nm = re.match(r"(\w+)", ch).group(1)
        if "__syncthreads" in ch.split("__global__")[0]:
            names.add(nm)
    return names


def build(force: bool = False, jobs: int = 8) -> list:
    root = os.path.join(reference_root(), "CUDA")
    if not os.path.isdir(root):
        raise FileNotFoundError(f"reference tree not found at {root}")
    os.makedirs(OUT, exist_ok=True)
    targets = parse_compile_m(os.path.join(root, "compile.m"))
    libs = []
    tmp = tempfile.mkdtemp(prefix="sa_refbuild_")
    try:
        runtime_obj = os.path.join(tmp, "emu_runtime.o")
        base = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-w",
                "-include", os.path.join(SHIM, "cuda_emu.h"), "-I", SHIM]
        subprocess.check_call(base + ["-c", os.path.join(SHIM, "emu_runtime.cpp"), "-o", runtime_obj])
        jobs_list = []
        for out, dim, files in targets:
            lib = os.path.join(OUT, f"libref_{out}.so")
            libs.append(lib)
            if os.path.exists(lib) and not force:
                continue
            tdir = os.path.join(tmp, out)
            os.makedirs(tdir)
            objs = []
            for f in files:
                src_path = os.path.join(root, f)
                text = open(src_path).read()
                text = rewrite_launches(text, barrier_kernels(text))
                dst = os.path.join(tdir, os.path.basename(f))
                with open(dst, "w") as fh:
                    fh.write(text)
                obj = dst[:-3] + ".o"
                objs.append(obj)
                cmd = base + [f"-D{dim}", "-I", os.path.join(root, "include"),
                              "-I", os.path.join(root, os.path.dirname(f)), "-x", "c++", "-c", dst, "-o", obj]
                jobs_list.append(cmd)
            libs_link = (lib, objs)
            jobs_list.append(("LINK", libs_link))
        compiles = [j for j in jobs_list if j[0] != "LINK"]
        links = [j[1] for j in jobs_list if j[0] == "LINK"]
        with ThreadPoolExecutor(jobs) as ex:
            rcs = list(ex.map(lambda c: subprocess.call(c), compiles))
        if any(rcs):
            raise RuntimeError("compiling the reference sources failed")
        for lib, objs in links:
            subprocess.check_call(["g++", "-shared", "-o", lib + ".tmp"] + objs + [runtime_obj])
            os.replace(lib + ".tmp", lib)
    finally:
        shutil.rmtree(tmp, ignore_errors=True)
    return libs


def build_ops(force: bool = False) -> str:
    """oracle/_ref/libref_ops_2D.so: oracle/ref_ops.cpp (single-operator entry points) linked against the
    reference's 2D library built above."""
    build()
    lib = os.path.join(OUT, "libref_ops_2D.so")
    src = os.path.join(HERE, "ref_ops.cpp")
    if os.path.exists(lib) and not force and os.path.getmtime(lib) >= os.path.getmtime(src):
        return lib
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-shared", src,
                           "-L", OUT, "-lref_deformation_2D_frame", f"-Wl,-rpath,{OUT}", "-o", lib + ".tmp"])
    os.replace(lib + ".tmp", lib)
    return lib


if __name__ == "__main__":
    print("\n".join(build(force="--force" in sys.argv)))
