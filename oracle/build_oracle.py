"""Build the CPU oracle (test infrastructure, never linked by the product).

Produces, from oracle.c with -DDIM=2 / -DDIM=3 (like the reference's
-DDIM2 / -DDIM3 trees):

* oracle/_build/liboracle2d.so, liboracle3d.so -- the parity build: plain
  gcc -O2, portable flags and -ffp-contract=off, so the x86 and Arm hosts
  give identical FP64 results;
* oracle/_build/liboracle2d_fast.so, liboracle3d_fast.so -- the timing
  build for the CPU baseline: -O3 -march=native (-mcpu=native where gcc
  does not take -march=native, plain -O3 where neither works), still
  -ffp-contract=off, so its results equal the parity build's.

A library is rebuilt when its source is newer or when the key file beside
it names another machine architecture, compiler or flags.
"""
import os
import platform
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build")
PORTABLE = ["-O2", "-fopenmp", "-ffp-contract=off"]
FAST_CANDIDATES = (["-O3", "-march=native"], ["-O3", "-mcpu=native"], ["-O3"])


def _gcc_version() -> str:
    try:
        out = subprocess.run(["gcc", "--version"], capture_output=True, text=True).stdout.splitlines()
        return out[0] if out else "unknown"
    except OSError:
        return "unknown"


def _accepts(flags) -> bool:
    r = subprocess.run(["gcc"] + flags + ["-x", "c", "-c", "-o", os.devnull, "-"], input="int x;\n",
                       capture_output=True, text=True)
    return r.returncode == 0


def fast_flags() -> list:
    """Flags of the timing build on this host."""
    for c in FAST_CANDIDATES:
        if _accepts(c):
            return c + ["-fopenmp", "-ffp-contract=off"]
    return ["-O2", "-fopenmp", "-ffp-contract=off"]


def _key(flags) -> str:
    return "\n".join([platform.machine(), _gcc_version(), " ".join(flags)]) + "\n"


def _stale(lib: str, key: str, deps) -> bool:
    kf = lib + ".key"
    if not os.path.exists(lib) or not os.path.exists(kf):
        return True
    with open(kf) as f:
        if f.read() != key:
            return True
    return os.path.getmtime(lib) < max(os.path.getmtime(d) for d in deps)


def build(force: bool = False, fast: bool = True) -> list:
    """Build (when stale) and return [liboracle2d.so, liboracle3d.so]; with fast=True also the timing build."""
    os.makedirs(OUT, exist_ok=True)
    src = os.path.join(HERE, "oracle.c")
    hdr = os.path.join(HERE, "oracle.h")
    variants = [("", PORTABLE)] + ([("_fast", fast_flags())] if fast else [])
    libs, procs = [], []
    for suffix, flags in variants:
        key = _key(flags)
        for d in (2, 3):
            lib = os.path.join(OUT, f"liboracle{d}d{suffix}.so")
            if not suffix:
                libs.append(lib)
            if not force and not _stale(lib, key, (src, hdr)):
                continue
            cmd = ["gcc"] + flags + ["-fPIC", "-shared", f"-DDIM={d}", "-o", lib + ".tmp", src, "-lm"]
            procs.append((subprocess.Popen(cmd), lib, key))
    for p, lib, key in procs:
        if p.wait() != 0:
            raise RuntimeError(f"oracle build failed for {lib}")
        os.replace(lib + ".tmp", lib)
        with open(lib + ".key", "w") as f:
            f.write(key)
    return libs


def fast_paths() -> list:
    """[liboracle2d_fast.so, liboracle3d_fast.so] (built by build())."""
    return [os.path.join(OUT, f"liboracle{d}d_fast.so") for d in (2, 3)]


if __name__ == "__main__":
    print("\n".join(build(force="--force" in sys.argv)))
