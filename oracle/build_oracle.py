"""Build the CPU oracle (test infrastructure, never linked by the product).

Produces oracle/_build/liboracle2d.so and liboracle3d.so from oracle.c with
-DDIM=2 / -DDIM=3, like the reference's -DDIM2 / -DDIM3 trees.  Plain gcc,
portable flags (no -march=native) and -ffp-contract=off so the x86 and Arm
hosts give identical FP64 results.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build")


def build(force: bool = False) -> list:
    os.makedirs(OUT, exist_ok=True)
    src = os.path.join(HERE, "oracle.c")
    hdr = os.path.join(HERE, "oracle.h")
    libs = []
    procs = []
    for d in (2, 3):
        lib = os.path.join(OUT, f"liboracle{d}d.so")
        libs.append(lib)
        if (not force and os.path.exists(lib)
                and os.path.getmtime(lib) >= max(os.path.getmtime(src), os.path.getmtime(hdr))):
            continue
        cmd = ["gcc", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", f"-DDIM={d}",
               "-o", lib + ".tmp", src, "-lm"]
        procs.append((subprocess.Popen(cmd), lib))
    for p, lib in procs:
        if p.wait() != 0:
            raise RuntimeError(f"oracle build failed for {lib}")
        os.replace(lib + ".tmp", lib)
    return libs


if __name__ == "__main__":
    print("\n".join(build(force="--force" in sys.argv)))
