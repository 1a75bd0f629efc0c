"""Compile the MEX gateways of shape_atrophy_gb300/mex/ against the test
stand-in of the MEX API (tests/mex_stub) and the CUDA library, one shared
library per entry point (deformation / computeObjfcn x 2D / 3D x frame /
isotropic), into tests/mex_stub/_build/.  Used by
tests/test_gpu_mex_gateway.py.  Keys: (name, dim) for the frame gateways,
(name, dim, "isotropic") for the layered ones."""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.abspath(os.path.join(HERE, "..", ".."))
OUT = os.path.join(HERE, "_build")
GATEWAYS = {("deformation", "frame"): "sa_mex_deformation.cpp",
            ("computeObjfcn", "frame"): "sa_mex_computeObjfcn.cpp",
            ("deformation", "isotropic"): "sa_mex_deformation_isotropic.cpp",
            ("computeObjfcn", "isotropic"): "sa_mex_computeObjfcn_isotropic.cpp"}


def path(name: str, dim: int, model: str = "frame") -> str:
    return os.path.join(OUT, f"lib{name}_{dim}D_{model}.so")


def build() -> dict:
    sys.path.insert(0, ROOT)
    from shape_atrophy_gb300 import build as libbuild
    lib = libbuild.build()
    libdir = os.path.dirname(lib)
    os.makedirs(OUT, exist_ok=True)
    out = {}
    for (name, model), src in GATEWAYS.items():
        for dim in (2, 3):
            so = path(name, dim, model)
            cmd = ["g++", "-O2", "-std=c++17", "-shared", "-fPIC", f"-DSA_DIM={dim}",
                   os.path.join(ROOT, "shape_atrophy_gb300", "mex", src), os.path.join(HERE, "mex_stub.cpp"),
                   "-I", HERE, "-I", os.path.join(ROOT, "include"), "-L", libdir, "-lshape_atrophy_gb300",
                   f"-Wl,-rpath,{libdir}", "-o", so]
            subprocess.run(cmd, check=True)
            out[(name, dim) if model == "frame" else (name, dim, model)] = so
    return out


if __name__ == "__main__":
    print(build())
