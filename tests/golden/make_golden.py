"""Generate the golden vectors in tests/golden/*.npz from the reference itself.

Run in the development container, where the reference tree exists:

    python tests/golden/make_golden.py

Each case is built with shape_atrophy_gb300.problems / mesh, then the
reference's own MEX gateways (compiled for the CPU by oracle/build_ref.py)
produce the outputs.  Every input array and scalar is stored next to the
outputs, so the fixtures are self-contained: tests read them without the
reference tree and without rebuilding meshes.
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), "..", ".."))
sys.path.insert(0, ROOT)

from oracle import ref  # noqa: E402
from shape_atrophy_gb300 import mesh, problems  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))

OBJ_KEYS = ["elmVtxMat", "vtxElmMat", "tanVtxMat", "nmlVtxMat", "tsvVtxMat", "bdrVtxMat", "vtxBdrMat",
            "btmVtxMat", "vtxBtmMat", "femVtxMat", "femIfoMat", "vfdVtxMat", "vfdIfoMat"]
SCALARS = ["dim", "ldmWgt", "knlOrder", "knlWidth", "knlEps", "spdTanVal", "spdTsvVal", "btmWgt",
           "timeStp", "timeNum", "cgItrMax", "cgTolSqu"]


def save(name: str, spec: dict, tauVarMat: np.ndarray):
    tv = np.atleast_2d(np.asarray(tauVarMat, dtype=np.float64))
    lmk, tau, objd = ref.deformation(spec, tv)
    objf = ref.compute_objfcn(spec, tv)
    data = {f"obj_{k}": v for k, v in spec["elmObj"].items() if k in OBJ_KEYS}
    data.update({k: np.asarray(spec[k]) for k in SCALARS})
    data.update(lmkIniMat=spec["lmkIniMat"], tauPrmVec=spec["tauPrmVec"], modVec=spec["modVec"],
                ynkActPrmVec=spec["ynkActPrmVec"], reaActPrmVec=spec["reaActPrmVec"],
                tgtCen=spec["tgt"][0], tgtDir=spec["tgt"][1], tgtVol=spec["tgt"][2],
                vfdKnl=np.array([ord(spec["vfd"][0]), spec["vfd"][1], ord(spec["vfd"][2]), spec["vfd"][3]]),
                tauVarMat=tv, ref_lmkStk=lmk, ref_tauMat=tau, ref_deformation_obj=objd, ref_objfcn=objf)
    np.savez_compressed(os.path.join(OUT, name + ".npz"), **data)
    print(name, "N", spec["lmkIniMat"].shape[1], "obj", objf)


def main():
    # 2D: the demo parameters on a coarse strip, Matern order 3 (demo), Gaussian/Binet varifold
    s = problems.demo_strip(21, 7, timeEnd=0.1)
    save("frame2d_demo_m3", s, s["tauVarVec"])

    # 2D: Gaussian RKHS kernel, Cauchy/oriented varifold, two parameter columns
    s = problems.demo_strip(15, 5, timeEnd=0.06)
    s.update(knlOrder=-1, knlWidth=0.5)
    s["vfd"] = ("C", 0.4, "O", 0.8)
    save("frame2d_gauss_2col", s, np.stack([s["tauVarVec"], np.array([-0.5, 0.2, 0.3, 0.4])]))

    # 2D: remaining Matern orders 0, 1, 2, 4 (Bessel-function branches) and varifold kernels L / U
    for order, vk in [(0, ("G", 0.3, "L", 1.0)), (1, ("C", 0.3, "U", 0.7)), (2, ("G", 0.6, "B", 1.0)),
                      (4, ("G", 0.5, "O", 0.5))]:
        s = problems.demo_strip(13, 5, timeEnd=0.03)
        s.update(knlOrder=order, knlWidth=0.4)
        s["vfd"] = vk
        save(f"frame2d_matern{order}", s, s["tauVarVec"])

    # 2D: more target than deformed elements (TT_TD / DD branch, 2D/varifold.cu:518-536)
    s = problems.demo_strip(13, 5, timeEnd=0.03)
    c, u, v = s["tgt"]
    s["tgt"] = (np.concatenate([c, c + 0.05], 1), np.concatenate([u, u], 1), np.concatenate([v, v]))
    save("frame2d_target_larger", s, s["tauVarVec"])

    # 2D: CG cannot converge in 2 iterations -> objective DBL_MAX (2D/deform.cu:68-73)
    s = problems.demo_strip(13, 5, timeEnd=0.03)
    s.update(cgItrMax=2)
    save("frame2d_cgfail", s, s["tauVarVec"])

    # 2D: bottom penalty switched on (btmWgt > 0) with the K term
    s = problems.demo_strip(13, 5, timeEnd=0.03)
    s.update(btmWgt=5.0)
    save("frame2d_btm", s, s["tauVarVec"])

    # 3D: frame shell, icosphere level 1 x 3 node layers, Matern 1 (closed form), Gaussian/unoriented
    s = problems.frame_shell(1, 3, timeEnd=0.04, knlOrder=1)
    s["vfd"] = ("G", 0.4, "U", 0.6)
    save("frame3d_l1_m1", s, s["tauVarVec"])

    # 3D: level 2 x 4, Gaussian RKHS kernel, Binet, bottom penalty (projected-area quirk)
    s = problems.frame_shell(2, 4, timeEnd=0.03, knlOrder=-1)
    s.update(btmWgt=2.0, knlWidth=0.4)
    save("frame3d_l2_gauss_btm", s, s["tauVarVec"])

    # 3D: Matern orders 0, 2, 3, 4, varifold kernels C/L and O
    for order, vk in [(0, ("C", 0.4, "L", 1.0)), (2, ("G", 0.3, "O", 0.6)), (3, ("G", 0.5, "B", 1.0)),
                      (4, ("C", 0.5, "U", 0.9))]:
        s = problems.frame_shell(1, 3, timeEnd=0.02, knlOrder=order)
        s["vfd"] = vk
        save(f"frame3d_matern{order}", s, s["tauVarVec"])


if __name__ == "__main__":
    main()
