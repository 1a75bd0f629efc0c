"""Ready-made problem specs.

A *spec* is a plain dict holding everything one forward solve needs: the
initial nodes ``lmkIniMat`` (D, N), the element object ``elmObj`` (see
mesh.py), model parameters in the reference's argument vocabulary, and
optionally a varifold target ``tgt`` = (cenPosMat (D, Vt), uniDirMat (D, Vt),
elmVolVec (Vt,)) with kernel choice ``vfd`` = (cenKnlType, cenKnlWidth,
dirKnlType, dirKnlWidth).

* ``demo_strip``   -- the reference demo (demo/run_demo.m:1-28) on a
  lyrNdeNum x lyrCntNum strip of [-3,3] x [-1,1] (frame elasticity, 2D).
* ``frame_shell``  -- frame elasticity on a small icosphere shell (3D).
* ``annulus_layered`` -- layered 2D annulus: 16 radial x 256 angular nodes,
  7680 triangles, 4 layers, Fisher-KPP, Gaussian bump, block-Jacobi PCG 1e-8,
  Gaussian varifold (width 0.1) on inner+outer boundary (512 segments).
* ``shell_layered`` -- layered 3D shell: icosphere level 5 x 9 node layers
  (92178 nodes, 491520 tets), 3 material layers, 100 steps dt 0.01,
  block-Jacobi PCG 1e-8, Matern-3/2 varifold (width 0.08) on the 20480 outer
  triangles.

Choices the layered workloads leave open are fixed here: bottom penalty weight ``btmWgt`` (anchors the inner boundary;
pure elasticity has rigid-body null modes), the direction kernel ('B',
Binet), the bump centre (outer surface, angle 0 / +z pole) and the
target (seeded smooth displacement of the initial boundary).
"""
from __future__ import annotations

import numpy as np

from . import mesh


def _attach_target(spec: dict, amplitude: float, seed: int, vfd):
    obj = spec["elmObj"]
    lmk = spec["lmkIniMat"]
    obj["vfdIfoMat"] = mesh.vfd_gradient_table(obj["vfdVtxMat"], lmk.shape[1])
    tgt_nodes = mesh.smooth_displacement(lmk, amplitude, seed)
    spec["tgt"] = mesh.varifold_target(tgt_nodes, obj["vfdVtxMat"])
    spec["vfd"] = vfd
    return spec


def demo_strip(lyrNdeNum: int = 101, lyrCntNum: int = 31, timeEnd: float = 1.0, timeStp: float = 0.01,
               cgTolVal: float = 1e-12, target_seed: int = 7) -> dict:
    """Reference demo parameters (demo/run_demo.m:1-28) on a strip mesh."""
    obj = mesh.generate_element_object_2d(lyrNdeNum, lyrCntNum, [1, lyrCntNum])
    lmk = mesh.strip_nodes(lyrNdeNum, lyrCntNum)
    actMax = 4.0
    spec = dict(
        dim=2, elaType="frame", lmkIniMat=lmk, elmObj=obj,
        tauVarVec=np.array([0.5, 0.5, 0.2, 0.3]), tauPrmVec=np.array([1.0]),
        modVec=3.0 * np.array([1.0, 1.0, 5.0]), spdTanVal=0.625, spdTsvVal=0.125,
        ynkActPrmVec=np.array([0.01, 1.0, actMax, 0.5]), reaActPrmVec=np.array([0.01, 1.0, actMax, 0.5, 0.3]),
        ldmWgt=1e-2, knlOrder=3, knlWidth=0.2, knlEps=1e-10, btmWgt=0.0,
        timeStp=timeStp, timeNum=int(np.floor(timeEnd / timeStp + 1e-9)) + 1,
        cgItrMax=10000, cgTolSqu=cgTolVal ** 2,
    )
    return _attach_target(spec, 0.05, target_seed, ("G", 0.5, "B", 1.0))


def frame_shell(level: int = 2, lyrCntNum: int = 4, timeEnd: float = 0.1, timeStp: float = 0.01,
                cgTolVal: float = 1e-12, knlOrder: int = 1, target_seed: int = 11) -> dict:
    """Frame elasticity (3D reference moduli [ldT, muT, muS, muA]) on a small shell."""
    surf, tri, tet, nml, tsv, obj = mesh.shell_element_object(level, lyrCntNum)
    lmk = mesh.shell_nodes(surf, lyrCntNum, 0.7, 1.0)
    spec = dict(
        dim=3, elaType="frame", lmkIniMat=lmk, elmObj=obj,
        tauVarVec=np.array([0.0, 0.0, 1.0, 0.5]), tauPrmVec=np.array([0.6, 1.0]),
        modVec=np.array([1.0, 1.0, 1.0, 5.0]), spdTanVal=0.625, spdTsvVal=0.125,
        ynkActPrmVec=np.array([0.01, 1.0, 4.0, 0.5]), reaActPrmVec=np.array([0.01, 1.0, 4.0, 0.5, 0.3]),
        ldmWgt=1e-2, knlOrder=knlOrder, knlWidth=0.3, knlEps=1e-10, btmWgt=0.0,
        timeStp=timeStp, timeNum=int(np.floor(timeEnd / timeStp + 1e-9)) + 1,
        cgItrMax=10000, cgTolSqu=cgTolVal ** 2,
    )
    return _attach_target(spec, 0.03, target_seed, ("G", 0.3, "B", 1.0))


def annulus_layered(angNum: int = 256, radNum: int = 16, steps: int = 50, timeStp: float = 0.02,
                    cgTolVal: float = 1e-8, btmWgt: float = 10.0, target_seed: int = 1, layers: int = 4,
                    native: bool = False) -> dict:
    """Layered 2D annulus, radii 0.6-1.0 (periodic in angle); ``layers`` equal radial material layers with
    (lambda, mu) = (2^k, 2^k / 2) and D = 0.01 * 2^k, k = 0 .. layers-1 (the default 4 layers: (1, 0.5) ..
    (8, 4), D = 0.01 .. 0.08).  native=True builds the element object with the C library (identical arrays)."""
    if native:
        from . import api
        obj = api.build_element_object_2d(angNum, radNum, [1, radNum], periodic=True)
    else:
        obj = mesh.generate_element_object_2d(angNum, radNum, [1, radNum], periodic=True)
    lmk = mesh.annulus_nodes(angNum, radNum, 0.6, 1.0)
    E = obj["elmVtxMat"].shape[1]
    rings = radNum - 1
    L = int(layers)
    ring_layer = np.minimum((L * np.arange(rings)) // rings, L - 1)
    obj["elmLyrVec"] = mesh.element_layers(E, obj["elmPerLayer"], ring_layer)
    lam = 2.0 ** np.arange(L)
    spec = dict(
        dim=2, elaType="isotropic", lmkIniMat=lmk, elmObj=obj, elmLyrVec=obj["elmLyrVec"],
        tauVarVec=np.array([1.0, 0.0, 1.0, 0.1]),          # centre (r=1, angle 0), height 1, sigma 0.1
        tauPrmVec=np.array([0.0]),
        modVec=np.column_stack([lam, lam / 2]).reshape(-1),
        spdLyrVec=0.01 * lam,
        ynkActPrmVec=np.array([0.5]), reaActPrmVec=np.array([2.0]),
        ldmWgt=0.0, knlOrder=1, knlWidth=0.1, knlEps=0.0, btmWgt=btmWgt,
        timeStp=timeStp, timeNum=steps + 1, cgItrMax=20000, cgTolSqu=cgTolVal ** 2,
        rdItrMax=20000, rdTolSqu=cgTolVal ** 2,
    )
    return _attach_target(spec, 0.05, target_seed, ("G", 0.1, "B", 1.0))


def shell_layered(level: int = 5, lyrCntNum: int = 9, steps: int = 100, timeStp: float = 0.01,
                  cgTolVal: float = 1e-8, btmWgt: float = 10.0, target_seed: int = 2,
                  material_of_prism=None, native: bool = False) -> dict:
    """Layered 3D shell, radii 0.7-1.0; default = icosphere 5 x 8 prism layers.
    native=True builds the element object with the C library (identical arrays)."""
    surf, tri, tet, nml, tsv, obj = mesh.shell_element_object(level, lyrCntNum, native=native)
    lmk = mesh.shell_nodes(surf, lyrCntNum, 0.7, 1.0)
    E = obj["elmVtxMat"].shape[1]
    nl = lyrCntNum - 1
    if material_of_prism is None:
        # three material layers: prisms 1-3, 4-6, 7-8 of 8 (scaled for other counts)
        material_of_prism = np.minimum((3 * np.arange(nl)) // nl, 2) if nl != 8 else [0, 0, 0, 1, 1, 1, 2, 2]
    obj["elmLyrVec"] = mesh.element_layers(E, obj["elmPerLayer"], material_of_prism)
    spec = dict(
        dim=3, elaType="isotropic", lmkIniMat=lmk, elmObj=obj, elmLyrVec=obj["elmLyrVec"],
        tauVarVec=np.array([0.0, 0.0, 1.0, 1.0, 0.15]),     # bump centre at the outer +z pole
        tauPrmVec=np.array([0.0, 0.0]),
        modVec=np.array([1.0, 0.5, 3.0, 1.5, 9.0, 4.5]),
        spdLyrVec=np.array([0.01, 0.03, 0.09]),
        ynkActPrmVec=np.array([0.5]), reaActPrmVec=np.array([2.0]),
        ldmWgt=0.0, knlOrder=1, knlWidth=0.1, knlEps=0.0, btmWgt=btmWgt,
        timeStp=timeStp, timeNum=steps + 1, cgItrMax=20000, cgTolSqu=cgTolVal ** 2,
        rdItrMax=20000, rdTolSqu=cgTolVal ** 2,
    )
    return _attach_target(spec, 0.03, target_seed, ("M", 0.08, "B", 1.0))
