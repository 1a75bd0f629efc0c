"""Generate tests/golden/layered_pin_2d.npz: reference outputs that pin the
layered (isotropic) operators of the oracle where they coincide with the
reference's frame-model operators.

Run in the development container, where the reference tree exists:

    python tests/golden/make_layered_pin.py

The reference's own 2D kernels run on the CPU through oracle/ref_ops.cpp
(built by oracle/build_ref.py.build_ops).  The reference has no layered
model (CUDA/deformation.m:22-24 is empty), but on a mesh whose element
frames are orthonormal its operators reduce to the layered ones:

* elasticity: the frame stress (2D_frame/applyFrameElasticOperator.cu:7-39)
  with mu_tan = mu_tsv = mu_ang = 2 mu is sigma = 2 mu eps, the isotropic
  stress with lambda = 0;
* diffusion: spdTan = spdTsv = D (2D_frame/assembleFemMatrix.cu:5-59) is the
  isotropic D grad(phi_i) . grad(phi_j);
* mass, yank load and reaction load are the same operators given the same
  nodal activity (c u and rate u (1 - u) for the layered model).

Per-layer coefficients are pinned by linearity: the reference operator of
each layer's sub-mesh (its ring band of the annulus), scattered into the
full node numbering and summed over the layers.  Cases: a periodic annulus
(96 angles x 9 rings, 4 material layers; element frames tangential and
radial, orthonormal up to rounding) and a rotated, stretched strip (one
layer).  Every input array is stored beside the outputs.
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), "..", ".."))
sys.path.insert(0, ROOT)

from oracle import build_ref  # noqa: E402
from shape_atrophy_gb300 import mesh  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "layered_pin_2d.npz")
OBJ_KEYS = ["elmVtxMat", "vtxElmMat", "tanVtxMat", "tsvVtxMat", "bdrVtxMat", "vtxBdrMat", "btmVtxMat",
            "vtxBtmMat", "femVtxMat", "femIfoMat"]

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


def _d(a):
    return np.ascontiguousarray(a, dtype=np.float64).ctypes.data_as(_dp)


def _i(a):
    return np.ascontiguousarray(a, dtype=np.int32).ctypes.data_as(_ip)


class RefOps:
    def __init__(self):
        self.lib = C.CDLL(build_ref.build_ops())

    def elastic(self, obj, lmk, modVec, v):
        N, E = lmk.shape[1], obj["elmVtxMat"].shape[1]
        y = np.zeros((2, N))
        keep = [np.ascontiguousarray(x) for x in (lmk, v)]
        self.lib.refop_elastic(N, E, _d(keep[0]), _i(obj["elmVtxMat"]), _i(obj["vtxElmMat"]), _i(obj["tanVtxMat"]),
                               _i(obj["tsvVtxMat"]), _d(np.asarray(modVec, float)), _d(keep[1]), _d(y))
        return y

    def fem_matrix(self, obj, lmk, spd):
        N, E, Z = lmk.shape[1], obj["elmVtxMat"].shape[1], obj["femVtxMat"].shape[1]
        ppd, ggd = np.zeros((N, N)), np.zeros((N, N))   # [col, row]: column-major N x N
        self.lib.refop_fem_matrix(N, E, Z, _d(lmk), _i(obj["elmVtxMat"]), _i(obj["tanVtxMat"]),
                                  _i(obj["tsvVtxMat"]), _i(obj["femVtxMat"]), _i(obj["femIfoMat"]),
                                  C.c_double(spd), C.c_double(spd), _d(ppd), _d(ggd))
        return ppd.T.copy(), ggd.T.copy()                # [row, col]

    def fem_vector(self, obj, lmk, act):
        N, E = lmk.shape[1], obj["elmVtxMat"].shape[1]
        y = np.zeros(N)
        self.lib.refop_fem_vector(N, E, _d(lmk), _i(obj["elmVtxMat"]), _i(obj["vtxElmMat"]), _d(act), _d(y))
        return y

    def yank(self, obj, lmk, act):
        N, E = lmk.shape[1], obj["elmVtxMat"].shape[1]
        y = np.zeros((2, N))
        self.lib.refop_yank(N, E, obj["bdrVtxMat"].shape[1], _d(lmk), _i(obj["elmVtxMat"]), _i(obj["vtxElmMat"]),
                            _i(obj["bdrVtxMat"]), _i(obj["vtxBdrMat"]), _d(act), _d(y))
        return y

    def penalty(self, obj, lmk, v):
        N = lmk.shape[1]
        y = np.zeros((2, N))
        self.lib.refop_penalty(N, obj["btmVtxMat"].shape[1], obj["vtxBtmMat"].shape[1], _d(lmk),
                               _i(obj["btmVtxMat"]), _i(obj["vtxBtmMat"]), _d(v), _d(y))
        return y


def csr_values(dense, obj):
    fv = obj["femVtxMat"]
    vals = dense[fv[0], fv[1]]
    mask = np.ones_like(dense, dtype=bool)
    mask[fv[0], fv[1]] = False
    assert not np.any(dense[mask]), "reference matrix has entries outside the femVtxMat pattern"
    return vals


def annulus_case(R, rng):
    A, rings, L = 96, 9, 4
    obj = mesh.generate_element_object_2d(A, rings, [1, rings], periodic=True)
    lmk = mesh.annulus_nodes(A, rings, 0.6, 1.0)
    N = lmk.shape[1]
    bands = rings - 1
    band_layer = np.minimum((L * np.arange(bands)) // bands, L - 1)
    elmLyr = mesh.element_layers(obj["elmVtxMat"].shape[1], obj["elmPerLayer"], band_layer)
    mu = np.array([0.5, 1.0, 2.0, 4.0])
    D = np.array([0.01, 0.02, 0.04, 0.08])
    v = rng.standard_normal((2, N))
    tau = rng.uniform(0.0, 1.0, N)
    c, rate = 0.5, 2.0
    y = np.zeros((2, N))
    ppd, ggd = np.zeros((N, N)), np.zeros((N, N))
    for l in range(L):
        b = np.nonzero(band_layer == l)[0]
        r0, r1 = int(b[0]), int(b[-1]) + 1                  # rings r0 .. r1 of the layer's bands
        sub = mesh.generate_element_object_2d(A, r1 - r0 + 1, [1, r1 - r0 + 1], periodic=True)
        off = r0 * A
        per = obj["elmPerLayer"]
        np.testing.assert_array_equal(obj["elmVtxMat"][:, r0 * per:r1 * per], sub["elmVtxMat"] + off)
        nodes = slice(off, off + (r1 - r0 + 1) * A)
        y[:, nodes] += R.elastic(sub, lmk[:, nodes], [2 * mu[l]] * 3, v[:, nodes])
        p, g = R.fem_matrix(sub, lmk[:, nodes], D[l])
        ppd[nodes, nodes] += p
        ggd[nodes, nodes] += g
    out = {"obj": obj, "lmk": lmk, "elmLyrVec": elmLyr, "mu": mu, "D": D, "v": v, "tau": tau, "c": c, "rate": rate,
           "ref_elastic": y, "ref_ppd": csr_values(ppd, obj), "ref_ggd": csr_values(ggd, obj),
           "ref_yank": R.yank(obj, lmk, c * tau), "ref_rea": R.fem_vector(obj, lmk, (rate * tau) * (1.0 - tau)),
           "ref_pnl": R.penalty(obj, lmk, v)}
    return out


def strip_case(R, rng):
    nx, ny = 21, 7
    obj = mesh.generate_element_object_2d(nx, ny, [1, ny])
    base = mesh.strip_nodes(nx, ny, x=(-3.0, 3.0), y=(-0.7, 0.9))
    th = 0.3
    rot = np.array([[np.cos(th), -np.sin(th)], [np.sin(th), np.cos(th)]])
    lmk = rot @ base
    N = lmk.shape[1]
    mu, D = np.array([0.7]), np.array([0.05])
    v = rng.standard_normal((2, N))
    tau = rng.uniform(0.0, 1.0, N)
    c, rate = 0.8, 1.5
    p, g = R.fem_matrix(obj, lmk, D[0])
    return {"obj": obj, "lmk": lmk, "elmLyrVec": np.zeros(obj["elmVtxMat"].shape[1], np.int32), "mu": mu, "D": D,
            "v": v, "tau": tau, "c": c, "rate": rate, "ref_elastic": R.elastic(obj, lmk, [2 * mu[0]] * 3, v),
            "ref_ppd": csr_values(p, obj), "ref_ggd": csr_values(g, obj), "ref_yank": R.yank(obj, lmk, c * tau),
            "ref_rea": R.fem_vector(obj, lmk, (rate * tau) * (1.0 - tau)), "ref_pnl": R.penalty(obj, lmk, v)}


def main():
    R = RefOps()
    rng = np.random.default_rng(20261204)
    data = {}
    for name, case in (("annulus", annulus_case(R, rng)), ("strip", strip_case(R, rng))):
        for k, val in case.items():
            if k == "obj":
                for ok in OBJ_KEYS:
                    data[f"{name}_obj_{ok}"] = val[ok]
            else:
                data[f"{name}_{k}"] = np.asarray(val)
        print(name, "N", case["lmk"].shape[1], "E", case["obj"]["elmVtxMat"].shape[1])
    np.savez_compressed(OUT, **data)
    print("wrote", OUT)


if __name__ == "__main__":
    main()
