"""Call the reference's own MEX gateways compiled for the CPU (checker only).

TEST INFRASTRUCTURE ONLY.  Requires the libraries built by
oracle/build_ref.py from the reference tree, which exists only in the
development container; on other hosts ``available()`` is False and tests
fall back to the committed golden vectors.

Arguments are packed in the gateways' prhs order
(2D_frame/deformation.cu:24-50, 2D_frame/computeObjfcn.cu:25-59).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build_ref

_LIBS = {}


def available() -> bool:
    root = build_ref.reference_root()
    return bool(root) and os.path.isdir(os.path.join(root, "CUDA"))


def _lib(name: str):
    if name not in _LIBS:
        build_ref.build()
        l = C.CDLL(os.path.join(build_ref.OUT, f"libref_{name}.so"))
        l.sa_ref_wrap.restype = C.c_void_p
        l.sa_ref_wrap.argtypes = [C.c_size_t, C.c_size_t, C.c_void_p]
        l.sa_ref_data.restype = C.c_void_p
        l.sa_ref_data.argtypes = [C.c_void_p]
        l.sa_ref_free.argtypes = [C.c_void_p]
        l.sa_ref_error.restype = C.c_char_p
        l.sa_ref_mex.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_void_p]
        _LIBS[name] = l
    return _LIBS[name]


class _Args:
    def __init__(self, lib):
        self.lib, self.keep, self.ptrs = lib, [], []

    def mat(self, a, dtype):
        """numpy (k, n) C-order == MATLAB n x k column-major."""
        a = np.ascontiguousarray(np.asarray(a, dtype=dtype))
        if a.ndim == 1:
            m, n = a.shape[0], 1
        else:
            m, n = a.shape[-1], int(np.prod(a.shape[:-1]))
        self.keep.append(a)
        self.ptrs.append(self.lib.sa_ref_wrap(m, n, a.ctypes.data))

    def scalar(self, v):
        self.mat(np.array([float(v)]), np.float64)


def _common_head(A: _Args, spec: dict, tauVarMat):
    obj, D = spec["elmObj"], spec["dim"]
    tv = np.asarray(tauVarMat, dtype=np.float64)
    if tv.ndim == 1:
        tv = tv[None, :]                     # one column: nObj = 1
    A.mat(tv, np.float64)                    # prhs[0] tauVarMat (nVar x nObj)
    A.mat(spec["tauPrmVec"], np.float64)     # prhs[1]
    A.mat(spec["lmkIniMat"], np.float64)     # prhs[2] N x D
    for k in ["elmVtxMat", "vtxElmMat", "tanVtxMat" if D == 2 else "nmlVtxMat", "tsvVtxMat", "bdrVtxMat",
              "vtxBdrMat", "btmVtxMat", "vtxBtmMat", "femVtxMat", "femIfoMat"]:
        A.mat(obj[k], np.int32)              # prhs[3..12]
    return tv.shape[0]


def _common_tail(A: _Args, spec: dict):
    for k in ["ldmWgt", "knlOrder", "knlWidth", "knlEps"]:
        A.scalar(spec[k])
    A.mat(spec["modVec"], np.float64)
    A.scalar(spec["spdTanVal"]); A.scalar(spec["spdTsvVal"])
    A.mat(spec["ynkActPrmVec"], np.float64); A.mat(spec["reaActPrmVec"], np.float64)
    for k in ["btmWgt", "timeStp", "timeNum", "cgItrMax", "cgTolSqu"]:
        A.scalar(spec[k])


def _call(lib, A: _Args, nlhs: int):
    plhs = (C.c_void_p * nlhs)()
    prhs = (C.c_void_p * len(A.ptrs))(*A.ptrs)
    rc = lib.sa_ref_mex(nlhs, plhs, len(A.ptrs), prhs)
    for p in A.ptrs:
        lib.sa_ref_free(p)
    if rc != 0:
        raise RuntimeError(lib.sa_ref_error().decode())
    return plhs


def _take(lib, p, count):
    buf = (C.c_double * count).from_address(lib.sa_ref_data(p))
    out = np.frombuffer(buf, dtype=np.float64).copy()
    lib.sa_ref_free(p)
    return out


def deformation(spec: dict, tauVarMat):
    """Reference deformation_{2D,3D}_frame -> (lmkStk (T, D, N), tauMat (T, N), objVec)."""
    D = spec["dim"]
    lib = _lib(f"deformation_{D}D_frame")
    A = _Args(lib)
    _common_head(A, spec, tauVarMat)
    _common_tail(A, spec)
    nobj = np.asarray(tauVarMat).reshape(-1, np.asarray(tauVarMat).shape[-1]).shape[0]
    plhs = _call(lib, A, 3)
    N, T = spec["lmkIniMat"].shape[1], int(spec["timeNum"])
    lmk = _take(lib, plhs[0], N * D * T).reshape(T, D, N)
    tau = _take(lib, plhs[1], N * T).reshape(T, N)
    obj = _take(lib, plhs[2], nobj)
    return lmk, tau, obj


def compute_objfcn(spec: dict, tauVarMat):
    """Reference computeObjfcn_{2D,3D}_frame -> objVec (nObj,)."""
    D = spec["dim"]
    lib = _lib(f"computeObjfcn_{D}D_frame")
    A = _Args(lib)
    _common_head(A, spec, tauVarMat)
    obj = spec["elmObj"]
    A.mat(obj["vfdVtxMat"], np.int32)                    # prhs[13]
    cen, udir, vol = spec["tgt"]
    A.mat(cen, np.float64); A.mat(udir, np.float64); A.mat(vol, np.float64)   # prhs[14..16]
    ck, cw, dk, dw = spec["vfd"]
    A.scalar(ord(ck)); A.scalar(cw); A.scalar(ord(dk)); A.scalar(dw)         # prhs[17..20]
    _common_tail(A, spec)                                # prhs[21..34]
    nobj = np.asarray(tauVarMat).reshape(-1, np.asarray(tauVarMat).shape[-1]).shape[0]
    plhs = _call(lib, A, 1)
    return _take(lib, plhs[0], nobj)
