"""ctypes front end of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use
this module, as the checker.  The product never imports it.

A problem is the same ``spec`` dict the product API takes (see
shape_atrophy_gb300.api.make_spec); this module packs it into the C
``orc_problem`` struct of oracle.h.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build_oracle

_LIBS = {}

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


class OrcProblem(C.Structure):
    _fields_ = [
        ("dim", C.c_int), ("lmkNum", C.c_int), ("elmNum", C.c_int), ("nzrNum", C.c_int),
        ("btmLmkNum", C.c_int), ("btmElmNum", C.c_int), ("vfdElmNum", C.c_int), ("tgtElmNum", C.c_int),
        ("vtxElmCols", C.c_int), ("vtxBtmCols", C.c_int), ("femIfoCols", C.c_int), ("vfdIfoCols", C.c_int),
        ("lmkIniMat", _dp), ("elmVtxMat", _ip), ("vtxElmMat", _ip), ("frmVtxMat", _ip), ("tsvVtxMat", _ip),
        ("btmVtxMat", _ip), ("vtxBtmMat", _ip), ("femVtxMat", _ip), ("femIfoMat", _ip), ("vfdVtxMat", _ip),
        ("vfdIfoMat", _ip), ("tgtCenPosMat", _dp), ("tgtUniDirMat", _dp), ("tgtElmVolVec", _dp),
        ("cenKnlType", C.c_char), ("dirKnlType", C.c_char), ("cenKnlWidth", C.c_double), ("dirKnlWidth", C.c_double),
        ("elaType", C.c_int), ("lyrNum", C.c_int), ("elmLyrVec", _ip), ("modVec", _dp), ("spdLyrVec", _dp),
        ("spdTanVal", C.c_double), ("spdTsvVal", C.c_double), ("ynkActPrmVec", _dp), ("reaActPrmVec", _dp),
        ("tauPrmVec", _dp), ("ldmWgt", C.c_double), ("knlOrder", C.c_int), ("knlWidth", C.c_double),
        ("knlEps", C.c_double), ("btmWgt", C.c_double), ("timeStp", C.c_double), ("timeNum", C.c_int),
        ("cgItrMax", C.c_int), ("cgTolSqu", C.c_double), ("rdItrMax", C.c_int), ("rdTolSqu", C.c_double),
        ("velocityGuess", C.c_int),
    ]


def lib(dim: int, fast: bool = False):
    """The parity build of the oracle, or with fast=True the -O3 -march=native timing build (same results)."""
    key = (dim, fast)
    if key not in _LIBS:
        paths = build_oracle.build()
        if fast:
            paths = build_oracle.fast_paths()
        l = C.CDLL(paths[0 if dim == 2 else 1])
        l.orc_forward.restype = C.c_int
        l.orc_forward_timed.restype = C.c_int
        l.orc_varifold.restype = C.c_double
        l.orc_dsum.restype = C.c_double
        _LIBS[key] = l
    return _LIBS[key]


def _d(a):
    return a.ctypes.data_as(_dp) if a is not None else None


def _i(a):
    return a.ctypes.data_as(_ip) if a is not None else None


class Problem:
    """Holds the numpy arrays alive and the packed struct."""

    def __init__(self, spec: dict, fast: bool = False):
        self.spec = spec
        obj = spec["elmObj"]
        D = spec["dim"]
        keep = []

        def f64(x):
            a = np.ascontiguousarray(np.asarray(x, dtype=np.float64))
            keep.append(a)
            return a

        def i32(x):
            a = np.ascontiguousarray(np.asarray(x, dtype=np.int32))
            keep.append(a)
            return a

        p = OrcProblem()
        lmk = f64(spec["lmkIniMat"])
        N = lmk.shape[1]
        elm = i32(obj["elmVtxMat"])
        p.dim, p.lmkNum, p.elmNum = D, N, elm.shape[1]
        fv = i32(obj["femVtxMat"]); fi = i32(obj["femIfoMat"])
        ve = i32(obj["vtxElmMat"]); vb = i32(obj["vtxBtmMat"]); bt = i32(obj["btmVtxMat"])
        p.nzrNum = fv.shape[1]
        p.btmLmkNum, p.btmElmNum = vb.shape[1], bt.shape[1]
        p.vtxElmCols, p.vtxBtmCols, p.femIfoCols = ve.shape[0], vb.shape[0], fi.shape[0]
        p.lmkIniMat, p.elmVtxMat, p.vtxElmMat = _d(lmk), _i(elm), _i(ve)
        p.frmVtxMat = _i(i32(obj["tanVtxMat"] if D == 2 else obj["nmlVtxMat"]))
        p.tsvVtxMat = _i(i32(obj["tsvVtxMat"]))
        p.btmVtxMat, p.vtxBtmMat, p.femVtxMat, p.femIfoMat = _i(bt), _i(vb), _i(fv), _i(fi)
        vd = i32(obj["vfdVtxMat"])
        p.vfdElmNum = vd.shape[1]
        p.vfdVtxMat = _i(vd)
        if "vfdIfoMat" in obj:
            vi = i32(obj["vfdIfoMat"])
            p.vfdIfoMat, p.vfdIfoCols = _i(vi), vi.shape[0]
        tgt = spec.get("tgt")
        if tgt is not None:
            tc, tu, tv = f64(tgt[0]), f64(tgt[1]), f64(tgt[2])
            p.tgtElmNum = tv.shape[0]
            p.tgtCenPosMat, p.tgtUniDirMat, p.tgtElmVolVec = _d(tc), _d(tu), _d(tv)
        vfd = spec.get("vfd") or ("G", 1.0, "B", 1.0)
        p.cenKnlType, p.cenKnlWidth = vfd[0].encode(), float(vfd[1])
        p.dirKnlType, p.dirKnlWidth = vfd[2].encode(), float(vfd[3])
        p.elaType = 0 if spec["elaType"] == "frame" else 1
        if p.elaType == 1:
            ly = i32(spec["elmLyrVec"])
            p.elmLyrVec = _i(ly)
            sp = f64(spec["spdLyrVec"])
            p.spdLyrVec, p.lyrNum = _d(sp), sp.shape[0]
        p.modVec = _d(f64(spec["modVec"]))
        p.spdTanVal, p.spdTsvVal = float(spec.get("spdTanVal", 0.0)), float(spec.get("spdTsvVal", 0.0))
        p.ynkActPrmVec = _d(f64(spec["ynkActPrmVec"]))
        p.reaActPrmVec = _d(f64(spec["reaActPrmVec"]))
        p.tauPrmVec = _d(f64(spec.get("tauPrmVec", [0.0, 0.0])))
        p.ldmWgt, p.knlOrder = float(spec["ldmWgt"]), int(spec["knlOrder"])
        p.knlWidth, p.knlEps = float(spec["knlWidth"]), float(spec["knlEps"])
        p.btmWgt, p.timeStp, p.timeNum = float(spec["btmWgt"]), float(spec["timeStp"]), int(spec["timeNum"])
        p.cgItrMax, p.cgTolSqu = int(spec["cgItrMax"]), float(spec["cgTolSqu"])
        p.rdItrMax, p.rdTolSqu = int(spec.get("rdItrMax", 10000)), float(spec.get("rdTolSqu", 1e-26))
        g = spec.get("velocityGuess", "cubic")     # the layered model's default start (polynomial order 3)
        p.velocityGuess = {"previous": 0, "extrapolate": 1, "linear": 1, "quadratic": 2, "cubic": 3, "quartic": 4,
                           "quintic": 5}[g] if isinstance(g, str) else int(g)
        if not 0 <= p.velocityGuess <= 5:
            raise ValueError("velocityGuess order outside 0 .. 5")
        self.p = p
        self.keep = keep
        self.dim, self.N = D, N
        self.lib = lib(D, fast)

    # -- full model ------------------------------------------------------
    def forward(self, tauVarVec, with_obj: bool = False):
        """Whole trajectory: dict(status, lmkStk (T, D, N), tauMat (T, N), obj, cgItr (T-1,), stepSec (T-1,))
        -- stepSec is the wall time of each time step."""
        N, D, T = self.N, self.dim, self.p.timeNum
        lmk = np.zeros((T, D, N))
        tau = np.zeros((T, N))
        obj = C.c_double(0.0)
        itr = np.zeros(max(T - 1, 1), dtype=np.int32)
        sec = np.zeros(max(T - 1, 1))
        tv = np.ascontiguousarray(np.asarray(tauVarVec, dtype=np.float64))
        st = self.lib.orc_forward_timed(C.byref(self.p), _d(tv), _d(lmk), _d(tau),
                                        C.byref(obj) if with_obj else None, _i(itr), _d(sec))
        return dict(status=st, lmkStk=lmk, tauMat=tau, obj=obj.value if with_obj else None, cgItr=itr,
                    stepSec=sec)

    # -- operators -------------------------------------------------------
    def _vec(self, name, lmk, x, out_shape):
        y = np.zeros(out_shape)
        getattr(self.lib, name)(C.byref(self.p), _d(np.ascontiguousarray(lmk, dtype=np.float64)),
                                _d(np.ascontiguousarray(x, dtype=np.float64)), _d(y))
        return y

    def elastic(self, lmk, v):
        return self._vec("orc_elastic_apply", lmk, v, (self.dim, self.N))

    def penalty(self, lmk, v):
        return self._vec("orc_penalty_apply", lmk, v, (self.dim, self.N))

    def yank(self, lmk, tau):
        return self._vec("orc_yank", lmk, tau, (self.dim, self.N))

    def reaction_load(self, lmk, tau):
        return self._vec("orc_reaction_load", lmk, tau, (self.N,))

    def elastic_diag(self, lmk):
        y = np.zeros((self.dim, self.N))
        self.lib.orc_elastic_diag(C.byref(self.p), _d(np.ascontiguousarray(lmk, dtype=np.float64)), _d(y))
        return y

    def elastic_blocks(self, lmk, inverse: bool = False):
        """(N, D, D): every node's diagonal block of E + btmWgt P, or its inverse."""
        y = np.zeros((self.dim, self.dim, self.N))
        self.lib.orc_elastic_blocks(C.byref(self.p), _d(np.ascontiguousarray(lmk, dtype=np.float64)),
                                    C.c_int(1 if inverse else 0), _d(y))
        return np.moveaxis(y, -1, 0)

    def fem_csr(self, lmk):
        Z = self.p.nzrNum
        a, b = np.zeros(Z), np.zeros(Z)
        self.lib.orc_fem_csr(C.byref(self.p), _d(np.ascontiguousarray(lmk, dtype=np.float64)), _d(a), _d(b))
        return a, b

    def kernel_matrix(self, lmk):
        K = np.zeros((self.N, self.N))   # K[j, i] = column-major (i, j)
        self.lib.orc_kernel_matrix(C.byref(self.p), _d(np.ascontiguousarray(lmk, dtype=np.float64)), _d(K))
        return K

    def initial_tau(self, tauVarVec):
        t = np.zeros(self.N)
        self.lib.orc_initial_tau(C.byref(self.p), _d(np.ascontiguousarray(tauVarVec, dtype=np.float64)), _d(t))
        return t

    def frame(self, lmk):
        E = self.p.elmNum
        a, s = np.zeros((self.dim, E)), np.zeros((self.dim, E))
        self.lib.orc_frame(C.byref(self.p), _d(np.ascontiguousarray(lmk, dtype=np.float64)), _d(a), _d(s))
        return a, s

    def activity(self, tau, kind: str):
        tau = np.ascontiguousarray(tau, dtype=np.float64)
        f = np.zeros_like(tau)
        fn = self.lib.orc_yank_activity if kind == "yank" else self.lib.orc_reaction_activity
        fn(C.byref(self.p), _d(tau), _d(f), C.c_int(tau.size))
        return f

    def varifold(self, lmk, grad: bool = False):
        g = np.zeros((self.dim, self.N)) if grad else None
        v = self.lib.orc_varifold(C.byref(self.p), _d(np.ascontiguousarray(lmk, dtype=np.float64)), _d(g))
        return (v, g) if grad else v


def dsum(vec) -> float:
    v = np.ascontiguousarray(vec, dtype=np.float64)
    return lib(2).orc_dsum(_d(v), C.c_int(v.size))


def besselk(x: float):
    f0, f1 = C.c_double(), C.c_double()
    lib(2).orc_besselk(C.c_double(x), C.byref(f0), C.byref(f1))
    return f0.value, f1.value
