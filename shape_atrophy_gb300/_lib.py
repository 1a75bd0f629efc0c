"""ctypes binding of include/shape_atrophy_gb300.h.

The library is built in-tree by shape_atrophy_gb300.build (called from
__graft_entry__.build()).  There is no fallback: if the library is missing
or no GPU is visible, load() raises.
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

_LIB = None

_ip = C.POINTER(C.c_int)
_dp = C.POINTER(C.c_double)

SA_OK, SA_ERR_ARG, SA_ERR_CUDA, SA_ERR_UNSUPPORTED = 0, 1, 2, 3
SA_ERR_NOT_CONVERGED, SA_ERR_BREAKDOWN, SA_ERR_NONFINITE, SA_ERR_TIMEOUT = 4, 5, 6, 7
SA_CG_AUTO, SA_CG_PERSISTENT, SA_CG_TWO_KERNEL, SA_CG_PERSISTENT_GLOBAL = 0, 1, 2, 3
SA_GUESS_PREVIOUS, SA_GUESS_EXTRAPOLATE, SA_GUESS_QUADRATIC = 0, 1, 2
SA_ELA_FRAME, SA_ELA_ISOTROPIC = 0, 1
SA_PREC_FP64, SA_PREC_MIXED = 0, 1


class ElementObject(C.Structure):
    _fields_ = [
        ("dim", C.c_int), ("lmkNum", C.c_int), ("elmNum", C.c_int),
        ("elmVtxMat", _ip), ("vtxElmMat", _ip), ("vtxElmCols", C.c_int),
        ("frmVtxMat", _ip), ("tsvVtxMat", _ip),
        ("bdrVtxMat", _ip), ("bdrElmNum", C.c_int), ("vtxBdrMat", _ip), ("vtxBdrCols", C.c_int),
        ("btmVtxMat", _ip), ("btmElmNum", C.c_int), ("vtxBtmMat", _ip), ("btmLmkNum", C.c_int),
        ("vtxBtmCols", C.c_int), ("femVtxMat", _ip), ("nzrNum", C.c_int), ("femIfoMat", _ip),
        ("femIfoCols", C.c_int), ("vfdVtxMat", _ip), ("vfdElmNum", C.c_int), ("vfdIfoMat", _ip),
        ("vfdIfoCols", C.c_int), ("elmLyrVec", _ip),
    ]


class Params(C.Structure):
    _fields_ = [
        ("elaType", C.c_int), ("precision", C.c_int), ("tauPrmVec", _dp), ("tauPrmNum", C.c_int),
        ("ldmWgt", C.c_double), ("knlOrder", C.c_int), ("knlWidth", C.c_double), ("knlEps", C.c_double),
        ("modVec", _dp), ("modNum", C.c_int), ("spdTanVal", C.c_double), ("spdTsvVal", C.c_double),
        ("spdLyrVec", _dp), ("lyrNum", C.c_int), ("ynkActPrmVec", _dp), ("reaActPrmVec", _dp),
        ("btmWgt", C.c_double), ("timeStp", C.c_double), ("timeNum", C.c_int), ("cgItrMax", C.c_int),
        ("cgTolSqu", C.c_double), ("rdItrMax", C.c_int), ("rdTolSqu", C.c_double), ("cgKernel", C.c_int),
        ("velocityGuess", C.c_int),
    ]


class Target(C.Structure):
    _fields_ = [
        ("cenPosMat", _dp), ("uniDirMat", _dp), ("elmVolVec", _dp), ("tgtElmNum", C.c_int),
        ("cenKnlType", C.c_char), ("cenKnlWidth", C.c_double), ("dirKnlType", C.c_char),
        ("dirKnlWidth", C.c_double),
    ]


class SolveInfo(C.Structure):
    _fields_ = [
        ("status", C.c_int), ("cgIterTotal", C.c_int), ("rdIterTotal", C.c_int), ("cgIterMax", C.c_int),
        ("invertedElements", C.c_int), ("elapsedMs", C.c_double), ("kernelLaunches", C.c_longlong),
    ]


class ServerCounters(C.Structure):
    _fields_ = [
        ("submitted", C.c_longlong), ("completed", C.c_longlong), ("failed", C.c_longlong),
        ("queued", C.c_int), ("running", C.c_int), ("bytesInUse", C.c_double), ("peakBytes", C.c_double),
        ("ticks", C.c_longlong), ("busyMs", C.c_double),
    ]


SA_REQ_QUEUED, SA_REQ_RUNNING, SA_REQ_DONE, SA_REQ_FAILED = 0, 1, 2, 3


def library_path() -> str:
    return _build.LIB


def load():
    """Load the CUDA library (raises if it has not been built)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = library_path()
    if not os.path.exists(path):
        raise RuntimeError(f"CUDA library not built: {path} (run __graft_entry__.build())")
    lib = C.CDLL(path)
    vp = C.c_void_p
    lib.sa_create.argtypes = [C.POINTER(vp), C.c_int]
    lib.sa_destroy.argtypes = [vp]
    lib.sa_error_message.argtypes = [vp]
    lib.sa_error_message.restype = C.c_char_p
    lib.sa_forward.argtypes = [vp, C.POINTER(ElementObject), _dp, C.POINTER(Params), C.POINTER(Target), _dp,
                               C.c_int, C.c_int, _dp, _dp, _dp, C.POINTER(SolveInfo)]
    lib.sa_varifold.argtypes = [vp, C.POINTER(ElementObject), _dp, C.POINTER(Target), C.c_int, _dp, _dp]
    lib.sa_session_create.argtypes = [vp, C.POINTER(ElementObject), _dp, C.POINTER(Params), C.POINTER(Target),
                                      _dp, C.c_int, C.POINTER(vp)]
    lib.sa_session_step.argtypes = [vp, C.c_int, _ip]
    lib.sa_session_state.argtypes = [vp, _dp, _dp, _ip]
    lib.sa_session_stream.argtypes = [vp, C.c_int, C.c_int, _dp, _dp, C.c_int, _ip, _ip]
    lib.sa_objective_gradient.argtypes = [vp, C.POINTER(ElementObject), _dp, C.POINTER(Params), C.POINTER(Target),
                                          _dp, C.c_int, _dp, _dp, C.POINTER(SolveInfo)]
    lib.sa_objective_adjoint.argtypes = [vp, C.POINTER(ElementObject), _dp, C.POINTER(Params), C.POINTER(Target),
                                         _dp, C.c_int, _dp, _dp, _dp, _dp, _dp, C.POINTER(SolveInfo)]
    lib.sa_session_objective.argtypes = [vp, _dp]
    lib.sa_session_info.argtypes = [vp, C.POINTER(SolveInfo)]
    lib.sa_session_profile.argtypes = [vp, C.c_int, _dp, C.POINTER(C.c_longlong), _dp, _dp]
    lib.sa_session_destroy.argtypes = [vp]
    lib.sa_tri2tetra.argtypes = [_ip, C.c_int, C.c_int, _ip, _ip, _ip]
    lib.sa_build_element_object_3d.argtypes = [_ip, C.c_int, _ip, C.c_int, _ip, _ip, _ip, C.c_int, C.POINTER(vp)]
    lib.sa_build_element_object_2d.argtypes = [C.c_int, C.c_int, _ip, C.c_int, C.c_int, C.POINTER(vp)]
    lib.sa_elmobj_view.argtypes = [vp, C.POINTER(ElementObject)]
    lib.sa_elmobj_layers.argtypes = [vp, _ip, _ip, _ip]
    lib.sa_elmobj_free.argtypes = [vp]
    lib.sa_server_create.argtypes = [vp, C.c_double, C.c_int, C.POINTER(vp)]
    lib.sa_server_submit.argtypes = [vp, C.POINTER(ElementObject), _dp, C.POINTER(Params), C.POINTER(Target), _dp,
                                     C.c_int, C.POINTER(C.c_longlong)]
    lib.sa_server_poll.argtypes = [vp, C.c_longlong, _ip]
    lib.sa_server_wait.argtypes = [vp, C.c_longlong, C.c_double, _ip]
    lib.sa_server_result.argtypes = [vp, C.c_longlong, _dp, _dp, _dp, C.POINTER(SolveInfo), _dp]
    lib.sa_server_stats.argtypes = [vp, C.POINTER(ServerCounters)]
    lib.sa_server_destroy.argtypes = [vp]
    lib.sa_set_tuning.argtypes = [C.c_char_p, C.c_int]
    lib.sa_get_tuning.argtypes = [C.c_char_p, _ip]
    lib.sa_device_name.argtypes = [C.c_int, C.c_char_p, C.c_int, _ip]
    lib.sa_selftest_math.argtypes = [vp, C.c_int, C.c_long, _dp, _dp, _dp]
    lib.sa_selftest_fma_peak.argtypes = [vp, C.c_int, _dp, _dp, _dp]
    _LIB = lib
    return lib


class Context:
    """One device context (stream, events) of the C library."""

    def __init__(self, device: int = 0):
        self.lib = load()
        self.h = C.c_void_p()
        rc = self.lib.sa_create(C.byref(self.h), device)
        if rc != SA_OK:
            raise RuntimeError(f"sa_create failed with code {rc} (no usable CUDA device {device})")

    def check(self, rc: int, what: str):
        if rc != SA_OK:
            msg = self.lib.sa_error_message(self.h).decode()
            raise RuntimeError(f"{what} failed (code {rc}): {msg}")

    def close(self):
        if self.h:
            self.lib.sa_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
