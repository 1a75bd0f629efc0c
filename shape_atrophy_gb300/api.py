"""Host API of the GB300 forward model.

Two layers:

* ``forward(spec, ...)`` / ``varifold(spec, lmk, ...)`` -- spec-dict front
  end of the C-ABI (see problems.py for the spec keys);
* ``deformation(...)`` / ``computeObjfcn(...)`` -- the reference's MATLAB
  wrappers (CUDA/deformation.m:1-62, CUDA/computeObjfcn.m:1-62) with the
  same argument names, order and meaning: ``timeNum = floor(timeEnd /
  timeStp) + 1``, the CG tolerance is squared before the call, landmarks
  are given as D x N and the trajectory is returned as (D, N, timeNum).
  ``elaType='frame'`` is the reference's model; ``elaType='isotropic'``
  fills the branch the reference leaves empty (deformation.m:12-13,22-24):
  ``h_modVec`` holds (lambda, mu) per layer (reshape(h_modVec, 2, [])'),
  ``spdTanVal`` the per-layer diffusivities, ``elmObj['elmLyrVec']`` the
  layer of each element, ``h_ynkActPrmVec = [c]`` (load -c u I) and
  ``h_reaActPrmVec = [rate]`` (Fisher-KPP rate u (1 - u)).
"""
from __future__ import annotations

import ctypes as C
import json
import math
import os

import numpy as np

from . import _lib

_CTX = {}

TUNING_NAMES = ("persistMaxWarps", "batchBlock", "batchSlicesPerWarp", "vfdCtasPerSm", "mixedInnerFloor",
                "kernelMatrixFree")
TUNING_FILE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tuning.json")
_TUNED = {"applied": None}


def device_name(device: int = 0):
    """(name, SM count) of a CUDA device: the key of the tuning table."""
    lib = _lib.load()
    buf = C.create_string_buffer(256)
    sms = C.c_int()
    rc = lib.sa_device_name(int(device), buf, 256, C.byref(sms))
    if rc != _lib.SA_OK:
        raise RuntimeError(f"sa_device_name failed with code {rc}")
    return buf.value.decode(), sms.value


def set_tuning(**values):
    """Set launch shapes (process-wide; see TUNING_NAMES).  Raises on an unknown name or a value out of range."""
    lib = _lib.load()
    for k, v in values.items():
        if lib.sa_set_tuning(k.encode(), int(v)) != _lib.SA_OK:
            raise ValueError(f"bad tuning {k}={v}")


def get_tuning() -> dict:
    lib = _lib.load()
    out = {}
    for k in TUNING_NAMES:
        v = C.c_int()
        if lib.sa_get_tuning(k.encode(), C.byref(v)) != _lib.SA_OK:
            raise RuntimeError(f"sa_get_tuning({k}) failed")
        out[k] = v.value
    return out


def tuning_entry(device: int = 0, path: str = TUNING_FILE):
    """The tuning-table entry for this device (matched by name and SM count), or None."""
    if not os.path.exists(path):
        return None
    with open(path) as f:
        table = json.load(f)
    name, sms = device_name(device)
    for e in table.get("devices", []):
        if e.get("name") == name and int(e.get("smCount", -1)) == sms:
            return e
    return None


def apply_tuning(device: int = 0, path: str = TUNING_FILE):
    """Apply the autotuner's table for this device (compiled defaults stay when it has no entry).
    Set SA_TUNING=off in the environment to keep the compiled defaults."""
    if os.environ.get("SA_TUNING", "").lower() == "off":
        return None
    e = tuning_entry(device, path)
    if e is not None:
        set_tuning(**{k: e["values"][k] for k in TUNING_NAMES if k in e["values"]})
    _TUNED["applied"] = e
    return e


def fma_peak(fp64: bool = True, device: int = 0) -> dict:
    """Measured FMA throughput of the device's FP64 or FP32 pipe (sa_selftest_fma_peak):
    dict(tflops, flops_per_clock_sm, sm_mhz)."""
    ctx = context(device)
    v, pc, mhz = C.c_double(), C.c_double(), C.c_double()
    ctx.check(ctx.lib.sa_selftest_fma_peak(ctx.h, 1 if fp64 else 0, C.byref(v), C.byref(pc), C.byref(mhz)),
              "sa_selftest_fma_peak")
    return {"tflops": v.value, "flops_per_clock_sm": pc.value, "sm_mhz": mhz.value}


# Layered model: where each step's velocity CG starts -- the polynomial through the last k + 1 velocities,
# evaluated one step ahead (k = 0: the previous velocity, the reference's warm start).  Names or orders.
GUESS_ORDERS = {"previous": 0, "extrapolate": 1, "linear": 1, "quadratic": 2, "cubic": 3, "quartic": 4, "quintic": 5}
DEFAULT_GUESS = "cubic"


def guess_order(g) -> int:
    k = GUESS_ORDERS[g] if isinstance(g, str) else int(g)
    if not 0 <= k <= 5:
        raise ValueError(f"velocityGuess order {k} outside 0 .. 5")
    return k


def context(device: int = 0) -> _lib.Context:
    if device not in _CTX:
        _CTX[device] = _lib.Context(device)
        if _TUNED["applied"] is None:
            apply_tuning(device)
    return _CTX[device]


class _Keep:
    def __init__(self):
        self.arrays = []

    def i32(self, a):
        if a is None:
            return None
        a = np.ascontiguousarray(np.asarray(a, dtype=np.int32))
        self.arrays.append(a)
        return a.ctypes.data_as(_lib._ip)

    def f64(self, a):
        if a is None:
            return None
        a = np.ascontiguousarray(np.asarray(a, dtype=np.float64))
        self.arrays.append(a)
        return a.ctypes.data_as(_lib._dp)


def _element_object(obj: dict, dim: int, N: int, K: _Keep, with_vfd=True, with_grad=False) -> _lib.ElementObject:
    o = _lib.ElementObject()
    o.dim, o.lmkNum = dim, N
    o.elmVtxMat = K.i32(obj["elmVtxMat"]); o.elmNum = obj["elmVtxMat"].shape[1]
    o.vtxElmMat = K.i32(obj["vtxElmMat"]); o.vtxElmCols = obj["vtxElmMat"].shape[0]
    o.frmVtxMat = K.i32(obj["tanVtxMat"] if dim == 2 else obj["nmlVtxMat"])
    o.tsvVtxMat = K.i32(obj["tsvVtxMat"])
    if "bdrVtxMat" in obj:
        o.bdrVtxMat = K.i32(obj["bdrVtxMat"]); o.bdrElmNum = obj["bdrVtxMat"].shape[1]
        o.vtxBdrMat = K.i32(obj["vtxBdrMat"]); o.vtxBdrCols = obj["vtxBdrMat"].shape[0]
    o.btmVtxMat = K.i32(obj["btmVtxMat"]); o.btmElmNum = obj["btmVtxMat"].shape[1]
    o.vtxBtmMat = K.i32(obj["vtxBtmMat"]); o.btmLmkNum = obj["vtxBtmMat"].shape[1]
    o.vtxBtmCols = obj["vtxBtmMat"].shape[0]
    o.femVtxMat = K.i32(obj["femVtxMat"]); o.nzrNum = obj["femVtxMat"].shape[1]
    o.femIfoMat = K.i32(obj["femIfoMat"]); o.femIfoCols = obj["femIfoMat"].shape[0]
    if with_vfd and "vfdVtxMat" in obj:
        o.vfdVtxMat = K.i32(obj["vfdVtxMat"]); o.vfdElmNum = obj["vfdVtxMat"].shape[1]
    if with_grad and "vfdIfoMat" in obj:
        o.vfdIfoMat = K.i32(obj["vfdIfoMat"]); o.vfdIfoCols = obj["vfdIfoMat"].shape[0]
    if "elmLyrVec" in obj:
        o.elmLyrVec = K.i32(obj["elmLyrVec"])
    return o


def _params(spec: dict, K: _Keep, precision: str) -> _lib.Params:
    p = _lib.Params()
    iso = spec["elaType"] == "isotropic"
    p.elaType = _lib.SA_ELA_ISOTROPIC if iso else _lib.SA_ELA_FRAME
    p.precision = _lib.SA_PREC_MIXED if precision == "mixed" else _lib.SA_PREC_FP64
    tp = np.atleast_1d(np.asarray(spec.get("tauPrmVec", [0.0]), dtype=np.float64))
    p.tauPrmVec, p.tauPrmNum = K.f64(tp), tp.size
    p.ldmWgt, p.knlOrder = float(spec["ldmWgt"]), int(spec["knlOrder"])
    p.knlWidth, p.knlEps = float(spec["knlWidth"]), float(spec["knlEps"])
    mv = np.asarray(spec["modVec"], dtype=np.float64).reshape(-1)
    p.modVec, p.modNum = K.f64(mv), mv.size
    p.spdTanVal, p.spdTsvVal = float(spec.get("spdTanVal", 0.0)), float(spec.get("spdTsvVal", 0.0))
    if iso:
        sp = np.asarray(spec["spdLyrVec"], dtype=np.float64).reshape(-1)
        p.spdLyrVec, p.lyrNum = K.f64(sp), sp.size
    p.ynkActPrmVec = K.f64(spec["ynkActPrmVec"])
    p.reaActPrmVec = K.f64(spec["reaActPrmVec"])
    p.btmWgt, p.timeStp, p.timeNum = float(spec["btmWgt"]), float(spec["timeStp"]), int(spec["timeNum"])
    p.cgItrMax, p.cgTolSqu = int(spec["cgItrMax"]), float(spec["cgTolSqu"])
    p.rdItrMax = int(spec.get("rdItrMax", 0))
    p.rdTolSqu = float(spec.get("rdTolSqu", 0.0))
    p.cgKernel = {"auto": _lib.SA_CG_AUTO, "persistent": _lib.SA_CG_PERSISTENT,
                  "two-kernel": _lib.SA_CG_TWO_KERNEL,
                  "persistent-global": _lib.SA_CG_PERSISTENT_GLOBAL}[spec.get("cgKernel", "auto")]
    p.velocityGuess = guess_order(spec.get("velocityGuess", DEFAULT_GUESS))
    return p


def _target(spec: dict, K: _Keep) -> _lib.Target:
    t = _lib.Target()
    cen, udir, vol = spec["tgt"]
    t.cenPosMat, t.uniDirMat, t.elmVolVec = K.f64(cen), K.f64(udir), K.f64(vol)
    t.tgtElmNum = int(np.asarray(vol).size)
    ck, cw, dk, dw = spec["vfd"]
    t.cenKnlType, t.cenKnlWidth = ck.encode(), float(cw)
    t.dirKnlType, t.dirKnlWidth = dk.encode(), float(dw)
    return t


def _host_out(shape):
    """Host array for a device-to-host copy, its pages touched first: a copy into freshly mapped pages spends
    most of its time in page faults (46 MB of trajectory: 14 ms untouched, 2 ms after a 2 ms fill)."""
    a = np.empty(shape)
    a.fill(0.0)
    return a


def forward(spec: dict, tauVarMat=None, precision: str = "fp64", trajectory: bool = True,
            objective: bool = True, device: int = 0) -> dict:
    """Run the forward model for every row of ``tauVarMat`` (nObj x nVar).

    Returns dict(lmkStk (T, D, N) and tauMat (T, N) of the last row (as the
    reference returns them), obj (nObj,) -- DBL_MAX where the CG failed --
    and info (solve diagnostics of the last row)).
    """
    ctx = context(device)
    D = int(spec["dim"])
    lmk = np.ascontiguousarray(np.asarray(spec["lmkIniMat"], dtype=np.float64))
    N = lmk.shape[1]
    T = int(spec["timeNum"])
    tv = np.atleast_2d(np.asarray(spec["tauVarVec"] if tauVarMat is None else tauVarMat, dtype=np.float64))
    K = _Keep()
    with_obj = objective and spec.get("tgt") is not None
    o = _element_object(spec["elmObj"], D, N, K, with_vfd=with_obj)
    if spec["elaType"] == "isotropic" and "elmLyrVec" in spec:
        o.elmLyrVec = K.i32(spec["elmLyrVec"])
    p = _params(spec, K, precision)
    t = _target(spec, K) if with_obj else None
    lmkStk = _host_out((T, D, N)) if trajectory else None
    tauMat = _host_out((T, N)) if trajectory else None
    obj = np.zeros(tv.shape[0])
    info = _lib.SolveInfo()
    tvc = np.ascontiguousarray(tv)
    rc = ctx.lib.sa_forward(ctx.h, C.byref(o), lmk.ctypes.data_as(_lib._dp), C.byref(p),
                            C.byref(t) if t is not None else None, tvc.ctypes.data_as(_lib._dp), tv.shape[1],
                            tv.shape[0], lmkStk.ctypes.data_as(_lib._dp) if trajectory else None,
                            tauMat.ctypes.data_as(_lib._dp) if trajectory else None, obj.ctypes.data_as(_lib._dp),
                            C.byref(info))
    ctx.check(rc, "sa_forward")
    return dict(lmkStk=lmkStk, tauMat=tauMat, obj=obj,
                info=dict(status=info.status, cgIterTotal=info.cgIterTotal, rdIterTotal=info.rdIterTotal,
                          cgIterMax=info.cgIterMax, invertedElements=info.invertedElements,
                          elapsedMs=info.elapsedMs))


def gradient(spec: dict, tauVarVec=None, precision: str = "fp64", device: int = 0) -> dict:
    """Objective and its gradient with respect to the bump parameters [c (dim), h, sigma] of one parameter
    vector (layered model): the forward solve with the tangent-linear model of every step
    (sa_objective_gradient).  precision="mixed" runs the velocity solves (forward and tangent) as FP32 inner
    CG with FP64 refinement and the objective in FP32 pair sums.  Returns dict(obj, grad (dim + 2,), info)."""
    ctx = context(device)
    D = int(spec["dim"])
    lmk = np.ascontiguousarray(np.asarray(spec["lmkIniMat"], dtype=np.float64))
    N = lmk.shape[1]
    tv = np.ascontiguousarray(np.asarray(spec["tauVarVec"] if tauVarVec is None else tauVarVec,
                                         dtype=np.float64).reshape(-1))
    K = _Keep()
    o = _element_object(spec["elmObj"], D, N, K, with_vfd=True, with_grad=True)
    if "elmLyrVec" in spec:
        o.elmLyrVec = K.i32(spec["elmLyrVec"])
    p = _params(spec, K, precision)
    t = _target(spec, K)
    obj = np.zeros(1)
    grad = np.zeros(D + 2)
    info = _lib.SolveInfo()
    rc = ctx.lib.sa_objective_gradient(ctx.h, C.byref(o), lmk.ctypes.data_as(_lib._dp), C.byref(p), C.byref(t),
                                       tv.ctypes.data_as(_lib._dp), tv.size, obj.ctypes.data_as(_lib._dp),
                                       grad.ctypes.data_as(_lib._dp), C.byref(info))
    ctx.check(rc, "sa_objective_gradient")
    return dict(obj=float(obj[0]), grad=grad,
                info=dict(status=info.status, cgIterTotal=info.cgIterTotal, rdIterTotal=info.rdIterTotal,
                          tangentIters=info.cgIterMax, elapsedMs=info.elapsedMs))


def adjoint(spec: dict, tauVarVec=None, layers: bool = True, tau0: bool = True, x0: bool = True,
            device: int = 0) -> dict:
    """Objective and its gradient by the discrete adjoint (sa_objective_adjoint), FP64: dict(obj, grad,
    grad_layer, grad_tau0 (N,), grad_x0 (D, N), info).  Layered model: grad = d/d[c, h, sigma] (dim + 2),
    grad_layer (lyrNum, 3) = d/d(lambda, mu, D) per layer.  Frame model (the reference's): grad = d/d tauVar
    (2D [cx, cy, h, R], 3D [cx, cy, cz, h]), grad_layer None.  About twice (layered) the cost of one forward
    solve for all of them together."""
    ctx = context(device)
    D = int(spec["dim"])
    lmk = np.ascontiguousarray(np.asarray(spec["lmkIniMat"], dtype=np.float64))
    N = lmk.shape[1]
    tv = np.ascontiguousarray(np.asarray(spec["tauVarVec"] if tauVarVec is None else tauVarVec,
                                         dtype=np.float64).reshape(-1))
    K = _Keep()
    o = _element_object(spec["elmObj"], D, N, K, with_vfd=True, with_grad=True)
    if "elmLyrVec" in spec:
        o.elmLyrVec = K.i32(spec["elmLyrVec"])
    p = _params(spec, K, "fp64")
    t = _target(spec, K)
    frame = spec["elaType"] == "frame"
    L = 0 if frame else int(np.asarray(spec["spdLyrVec"]).size)
    obj, gb = np.zeros(1), np.zeros(4 if frame else D + 2)
    gl = np.zeros((L, 3)) if (layers and not frame) else None
    gt = np.zeros(N) if tau0 else None
    gx = np.zeros((D, N)) if x0 else None
    info = _lib.SolveInfo()
    ptr = lambda a: a.ctypes.data_as(_lib._dp) if a is not None else None
    rc = ctx.lib.sa_objective_adjoint(ctx.h, C.byref(o), lmk.ctypes.data_as(_lib._dp), C.byref(p), C.byref(t),
                                      tv.ctypes.data_as(_lib._dp), tv.size, ptr(obj), ptr(gb), ptr(gl), ptr(gt),
                                      ptr(gx), C.byref(info))
    ctx.check(rc, "sa_objective_adjoint")
    return dict(obj=float(obj[0]), grad=gb, grad_layer=gl, grad_tau0=gt, grad_x0=gx,
                info=dict(status=info.status, cgIterTotal=info.cgIterTotal, rdIterTotal=info.rdIterTotal,
                          adjointIters=info.cgIterMax, elapsedMs=info.elapsedMs))


def varifold(spec: dict, lmk, grad: bool = False, precision: str = "fp64", device: int = 0):
    """Varifold objective of the shape ``lmk`` (D, N) against spec['tgt'];
    with grad=True also its gradient with respect to the nodes, (D, N)."""
    ctx = context(device)
    D = int(spec["dim"])
    lmk = np.ascontiguousarray(np.asarray(lmk, dtype=np.float64))
    N = lmk.shape[1]
    K = _Keep()
    o = _element_object(spec["elmObj"], D, N, K, with_vfd=True, with_grad=grad)
    t = _target(spec, K)
    out = C.c_double()
    g = np.zeros((D, N)) if grad else None
    rc = ctx.lib.sa_varifold(ctx.h, C.byref(o), lmk.ctypes.data_as(_lib._dp), C.byref(t),
                             _lib.SA_PREC_MIXED if precision == "mixed" else _lib.SA_PREC_FP64, C.byref(out),
                             g.ctypes.data_as(_lib._dp) if grad else None)
    ctx.check(rc, "sa_varifold")
    return (out.value, g) if grad else out.value


class Session:
    """Stepwise solve of one parameter vector with device-resident state."""

    def __init__(self, spec: dict, tauVarVec=None, precision: str = "fp64", objective: bool = True,
                 device: int = 0):
        self.ctx = context(device)
        self.D = int(spec["dim"])
        self.K = _Keep()
        lmk = np.ascontiguousarray(np.asarray(spec["lmkIniMat"], dtype=np.float64))
        self.N = lmk.shape[1]
        with_obj = objective and spec.get("tgt") is not None
        o = _element_object(spec["elmObj"], self.D, self.N, self.K, with_vfd=with_obj)
        if spec["elaType"] == "isotropic" and "elmLyrVec" in spec:
            o.elmLyrVec = self.K.i32(spec["elmLyrVec"])
        p = _params(spec, self.K, precision)
        t = _target(spec, self.K) if with_obj else None
        tv = np.ascontiguousarray(np.asarray(spec["tauVarVec"] if tauVarVec is None else tauVarVec,
                                             dtype=np.float64).reshape(-1))
        self.h = C.c_void_p()
        rc = self.ctx.lib.sa_session_create(self.ctx.h, C.byref(o), lmk.ctypes.data_as(_lib._dp), C.byref(p),
                                            C.byref(t) if t is not None else None, tv.ctypes.data_as(_lib._dp),
                                            tv.size, C.byref(self.h))
        self.ctx.check(rc, "sa_session_create")

    def step(self, n: int = 1) -> int:
        done = C.c_int()
        self.ctx.check(self.ctx.lib.sa_session_step(self.h, int(n), C.byref(done)), "sa_session_step")
        return done.value

    def state(self):
        lmk = np.zeros((self.D, self.N))
        tau = np.zeros(self.N)
        t = C.c_int()
        self.ctx.check(self.ctx.lib.sa_session_state(self.h, lmk.ctypes.data_as(_lib._dp),
                                                     tau.ctypes.data_as(_lib._dp), C.byref(t)), "sa_session_state")
        return lmk, tau, t.value

    def stream(self, nsteps: int, stride: int = 1, max_snapshots: int = None, positions: bool = True,
               concentration: bool = True):
        """Advance up to nsteps steps, collecting the state after every step whose session step number is a
        multiple of stride (copied to the host while the next steps run).  Returns (lmk (K, D, N) or None,
        tau (K, N) or None, steps taken); K = snapshots written."""
        K = nsteps // stride + 1 if max_snapshots is None else int(max_snapshots)
        lmk = _host_out((K, self.D, self.N)) if positions else None
        tau = _host_out((K, self.N)) if concentration else None
        wr, done = C.c_int(), C.c_int()
        self.ctx.check(self.ctx.lib.sa_session_stream(
            self.h, int(nsteps), int(stride), lmk.ctypes.data_as(_lib._dp) if positions else None,
            tau.ctypes.data_as(_lib._dp) if concentration else None, K, C.byref(wr), C.byref(done)),
            "sa_session_stream")
        k = wr.value
        return (lmk[:k] if positions else None), (tau[:k] if concentration else None), done.value

    def objective(self) -> float:
        v = C.c_double()
        self.ctx.check(self.ctx.lib.sa_session_objective(self.h, C.byref(v)), "sa_session_objective")
        return v.value

    def info(self) -> dict:
        i = _lib.SolveInfo()
        self.ctx.check(self.ctx.lib.sa_session_info(self.h, C.byref(i)), "sa_session_info")
        return dict(status=i.status, cgIterTotal=i.cgIterTotal, rdIterTotal=i.rdIterTotal, cgIterMax=i.cgIterMax,
                    invertedElements=i.invertedElements, lastStepMs=i.elapsedMs, kernelLaunches=i.kernelLaunches)

    def profile(self, enable: int = -1):
        """enable=1/0 switches timing of the velocity CG's dominant kernel on/off (and resets the totals);
        returns (ms, launches, algorithmic bytes, flops) accumulated over the timed launches."""
        ms, cnt, by, fl = C.c_double(), C.c_longlong(), C.c_double(), C.c_double()
        self.ctx.check(self.ctx.lib.sa_session_profile(self.h, int(enable), C.byref(ms), C.byref(cnt),
                                                       C.byref(by), C.byref(fl)), "sa_session_profile")
        return ms.value, cnt.value, by.value, fl.value

    def close(self):
        if self.h:
            self.ctx.lib.sa_session_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------------------
# the reference's MATLAB wrappers
# ---------------------------------------------------------------------------
def _matlab_spec(elaType, h_lmkIniMat, elmObj, ldmWgt, knlOrder, knlWidth, knlEps, h_modVec, h_ynkActPrmVec,
                 spdTanVal, spdTsvVal, h_reaActPrmVec, btmWgt, timeStp, timeEnd, cgItrMax, cgTolVal, h_tauPrmVec):
    et = str(elaType).lower()
    if et not in ("frame", "isotropic"):
        raise ValueError(f"Unknown elasticity type {elaType}.")       # deformation.m:18
    lmk = np.asarray(h_lmkIniMat, dtype=np.float64)
    D = lmk.shape[0]
    if D not in (2, 3):
        raise ValueError(f"Dimension {D} is not supported.")            # deformation.m:55
    spec = dict(dim=D, elaType=et, lmkIniMat=lmk, elmObj=elmObj, tauPrmVec=np.atleast_1d(h_tauPrmVec),
                modVec=np.asarray(h_modVec, dtype=np.float64).reshape(-1), ynkActPrmVec=h_ynkActPrmVec,
                reaActPrmVec=h_reaActPrmVec, ldmWgt=ldmWgt, knlOrder=knlOrder, knlWidth=knlWidth, knlEps=knlEps,
                btmWgt=btmWgt, timeStp=timeStp, timeNum=int(math.floor(timeEnd / timeStp)) + 1,
                cgItrMax=cgItrMax, cgTolSqu=cgTolVal ** 2)
    if et == "isotropic":
        spec["spdLyrVec"] = np.atleast_1d(np.asarray(spdTanVal, dtype=np.float64))
        spec["elmLyrVec"] = elmObj["elmLyrVec"]
    else:
        spec["spdTanVal"], spec["spdTsvVal"] = float(spdTanVal), float(spdTsvVal)
    return spec


def deformation(h_tauVarVec, h_tauPrmVec, elaType, h_lmkIniMat, elmObj, ldmWgt, knlOrder, knlWidth, knlEps,
                h_modVec, h_ynkActPrmVec, spdTanVal, spdTsvVal, h_reaActPrmVec, btmWgt, timeStp, timeEnd,
                cgItrMax, cgTolVal):
    """deformation.m: returns (h_lmkStk (D, N, timeNum), h_tauMat (N, timeNum))."""
    spec = _matlab_spec(elaType, h_lmkIniMat, elmObj, ldmWgt, knlOrder, knlWidth, knlEps, h_modVec,
                        h_ynkActPrmVec, spdTanVal, spdTsvVal, h_reaActPrmVec, btmWgt, timeStp, timeEnd, cgItrMax,
                        cgTolVal, h_tauPrmVec)
    tv = np.asarray(h_tauVarVec, dtype=np.float64)
    tv = tv.T if tv.ndim == 2 else tv[None, :]          # MATLAB columns are parameter sets
    r = forward(spec, tv, trajectory=True, objective=False)
    return np.transpose(r["lmkStk"], (1, 2, 0)), r["tauMat"].T


def computeObjfcn(h_tauVarMat, h_tauPrmVec, elaType, h_lmkIniMat, elmObj, tgtObj, vfdObj, ldmWgt, knlOrder,
                  knlWidth, knlEps, h_modVec, h_ynkActPrmVec, spdTanVal, spdTsvVal, h_reaActPrmVec, btmWgt,
                  timeStp, timeEnd, cgItrMax, cgTolVal):
    """computeObjfcn.m: objective per column of h_tauVarMat (DBL_MAX where the CG failed)."""
    spec = _matlab_spec(elaType, h_lmkIniMat, elmObj, ldmWgt, knlOrder, knlWidth, knlEps, h_modVec,
                        h_ynkActPrmVec, spdTanVal, spdTsvVal, h_reaActPrmVec, btmWgt, timeStp, timeEnd, cgItrMax,
                        cgTolVal, h_tauPrmVec)
    spec["tgt"] = (tgtObj["cenPosMat"], tgtObj["uniDirMat"], tgtObj["elmVolVec"])
    spec["vfd"] = (vfdObj["cenKnlType"], vfdObj["cenKnlWidth"], vfdObj["dirKnlType"], vfdObj["dirKnlWidth"])
    tv = np.asarray(h_tauVarMat, dtype=np.float64)
    tv = tv.T if tv.ndim == 2 else tv[None, :]
    return forward(spec, tv, trajectory=False, objective=True)["obj"]


class Server:
    """Continuous-batching solver service (layered model): submit() returns at once; result() waits.

    hbm_budget: device bytes the running instances may hold; max_instances: limit on concurrent solves.
    """

    def __init__(self, hbm_budget: float = 64e9, max_instances: int = 256, device: int = 0):
        self.ctx = context(device)
        self.h = C.c_void_p()
        self.ctx.check(self.ctx.lib.sa_server_create(self.ctx.h, float(hbm_budget), int(max_instances),
                                                     C.byref(self.h)), "sa_server_create")
        self.meta = {}

    def submit(self, spec: dict, tauVarVec=None, precision: str = "fp64", objective: bool = True) -> int:
        D = int(spec["dim"])
        K = _Keep()
        lmk = np.ascontiguousarray(np.asarray(spec["lmkIniMat"], dtype=np.float64))
        N = lmk.shape[1]
        with_obj = objective and spec.get("tgt") is not None
        o = _element_object(spec["elmObj"], D, N, K, with_vfd=with_obj)
        if "elmLyrVec" in spec:
            o.elmLyrVec = K.i32(spec["elmLyrVec"])
        p = _params(spec, K, precision)
        t = _target(spec, K) if with_obj else None
        tv = np.ascontiguousarray(np.asarray(spec["tauVarVec"] if tauVarVec is None else tauVarVec,
                                             dtype=np.float64).reshape(-1))
        rid = C.c_longlong()
        self.ctx.check(self.ctx.lib.sa_server_submit(self.h, C.byref(o), lmk.ctypes.data_as(_lib._dp), C.byref(p),
                                                     C.byref(t) if t is not None else None,
                                                     tv.ctypes.data_as(_lib._dp), tv.size, C.byref(rid)),
                       "sa_server_submit")
        self.meta[rid.value] = (D, N)
        return rid.value

    def poll(self, rid: int) -> int:
        st = C.c_int()
        self.ctx.check(self.ctx.lib.sa_server_poll(self.h, int(rid), C.byref(st)), "sa_server_poll")
        return st.value

    def result(self, rid: int, timeout_ms: float = -1.0) -> dict:
        """Waits for the request, then returns dict(lmk (D, N), tau (N,), obj, info, latency_ms)."""
        st = C.c_int()
        self.ctx.check(self.ctx.lib.sa_server_wait(self.h, int(rid), float(timeout_ms), C.byref(st)),
                       "sa_server_wait")
        if st.value not in (_lib.SA_REQ_DONE, _lib.SA_REQ_FAILED):
            raise TimeoutError(f"request {rid} not finished")
        D, N = self.meta.pop(rid)
        lmk, tau = np.zeros((D, N)), np.zeros(N)
        obj, lat = C.c_double(), C.c_double()
        info = _lib.SolveInfo()
        self.ctx.check(self.ctx.lib.sa_server_result(self.h, int(rid), lmk.ctypes.data_as(_lib._dp),
                                                     tau.ctypes.data_as(_lib._dp), C.byref(obj), C.byref(info),
                                                     C.byref(lat)), "sa_server_result")
        return dict(lmk=lmk, tau=tau, obj=obj.value, latency_ms=lat.value,
                    info=dict(status=info.status, cgIterTotal=info.cgIterTotal, rdIterTotal=info.rdIterTotal,
                              cgIterMax=info.cgIterMax, invertedElements=info.invertedElements,
                              elapsedMs=info.elapsedMs))

    def stats(self) -> dict:
        c = _lib.ServerCounters()
        self.ctx.check(self.ctx.lib.sa_server_stats(self.h, C.byref(c)), "sa_server_stats")
        return {k: getattr(c, k) for k, _ in c._fields_}

    def close(self):
        if self.h:
            self.ctx.lib.sa_server_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# --------------------------------------------------------------------------
# native element-object builders (host code of the C library)
# --------------------------------------------------------------------------
def _i32(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.int32))


def _elmobj_dict(h, lib, dim: int) -> dict:
    """Copy a built sa_elmobj into the dict layout of mesh.generate_element_object_2d/3d."""
    v = _lib.ElementObject()
    lib.sa_elmobj_view(h, C.byref(v))
    N, E = v.lmkNum, v.elmNum

    def arr(ptr, rows, cols):
        return np.ctypeslib.as_array(ptr, shape=(rows, cols)).copy()

    fcols = 4 if dim == 2 else 6
    obj = {"elmVtxMat": arr(v.elmVtxMat, dim + 1, E), "vtxElmMat": arr(v.vtxElmMat, v.vtxElmCols, N),
           ("tanVtxMat" if dim == 2 else "nmlVtxMat"): arr(v.frmVtxMat, fcols, E),
           "tsvVtxMat": arr(v.tsvVtxMat, fcols, E), "bdrVtxMat": arr(v.bdrVtxMat, dim, v.bdrElmNum),
           "vtxBdrMat": arr(v.vtxBdrMat, v.vtxBdrCols, N), "btmVtxMat": arr(v.btmVtxMat, dim, v.btmElmNum),
           "vtxBtmMat": arr(v.vtxBtmMat, v.vtxBtmCols, v.btmLmkNum), "femVtxMat": arr(v.femVtxMat, 2, v.nzrNum),
           "femIfoMat": arr(v.femIfoMat, v.femIfoCols, v.nzrNum), "vfdVtxMat": arr(v.vfdVtxMat, dim, v.vfdElmNum),
           "vfdIfoMat": arr(v.vfdIfoMat, v.vfdIfoCols, N), "dim": dim}
    L, Cn, per = C.c_int(), C.c_int(), C.c_int()
    lib.sa_elmobj_layers(h, C.byref(L), C.byref(Cn), C.byref(per))
    obj["lyrLmkNum"], obj["lyrCntNum"], obj["elmPerLayer"] = L.value, Cn.value, per.value
    return obj


def tri2tetra(triVtxMat, lyrCntNum: int):
    """tri2tetra.m in the C library: (3, T) triangles -> tet (4, E), nml (6, E), tsv (6, E)."""
    lib = _lib.load()
    tri = _i32(triVtxMat)
    T = tri.shape[1]
    E = 3 * T * (int(lyrCntNum) - 1)
    tet, nml, tsv = np.zeros((4, E), np.int32), np.zeros((6, E), np.int32), np.zeros((6, E), np.int32)
    rc = lib.sa_tri2tetra(tri.ctypes.data_as(_lib._ip), T, int(lyrCntNum), tet.ctypes.data_as(_lib._ip),
                          nml.ctypes.data_as(_lib._ip), tsv.ctypes.data_as(_lib._ip))
    if rc != _lib.SA_OK:
        raise ValueError(f"sa_tri2tetra failed (code {rc})")
    return tet, nml, tsv


def build_element_object_3d(tetVtxMat, btmVtxMat, nmlVtxMat, tsvVtxMat, vfdLyrVec) -> dict:
    """generateElementObject3D.m in the C library (same arrays as mesh.generate_element_object_3d)."""
    lib = _lib.load()
    tet, btm, nml, tsv, vl = (_i32(a) for a in (tetVtxMat, btmVtxMat, nmlVtxMat, tsvVtxMat, vfdLyrVec))
    h = C.c_void_p()
    rc = lib.sa_build_element_object_3d(tet.ctypes.data_as(_lib._ip), tet.shape[1], btm.ctypes.data_as(_lib._ip),
                                        btm.shape[1], nml.ctypes.data_as(_lib._ip), tsv.ctypes.data_as(_lib._ip),
                                        vl.ctypes.data_as(_lib._ip), vl.size, C.byref(h))
    if rc != _lib.SA_OK:
        raise ValueError(f"sa_build_element_object_3d failed (code {rc})")
    try:
        return _elmobj_dict(h, lib, 3)
    finally:
        lib.sa_elmobj_free(h)


def build_element_object_2d(lyrLmkNum: int, lyrCntNum: int, vfdLyrVec, periodic: bool = False) -> dict:
    """generateElementObject2D.m in the C library (same arrays as mesh.generate_element_object_2d)."""
    lib = _lib.load()
    vl = _i32(vfdLyrVec)
    h = C.c_void_p()
    rc = lib.sa_build_element_object_2d(int(lyrLmkNum), int(lyrCntNum), vl.ctypes.data_as(_lib._ip), vl.size,
                                        int(bool(periodic)), C.byref(h))
    if rc != _lib.SA_OK:
        raise ValueError(f"sa_build_element_object_2d failed (code {rc})")
    try:
        return _elmobj_dict(h, lib, 2)
    finally:
        lib.sa_elmobj_free(h)
