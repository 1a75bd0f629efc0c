"""The drop-in boundary end to end: the MEX gateways of shape_atrophy_gb300/mex/
(the files a maintainer compiles with `mex` to replace deformation_{2D,3D}_frame
and computeObjfcn_{2D,3D}_frame, and to fill the empty isotropic branch with
deformation_{2D,3D}_isotropic and computeObjfcn_{2D,3D}_isotropic) are compiled
against a stand-in of the MEX API and called with 27 / 35 right-hand sides,
gpuArray arguments in device memory (zero-copy, as MATLAB passes them).  Frame
outputs are compared with the reference's own outputs (golden vectors) at
1e-10; isotropic outputs with sa_forward bit for bit and with the oracle at
1e-10."""
import ctypes as C

import numpy as np
import pytest

from golden_io import load, names

pytestmark = pytest.mark.gpu

DBL_MAX = np.finfo(np.float64).max


@pytest.fixture(scope="module")
def gateways():
    import sys, os
    sys.path.insert(0, os.path.join(os.path.dirname(__file__), "mex_stub"))
    import build_gateways
    libs = {}
    for key, so in build_gateways.build().items():
        lib = C.CDLL(so)
        lib.stub_wrap.restype = C.c_void_p
        lib.stub_wrap.argtypes = [C.c_size_t, C.c_size_t, C.c_void_p]
        lib.stub_data.restype = C.c_void_p
        lib.stub_data.argtypes = [C.c_void_p]
        lib.stub_free.argtypes = [C.c_void_p]
        lib.stub_call.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_char_p, C.c_int]
        libs[key] = lib
    yield libs
    for lib in libs.values():
        lib.stub_atexit()


class _Rhs:
    """prhs builder: host matrices, or device matrices for the gpuArray arguments."""

    def __init__(self, lib, torch):
        self.lib, self.torch, self.ptrs, self.keep = lib, torch, [], []

    def host(self, a, dtype=np.float64):
        a = np.ascontiguousarray(np.asarray(a, dtype=dtype))
        a2 = a.reshape(a.shape[0], -1) if a.ndim > 1 else a.reshape(1, -1)
        self.keep.append(a)
        # a (k, n) C-contiguous array is the column-major n x k MATLAB matrix of the reference
        m, n = (a2.shape[1], a2.shape[0]) if a.ndim > 1 else (1, a2.shape[1])
        self.ptrs.append(self.lib.stub_wrap(m, n, a.ctypes.data))

    def scalar(self, v):
        self.host(np.array([float(v)]))

    def gpu(self, a, dtype):
        a = np.ascontiguousarray(np.asarray(a, dtype=dtype))
        t = self.torch.as_tensor(a, device="cuda:0")
        self.keep.append(t)
        m, n = (a.shape[1], a.shape[0]) if a.ndim > 1 else (a.shape[0], 1)
        self.ptrs.append(self.lib.stub_wrap(m, n, t.data_ptr()))


def _common_head(R, spec, tv):
    obj, D = spec["elmObj"], spec["dim"]
    R.host(tv)                                              # prhs[0] tauVarMat (nVar x nObj)
    R.host(spec["tauPrmVec"])                               # prhs[1]
    R.gpu(spec["lmkIniMat"], np.float64)                    # prhs[2] gpuArray N x D
    for k in ["elmVtxMat", "vtxElmMat", "tanVtxMat" if D == 2 else "nmlVtxMat", "tsvVtxMat", "bdrVtxMat",
              "vtxBdrMat", "btmVtxMat", "vtxBtmMat", "femVtxMat", "femIfoMat"]:
        R.gpu(obj[k], np.int32)                             # prhs[3..12] gpuArray int32


def _common_tail(R, spec):
    for k in ["ldmWgt", "knlOrder", "knlWidth", "knlEps"]:
        R.scalar(spec[k])
    R.host(spec["modVec"])
    R.scalar(spec["spdTanVal"]); R.scalar(spec["spdTsvVal"])
    R.host(spec["ynkActPrmVec"]); R.host(spec["reaActPrmVec"])
    for k in ["btmWgt", "timeStp", "timeNum", "cgItrMax", "cgTolSqu"]:
        R.scalar(spec[k])


def _call(lib, R, nlhs):
    torch = R.torch
    torch.cuda.synchronize()
    plhs = (C.c_void_p * nlhs)()
    prhs = (C.c_void_p * len(R.ptrs))(*R.ptrs)
    err = C.create_string_buffer(1024)
    rc = lib.stub_call(nlhs, plhs, len(R.ptrs), prhs, err, 1024)
    for p in R.ptrs:
        lib.stub_free(p)
    assert rc == 0, err.value.decode()
    return list(plhs)


def _take(lib, p, count):
    a = np.ctypeslib.as_array(C.cast(lib.stub_data(p), C.POINTER(C.c_double)), shape=(count,)).copy()
    lib.stub_free(p)
    return a


@pytest.mark.parametrize("name", names())
def test_gateways_reproduce_the_reference(gateways, name):
    torch = pytest.importorskip("torch")
    spec, ref = load(name)
    D, N, T = spec["dim"], spec["lmkIniMat"].shape[1], int(spec["timeNum"])
    tv = ref["tauVarMat"]
    # deformation_{D}D_frame: plhs lmkStk (N*D x T), tauMat (N x T), objVec
    lib = gateways[("deformation", D)]
    R = _Rhs(lib, torch)
    _common_head(R, spec, tv)
    _common_tail(R, spec)
    assert len(R.ptrs) == 27
    p = _call(lib, R, 3)
    lmk = _take(lib, p[0], N * D * T).reshape(T, D, N)
    tau = _take(lib, p[1], N * T).reshape(T, N)
    obj = _take(lib, p[2], tv.shape[0])
    if ref["objfcn"][-1] != DBL_MAX:
        scale = np.abs(ref["lmkStk"]).max()
        assert np.abs(lmk - ref["lmkStk"]).max() <= 1e-10 * scale
        assert np.abs(tau - ref["tauMat"]).max() <= 1e-10 * max(np.abs(ref["tauMat"]).max(), 1e-300)
    assert np.all((obj == 0.0) | (obj == DBL_MAX))
    # computeObjfcn_{D}D_frame: plhs objVec
    lib = gateways[("computeObjfcn", D)]
    R = _Rhs(lib, torch)
    _common_head(R, spec, tv)
    R.gpu(spec["elmObj"]["vfdVtxMat"], np.int32)            # prhs[13]
    cen, udir, vol = spec["tgt"]
    R.gpu(cen, np.float64); R.gpu(udir, np.float64); R.gpu(vol, np.float64)   # prhs[14..16]
    ck, cw, dk, dw = spec["vfd"]
    R.scalar(ord(ck)); R.scalar(cw); R.scalar(ord(dk)); R.scalar(dw)          # prhs[17..20]
    _common_tail(R, spec)                                   # prhs[21..34]
    assert len(R.ptrs) == 35
    p = _call(lib, R, 1)
    obj = _take(lib, p[0], tv.shape[0])
    for k in range(tv.shape[0]):
        if ref["objfcn"][k] == DBL_MAX:
            assert obj[k] == DBL_MAX
        else:
            assert abs(obj[k] - ref["objfcn"][k]) <= 1e-10 * abs(ref["objfcn"][k])


# ---------------------------------------------------------------------------
# the layered (isotropic) model: deformation_{2D,3D}_isotropic, computeObjfcn_{2D,3D}_isotropic
# ---------------------------------------------------------------------------
def _layered_case(dim):
    from shape_atrophy_gb300 import problems
    if dim == 2:
        spec = problems.annulus_layered(angNum=48, radNum=7, steps=6, cgTolVal=1e-12)
        tv = np.array([[1.0, 0.0, 1.0, 0.1], [0.0, 1.0, 0.8, 0.15]])
    else:
        spec = problems.shell_layered(level=2, lyrCntNum=4, steps=4, cgTolVal=1e-12)
        tv = np.array([[0.0, 0.0, 1.0, 1.0, 0.15], [1.0, 0.0, 0.0, 0.7, 0.2]])
    return spec, tv


def _isotropic_middle(R, spec):
    """prhs[13]: elmObj.elmLyrVec, gpuArray int32."""
    R.gpu(spec["elmLyrVec"], np.int32)


def _isotropic_tail(R, spec):
    for k in ["ldmWgt", "knlOrder", "knlWidth", "knlEps"]:
        R.scalar(spec[k])
    mv = np.asarray(spec["modVec"], dtype=np.float64)
    R.gpu(np.stack([mv[0::2], mv[1::2]]), np.float64)       # d_modMat = reshape(h_modVec, 2, [])': L x 2
    R.host(spec["spdLyrVec"])                                # per-layer diffusivities
    R.host(spec["ynkActPrmVec"]); R.host(spec["reaActPrmVec"])
    for k in ["btmWgt", "timeStp", "timeNum", "cgItrMax", "cgTolSqu"]:
        R.scalar(spec[k])


@pytest.mark.parametrize("dim", [2, 3])
def test_isotropic_gateways_match_forward(gateways, dim):
    """The isotropic gateways give sa_forward's results bit for bit (same solves), and the oracle's to 1e-10."""
    torch = pytest.importorskip("torch")
    from oracle.oracle import Problem
    from shape_atrophy_gb300 import api
    spec, tv = _layered_case(dim)
    N, T = spec["lmkIniMat"].shape[1], int(spec["timeNum"])
    want = api.forward(spec, tv, trajectory=True, objective=True)
    assert want["info"]["status"] == 0

    lib = gateways[("deformation", dim, "isotropic")]
    R = _Rhs(lib, torch)
    _common_head(R, spec, tv)                                # prhs[0..12]
    _isotropic_middle(R, spec)                               # prhs[13]
    _isotropic_tail(R, spec)                                 # prhs[14..26]
    assert len(R.ptrs) == 27
    p = _call(lib, R, 3)
    lmk = _take(lib, p[0], N * dim * T).reshape(T, dim, N)
    tau = _take(lib, p[1], N * T).reshape(T, N)
    obj = _take(lib, p[2], tv.shape[0])
    np.testing.assert_array_equal(lmk, want["lmkStk"])
    np.testing.assert_array_equal(tau, want["tauMat"])
    assert np.all(obj == 0.0)

    lib = gateways[("computeObjfcn", dim, "isotropic")]
    R = _Rhs(lib, torch)
    _common_head(R, spec, tv)                                # prhs[0..12]
    _isotropic_middle(R, spec)                               # prhs[13]
    R.gpu(spec["elmObj"]["vfdVtxMat"], np.int32)             # prhs[14]
    cen, udir, vol = spec["tgt"]
    R.gpu(cen, np.float64); R.gpu(udir, np.float64); R.gpu(vol, np.float64)   # prhs[15..17]
    ck, cw, dk, dw = spec["vfd"]
    R.scalar(ord(ck)); R.scalar(cw); R.scalar(ord(dk)); R.scalar(dw)          # prhs[18..21]
    _isotropic_tail(R, spec)                                 # prhs[22..34]
    assert len(R.ptrs) == 35
    p = _call(lib, R, 1)
    obj = _take(lib, p[0], tv.shape[0])
    np.testing.assert_array_equal(obj, want["obj"])
    P = Problem(spec)
    for k in range(tv.shape[0]):
        r = P.forward(tv[k], with_obj=True)
        assert abs(obj[k] - r["obj"]) <= 1e-10 * abs(r["obj"])
    assert np.abs(lmk - r["lmkStk"]).max() <= 1e-10 * np.abs(r["lmkStk"]).max()


def test_isotropic_gateway_rejects_bad_layer_table(gateways):
    """modMat must be lyrNum x 2 with lyrNum diffusivities: a mismatch is a MEX error, not a fault."""
    torch = pytest.importorskip("torch")
    spec, tv = _layered_case(2)
    lib = gateways[("deformation", 2, "isotropic")]
    R = _Rhs(lib, torch)
    _common_head(R, spec, tv)
    _isotropic_middle(R, spec)
    for k in ["ldmWgt", "knlOrder", "knlWidth", "knlEps"]:
        R.scalar(spec[k])
    mv = np.asarray(spec["modVec"], dtype=np.float64)
    R.gpu(np.stack([mv[0::2], mv[1::2]]), np.float64)
    R.host(spec["spdLyrVec"][:-1])                           # one diffusivity short
    R.host(spec["ynkActPrmVec"]); R.host(spec["reaActPrmVec"])
    for k in ["btmWgt", "timeStp", "timeNum", "cgItrMax", "cgTolSqu"]:
        R.scalar(spec[k])
    torch.cuda.synchronize()
    plhs = (C.c_void_p * 3)()
    prhs = (C.c_void_p * len(R.ptrs))(*R.ptrs)
    err = C.create_string_buffer(1024)
    rc = lib.stub_call(3, plhs, len(R.ptrs), prhs, err, 1024)
    for p in R.ptrs:
        lib.stub_free(p)
    assert rc != 0 and b"lyrNum" in err.value
