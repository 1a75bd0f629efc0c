"""sa_varifold_noalloc: the allocation-free varifold objective.

It exists for callers that must not allocate device memory while they
evaluate the objective (an optimiser's line search on a GPU whose memory
belongs to MATLAB's gpuArray pool or to a serving process with a fixed
budget).  This test calls it through the C-ABI with inputs the test places
in device memory itself, twice in a row, and compares both results with
the allocating entry point sa_varifold (same tolerance as the other
varifold tests: 1e-12 relative), then checks the size limit.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SA_OK, SA_ERR_ARG = 0, 1


def _device(torch, a, dtype):
    return torch.as_tensor(np.ascontiguousarray(a), dtype=dtype, device="cuda:0")


@pytest.mark.parametrize("dim", [2, 3])
def test_noalloc_matches_allocating_entry(dim):
    torch = pytest.importorskip("torch")
    from shape_atrophy_gb300 import _lib, api, mesh, problems

    spec = problems.demo_strip(33, 9) if dim == 2 else problems.frame_shell(2, 3)
    spec["vfd"] = ("G", 0.4, "B", 1.0)
    lmk = mesh.smooth_displacement(spec["lmkIniMat"], 0.02, 3)
    want = api.varifold(spec, lmk)                       # allocating entry point

    lib = _lib.load()
    fn = lib.sa_varifold_noalloc
    fn.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p,
                   C.c_void_p, C.c_char, C.c_double, C.c_char, C.c_double, C.c_void_p, C.POINTER(C.c_double)]
    fn.restype = C.c_int
    cen, udir, vol = spec["tgt"]
    x_d = _device(torch, lmk, torch.float64)
    v_d = _device(torch, spec["elmObj"]["vfdVtxMat"], torch.int32)
    c_d = _device(torch, cen, torch.float64)
    u_d = _device(torch, udir, torch.float64)
    w_d = _device(torch, vol, torch.float64)
    torch.cuda.synchronize()
    N, Vd, Vt = lmk.shape[1], spec["elmObj"]["vfdVtxMat"].shape[1], vol.size
    got = []
    for _ in range(2):                                   # two calls in a row share the scratch array
        out = C.c_double(0.0)
        rc = fn(dim, N, x_d.data_ptr(), Vd, v_d.data_ptr(), Vt, c_d.data_ptr(), u_d.data_ptr(), w_d.data_ptr(),
                b"G", 0.4, b"B", 1.0, None, C.byref(out))
        assert rc == SA_OK
        got.append(out.value)
    for g in got:
        assert abs(g - want) <= 1e-12 * abs(want), (g, want)

    # beyond the scratch limit: rejected, not truncated
    out = C.c_double(0.0)
    rc = fn(dim, N, x_d.data_ptr(), 40000, v_d.data_ptr(), Vt, c_d.data_ptr(), u_d.data_ptr(), w_d.data_ptr(),
            b"G", 0.4, b"B", 1.0, None, C.byref(out))
    assert rc == SA_ERR_ARG
    # host memory inputs: rejected (the entry point copies nothing)
    h = np.ascontiguousarray(lmk)
    rc = fn(dim, N, h.ctypes.data, Vd, v_d.data_ptr(), Vt, c_d.data_ptr(), u_d.data_ptr(), w_d.data_ptr(),
            b"G", 0.4, b"B", 1.0, None, C.byref(out))
    assert rc == SA_ERR_ARG
    # a zero centre width: rejected before any launch
    rc = fn(dim, N, x_d.data_ptr(), Vd, v_d.data_ptr(), Vt, c_d.data_ptr(), u_d.data_ptr(), w_d.data_ptr(),
            b"G", 0.0, b"B", 1.0, None, C.byref(out))
    assert rc == SA_ERR_ARG
    # a node index equal to N (one past the end, e.g. a 1-based index): found on the device, no read made
    bad = np.array(spec["elmObj"]["vfdVtxMat"], dtype=np.int32, copy=True)
    bad[0, Vd // 2] = N
    b_d = _device(torch, bad, torch.int32)
    torch.cuda.synchronize()
    rc = fn(dim, N, x_d.data_ptr(), Vd, b_d.data_ptr(), Vt, c_d.data_ptr(), u_d.data_ptr(), w_d.data_ptr(),
            b"G", 0.4, b"B", 1.0, None, C.byref(out))
    assert rc == SA_ERR_ARG
    # the next valid call is unaffected by the rejected one
    out = C.c_double(0.0)
    rc = fn(dim, N, x_d.data_ptr(), Vd, v_d.data_ptr(), Vt, c_d.data_ptr(), u_d.data_ptr(), w_d.data_ptr(),
            b"G", 0.4, b"B", 1.0, None, C.byref(out))
    assert rc == SA_OK and abs(out.value - want) <= 1e-12 * abs(want)
