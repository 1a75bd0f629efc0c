"""Failure detection without a GPU fault.

The CG kernels' grid waits are bounded (1 s by the GPU global timer).  A
cooperative launch on a barrier that can never complete (its count starts
2^31 below the target: a flag nothing sets) must end with every CTA giving
up and the abort flag set -- no hang, no fault -- and the context must
still run a solve afterwards.  Failures of a solve itself (no convergence)
are per-request statuses, covered in test_gpu_server.py."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_bounded_grid_wait_gives_up_and_context_survives():
    from shape_atrophy_gb300 import api, problems
    ctx = api.context(0)
    fn = ctx.lib.sa_selftest_wait_timeout
    fn.argtypes = [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_double)]
    gave, ms = C.c_int(), C.c_double()
    rc = fn(ctx.h, C.byref(gave), C.byref(ms))
    assert rc == 0, ctx.lib.sa_error_message(ctx.h)
    assert gave.value == 2
    assert 900.0 <= ms.value < 10_000.0               # waited for the limit, then returned
    spec = problems.annulus_layered(angNum=32, radNum=6, steps=2)
    got = api.forward(spec)
    assert got["info"]["status"] == 0 and np.all(np.isfinite(got["lmkStk"]))
