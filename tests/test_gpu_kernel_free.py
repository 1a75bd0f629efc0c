"""The frame model's K-preconditioned CG: the persistent kernel against the launch loop, and the RKHS
products with and without the stored N x N kernel matrix.

The velocity solve runs as one persistent cooperative launch (three exact grid sums per iteration) unless
cgKernel = "two-kernel" asks for the launch loop (six launches per iteration); the two sum in different
orders, so they agree to the CG tolerance, not bit for bit: every golden frame case is compared at 1e-10
(positions, concentration, objective; CG tolerance 1e-12 there), as each is against the reference.

K-preconditioned CG multiplies by K = [k(|q_i - q_j| / w) + eps delta_ij] once per iteration.  Up to 96 GiB
(N <= 113 511, memory permitting) the matrix is built once per step and streamed; beyond that, or with the
tuning switch kernelMatrixFree = 1, each product evaluates the entries from the node positions with the same
instructions in the same order.  Checked:
- every reference golden case (2D and 3D, Matern orders 0-4 and Gaussian, CG failure): the matrix-free
  forward equals the stored-matrix forward bit for bit (positions, concentration, objective);
- the frame adjoint (2D demo strip): bit for bit;
- the layered model with the LDDMM term switched on (annulus and shell): the CPU oracle at 1e-10, the launch
  loop at 1e-10, matrix-free bit for bit;
- a 30 744-node shell (7.6 GB matrix, one step): bit for bit at that size;
- a 71 694-node shell, whose 41 GB matrix has more than 65 535 columns: the solve runs, and its
  displacement is invariant to a translation of the mesh and the bump centre, to 1e-6 of its largest
  component (the two CG solves stop at a relative residual of 1e-5, possibly one iteration apart).
"""
import numpy as np
import pytest

from golden_io import load, names

pytestmark = pytest.mark.gpu


@pytest.fixture
def matrix_free():
    from shape_atrophy_gb300 import api
    api.context(0)
    before = api.get_tuning()
    yield lambda on: api.set_tuning(kernelMatrixFree=int(on))
    api.set_tuning(**before)


def _both(fn, matrix_free):
    matrix_free(False)
    a = fn()
    matrix_free(True)
    b = fn()
    matrix_free(False)
    return a, b


def test_stored_matrix_path_reproducible():
    """The comparisons below are meaningful: two stored-matrix runs give the same bits."""
    from shape_atrophy_gb300 import api
    spec, ref = load(names()[0])
    a = api.forward(spec, ref["tauVarMat"], trajectory=True, objective=True)
    b = api.forward(spec, ref["tauVarMat"], trajectory=True, objective=True)
    np.testing.assert_array_equal(a["obj"], b["obj"])
    np.testing.assert_array_equal(a["lmkStk"], b["lmkStk"])


def rel(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300))


@pytest.mark.parametrize("name", names())
def test_persistent_matches_launch_loop(name):
    from shape_atrophy_gb300 import api
    spec, ref = load(name)
    tv = ref["tauVarMat"]
    a = api.forward(spec, tv, trajectory=True, objective=True)
    loop = dict(spec, cgKernel="two-kernel")
    b = api.forward(loop, tv, trajectory=True, objective=True)
    assert a["info"]["status"] == b["info"]["status"]
    if a["info"]["status"] == 0:
        assert abs(a["info"]["cgIterTotal"] - b["info"]["cgIterTotal"]) <= 0.02 * b["info"]["cgIterTotal"] + 2
        assert rel(a["lmkStk"], b["lmkStk"]) < 1e-10
        assert rel(a["tauMat"], b["tauMat"]) < 1e-10
        assert rel(a["obj"], b["obj"]) < 1e-10
    else:
        np.testing.assert_array_equal(a["obj"], b["obj"])


@pytest.mark.parametrize("name", names())
def test_goldens_bitwise(matrix_free, name):
    from shape_atrophy_gb300 import api
    spec, ref = load(name)
    tv = ref["tauVarMat"]
    a, b = _both(lambda: api.forward(spec, tv, trajectory=True, objective=True), matrix_free)
    assert a["info"]["status"] == b["info"]["status"]
    np.testing.assert_array_equal(a["obj"], b["obj"])
    np.testing.assert_array_equal(a["lmkStk"], b["lmkStk"])
    np.testing.assert_array_equal(a["tauMat"], b["tauMat"])


def test_adjoint_bitwise(matrix_free):
    from shape_atrophy_gb300 import api, problems
    spec = problems.demo_strip(21, 7, timeEnd=0.05)
    a, b = _both(lambda: api.adjoint(spec), matrix_free)
    assert a["info"]["status"] == 0 and b["info"]["status"] == 0
    assert a["obj"] == b["obj"]
    for k in ("grad", "grad_tau0", "grad_x0"):
        np.testing.assert_array_equal(a[k], b[k])


@pytest.mark.slow
def test_large_shell_bitwise(matrix_free):
    from shape_atrophy_gb300 import api, problems
    spec = problems.frame_shell(level=4, lyrCntNum=12, timeEnd=0.01, cgTolVal=1e-6)
    assert spec["lmkIniMat"].shape[1] == 2562 * 12
    a, b = _both(lambda: api.forward(spec, trajectory=True, objective=True), matrix_free)
    assert a["info"]["status"] == 0 and b["info"]["status"] == 0
    print("K-PCG iterations", a["info"]["cgIterTotal"], b["info"]["cgIterTotal"],
          "ms", a["info"]["elapsedMs"], b["info"]["elapsedMs"])
    np.testing.assert_array_equal(a["lmkStk"], b["lmkStk"])
    np.testing.assert_array_equal(a["tauMat"], b["tauMat"])
    np.testing.assert_array_equal(a["obj"], b["obj"])


@pytest.mark.slow
def test_large_stored_matrix_translation_invariant():
    from shape_atrophy_gb300 import api, problems
    spec = problems.frame_shell(level=5, lyrCntNum=7, timeEnd=0.01, cgTolVal=1e-5)
    N = spec["lmkIniMat"].shape[1]
    assert N == 10242 * 7 and N > 65535 and N * N * 8 > 16 << 30
    a = api.forward(spec, trajectory=True, objective=False)
    assert a["info"]["status"] == 0
    shift = np.array([[0.25], [-0.5], [0.125]])
    sp = dict(spec)
    sp["lmkIniMat"] = spec["lmkIniMat"] + shift
    sp["tauVarVec"] = np.asarray(spec["tauVarVec"], dtype=float).copy()
    sp["tauVarVec"][:3] += shift[:, 0]                  # the bump centre moves with the mesh
    b = api.forward(sp, trajectory=True, objective=False)
    assert b["info"]["status"] == 0
    da = a["lmkStk"][-1] - a["lmkStk"][0]
    db = b["lmkStk"][-1] - b["lmkStk"][0]
    assert np.isfinite(da).all() and np.abs(da).max() > 0
    print("K-PCG iterations", a["info"]["cgIterTotal"], b["info"]["cgIterTotal"], "ms", a["info"]["elapsedMs"],
          "translation difference", np.abs(da - db).max() / np.abs(da).max())
    assert np.abs(da - db).max() <= 1e-6 * np.abs(da).max()
    assert np.abs(a["tauMat"] - b["tauMat"]).max() <= 1e-6 * np.abs(a["tauMat"]).max()


def _layered_rkhs(case):
    from shape_atrophy_gb300 import problems
    if case == "annulus":
        spec = problems.annulus_layered(angNum=48, radNum=7, steps=4, cgTolVal=1e-12)
    else:
        spec = problems.shell_layered(level=2, lyrCntNum=4, steps=3, cgTolVal=1e-12)
    return dict(spec, ldmWgt=1e-2, knlOrder=1, knlWidth=0.2, knlEps=1e-10)


@pytest.mark.parametrize("case", ["annulus", "shell"])
def test_layered_model_with_rkhs_term(matrix_free, case):
    """The layered model with the LDDMM term switched on (ldmWgt != 0) runs the same K-preconditioned CG on
    the layered operator: oracle parity at 1e-10, the launch loop at 1e-10, matrix-free bit for bit."""
    from oracle.oracle import Problem
    from shape_atrophy_gb300 import api
    spec = _layered_rkhs(case)
    want = Problem(spec).forward(spec["tauVarVec"], with_obj=True)
    assert want["status"] == 0
    a, b = _both(lambda: api.forward(spec, trajectory=True, objective=True), matrix_free)
    loop = api.forward(dict(spec, cgKernel="two-kernel"), trajectory=True, objective=True)
    for got in (a, b, loop):
        assert got["info"]["status"] == 0
        assert rel(got["lmkStk"], want["lmkStk"]) < 1e-10
        assert rel(got["tauMat"], want["tauMat"]) < 1e-10
        assert abs(got["obj"][0] - want["obj"]) <= 1e-10 * abs(want["obj"])
    np.testing.assert_array_equal(a["lmkStk"], b["lmkStk"])
    np.testing.assert_array_equal(a["obj"], b["obj"])
