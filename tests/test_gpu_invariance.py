"""Size-independent properties of the CUDA path at the workload's sizes.

* The layered model is invariant under rigid motions: moving the initial
  shape, the bump centre and the varifold target by a translation and a
  rotation moves the whole trajectory the same way and leaves the
  concentration and the objective unchanged (isotropic per-layer
  elasticity, P1 mass and diffusion, bottom penalty, Gaussian bump and the
  varifold are all frame-indifferent; a wrong index in an assembled 3x3
  block would break the rotation case).
* The varifold distance of a shape to its own varifold is zero, FP64 and
  mixed precision."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _rotation(seed):
    q, r = np.linalg.qr(np.random.default_rng(seed).normal(size=(3, 3)))
    q = q * np.sign(np.diag(r))
    if np.linalg.det(q) < 0:
        q[:, 0] = -q[:, 0]
    return q


def _moved(spec, R, t):
    s = dict(spec)
    s["lmkIniMat"] = R @ spec["lmkIniMat"] + t[:, None]
    tv = np.array(spec["tauVarVec"], dtype=float)
    tv[:3] = R @ tv[:3] + t
    s["tauVarVec"] = tv
    cen, dirs, vol = spec["tgt"]
    s["tgt"] = (np.ascontiguousarray(R @ cen + t[:, None]), np.ascontiguousarray(R @ dirs), vol.copy())
    return s


@pytest.mark.parametrize("level", [4, 5])
def test_layered_shell_is_invariant_under_rigid_motions(level):
    from shape_atrophy_gb300 import api, problems
    spec = problems.shell_layered(level=level, lyrCntNum=9, steps=6, native=True)
    spec["cgTolSqu"] = 1e-24
    spec["rdTolSqu"] = 1e-24
    base = api.forward(spec, trajectory=True, objective=True)
    R, t = _rotation(level), np.array([0.37, -1.25, 2.5])
    got = api.forward(_moved(spec, R, t), trajectory=True, objective=True)
    assert base["info"]["status"] == 0 and got["info"]["status"] == 0
    disp = base["lmkStk"][-1] - base["lmkStk"][0]
    back = np.einsum("ij,tjn->tin", R.T, got["lmkStk"] - t[None, :, None])
    assert np.abs(back - base["lmkStk"]).max() <= 1e-8 * np.abs(disp).max()
    np.testing.assert_allclose(got["tauMat"], base["tauMat"], rtol=0, atol=1e-10 * np.abs(base["tauMat"]).max())
    assert got["obj"][0] == pytest.approx(base["obj"][0], rel=1e-9)


@pytest.mark.parametrize("precision, tol", [("fp64", 1e-13), ("mixed", 1e-8)])
def test_varifold_of_a_shape_against_itself_is_zero(precision, tol):
    from shape_atrophy_gb300 import api, mesh, problems
    spec = problems.shell_layered(level=5, lyrCntNum=9, steps=2, native=True)
    lmk = spec["lmkIniMat"]
    cen, dirs, vol = mesh.varifold_target(lmk, spec["elmObj"]["vfdVtxMat"])
    same = dict(spec, tgt=(cen, dirs, vol))
    far = dict(spec, tgt=(cen + 100.0, dirs, vol))             # DD + TT, the cross term vanishes
    j_same = api.varifold(same, lmk, precision=precision)
    j_far = api.varifold(far, lmk, precision=precision)
    assert j_far > 0.0
    assert abs(j_same) <= tol * j_far
