"""The element-Jacobian sign check (FP64): after every step the geometry kernel compares the sign of each
element's determinant with the initial mesh's and counts the elements whose orientation flipped
(info["invertedElements"], summed over the steps).  A 2D annulus driven with a time step 125x the
workload's (dt 2.5) inverts 41-42 elements in each of its last three steps; the count must equal the one
computed from the returned trajectory itself, and the oracle's trajectory (the same CG tolerance) flips the
same elements.  The smallest |det| stays above 3e-3 of the initial smallest, so the signs are not decided
by rounding.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dets(lmk, ev):
    q = [lmk[:, ev[k]] for k in range(3)]
    a, b = q[1] - q[0], q[2] - q[0]
    return a[0] * b[1] - a[1] * b[0]


def _flips(traj, ev):
    s0 = np.sign(_dets(traj[0], ev))
    return [int(np.sum(np.sign(_dets(traj[t], ev)) != s0)) for t in range(1, traj.shape[0])]


def _case():
    from shape_atrophy_gb300 import problems
    spec = problems.annulus_layered(angNum=48, radNum=7, steps=6, cgTolVal=1e-10)
    spec["timeStp"] = 2.5
    return spec


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_inverted_elements_are_counted_per_step(precision):
    """In both precisions the sign check runs on the FP64 geometry of the FP64 node positions."""
    from shape_atrophy_gb300 import api
    spec = _case()
    ev = spec["elmObj"]["elmVtxMat"]
    got = api.forward(spec, trajectory=True, objective=False, precision=precision)
    assert got["info"]["status"] == 0
    per = _flips(got["lmkStk"], ev)
    assert sum(per) > 0 and per[:3] == [0, 0, 0]
    assert got["info"]["invertedElements"] == sum(per)


def test_inverted_elements_match_the_oracle():
    from oracle.oracle import Problem
    from shape_atrophy_gb300 import api
    spec = _case()
    ev = spec["elmObj"]["elmVtxMat"]
    got = api.forward(spec, trajectory=True, objective=False)
    assert got["info"]["status"] == 0
    per = _flips(got["lmkStk"], ev)
    want = Problem(spec).forward(spec["tauVarVec"])
    assert want["status"] == 0
    assert _flips(want["lmkStk"], ev) == per
    scale = np.abs(want["lmkStk"]).max()
    assert np.abs(got["lmkStk"] - want["lmkStk"]).max() <= 1e-6 * scale
