"""Streamed trajectory (sa_session_stream) on the GPU.

- the snapshots of a streamed run are bitwise the trajectory of the one-call
  forward solve at the same steps (stride 1 and stride 3, shell and annulus);
- maxSnapshots bounds what is written, NULL outputs are allowed, and a
  stream continues a session stepped before (snapshots by session step);
- a stream stops at timeNum - 1 like sa_session_step.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _cases():
    from shape_atrophy_gb300 import problems
    return {"shell": problems.shell_layered(level=3, lyrCntNum=5, steps=9),
            "annulus": problems.annulus_layered(angNum=48, radNum=7, steps=9)}


@pytest.mark.parametrize("name", ["shell", "annulus"])
@pytest.mark.parametrize("stride", [1, 3])
def test_stream_equals_forward_trajectory(name, stride):
    from shape_atrophy_gb300 import api
    spec = _cases()[name]
    full = api.forward(spec, trajectory=True, objective=False)
    sess = api.Session(spec, objective=False)
    lmk, tau, done = sess.stream(spec["timeNum"] - 1, stride)
    sess.close()
    assert done == spec["timeNum"] - 1
    steps = list(range(stride, spec["timeNum"], stride))
    assert lmk.shape[0] == len(steps) and tau.shape[0] == len(steps)
    for k, t in enumerate(steps):
        np.testing.assert_array_equal(lmk[k], full["lmkStk"][t])
        np.testing.assert_array_equal(tau[k], full["tauMat"][t])


def test_stream_limits_and_continuation():
    from shape_atrophy_gb300 import api
    spec = _cases()["shell"]
    full = api.forward(spec, trajectory=True, objective=False)
    sess = api.Session(spec, objective=False)
    assert sess.step(2) == 2                                   # session at step 2
    lmk, tau, done = sess.stream(4, 2, max_snapshots=1, concentration=False)
    assert done == 4 and tau is None and lmk.shape[0] == 1     # steps 3..6; snapshots at 4 (6 over the limit)
    np.testing.assert_array_equal(lmk[0], full["lmkStk"][4])
    _, tau2, done2 = sess.stream(100, 1, positions=False)      # runs to timeNum - 1 = 9 only
    assert done2 == 3 and tau2.shape[0] == 3
    np.testing.assert_array_equal(tau2, full["tauMat"][7:10])
    sess.close()
