"""Launch shapes other than the tuned ones give the same answers.

The autotuner only picks among valid launch shapes; these tests run a
different setting of every shape (persistent CG CTAs capped at 8 warps,
varifold at 2 CTAs per SM, batched CG at 128 threads and 1 slice per warp)
and check:
- the forward solve and objective still match the FP64 oracle to 1e-10;
- at the icosphere-5 shell (where the warp cap changes the CTA count) the
  steps and the objective match the default shapes to 1e-10 (CG to 1e-12);
- a served request is still bitwise the same alone and in a mix.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

OTHER = {"persistMaxWarps": 8, "vfdCtasPerSm": 2, "batchBlock": 128, "batchSlicesPerWarp": 1}


def rel(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300))


@pytest.fixture
def other_shapes():
    from shape_atrophy_gb300 import api
    api.context(0)
    before = api.get_tuning()
    api.set_tuning(**OTHER)
    yield before
    api.set_tuning(**before)


def test_other_shapes_match_oracle(other_shapes):
    from oracle.oracle import Problem
    from shape_atrophy_gb300 import api, problems
    spec = problems.shell_layered(level=3, lyrCntNum=5, steps=3, cgTolVal=1e-12)
    want = Problem(spec).forward(spec["tauVarVec"], with_obj=True)
    got = api.forward(spec, trajectory=True, objective=True)
    assert got["info"]["status"] == 0
    assert rel(got["lmkStk"], want["lmkStk"]) < 1e-10
    assert rel(got["tauMat"], want["tauMat"]) < 1e-10
    assert abs(got["obj"][0] - want["obj"]) <= 1e-10 * abs(want["obj"])


def test_other_shapes_match_default_shapes_on_the_level5_shell(other_shapes):
    from shape_atrophy_gb300 import api, problems
    spec = problems.shell_layered(level=5, lyrCntNum=9, steps=3, cgTolVal=1e-12, native=True)
    runs = {}
    for name, shapes in (("default", other_shapes), ("other", OTHER)):
        api.set_tuning(**shapes)
        s = api.Session(spec, objective=True)
        s.step(3)
        x, u, _ = s.state()
        runs[name] = (x, u, s.objective())
        s.close()
        m = api.Session(spec, precision="mixed", objective=True)
        runs[name] += (m.objective(),)
        m.close()
    a, b = runs["default"], runs["other"]
    assert rel(b[0], a[0]) < 1e-10
    assert rel(b[1], a[1]) < 1e-10
    assert abs(b[2] - a[2]) <= 1e-10 * abs(a[2])
    assert abs(b[3] - a[3]) <= 1e-6 * abs(a[3])       # FP32 pair sums regrouped by the chunk count


def test_served_identity_under_other_shapes(other_shapes):
    from shape_atrophy_gb300 import api, problems
    specs = [problems.annulus_layered(angNum=48, radNum=7, steps=4),
             problems.shell_layered(level=3, lyrCntNum=5, steps=3),
             problems.shell_layered(level=2, lyrCntNum=4, steps=4)]
    probe = specs[1]
    alone = api.Server(hbm_budget=8e9, max_instances=4)
    a = alone.result(alone.submit(probe))
    alone.close()
    mix = api.Server(hbm_budget=8e9, max_instances=16)
    ids = [mix.submit(specs[0])]
    pid = mix.submit(probe)
    ids.append(mix.submit(specs[2]))
    b = mix.result(pid)
    for i in ids:
        assert mix.result(i)["info"]["status"] == 0
    mix.close()
    np.testing.assert_array_equal(a["lmk"], b["lmk"])
    np.testing.assert_array_equal(a["tau"], b["tau"])
    assert a["obj"] == b["obj"]
