"""Serving path (continuous batching of layered forward solves) on the GPU.

- every served result matches the one-call forward solve of the same
  request (1e-10 relative; the batched CG adds its partial sums in another
  grouping than the single-solve kernel);
- a request's result is bitwise the same alone and in a mix of other
  requests (its CG partial sums are grouped by its own size only);
- the device-memory budget bounds the running set, and every request
  still completes;
- a solve that does not converge fails only its own request (objective
  DBL_MAX, status SA_ERR_NOT_CONVERGED), the others are unaffected;
- mixed precision served results stay within 1e-6 of FP64;
- with more requests than the server's instance streams (eight), so that
  instances share streams with others, a request is still bitwise the same
  alone and in the mix, in FP64 and in mixed precision;
- requests the server does not run (frame model) are rejected at submit.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DBL_MAX = np.finfo(np.float64).max
SA_ERR_NOT_CONVERGED = 4


def rel(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300))


def _requests():
    from shape_atrophy_gb300 import problems
    return [
        problems.annulus_layered(angNum=48, radNum=7, steps=5),
        problems.shell_layered(level=2, lyrCntNum=4, steps=4),
        problems.annulus_layered(angNum=96, radNum=9, steps=3, target_seed=3),
        problems.shell_layered(level=3, lyrCntNum=5, steps=3),
    ]


def test_served_results_match_forward():
    from shape_atrophy_gb300 import api
    specs = _requests()
    sv = api.Server(hbm_budget=8e9, max_instances=16)
    ids = [sv.submit(sp) for sp in specs]
    res = [sv.result(i) for i in ids]
    sv.close()
    for sp, r in zip(specs, res):
        want = api.forward(sp, trajectory=True, objective=True)
        assert r["info"]["status"] == 0
        assert rel(r["lmk"], want["lmkStk"][-1]) < 1e-10
        assert rel(r["tau"], want["tauMat"][-1]) < 1e-10
        assert abs(r["obj"] - want["obj"][0]) <= 1e-10 * abs(want["obj"][0])
        assert r["latency_ms"] > 0.0


def test_result_alone_equals_result_in_mix():
    from shape_atrophy_gb300 import api
    specs = _requests()
    probe = specs[1]
    alone = api.Server(hbm_budget=8e9, max_instances=4)
    a = alone.result(alone.submit(probe))
    alone.close()
    mix = api.Server(hbm_budget=8e9, max_instances=16)
    ids = [mix.submit(sp) for sp in specs[:1]]
    pid = mix.submit(probe)
    ids += [mix.submit(sp) for sp in specs[2:]]
    b = mix.result(pid)
    for i in ids:
        mix.result(i)
    mix.close()
    np.testing.assert_array_equal(a["lmk"], b["lmk"])
    np.testing.assert_array_equal(a["tau"], b["tau"])
    assert a["obj"] == b["obj"]
    assert a["info"]["cgIterTotal"] == b["info"]["cgIterTotal"]


def test_memory_budget_bounds_running_set():
    from shape_atrophy_gb300 import api, problems
    specs = [problems.annulus_layered(angNum=64, radNum=8, steps=3, target_seed=k) for k in range(6)]
    for k, sp in enumerate(specs):
        sp["tauVarVec"] = np.array([1.0, 0.5 * k, 1.0, 0.1])    # bump at a different angle each
    # measure one instance's footprint, then allow about two and a half of them
    probe = api.Server(hbm_budget=8e9, max_instances=1)
    probe.result(probe.submit(specs[0]))
    one = probe.stats()["peakBytes"]
    probe.close()
    sv = api.Server(hbm_budget=2.5 * one, max_instances=16)
    ids = [sv.submit(sp) for sp in specs]
    res = [sv.result(i) for i in ids]
    st = sv.stats()
    sv.close()
    assert all(r["info"]["status"] == 0 for r in res)
    assert st["completed"] == len(specs)
    assert st["peakBytes"] <= 2.5 * one


def test_failed_solve_is_isolated():
    from shape_atrophy_gb300 import api
    specs = _requests()[:3]
    bad = dict(specs[1])
    bad["cgItrMax"] = 2
    sv = api.Server(hbm_budget=8e9, max_instances=16)
    ok0 = sv.submit(specs[0])
    b = sv.submit(bad)
    ok2 = sv.submit(specs[2])
    r0, rb, r2 = sv.result(ok0), sv.result(b), sv.result(ok2)
    sv.close()
    assert rb["info"]["status"] == SA_ERR_NOT_CONVERGED and rb["obj"] == DBL_MAX
    solo = api.Server(hbm_budget=8e9, max_instances=4)
    s0 = solo.result(solo.submit(specs[0]))
    s2 = solo.result(solo.submit(specs[2]))
    solo.close()
    np.testing.assert_array_equal(r0["lmk"], s0["lmk"])
    np.testing.assert_array_equal(r2["lmk"], s2["lmk"])


def test_mixed_precision_served_within_1e6():
    from shape_atrophy_gb300 import api
    specs = _requests()
    sv = api.Server(hbm_budget=8e9, max_instances=16)
    f = [sv.submit(sp) for sp in specs]
    m = [sv.submit(sp, precision="mixed") for sp in specs]
    rf = [sv.result(i) for i in f]
    rm = [sv.result(i) for i in m]
    sv.close()
    for a, b in zip(rm, rf):
        assert a["info"]["status"] == 0
        assert rel(a["lmk"], b["lmk"]) < 1e-6
        assert rel(a["tau"], b["tau"]) < 1e-6
        assert abs(a["obj"] - b["obj"]) <= 1e-6 * abs(b["obj"])


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_alone_equals_mix_with_shared_instance_streams(precision):
    from shape_atrophy_gb300 import api, problems
    specs = [problems.annulus_layered(angNum=32 + 8 * k, radNum=6, steps=3, target_seed=k) for k in range(6)]
    specs += [problems.shell_layered(level=2, lyrCntNum=3 + k % 2, steps=3, target_seed=k) for k in range(5)]
    probe = 9                                     # the tenth instance shares a stream with the second
    alone = api.Server(hbm_budget=8e9, max_instances=4)
    a = alone.result(alone.submit(specs[probe], precision=precision))
    alone.close()
    mix = api.Server(hbm_budget=8e9, max_instances=32)
    ids = [mix.submit(sp, precision=precision) for sp in specs]
    res = [mix.result(i) for i in ids]
    mix.close()
    b = res[probe]
    assert all(r["info"]["status"] == 0 for r in res)
    np.testing.assert_array_equal(a["lmk"], b["lmk"])
    np.testing.assert_array_equal(a["tau"], b["tau"])
    assert a["obj"] == b["obj"]


def test_frame_request_is_rejected():
    from shape_atrophy_gb300 import api, problems
    sv = api.Server(hbm_budget=8e9, max_instances=4)
    with pytest.raises(RuntimeError, match="layered"):
        sv.submit(problems.demo_strip(9, 4, timeEnd=0.02))
    sv.close()
