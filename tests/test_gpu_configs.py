"""The CUDA path against the FP64 CPU oracle at the workloads' own sizes.

* 2D layered annulus: 16 radial x 256 angular nodes (4096 nodes, 7680
  triangles), 4 material layers, 50 steps of dt 0.02 -- the whole workload,
  every step compared: 1e-10 relative at CG tolerance 1e-12, and at the
  workload's own tolerance 1e-8 1e-9 in positions, 1e-8 in concentration
  and objective.  At 1e-8 the concentration is known only to its solve's
  tolerance: the oracle itself moves by ~1e-9 in concentration when the
  initial nodes are perturbed by 1e-15 relative (the velocity and
  reaction-diffusion solves stop an iteration earlier or later), so the
  bound there is the solves' relative residual; the test prints that
  spread beside the GPU's difference.
* 3D layered shell: icosphere 5 x 8 prism layers (92 178 nodes, 491 520
  tets), 3 material layers, dt 0.01: the first 20 steps at the workload's
  tolerance 1e-8 (1e-9 in positions and concentration, 1e-8 in the
  objective), the first 5 steps at 1e-12 (1e-10).
* Mixed precision on the same shell (FP32 operator and inner CG, FP64 dots
  and refinement, FP32 pair sums): against the FP64 oracle at steps 10 and
  20, at most 1e-6 relative in positions, concentration and objective.

Relative error = max |a - b| / max |b| over the whole trajectory (or the
step compared).  The oracle runs in its -O3 -march=native build, whose
results equal the parity build's bit for bit (tests/test_oracle_golden.py).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300))


def oracle(spec):
    from oracle.oracle import Problem
    P = Problem(spec, fast=True)
    r = P.forward(spec["tauVarVec"], with_obj=True)
    assert r["status"] == 0
    r["problem"] = P
    return r


def report(name, **errs):
    print(f"[{name}] " + ", ".join(f"{k} {v:.2e}" for k, v in errs.items()))


# ---------------------------------------------------------------------------
# 2D annulus, the whole workload
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("tol,bound,tau_bound,obj_bound", [(1e-12, 1e-10, 1e-10, 1e-10), (1e-8, 1e-9, 1e-8, 1e-8)])
def test_annulus_workload_matches_oracle(tol, bound, tau_bound, obj_bound):
    from shape_atrophy_gb300 import api, problems
    spec = problems.annulus_layered(cgTolVal=tol)
    assert spec["lmkIniMat"].shape[1] == 4096 and spec["elmObj"]["elmVtxMat"].shape[1] == 7680
    assert spec["timeNum"] == 51
    got = api.forward(spec, trajectory=True, objective=True)
    want = oracle(spec)
    assert got["info"]["status"] == 0
    e = dict(positions=rel(got["lmkStk"], want["lmkStk"]), concentration=rel(got["tauMat"], want["tauMat"]),
             displacement=rel(got["lmkStk"] - got["lmkStk"][0], want["lmkStk"] - want["lmkStk"][0]),
             objective=abs(got["obj"][0] - want["obj"]) / abs(want["obj"]))
    report(f"annulus 4096 nodes, 50 steps, cg tol {tol:g}", **e)
    if tol > 1e-10:
        # the oracle against itself, initial nodes perturbed by 1e-15 relative
        pert = dict(spec)
        pert["lmkIniMat"] = spec["lmkIniMat"] * (1.0 + 1e-15 * np.random.default_rng(1).standard_normal(
            spec["lmkIniMat"].shape))
        again = oracle(pert)
        report("oracle, initial nodes perturbed by 1e-15", positions=rel(again["lmkStk"], want["lmkStk"]),
               concentration=rel(again["tauMat"], want["tauMat"]))
    assert e["positions"] < bound and e["concentration"] < tau_bound
    assert e["objective"] < obj_bound


# ---------------------------------------------------------------------------
# 3D shell, icosphere 5 x 8 prism layers
# ---------------------------------------------------------------------------
@pytest.fixture(scope="module")
def shell20():
    from shape_atrophy_gb300 import problems
    spec = problems.shell_layered(steps=20, native=True)
    assert spec["lmkIniMat"].shape[1] == 92178 and spec["elmObj"]["elmVtxMat"].shape[1] == 491520
    return spec, oracle(spec)


def test_shell_workload_20_steps_match_oracle(shell20):
    from shape_atrophy_gb300 import api
    spec, want = shell20
    got = api.forward(spec, trajectory=True, objective=True)
    assert got["info"]["status"] == 0
    e = dict(positions=rel(got["lmkStk"], want["lmkStk"]), concentration=rel(got["tauMat"], want["tauMat"]),
             displacement=rel(got["lmkStk"] - got["lmkStk"][0], want["lmkStk"] - want["lmkStk"][0]),
             objective=abs(got["obj"][0] - want["obj"]) / abs(want["obj"]))
    report("shell 92178 nodes, 20 steps, cg tol 1e-8", **e)
    assert e["positions"] < 1e-9 and e["concentration"] < 1e-9
    assert e["objective"] < 1e-8


def test_shell_parity_tolerance_5_steps_match_oracle():
    from shape_atrophy_gb300 import api, problems
    spec = problems.shell_layered(steps=5, cgTolVal=1e-12, native=True)
    got = api.forward(spec, trajectory=True, objective=True)
    want = oracle(spec)
    assert got["info"]["status"] == 0
    e = dict(positions=rel(got["lmkStk"], want["lmkStk"]), concentration=rel(got["tauMat"], want["tauMat"]),
             objective=abs(got["obj"][0] - want["obj"]) / abs(want["obj"]))
    report("shell 92178 nodes, 5 steps, cg tol 1e-12", **e)
    assert max(e.values()) < 1e-10


def test_shell_mixed_precision_against_fp64_oracle(shell20):
    """Mixed precision at every 10th step against the FP64 oracle (positions, concentration, objective)."""
    from shape_atrophy_gb300 import api
    spec, want = shell20
    P = want["problem"]
    sess = api.Session(spec, precision="mixed", objective=True)
    try:
        for t in (10, 20):
            assert sess.step(10) == 10
            x, u, _ = sess.state()
            o = sess.objective()
            o_ref = P.varifold(want["lmkStk"][t])
            e = dict(positions=rel(x, want["lmkStk"][t]), concentration=rel(u, want["tauMat"][t]),
                     objective=abs(o - o_ref) / abs(o_ref))
            report(f"shell mixed vs FP64 oracle, step {t}", **e)
            assert max(e.values()) <= 1e-6, (t, e)
    finally:
        sess.close()
