"""Discrete adjoint of the reference's own (frame) model on the GPU.

The frame model's sweep differentiates what the layered one does not have: element frames built from other
nodes (normalised sums of edge directions, 3D triangle normals), the frame stress and the anisotropic
diffusion, the projected 3D bottom penalty, the activity templates, the dense RKHS term ldmWgt K^{-1} of
the velocity operator (an N-body sum of kernel gradients) and the polynomial bump.  Checked against central
differences of the CPU oracle's objective (the oracle agrees with the reference's compiled frame model bit
for bit): dJ/d tauVar (2D [cx, cy, h, R], 3D [cx, cy, cz, h]) and dJ/d(initial node positions) at a few
nodes, to 1e-5 of the largest component; dJ/dtau_0 carries dJ/dh by the chain rule.  The reference demo
on a 21 x 7 strip (5 steps, Matern order 3) and a frame shell (icosphere 2 x 2 prism layers, 3 steps),
CG tolerance 1e-12.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _case(dim):
    from shape_atrophy_gb300 import problems
    if dim == 2:
        return problems.demo_strip(21, 7, timeEnd=0.05)
    return problems.frame_shell(2, 3, timeEnd=0.03)


def _oracle_obj(spec, tv):
    from oracle.oracle import Problem
    r = Problem(spec).forward(tv, with_obj=True)
    assert r["status"] == 0
    return r["obj"]


@pytest.fixture(scope="module", params=[2, 3])
def run(request):
    from shape_atrophy_gb300 import api
    spec = _case(request.param)
    adj = api.adjoint(spec)
    assert adj["info"]["status"] == 0
    return spec, adj


def test_objective_equals_forward(run):
    from shape_atrophy_gb300 import api
    spec, adj = run
    f = api.forward(spec, trajectory=False, objective=True)
    assert abs(adj["obj"] - f["obj"][0]) <= 1e-12 * abs(f["obj"][0])


def test_tauvar_gradient_matches_oracle_differences(run):
    spec, adj = run
    tv0 = np.asarray(spec["tauVarVec"], dtype=float)
    fd = np.zeros(4)
    for k in range(4):
        h = 1e-5 * max(1.0, abs(tv0[k]))
        a, b = tv0.copy(), tv0.copy()
        a[k] += h
        b[k] -= h
        fd[k] = (_oracle_obj(spec, a) - _oracle_obj(spec, b)) / (2 * h)
    print("adjoint", adj["grad"], "oracle differences", fd)
    assert np.abs(adj["grad"] - fd).max() <= 1e-5 * np.abs(fd).max(), (adj["grad"], fd)


def test_shape_gradient_matches_oracle_differences(run):
    spec, adj = run
    x0 = np.asarray(spec["lmkIniMat"], dtype=float)
    N = x0.shape[1]
    rng = np.random.default_rng(5)
    got, fd = [], []
    for i in rng.choice(N, 4, replace=False):
        for d in range(spec["dim"]):
            h = 1e-5
            sp = dict(spec)
            x = x0.copy(); x[d, i] += h; sp["lmkIniMat"] = x
            jp = _oracle_obj(sp, spec["tauVarVec"])
            x = x0.copy(); x[d, i] -= h; sp["lmkIniMat"] = x
            jm = _oracle_obj(sp, spec["tauVarVec"])
            fd.append((jp - jm) / (2 * h))
            got.append(adj["grad_x0"][d, i])
    got, fd = np.array(got), np.array(fd)
    print("adjoint", got, "oracle differences", fd)
    assert np.abs(got - fd).max() <= 1e-5 * np.abs(adj["grad_x0"]).max(), (got, fd)


def test_concentration_gradient_chains_to_height(run):
    """dJ/dh = sum_i dJ/dtau0_i tau0_i / h (tau_0 is linear in the height)."""
    from oracle.oracle import Problem
    spec, adj = run
    tv = np.asarray(spec["tauVarVec"], dtype=float)
    k_h = 2 if spec["dim"] == 2 else 3
    tau0 = Problem(spec).initial_tau(tv)
    dh = float(np.dot(adj["grad_tau0"], tau0 / tv[k_h]))
    assert abs(dh - adj["grad"][k_h]) <= 1e-10 * np.abs(adj["grad"]).max()
