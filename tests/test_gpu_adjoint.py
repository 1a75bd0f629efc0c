"""Discrete adjoint of the layered model (sa_objective_adjoint) on the GPU.

- its bump gradient equals the tangent-linear model's (sa_objective_gradient) to 1e-8 of the largest
  component: two exact differentiations of the same discrete model, each up to its CG tolerance;
- every kind of gradient it returns (bump [c, h, sigma], per-layer lambda, mu, D, initial node
  positions at a few nodes) matches central differences of the CPU oracle's objective (not the GPU's
  own forward solve) to 1e-5 of the largest component of that kind of gradient;
- the gradient with respect to the initial concentration is consistent with the bump gradient
  (chain rule through tau_0 = h exp(-|x - c|^2 / (2 sigma^2))).

Small layered annulus (48 x 7 nodes, 4 material layers, 6 steps) and shell (icosphere 2 x 3 prism
layers, 3 material layers, 4 steps), CG tolerance 1e-12.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _case(dim):
    from shape_atrophy_gb300 import problems
    if dim == 2:
        return problems.annulus_layered(angNum=48, radNum=7, steps=6, cgTolVal=1e-12)
    return problems.shell_layered(level=2, lyrCntNum=4, steps=4, cgTolVal=1e-12)


def _oracle_obj(spec, tv=None):
    from oracle.oracle import Problem
    r = Problem(spec).forward(spec["tauVarVec"] if tv is None else tv, with_obj=True)
    assert r["status"] == 0
    return r["obj"]


def _central(spec, setter, value, h):
    sp = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in spec.items()}
    setter(sp, value + h)
    jp = _oracle_obj(sp)
    sp = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in spec.items()}
    setter(sp, value - h)
    jm = _oracle_obj(sp)
    return (jp - jm) / (2.0 * h)


@pytest.fixture(scope="module", params=[2, 3])
def run(request):
    from shape_atrophy_gb300 import api
    spec = _case(request.param)
    adj = api.adjoint(spec)
    assert adj["info"]["status"] == 0
    return spec, adj


def test_adjoint_equals_tangent_linear(run):
    from shape_atrophy_gb300 import api
    spec, adj = run
    tan = api.gradient(spec)
    assert abs(adj["obj"] - tan["obj"]) <= 1e-12 * abs(tan["obj"])
    scale = np.abs(tan["grad"]).max()
    assert np.abs(adj["grad"] - tan["grad"]).max() <= 1e-8 * scale, (adj["grad"], tan["grad"])


def test_bump_gradient_matches_oracle_differences(run):
    spec, adj = run
    D = spec["dim"]
    tv0 = np.asarray(spec["tauVarVec"], dtype=float)
    fd = np.zeros(D + 2)
    for k in range(D + 2):
        def setter(sp, val, k=k):
            t = tv0.copy()
            t[k] = val
            sp["tauVarVec"] = t
        fd[k] = _central(spec, setter, tv0[k], 1e-6 * max(1.0, abs(tv0[k])))
    assert np.abs(adj["grad"] - fd).max() <= 1e-5 * np.abs(fd).max(), (adj["grad"], fd)


def test_layer_gradients_match_oracle_differences(run):
    spec, adj = run
    mv0 = np.asarray(spec["modVec"], dtype=float)
    sp0 = np.asarray(spec["spdLyrVec"], dtype=float)
    L = sp0.size
    got, fd = [], []
    for l in range(L):
        for j, name in enumerate(("lambda", "mu", "D")):
            if name == "D":
                def setter(sp, val, l=l):
                    a = sp0.copy(); a[l] = val; sp["spdLyrVec"] = a
                v0 = sp0[l]
            else:
                def setter(sp, val, l=l, j=j):
                    a = mv0.copy(); a[2 * l + j] = val; sp["modVec"] = a
                v0 = mv0[2 * l + j]
            fd.append(_central(spec, setter, v0, 1e-3 * v0))     # the objective moves little with a modulus:
                                                                  # smaller steps are dominated by solve noise
            got.append(adj["grad_layer"][l, j])
    got, fd = np.array(got), np.array(fd)
    for j in range(3):                        # each kind of modulus against its own scale
        g, f = got[j::3], fd[j::3]
        assert np.abs(g - f).max() <= 1e-5 * np.abs(f).max(), (j, g, f)


def test_shape_gradient_matches_oracle_differences(run):
    spec, adj = run
    x0 = np.asarray(spec["lmkIniMat"], dtype=float)
    N = x0.shape[1]
    rng = np.random.default_rng(3)
    nodes = rng.choice(N, 4, replace=False)
    got, fd = [], []
    for i in nodes:
        for d in range(spec["dim"]):
            def setter(sp, val, i=i, d=d):
                x = x0.copy(); x[d, i] = val; sp["lmkIniMat"] = x
            fd.append(_central(spec, setter, x0[d, i], 1e-4))
            got.append(adj["grad_x0"][d, i])
    got, fd = np.array(got), np.array(fd)
    assert np.abs(got - fd).max() <= 1e-5 * np.abs(adj["grad_x0"]).max(), (got, fd)


def test_concentration_gradient_chains_to_bump_gradient(run):
    """dJ/dh = sum_i dJ/dtau0_i exp(-|x_i - c|^2 / (2 sigma^2)): the per-node gradient carries the bump's."""
    spec, adj = run
    D = spec["dim"]
    tv = np.asarray(spec["tauVarVec"], dtype=float)
    x = np.asarray(spec["lmkIniMat"], dtype=float)
    r2 = ((x - tv[:D, None]) ** 2).sum(0)
    dh = float(np.dot(adj["grad_tau0"], np.exp(-r2 / (2 * tv[D + 1] ** 2))))
    assert abs(dh - adj["grad"][D]) <= 1e-10 * np.abs(adj["grad"]).max()
