"""The oracle's layered (isotropic) operators against the reference's own
kernels where the two models coincide (tests/golden/make_layered_pin.py):
2D elasticity with lambda = 0 (frame moduli 2 mu on an orthonormal frame),
isotropic diffusion (spdTan = spdTsv = D), mass, yank load, reaction load and
bottom penalty, per material layer on a 4-layer periodic annulus and on a
rotated, stretched strip.  The lambda part of the layered stress has no
counterpart in the reference; it is checked against the closed form
lambda * vol * (g_a . v_a)(sum_b g_b) of the div-div form below.

The reference outputs were produced by the reference's CUDA sources compiled
for the CPU; where the reference tree is present the fixture is regenerated
and compared bit for bit.
"""
import os

import numpy as np
import pytest

from oracle.oracle import Problem

FIX = os.path.join(os.path.dirname(__file__), "golden", "layered_pin_2d.npz")
OBJ_KEYS = ["elmVtxMat", "vtxElmMat", "tanVtxMat", "tsvVtxMat", "bdrVtxMat", "vtxBdrMat", "btmVtxMat",
            "vtxBtmMat", "femVtxMat", "femIfoMat"]


def rel(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300))


def case(name, lam=None):
    z = np.load(FIX)
    g = lambda k: z[f"{name}_{k}"]
    obj = {k: g(f"obj_{k}") for k in OBJ_KEYS}
    obj["vfdVtxMat"] = obj["bdrVtxMat"]                     # unused by these operators
    mu, D = g("mu"), g("D")
    lam = np.zeros_like(mu) if lam is None else lam
    spec = dict(dim=2, elaType="isotropic", lmkIniMat=g("lmk"), elmObj=obj, elmLyrVec=g("elmLyrVec"),
                modVec=np.column_stack([lam, mu]).reshape(-1), spdLyrVec=D, ynkActPrmVec=np.array([float(g("c"))]),
                reaActPrmVec=np.array([float(g("rate"))]), tauPrmVec=np.array([0.0]), ldmWgt=0.0, knlOrder=1,
                knlWidth=0.1, knlEps=0.0, btmWgt=1.0, timeStp=0.01, timeNum=2, cgItrMax=100, cgTolSqu=1e-16)
    return spec, z, g


@pytest.mark.parametrize("name", ["annulus", "strip"])
def test_layered_operators_match_reference_kernels(name):
    spec, z, g = case(name)
    P = Problem(spec)
    lmk, v, tau = g("lmk"), g("v"), g("tau")
    errs = {"elastic": rel(P.elastic(lmk, v), g("ref_elastic"))}
    ppd, ggd = P.fem_csr(lmk)
    errs["mass"] = rel(ppd, g("ref_ppd"))
    errs["diffusion"] = rel(ggd, g("ref_ggd"))
    errs["yank"] = rel(P.yank(lmk, tau), g("ref_yank"))
    errs["reaction"] = rel(P.reaction_load(lmk, tau), g("ref_rea"))
    errs["penalty"] = rel(P.penalty(lmk, v), g("ref_pnl"))
    print(name, {k: f"{e:.1e}" for k, e in errs.items()})
    for k, e in errs.items():
        assert e <= 1e-14, (k, e)


@pytest.mark.parametrize("name", ["annulus", "strip"])
def test_lambda_term_is_the_div_div_form(name):
    """E(lambda, mu = 0) v = sum_e lambda_e vol_e (sum_b g_b . v_b) g_a, g_a the P1 basis gradients."""
    spec0, z, g = case(name)
    L = g("mu").size
    lam = np.linspace(1.0, 3.0, L)
    spec, _, _ = case(name, lam=lam)
    spec["modVec"] = np.column_stack([lam, np.zeros(L)]).reshape(-1)
    P = Problem(spec)
    lmk, v = g("lmk"), g("v")
    got = P.elastic(lmk, v)
    elm = spec["elmObj"]["elmVtxMat"]
    ly = spec["elmLyrVec"]
    want = np.zeros_like(v)
    for e in range(elm.shape[1]):
        q = lmk[:, elm[:, e]]
        Q = np.column_stack([q[:, 1] - q[:, 0], q[:, 2] - q[:, 0]])
        Qi = np.linalg.inv(Q)
        gr = np.column_stack([-Qi[0] - Qi[1], Qi[0], Qi[1]])      # basis gradients, one column per vertex
        vol = abs(np.linalg.det(Q)) / 2.0
        div = sum(gr[:, b] @ v[:, elm[b, e]] for b in range(3))
        for a in range(3):
            want[:, elm[a, e]] += lam[ly[e]] * vol * div * gr[:, a]
    assert rel(got, want) <= 1e-12


def test_fixture_is_current():
    """Regenerate from the reference (only where its tree exists) and compare bit for bit."""
    from oracle import ref
    if not ref.available():
        pytest.skip("reference tree not present on this host")
    import importlib.util
    spec = importlib.util.spec_from_file_location("mk", os.path.join(os.path.dirname(FIX), "make_layered_pin.py"))
    mk = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mk)
    R = mk.RefOps()
    z = np.load(FIX)
    rng = np.random.default_rng(20261204)
    for name, fn in (("annulus", mk.annulus_case), ("strip", mk.strip_case)):
        c = fn(R, rng)
        for k in ("ref_elastic", "ref_ppd", "ref_ggd", "ref_yank", "ref_rea", "ref_pnl"):
            np.testing.assert_array_equal(c[k], z[f"{name}_{k}"])


@pytest.mark.parametrize("name", ["annulus", "strip"])
def test_bump_and_fisher_kpp_closed_forms(name):
    """The layered model's initial concentration h exp(-|x - c|^2 / (2 sigma^2)) and reaction rate u (1 - u)."""
    spec, z, g = case(name)
    P = Problem(spec)
    lmk = g("lmk")
    tv = np.array([0.3, -0.2, 0.9, 0.25])
    want = 0.9 * np.exp(-((lmk[0] - 0.3) ** 2 + (lmk[1] + 0.2) ** 2) / (2 * 0.25 ** 2))
    assert rel(P.initial_tau(tv), want) <= 1e-15
    tau = g("tau")
    np.testing.assert_array_equal(P.activity(tau, "reaction"), (float(g("rate")) * tau) * (1.0 - tau))
    np.testing.assert_array_equal(P.activity(tau, "yank"), float(g("c")) * tau)
