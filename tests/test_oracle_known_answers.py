"""Known-answer tests of the CPU oracle from the mathematics of the model.

The reference ships no tests; these properties hold for the exact operators
whatever the mesh, so they check the oracle's restatement independently of
the golden vectors:

* the assembled P1 mass matrix sums to the mesh's area / volume;
* the diffusion (stiffness) matrix annihilates constants (zero row sums);
* the elasticity operator annihilates rigid translations and infinitesimal
  rotations and is symmetric
  (x . E y = y . E x), frame and layered models, 2D and 3D; the bottom
  penalty is symmetric;
* the layered velocity solve's block-Jacobi blocks are the diagonal blocks of
  E + btmWgt P (probed with unit fields), symmetric, and inverted exactly;
* the RKHS kernel matrix equals the closed forms of the half-integer Matern
  kernels (nu = p + 1/2: e^-r times a degree-p polynomial, generated here
  from the general formula) and the Gaussian in 3D; in 2D (rational Bessel
  approximations) its diagonal is 1 and it is symmetric;
* the varifold distance of a shape to its own varifold is zero;
* the varifold node gradient agrees with central differences.
"""
import math

import numpy as np
import pytest

from oracle.oracle import Problem
from shape_atrophy_gb300 import mesh, problems


def _cases():
    return {
        "strip2d_frame": lambda: problems.demo_strip(21, 5, timeEnd=0.02),
        "shell3d_frame": lambda: problems.frame_shell(level=1, lyrCntNum=3, timeEnd=0.02),
        "annulus2d_layered": lambda: problems.annulus_layered(angNum=32, radNum=6, steps=2),
        "shell3d_layered": lambda: problems.shell_layered(level=2, lyrCntNum=3, steps=2),
    }


CASES = _cases()


def _volumes(lmk, elm):
    D = lmk.shape[0]
    q = [lmk[:, elm[k]] for k in range(D + 1)]
    if D == 2:
        a, b = q[1] - q[0], q[2] - q[0]
        return np.abs(a[0] * b[1] - a[1] * b[0]) / 2.0
    a, b, c = q[1] - q[0], q[2] - q[0], q[3] - q[0]
    det = (a[0] * (b[1] * c[2] - b[2] * c[1]) - a[1] * (b[0] * c[2] - b[2] * c[0]) +
           a[2] * (b[0] * c[1] - b[1] * c[0]))
    return np.abs(det) / 6.0


@pytest.mark.parametrize("name", list(CASES))
def test_mass_sums_to_volume_and_stiffness_annihilates_constants(name):
    spec = CASES[name]()
    P = Problem(spec)
    lmk = spec["lmkIniMat"]
    mass, stiff = P.fem_csr(lmk)
    vol = _volumes(lmk, spec["elmObj"]["elmVtxMat"]).sum()
    assert mass.sum() == pytest.approx(vol, rel=1e-13)
    rows = spec["elmObj"]["femVtxMat"][0]
    rowsum = np.bincount(rows, weights=stiff, minlength=lmk.shape[1])
    diag = np.abs(stiff[rows == spec["elmObj"]["femVtxMat"][1]])
    assert np.abs(rowsum).max() <= 1e-12 * diag.max()


@pytest.mark.parametrize("name", list(CASES))
def test_elasticity_annihilates_rigid_motions_and_is_symmetric(name):
    spec = CASES[name]()
    P = Problem(spec)
    lmk = spec["lmkIniMat"]
    D, N = lmk.shape
    rng = np.random.default_rng(3)
    x, y = rng.normal(size=(D, N)), rng.normal(size=(D, N))
    Ex, Ey = P.elastic(lmk, x), P.elastic(lmk, y)
    scale = np.abs(Ex).max()
    for d in range(D):
        t = np.zeros((D, N))
        t[d] = 1.7
        assert np.abs(P.elastic(lmk, t)).max() <= 1e-12 * scale
    # infinitesimal rigid rotations v = W x (W skew) have zero linear strain
    w = rng.normal(size=3)
    W = (np.array([[0.0, -1.0], [1.0, 0.0]]) if D == 2 else
         np.array([[0.0, -w[2], w[1]], [w[2], 0.0, -w[0]], [-w[1], w[0], 0.0]]))
    assert np.abs(P.elastic(lmk, W @ lmk)).max() <= 1e-12 * scale
    assert np.vdot(x, Ey) == pytest.approx(np.vdot(y, Ex), rel=1e-12)
    if spec["btmWgt"] != 0.0 or spec["elmObj"]["btmVtxMat"].shape[1] > 0:
        Px, Py = P.penalty(lmk, x), P.penalty(lmk, y)
        assert np.vdot(x, Py) == pytest.approx(np.vdot(y, Px), rel=1e-12, abs=1e-14)


@pytest.mark.parametrize("name", [k for k in CASES if k.endswith("layered")])
def test_block_jacobi_blocks_are_the_operator_diagonal_blocks(name):
    """The velocity solve's block-Jacobi preconditioner: node i's D x D block equals rows i of
    (E + btmWgt P) applied to the unit fields e_(i,c), every block is symmetric, and the inverse
    returned times the block is the identity."""
    spec = CASES[name]()
    P = Problem(spec)
    lmk = spec["lmkIniMat"]
    D, N = lmk.shape
    blk = P.elastic_blocks(lmk)
    inv = P.elastic_blocks(lmk, inverse=True)
    rng = np.random.default_rng(5)
    nodes = rng.choice(N, size=min(N, 12), replace=False)
    btm = spec["elmObj"]["btmVtxMat"]
    if btm.shape[1] > 0:
        nodes = np.concatenate([nodes, btm[0, :3]])    # some with the bottom penalty
    scale = np.abs(blk).max()
    for i in nodes:
        for c in range(D):
            e = np.zeros((D, N))
            e[c, i] = 1.0
            col = P.elastic(lmk, e)[:, i] + spec["btmWgt"] * P.penalty(lmk, e)[:, i]
            np.testing.assert_allclose(blk[i][:, c], col, rtol=0, atol=1e-13 * scale)
    np.testing.assert_allclose(blk, np.swapaxes(blk, 1, 2), rtol=0, atol=1e-14 * scale)
    eye = np.einsum("nab,nbc->nac", inv, blk)
    np.testing.assert_allclose(eye, np.broadcast_to(np.eye(D), eye.shape), rtol=0, atol=1e-12)
    np.testing.assert_array_equal(np.stack([blk[:, d, d] for d in range(D)]), P.elastic_diag(lmk))


def _matern_half_integer(p, r):
    """Matern nu = p + 1/2 in the scaled distance r: e^-r (p!/(2p)!) sum_i (p+i)!/(i!(p-i)!) (2r)^(p-i)."""
    s = sum(math.factorial(p + i) / (math.factorial(i) * math.factorial(p - i)) * (2.0 * r) ** (p - i)
            for i in range(p + 1))
    return np.exp(-r) * s * math.factorial(p) / math.factorial(2 * p)


@pytest.mark.parametrize("order", [-1, 0, 1, 2, 3, 4])
def test_kernel_matrix_closed_forms_3d(order):
    spec = problems.frame_shell(level=1, lyrCntNum=3, timeEnd=0.02, knlOrder=order)
    P = Problem(spec)
    lmk = spec["lmkIniMat"]
    K = P.kernel_matrix(lmk)
    d = np.sqrt(((lmk[:, :, None] - lmk[:, None, :]) ** 2).sum(0))
    w = spec["knlWidth"]
    want = np.exp(-(d / w) ** 2) if order == -1 else _matern_half_integer(order, d / w)
    np.testing.assert_allclose(K, want, rtol=1e-13, atol=1e-15)


@pytest.mark.parametrize("order", [0, 1, 2, 3, 4])
def test_kernel_matrix_2d_unit_diagonal_and_symmetric(order):
    spec = problems.demo_strip(21, 5, timeEnd=0.02)
    spec["knlOrder"] = order
    P = Problem(spec)
    K = P.kernel_matrix(spec["lmkIniMat"])
    np.testing.assert_allclose(np.diag(K), 1.0, rtol=1e-12)
    np.testing.assert_allclose(K, K.T, rtol=1e-13, atol=1e-15)
    assert np.all(K <= 1.0 + 1e-12) and np.all(K > 0.0)


def _self_target(spec, lmk):
    s = dict(spec)
    cen, dirs, vol = mesh.varifold_target(lmk, spec["elmObj"]["vfdVtxMat"])
    s["tgt"] = (cen, dirs, vol)
    return s


@pytest.mark.parametrize("name", list(CASES))
def test_varifold_of_a_shape_against_itself_is_zero(name):
    spec = CASES[name]()
    lmk = spec["lmkIniMat"]
    same = Problem(_self_target(spec, lmk)).varifold(lmk)
    far = Problem(_self_target(spec, lmk + 100.0)).varifold(lmk)   # DD + TT, the cross term vanishes
    assert far > 0.0
    assert abs(same) <= 1e-13 * far


@pytest.mark.parametrize("name", ["strip2d_frame", "shell3d_layered"])
def test_varifold_gradient_matches_central_differences(name):
    spec = CASES[name]()
    P = Problem(spec)
    lmk = spec["lmkIniMat"]
    _, g = P.varifold(lmk, grad=True)
    nodes = np.unique(spec["elmObj"]["vfdVtxMat"])
    rng = np.random.default_rng(7)
    h = 1e-6
    for k in rng.choice(nodes, 6, replace=False):
        for d in range(lmk.shape[0]):
            xp, xm = lmk.copy(), lmk.copy()
            xp[d, k] += h
            xm[d, k] -= h
            fd = (P.varifold(xp) - P.varifold(xm)) / (2 * h)
            assert fd == pytest.approx(g[d, k], rel=1e-6, abs=1e-9 * np.abs(g).max())
