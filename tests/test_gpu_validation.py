"""Index validation of the element object on the one-call path (host inputs,
arrays large enough that the checks run split over host threads): each
corrupted array is rejected with its own message, and the call returns an
error instead of faulting.  The corruption is made on the host, in numpy
copies of a valid icosphere-3 shell element object."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def spec():
    from shape_atrophy_gb300 import problems
    return problems.shell_layered(level=3, lyrCntNum=5, steps=2)


def _run(spec, key, mutate):
    from shape_atrophy_gb300 import api
    sp = dict(spec)
    obj = dict(sp["elmObj"])
    arr = np.array(obj[key], copy=True)
    mutate(arr)
    obj[key] = arr
    sp["elmObj"] = obj
    return api.forward(sp, trajectory=False, objective=False)


def test_valid_object_runs(spec):
    from shape_atrophy_gb300 import api
    assert api.forward(spec, trajectory=False, objective=False)["info"]["status"] == 0


def test_unsorted_pattern_rejected(spec):
    def m(a):
        z = a.shape[1] // 2
        a[:, [z, z + 1]] = a[:, [z + 1, z]]
    with pytest.raises(RuntimeError, match="sorted"):
        _run(spec, "femVtxMat", m)


def test_pattern_index_out_of_range_rejected(spec):
    def m(a):
        a[1, -1] = 10 ** 7
    with pytest.raises(RuntimeError, match="femVtxMat index out of range"):
        _run(spec, "femVtxMat", m)


def test_asymmetric_element_lists_rejected(spec):
    def m(a):
        fv = spec["elmObj"]["femVtxMat"]
        z = int(np.nonzero((fv[0] != fv[1]) & (a[0] > 1))[0][10])
        a[0, z] -= 1                                        # (i, j) lists one element fewer than (j, i)
    with pytest.raises(RuntimeError, match="differ between"):
        _run(spec, "femIfoMat", m)


def test_count_beyond_columns_rejected(spec):
    def m(a):
        a[0, 5] = a.shape[0]
    with pytest.raises(RuntimeError, match="femIfoMat count exceeds"):
        _run(spec, "femIfoMat", m)


def test_adjacency_mismatch_rejected(spec):
    def m(a):
        E = spec["elmObj"]["elmVtxMat"].shape[1]
        a[1, 100] = (a[1, 100] + E // 2) % E                   # an element of another layer
    with pytest.raises(RuntimeError, match="vtxElmMat entry does not match"):
        _run(spec, "vtxElmMat", m)


@pytest.mark.parametrize("vfd", [("M", 0.0, "B", 1.0), ("G", float("nan"), "B", 1.0), ("G", 0.1, "O", 0.0),
                                 ("G", 0.1, "U", -1.0)])
def test_bad_kernel_width_rejected(spec, vfd):
    """A varifold width that divides must be finite and > 0 (the forward objective and sa_varifold)."""
    from shape_atrophy_gb300 import api
    sp = dict(spec, vfd=vfd)
    with pytest.raises(RuntimeError, match="must be finite and > 0"):
        api.forward(sp, trajectory=False, objective=True)
    with pytest.raises(RuntimeError, match="must be finite and > 0"):
        api.varifold(sp, sp["lmkIniMat"])


def test_unused_direction_width_accepted(spec):
    """The Binet kernel does not use dirKnlWidth (2D_frame/varifold.cu:91-120): any value passes."""
    from shape_atrophy_gb300 import api
    sp = dict(spec, vfd=("M", 0.08, "B", 0.0))
    assert np.isfinite(api.varifold(sp, sp["lmkIniMat"]))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("where", ["node", "bump"])
def test_nonfinite_input_ends_the_solve_with_dbl_max(spec, where, precision):
    """A NaN in the initial nodes or in the bump parameters reaches the first velocity solve's right-hand
    side: the solve stops with SA_ERR_NONFINITE and the column's objective is DBL_MAX, as for a failed CG
    (2D_frame/deform.cu:68-73); the call itself returns normally."""
    from shape_atrophy_gb300 import _lib, api
    sp = dict(spec)
    if where == "node":
        x = np.array(sp["lmkIniMat"], copy=True)
        x[0, 7] = float("nan")
        sp["lmkIniMat"] = x
    else:
        tv = np.array(sp["tauVarVec"], dtype=float, copy=True)
        tv[-1] = float("nan")                                  # the bump's width
        sp["tauVarVec"] = tv
    got = api.forward(sp, trajectory=False, objective=True, precision=precision)
    assert got["info"]["status"] == _lib.SA_ERR_NONFINITE
    assert got["obj"][0] == np.finfo(np.float64).max
