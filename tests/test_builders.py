"""The C library's element-object builders (host code) against the Python
restatement of generateElementObject2D/3D and tri2tetra: every array bit
for bit, on the demo strip, a periodic annulus and icosphere shells.  No
GPU involved."""
import numpy as np
import pytest

KEYS_2D = ["elmVtxMat", "vtxElmMat", "tanVtxMat", "tsvVtxMat", "bdrVtxMat", "vtxBdrMat", "btmVtxMat", "vtxBtmMat",
           "femVtxMat", "femIfoMat", "vfdVtxMat"]
KEYS_3D = ["elmVtxMat", "vtxElmMat", "nmlVtxMat", "tsvVtxMat", "bdrVtxMat", "vtxBdrMat", "btmVtxMat", "vtxBtmMat",
           "femVtxMat", "femIfoMat", "vfdVtxMat"]


@pytest.fixture(scope="module")
def api():
    from shape_atrophy_gb300 import api as a, build
    build.build()
    return a


def _same(a, b, keys):
    for k in keys:
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)
    for k in ("lyrLmkNum", "lyrCntNum", "elmPerLayer"):
        assert a[k] == b[k], k


@pytest.mark.parametrize("L,C,vfd,periodic", [(21, 7, [1, 7], False), (101, 31, [1, 31], False),
                                              (48, 7, [1, 7], True), (256, 16, [1, 16], True)])
def test_2d_builder_bit_exact(api, L, C, vfd, periodic):
    from shape_atrophy_gb300 import mesh
    want = mesh.generate_element_object_2d(L, C, vfd, periodic=periodic)
    got = api.build_element_object_2d(L, C, vfd, periodic=periodic)
    _same(got, want, KEYS_2D)
    np.testing.assert_array_equal(got["vfdIfoMat"], mesh.vfd_gradient_table(want["vfdVtxMat"], L * C))


@pytest.mark.parametrize("level,layers", [(1, 3), (2, 5), (3, 9)])
def test_3d_builder_bit_exact(api, level, layers):
    from shape_atrophy_gb300 import mesh
    surf, tri = mesh.icosphere(level)
    tet, nml, tsv = mesh.tri2tetra(tri, layers)
    t2, n2, s2 = api.tri2tetra(tri, layers)
    np.testing.assert_array_equal(t2, tet)
    np.testing.assert_array_equal(n2, nml)
    np.testing.assert_array_equal(s2, tsv)
    want = mesh.generate_element_object_3d(tet, tri, nml, tsv, [layers])
    got = api.build_element_object_3d(tet, tri, nml, tsv, [layers])
    _same(got, want, KEYS_3D)
    np.testing.assert_array_equal(got["vfdIfoMat"], mesh.vfd_gradient_table(want["vfdVtxMat"], tet.max() + 1))


def test_builder_rejects_bad_input(api):
    from shape_atrophy_gb300 import mesh
    surf, tri = mesh.icosphere(1)
    bad = tri.copy()
    bad[:, 0] = bad[0, 0]                              # one vertex three times: no label case applies
    with pytest.raises(ValueError):
        mesh.tri2tetra(bad, 3)
    with pytest.raises(ValueError):
        api.tri2tetra(bad, 3)
    with pytest.raises(ValueError):
        api.build_element_object_2d(10, 4, [7])        # layer 7 of 4
