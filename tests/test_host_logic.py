"""Host-side logic without a GPU: mesh builders and the invariants the
library relies on (CSR order, symmetric pattern, symmetric element lists),
the seeded served-request stream, and the replica reduction of bench.py
over two gloo ranks."""
import os
import socket

import numpy as np
import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))


def _check_element_object(obj, N):
    fv = obj["femVtxMat"]
    r, c = fv[0].astype(np.int64), fv[1].astype(np.int64)
    key = r * N + c
    assert np.all(np.diff(key) > 0)                      # sorted by (row, col), no duplicates
    assert set(np.unique(r)) == set(range(N))            # every node has a row
    pos = {k: z for z, k in enumerate(key.tolist())}
    fi = obj["femIfoMat"]
    for z in range(0, fv.shape[1], max(1, fv.shape[1] // 500)):
        zt = pos[int(c[z]) * N + int(r[z])]                # the transposed slot exists ...
        assert fi[0, z] == fi[0, zt]                       # ... with the same number of elements
        assert set(fi[2::2, z][:fi[0, z]]) == set(fi[2::2, zt][:fi[0, zt]])


@pytest.mark.parametrize("kind", ["annulus", "shell"])
def test_layered_meshes_satisfy_library_invariants(kind):
    from shape_atrophy_gb300 import problems
    sp = (problems.annulus_layered(angNum=32, radNum=6, steps=2) if kind == "annulus"
          else problems.shell_layered(level=2, lyrCntNum=4, steps=2))
    N = sp["lmkIniMat"].shape[1]
    _check_element_object(sp["elmObj"], N)
    lyr = np.asarray(sp["elmLyrVec"])
    assert lyr.min() >= 0 and lyr.max() < len(sp["spdLyrVec"])


def test_shell_sizes_of_the_workload_family():
    from shape_atrophy_gb300 import problems
    sp = problems.shell_layered(level=3, lyrCntNum=5, steps=1)
    assert sp["lmkIniMat"].shape[1] == 642 * 5
    assert sp["elmObj"]["elmVtxMat"].shape[1] == 1280 * 4 * 3


def test_served_request_stream_is_seeded():
    import bench
    a = bench.served_requests(6, seed=3)
    b = bench.served_requests(6, seed=3)
    assert [g for _, g in a] == [g for _, g in b]
    for (sa, _), (sb, _) in zip(a, b):
        np.testing.assert_array_equal(sa["tauVarVec"], sb["tauVarVec"])
        np.testing.assert_array_equal(sa["modVec"], sb["modVec"])
        assert sa["timeNum"] == sb["timeNum"] and 21 <= sa["timeNum"] <= 61


@pytest.mark.parametrize("layers", [2, 3, 5, 6])
def test_annulus_material_layers(layers):
    from shape_atrophy_gb300 import problems
    sp = problems.annulus_layered(angNum=32, radNum=8, steps=2, layers=layers)
    lyr = np.asarray(sp["elmLyrVec"])
    assert sorted(set(lyr.tolist())) == list(range(layers))          # every material layer has elements
    assert len(sp["spdLyrVec"]) == layers and len(sp["modVec"]) == 2 * layers
    np.testing.assert_array_equal(sp["modVec"][1::2], sp["modVec"][0::2] / 2)   # mu = lambda / 2
    # material layers follow the radial rings outward: element layer ids never decrease with the ring
    per = sp["elmObj"]["elmPerLayer"]
    ring = np.arange(lyr.size) // per
    assert np.all(np.diff([lyr[ring == k].max() for k in range(ring.max() + 1)]) >= 0)


def test_batched_instance_batch_is_seeded_and_in_range():
    import bench
    a, b = bench.batched_requests(24, seed=5, steps=3), bench.batched_requests(24, seed=5, steps=3)
    dims = [sp["dim"] for sp in a]
    assert 2 in dims and 3 in dims
    for sa, sb in zip(a, b):
        np.testing.assert_array_equal(sa["tauVarVec"], sb["tauVarVec"])
        np.testing.assert_array_equal(sa["modVec"], sb["modVec"])
        assert sa["timeNum"] == 4
        N = sa["lmkIniMat"].shape[1]
        L = len(sa["spdLyrVec"])
        assert len(sa["modVec"]) == 2 * L
        assert np.all((sa["modVec"][0::2] >= 0.5) & (sa["modVec"][0::2] <= 10.0))
        assert np.all((sa["spdLyrVec"] >= 0.005) & (sa["spdLyrVec"] <= 0.1))
        if sa["dim"] == 2:
            assert 1500 <= N <= 45000 and 2 <= L <= 6
            assert np.hypot(*sa["tauVarVec"][:2]) == pytest.approx(1.0)     # bump on the outer circle
        else:
            assert N in {642 * k for k in range(5, 10)} | {2562 * k for k in range(5, 10)} and L == 3
            assert np.linalg.norm(sa["tauVarVec"][:3]) == pytest.approx(1.0)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE="2",
                      LOCAL_RANK=str(rank))
    import sys
    sys.path.insert(0, ROOT)
    import bench
    r, local, ws, dist = bench.dist_init()
    t = bench.reduce_max(1.5 + rank, dist, local)        # per-rank times 1.5 and 2.5
    bench.barrier(dist)
    q.put((r, ws, t))
    dist.destroy_process_group()


def test_bench_replicas_take_the_max_time_over_two_gloo_ranks():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(k, port, q)) for k in range(2)]
    for p in ps:
        p.start()
    got = [q.get(timeout=120) for _ in ps]
    for p in ps:
        p.join(timeout=60)
    assert sorted(g[0] for g in got) == [0, 1]
    assert all(g[1] == 2 and g[2] == 2.5 for g in got)
