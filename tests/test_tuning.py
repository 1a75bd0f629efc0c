"""Launch-shape tuning on the host: sa_set_tuning / sa_get_tuning round
trip, out-of-range values and unknown names are refused, and the committed
tuning table (written by shape_atrophy_gb300/autotune.py) holds only known
names with values the library accepts.  No compute call runs here."""
import json
import os

import pytest

from shape_atrophy_gb300 import api

DEFAULTS = {"persistMaxWarps": 20, "batchBlock": 256, "batchSlicesPerWarp": 2, "vfdCtasPerSm": 8,
            "mixedInnerFloor": 10, "kernelMatrixFree": 0}


@pytest.fixture
def restore():
    from shape_atrophy_gb300 import build
    build.build()
    before = api.get_tuning()
    yield
    api.set_tuning(**before)


def test_compiled_defaults(restore):
    assert api.get_tuning() == DEFAULTS


def test_set_get_round_trip(restore):
    api.set_tuning(persistMaxWarps=8, batchBlock=128, batchSlicesPerWarp=4, vfdCtasPerSm=2, mixedInnerFloor=12,
                   kernelMatrixFree=1)
    assert api.get_tuning() == {"persistMaxWarps": 8, "batchBlock": 128, "batchSlicesPerWarp": 4,
                                "vfdCtasPerSm": 2, "mixedInnerFloor": 12, "kernelMatrixFree": 1}


@pytest.mark.parametrize("name,value", [("persistMaxWarps", 0), ("persistMaxWarps", 21), ("batchBlock", 192),
                                        ("batchBlock", 512), ("batchSlicesPerWarp", 0), ("vfdCtasPerSm", 33),
                                        ("mixedInnerFloor", 3), ("mixedInnerFloor", 17),
                                        ("kernelMatrixFree", 2),
                                        ("noSuchShape", 1)])
def test_bad_values_refused(restore, name, value):
    before = api.get_tuning()
    with pytest.raises(ValueError):
        api.set_tuning(**{name: value})
    assert api.get_tuning() == before


def test_committed_table_is_valid(restore, tmp_path):
    if not os.path.exists(api.TUNING_FILE):
        pytest.skip("no tuning table committed")
    table = json.load(open(api.TUNING_FILE))
    assert table["devices"]
    for e in table["devices"]:
        assert isinstance(e["name"], str) and int(e["smCount"]) > 0
        assert set(e["values"]) <= set(api.TUNING_NAMES)
        api.set_tuning(**e["values"])          # every value in range


def test_write_entry_replaces_same_device(restore, tmp_path):
    from shape_atrophy_gb300 import autotune
    p = str(tmp_path / "t.json")
    a = {"name": "X", "smCount": 10, "values": {"batchBlock": 128}}
    b = {"name": "X", "smCount": 10, "values": {"batchBlock": 256}}
    c = {"name": "Y", "smCount": 10, "values": {"batchBlock": 128}}
    for e in (a, c, b):
        autotune.write_entry(e, p)
    t = json.load(open(p))
    assert sorted((e["name"], e["values"]["batchBlock"]) for e in t["devices"]) == [("X", 256), ("Y", 128)]
