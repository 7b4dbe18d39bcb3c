"""Autotuner table: storage and nearest-size lookup (host logic, no GPU)."""
import json

from astronbodysim import autotune


def test_save_and_lookup_nearest_size(tmp_path):
    p = str(tmp_path / "t.json")
    table = {"law": "spline", "entries": [
        {"n": 4096, "best": "worklist", "ms": {}},
        {"n": 65536, "best": "128x1x2", "ms": {}},
        {"n": 262144, "best": "128x2x4x512x3", "ms": {}},
        {"n": 1048576, "best": "256x2x1", "ms": {}}]}
    autotune.save(table, p)
    assert autotune.lookup(3000, law="spline", path=p) == (-1, 0, 0, 0, 0)
    # three-field keys (block x targets x j-split) mean tiles of 256, 4 stages
    assert autotune.lookup(50000, law="spline", path=p) == (128, 1, 2, 256, 4)
    assert autotune.lookup(300000, law="spline", path=p) == (128, 2, 4, 512, 3)
    assert autotune.lookup(2 ** 21, law="spline", path=p) == (256, 2, 1, 256, 4)
    assert autotune.lookup(1000, law="plummer", path=p) is None


def test_batch_entry_does_not_disturb_single_system_entries(tmp_path):
    p = str(tmp_path / "t.json")
    autotune.save({"law": "spline", "entries": [{"n": 1024, "best": "128x2x1", "ms": {}}]}, p)
    autotune.save_batch({"law": "spline", "best": "256x1", "g_interactions_per_s": {}}, p)
    assert autotune.lookup_batch(law="spline", path=p) == (256, 1)
    assert autotune.lookup_batch(law="plummer", path=p) is None
    assert autotune.lookup(1024, law="spline", path=p) == (128, 2, 1, 256, 4)
    with open(p) as f:
        t = json.load(f)
    assert set(t) == {"spline", "batch"}


def test_missing_table(tmp_path):
    p = str(tmp_path / "none.json")
    assert autotune.lookup(1024, path=p) is None
    assert autotune.lookup_batch(path=p) is None


def test_shipped_table_parses():
    t = autotune.load()
    if t is None:
        return
    for law, entries in t.items():
        if law == "batch":
            for e in entries.values():
                b, i = e["best"].split("x")
                assert int(b) in (128, 256) and int(i) in (1, 2)
            continue
        for e in entries:
            if e["best"] == "worklist":
                continue
            v = [int(x) for x in e["best"].split("x")]
            assert len(v) in (3, 5)
            assert v[0] in (128, 256) and v[1] in (1, 2, 4) and 1 <= v[2] <= 8
            if len(v) == 5:
                assert v[3] in (128, 256, 512) and v[4] in (3, 4, 6)
