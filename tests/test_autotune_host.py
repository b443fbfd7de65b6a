"""Schedule-cache logic of the autotuner on the host: keys, atomic stores, tolerance of a
missing or foreign cache file, and the choice rule (fastest within 1 %, lowest mask)."""
import importlib
import json

import pytest


@pytest.fixture(scope="module")
def at():
    return importlib.import_module("3d_ravesim_gb300.autotune")


def test_cache_round_trip(at, tmp_path, monkeypatch):
    path = tmp_path / "sub" / "schedules.json"
    monkeypatch.setenv("RS_SCHEDULE_CACHE", str(path))
    assert at.cache_path() == path
    assert at.load_cache() == {}
    key = at.entry_key("GB300|sm103|152sm", 4096, 4096, "multislice")
    assert key == "GB300|sm103|152sm|4096x4096|multislice"
    at.store_entry(key, {"mask": 2, "timings_ms": {"0": 1.0, "2": 0.9}})
    at.store_entry(at.entry_key("GB300|sm103|152sm", 1024, 1024, "multislice"), {"mask": 0})
    data = json.loads(path.read_text())
    assert data["version"] == at.CACHE_VERSION and data["entries"][key]["mask"] == 2
    assert len(at.load_cache()) == 2
    assert not [p for p in path.parent.iterdir() if p.name != "schedules.json"]  # no temp files left


def test_cache_ignores_corrupt_or_foreign_files(at, tmp_path):
    p = tmp_path / "c.json"
    p.write_text("{not json")
    assert at.load_cache(p) == {}
    p.write_text(json.dumps({"version": 999, "entries": {"k": {"mask": 1}}}))
    assert at.load_cache(p) == {}
    p.write_text(json.dumps([1, 2]))
    assert at.load_cache(p) == {}


def test_pick_fastest(at):
    assert at.pick_fastest({0: 1.0, 2: 0.8, 3: 0.9}) == 2
    assert at.pick_fastest({0: 0.805, 2: 0.8, 6: 0.95}) == 0  # within 1 %: the lower mask
    assert at.pick_fastest({4: 1.0}) == 4


def test_choice_json(at):
    c = at.Choice(2, {2: 0.51234567, 0: 0.6}, 4, {0: 0.0, 2: 0.0})
    assert c.as_json() == {"mask": 2, "slices": 4, "timings_ms": {"0": 0.6, "2": 0.5123},
                           "rel_diff": {"0": 0.0, "2": 0.0}}
