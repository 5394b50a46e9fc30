"""The shape autotuner's search and cache (host logic, no GPU): coordinate
descent from the default shape over every dimension, each shape timed once,
the winner and all timings cached per device, workload and search space."""
import json

from sdbe_gb300 import autotune as A


def _cost(shape):
    wave = {16: 5.0, 32: 4.0, 48: 3.5, 64: 3.8}[shape["wave"]]
    per = {1: 1.0, 2: 0.5, 4: 0.2}[shape["per_launch"]]
    return wave + per + (0.1 if shape["precision"] == "fp32" else 0.0)


def test_tune_shape_descends_and_caches(tmp_path, monkeypatch):
    monkeypatch.setenv("SDBE_AUTOTUNE_CACHE", str(tmp_path / "cache.json"))
    monkeypatch.setattr(A, "device_key", lambda: "dev0")
    calls = []

    def measure(shape):
        calls.append(dict(shape))
        return _cost(shape)

    space = {"wave": [16, 32, 48, 64], "per_launch": [1, 2, 4], "precision": ["fp32", "tc16fast"]}
    default = {"wave": 64, "per_launch": 4, "precision": "fp32"}
    best, table = A.tune_shape("w8", measure, space, default)
    assert best == {"wave": 48, "per_launch": 4, "precision": "tc16fast"}
    assert len(calls) == len({A._shape_key(c) for c in calls}) == len(table)  # no shape timed twice
    assert table[A._shape_key(default)] == _cost(default)
    # cached: no measuring the second time; another search space is another entry
    best2, table2 = A.tune_shape("w8", lambda s: 1 / 0, space, default)
    assert best2 == best and table2 == table
    d = json.loads((tmp_path / "cache.json").read_text())
    assert len(d) == 1 and next(iter(d)).startswith("dev0|w8|")
    best3, _ = A.tune_shape("w8", measure, {"wave": [16, 64]}, {"wave": 64, "per_launch": 4, "precision": "fp32"})
    assert best3["wave"] == 64 and len(json.loads((tmp_path / "cache.json").read_text())) == 2
