"""The tuner's result cache (no GPU): results keyed by a device persist to the
JSON file and come back in a fresh load; results without a device key stay in
the process."""

import json

from py4dstem_gb300 import autotune


def test_results_persist_per_device(tmp_path, monkeypatch):
    path = tmp_path / "tune.json"
    monkeypatch.setenv("PY4DSTEM_GB300_TUNE_CACHE", str(path))
    autotune.clear_cache(disk=True)
    key = ("multiscan", (100, 200), ((64, 64), (128, 128)))
    timings = [({"concurrent": True, "schedule": 1}, 2.5),
               ({"concurrent": False, "schedule": 1}, 3.0)]
    autotune.remember(key, timings[0][0], timings, device="GPU|sm152|abi2")
    autotune.remember(("local",), {"batch": 256}, [({"batch": 256}, 1.0)])
    data = json.loads(path.read_text())
    assert len(data) == 1  # the entry without a device key is not written
    autotune.clear_cache()  # memory only: the next lookup reads the file
    best, tm = autotune.lookup(key, "GPU|sm152|abi2")
    assert best == {"concurrent": True, "schedule": 1}
    assert tm == timings
    assert autotune.lookup(key, "GPU|sm148|abi2") is None  # another device tunes anew
    assert autotune.lookup(("local",)) is None
    autotune.clear_cache(disk=True)
    assert not path.exists()


def test_disabled_cache_keeps_results_in_memory(tmp_path, monkeypatch):
    monkeypatch.setenv("PY4DSTEM_GB300_TUNE_CACHE", "")
    autotune.clear_cache()
    autotune.remember(("k",), {"batch": 128}, [({"batch": 128}, 1.0)], device="D")
    assert autotune.lookup(("k",), "D")[0] == {"batch": 128}
    assert not list(tmp_path.iterdir())
    autotune.clear_cache()
