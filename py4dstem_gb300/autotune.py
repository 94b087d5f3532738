"""The launch-configuration tuner: time candidate configurations with CUDA
events and remember the fastest.

Each candidate is a dict of settings; `run(candidate)` issues the work to time
on the current stream. The tuner runs every candidate `warmup` times untimed and
`reps` times timed (events on the current stream, synchronised) and returns the
fastest candidate with all timings.

Results are kept in memory for the life of the process and on disk, so that a
configuration is tuned once per GPU model: a JSON file (the path in the
environment variable PY4DSTEM_GB300_TUNE_CACHE, else
~/.cache/py4dstem_gb300/autotune.json) maps a key to the chosen candidate and
its timings. The key joins the caller's description of the work (scan sizes,
slices, probe modes, batch sizes...) with the device name, its SM count and
this library's ABI version, so a different GPU, library or workload tunes
anew. Set PY4DSTEM_GB300_TUNE_CACHE to an empty string to keep results in
memory only.
"""

from __future__ import annotations

import json
import os
import tempfile
import threading
from typing import Callable, Dict, Hashable, List, Optional, Sequence, Tuple

_CACHE: Dict[str, Tuple[dict, List[Tuple[dict, float]]]] = {}
_LOCK = threading.Lock()
_LOADED = False


def cache_path() -> Optional[str]:
    """The on-disk cache file, or None when disabled."""
    path = os.environ.get("PY4DSTEM_GB300_TUNE_CACHE")
    if path is None:
        path = os.path.join(os.path.expanduser("~"), ".cache", "py4dstem_gb300",
                            "autotune.json")
    return path or None


def device_key() -> str:
    """Device name, SM count and library ABI version of the current device."""
    import torch

    from . import _native

    props = torch.cuda.get_device_properties(torch.cuda.current_device())
    return f"{props.name}|sm{props.multi_processor_count}|abi{_native.lib().ptycho_abi_version()}"


def _key_string(key: Hashable, device: Optional[str]) -> str:
    return json.dumps([device, repr(key)])


def _load() -> None:
    global _LOADED
    if _LOADED:
        return
    _LOADED = True
    path = cache_path()
    if not path or not os.path.exists(path):
        return
    try:
        with open(path) as f:
            data = json.load(f)
    except (OSError, ValueError):
        return  # an unreadable cache is ignored and rewritten
    for k, v in data.items():
        try:
            _CACHE.setdefault(k, (dict(v["best"]), [(dict(c), float(t)) for c, t in v["timings"]]))
        except (KeyError, TypeError, ValueError):
            continue


def _save() -> None:
    path = cache_path()
    if not path:
        return
    # entries tuned without a device key belong to this process only
    data = {k: {"best": b, "timings": [[c, t] for c, t in tm]} for k, (b, tm) in _CACHE.items()
            if json.loads(k)[0] is not None}
    try:
        os.makedirs(os.path.dirname(path), exist_ok=True)
        fd, tmp = tempfile.mkstemp(dir=os.path.dirname(path), suffix=".tmp")
        with os.fdopen(fd, "w") as f:
            json.dump(data, f, indent=1, sort_keys=True)
        os.replace(tmp, path)
    except OSError:
        pass  # a read-only home: results stay in memory


def time_candidates(candidates: Sequence[dict], run: Callable[[dict], None], *, warmup: int = 1,
                    reps: int = 3) -> List[Tuple[dict, float]]:
    """[(candidate, median ms)] in the given order."""
    import torch

    out = []
    for cand in candidates:
        for _ in range(warmup):
            run(cand)
        times = []
        for _ in range(reps):
            start = torch.cuda.Event(enable_timing=True)
            stop = torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            start.record()
            run(cand)
            stop.record()
            stop.synchronize()
            times.append(start.elapsed_time(stop))
        times.sort()
        out.append((dict(cand), times[len(times) // 2]))
    return out


def lookup(key: Hashable, device: Optional[str] = None):
    """The cached (best, timings) for `key` on `device`, or None."""
    with _LOCK:
        _load()
        return _CACHE.get(_key_string(key, device))


def tune(key: Hashable, candidates: Sequence[dict], run: Callable[[dict], None], *,
         warmup: int = 1, reps: int = 3,
         device: Optional[str] = None) -> Tuple[dict, List[Tuple[dict, float]]]:
    """Fastest candidate for `key` (from the cache when present) and the timings
    it was chosen from. `device` (device_key()) makes the entry persistent; a
    key without it is kept for this process only."""
    ks = _key_string(key, device)
    with _LOCK:
        _load()
        if ks in _CACHE:
            return _CACHE[ks]
    timings = time_candidates(candidates, run, warmup=warmup, reps=reps)
    best = min(timings, key=lambda t: t[1])[0]
    with _LOCK:
        _CACHE[ks] = (best, timings)
        if device is not None:
            _save()
    return best, timings


def remember(key: Hashable, best: dict, timings: List[Tuple[dict, float]],
             device: Optional[str] = None) -> None:
    """Store a result timed by the caller (same semantics as tune())."""
    with _LOCK:
        _load()
        _CACHE[_key_string(key, device)] = (dict(best), [(dict(c), float(t)) for c, t in timings])
        if device is not None:
            _save()


def clear_cache(disk: bool = False) -> None:
    """Forget the in-memory results; with disk=True remove the file too."""
    global _LOADED
    with _LOCK:
        _CACHE.clear()
        # memory only: the file is read again on the next use
        _LOADED = disk
        path = cache_path()
        if disk and path and os.path.exists(path):
            os.remove(path)
