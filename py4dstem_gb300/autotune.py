"""A small autotuner: time candidate launch configurations with CUDA events.

Each candidate is a dict of settings; `run(candidate)` issues the work to time
on the current stream. The tuner runs every candidate `warmup` times untimed and
`reps` times timed (events on the current stream, synchronised), and returns the
fastest candidate with all timings. Results are cached per key for the life of
the process so that a configuration is tuned once.
"""

from __future__ import annotations

from typing import Callable, Dict, Hashable, List, Sequence, Tuple

_CACHE: Dict[Hashable, Tuple[dict, List[Tuple[dict, float]]]] = {}


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


def tune(key: Hashable, candidates: Sequence[dict], run: Callable[[dict], None], *,
         warmup: int = 1, reps: int = 3) -> Tuple[dict, List[Tuple[dict, float]]]:
    """Fastest candidate for `key` (cached) and the timings it was chosen from."""
    if key in _CACHE:
        return _CACHE[key]
    timings = time_candidates(candidates, run, warmup=warmup, reps=reps)
    best = min(timings, key=lambda t: t[1])[0]
    _CACHE[key] = (best, timings)
    return best, timings


def clear_cache() -> None:
    _CACHE.clear()
