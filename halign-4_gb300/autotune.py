"""Autotuner for the launch shape of the batched stages and the DP tier
boundaries.

The stages run persistent grids (CTAs pulling queries or segments from atomic
queues), so the grid size per SM trades occupancy against tail and queue
contention, and the best point depends on the workload (query length, number
of segments per query).  The two tier knobs move gap-fill segments between
the thin, square and wavefront DP tiers (all bit-identical), trading one
tier's latency tail against another's occupancy, and an on/off knob picks
the small tier's int32 or packed int16x2 form.  The band width is not a
knob: bit-exactness fixes it to the reference's auto_band.  `tune` runs a coordinate descent over the
CTAs-per-SM knobs of a context (`Context.set_launch`), scoring each candidate
with `measure` (by default the CUDA-event time of a staged run of the batch
already resident in the context) and keeping a change only when it is faster
by more than `min_gain`.  `TuneCache` stores the result per
(device, workload signature) in a JSON file.
"""
from __future__ import annotations

import json
from pathlib import Path
from typing import Callable, Sequence

from . import LAUNCH_BOUNDS, LAUNCH_KNOBS


def candidates(value: int, lo: int, hi: int) -> list[int]:
    """Neighbours of a knob value: halved, 3/4, 3/2 and doubled, within bounds
    (both values of an on/off knob)."""
    if (lo, hi) == (0, 1):
        return [0, 1]
    out = {value}
    for v in (value // 2, (value * 3) // 4, (value * 3 + 1) // 2, value * 2):
        if lo <= v <= hi:
            out.add(v)
    return sorted(out)


def tune(measure: Callable[[Sequence[int]], float], start: Sequence[int],
         bounds: Sequence[tuple[int, int]] = LAUNCH_BOUNDS, rounds: int = 2, min_gain: float = 0.01):
    """Coordinate descent: returns (best knobs, best time, list of (knobs, time) tried)."""
    best = [int(x) for x in start]
    bounds = list(bounds)[: len(best)]  # a shorter start tunes the leading knobs only
    best_t = measure(best)
    tried = [(list(best), best_t)]
    for _ in range(rounds):
        improved = False
        for i, (lo, hi) in enumerate(bounds):
            for v in candidates(best[i], lo, hi):
                if v == best[i]:
                    continue
                cand = list(best)
                cand[i] = v
                t = measure(cand)
                tried.append((cand, t))
                if t < best_t * (1.0 - min_gain):
                    best, best_t, improved = cand, t, True
        if not improved:
            break
    return best, best_t, tried


def staged_measure(ctx, reps: int = 2) -> Callable[[Sequence[int]], float]:
    """Score = minimum CUDA-event time (ms) over `reps` staged runs after one
    warm-up run (which also captures the graph of the new launch shape)."""
    def measure(knobs: Sequence[int]) -> float:
        ctx.set_launch(knobs)
        ctx.run_staged()
        ctx.last_timing()
        t = float("inf")
        for _ in range(reps):
            ctx.run_staged()
            t = min(t, ctx.last_timing()[0])
        return t
    return measure


class TuneCache:
    """Tuned knobs per (device name, workload signature), kept in a JSON file."""

    def __init__(self, path: str | Path):
        self.path = Path(path)
        self.data = json.loads(self.path.read_text()) if self.path.exists() else {}

    @staticmethod
    def key(device: str, center_len: int, mean_query_len: float, n_queries: int) -> str:
        return f"{device}|L={center_len}|q~{int(round(mean_query_len, -2))}|n~{1 << max(0, int(n_queries).bit_length() - 1)}"

    def get(self, key: str):
        v = self.data.get(key)
        return list(v) if v is not None else None

    def put(self, key: str, knobs: Sequence[int]) -> None:
        self.data[key] = [int(x) for x in knobs]
        self.path.write_text(json.dumps(self.data, indent=1, sort_keys=True))


__all__ = ["LAUNCH_KNOBS", "candidates", "tune", "staged_measure", "TuneCache"]
