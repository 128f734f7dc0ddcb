"""Autotuner of the batched decode's launch shape.

For a set of streams it tries candidate settings of the batch engine —
frames per stream per round (lookahead), rounds in flight (pipeline depth),
entropy launches per round and intra-stage warps per CTA (the tile-to-CTA
mapping of the reconstruction) — on a prefix of every stream, measures each
with the wall clock of whole rounds, and returns the best under the
objective:

* ``throughput``: most frames per second;
* ``latency``: most frames per second among the settings whose 99th
  percentile round-call time stays within ``round_budget_ms`` (the fastest
  setting when none does).

Results do not depend on the setting (the engine's outputs are identical for
every shape; the parity tests run several), so the tuner only measures time.
"""
from __future__ import annotations

import itertools
import statistics
import time

from . import ebiv

LOOKAHEADS = (1, 2, 4, 8)
DEPTHS = (1, 2, 3)
GROUPS = (1, 2, 4)
INTRA_WARPS = (0, 4, 8, 16)


def _trial(streams: list[list[bytes]], lookahead: int, depth: int, groups: int, warps: int, frames: int) -> dict:
    b = ebiv.Batch(lookahead=lookahead, pipeline=depth)
    b.set_tuning(groups, warps)
    ids = [b.add_stream(pk[:frames], ring=3) for pk in streams]
    lat: list[float] = []
    n, dt = 0, 1.0
    for _ in range(2):  # the first pass sizes the frame pools; the second is timed
        for sid in ids:
            b.seek(sid, 0)
        lat.clear()
        n = 0
        t0 = time.perf_counter()
        empty = 0
        while empty < b.depth + 1:
            c0 = time.perf_counter()
            res = b.round()
            if res:
                lat.append(time.perf_counter() - c0)
            n += len(res)
            empty = empty + 1 if not res else 0
        n += len(b.drain())
        dt = time.perf_counter() - t0
    b.close()
    lat.sort()
    return {"lookahead": lookahead, "pipeline_depth": depth, "entropy_groups": groups, "intra_warps": warps,
            "frames_per_s": n / dt, "round_p99_ms": 1000 * lat[int(0.99 * (len(lat) - 1))] if lat else 0.0,
            "round_p50_ms": 1000 * statistics.median(lat) if lat else 0.0}


def tune(streams: list[list[bytes]], frames: int = 16, objective: str = "throughput", round_budget_ms: float = 16.7,
         lookaheads=LOOKAHEADS, depths=DEPTHS, groups=GROUPS, intra_warps=INTRA_WARPS) -> dict:
    """Searches lookahead x depth (entropy groups 4, intra warps by tile
    count), then entropy groups x intra warps at the best of those; returns
    the chosen setting and every trial."""

    def pick(cands):
        if objective == "latency":
            ok = [t for t in cands if t["round_p99_ms"] <= round_budget_ms]
            if ok:
                return max(ok, key=lambda t: t["frames_per_s"])
        return max(cands, key=lambda t: t["frames_per_s"])

    first = [_trial(streams, la, d, 4, 0, frames) for la, d in itertools.product(lookaheads, depths)]
    best = pick(first)
    second = [_trial(streams, best["lookahead"], best["pipeline_depth"], g, w, frames)
              for g, w in itertools.product(groups, intra_warps) if (g, w) != (4, 0)]
    best = pick(first + second)
    return {"objective": objective, "frames_per_stream_tried": frames, "choice": best, "trials": first + second}
