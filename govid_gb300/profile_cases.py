"""Small, fixed decode cases to run under a profiler (ncu) on one GPU.

    python -m govid_gb300.profile_cases passes  [--frames 60] [--passes 2]
        pipelined passes (32-frame lookahead, depth 3) over the first frames
        of the 1080p benchmark clip: the launch list and DRAM traffic of the
        single-stream decode;
    python -m govid_gb300.profile_cases frames  [--frames 3]
        one frame per synchronous round: each stage's kernels of a key frame
        (frame 0) and an inter frame (frame 1), launched in that order;
    python -m govid_gb300.profile_cases batched [--frames 8]
        one 64-stream round of the benchmark's mix (each stream's first
        frames, lookahead 1): the batched stages;
    python -m govid_gb300.profile_cases helpers
        the alt-ref filter over 16 1080p frames, then forwardDCT + satd of
        262144 8x8 blocks.

Every case checks its statuses; the decode cases use the content cache
(govid_gb300/workloads.py).
"""
from __future__ import annotations

import argparse
import sys

import numpy as np

from . import ebiv, workloads


def _clip(frames: int) -> list[bytes]:
    data = workloads.load([workloads.single_1080()], in_child=False)[0]
    return [p.data for p in ebiv.Reader(data).packets()][:frames]


def _rounds(b: ebiv.Batch) -> int:
    n, empty = 0, 0
    while empty < b.depth + 1:
        res = b.round()
        empty = empty + 1 if not res else 0
        if any(r.status for r in res):
            raise RuntimeError("decode failed")
        n += len(res)
    return n + len(b.drain())


def passes(frames: int, reps: int) -> None:
    b = ebiv.Batch(lookahead=32, pipeline=3)
    sid = b.add_stream(_clip(frames), ring=3)
    for _ in range(reps):
        b.seek(sid, 0)
        print("frames", _rounds(b))


def single_frames(frames: int) -> None:
    b = ebiv.Batch(lookahead=1)
    sid = b.add_stream(_clip(frames), ring=3)
    for _ in range(frames):
        res = b.round([sid])
        if not res or res[0].status:
            raise RuntimeError("decode failed")
    print("frames", frames)


def batched(frames: int) -> None:
    conts = workloads.load(workloads.mix(), in_child=False)
    b = ebiv.Batch(lookahead=1)
    for c in conts:
        b.add_stream([p.data for p in ebiv.Reader(c).packets()][:frames], ring=3)
    print("frames", _rounds(b))


def helpers() -> None:
    sc = ebiv.Scene(ebiv.SceneSpec(width=1920, height=1080, seed=9, sprites=24, noise_y16=16, noise_c16=8))
    frames = [sc.render(i) for i in range(16)]
    a = ebiv.AltRef()
    a.build(frames, 1920, 1080, 16)
    blocks = np.random.default_rng(1).integers(-255, 256, size=(1 << 18, 8, 8), dtype=np.int64).astype(np.int32)
    ebiv.BlockAnalysis().fdct_satd(blocks)
    print("altref accepted", a.accepted)


def main(argv: list[str]) -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("case", choices=["passes", "frames", "batched", "helpers"])
    ap.add_argument("--frames", type=int, default=0)
    ap.add_argument("--passes", type=int, default=2)
    a = ap.parse_args(argv)
    if a.case == "passes":
        passes(a.frames or 60, a.passes)
    elif a.case == "frames":
        single_frames(a.frames or 3)
    elif a.case == "batched":
        batched(a.frames or 8)
    else:
        helpers()


if __name__ == "__main__":
    main(sys.argv[1:])
