"""Learned MV proposer against the exhaustive search: encode time and EBIV
bytes at matched PSNR, and the GPU decode of every bitstream checked frame
by frame against the encoder's own reconstruction (tests/test_gpu_mvnet.py
checks the same bitstream kind against the CPU oracle).

The clip is a seeded sprite scene (fractional velocities in [-8, 8]
px/frame, global pan up to 3 px/frame, 24 sprites).  The exhaustive search
encodes at q; the proposer encodes at q-1, q and q+1.  PSNR per frame is
taken over all three planes (framePSNR, ebiv/coded_test.go:42-59) and
averaged over the clip; the proposer's size at the exhaustive encode's PSNR
is interpolated with ln(size) linear in PSNR between the bracketing points
(interpolateSize, examples/ebiv/corpus_test.go:326-347).

    python -m govid_gb300.eval_mvnet [--frames 120] [--width 1920 --height 1080]
"""
from __future__ import annotations

import argparse
import json
import math
import os
import time

import numpy as np

from . import ebiv, mvnet


def frame_psnr(dec: bytes, src: bytes) -> float:
    a = np.frombuffer(dec, np.uint8).astype(np.int64)
    b = np.frombuffer(src, np.uint8).astype(np.int64)
    mse = float(((a - b) ** 2).sum()) / a.size
    return 1e9 if mse == 0 else 10.0 * math.log10(255.0 * 255.0 / mse)


def interpolate_size(points: list[tuple[float, int]], target: float) -> float:
    """points: (psnr, size); ln(size) linear in PSNR between the two points
    bracketing target (the nearest two when none brackets it)."""
    pts = sorted(points)
    if len(pts) == 1:
        return float(pts[0][1])
    i = next((k for k, p in enumerate(pts) if p[0] >= target), len(pts))
    i = min(max(i, 1), len(pts) - 1)
    (pa, sa), (pb, sb) = pts[i - 1], pts[i]
    if pb == pa:
        return float(sa)
    f = (target - pa) / (pb - pa)
    return math.exp(math.log(sa) + f * (math.log(sb) - math.log(sa)))


def encode(frames: list[bytes], w: int, h: int, qp: int, search: str, threads: int, net=None, gop: int = 60,
           fallback_sad: int = 0) -> dict:
    enc = ebiv.Encoder(ebiv.Config(w, h), intra=qp, gop=gop, tiles=(4, 3), search=search, threads=threads,
                       fallback_sad=fallback_sad, keep_recon=True)
    if net is not None:
        net.attach(enc)
    t0 = time.perf_counter()
    for f in frames:
        enc.write_frame(f)
    enc.close()
    wall = time.perf_counter() - t0
    data = enc.output()
    recons = enc.recons()
    return {"recons": recons, "search": search, "qp": qp, "bytes": len(data), "encode_s": wall, "search_thread_s": enc.search_seconds(),
            "propose_s": enc.propose_seconds(), "sad_evaluations": enc.sad_evaluations(),
            "fallbacks": enc.search_fallbacks(), "data": data}


def decode_check(data: bytes, frames: list[bytes], recons: list[bytes]) -> tuple[float, bool]:
    """Mean PSNR of the GPU decode, and whether every decoded frame equals
    the encoder's reconstruction of it."""
    pk = [p.data for p in ebiv.Reader(data).packets()]
    c = ebiv.Codec()
    same = len(pk) == len(recons)
    ps = []
    for i, p in enumerate(pk):
        got = c.decode(p).packed()
        same = same and got == recons[i]
        ps.append(frame_psnr(got, frames[i]))
    c.close()
    return float(np.mean(ps)), same


def compare(w: int = 1920, h: int = 1080, nframes: int = 120, qp: int = 22, seed: int = 77, threads: int = 0,
            weights=mvnet.WEIGHTS, fallback_sad: int = 0, log=print) -> dict:
    threads = threads or os.cpu_count() or 8
    sc = ebiv.Scene(mvnet.clip_spec(seed, w, h))
    frames = [sc.render(i) for i in range(nframes)]
    pad_w, pad_h = (w + 15) // 16 * 16, (h + 15) // 16 * 16
    net = mvnet.MvNet(pad_w, pad_h).load(weights)
    runs = []
    ex = encode(frames, w, h, qp, "exhaustive", threads)
    runs.append(ex)
    for q in (qp - 1, qp, qp + 1):
        runs.append(encode(frames, w, h, q, "proposed", threads, net=net, fallback_sad=fallback_sad))
    for r in runs:
        r["psnr"], r["bit_exact"] = decode_check(r.pop("data"), frames, r.pop("recons"))
        if log:
            log(f"[mvnet-eval] {r['search']} q{r['qp']}: {r['bytes']} B, {r['psnr']:.3f} dB, "
                f"encode {r['encode_s']:.2f} s, search {r['search_thread_s']:.2f} thread-s, "
                f"bit-exact {r['bit_exact']}")
    prop = [r for r in runs if r["search"] == "proposed"]
    pq = next(r for r in prop if r["qp"] == qp)
    size_at = interpolate_size([(r["psnr"], r["bytes"]) for r in prop], ex["psnr"])
    return {
        "workload": f"{w}x{h} {nframes} frames, seeded sprites (24, fractional velocity <= 8 px/frame, "
                    f"pan <= 3 px/frame), gop 60, tiles 4x3, q{qp}",
        "encoder_threads": threads,
        "exhaustive": {k: ex[k] for k in ("bytes", "psnr", "encode_s", "search_thread_s", "sad_evaluations")},
        "proposed": {k: pq[k] for k in ("bytes", "psnr", "encode_s", "search_thread_s", "propose_s",
                                         "sad_evaluations", "fallbacks")},
        "encode_speedup": ex["encode_s"] / pq["encode_s"],
        "search_speedup": ex["search_thread_s"] / (pq["search_thread_s"] + pq["propose_s"] * threads),
        "bits_at_matched_psnr": size_at / ex["bytes"] - 1.0,
        "matched_psnr_db": ex["psnr"],
        "gpu_decode_equals_encoder_recon": all(r["bit_exact"] for r in runs),
        "rate_points": [{k: r[k] for k in ("search", "qp", "bytes", "psnr")} for r in runs],
    }


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--width", type=int, default=1920)
    ap.add_argument("--height", type=int, default=1080)
    ap.add_argument("--frames", type=int, default=120)
    ap.add_argument("--qp", type=int, default=22)
    ap.add_argument("--threads", type=int, default=0)
    ap.add_argument("--fallback-sad", type=int, default=0)
    a = ap.parse_args()
    r = compare(a.width, a.height, a.frames, a.qp, threads=a.threads, fallback_sad=a.fallback_sad)
    print(json.dumps(r))


if __name__ == "__main__":
    main()
