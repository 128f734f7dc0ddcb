"""Trains the learned motion-vector proposer on the GPU and writes
govid_gb300/mvnet_weights.f32.

Training set: seeded 1280x720 sprite clips (fractional velocities in
[-8, 8] px/frame, global pan up to 3 px/frame, noise sigma 2); every
consecutive frame pair is labelled by the GPU exhaustive full-pel search
(+-16 px).  Adam, batch of frame pairs, learning rate decayed linearly.

    python -m govid_gb300.train_mvnet [--clips 200] [--frames 4] [--steps 3000]
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import mvnet


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--clips", type=int, default=200)
    ap.add_argument("--frames", type=int, default=4, help="frames rendered per clip (frames-1 pairs)")
    ap.add_argument("--width", type=int, default=1280)
    ap.add_argument("--height", type=int, default=720)
    ap.add_argument("--steps", type=int, default=3000)
    ap.add_argument("--batch", type=int, default=8)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--out", default=str(mvnet.WEIGHTS))
    a = ap.parse_args()
    pairs = a.clips * (a.frames - 1)
    net = mvnet.MvNet(a.width, a.height, max_batch=a.batch, max_pairs=pairs, seed=a.seed)
    data = mvnet.build_training_set(net, a.clips, a.frames)
    t0 = time.time()
    hist = mvnet.train(net, a.steps, a.batch, a.lr)
    train_s = time.time() - t0
    net.save(a.out)
    tail = np.mean(hist[-200:], axis=0)
    print(json.dumps({"training_set": data, "steps": a.steps, "batch": a.batch, "train_seconds": round(train_s, 1),
                      "final": {"loss": float(tail[0]), "top1": float(tail[1]), "top8": float(tail[2])},
                      "weights": a.out}))


if __name__ == "__main__":
    main()
