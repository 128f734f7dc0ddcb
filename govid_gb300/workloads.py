"""Seeded synthetic EBIV workloads of the decode benchmarks and the full-size
parity tests, and their content cache.

The reference publishes no dataset for its EBIV decode path, so every clip is
a seeded sprite scene (a luma gradient, textured sprites moving at seeded
velocities, Gaussian noise) encoded by this repository's EBIV encoder:

* ``single_640``: 640x360, 60 frames, 6 sprites, q22, gop 60, 2x2 tiles;
* ``single_1080``: 1920x1080, 300 frames, 24 sprites, a +40 luma flash for 3
  frames every 60 frames, q22, gop 60, 4x3 tiles (the single-stream bench clip);
* ``mix``: 64 streams (24 x 640x360, 24 x 1280x720, 16 x 1920x1080), each with
  its own seed and its own draw of tile grid from {1x1, 2x2, 4x3}, q from
  {18, 22, 28} and gop from 30-120, 120 frames each: 64 distinct bitstreams;
* ``serve``: 600-frame clips with the mix's settings for the serving loop.

Encoding is slow next to decoding (about 2 s of one host core per 1080p
frame), so clips are cached on disk under ``EBIV_CONTENT_DIR`` (default: the
``.content_cache`` folder at the repository root) keyed by their parameters
and by a hash of the encoder sources.  A missing clip is encoded by
``python -m govid_gb300.workloads <names>`` in a child process, so that a
process which must not load the decoder library (the CPU reference arm of the
benchmark) can still obtain its input.  This module itself loads no native
code unless it encodes.
"""
from __future__ import annotations

import hashlib
import os
import random
import subprocess
import sys
import time
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent

# Encoder settings are part of every cache key: a change to the encoder or the
# scene generator invalidates the cached clips.
_SOURCES = ["csrc/encoder.cpp", "csrc/encoder.h", "csrc/synth.cpp", "csrc/synth.h"]

MIX_RES = [((640, 360), 24), ((1280, 720), 24), ((1920, 1080), 16)]
GRIDS = [(1, 1), (2, 2), (4, 3)]
QPS = [18, 22, 28]


def content_dir() -> Path:
    d = Path(os.environ.get("EBIV_CONTENT_DIR", ROOT / ".content_cache"))
    d.mkdir(parents=True, exist_ok=True)
    return d


def _src_hash() -> str:
    h = hashlib.sha1()
    for s in _SOURCES:
        h.update((PKG / s).read_bytes())
    return h.hexdigest()[:12]


def sprites_for(w: int) -> int:
    return 6 if w <= 640 else (12 if w <= 1280 else 24)


class Clip:
    """One seeded clip: scene parameters plus encoder settings."""

    def __init__(self, name, w, h, frames, seed, qp, gop, grid, sprites=None, flash=False):
        self.name, self.w, self.h, self.frames, self.seed = name, w, h, frames, seed
        self.qp, self.gop, self.grid = qp, gop, tuple(grid)
        self.sprites = sprites_for(w) if sprites is None else sprites
        self.flash = flash

    def scene(self):
        from . import ebiv

        kw = dict(flash_period=60, flash_start=30, flash_len=3, flash_amp=40) if self.flash else {}
        return ebiv.SceneSpec(width=self.w, height=self.h, seed=self.seed, sprites=self.sprites, vel_max_q=16,
                              integer_vel=True, noise_y16=32, noise_c16=16, **kw)

    def key(self) -> str:
        k = (f"v2|{self.w}x{self.h}|{self.frames}|s{self.seed}|sp{self.sprites}|f{int(self.flash)}|q{self.qp}|"
             f"g{self.gop}|{self.grid[0]}x{self.grid[1]}|fast|{_src_hash()}")
        return hashlib.sha1(k.encode()).hexdigest()[:20]

    def path(self) -> Path:
        return content_dir() / f"{self.name}-{self.key()}.ebiv"

    def describe(self) -> dict:
        return {"w": self.w, "h": self.h, "frames": self.frames, "seed": self.seed, "qp": self.qp, "gop": self.gop,
                "grid": f"{self.grid[0]}x{self.grid[1]}", "sprites": self.sprites, "flash": self.flash}

    def encode(self, threads: int) -> bytes:
        from . import ebiv

        return ebiv.encode_scene(self.scene(), self.frames, qp=self.qp, gop=self.gop, tiles=self.grid, fast=True,
                                 threads=threads)

    def cost(self) -> float:
        return self.w * self.h * self.frames


def single_640() -> Clip:
    return Clip("single640", 640, 360, 60, 7, 22, 60, (2, 2))


def single_1080(frames: int = 300) -> Clip:
    return Clip("single1080", 1920, 1080, frames, 2024, 22, 60, (4, 3), sprites=24, flash=True)


def mix(frames: int = 120, seed: int = 3) -> list[Clip]:
    """The 64-stream mix: per stream a seeded draw of grid, q and gop."""
    rng = random.Random(seed)
    out = []
    for (w, h), count in MIX_RES:
        for i in range(count):
            grid = rng.choice(GRIDS)
            qp = rng.choice(QPS)
            gop = rng.randint(30, 120)
            out.append(Clip(f"mix{frames}", w, h, frames, 1000 + len(out), qp, gop, grid))
    return out


def serve(frames: int = 600, distinct: int = 16, seed: int = 5) -> list[Clip]:
    """Clips of the serving loop: `distinct` 600-frame clips in the mix's
    proportions (1080p : 720p : 360p = 16 : 24 : 24) with the mix's per-stream
    draws; the serving streams cycle through them."""
    rng = random.Random(seed)
    total = sum(c for _, c in MIX_RES)
    out = []
    for (w, h), count in MIX_RES:
        n = max(1, round(distinct * count / total))
        for i in range(n):
            out.append(Clip(f"serve{frames}", w, h, frames, 5000 + len(out), rng.choice(QPS), rng.randint(30, 120),
                            rng.choice(GRIDS)))
    return out


def named(name: str) -> list[Clip]:
    return {"single640": lambda: [single_640()], "single1080": lambda: [single_1080()], "mix": mix,
            "serve": serve}[name]()


def ensure(clips: list[Clip], threads: int | None = None, log=None) -> None:
    """Encodes every missing clip in this process, largest first: each
    clip's encoder parallelises over its tiles and GOPs, and up to one clip
    per core runs at a time so no core idles behind one long clip."""
    import concurrent.futures as cf

    todo = [c for c in clips if not c.path().exists()]
    if not todo:
        return
    cores = threads or os.cpu_count() or 1
    todo.sort(key=lambda c: -c.cost())
    t0 = time.time()

    def one(c: Clip):
        data = c.encode(cores)
        tmp = c.path().with_suffix(f".tmp{os.getpid()}.{id(c)}")
        tmp.write_bytes(data)
        tmp.replace(c.path())
        return len(data)

    with cf.ThreadPoolExecutor(max_workers=min(len(todo), max(2, cores))) as ex:
        total = sum(ex.map(one, todo))
    if log:
        log(f"[workloads] encoded {len(todo)} clip(s), {total} bytes, in {time.time() - t0:.1f}s")


def load(clips: list[Clip], in_child: bool = True, log=None) -> list[bytes]:
    """Container bytes of every clip.  Missing clips are encoded first: in a
    child process when in_child (the caller then loads no encoder), else here."""
    missing = [c for c in clips if not c.path().exists()]
    if missing:
        if in_child:
            names = sorted({c.name for c in missing})
            env = dict(os.environ, EBIV_CONTENT_DIR=str(content_dir()))
            args = [sys.executable, "-m", "govid_gb300.workloads"] + [_cli_name(n) for n in names]
            subprocess.run(args, check=True, cwd=str(ROOT), env=env)
        else:
            ensure(missing, log=log)
    return [c.path().read_bytes() for c in clips]


def _cli_name(n: str) -> str:
    return "mix" if n.startswith("mix") else ("serve" if n.startswith("serve") else n)


def main(argv: list[str]) -> None:
    names = argv or ["single1080", "mix", "serve"]
    clips = [c for n in names for c in named(n)]
    ensure(clips, log=lambda *a: print(*a, file=sys.stderr, flush=True))


if __name__ == "__main__":
    main(sys.argv[1:])
