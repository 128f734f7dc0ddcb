"""Learned motion-vector proposer for the EBIV encoder (include/ebiv_mvnet.h).

A 4-layer 3x3 conv net on quarter-resolution luma pairs proposes the top-8
full-pel motion vectors per 16x16 macroblock; the encoder's search="proposed"
mode evaluates them (with a one-pixel polish and the usual half/quarter-pel
refinement) instead of walking the diamond of ebiv/encode_inter.go:381-419.
Training and inference run in the project's own CUDA kernels; this module is
the host harness: it builds the training set from seeded synthetic clips
labelled by the GPU exhaustive search, runs the training loop and installs
the net in an encoder.
"""
from __future__ import annotations

import ctypes as C
import time
from pathlib import Path

import numpy as np

from . import _native
from .ebiv import Encoder, Scene, SceneSpec, _check

PARAMS = 28930
TOPK = 8
RANGE = 16
WEIGHTS = Path(__file__).resolve().parent / "mvnet_weights.f32"


def _u8(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_uint8))


def _i16(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_int16))


def _f32(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_float))


class MvNet:
    """One net for luma planes padded to pad_w x pad_h (multiples of 16)."""

    def __init__(self, pad_w: int, pad_h: int, max_batch: int = 1, max_pairs: int = 0, seed: int = 1):
        L = _native.lib()
        h = C.c_void_p()
        _check(L.ebiv_mvnet_create(int(max_batch), int(pad_w), int(pad_h), int(max_pairs), int(seed), C.byref(h)),
               "mvnet")
        self._h, self._L = h, L
        self.pad_w, self.pad_h, self.max_batch = pad_w, pad_h, max_batch
        self.mbs = (pad_w // 16) * (pad_h // 16)

    # parameters -----------------------------------------------------------
    @property
    def params(self) -> np.ndarray:
        p = np.empty(PARAMS, np.float32)
        _check(self._L.ebiv_mvnet_get_params(self._h, _f32(p)))
        return p

    @params.setter
    def params(self, p: np.ndarray) -> None:
        a = np.ascontiguousarray(p, dtype=np.float32)
        assert a.size == PARAMS
        _check(self._L.ebiv_mvnet_set_params(self._h, _f32(a)))

    def save(self, path: str | Path = WEIGHTS) -> None:
        self.params.astype("<f4").tofile(str(path))

    def load(self, path: str | Path = WEIGHTS) -> "MvNet":
        self.params = np.fromfile(str(path), dtype="<f4")
        return self

    # search and training ---------------------------------------------------
    def _planes(self, cur: np.ndarray, ref: np.ndarray):
        cur = np.ascontiguousarray(cur, dtype=np.uint8)
        ref = np.ascontiguousarray(ref, dtype=np.uint8)
        assert cur.shape == ref.shape and cur.shape[0] >= self.pad_h and cur.shape[1] >= self.pad_w
        return cur, ref

    def exhaustive(self, cur: np.ndarray, ref: np.ndarray, rng: int = RANGE):
        cur, ref = self._planes(cur, ref)
        mv = np.empty((self.mbs, 2), np.int16)
        sad = np.empty(self.mbs, np.int32)
        _check(self._L.ebiv_mvnet_exhaustive(self._h, _u8(cur), _u8(ref), cur.shape[1], int(rng), _i16(mv),
                                             sad.ctypes.data_as(C.POINTER(C.c_int32))))
        return mv, sad

    def add_pair(self, cur: np.ndarray, ref: np.ndarray, labels: np.ndarray) -> None:
        cur, ref = self._planes(cur, ref)
        lab = np.ascontiguousarray(labels, dtype=np.int16)
        _check(self._L.ebiv_mvnet_add_pair(self._h, _u8(cur), _u8(ref), cur.shape[1], _i16(lab)))

    @property
    def pairs(self) -> int:
        return int(self._L.ebiv_mvnet_pairs(self._h))

    def set_input(self, slot: int, cur: np.ndarray, ref: np.ndarray, labels: np.ndarray | None = None) -> None:
        cur, ref = self._planes(cur, ref)
        lab = None if labels is None else np.ascontiguousarray(labels, dtype=np.int16)
        _check(self._L.ebiv_mvnet_set_input(self._h, int(slot), _u8(cur), _u8(ref), cur.shape[1],
                                            None if lab is None else _i16(lab)))

    def gather(self, idx) -> None:
        a = np.ascontiguousarray(idx, dtype=np.int32)
        _check(self._L.ebiv_mvnet_gather(self._h, a.ctypes.data_as(C.POINTER(C.c_int32)), a.size))

    def gradients(self, batch: int):
        g = np.empty(PARAMS, np.float32)
        s = np.empty(3, np.float32)
        _check(self._L.ebiv_mvnet_gradients(self._h, int(batch), _f32(g), _f32(s)))
        return g, s

    def train_step(self, batch: int, lr: float) -> np.ndarray:
        s = np.empty(3, np.float32)
        _check(self._L.ebiv_mvnet_train_step(self._h, int(batch), float(lr), _f32(s)))
        return s

    def head(self, batch: int) -> np.ndarray:
        out = np.empty((batch, 34, self.pad_h // 4, self.pad_w // 4), np.float32)
        _check(self._L.ebiv_mvnet_head(self._h, int(batch), _f32(out)))
        return out

    def propose(self, cur: np.ndarray, ref: np.ndarray) -> np.ndarray:
        """Top-8 full-pel candidates per macroblock, (mbs, 8, 2)."""
        cur, ref = self._planes(cur, ref)
        out = np.empty((self.mbs, TOPK, 2), np.int16)
        _check(self._L.ebiv_mvnet_propose(self._h, _u8(cur), _u8(ref), cur.shape[1], _i16(out)))
        return out

    def attach(self, enc: Encoder) -> None:
        """Makes this net the candidate source of an encoder (search="proposed")."""
        _check(self._L.ebiv_encoder_set_mvnet(enc._h, self._h), "mvnet")
        enc._mvnet = self

    def __del__(self):
        try:
            if self._h:
                self._L.ebiv_mvnet_destroy(self._h)
                self._h = None
        except Exception:
            pass


def luma(packed: bytes, w: int, h: int) -> np.ndarray:
    return np.frombuffer(packed, np.uint8, count=w * h).reshape(h, w)


def clip_spec(seed: int, w: int, h: int, sprites: int = 24) -> SceneSpec:
    """Seeded sprite clip: velocities fractional in [-8, 8] px/frame, global
    pan up to 3 px/frame, noise sigma 2."""
    return SceneSpec(width=w, height=h, seed=seed, sprites=sprites, vel_max_q=32, integer_vel=False, pan_max_q=12)


def build_training_set(net: MvNet, clips: int, frames: int, seed0: int = 1000, log=print) -> dict:
    """Renders `clips` seeded clips of net's size, labels every consecutive
    frame pair with the GPU exhaustive search and adds it to the net's
    training set."""
    w, h = net.pad_w, net.pad_h
    t0 = time.time()
    for c in range(clips):
        sc = Scene(clip_spec(seed0 + c, w, h))
        prev = luma(sc.render(0), w, h)
        for i in range(1, frames):
            cur = luma(sc.render(i), w, h)
            mv, _ = net.exhaustive(cur, prev)
            net.add_pair(cur, prev, mv)
            prev = cur
        if log and (c + 1) % 25 == 0:
            log(f"[mvnet] clips {c + 1}/{clips}, pairs {net.pairs}, {time.time() - t0:.1f}s")
    return {"clips": clips, "frames_per_clip": frames, "pairs": net.pairs, "seconds": time.time() - t0}


def train(net: MvNet, steps: int, batch: int, lr: float = 2e-3, seed: int = 7, log=print, log_every: int = 200):
    """Adam on random batches of the training set, learning rate decayed
    linearly to 10 % over the run.  Returns the per-step statistics."""
    rng = np.random.default_rng(seed)
    hist = []
    t0 = time.time()
    for s in range(steps):
        net.gather(rng.integers(0, net.pairs, size=batch))
        st = net.train_step(batch, lr * (1.0 - 0.9 * s / max(1, steps - 1)))
        hist.append(st.copy())
        if log and (s + 1) % log_every == 0:
            m = np.mean(hist[-log_every:], axis=0)
            log(f"[mvnet] step {s + 1}/{steps} loss {m[0]:.3f} top1 {m[1]:.3f} top8 {m[2]:.3f} "
                f"{time.time() - t0:.1f}s")
    return np.array(hist)
