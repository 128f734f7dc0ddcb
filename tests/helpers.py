"""Shared helpers for the EBIV tests: clip encoders restating the reference
test harness (ebiv/harness_test.go, ebiv/coded_test.go) and a differential
decode against the CPU oracle."""
from __future__ import annotations

import numpy as np

from govid_gb300 import ebiv


def encode_gen(w, h, n, gen, **opts) -> tuple[bytes, list[bytes], list[bytes]]:
    """encodeCodedGen (ebiv/coded_test.go:111-130): returns (container, sources, reconstructions)."""
    opts.setdefault("keep_recon", True)
    enc = ebiv.Encoder(ebiv.Config(w, h), **opts)
    srcs = []
    for i in range(n):
        f = gen(w, h, i)
        srcs.append(f)
        enc.write_frame(f)
    enc.close()
    return enc.output(), srcs, enc.recons()


def flash_gen(w, h, i):
    """TestGoldenRefFlashingSequence's generator (ebiv/coded_test.go:436-447)."""
    return ebiv.synth_frame(w, h, 1 if i % 2 == 0 else 2)


def noisy_gen(w, h, i):
    """TestAltRefGoldenOverride's hold-under-noise generator (ebiv/coded_test.go:664-674)."""
    img = np.frombuffer(ebiv.synth_frame(w, h, 3), np.uint8).copy()
    y = img[: w * h].reshape(h, w).astype(np.int32)
    yy, xx = np.mgrid[0:h, 0:w]
    n = ((xx * 31 + yy * 17 + i * 97) % 13) - 6
    img[: w * h] = np.clip(y + n, 0, 255).astype(np.uint8).ravel()
    return img.tobytes()


def psnr(a: bytes, b: bytes) -> float:
    x = np.frombuffer(a, np.uint8).astype(np.float64)
    y = np.frombuffer(b, np.uint8).astype(np.float64)
    mse = np.mean((x - y) ** 2)
    return float("inf") if mse == 0 else 10 * np.log10(255 * 255 / mse)


def gpu_decode_all(packets: list[bytes], ring: int = 3) -> list[tuple[int, bytes | None]]:
    c = ebiv.Codec(ring)
    out = []
    for p in packets:
        try:
            f = c.decode(p)
            out.append((0, f.packed()))
        except ebiv.EbivError as e:
            out.append((e.status, None))
    return out


def first_diff(a: bytes, b: bytes, w: int, h: int) -> str:
    x = np.frombuffer(a, np.uint8)
    y = np.frombuffer(b, np.uint8)
    d = np.nonzero(x != y)[0]
    if len(d) == 0:
        return "identical"
    i = int(d[0])
    plane, off = ("Y", i) if i < w * h else (("Cb", i - w * h) if i < w * h + ((w + 1) // 2) * ((h + 1) // 2)
                                             else ("Cr", i - w * h - ((w + 1) // 2) * ((h + 1) // 2)))
    pw = w if plane == "Y" else (w + 1) // 2
    return f"{len(d)} bytes differ; first in {plane} at ({off % pw},{off // pw}): got {x[i]} want {y[i]}"
