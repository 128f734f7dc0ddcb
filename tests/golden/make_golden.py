"""Generates the committed EBIV fixtures in this directory.

Each fixture is a container written by this repo's encoder plus, in
golden.json, the container's SHA-256 and the SHA-256 of every frame the CPU
oracle decodes from it.  The CPU tests regenerate the containers (encoder
determinism on every host) and re-decode them; the GPU tests decode the
committed bytes and compare hashes.  The reference decoder cannot run here,
so these pin this build across hosts and changes; parity with the reference
rests on the gate-clip size and the restated known-answer tests.

Run from the repository root:  python tests/golden/make_golden.py
"""
import hashlib
import json
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path[:0] = [str(ROOT), str(ROOT / "oracle"), str(ROOT / "tests")]

import ebiv_oracle  # noqa: E402
from govid_gb300 import ebiv  # noqa: E402
from helpers import encode_gen, flash_gen, noisy_gen  # noqa: E402


def fixtures():
    """name -> (width, height, builder)."""
    return {
        "gate_clip": (256, 192, lambda: encode_gen(256, 192, 16, ebiv.synth_pan, intra=18, gop=8, tiles=(2, 2),
                                                   keep_recon=False)[0]),
        "flash_128x96": (128, 96, lambda: encode_gen(128, 96, 9, flash_gen, intra=16, gop=9, keep_recon=False)[0]),
        "altref_64x48": (64, 48, lambda: encode_gen(64, 48, 10, noisy_gen, intra=16, gop=10, altref=4,
                                                    keep_recon=False)[0]),
        "scene_160x96": (160, 96, lambda: ebiv.encode_scene(ebiv.SceneSpec(width=160, height=96, seed=7, sprites=3),
                                                            8, qp=22, gop=8, tiles=(2, 1), fast=True)),
        "odd_37x21": (37, 21, lambda: encode_gen(37, 21, 4, ebiv.synth_pan, intra=20, gop=4, keep_recon=False)[0]),
    }


def digest(b: bytes) -> str:
    return hashlib.sha256(b).hexdigest()


def main():
    out = {}
    for name, (w, h, build) in fixtures().items():
        cont = build()
        (HERE / f"{name}.ebiv").write_bytes(cont)
        pk = [p.data for p in ebiv.Reader(cont).packets()]
        dec = ebiv_oracle.decode_all(pk)
        out[name] = {"width": w, "height": h, "bytes": len(cont), "sha256": digest(cont),
                     "frames": [{"status": s, "sha256": digest(p) if p else None} for s, p in dec]}
    (HERE / "golden.json").write_text(json.dumps(out, indent=1) + "\n")
    print(json.dumps({k: v["bytes"] for k, v in out.items()}))


if __name__ == "__main__":
    main()
