"""Fuzzing the GPU decoder's host-side packet planning on the CPU.

The decode kernels read only byte ranges, macroblock bounds and tables that
the host planner (govid_gb300/csrc/payload.cpp, container.cpp) produced and
checked, so malformed packets must be stopped there or produce a plan whose
invariants hold. tests/native/plan_fuzz.cpp replays the Codec contract's host
steps over seeded mutations of the golden clips, built with AddressSanitizer
and UBSan, checks each accepted plan's invariants and that every packet the
host rejects, the oracle rejects with the same status (the reference's
errors, ebiv/codec.go:70-192, ebiv/frame.go:197-274, ebiv/rans.go:396-471).
"""
import os
import shutil
import struct
import subprocess
from pathlib import Path

import numpy as np
import pytest

import ebiv_oracle
from govid_gb300 import ebiv

ROOT = Path(__file__).resolve().parent.parent
CSRC = ROOT / "govid_gb300" / "csrc"
GOLDEN = Path(__file__).resolve().parent / "golden"
CLIPS = ["gate_clip", "flash_128x96", "altref_64x48", "odd_37x21", "scene_160x96"]


def _build(out: Path) -> Path:
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    exe = out / "plan_fuzz"
    srcs = [str(Path(__file__).parent / "native" / "plan_fuzz.cpp"), str(CSRC / "payload.cpp"), str(CSRC / "container.cpp")]
    base = [gxx, "-std=c++17", "-O1", "-g", f"-I{CSRC}", *srcs, "-o", str(exe)]
    san = ["-fsanitize=address,undefined", "-fno-sanitize-recover=all", "-fno-omit-frame-pointer"]
    r = subprocess.run(base[:1] + san + base[1:], capture_output=True, text=True)
    if r.returncode != 0:  # no sanitizer runtime: the invariants and statuses are still checked
        r = subprocess.run(base, capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
    return exe


def _mutate(pk: bytes, rng) -> bytes:
    """One seeded mutation, aimed at the planned fields: the frame header, the
    coded header (qp, tile counts), the table block and the tile length
    varints, which all sit near the start of a packet."""
    b = bytearray(pk)
    kind = rng.integers(0, 6)
    head = max(1, min(len(b), 96 if rng.integers(0, 2) else 600))  # the coded header, or into the tables
    if kind == 0:  # flip one bit near the start
        i = int(rng.integers(0, head))
        b[i] ^= 1 << int(rng.integers(0, 8))
    elif kind == 1:  # a random byte anywhere
        i = int(rng.integers(0, len(b)))
        b[i] = int(rng.integers(0, 256))
    elif kind == 2:  # truncate
        b = b[: int(rng.integers(0, len(b)))]
    elif kind == 3:  # a varint continuation run near the start
        i = int(rng.integers(0, head))
        for j in range(i, min(len(b), i + int(rng.integers(1, 10)))):
            b[j] = 0xFF
    elif kind == 4:  # insert or delete a byte near the start
        i = int(rng.integers(0, head))
        if rng.integers(0, 2):
            b.insert(i, int(rng.integers(0, 256)))
        else:
            del b[i]
    else:  # rewrite the coded header's tile counts (key frames: body at 6, inter: at 1)
        off = 6 if (b and (b[0] & 3) == 0) else 1
        if len(b) > off + 2:
            b[off + 1] = int(rng.integers(0, 130))
            b[off + 2] = int(rng.integers(0, 130))
    return bytes(b)


def _streams(seed: int, per_clip: int):
    rng = np.random.default_rng(seed)
    out = []
    for name in CLIPS:
        pk = [p.data for p in ebiv.Reader((GOLDEN / f"{name}.ebiv").read_bytes()).packets()]
        out.append(list(pk))  # the intact clip
        for _ in range(per_clip):
            s = list(pk)
            for _ in range(int(rng.integers(1, 4))):
                i = int(rng.integers(0, len(s)))
                s[i] = _mutate(s[i], rng)
            out.append(s)
    return out


def test_planner_invariants_and_statuses_under_fuzz(tmp_path):
    exe = _build(tmp_path)
    streams = _streams(seed=2024, per_clip=160)
    blob = bytearray(struct.pack("<I", len(streams)))
    for s in streams:
        statuses = [st for st, _ in ebiv_oracle.decode_all(s)]
        blob += struct.pack("<I", len(s))
        for p, st in zip(s, statuses):
            blob += struct.pack("<Ii", len(p), st) + p
    inp = tmp_path / "streams.bin"
    inp.write_bytes(bytes(blob))
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=0:abort_on_error=0", UBSAN_OPTIONS="print_stacktrace=1")
    r = subprocess.run([str(exe), str(inp)], capture_output=True, text=True, timeout=600, env=env)
    assert r.returncode == 0, r.stdout + r.stderr[-4000:]
    f = r.stdout.split()
    counts = dict(zip(f[0::2], map(int, f[1::2])))
    assert counts["streams"] == len(streams) and counts["mismatches"] == 0
    # The mutations reach both the host checks and the kernels' own checks.
    assert counts["host_rejects"] > 500 and counts["kernel_rejects"] > 40 and counts["accepted"] > 3000
