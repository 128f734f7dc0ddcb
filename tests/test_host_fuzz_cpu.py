"""Fuzzing the host code in front of the GPU decoder, on the CPU, built with
AddressSanitizer and UBSan.

* Packet planning. The decode kernels read only byte ranges, macroblock
  bounds and tables that the host planner (govid_gb300/csrc/payload.cpp,
  container.cpp) produced and checked, so malformed packets must be stopped
  there or produce a plan whose invariants hold. tests/native/plan_fuzz.cpp
  replays the Codec contract's host steps over seeded mutations of the golden
  clips, checks each accepted plan's invariants and that every packet the
  host rejects, the oracle rejects with the same status (the reference's
  errors, ebiv/codec.go:70-192, ebiv/frame.go:197-274, ebiv/rans.go:396-471).
* The demuxer. tests/native/container_fuzz.cpp opens seeded mutations of the
  golden containers (header, frame records, footer, index entries with the
  CRC recomputed, truncations) with the product's reader and reads every
  packet; statuses, indexes and packet bytes must equal the oracle's demuxer
  (ebiv/reader.go:32-217).
"""
import os
import shutil
import struct
import subprocess
import zlib
from pathlib import Path

import numpy as np
import pytest

import ebiv_oracle
from govid_gb300 import ebiv

ROOT = Path(__file__).resolve().parent.parent
CSRC = ROOT / "govid_gb300" / "csrc"
GOLDEN = Path(__file__).resolve().parent / "golden"
CLIPS = ["gate_clip", "flash_128x96", "altref_64x48", "odd_37x21", "scene_160x96"]


def _build(out: Path, harness: str, sources) -> Path:
    """The harness and the product sources under test with the sanitizers;
    encoder.cpp (which holds the container's CRC-32) plain, as it is only
    linked, not fuzzed."""
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    exe = out / harness
    enc = out / "encoder.o"
    r = subprocess.run([gxx, "-std=c++17", "-O0", f"-I{CSRC}", "-c", str(CSRC / "encoder.cpp"), "-o", str(enc)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    srcs = [str(Path(__file__).parent / "native" / f"{harness}.cpp")] + [str(CSRC / f) for f in sources]
    base = [gxx, "-std=c++17", "-O1", "-g", f"-I{CSRC}", *srcs, str(enc), "-lpthread", "-o", str(exe)]
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
    exe = _build(tmp_path, "plan_fuzz", ("payload.cpp", "container.cpp"))
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


U64 = (1 << 64) - 1
_OFFSETS = [0, 47, 48, U64, U64 - 7, U64 - 8, U64 - 15, U64 - 16, 1 << 63, (1 << 63) - 1]
_SIZES = [0, 1, 40, 256 << 20, (256 << 20) + 1, 0xFFFFFFFF]


def _index_at(b: bytes):
    if len(b) < 68 or b[-4:] != b"EBIX":
        return None
    off, count, _ = struct.unpack_from("<QII", b, len(b) - 20)
    if off < 48 or off + 16 * count != len(b) - 20:
        return None
    return off, count


def _mutate_container(data: bytes, rng) -> bytes:
    b = bytearray(data)
    kind = int(rng.integers(0, 7))
    if not b:  # an earlier truncation left nothing to change
        return bytes(b)
    if kind == 0:  # a file header byte
        b[int(rng.integers(0, min(48, len(b))))] = int(rng.integers(0, 256))
    elif kind == 1:  # a footer byte
        b[len(b) - 1 - int(rng.integers(0, min(20, len(b))))] ^= 1 << int(rng.integers(0, 8))
    elif kind == 2:  # any byte (frame records included)
        i = int(rng.integers(0, len(b)))
        b[i] = int(rng.integers(0, 256))
    elif kind == 3:  # truncated
        b = b[: int(rng.integers(0, len(b)))]
    elif kind == 4:  # trailing bytes after the footer
        b += bytes(rng.integers(0, 256, int(rng.integers(1, 40)), dtype=np.uint8))
    else:  # an index entry or the footer's count, with the CRC recomputed
        at = _index_at(bytes(b))
        if at is None:
            return bytes(b)
        off, count = at
        if kind == 5 and count:
            i = int(rng.integers(0, count))
            o, n, fl = struct.unpack_from("<QII", b, off + 16 * i)
            field = int(rng.integers(0, 3))
            if field == 0:
                pick = int(rng.integers(0, len(_OFFSETS) + 2))
                o = _OFFSETS[pick] if pick < len(_OFFSETS) else int(rng.integers(0, len(b)))
            elif field == 1:
                pick = int(rng.integers(0, len(_SIZES) + 1))
                n = _SIZES[pick] if pick < len(_SIZES) else int(rng.integers(1, 4096))
            else:
                fl = int(rng.integers(0, 4)) | (0xFFFFFFF0 if rng.integers(0, 2) else 0)
            struct.pack_into("<QII", b, off + 16 * i, o, n & 0xFFFFFFFF, fl)
        elif kind == 6:  # drop trailing entries: the footer moves with them
            keep = int(rng.integers(0, count + 1))
            entries = bytes(b[off:off + 16 * keep])
            tail = struct.pack("<QII", off, keep, 0) + b"EBIX"
            b = b[:off] + bytearray(entries) + bytearray(tail)
        raw = bytes(b[off:len(b) - 20])
        struct.pack_into("<I", b, len(b) - 8, zlib.crc32(raw) & 0xFFFFFFFF)
    return bytes(b)


def _oracle_line(data: bytes) -> str:
    import ebiv_container

    try:
        _, entries, rebuilt = ebiv_container.demux(data)
    except ebiv_container.ContainerError as e:
        return str(e.status)
    parts = ["0", str(len(entries)), str(int(rebuilt))]
    for p, n, k in entries:
        if p is None:
            parts.append(f"-1:{n}:{int(k)}")
        else:
            parts.append(f"{p}:{n}:{int(k)}:{zlib.crc32(data[p:p + n]) & 0xFFFFFFFF:08x}")
    return " ".join(parts)


def test_demuxer_matches_the_oracle_under_fuzz(tmp_path):
    exe = _build(tmp_path, "container_fuzz", ("container.cpp",))
    rng = np.random.default_rng(77)
    files = []
    for name in CLIPS:
        data = (GOLDEN / f"{name}.ebiv").read_bytes()
        files.append(data)
        for _ in range(240):
            m = data
            for _ in range(int(rng.integers(1, 3))):
                m = _mutate_container(m, rng)
            files.append(m)
    blob = bytearray(struct.pack("<I", len(files)))
    for f in files:
        blob += struct.pack("<I", len(f)) + f
    inp = tmp_path / "containers.bin"
    inp.write_bytes(bytes(blob))
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=0", UBSAN_OPTIONS="print_stacktrace=1")
    r = subprocess.run([str(exe), str(inp)], capture_output=True, text=True, timeout=600, env=env)
    assert r.returncode == 0, r.stderr[-4000:]
    got = r.stdout.splitlines()
    assert len(got) == len(files)
    want = [_oracle_line(f) for f in files]
    bad = [i for i in range(len(files)) if got[i] != want[i]]
    assert not bad, f"{len(bad)} containers differ; first {bad[0]}:\n got {got[bad[0]][:300]}\nwant {want[bad[0]][:300]}"
    statuses = [int(w.split()[0]) for w in want]
    # The mutations reach every outcome: opened from the index, rebuilt by
    # scanning, each header error, and entries NextPacket cannot read.
    assert statuses.count(0) > 300 and {1, 4, 5, 6} <= set(statuses)
    assert sum(1 for w in want if w.startswith("0 ") and w.split()[2] == "1") > 50
    assert sum(1 for w in want if " -1:" in w) > 3
