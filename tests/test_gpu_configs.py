"""Bit-exact decode of the benchmark workloads at their full sizes.

Every frame of every clip, decoded on the GPU through the drop-in Codec
contract (``ebivgpu_decode``) and through the pipelined Batch path, must hash
(SHA-256 of the packed planes) to the CPU oracle's decode of the same packets
— the reference's own regression and tiling tests compare whole clips the
same way (ebiv/regression_test.go:15-39, ebiv/tile_test.go:52-70):

* the 640x360 60-frame 2x2-tile clip, q22, gop 60;
* the 1920x1080 300-frame 4x3-tile clip with flashes (the single-stream
  benchmark clip);
* streams of the 64-stream mix at their real resolutions: a 1920x1080 stream
  coded as one tile and a 1280x720 stream coded as 4x3 tiles, 120 frames,
  decoded together in one batch;
* a tile wider than 128 macroblocks (2304x256, one tile), whose rows the
  entropy stage keeps in global memory instead of shared memory.

Clips come from the content cache (govid_gb300/workloads.py), encoded on the
first run.
"""
import hashlib
import os

import pytest

import ebiv_oracle
from govid_gb300 import ebiv, workloads

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 1


def sha(b: bytes) -> str:
    return hashlib.sha256(b).hexdigest()


def oracle_hashes(pkts):
    c = ebiv_oracle.OracleCodec(3, THREADS)
    out = []
    for p in pkts:
        st, planes = c.decode(p)
        out.append((st, sha(planes) if st == 0 else None))
    return out


def packets(cont):
    return [p.data for p in ebiv.Reader(cont).packets()]


def codec_hashes(pkts):
    c = ebiv.Codec(3)
    out = []
    for p in pkts:
        try:
            out.append((0, sha(c.decode(p).packed())))
        except ebiv.EbivError as e:
            out.append((e.status, None))
    c.close()
    return out


def batch_hashes(streams, lookahead=32, depth=3):
    """streams: [(packets, w, h)] decoded together; per stream the list of
    (status, hash) in frame order."""
    b = ebiv.Batch(lookahead=lookahead, pipeline=depth)
    ids = [b.add_stream(pk, ring=3) for pk, _, _ in streams]
    got = {sid: {} for sid in ids}
    dims = {sid: (w, h) for sid, (_, w, h) in zip(ids, streams)}
    empty = 0
    res_all = []
    while empty < b.depth + 1:
        res = b.round()
        empty = empty + 1 if not res else 0
        for r in res:
            w, h = dims[r.stream]
            got[r.stream][r.frame_index] = (r.status, sha(b.download(r, w, h)) if r.status == 0 else None)
        res_all += res
    for r in b.drain():
        w, h = dims[r.stream]
        got[r.stream][r.frame_index] = (r.status, sha(b.download(r, w, h)) if r.status == 0 else None)
    b.close()
    return [[got[sid][i] for i in range(len(streams[k][0]))] for k, sid in enumerate(ids)]


def _compare(got, want, what):
    assert len(got) == len(want), what
    bad = [i for i, (g, w) in enumerate(zip(got, want)) if g != w]
    assert not bad, f"{what}: {len(bad)} frame(s) differ from the oracle, first {bad[0]}: {got[bad[0]]} vs {want[bad[0]]}"
    assert all(s == 0 for s, _ in want), f"{what}: the oracle failed a frame"


def test_config_640x360_60_frames(gpu_required):
    clip = workloads.single_640()
    pk = packets(workloads.load([clip], in_child=False)[0])
    assert len(pk) == 60
    want = oracle_hashes(pk)
    _compare(codec_hashes(pk), want, "Codec 640x360")
    _compare(batch_hashes([(pk, clip.w, clip.h)])[0], want, "Batch 640x360")


def test_config_1080p_300_frames_flashes(gpu_required):
    clip = workloads.single_1080()
    pk = packets(workloads.load([clip], in_child=False)[0])
    assert len(pk) == 300
    assert sum(1 for p in pk if (p[0] & 3) == 0) >= 5  # gop 60, plus scene cuts at flashes
    want = oracle_hashes(pk)
    _compare(codec_hashes(pk), want, "Codec 1080p")
    _compare(batch_hashes([(pk, clip.w, clip.h)])[0], want, "Batch 1080p")


def test_config_mix_streams_real_resolutions(gpu_required):
    mix = workloads.mix()
    # the shortest-GOP draws keep a first encode short (GOPs encode in parallel)
    a = min((c for c in mix if c.w == 1920 and c.grid == (1, 1)), key=lambda c: c.gop)
    b = min((c for c in mix if c.w == 1280 and c.grid == (4, 3)), key=lambda c: c.gop)
    conts = workloads.load([a, b], in_child=False)
    pa, pb = packets(conts[0]), packets(conts[1])
    assert len(pa) == len(pb) == 120
    wa, wb = oracle_hashes(pa), oracle_hashes(pb)
    _compare(codec_hashes(pa), wa, "Codec 1080p 1x1")
    ga, gb = batch_hashes([(pa, a.w, a.h), (pb, b.w, b.h)], lookahead=4, depth=2)
    _compare(ga, wa, "Batch 1080p 1x1")
    _compare(gb, wb, "Batch 720p 4x3")


def test_tile_wider_than_shared_rows(gpu_required):
    # 2304 px = 144 macroblocks in one tile: above the 128 the entropy stage
    # keeps in shared memory, so the vector and level rows live in the frame grid.
    spec = ebiv.SceneSpec(width=2304, height=256, seed=21, sprites=10)
    cont = ebiv.encode_scene(spec, 8, qp=22, gop=8, tiles=(1, 1), fast=True, threads=THREADS)
    pk = packets(cont)
    want = oracle_hashes(pk)
    _compare(codec_hashes(pk), want, "Codec 2304x256")
    _compare(batch_hashes([(pk, 2304, 256)], lookahead=4, depth=2)[0], want, "Batch 2304x256")
