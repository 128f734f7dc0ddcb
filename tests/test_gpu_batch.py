"""Batched decode parity: many streams of uneven resolution, tile grid and
quantizer decoded together in rounds; every frame of every stream must be
bit-exact against the CPU oracle decoding that stream alone."""
import pytest

import ebiv_oracle
from govid_gb300 import ebiv

from helpers import encode_gen, first_diff, flash_gen, noisy_gen

pytestmark = pytest.mark.gpu


def _streams():
    out = []
    specs = [((160, 96), (1, 1), 18, 8, 1), ((320, 192), (2, 2), 22, 5, 2), ((96, 64), (4, 3), 28, 3, 3),
             ((200, 120), (2, 1), 22, 6, 4)]
    for (w, h), tiles, qp, gop, seed in specs:
        spec = ebiv.SceneSpec(width=w, height=h, seed=seed, sprites=3)
        cont = ebiv.encode_scene(spec, 9, qp=qp, gop=gop, tiles=tiles, fast=True, threads=4)
        out.append((cont, w, h))
    cont, _, _ = encode_gen(128, 96, 7, flash_gen, intra=16, gop=7)
    out.append((cont, 128, 96))
    cont, _, _ = encode_gen(64, 48, 10, noisy_gen, intra=16, gop=10, altref=4)
    out.append((cont, 64, 48))
    return out


def test_batch_matches_oracle(gpu_required):
    streams = _streams()
    b = ebiv.Batch()
    want, ids, dims = {}, [], {}
    for cont, w, h in streams:
        pkts = [p.data for p in ebiv.Reader(cont).packets()]
        sid = b.add_stream(pkts, ring=3)
        ids.append(sid)
        dims[sid] = (w, h)
        want[sid] = ebiv_oracle.decode_all(pkts)
    seen = 0
    while True:
        res = b.round()
        if not res:
            break
        for r in res:
            ws, wp = want[r.stream][r.frame_index]
            assert r.status == ws, f"stream {r.stream} frame {r.frame_index}: status {r.status} vs {ws}"
            if ws == 0:
                w, h = dims[r.stream]
                got = b.download(r, w, h)
                assert got == wp, f"stream {r.stream} frame {r.frame_index}: {first_diff(got, wp, w, h)}"
            seen += 1
    assert seen == sum(len(v) for v in want.values())


def test_batch_streaming_submit(gpu_required):
    # Streams fed one packet per round (the serving path) match the oracle.
    streams = _streams()[:3]
    b = ebiv.Batch()
    pk = []
    for cont, w, h in streams:
        pkts = [p.data for p in ebiv.Reader(cont).packets()]
        pk.append((b.add_streaming(3), pkts, ebiv_oracle.decode_all(pkts), w, h))
    for i in range(max(len(p[1]) for p in pk)):
        for sid, pkts, _, _, _ in pk:
            if i < len(pkts):
                b.submit(sid, pkts[i])
        for r in b.round():
            sid, pkts, want, w, h = next(p for p in pk if p[0] == r.stream)
            assert r.status == want[i][0]
            if r.status == 0:
                assert b.download(r, w, h) == want[i][1]


def test_batch_seek_replays_exactly(gpu_required):
    # Seeking a stream back to a key frame reproduces the same frames
    # (key frames are self-contained: ebiv/rans.go:397-405, codec.go:156-161).
    spec = ebiv.SceneSpec(width=160, height=96, seed=9, sprites=3)
    cont = ebiv.encode_scene(spec, 12, qp=22, gop=4, tiles=(2, 1), fast=True)
    pkts = [p.data for p in ebiv.Reader(cont).packets()]
    want = ebiv_oracle.decode_all(pkts)
    b = ebiv.Batch()
    sid = b.add_stream(pkts)
    for _ in range(9):
        b.round()
    b.seek(sid, 4)  # the key frame at index 4
    for i in range(4, 12):
        (r,) = b.round()
        assert r.frame_index == i and r.status == 0
        assert b.download(r, 160, 96) == want[i][1]
