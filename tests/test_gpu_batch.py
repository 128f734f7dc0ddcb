"""Batched decode parity: many streams of uneven resolution, tile grid and
quantizer decoded together in rounds; every frame of every stream must be
bit-exact against the CPU oracle decoding that stream alone."""
import pytest

import ebiv_oracle
from govid_gb300 import ebiv

from helpers import encode_gen, first_diff, flash_gen, noisy_gen

pytestmark = pytest.mark.gpu


def run_rounds(b):
    """All results of a batch, synchronous or pipelined: a pipelined round
    returns the results of the round planned b.depth calls before, so stop
    after depth + 1 empty rounds and collect the rounds still in flight."""
    empty = 0
    while empty < b.depth + 1:
        res = b.round()
        empty = empty + 1 if not res else 0
        yield from res
    yield from b.drain()


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


@pytest.mark.parametrize("lookahead,pipeline,tuning", [(1, False, None), (4, False, None), (1, True, None),
                                                        (4, True, None), (1, 2, None), (4, 2, None), (4, 3, None),
                                                        (4, 2, (1, 4)), (8, 3, (2, 16)), (2, 1, (4, 8))])
def test_batch_matches_oracle(gpu_required, lookahead, pipeline, tuning):
    # Every launch shape the autotuner may pick gives the same frames.
    streams = _streams()
    b = ebiv.Batch(lookahead=lookahead, pipeline=pipeline)
    if tuning:
        b.set_tuning(*tuning)
    want, ids, dims = {}, [], {}
    for cont, w, h in streams:
        pkts = [p.data for p in ebiv.Reader(cont).packets()]
        sid = b.add_stream(pkts, ring=3)
        ids.append(sid)
        dims[sid] = (w, h)
        want[sid] = ebiv_oracle.decode_all(pkts)
    seen = 0
    for r in run_rounds(b):
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


def _zero_tile(pkt: bytes, tile: int) -> bytes:
    """Zeroes one tile's rANS bytes: the decoder underruns inside that tile."""
    from govid_gb300 import ebiv as E

    hdr = E.parse_frame_header(pkt)
    b = bytearray(pkt)
    pos = hdr["body_offset"] + 1  # skip qp

    def uvar(p):
        x, s = 0, 0
        while True:
            c = b[p]
            x |= (c & 0x7F) << s
            p += 1
            if c < 0x80:
                return x, p
            s += 7

    _, pos = uvar(pos)  # tile cols
    _, pos = uvar(pos)  # tile rows
    tl, pos = uvar(pos)
    pos += tl  # tables
    for t in range(tile + 1):
        n, pos = uvar(pos)
        if t == tile:
            b[pos:pos + n] = bytes(n)
        pos += n
    return bytes(b)


@pytest.mark.parametrize("lookahead,pipeline", [(1, False), (4, False), (1, True), (4, True), (4, 2)])
def test_batch_error_mid_chain_matches_oracle(gpu_required, lookahead, pipeline):
    # A frame that fails on the GPU leaves its references untouched
    # (ebiv/codec.go:174-191); later frames of the same round are re-planned.
    spec = ebiv.SceneSpec(width=160, height=96, seed=21, sprites=3)
    cont = ebiv.encode_scene(spec, 12, qp=22, gop=12, tiles=(2, 1), fast=True)
    pkts = [p.data for p in ebiv.Reader(cont).packets()]
    pkts[3] = _zero_tile(pkts[3], 1)
    pkts[8] = _zero_tile(pkts[8], 0)
    want = ebiv_oracle.decode_all(pkts)
    assert want[3][0] == ebiv.ErrCorrupt.status and want[8][0] == ebiv.ErrCorrupt.status
    b = ebiv.Batch(lookahead=lookahead, pipeline=pipeline)
    b.add_stream(pkts)
    got = {}
    for r in run_rounds(b):
        assert r.frame_index not in got, f"frame {r.frame_index} delivered twice"
        got[r.frame_index] = (r.status, b.download(r, 160, 96) if r.status == 0 else None)
    assert sorted(got) == list(range(len(pkts)))
    for i, (ws, wp) in enumerate(want):
        assert got[i][0] == ws, f"frame {i}: status {got[i][0]} vs oracle {ws}"
        assert got[i][1] == wp, f"frame {i} differs from the oracle"


def test_fuzzed_packets_match_oracle(gpu_required):
    # FuzzDecodePacket-style (ebiv/fuzz_test.go): seeded byte flips in the
    # seed clip's packets; statuses and every decoded plane match the oracle.
    import random

    from helpers import encode_gen

    cont, _, _ = encode_gen(64, 48, 6, lambda w, h, i: ebiv.synth_frame(w, h, 1 if i < 3 else 2), intra=20, gop=4,
                            altref=4, fast=True, keep_recon=False)
    clean = [p.data for p in ebiv.Reader(cont).packets()]
    rng = random.Random(1234)
    for case in range(24):
        pkts = []
        for p in clean:
            b = bytearray(p)
            for _ in range(rng.randint(0, 3)):
                i = rng.randrange(len(b))
                b[i] ^= 1 << rng.randrange(8)
            if rng.random() < 0.1:
                b = b[: rng.randrange(1, len(b) + 1)]
            pkts.append(bytes(b))
        want = ebiv_oracle.decode_all(pkts)
        c = ebiv.Codec()
        for i, p in enumerate(pkts):
            try:
                g = (0, c.decode(p).packed())
            except ebiv.EbivError as e:
                g = (e.status, None)
            assert g[0] == want[i][0], f"case {case} frame {i}: status {g[0]} vs oracle {want[i][0]}"
            assert g[1] == want[i][1], f"case {case} frame {i}: planes differ from the oracle"


@pytest.mark.parametrize("lookahead,depth", [(1, 1), (3, 1), (3, 2), (2, 3)])
def test_fuzzed_streams_pipelined_batch_match_oracle(gpu_required, lookahead, depth):
    # Corrupted packets in several streams decoded together by a pipelined
    # batch: every status and plane equals the oracle decoding each stream
    # alone, through the rollbacks that failures force on rounds planned
    # ahead of them.
    import random

    rng = random.Random(77 + lookahead)
    streams = []
    for k in range(4):
        spec = ebiv.SceneSpec(width=96 + 32 * k, height=64, seed=300 + k, sprites=2)
        cont = ebiv.encode_scene(spec, 14, qp=22, gop=5 + k, tiles=(2, 1), fast=True)
        pkts = []
        for p in (q.data for q in ebiv.Reader(cont).packets()):
            b = bytearray(p)
            if rng.random() < 0.3:
                for _ in range(rng.randint(1, 3)):
                    i = rng.randrange(len(b))
                    b[i] ^= 1 << rng.randrange(8)
            pkts.append(bytes(b))
        streams.append((pkts, 96 + 32 * k, 64))
    b = ebiv.Batch(lookahead=lookahead, pipeline=depth)
    want, dims = {}, {}
    for pkts, w, h in streams:
        sid = b.add_stream(pkts)
        want[sid] = ebiv_oracle.decode_all(pkts)
        dims[sid] = (w, h)
    got = {}
    for r in run_rounds(b):
        key = (r.stream, r.frame_index)
        assert key not in got, f"{key} delivered twice"
        got[key] = (r.status, b.download(r, *dims[r.stream]) if r.status == 0 else None)
    for sid, frames in want.items():
        for i, (ws, wp) in enumerate(frames):
            assert (sid, i) in got, f"stream {sid} frame {i} never delivered"
            assert got[(sid, i)][0] == ws, f"stream {sid} frame {i}: status {got[(sid, i)][0]} vs {ws}"
            assert got[(sid, i)][1] == wp, f"stream {sid} frame {i} differs from the oracle"


def test_async_downloads_of_a_deep_pipeline_match_oracle(gpu_required):
    # Every result of a depth-3 pipelined batch queued into pinned host memory
    # on the engine's copy stream while later rounds decode: after sync() each
    # frame equals the oracle (later rounds never overwrite a frame whose copy
    # is still queued).
    torch = pytest.importorskip("torch")
    streams = _streams()
    b = ebiv.Batch(lookahead=4, pipeline=3)
    want, dims = {}, {}
    for cont, w, h in streams:
        pkts = [p.data for p in ebiv.Reader(cont).packets()]
        sid = b.add_stream(pkts, ring=3)
        dims[sid] = (w, h)
        want[sid] = ebiv_oracle.decode_all(pkts)
    total = sum(ebiv_frame_bytes(*dims[s]) * len(want[s]) for s in want)
    host = torch.empty(total, dtype=torch.uint8, pin_memory=True)
    placed, off = [], 0
    for r in run_rounds(b):
        ws, _ = want[r.stream][r.frame_index]
        assert r.status == ws
        if ws != 0:
            continue
        n = ebiv_frame_bytes(*dims[r.stream])
        b.download_async(r, host.data_ptr() + off, n)
        placed.append((r.stream, r.frame_index, off, n))
        off += n
    b.sync()
    data = host.numpy().tobytes()
    assert placed
    for sid, i, o, n in placed:
        assert data[o:o + n] == want[sid][i][1], f"stream {sid} frame {i} differs from the oracle"


def ebiv_frame_bytes(w, h):
    return w * h + 2 * ((w + 1) // 2) * ((h + 1) // 2)
