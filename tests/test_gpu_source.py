"""The decode-ahead frame source (ebivgpu_source_*, govid's asyncSource,
source.go:84-266) on the GPU: the behaviour govid's AsyncPlayer tests check
(async_test.go: frames in order, decode-ahead with a bounded queue, seek
generations, seek after the end, close, prepared RGBA and its pooled
buffers), with real EBIV streams whose every frame must equal the oracle's
decode."""
import hashlib
import json
import time
from pathlib import Path

import numpy as np
import pytest

import ebiv_oracle
from govid_gb300 import ebiv

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"
META = json.loads((GOLDEN / "golden.json").read_text())


def sha(b: bytes) -> str:
    return hashlib.sha256(b).hexdigest()


def drain_all(src, release=True):
    """next() until EOF: [(frame_index, timestamp, sha)]."""
    out = []
    while True:
        try:
            f = src.next()
        except ebiv.EOF:
            return out
        out.append((f.frame_index, f.timestamp_ns, sha(f.packed())))
        if release:
            src.release(f)


def scene(frames=40, gop=12):
    spec = ebiv.SceneSpec(width=160, height=96, seed=5, sprites=4)
    return ebiv.encode_scene(spec, frames, qp=22, gop=gop, tiles=(2, 1), fast=True)


@pytest.mark.parametrize("name", ["gate_clip", "flash_128x96", "altref_64x48", "odd_37x21"])
@pytest.mark.parametrize("depth", [1, 4, 32])
def test_source_delivers_every_frame_in_order_bit_exact(gpu_required, name, depth):
    # TestAsyncPlayerDeliversFramesInOrder with the golden clips' decoded planes.
    data = (GOLDEN / f"{name}.ebiv").read_bytes()
    want = META[name]["frames"]
    rd = ebiv.Reader(data)
    src = ebiv.AsyncSource(data, depth=depth)
    got = drain_all(src)
    src.destroy()
    ok = [w["sha256"] for w in want if w["status"] == 0]
    assert len(ok) == len(want), "golden clips decode without errors"
    assert [g[0] for g in got] == list(range(len(want)))
    assert [g[1] for g in got] == [rd.frame_time(i) for i in range(len(want))]
    assert [g[2] for g in got] == ok


def test_source_decodes_ahead_with_a_bounded_queue(gpu_required):
    # TestAsyncPlayerDecodesAhead: with nothing consumed the worker fills the
    # queue, then stops (frames are decoded a round of `lookahead` at a time).
    data = scene(60)
    depth = 4
    src = ebiv.AsyncSource(data, depth=depth)
    deadline = time.time() + 10
    while src.decoded < depth and time.time() < deadline:
        time.sleep(0.001)
    assert src.decoded >= depth
    time.sleep(0.05)
    bound = depth + 2 * src.lookahead
    assert src.decoded <= bound, f"decoded {src.decoded} frames ahead with depth {depth}"
    f = src.next()
    assert f.frame_index == 0
    src.release(f)
    src.destroy()


def test_source_poll_never_blocks_and_delivers_in_order(gpu_required):
    data = scene(30)
    src = ebiv.AsyncSource(data, depth=2)
    got, polls = [], 0
    deadline = time.time() + 20
    while time.time() < deadline:
        try:
            f = src.poll()
        except ebiv.EOF:
            break
        polls += 1
        if f is None:
            time.sleep(0.0005)
            continue
        got.append(f.frame_index)
        src.release(f)
    assert got == list(range(30))
    src.destroy()


def test_source_seek_drops_frames_of_the_old_generation(gpu_required):
    # TestAsyncPlayerSeek / TestAsyncPlayerSeekRecyclesDiscardedFrames: after
    # Seek(t) the next frame is the last key frame at or before t, and no frame
    # decoded before the seek comes through.
    data = scene(40, gop=12)
    rd = ebiv.Reader(data)
    want = ebiv_oracle.decode_all([p.data for p in rd.packets()])
    src = ebiv.AsyncSource(data, depth=4)
    for _ in range(5):
        src.release(src.next())
    time.sleep(0.02)  # let the worker run ahead of the seek point
    t = rd.frame_time(27)
    landed = src.seek(t)
    assert landed == rd.frame_time(24)  # key frames every 12
    got = drain_all(src)
    assert [g[0] for g in got] == list(range(24, 40))
    assert [g[2] for g in got] == [sha(want[i][1]) for i in range(24, 40)]
    # backwards, twice in a row (the first seek's frames never surface)
    src.seek(rd.frame_time(13))
    src.seek(0)
    got = drain_all(src)
    assert [g[0] for g in got] == list(range(40))
    assert [g[2] for g in got] == [sha(w[1]) for w in want]
    src.destroy()


def test_source_parks_at_the_end_and_a_seek_revives_it(gpu_required):
    # TestAsyncPlayerSeekAfterEOF
    data = scene(6, gop=6)
    src = ebiv.AsyncSource(data, depth=4)
    assert [g[0] for g in drain_all(src)] == list(range(6))
    with pytest.raises(ebiv.EOF):
        src.next()  # parked: the end is reported again
    with pytest.raises(ebiv.EOF):
        src.poll()
    assert src.seek(0) == 0
    f = src.next()
    assert f.frame_index == 0
    src.release(f)
    src.destroy()


def test_source_error_parks_until_seek(gpu_required):
    # readNextFrame's error (source.go:164-170): the frames before the bad one
    # are delivered, then its error; nothing after it until a seek.
    from test_gpu_batch import _zero_tile

    data = bytearray(scene(20, gop=10))
    pk = [p.data for p in ebiv.Reader(bytes(data)).packets()]
    bad = _zero_tile(pk[13], 1)
    off = bytes(data).find(pk[13])
    assert off > 0 and len(bad) == len(pk[13])
    data[off:off + len(bad)] = bad
    data = bytes(data)
    want = ebiv_oracle.decode_all([p.data for p in ebiv.Reader(data).packets()])
    assert want[13][0] == ebiv.ErrCorrupt.status and all(w[0] == 0 for w in want[:13])
    src = ebiv.AsyncSource(data, depth=8)
    got = []
    with pytest.raises(ebiv.ErrCorrupt):
        while True:
            f = src.next()
            got.append((f.frame_index, sha(f.packed())))
            src.release(f)
    assert got == [(i, sha(want[i][1])) for i in range(13)]
    with pytest.raises(ebiv.ErrCorrupt):
        src.next()
    time.sleep(0.02)
    n = src.decoded
    time.sleep(0.03)
    assert src.decoded == n  # parked: no decoding
    src.seek(ebiv.Reader(data).frame_time(15))  # key frame 10
    f = src.next()
    assert f.frame_index == 10 and sha(f.packed()) == sha(want[10][1])
    src.release(f)
    src.destroy()


def test_source_close_stops_decoding(gpu_required):
    # TestAsyncPlayerCloseStopsDecoding
    data = scene(60)
    src = ebiv.AsyncSource(data, depth=4)
    src.release(src.next())
    src.close()
    after = src.decoded
    time.sleep(0.05)
    assert src.decoded == after
    src.close()  # a second close is fine
    with pytest.raises(ebiv.EOF):
        src.next()
    src.destroy()


def test_source_prepares_rgba_matching_the_oracle(gpu_required):
    # TestAsyncPlayerPreparesRGBAOnDecodeGoroutine with the oracle's
    # convertYCbCr420ToRGBA (frame.go:8-67); odd sizes included.
    for name in ("odd_37x21", "flash_128x96"):
        data = (GOLDEN / f"{name}.ebiv").read_bytes()
        w, h = META[name]["width"], META[name]["height"]
        src = ebiv.AsyncSource(data, depth=4, rgba=True)
        n = 0
        while True:
            try:
                f = src.next()
            except ebiv.EOF:
                break
            assert f.rgba is not None and f.rgba.shape == (h, w, 4)
            want = np.frombuffer(ebiv_oracle.rgba(f.packed(), w, h), np.uint8).reshape(h, w, 4)
            assert np.array_equal(f.rgba, want), f"{name} frame {f.frame_index}"
            src.release(f)
            n += 1
        assert n == len(META[name]["frames"])
        src.destroy()
    plain = ebiv.AsyncSource((GOLDEN / "odd_37x21.ebiv").read_bytes(), depth=4)
    f = plain.next()
    assert f.rgba is None  # TestAsyncPlayerWithoutRGBAOptionDefersConversion
    plain.release(f)
    plain.destroy()


def test_source_recycles_buffers_and_retired_frames_survive_one_change(gpu_required):
    # TestAsyncPlayerRecyclesRGBABuffers / TestAsyncPlayerRetiredFrameSurvivesOneChange,
    # driven the way the Player drives its source (player.go:130-159): current,
    # next and retired frames held, the retired one released at each change.
    data = scene(40)
    want = ebiv_oracle.decode_all([p.data for p in ebiv.Reader(data).packets()])
    src = ebiv.AsyncSource(data, depth=4, rgba=True)
    cur, nxt, retired = src.next(), src.next(), None
    seen, delivered = set(), 0
    while True:
        if retired is not None:
            # the frame displaced one change ago is still intact
            assert sha(retired.packed()) == sha(want[retired.frame_index][1])
            src.release(retired)
        retired, cur = cur, nxt
        try:
            nxt = src.next()
        except ebiv.EOF:
            nxt = None
        seen.add(cur.rgba.ctypes.data)
        delivered += 1
        assert sha(cur.packed()) == sha(want[cur.frame_index][1])
        if nxt is not None:
            assert nxt.rgba.ctypes.data != cur.rgba.ctypes.data
            assert nxt.y.ctypes.data != cur.y.ctypes.data
        else:
            break
    assert len(seen) < delivered, f"no buffer reuse: {len(seen)} buffers for {delivered} frames"
    src.destroy()


def test_source_holding_too_many_frames_is_an_error_not_a_hang(gpu_required):
    # Frames stay valid until released; a consumer that holds so many that no
    # frame can be decoded gets ErrArgument instead of a wait that never ends,
    # and decoding resumes at the next release.
    data = scene(60)
    want = ebiv_oracle.decode_all([p.data for p in ebiv.Reader(data).packets()])
    src = ebiv.AsyncSource(data, depth=2)
    held = []
    with pytest.raises(ebiv.ErrArgument):
        for _ in range(60):
            held.append(src.next())
    assert len(held) >= 2 + src.lookahead + 4
    assert [sha(f.packed()) for f in held] == [sha(want[i][1]) for i in range(len(held))]
    for f in held:
        src.release(f)
    rest = drain_all(src)
    assert [g[0] for g in rest] == list(range(len(held), 60))
    assert [g[2] for g in rest] == [sha(want[i][1]) for i in range(len(held), 60)]
    src.destroy()
