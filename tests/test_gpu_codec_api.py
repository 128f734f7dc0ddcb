"""The reference-facing C-ABI codec (include/ebivgpu.h) against the
ebiv.Codec contract (ebiv/codec.go:70-192): error statuses, ring cursor and
Flush, RGBA conversion (frame.go:8-67), and side effects of failing frames,
each checked against the CPU oracle."""
import numpy as np
import pytest

import ebiv_oracle
from govid_gb300 import ebiv

from helpers import encode_gen, noisy_gen
from test_gpu_batch import _zero_tile

pytestmark = pytest.mark.gpu


def _raw_key(w, h, extra=0):
    return bytes([0, w & 255, w >> 8, h & 255, h >> 8, 0]) + bytes(ebiv.packed_size(w, h) + extra)


def _status(codec, pkt):
    try:
        codec.decode(pkt)
        return 0
    except ebiv.EbivError as e:
        return e.status


@pytest.mark.parametrize("w,h,cw,ch,ys,cs", [(64, 48, 32, 24, 64, 64), (1920, 1080, 960, 540, 1920, 960),
                                             (65, 49, 33, 25, 128, 64), (1, 1, 1, 1, 64, 64)])
def test_frame_geometry_matches_the_reference_table(gpu_required, w, h, cw, ch, ys, cs):
    # TestGeometry (ebiv/format_test.go:188-219): the chroma sizes and the
    # 64-byte-aligned strides of the frames the Codec returns, and a raw key
    # frame's bytes round-trip.
    rng = np.random.default_rng(7 * w + h)
    body = rng.integers(0, 256, w * h + 2 * cw * ch, dtype=np.uint8).tobytes()
    assert len(body) == ebiv.packed_size(w, h)
    f = ebiv.Codec().decode(_raw_key(w, h)[:6] + body)
    assert (f.width, f.height) == (w, h)
    assert f.y.shape == (h, ys) and f.cb.shape == (ch, cs) and f.cr.shape == (ch, cs)
    assert f.packed() == body


def test_bad_packets(gpu_required):
    assert _status(ebiv.Codec(), b"") == ebiv.ErrCorrupt.status
    assert _status(ebiv.Codec(), bytes([1])) == ebiv.ErrNoKeyframe.status
    assert _status(ebiv.Codec(), bytes([0, 1, 0])) == ebiv.ErrCorrupt.status
    c = ebiv.Codec()
    assert _status(c, _raw_key(16, 16)[:6]) == ebiv.ErrCorrupt.status
    assert _status(c, _raw_key(16, 16, 1)) == ebiv.ErrCorrupt.status
    assert _status(c, _raw_key(16, 16)) == 0
    assert _status(c, _raw_key(32, 32)) == ebiv.ErrDimensions.status
    assert _status(ebiv.Codec(), bytes([0, 16, 0, 16, 0, 0x10])) == ebiv.ErrUnsupported.status
    assert _status(ebiv.Codec(), bytes([0 | (5 << 2), 16, 0, 16, 0, 0])) == ebiv.ErrUnsupported.status


def test_ring_cursor_and_flush(gpu_required):
    cont, _, _ = encode_gen(64, 48, 6, ebiv.synth_frame, intra=20, gop=3)
    pk = [p.data for p in ebiv.Reader(cont).packets()]
    c = ebiv.Codec(3)
    slots = [c.decode(p).ring_slot for p in pk[:4]]
    assert slots == [0, 1, 2, 0]
    c.flush()
    assert c.decode(pk[3]).ring_slot == 0  # pk[3] is a key frame


def test_rgba_matches_oracle(gpu_required):
    spec = ebiv.SceneSpec(width=97, height=55, seed=4, sprites=2)
    cont = ebiv.encode_scene(spec, 2, qp=22, gop=2, tiles=(1, 1), fast=True)
    pk = [p.data for p in ebiv.Reader(cont).packets()]
    c = ebiv.Codec()
    for p in pk:
        f = c.decode(p)
        want = np.frombuffer(ebiv_oracle.rgba(f.packed(), 97, 55), np.uint8).reshape(55, 97, 4)
        got = f.rgba()
        assert (got == want).all()
        assert (got[..., 3] == 255).all()


def test_with_rgba_pooled_matches_oracle_and_lives_as_long_as_the_frame(gpu_required):
    # WithRGBA (source.go:61-74): the decode round converts each frame on the
    # GPU into a per-slot pooled buffer; odd sizes exercise the last chroma column.
    spec = ebiv.SceneSpec(width=97, height=55, seed=6, sprites=3)
    cont = ebiv.encode_scene(spec, 7, qp=22, gop=4, tiles=(2, 1), fast=True)
    pk = [p.data for p in ebiv.Reader(cont).packets()]
    c = ebiv.Codec(3)
    f0 = c.decode(pk[0])
    assert c.pooled_rgba(f0) is None  # decoded before WithRGBA
    c.with_rgba(True)
    frames, want = [], []
    for p in pk[1:]:
        f = c.decode(p)
        frames.append(f)
        want.append(np.frombuffer(ebiv_oracle.rgba(f.packed(), 97, 55), np.uint8).reshape(55, 97, 4))
        # every frame still inside its ring lifetime keeps its own RGBA
        for g, w in list(zip(frames, want))[-3:]:
            got = c.pooled_rgba(g)
            assert got is not None and (got == w).all()
    c.with_rgba(False)
    f = c.decode(pk[4])  # a key frame (gop 4): decodable out of order
    assert c.pooled_rgba(f) is None


def _zero_override_tile(pkt: bytes, tile: int) -> bytes:
    """Zeroes one tile of a key packet's golden-override payload."""
    b = bytearray(pkt)
    pos = 6

    def uvar(p):
        x, s = 0, 0
        while True:
            c = b[p]
            x |= (c & 0x7F) << s
            p += 1
            if c < 0x80:
                return x, p
            s += 7

    keylen, pos = uvar(pos)
    ov = pos + keylen
    head = bytes([0x01 | (2 << 2)]) + bytes(b[ov:])  # decode the override body as an inter packet
    zeroed = _zero_tile(head, tile)
    return bytes(b[:ov]) + zeroed[1:]


def test_failed_override_leaves_partial_golden(gpu_required):
    cont, _, _ = encode_gen(64, 48, 10, noisy_gen, intra=16, gop=10, altref=4)
    pk = [p.data for p in ebiv.Reader(cont).packets()]
    assert ebiv.parse_frame_header(pk[0])["golden_override"]
    bad = list(pk)
    bad[0] = _zero_override_tile(pk[0], 0)
    # a second, clean key with the same geometry restarts from a known state
    seq = bad + pk
    want = ebiv_oracle.decode_all(seq)
    assert want[0][0] == ebiv.ErrCorrupt.status
    c = ebiv.Codec()
    for i, p in enumerate(seq):
        try:
            got = (0, c.decode(p).packed())
        except ebiv.EbivError as e:
            got = (e.status, None)
        assert got[0] == want[i][0], f"frame {i}"
        assert got[1] == want[i][1], f"frame {i} differs from the oracle"


def test_failed_inter_frame_keeps_references(gpu_required):
    spec = ebiv.SceneSpec(width=160, height=96, seed=8, sprites=3)
    cont = ebiv.encode_scene(spec, 8, qp=22, gop=8, tiles=(2, 1), fast=True)
    pk = [p.data for p in ebiv.Reader(cont).packets()]
    pk[2] = _zero_tile(pk[2], 0)
    want = ebiv_oracle.decode_all(pk)
    c = ebiv.Codec()
    for i, p in enumerate(pk):
        try:
            got = (0, c.decode(p).packed())
        except ebiv.EbivError as e:
            got = (e.status, None)
        assert got == want[i], f"frame {i}"
