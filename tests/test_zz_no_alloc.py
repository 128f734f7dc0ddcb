"""ebivgpu_decode_key_noalloc (include/ebivgpu.h): key frames decoded with
all scratch in a static device array equal the stateful codec's first frame
(ebivgpu_decode on a new codec) and the oracle, for two different streams
decoded back to back through the one scratch, including an alt-ref key packet
whose golden override is checked too, and a frame at the limits (3600
macroblocks, 3600 tiles per payload, a packet near 2 MiB).  Size limits are
refused with their own status before any device work.

This file is named to be collected last: the entry point's first call on a
device does its setup, and it must work after every other test has run."""
import ctypes as C
from pathlib import Path

import numpy as np
import pytest

import ebiv_oracle
from govid_gb300 import _native, ebiv

GOLDEN = Path(__file__).resolve().parent / "golden"
EBIV_ERR_CORRUPT, EBIV_ERR_NOKEYFRAME, EBIV_ERR_UNSUPPORTED, EBIV_ERR_ARG, EBIV_ERR_TOO_LARGE = 1, 2, 4, 12, 13
KEY = 0  # frame type of a key frame (ebiv/format.go)


def _packets(name):
    return [p.data for p in ebiv.Reader((GOLDEN / f"{name}.ebiv").read_bytes()).packets()]


def _dims(pkt):
    w, h = C.c_int32(), C.c_int32()
    st = _native.lib().ebivgpu_decode_key_noalloc(pkt, len(pkt), None, 0, 0, None, None, 0, 0, None,
                                                  C.byref(w), C.byref(h))
    return st, w.value, h.value


def _noalloc(pkt):
    """Decode into caller-owned device planes (torch memory, pre-filled with
    garbage) and return (status, packed visible planes)."""
    import torch

    st, w, h = _dims(pkt)
    assert st == 0
    mbc, mbr = (w + 15) // 16, (h + 15) // 16
    ys, cs = mbc * 16 + 32, mbc * 8 + 16  # strides wider than required
    yp = torch.full((mbr * 16 * ys,), 0xAB, dtype=torch.uint8, device="cuda")
    cbp = torch.full((mbr * 8 * cs,), 0xCD, dtype=torch.uint8, device="cuda")
    crp = torch.full((mbr * 8 * cs,), 0xEF, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    ow, oh = C.c_int32(), C.c_int32()
    st = _native.lib().ebivgpu_decode_key_noalloc(pkt, len(pkt), yp.data_ptr(), ys, yp.numel(), cbp.data_ptr(),
                                                  crp.data_ptr(), cs, cbp.numel(), None, C.byref(ow), C.byref(oh))
    if st:
        return st, None
    assert (ow.value, oh.value) == (w, h)
    cw, ch = (w + 1) // 2, (h + 1) // 2
    y = yp.cpu().numpy().reshape(mbr * 16, ys)[:h, :w]
    cb = cbp.cpu().numpy().reshape(mbr * 8, cs)[:ch, :cw]
    cr = crp.cpu().numpy().reshape(mbr * 8, cs)[:ch, :cw]
    return 0, np.ascontiguousarray(y).tobytes() + np.ascontiguousarray(cb).tobytes() + np.ascontiguousarray(cr).tobytes()


def _codec_first(pkt):
    c = ebiv.Codec()
    try:
        return 0, c.decode(pkt).packed()
    except ebiv.EbivError as e:
        return e.status, None
    finally:
        c.close()


@pytest.mark.gpu
def test_two_calls_in_a_row_match_the_stateful_codec(gpu_required):
    # Two streams of different sizes and tilings back to back through the
    # one scratch, then the first again.
    a = _packets("scene_160x96")[0]
    b = _packets("odd_37x21")[0]
    want = {k: _codec_first(p) for k, p in (("a", a), ("b", b))}
    assert want["a"][0] == 0 and want["b"][0] == 0
    for k, p in (("a", a), ("b", b), ("a", a)):
        st, got = _noalloc(p)
        assert st == 0 and got == want[k][1], f"stream {k}"
        assert got == ebiv_oracle.decode_all([p])[0][1]


@pytest.mark.gpu
def test_altref_key_packet_and_its_override_status(gpu_required):
    pk = _packets("altref_64x48")
    keys = [p for p in pk if ebiv.parse_frame_header(p)["golden_override"]]
    assert keys, "fixture carries an alt-ref key packet"
    p = keys[0]
    assert _noalloc(p) == _codec_first(p)
    # A damaged override payload: the key still decodes, the override's
    # status decides the result, the same in both entry points.
    bad = bytearray(p)
    for i in range(len(bad) - 6, len(bad)):
        bad[i] ^= 0x5A
    bad = bytes(bad)
    got, want = _noalloc(bad), _codec_first(bad)
    assert got[0] == want[0]
    assert got == want


@pytest.mark.gpu
def test_consecutive_key_frames_of_one_stream(gpu_required):
    cont = ebiv.encode_scene(ebiv.SceneSpec(width=96, height=64, seed=9, sprites=2), 9, qp=24, gop=3, tiles=(2, 2),
                             fast=True)
    keys = [p.data for p in ebiv.Reader(cont).packets() if ebiv.parse_frame_header(p.data)["type"] == KEY]
    assert len(keys) >= 2
    for p in keys:
        st, got = _noalloc(p)
        assert (st, got) == _codec_first(p)


@pytest.mark.gpu
def test_at_the_limits_3600_macroblocks_3600_tiles_near_2mib(gpu_required):
    # The far end of every scratch region: a 1280x720 key frame (exactly the
    # 3600-macroblock limit) coded as 80x45 one-macroblock tiles at q2, with an
    # alt-ref override payload (its own 3600 tiles), in one 1.86 MB packet.
    from helpers import encode_gen, noisy_gen

    cont, _, _ = encode_gen(1280, 720, 8, noisy_gen, intra=2, gop=8, altref=4, tiles=(80, 45), threads=8,
                            keep_recon=False, fast=True)
    p = next(iter(ebiv.Reader(cont).packets())).data
    hdr = ebiv.parse_frame_header(p)
    assert hdr["golden_override"] and (hdr["width"], hdr["height"]) == (1280, 720)
    assert 1_700_000 < len(p) <= 2 << 20
    want = _codec_first(p)
    assert want[0] == 0 and want[1] == ebiv_oracle.decode_all([p])[0][1]
    for _ in range(2):  # two calls in a row through the one scratch
        assert _noalloc(p) == want


def test_size_limits_and_frame_types_are_refused_before_device_work():
    # No GPU needed: each refusal happens on the host.
    big = ebiv.encode_scene(ebiv.SceneSpec(width=1296, height=720, seed=1, sprites=1), 1, qp=40, gop=1,
                            tiles=(1, 1), fast=True)
    big_key = next(iter(ebiv.Reader(big).packets())).data  # 81 x 45 = 3645 macroblocks
    assert _dims(big_key)[0] == EBIV_ERR_TOO_LARGE
    ok_key = _packets("scene_160x96")[0]
    assert _dims(ok_key) == (0, 160, 96)
    inter = _packets("scene_160x96")[1]
    assert _dims(inter)[0] == EBIV_ERR_NOKEYFRAME
    assert _dims(b"")[0] == EBIV_ERR_CORRUPT
    assert b"no-allocation" in _native.lib().ebivgpu_status_string(EBIV_ERR_TOO_LARGE)
