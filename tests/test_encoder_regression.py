"""Encoder gates restated from the reference's tests, checked on the CPU:
exact gate-clip size (ebiv/regression_test.go:15-39), intra quality and size
ceilings (ebiv/coded_test.go:221-261), GOP cadence (336-355), static skip
collapse (267-332), golden flash returns (436-477), scene-cut keys (599-647),
and the encoder's reconstruction equal to the oracle's decode of its output
(the format's core contract, coded_test.go:199-216)."""
import pytest

import ebiv_oracle
from govid_gb300 import ebiv

from helpers import encode_gen, flash_gen, psnr


def _decode_check(cont, recons):
    pkts = [p.data for p in ebiv.Reader(cont).packets()]
    out = ebiv_oracle.decode_all(pkts)
    for i, (st, planes) in enumerate(out):
        assert st == 0, f"frame {i}: oracle status {st}"
        if recons:
            assert planes == recons[i], f"frame {i}: oracle decode differs from the encoder reconstruction"
    return [p for _, p in out]


def test_gate_clip_size_is_pinned():
    cont, _, rec = encode_gen(256, 192, 16, ebiv.synth_pan, intra=18, gop=8, tiles=(2, 2), threads=4)
    assert len(cont) == 54486
    _decode_check(cont, rec)


@pytest.mark.parametrize("qp,min_psnr,max_bytes", [(8, 40, 42000), (20, 30, 28000), (32, 24, 14000)])
def test_intra_quality(qp, min_psnr, max_bytes):
    cont, srcs, rec = encode_gen(256, 192, 4, ebiv.synth_frame, intra=qp)
    dec = _decode_check(cont, rec)
    assert min(psnr(d, s) for d, s in zip(dec, srcs)) >= min_psnr
    assert (len(cont) - 48 - 20) // 4 <= max_bytes


@pytest.mark.parametrize("gop", [1, 2, 3, 5])
def test_gop_cadence(gop):
    cont, _, _ = encode_gen(64, 48, 7, ebiv.synth_frame, intra=20, gop=gop)
    keys = [e.keyframe for e in ebiv.Reader(cont).index()]
    assert keys == [i % gop == 0 for i in range(7)]


def test_static_sequence_collapses_to_skip():
    cont, srcs, rec = encode_gen(256, 192, 10, lambda w, h, i: ebiv.synth_frame(w, h, 0), intra=20, gop=10)
    sizes = [e.size for e in ebiv.Reader(cont).index()]
    assert max(sizes[1:]) * 20 <= sizes[0]
    dec = _decode_check(cont, rec)
    first = psnr(dec[0], srcs[0])
    assert all(psnr(d, s) >= first - 0.5 for d, s in zip(dec, srcs))


def test_golden_flash_returns_are_cheap():
    cont, srcs, rec = encode_gen(128, 96, 9, flash_gen, intra=16, gop=9)
    sizes = [e.size for e in ebiv.Reader(cont).index()]
    for i in range(2, 9, 2):
        assert sizes[i] < sizes[1] / 10
    dec = _decode_check(cont, rec)
    assert all(psnr(d, s) >= 30 for d, s in zip(dec, srcs))


def test_scene_cut_starts_a_gop():
    cut = 12
    cont, _, _ = encode_gen(128, 96, 30, lambda w, h, i: ebiv.synth_frame(w, h, 1 if i < cut else 9), intra=16, gop=20)
    keys = [e.keyframe for e in ebiv.Reader(cont).index()]
    want = [i == 0 or i == cut or (i > cut and (i - cut) % 20 == 0) for i in range(30)]
    assert keys == want
    cont2, _, _ = encode_gen(128, 96, 6, lambda w, h, i: ebiv.synth_frame(w, h, 1 if i < 2 else 9), intra=16, gop=20)
    assert [e.keyframe for e in ebiv.Reader(cont2).index()] == [True] + [False] * 5


def test_parallel_encode_is_deterministic():
    a, _, _ = encode_gen(320, 224, 6, ebiv.synth_frame, intra=18, gop=4, tiles=(4, 4), threads=4, keep_recon=False)
    b, _, _ = encode_gen(320, 224, 6, ebiv.synth_frame, intra=18, gop=4, tiles=(4, 4), threads=1, keep_recon=False)
    assert a == b


def test_sprite_scene_decodes_exactly():
    spec = ebiv.SceneSpec(width=320, height=180, seed=5, sprites=4, flash_period=8, flash_start=4)
    cont = ebiv.encode_scene(spec, 10, qp=22, gop=10, tiles=(2, 2), fast=True, threads=4)
    enc = ebiv.Encoder(ebiv.Config(320, 180), intra=22, gop=10, tiles=(2, 2), fast=True, keep_recon=True)
    sc = ebiv.Scene(spec)
    for i in range(10):
        enc.write_frame(sc.render(i))
    enc.close()
    assert enc.output() == cont
    _decode_check(cont, enc.recons())
