"""GPU decode parity: every plane of every frame bit-exact against the CPU
oracle (the restated pure-Go decoder) on the same bitstreams.

Clip shapes and options restate the reference's own decode tests
(ebiv/coded_test.go, ebiv/tile_test.go, ebiv/regression_test.go,
ebiv/codec_test.go) plus the sprite-scene workloads' shapes at small sizes.
"""
import numpy as np
import pytest

import ebiv_oracle
from govid_gb300 import ebiv

from helpers import encode_gen, first_diff, flash_gen, gpu_decode_all, noisy_gen

pytestmark = pytest.mark.gpu


def _check(container: bytes, w: int, h: int, recons=None):
    pkts = [p.data for p in ebiv.Reader(container).packets()]
    want = ebiv_oracle.decode_all(pkts)
    got = gpu_decode_all(pkts)
    assert len(got) == len(want)
    for i, ((gs, gp), (ws, wp)) in enumerate(zip(got, want)):
        assert gs == ws, f"frame {i}: status {gs} vs oracle {ws}"
        if ws == 0:
            assert gp == wp, f"frame {i}: {first_diff(gp, wp, w, h)}"
            if recons is not None and i < len(recons):
                assert wp == recons[i], f"frame {i}: oracle differs from encoder reconstruction"
    return got


def test_intra_deterministic(gpu_required):
    # TestIntraDeterministic: 96x64, 3 intra frames at qp 16
    cont, _, rec = encode_gen(96, 64, 3, ebiv.synth_frame, intra=16)
    _check(cont, 96, 64, rec)


@pytest.mark.parametrize("qp", [8, 20, 32])
def test_intra_quality_clips(gpu_required, qp):
    # TestIntraQuality clips: 256x192, 4 frames
    cont, _, rec = encode_gen(256, 192, 4, ebiv.synth_frame, intra=qp)
    _check(cont, 256, 192, rec)


def test_inter_pan(gpu_required):
    # TestInterCompressesMotion: 192x128 synthPan, 8 frames, gop 8
    cont, _, rec = encode_gen(192, 128, 8, ebiv.synth_pan, intra=20, gop=8)
    _check(cont, 192, 128, rec)


def test_gate_clip(gpu_required):
    # regressionClip: 256x192 synthPan, 16 frames, q18 gop8 tiles 2x2, two-pass
    cont, _, rec = encode_gen(256, 192, 16, ebiv.synth_pan, intra=18, gop=8, tiles=(2, 2), threads=4)
    assert len(cont) == 54486
    _check(cont, 256, 192, rec)


@pytest.mark.parametrize("grid", [(1, 1), (2, 1), (2, 2), (4, 3)])
def test_tiling_grids(gpu_required, grid):
    # TestTilingDifferential: 256x160, 3 frames, q18 gop3
    cont, _, rec = encode_gen(256, 160, 3, ebiv.synth_frame, intra=18, gop=3, tiles=grid)
    _check(cont, 256, 160, rec)


@pytest.mark.parametrize("split", [(10, 8, 4, 4), (5, 5, 8, 8), (1, 1, 2, 2)])
def test_tile_grids_larger_than_the_frame(gpu_required, split):
    # TestTileGridSplit's shapes (ebiv/tile_test.go:12-45): grids clamp to the
    # macroblock grid; a header asking for more tiles than that is corrupt on
    # the GPU exactly where the oracle says so (ebiv/decode_intra.go:60-63).
    from test_oracle_known_answers import _with_tile_counts

    mbc, mbr, cols, rows = split
    w, h = 16 * mbc, 16 * mbr
    cont, _, rec = encode_gen(w, h, 3, ebiv.synth_pan, intra=20, gop=3, tiles=(cols, rows))
    _check(cont, w, h, rec)
    pkts = [p.data for p in ebiv.Reader(cont).packets()]
    over = [_with_tile_counts(p, min(cols, mbc) + 1, min(rows, mbr)) for p in pkts]
    want = ebiv_oracle.decode_all(over)
    got = gpu_decode_all(over)
    assert [g[0] for g in got] == [x[0] for x in want]
    assert want[0][0] == ebiv.ErrCorrupt.status


def test_golden_flash(gpu_required):
    # TestGoldenRefFlashingSequence: 128x96, 9 frames, q16, gop 9
    cont, _, rec = encode_gen(128, 96, 9, flash_gen, intra=16, gop=9)
    _check(cont, 128, 96, rec)


def test_altref_override(gpu_required):
    # TestAltRefGoldenOverride: 128x96 noisy hold, 24 frames, gop 24, alt-ref 8
    cont, _, rec = encode_gen(128, 96, 24, noisy_gen, intra=16, gop=24, altref=8)
    hdr = ebiv.parse_frame_header(ebiv.Reader(cont).packet(0).data)
    assert hdr["golden_override"]
    _check(cont, 128, 96, rec)


@pytest.mark.parametrize("size", [(65, 49), (37, 21), (1, 1), (17, 33)])
def test_odd_sizes(gpu_required, size):
    # TestCodedOddSizes-style: partial macroblocks at the right/bottom edges
    w, h = size
    cont, _, rec = encode_gen(w, h, 4, ebiv.synth_pan, intra=20, gop=4)
    _check(cont, w, h, rec)


@pytest.mark.parametrize("size", [(16, 16), (17, 15), (64, 48), (31, 47), (160, 90)])
def test_coded_round_trip_sizes(gpu_required, size):
    # TestCodedRoundTripSizes: q16, gop 3, 3 frames
    w, h = size
    cont, _, rec = encode_gen(w, h, 3, ebiv.synth_frame, intra=16, gop=3)
    _check(cont, w, h, rec)


def test_scene_cut_clip(gpu_required):
    # TestSceneCutKeyframes: 128x96, 30 frames, a hard cut at 12, gop 20 (key
    # frames at 0 and 12; the next one would be frame 32)
    cut = 12
    cont, _, rec = encode_gen(128, 96, 30, lambda w, h, i: ebiv.synth_frame(w, h, 1 if i < cut else 9),
                              intra=16, gop=20)
    assert [e.keyframe for e in ebiv.Reader(cont).index()].count(True) == 2
    _check(cont, 128, 96, rec)


def test_raw_frames(gpu_required):
    # TestRawRoundTrip: lossless raw key frames decode to the source
    cont, srcs, _ = encode_gen(64, 48, 3, ebiv.synth_frame)
    got = _check(cont, 64, 48)
    assert [g[1] for g in got] == srcs


def test_sprite_scene_640x360(gpu_required):
    # The single-stream workload's shape: 640x360 sprites, q22, 2x2 tiles
    spec = ebiv.SceneSpec(width=640, height=360, seed=7, sprites=6)
    cont = ebiv.encode_scene(spec, 10, qp=22, gop=60, tiles=(2, 2), fast=True, threads=4)
    _check(cont, 640, 360)


def test_fast_encode_scene_flash(gpu_required):
    spec = ebiv.SceneSpec(width=320, height=192, seed=3, sprites=4, flash_period=8, flash_start=3)
    cont = ebiv.encode_scene(spec, 16, qp=22, gop=16, tiles=(4, 3), fast=True, threads=4)
    _check(cont, 320, 192)


def _wide_levels(w, h, seed, dense):
    """Levels for ebiv.encode_key_from_levels: even macroblocks get escape
    levels near the grammar's largest (their residuals leave the 16-bit range;
    with `dense`, every coefficient is huge, so the transform's int32
    narrowing wraps), odd ones small levels."""
    rng = np.random.default_rng(seed)
    mbs = ((w + 15) // 16) * ((h + 15) // 16)
    lv = np.zeros((mbs, 384), np.int32)
    for m in range(mbs):
        if m % 2 == 0:
            n = 16 if dense else 2
            for b in range(16):
                lv[m, b * 16:b * 16 + n] = rng.choice([-1, 1], n) * rng.integers(20000, 32773, n)
            lv[m, 256:256 + (64 if dense else 1)] = 32772
            lv[m, 320] = -30000
        else:
            for b in range(16):
                lv[m, b * 16 + rng.integers(0, 16)] = rng.integers(-3, 4)
    return lv


@pytest.mark.parametrize("qp,dense", [(22, False), (51, False), (63, True), (40, True)])
def test_hostile_wide_residuals_match_oracle(gpu_required, qp, dense):
    # Residuals beyond 16 bits (only crafted streams have them) take the
    # reconstruction's int32 path between the residual and intra stages;
    # macroblocks with small residuals in the same frame take the 16-bit one.
    w, h = 80, 48
    pkts = [ebiv.encode_key_from_levels(w, h, qp, mode, _wide_levels(w, h, 7 + mode, dense)) for mode in range(4)]
    ebiv_oracle.wide_residuals(True)
    want = ebiv_oracle.decode_all(pkts)
    assert all(st == 0 for st, _ in want)
    assert ebiv_oracle.wide_residuals() > 0
    got = gpu_decode_all(pkts)
    for i, ((gs, gp), (ws, wp)) in enumerate(zip(got, want)):
        assert gs == ws and gp == wp, f"frame {i}: {first_diff(gp, wp, w, h) if gp and wp else (gs, ws)}"
    b = ebiv.Batch(lookahead=4, pipeline=2)
    sid = b.add_stream(pkts)
    res = []
    for _ in range(len(pkts) + 8):  # every frame is back after depth + frames rounds
        res += [(x.frame_index, x.status, b.download(x, w, h)) for x in b.round()]
    res += [(x.frame_index, x.status, b.download(x, w, h)) for x in b.drain()]
    assert sorted((i, s, p) for i, s, p in res) == [(i, 0, want[i][1]) for i in range(len(pkts))]
