"""Serving loop (include/ebivgpu.h, ebivgpu_server_*): requests from many
streams arriving at 30/60 fps are batched continuously; every delivered
frame is bit-identical to the same frame decoded from that stream alone
(the CPU oracle), including after seeks and loops; admission respects the
HBM budget."""
import pytest

import ebiv_oracle
from govid_gb300 import ebiv

pytestmark = pytest.mark.gpu


def _streams():
    out = []
    for k, ((w, h), tiles, gop) in enumerate([((160, 96), (1, 1), 4), ((128, 80), (2, 2), 5), ((96, 64), (2, 1), 3),
                                               ((160, 96), (4, 3), 6), ((64, 48), (1, 1), 4), ((200, 120), (2, 2), 8)]):
        spec = ebiv.SceneSpec(width=w, height=h, seed=40 + k, sprites=2)
        cont = ebiv.encode_scene(spec, 16, qp=22, gop=gop, tiles=tiles, fast=True)
        out.append(([p.data for p in ebiv.Reader(cont).packets()], w, h))
    return out


@pytest.mark.parametrize("lanes,side,long_key,cache", [(1, 1, 0, 0), (3, 1, 20, 0), (1, 3, 20, 0), (1, 2, 20, 1),
                                                        (2, 2, 20, 2), (1, 3, 0, 3)])
def test_mix_equals_alone_with_seeks_and_loops(gpu_required, lanes, side, long_key, cache):
    # long_key 20: every stream's key frames (tiles of more than 20
    # macroblocks for most of them) take the side lanes; with cache 1 those
    # streams reinstall key frames they decoded before, with 2 they decode
    # all of them at admission.
    streams = _streams()
    srv = ebiv.Server(duration_s=1.5, frames_per_stream=40, seek_prob=0.1, seed=3, record=True,
                      max_frames_per_round=3, decode_lanes=lanes, key_lane=side, long_key_mbs=long_key,
                      key_cache=cache)
    for i, (pk, w, h) in enumerate(streams):
        srv.add_stream(pk, fps=60 if i % 2 else 30, loop=(i % 3 == 0))
    st = srv.run()
    assert st["errors"] == 0 and st["frames"] > 0 and st["seeks"] > 0
    alone = [[ebiv.frame_hash(p) for _, p in ebiv_oracle.decode_all(pk)] for pk, _, _ in streams]
    seen = srv.frame_hashes()
    assert len(seen) == st["frames"]
    for s, f, h in seen:
        assert h == alone[s][f], f"stream {s} frame {f} differs in the mix"
    assert st["admitted_total"] == len(streams)
    if cache:
        assert st["key_installs"] > 0
    if cache == 2:
        assert st["warmed_streams"] == 2  # the two streams whose tiles exceed 20 macroblocks
    if cache == 3:
        assert st["warmed_streams"] == len(streams) and st["prepare_s"] > 0


def test_admission_respects_hbm_budget(gpu_required):
    # four streams of one size; the budget holds two footprints plus their
    # packets (the slack, half a footprint, is far above 16 small packets)
    s0 = _streams()[0]
    streams = [s0] * 4
    probe = ebiv.Server(max_frames_per_round=2)
    fp = probe.stream_footprint(s0[1], s0[2], s0[0])
    assert fp > ebiv.stream_footprint(s0[1], s0[2], 3, 2)
    srv = ebiv.Server(duration_s=0.6, frames_per_stream=10, seek_prob=0.0, seed=5, hbm_budget_bytes=2 * fp + fp // 2,
                      max_frames_per_round=2)
    for pk, w, h in streams:
        srv.add_stream(pk, fps=60, loop=False)
    st = srv.run()
    assert st["admitted_peak"] == 2 and st["peak_bytes"] <= 2 * fp + fp // 2
    assert st["admitted_total"] == 4 and st["errors"] == 0


def test_decode_ahead_serves_requests_from_ready_frames(gpu_required):
    # Under a light load every stream is kept ahead of its requests, so most
    # requests find their frame already decoded; seeks restart decoding at
    # their key frame and the frames that follow match the stream alone.
    streams = _streams()
    srv = ebiv.Server(duration_s=1.0, frames_per_stream=30, seek_prob=0.05, seed=11, record=True,
                      max_frames_per_round=2, decode_ahead=6)
    for i, (pk, w, h) in enumerate(streams):
        srv.add_stream(pk, fps=30, loop=True)
    st = srv.run()
    assert st["errors"] == 0 and st["frames"] > 0
    assert st["ready_at_arrival"] >= st["frames"] // 2, st
    assert st["frames"] + st["unserved"] == st["requests"]
    alone = [[ebiv.frame_hash(p) for _, p in ebiv_oracle.decode_all(pk)] for pk, _, _ in streams]
    for s, f, h in srv.frame_hashes():
        assert h == alone[s][f]


def test_stream_larger_than_the_budget_is_never_admitted(gpu_required):
    s0 = _streams()[0]
    srv = ebiv.Server(duration_s=0.3, frames_per_stream=10, seed=2, hbm_budget_bytes=64 << 10,
                      max_frames_per_round=2)
    srv.add_stream(s0[0], fps=60)
    st = srv.run()
    assert st["admitted_total"] == 0 and st["waiting_at_end"] == 1 and st["frames"] == 0
