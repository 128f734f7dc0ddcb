"""CPU tests of the content pipeline behind the benchmarks: the GOP-parallel
scene encoder must produce the serial encoder's bytes, the oracle's own
container parser must agree with the product demuxer, and the 64-stream mix
must draw what the workload names."""
import sys
from pathlib import Path

import pytest

from govid_gb300 import ebiv, workloads

sys.path.insert(0, str(Path(__file__).resolve().parent.parent / "oracle"))
import ebiv_container  # noqa: E402

GOLDEN = Path(__file__).resolve().parent / "golden"


@pytest.mark.parametrize("w,h,frames,gop,tiles,alt,flash", [
    (320, 192, 30, 12, (2, 2), 0, None),
    (160, 96, 24, 7, (1, 1), 4, None),
    # +120 luma flashes every 10 frames: scene cuts end GOPs early
    (200, 120, 45, 40, (1, 1), 0, dict(flash_period=10, flash_start=2, flash_amp=120)),
])
def test_gop_parallel_encode_matches_serial(w, h, frames, gop, tiles, alt, flash):
    spec = ebiv.SceneSpec(width=w, height=h, seed=9, sprites=4, **(flash or {}))
    serial = ebiv.encode_scene(spec, frames, qp=22, gop=gop, tiles=tiles, fast=True, threads=1, altref=alt)
    par = ebiv.encode_scene(spec, frames, qp=22, gop=gop, tiles=tiles, fast=True, threads=6, altref=alt)
    assert par == serial
    keys = sum(1 for p in ebiv.Reader(par).packets() if p.keyframe)
    if flash:
        assert keys > (frames + gop - 1) // gop  # the cuts added key frames


@pytest.mark.parametrize("name", ["gate_clip.ebiv", "flash_128x96.ebiv", "altref_64x48.ebiv", "odd_37x21.ebiv"])
def test_oracle_container_parser_matches_reader(name):
    data = (GOLDEN / name).read_bytes()
    want = [p.data for p in ebiv.Reader(data).packets()]
    assert ebiv_container.packets(data) == want
    # a damaged footer: both rebuild the index by scanning the frame records
    assert ebiv_container.packets(data[:-1]) == [p.data for p in ebiv.Reader(data[:-1]).packets()]
    assert [ebiv_container.frame_type(p) for p in want] == [ebiv.parse_frame_header(p)["type"] for p in want]


def test_mix_draws():
    mix = workloads.mix()
    assert len(mix) == 64
    assert [(c.w, c.h) for c in mix].count((640, 360)) == 24
    assert [(c.w, c.h) for c in mix].count((1280, 720)) == 24
    assert [(c.w, c.h) for c in mix].count((1920, 1080)) == 16
    assert len({c.seed for c in mix}) == 64
    assert {c.grid for c in mix} == {(1, 1), (2, 2), (4, 3)}
    assert {c.qp for c in mix} == {18, 22, 28}
    assert all(30 <= c.gop <= 120 and c.frames == 120 for c in mix)
    assert len({c.key() for c in mix}) == 64
    srv = workloads.serve()
    assert all(c.frames == 600 for c in srv) and len({c.key() for c in srv}) == len(srv)
