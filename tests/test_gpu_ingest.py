"""Container ingest on the GPU (ebivgpu_container_*): the device-built frame
index and seeks equal the host demuxer's (ebiv.Reader, a restatement of
ebiv/reader.go:32-238) on the reference-shaped fixtures, with the footer
intact, damaged (the index rebuilt by scanning the frame records) and
truncated; a batch stream decoding in place from the pinned container is
bit-exact against the oracle."""
import hashlib
from pathlib import Path

import pytest

import ebiv_oracle
from govid_gb300 import ebiv, workloads

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"
NAMES = ["gate_clip.ebiv", "flash_128x96.ebiv", "altref_64x48.ebiv", "odd_37x21.ebiv", "scene_160x96.ebiv"]


def _variants(data: bytes):
    yield "intact", data
    yield "footer magic damaged", data[:-1] + bytes([data[-1] ^ 0xFF])
    b = bytearray(data)
    b[-8] ^= 0x01  # the index CRC
    yield "index crc damaged", bytes(b)
    yield "truncated", data[: len(data) - 30]


def _same_index(dc, r, data):
    assert dc.frame_count == r.frame_count
    assert dc.rebuilt_index == r.rebuilt_index
    for i in range(r.frame_count):
        off, n, key = dc.entry(i)
        p = r.packet(i)
        assert key == p.keyframe and n == len(p.data)
        assert data[off:off + n] == p.data


@pytest.mark.parametrize("name", NAMES)
def test_device_index_and_seek_match_the_host_demuxer(gpu_required, name):
    for what, data in _variants((GOLDEN / name).read_bytes()):
        r = ebiv.Reader(data)
        dc = ebiv.DeviceContainer(data)
        _same_index(dc, r, data)
        period = 1_000_000_000 * r.fps_den // r.fps_num
        for t in [-5, 0, 1, period - 1, period, period + 1, 3 * period + 7, 10**12] + \
                 [k * period // 3 for k in range(3 * r.frame_count + 3)]:
            landed = r.seek(t)
            frame, dl = dc.seek(t)
            assert dl == landed, f"{name} {what} t={t}"
            assert frame == r.frame_index_at(landed)


def test_device_seek_with_a_wrapping_frame_rate_is_an_error(gpu_required):
    # The device seek caps frameIndexAt's correction walk exactly as the host
    # demuxer does: the same hostile frame rate is an error on both, and
    # ordinary seeks on that file land on the same frame.
    from test_container import _clip, _hostile_rate

    data = _hostile_rate(_clip(10, 4))
    r = ebiv.Reader(data)
    dc = ebiv.DeviceContainer(data)
    with pytest.raises(ebiv.ErrCorrupt):
        dc.seek(1 << 62)
    with pytest.raises(ebiv.ErrCorrupt):
        r.seek(1 << 62)
    for t in [-1, 0, 1, 2, 3, 10**9]:
        landed = r.seek(t)
        frame, dl = dc.seek(t)
        assert dl == landed, f"t={t}"


def test_device_index_keeps_wrapping_entries_and_never_reads_outside(gpu_required):
    # The device-built index keeps the entries whose offsets wrap
    # validateEntry's uint64 sum, as the reference and the host demuxer do
    # (ebiv/reader.go:115-123): the one that lands at position 0 reads the
    # file's first bytes, the one that lands at a negative position is an I/O
    # error, and an in-place stream over the file is refused before any
    # packet is read.
    from test_container import _clip, wrapping_entries

    bad = wrapping_entries(_clip(10, 4))
    r = ebiv.Reader(bad)
    dc = ebiv.DeviceContainer(bad)
    assert dc.frame_count == r.frame_count == 10 and not dc.rebuilt_index
    off, n, key = dc.entry(2)
    assert (off, n) == (0, 40) and bad[off:off + n] == r.packet(2).data
    with pytest.raises(ebiv.ErrIO):
        dc.entry(5)
    for i in (0, 1, 3, 4, 6, 7, 8, 9):
        off, n, key = dc.entry(i)
        assert bad[off:off + n] == r.packet(i).data and key == r.packet(i).keyframe
    b = ebiv.Batch(lookahead=2)
    with pytest.raises(ebiv.ErrIO):
        b.add_container(dc)
    b.close()


def test_batch_decodes_in_place_from_the_container(gpu_required):
    clip = workloads.single_640()
    data = workloads.load([clip], in_child=False)[0]
    pk = [p.data for p in ebiv.Reader(data).packets()]
    want = [hashlib.sha256(pl).hexdigest() for _, pl in ebiv_oracle.decode_all(pk)]
    dc = ebiv.DeviceContainer(data)
    for depth in (0, 2):
        b = ebiv.Batch(lookahead=8, pipeline=depth)
        sid = b.add_container(dc)
        got = {}
        empty = 0
        while empty < b.depth + 1:
            res = b.round()
            empty = empty + 1 if not res else 0
            for x in res:
                assert x.status == 0
                got[x.frame_index] = hashlib.sha256(b.download(x, clip.w, clip.h)).hexdigest()
        for x in b.drain():
            got[x.frame_index] = hashlib.sha256(b.download(x, clip.w, clip.h)).hexdigest()
        assert [got[i] for i in range(len(pk))] == want
        b.seek(sid, 0)
        b.close()
