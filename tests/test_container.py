"""Container behaviour (ebiv/container_test.go, ebiv/format_test.go,
ebiv/reader.go): index via the CRC-checked footer, rebuild by scan when the
footer is missing or corrupt, seeks land on governing key frames, exact
frame times for NTSC rates, sticky EOF."""
import pytest

from govid_gb300 import ebiv

from helpers import encode_gen


def _clip(n=10, gop=4, fps=(30, 1)):
    enc = ebiv.Encoder(ebiv.Config(64, 48, fps[0], fps[1]), intra=20, gop=gop)
    for i in range(n):
        enc.write_frame(ebiv.synth_frame(64, 48, i))
    enc.close()
    return enc.output()


def test_header_and_index():
    data = _clip()
    r = ebiv.Reader(data)
    assert (r.width, r.height, r.frame_count) == (64, 48, 10)
    assert not r.rebuilt_index
    assert [e.keyframe for e in r.index()] == [i % 4 == 0 for i in range(10)]
    assert data[:4] == b"EBIV" and data[-4:] == b"EBIX"


def test_packets_in_order_then_sticky_eof():
    r = ebiv.Reader(_clip(5, 5))
    pkts = [r.next_packet() for _ in range(5)]
    assert [p.keyframe for p in pkts] == [True, False, False, False, False]
    assert [p.timestamp_ns for p in pkts] == [r.frame_time(i) for i in range(5)]
    for _ in range(2):
        with pytest.raises(ebiv.EOF):
            r.next_packet()


def test_footerless_file_rebuilds_index():
    data = _clip()
    r = ebiv.Reader(data[:-20])
    assert r.rebuilt_index and r.frame_count == 10


def test_corrupt_index_falls_back_to_scan():
    data = bytearray(_clip())
    data[-30] ^= 0xFF  # inside the index: the CRC no longer matches
    r = ebiv.Reader(bytes(data))
    assert r.rebuilt_index and r.frame_count == 10


def test_truncated_trailing_record_is_dropped():
    data = _clip()
    r0 = ebiv.Reader(data)
    cut = len(data) - 20 - 16 * 10 - 5  # half of the last frame record gone
    r = ebiv.Reader(data[:cut])
    assert r.rebuilt_index and r.frame_count == 9 and r0.frame_count == 10


def test_seek_lands_on_key_frame():
    r = ebiv.Reader(_clip(10, 4))
    t6 = r.frame_time(6)
    assert r.seek(t6) == r.frame_time(4)
    assert r.next_packet().keyframe
    assert r.seek(10**15) == r.frame_time(8)
    assert r.seek(-5) == 0


def test_ntsc_frame_times_are_exact():
    r = ebiv.Reader(_clip(3, 3, (30000, 1001)))
    for i in range(0, 5000, 7):
        t = r.frame_time(i)
        assert t == i * 1001 * 10**9 // 30000
        assert r.frame_index_at(t) == i
        if i:
            assert r.frame_index_at(t - 1) == i - 1


def _hostile_rate(data: bytes) -> bytes:
    """The container with 2^32-1 frames per second (FileHeader FPSNum/FPSDen,
    ebiv/format.go:230-265); the index's CRC does not cover the header."""
    b = bytearray(data)
    b[16:20] = (0xFFFFFFFF).to_bytes(4, "little")
    b[20:24] = (1).to_bytes(4, "little")
    return bytes(b)


def test_seek_with_a_wrapping_frame_rate_is_an_error_not_a_hang():
    # frameIndexAt (ebiv/format.go:263-275) estimates from t*FPSNum in
    # wrapping int64; at 2^32-1 frames per second and t = 2^62 ns the estimate
    # is meaningless and the reference's correction walk would run for ~2^63
    # steps. Here the walk stops at 2^20 steps with an error, as on the GPU.
    r = ebiv.Reader(_hostile_rate(_clip(10, 4)))
    assert r.frame_index_at(1 << 62) == -1
    with pytest.raises(ebiv.ErrCorrupt):
        r.seek(1 << 62)
    assert r.seek(r.frame_time(9)) == r.frame_time(8)  # ordinary seeks still resolve


def with_index(data: bytes, edit) -> bytes:
    """The container with its footer index entries edited in place by
    edit([[offset, size, flags], ...]) and the index CRC recomputed
    (ebiv/reader.go:65-113)."""
    import struct
    import zlib

    b = bytearray(data)
    off, count, _ = struct.unpack_from("<QII", b, len(b) - 20)
    ents = [list(struct.unpack_from("<QII", b, off + 16 * i)) for i in range(count)]
    edit(ents)
    raw = b"".join(struct.pack("<QII", *e) for e in ents)
    b[off:off + 16 * count] = raw
    struct.pack_into("<I", b, len(b) - 8, zlib.crc32(raw) & 0xFFFFFFFF)
    return bytes(b)


def wrapping_entries(data: bytes) -> bytes:
    """Frame 2's offset wraps validateEntry's uint64 sum to position 0, frame
    5's to a negative position."""
    def edit(e):
        e[2][:2] = [2**64 - 8, 40]
        e[5][:2] = [2**64 - 16, 40]
    return with_index(data, edit)


def test_index_entries_whose_offset_wraps():
    # validateEntry (ebiv/reader.go:115-123) sums in uint64, so an offset near
    # 2^64 passes and the reference keeps the index. NextPacket then seeks to
    # int64(Offset)+8 (reader.go:203): position 0 for 2^64-8, so it returns
    # the file's first bytes; a negative position for 2^64-16, so it fails
    # and stays on that frame until a seek.
    import ebiv_container

    bad = wrapping_entries(_clip(10, 4))
    r = ebiv.Reader(bad)
    assert not r.rebuilt_index and r.frame_count == 10
    assert r.packet(2).data == bad[:40]
    with pytest.raises(ebiv.ErrIO):
        r.packet(5)
    got = []
    with pytest.raises(ebiv.ErrIO):
        while True:
            got.append(r.next_packet().data)
    assert len(got) == 5 and got[2] == bad[:40]
    with pytest.raises(ebiv.ErrIO):
        r.next_packet()
    r.seek(r.frame_time(8))
    assert r.next_packet().keyframe
    _, entries, rebuilt = ebiv_container.demux(bad)
    assert not rebuilt and entries[2][0] == 0 and entries[5][0] is None
    with pytest.raises(ebiv_container.ContainerError) as e:
        ebiv_container.packets(bad)
    assert e.value.status == ebiv.ErrIO.status


@pytest.mark.parametrize("bad,err", [(b"", ebiv.ErrBadMagic), (b"XXXX" + bytes(60), ebiv.ErrBadMagic)])
def test_bad_files(bad, err):
    with pytest.raises(err):
        ebiv.Reader(bad)


def test_version_mismatch():
    data = bytearray(_clip())
    data[4] = 9
    with pytest.raises(ebiv.ErrVersion):
        ebiv.Reader(bytes(data))


def test_raw_round_trip_sizes():
    # TestRawRoundTrip sizes, container level (the CPU oracle decodes them)
    import ebiv_oracle

    for w, h in [(64, 48), (1, 1), (65, 49), (37, 21)]:
        cont, srcs, _ = encode_gen(w, h, 2, ebiv.synth_frame)
        pk = [p.data for p in ebiv.Reader(cont).packets()]
        assert [p for _, p in ebiv_oracle.decode_all(pk)] == srcs
