"""Codec error mapping and side effects on the CPU oracle
(ebiv/codec_test.go:123-175): the statuses the GPU path must reproduce."""
import ebiv_oracle
from govid_gb300 import ebiv


def _raw_key(w, h, extra=0):
    hdr = bytes([0 | (0 << 2), w & 255, w >> 8, h & 255, h >> 8, 0])
    return hdr + bytes(ebiv.packed_size(w, h) + extra)


def test_bad_packets():
    c = ebiv_oracle.OracleCodec()
    assert c.decode(b"")[0] == ebiv.ErrCorrupt.status
    c = ebiv_oracle.OracleCodec()
    assert c.decode(bytes([1]))[0] == ebiv.ErrNoKeyframe.status
    c = ebiv_oracle.OracleCodec()
    assert c.decode(bytes([0, 1, 0]))[0] == ebiv.ErrCorrupt.status


def test_wrong_raw_length_and_resolution_change():
    c = ebiv_oracle.OracleCodec()
    assert c.decode(_raw_key(16, 16)[:6])[0] == ebiv.ErrCorrupt.status
    assert c.decode(_raw_key(16, 16, 1))[0] == ebiv.ErrCorrupt.status
    assert c.decode(_raw_key(16, 16))[0] == 0
    assert c.decode(_raw_key(32, 32))[0] == ebiv.ErrDimensions.status


def test_unsupported_features():
    c = ebiv_oracle.OracleCodec()
    assert c.decode(bytes([0, 16, 0, 16, 0, 0x10]))[0] == ebiv.ErrUnsupported.status  # chroma format
    assert c.decode(bytes([0 | (5 << 2), 16, 0, 16, 0, 0]))[0] == ebiv.ErrUnsupported.status  # coding mode
    assert c.decode(bytes([0, 0xFF, 0xFF, 0xFF, 0xFF, 0]))[0] == ebiv.ErrUnsupported.status  # > 8K pixels
