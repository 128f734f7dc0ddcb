"""Argument and container errors of the decode-ahead source, which it
reports before touching a GPU (so they run on CPU): govid's
TestAsyncPlayerEmptyStream (async_test.go) — an empty stream is io.EOF at
creation — NewDemuxer's container errors, and a container whose index holds
an entry NextPacket cannot read (the source reads every packet at creation)."""
import ctypes as C

import pytest

from govid_gb300 import _native, ebiv


def test_empty_stream_is_eof_at_creation():
    e = ebiv.Encoder(ebiv.Config(64, 48))
    e.close()
    data = e.output()
    assert len(ebiv.Reader(data).packets()) == 0
    with pytest.raises(ebiv.EOF):
        ebiv.AsyncSource(data, depth=4)


def test_container_errors_and_bad_arguments():
    with pytest.raises(ebiv.ErrBadMagic):
        ebiv.AsyncSource(b"not a container" * 8, depth=4)
    L = _native.lib()
    h = C.c_void_p()
    e = ebiv.Encoder(ebiv.Config(64, 48))
    e.close()
    data = e.output()
    assert L.ebivgpu_source_create(data, len(data), 4, 2, C.byref(h)) == ebiv.ErrArgument.status  # unknown flag
    assert L.ebivgpu_source_create(data, len(data), 4, 0, None) == ebiv.ErrArgument.status
    f = _native.SourceFrame()
    assert L.ebivgpu_source_next(None, C.byref(f)) == ebiv.ErrArgument.status
    assert L.ebivgpu_source_seek(None, 0, None) == ebiv.ErrArgument.status
    L.ebivgpu_source_release(None, 0)
    L.ebivgpu_source_destroy(None)


def test_unreadable_index_entry_is_refused_at_creation():
    from test_container import _clip, wrapping_entries

    with pytest.raises(ebiv.ErrIO):
        ebiv.AsyncSource(wrapping_entries(_clip(10, 4)), depth=4)
