"""TEST INFRASTRUCTURE — the EBIV container demuxer restated in plain Python.

The CPU reference arm of the benchmark and the CPU tests use it to read a
container without loading the GB300 product library.  It follows govid's
``ebiv.Reader`` (``ebiv/reader.go:32-160``) and the on-disk layout of
``ebiv/format.go``:

* 48-byte file header, magic ``EBIV``, version 4 (``format.go:28-36,230-265``);
* per frame an 8-byte record (sync ``0xEB17``, flags, payload size) before the
  payload (``format.go:296-328``);
* a trailing index of 16-byte entries and a 20-byte footer (index offset,
  count, CRC-32 of the index, magic ``EBIX``) (``reader.go:65-124``); when the
  footer does not validate the index is rebuilt by scanning the frame records
  (``reader.go:126-160``).

It is the checker's own parser: nothing in the product imports it.
"""
from __future__ import annotations

import struct
import zlib

FILE_HEADER = 48
FRAME_RECORD = 8
INDEX_ENTRY = 16
FOOTER = 20
VERSION = 4
MAX_FRAME = 256 << 20
FRAME_SYNC = 0xEB17


# Statuses of the reference's sentinel errors (ebiv/format.go:108-120), as the
# product's C-ABI numbers them.
ERR_CORRUPT, ERR_UNSUPPORTED, ERR_VERSION, ERR_BAD_MAGIC, ERR_IO = 1, 4, 5, 6, 10
U64 = (1 << 64) - 1


class ContainerError(ValueError):
    def __init__(self, msg: str, status: int = ERR_CORRUPT):
        super().__init__(msg)
        self.status = status


def parse_header(b: bytes) -> dict:
    """FileHeader.unmarshal — ebiv/format.go:207-245 (a short file is
    ErrBadMagic: NewDemuxer's ReadFull, ebiv/reader.go:38-44)."""
    if len(b) < FILE_HEADER or b[:4] != b"EBIV":
        raise ContainerError("bad magic", ERR_BAD_MAGIC)
    version, size, w, h, fn, fd = struct.unpack_from("<HHIIII", b, 4)
    if version != VERSION:
        raise ContainerError(f"version {version}", ERR_VERSION)
    if size != FILE_HEADER or not (0 < w <= 65535 and 0 < h <= 65535) or fn == 0 or fd == 0:
        raise ContainerError("corrupt header")
    if b[28] != 0 or b[29] != 0:
        raise ContainerError("chroma format or bit depth", ERR_UNSUPPORTED)
    tc, tr = struct.unpack_from("<HH", b, 32)
    return {"width": w, "height": h, "fps_num": fn, "fps_den": fd, "tile_cols": tc, "tile_rows": tr}


def _read_index(b: bytes) -> list[tuple[int, int, bool]] | None:
    """readIndex — ebiv/reader.go:65-113; None when the footer does not validate.
    Go's integer semantics: the bounds sum in int64, validateEntry's sum in
    wrapping uint64."""
    size = len(b)
    if size < FILE_HEADER + FOOTER or b[size - 4:] != b"EBIX":
        return None
    off, count, want = struct.unpack_from("<QII", b, size - FOOTER)
    if off < FILE_HEADER or off > size or off + count * INDEX_ENTRY != size - FOOTER:
        return None  # an offset past the file fails there or at the seek to it
    raw = b[off:off + count * INDEX_ENTRY]
    if zlib.crc32(raw) & 0xFFFFFFFF != want:
        return None
    idx = []
    for i in range(count):
        o, n, flags = struct.unpack_from("<QII", raw, i * INDEX_ENTRY)
        # validateEntry — ebiv/reader.go:115-123
        if o < FILE_HEADER or n == 0 or n > MAX_FRAME or (o + FRAME_RECORD + n) & U64 > off:
            return None
        idx.append((o, n, bool(flags & 1)))
    if idx and not idx[0][2]:
        return None
    return idx


def _scan_frames(b: bytes) -> list[tuple[int, int, bool]]:
    """scanFrames — ebiv/reader.go:126-160."""
    idx, off = [], FILE_HEADER
    while off + FRAME_RECORD <= len(b):
        sync, flags, n = struct.unpack_from("<HHI", b, off)
        if sync != FRAME_SYNC or n == 0 or n > MAX_FRAME or off + FRAME_RECORD + n > len(b):
            break
        idx.append((off, n, bool(flags & 1)))
        off += FRAME_RECORD + n
    if not idx or not idx[0][2]:
        raise ContainerError("no frames found")
    return idx


def payload_at(offset: int) -> int | None:
    """Where NextPacket reads an entry's payload: Seek(int64(Offset) +
    frameRecordSize) (ebiv/reader.go:203); None when that is negative (the
    seek fails and NextPacket returns the error)."""
    p = (offset + FRAME_RECORD) & U64
    return None if p >= 1 << 63 else p


def demux(container: bytes) -> tuple[dict, list[tuple[int | None, int, bool]], bool]:
    """NewDemuxer: (header, [(payload position or None, size, key)], index
    rebuilt by scanning)."""
    hdr = parse_header(container)
    idx = _read_index(container)
    rebuilt = idx is None
    if rebuilt:
        idx = _scan_frames(container)
    return hdr, [(payload_at(o), n, k) for o, n, k in idx], rebuilt


def packets(container: bytes) -> list[bytes]:
    """Every frame payload in order (NewDemuxer + NextPacket until EOF); an
    unreadable entry raises ContainerError with ERR_IO."""
    _, entries, _ = demux(container)
    out = []
    for p, n, _ in entries:
        if p is None:
            raise ContainerError("seek to a negative position", ERR_IO)
        out.append(bytes(container[p:p + n]))
    return out


def frame_type(pkt: bytes) -> int:
    """parseFrameHeader's type field (ebiv/format.go:376-383): 0 key, 1 inter."""
    return pkt[0] & 0x03
