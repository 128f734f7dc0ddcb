"""TEST INFRASTRUCTURE — ctypes wrapper over the CPU oracle (oracle/_build/).

Used only by the tests, the smoke check and the benchmark's CPU-baseline leg,
as the checker.  The oracle restates govid's pure-Go EBIV decoder; see
ebiv_oracle.h for what it covers and how its parity is pinned.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "libebiv_oracle.so"

_lib = None


def build() -> Path:
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        L = C.CDLL(str(LIB))
        L.eo_codec_create.restype = C.c_void_p
        L.eo_codec_create.argtypes = [C.c_int, C.c_int]
        L.eo_codec_destroy.argtypes = [C.c_void_p]
        L.eo_codec_decode.argtypes = [C.c_void_p, C.c_char_p, C.c_size_t, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                      C.POINTER(C.c_int)]
        L.eo_codec_flush.argtypes = [C.c_void_p]
        L.eo_codec_ring_image.argtypes = [C.c_void_p, C.c_int, C.c_char_p, C.c_size_t]
        L.eo_codec_reference.argtypes = [C.c_void_p, C.c_int, C.c_char_p, C.c_size_t]
        L.eo_decode_streams.restype = C.c_long
        L.eo_rgba.argtypes = [C.c_char_p, C.c_char_p, C.c_char_p, C.c_int, C.c_int, C.c_char_p]
        L.eo_wide_residuals.restype = C.c_long
        L.eo_wide_residuals.argtypes = [C.c_int]
        _lib = L
    return _lib


class OracleCodec:
    """The reference Codec restated on the CPU: decode(packet) -> (status, packed planes or None)."""

    def __init__(self, ring: int = 3, threads: int = 1):
        self._L = lib()
        self._h = self._L.eo_codec_create(ring, threads)
        self.width = self.height = 0

    def decode(self, pkt: bytes):
        slot, w, h = C.c_int(), C.c_int(), C.c_int()
        st = self._L.eo_codec_decode(self._h, pkt, len(pkt), C.byref(slot), C.byref(w), C.byref(h))
        self.width, self.height = w.value, h.value
        if st != 0:
            return st, None
        n = w.value * h.value + 2 * ((w.value + 1) // 2) * ((h.value + 1) // 2)
        buf = C.create_string_buffer(n)
        self._L.eo_codec_ring_image(self._h, slot.value, buf, n)
        return 0, buf.raw

    def flush(self):
        self._L.eo_codec_flush(self._h)

    def reference(self, which: int, nbytes: int) -> bytes:
        buf = C.create_string_buffer(nbytes)
        assert self._L.eo_codec_reference(self._h, which, buf, nbytes) == 0
        return buf.raw

    def __del__(self):
        try:
            self._L.eo_codec_destroy(self._h)
        except Exception:
            pass


def decode_all(packets, threads: int = 1):
    """Decodes a packet list; returns [(status, packed planes or None)]."""
    c = OracleCodec(3, threads)
    return [c.decode(p) for p in packets]


def rgba(packed: bytes, w: int, h: int) -> bytes:
    cw, ch = (w + 1) // 2, (h + 1) // 2
    y, cb, cr = packed[: w * h], packed[w * h: w * h + cw * ch], packed[w * h + cw * ch:]
    out = C.create_string_buffer(w * h * 4)
    lib().eo_rgba(y, cb, cr, w, h, out)
    return out.raw


def decode_streams(streams: list[list[bytes]], threads: int) -> int:
    """Decodes many independent packet sequences on `threads` host threads
    (streams spread over threads); returns frames decoded without error."""
    L = lib()
    keep = []
    arr_p = (C.POINTER(C.c_char_p) * len(streams))()
    arr_n = (C.POINTER(C.c_size_t) * len(streams))()
    nfr = (C.c_int * len(streams))()
    for i, s in enumerate(streams):
        ps = (C.c_char_p * len(s))(*s)
        ns = (C.c_size_t * len(s))(*[len(p) for p in s])
        keep += [ps, ns]
        arr_p[i] = C.cast(ps, C.POINTER(C.c_char_p))
        arr_n[i] = C.cast(ns, C.POINTER(C.c_size_t))
        nfr[i] = len(s)
    return int(L.eo_decode_streams(arr_p, arr_n, nfr, len(streams), threads))


def wide_residuals(reset: bool = False) -> int:
    """Intra residual samples outside the 16-bit range reconstructed so far
    (all oracle codecs of the process); reset clears the count."""
    return int(lib().eo_wide_residuals(1 if reset else 0))
