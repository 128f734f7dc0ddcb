"""Host-side mirror of govid's EBIV plugin API over the GB300 decoder.

The names, argument meaning and error behaviour follow the reference:

* ``Codec`` is ``ebiv.Codec`` (``NewCodec(WithFrameRing(n))``,
  ``Decode(Packet) (*Frame, error)``, ``Flush()``; ebiv/codec.go:48-117) —
  decoding runs on the GPU through the C-ABI in ``include/ebivgpu.h``.
* ``Reader`` is ``ebiv.Reader``, a ``govid.Demuxer`` (ebiv/reader.go).
* ``Encoder`` is ``ebiv.Encoder`` with its functional options
  (ebiv/encoder.go:50-148).
* Errors are exception classes matching the ``ebiv`` sentinels
  (ebiv/format.go:110-119); ``isinstance`` plays the role of ``errors.Is``.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _native

# ---------------------------------------------------------------------------
# Errors (ebiv/format.go:110-119)
# ---------------------------------------------------------------------------


class EbivError(Exception):
    status = -1


class ErrCorrupt(EbivError):
    status = 1


class ErrNoKeyframe(EbivError):
    status = 2


class ErrDimensions(EbivError):
    status = 3


class ErrUnsupported(EbivError):
    status = 4


class ErrVersion(EbivError):
    status = 5


class ErrBadMagic(EbivError):
    status = 6


class ErrConfig(EbivError):
    status = 7


class ErrWriterClosed(EbivError):
    status = 8


class EOF(EbivError):
    status = 9


class ErrIO(EbivError):
    status = 10


class ErrDevice(EbivError):
    status = 11


class ErrArgument(EbivError):
    status = 12


class ErrTooLarge(EbivError):
    status = 13


_ERRORS = {c.status: c for c in (ErrCorrupt, ErrNoKeyframe, ErrDimensions, ErrUnsupported, ErrVersion,
                                  ErrBadMagic, ErrConfig, ErrWriterClosed, EOF, ErrIO, ErrDevice, ErrArgument,
                                  ErrTooLarge)}


def _check(status: int, what: str = "") -> None:
    if status == 0:
        return
    L = _native.lib()
    msg = L.ebivgpu_status_string(status).decode()
    raise _ERRORS.get(status, EbivError)(f"{what}: {msg}" if what else msg)


# ---------------------------------------------------------------------------
# Packets and frames (govid.go:9-22)
# ---------------------------------------------------------------------------


@dataclass
class Packet:
    data: bytes
    timestamp_ns: int = 0
    keyframe: bool = False


@dataclass
class Frame:
    """A decoded 4:2:0 frame.  y/cb/cr are strided views into the codec's
    ring, valid for ``ring`` further decodes (ebiv/codec.go:15-22)."""
    y: np.ndarray
    cb: np.ndarray
    cr: np.ndarray
    timestamp_ns: int
    width: int
    height: int
    ring_slot: int = -1
    keyframe: bool = False
    _codec: "Codec | None" = field(default=None, repr=False)

    def packed(self) -> bytes:
        """Tightly packed Y, Cb, Cr planes (the on-disk raw layout)."""
        cw, ch = (self.width + 1) // 2, (self.height + 1) // 2
        return (np.ascontiguousarray(self.y[: self.height, : self.width]).tobytes()
                + np.ascontiguousarray(self.cb[:ch, :cw]).tobytes()
                + np.ascontiguousarray(self.cr[:ch, :cw]).tobytes())

    def rgba(self) -> np.ndarray:
        """RGBA (h, w, 4) computed on the GPU (frame.go:8-67, 127-135)."""
        if self._codec is None:
            raise ErrArgument("frame has no codec")
        return self._codec.rgba(self)


# ---------------------------------------------------------------------------
# Codec (ebiv/codec.go)
# ---------------------------------------------------------------------------


class Codec:
    """GPU EBIV decoder with the ebiv.Codec contract."""

    def __init__(self, ring: int = 3):
        L = _native.lib()
        h = C.c_void_p()
        _check(L.ebivgpu_create(int(ring), C.byref(h)), "NewCodec")
        self._h = h
        self._L = L

    def decode(self, pkt: Packet | bytes) -> Frame:
        data = pkt.data if isinstance(pkt, Packet) else bytes(pkt)
        ts = pkt.timestamp_ns if isinstance(pkt, Packet) else 0
        f = _native.Frame()
        _check(self._L.ebivgpu_decode(self._h, data, len(data), ts, C.byref(f)))
        w, h, ys, cs = f.width, f.height, f.y_stride, f.c_stride
        ch = (h + 1) // 2
        y = np.ctypeslib.as_array(f.y, shape=(h * ys,)).reshape(h, ys)
        cb = np.ctypeslib.as_array(f.cb, shape=(ch * cs,)).reshape(ch, cs)
        cr = np.ctypeslib.as_array(f.cr, shape=(ch * cs,)).reshape(ch, cs)
        return Frame(y, cb, cr, f.timestamp_ns, w, h, f.ring_slot, bool(f.keyframe), self)

    Decode = decode

    def flush(self) -> None:
        self._L.ebivgpu_flush(self._h)

    Flush = flush

    def with_rgba(self, on: bool = True) -> None:
        """WithRGBA (source.go:61-74): later decodes also convert each frame to
        RGBA on the GPU into a pinned buffer pooled per ring slot."""
        _check(self._L.ebivgpu_set_rgba(self._h, int(bool(on))))

    WithRGBA = with_rgba

    def pooled_rgba(self, frame: Frame) -> np.ndarray | None:
        """The frame's pooled RGBA (h, w, 4), copied out; None when the frame
        was decoded without WithRGBA or its slot has been reused."""
        p = self._L.ebivgpu_frame_rgba_pooled(self._h, frame.ring_slot)
        if not p:
            return None
        n = frame.width * frame.height * 4
        return np.frombuffer(C.string_at(p, n), np.uint8).reshape(frame.height, frame.width, 4)

    def rgba(self, frame: Frame) -> np.ndarray:
        out = np.empty((frame.height, frame.width, 4), np.uint8)
        _check(self._L.ebivgpu_frame_rgba(self._h, frame.ring_slot,
                                          out.ctypes.data_as(C.POINTER(C.c_uint8)), out.nbytes))
        return out

    def launches(self) -> int:
        return int(self._L.ebivgpu_codec_launches(self._h))

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._L.ebivgpu_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def NewCodec(ring: int = 3) -> Codec:
    return Codec(ring)


def device_available() -> bool:
    return bool(_native.lib().ebivgpu_device_available())


# ---------------------------------------------------------------------------
# Batched decode of many streams (include/ebivgpu.h, ebivgpu_batch_*)
# ---------------------------------------------------------------------------


@dataclass
class BatchResult:
    stream: int
    frame_index: int
    status: int
    keyframe: bool
    index: int  # position in the round's result list


class Batch:
    """Many independent EBIV streams decoded together: each round decodes the
    next packet of every active stream with one set of kernel launches."""

    def __init__(self, lookahead: int = 1, pipeline: bool | int = False):
        """pipeline (True or a depth of 1 to 3): each round() plans a round
        and starts its entropy stage while earlier rounds reconstruct, and
        returns the results of the round planned `depth` calls before; drain()
        returns those of the rounds still in flight (resident streams only).
        Each extra level starts a round's entropy stage one round earlier."""
        L = _native.lib()
        h = C.c_void_p()
        _check(L.ebivgpu_batch_create(C.byref(h)), "batch")
        self._h, self._L = h, L
        self.depth = int(pipeline)  # rounds between planning a round and getting its results
        if lookahead != 1:
            _check(L.ebivgpu_batch_set_lookahead(h, int(lookahead)), "lookahead")
        if pipeline:
            _check(L.ebivgpu_batch_set_pipeline(h, self.depth), "pipeline")

    def set_tuning(self, entropy_groups: int = 4, intra_warps: int = 0) -> None:
        """Launch shapes (results do not depend on them): entropy launches per
        pipelined round (1-4) and intra-stage warps per CTA (4/8/16, 0 = auto)."""
        _check(self._L.ebivgpu_batch_set_tuning(self._h, int(entropy_groups), int(intra_warps)), "tuning")

    def add_stream(self, packets: list[bytes], ring: int = 3) -> int:
        n = len(packets)
        arr = (C.c_char_p * n)(*packets)
        lens = (C.c_size_t * n)(*[len(p) for p in packets])
        sid = C.c_int()
        _check(self._L.ebivgpu_batch_add_stream(self._h, arr, lens, n, ring, C.byref(sid)), "add_stream")
        return sid.value

    def add_streaming(self, ring: int = 3) -> int:
        sid = C.c_int()
        _check(self._L.ebivgpu_batch_add_streaming(self._h, ring, C.byref(sid)))
        return sid.value

    def submit(self, sid: int, pkt: bytes) -> None:
        _check(self._L.ebivgpu_batch_submit(self._h, sid, pkt, len(pkt)))

    def seek(self, sid: int, packet_index: int) -> None:
        _check(self._L.ebivgpu_batch_seek(self._h, sid, packet_index))

    def set_active(self, sid: int, active: bool) -> None:
        _check(self._L.ebivgpu_batch_set_active(self._h, sid, int(active)))

    def remove_stream(self, sid: int) -> None:
        _check(self._L.ebivgpu_batch_remove_stream(self._h, sid))

    def remaining(self, sid: int) -> int:
        return int(self._L.ebivgpu_batch_remaining(self._h, sid))

    def round(self, ids: list[int] | None = None) -> list[BatchResult]:
        n = C.c_int()
        if ids is None:
            _check(self._L.ebivgpu_batch_round(self._h, C.byref(n)))
        else:
            arr = (C.c_int * len(ids))(*ids)
            _check(self._L.ebivgpu_batch_round_for(self._h, arr, len(ids), C.byref(n)))
        return self._results()

    def drain(self) -> list[BatchResult]:
        """Collects the round in flight (pipelined batches)."""
        n = C.c_int()
        _check(self._L.ebivgpu_batch_drain(self._h, C.byref(n)))
        return self._results()

    def _results(self) -> list[BatchResult]:
        out = []
        for i in range(self._L.ebivgpu_batch_result_count(self._h)):
            s, st, k = C.c_int(), C.c_int(), C.c_int()
            fi = C.c_int64()
            self._L.ebivgpu_batch_result(self._h, i, C.byref(s), C.byref(fi), C.byref(st), C.byref(k))
            out.append(BatchResult(s.value, fi.value, st.value, bool(k.value), i))
        return out

    def download(self, r: BatchResult, width: int, height: int) -> bytes:
        n = packed_size(width, height)
        buf = (C.c_uint8 * n)()
        _check(self._L.ebivgpu_batch_result_download(self._h, r.index, buf, n))
        return bytes(buf)

    def download_async(self, r: BatchResult, address: int, cap: int) -> None:
        """Queues the packed planes of r into host memory at address (pinned
        memory makes the copy asynchronous); complete after sync()."""
        _check(self._L.ebivgpu_batch_result_download_async(self._h, r.index, C.c_void_p(address), cap))

    def sync(self) -> None:
        _check(self._L.ebivgpu_batch_sync(self._h))

    def reload(self, sid: int, addresses: list[int], lengths: list[int]) -> None:
        """New packets (host addresses, e.g. in pinned memory) for a resident
        stream; rewinds it and keeps its frame pool (no round in flight)."""
        n = len(addresses)
        a = (C.c_void_p * n)(*addresses)
        ln = (C.c_size_t * n)(*lengths)
        _check(self._L.ebivgpu_batch_reload_stream(self._h, sid, a, ln, n), "reload")

    def add_container(self, container: "DeviceContainer", ring: int = 3) -> int:
        """A resident stream decoding in place from a DeviceContainer (no packet
        copies); the container must outlive the batch."""
        sid = C.c_int()
        _check(self._L.ebivgpu_batch_add_container(self._h, container._h, ring, C.byref(sid)), "add_container")
        self._keep = getattr(self, "_keep", []) + [container]
        return sid.value

    def planes(self, r: BatchResult) -> "_native.PlaneView":
        v = _native.PlaneView()
        _check(self._L.ebivgpu_batch_result_planes(self._h, r.index, C.byref(v)))
        return v

    def timing(self, enable: int = -1) -> tuple[float, float, float]:
        k, e, r = C.c_double(), C.c_double(), C.c_double()
        self._L.ebivgpu_batch_timing(self._h, enable, C.byref(k), C.byref(e), C.byref(r))
        return k.value, e.value, r.value

    def launches(self) -> int:
        return int(self._L.ebivgpu_batch_launches(self._h))

    def device_bytes(self) -> int:
        return int(self._L.ebivgpu_batch_device_bytes(self._h))

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._L.ebivgpu_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Serving loop: continuous batching of per-frame requests from many
    streams with HBM-budget admission, seeks and looping (include/ebivgpu.h,
    ebivgpu_server_*)."""

    def __init__(self, duration_s: float = 10.0, frames_per_stream: int = 600, seek_prob: float = 0.05,
                 seed: int = 1, hbm_budget_bytes: int = 120 << 30, max_frames_per_round: int = 4, ring: int = 3,
                 record: bool = False, key_lane: int = 1, start_spread_s: float = 0.0, decode_ahead: int = 0,
                 decode_lanes: int = 0, long_key_mbs: int = 0, key_cache: int = 0):
        L = _native.lib()
        o = _native.ServeOptions(duration_s, frames_per_stream, seek_prob, seed, hbm_budget_bytes,
                                 max_frames_per_round, ring, int(record), int(key_lane), float(start_spread_s),
                                 int(decode_ahead), int(decode_lanes), int(long_key_mbs), int(key_cache))
        h = C.c_void_p()
        _check(L.ebivgpu_server_create(C.byref(o), C.byref(h)), "server")
        self._h, self._L, self._o = h, L, o

    def stream_footprint(self, width: int, height: int, packets: list[bytes]) -> int:
        """The HBM bytes this server admits a stream of these packets by."""
        pb = sum((len(p) + 15) // 16 * 16 for p in packets)
        return int(self._L.ebivgpu_server_stream_footprint(C.byref(self._o), width, height, pb))

    def add_stream(self, packets: list[bytes], fps: float, loop: bool = False) -> None:
        n = len(packets)
        arr = (C.c_char_p * n)(*packets)
        lens = (C.c_size_t * n)(*[len(p) for p in packets])
        _check(self._L.ebivgpu_server_add_stream(self._h, arr, lens, n, float(fps), int(loop)))

    def run(self) -> dict:
        st = _native.ServeStats()
        _check(self._L.ebivgpu_server_run(self._h, C.byref(st)))
        return {k: getattr(st, k) for k, _ in _native.ServeStats._fields_}

    def request_log(self) -> dict[str, np.ndarray]:
        """Every delivered request: arrival (s), latency (ms), stream, frame, seek."""
        n = int(self._L.ebivgpu_server_request_log(self._h, None, None, None, None, None, 0))
        out = {"arrival_s": np.zeros(n), "latency_ms": np.zeros(n), "stream": np.zeros(n, np.int32),
               "frame": np.zeros(n, np.int64), "seek": np.zeros(n, np.int32)}
        self._L.ebivgpu_server_request_log(self._h, *(out[k].ctypes.data for k in out), n)
        return out

    def frame_hashes(self) -> list[tuple[int, int, int]]:
        n = self._L.ebivgpu_server_frame_hashes(self._h, None, None, None, 0)
        s = (C.c_int32 * n)()
        f = (C.c_int64 * n)()
        h = (C.c_uint64 * n)()
        self._L.ebivgpu_server_frame_hashes(self._h, s, f, h, n)
        return list(zip(s, f, h))

    def __del__(self):
        try:
            if self._h:
                self._L.ebivgpu_server_destroy(self._h)
                self._h = None
        except Exception:
            pass


class DeviceContainer:
    """An EBIV container in pinned, device-mapped host memory whose frame index
    and seeks are computed on the GPU (ebiv/reader.go:32-238); a Batch stream
    can decode from it in place (Batch.add_container)."""

    def __init__(self, data: bytes):
        L = _native.lib()
        h = C.c_void_p()
        _check(L.ebivgpu_container_open(data, len(data), C.byref(h)), "NewDemuxer")
        self._h, self._L = h, L
        info = (C.c_int64 * 6)()
        L.ebivgpu_container_info(h, info)
        self.width, self.height, self.fps_num, self.fps_den, self.frame_count, rebuilt = (int(v) for v in info)
        self.rebuilt_index = bool(rebuilt)

    def entry(self, i: int) -> tuple[int, int, bool]:
        """(payload offset, payload size, keyframe) of frame i."""
        o, n, k = C.c_uint64(), C.c_uint32(), C.c_int()
        _check(self._L.ebivgpu_container_entry(self._h, int(i), C.byref(o), C.byref(n), C.byref(k)))
        return o.value, n.value, bool(k.value)

    def seek(self, t_ns: int) -> tuple[int, int]:
        """Seek(t): (frame index, its presentation time), resolved on the GPU."""
        f, landed = C.c_int64(), C.c_int64()
        _check(self._L.ebivgpu_container_seek(self._h, int(t_ns), C.byref(f), C.byref(landed)))
        return f.value, landed.value

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._L.ebivgpu_container_close(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


@dataclass
class SourceFrame:
    """A frame from an AsyncSource: packed planes (and RGBA with rgba=True)
    in pinned host memory, valid until ``AsyncSource.release(frame)``."""
    y: np.ndarray
    cb: np.ndarray
    cr: np.ndarray
    timestamp_ns: int
    width: int
    height: int
    frame_index: int
    keyframe: bool
    rgba: np.ndarray | None
    handle: int

    def packed(self) -> bytes:
        return self.y.tobytes() + self.cb.tobytes() + self.cr.tobytes()


class AsyncSource:
    """govid's decode-ahead frame source (asyncSource, source.go:84-266; the
    source of NewAsyncPlayer(d, c, depth, WithRGBA), player.go:40-57) on the
    GPU: a native worker thread decodes the container's frames ahead of the
    consumer (include/ebivgpu.h, ebivgpu_source_*).

    next() blocks for the next frame; poll() returns None when none is ready.
    At the end of the stream both raise EOF, after a decode error they raise
    it; the worker then waits for seek().  Frames stay valid until release().
    """

    def __init__(self, container: bytes, depth: int = 4, rgba: bool = False):
        L = _native.lib()
        h = C.c_void_p()
        _check(L.ebivgpu_source_create(container, len(container), int(depth), 1 if rgba else 0, C.byref(h)),
               "NewAsyncPlayer")
        self._h, self._L = h, L
        self._f = _native.SourceFrame()

    def _frame(self) -> SourceFrame:
        f = self._f
        w, h = f.width, f.height
        cw, ch = (w + 1) // 2, (h + 1) // 2
        y = np.ctypeslib.as_array(f.y, shape=(h, w))
        cb = np.ctypeslib.as_array(f.cb, shape=(ch, cw))
        cr = np.ctypeslib.as_array(f.cr, shape=(ch, cw))
        rgba = np.ctypeslib.as_array(f.rgba, shape=(h, w, 4)) if f.rgba else None
        return SourceFrame(y, cb, cr, f.timestamp_ns, w, h, f.frame_index, bool(f.keyframe), rgba, f.handle)

    def next(self) -> SourceFrame:
        _check(self._L.ebivgpu_source_next(self._h, C.byref(self._f)), "next")
        return self._frame()

    def poll(self) -> SourceFrame | None:
        ready = C.c_int()
        _check(self._L.ebivgpu_source_poll(self._h, C.byref(self._f), C.byref(ready)), "poll")
        return self._frame() if ready.value else None

    def seek(self, t_ns: int) -> int:
        """Repositions at the last key frame at or before t; returns its time."""
        landed = C.c_int64()
        _check(self._L.ebivgpu_source_seek(self._h, int(t_ns), C.byref(landed)), "seek")
        return landed.value

    def release(self, frame: SourceFrame | None) -> None:
        if frame is not None and getattr(self, "_h", None):
            self._L.ebivgpu_source_release(self._h, frame.handle)

    @property
    def decoded(self) -> int:
        """Frames the worker has decoded so far."""
        return int(self._L.ebivgpu_source_decoded(self._h))

    @property
    def lookahead(self) -> int:
        return int(self._L.ebivgpu_source_lookahead(self._h))

    def duration(self) -> int:
        return int(self._L.ebivgpu_source_duration(self._h))

    def close(self) -> None:
        """Stops the worker (idempotent); frames already returned stay valid
        until destroy()."""
        if getattr(self, "_h", None):
            _check(self._L.ebivgpu_source_close(self._h))

    def destroy(self) -> None:
        if getattr(self, "_h", None):
            self._L.ebivgpu_source_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


class BlockAnalysis:
    """forwardDCT and satd (ebiv/transform.go:44-119) of a batch of residual
    blocks on the GPU."""

    def __init__(self):
        L = _native.lib()
        h = C.c_void_p()
        _check(L.ebivgpu_analysis_create(C.byref(h)), "analysis")
        self._h, self._L = h, L

    def fdct_satd(self, blocks: np.ndarray, coeffs: bool = True, satd: bool = True):
        """blocks: (count, n, n) int32 -> (coefficients or None, satd or None)."""
        b = np.ascontiguousarray(blocks, dtype=np.int32)
        count, n, _ = b.shape
        co = np.empty_like(b) if coeffs else None
        sa = np.empty(count, np.int64) if satd else None
        ms = C.c_double()
        _check(self._L.ebivgpu_fdct_satd(self._h, b.ctypes.data, n, count, co.ctypes.data if coeffs else None,
                                         sa.ctypes.data if satd else None, C.byref(ms)), "fdct_satd")
        self.kernel_ms = ms.value
        return co, sa

    def __del__(self):
        try:
            if self._h:
                self._L.ebivgpu_analysis_destroy(self._h)
                self._h = None
        except Exception:
            pass


class AltRef:
    """The encoder's alt-ref temporal filter on the GPU ((*Encoder).buildAltRef,
    ebiv/encoder.go:326-407): build(frames, w, h, window) returns the packed
    golden-override image, or None when the reference returns nil."""

    def __init__(self):
        L = _native.lib()
        h = C.c_void_p()
        _check(L.ebivgpu_altref_create(C.byref(h)), "altref")
        self._h, self._L = h, L

    def build(self, frames: list[bytes], width: int, height: int, window: int) -> bytes | None:
        n = len(frames)
        arr = (C.c_char_p * max(n, 1))(*frames)
        out = (C.c_uint8 * packed_size(width, height))()
        acc = C.c_int()
        _check(self._L.ebivgpu_altref_build(self._h, arr, n, width, height, window, out, len(out), C.byref(acc)),
               "altref")
        self.accepted = acc.value
        return bytes(out) if acc.value else None

    def time(self, window: int, reps: int = 10) -> float:
        """Mean kernel milliseconds on the frames of the last build."""
        ms = C.c_double()
        _check(self._L.ebivgpu_altref_time(self._h, window, reps, C.byref(ms)), "altref")
        return ms.value

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._L.ebivgpu_altref_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def frame_hash(packed: bytes) -> int:
    return int(_native.lib().ebivgpu_frame_hash(packed, len(packed)))


def stream_footprint(width: int, height: int, ring: int = 3, lookahead: int = 1) -> int:
    return int(_native.lib().ebivgpu_stream_footprint(width, height, ring, lookahead))


# ---------------------------------------------------------------------------
# Demuxer (ebiv/reader.go)
# ---------------------------------------------------------------------------


@dataclass
class VideoInfo:
    width: int
    height: int
    frame_rate: float


@dataclass
class IndexEntry:
    size: int
    keyframe: bool


class Reader:
    """In-memory EBIV demuxer (govid.Demuxer)."""

    def __init__(self, data: bytes):
        L = _native.lib()
        h = C.c_void_p()
        _check(L.ebiv_reader_open(data, len(data), C.byref(h)), "NewDemuxer")
        self._h, self._L = h, L
        info = (C.c_int64 * 8)()
        L.ebiv_reader_info(h, info)
        self.width, self.height = int(info[0]), int(info[1])
        self.fps_num, self.fps_den = int(info[2]), int(info[3])
        self.frame_count = int(info[4])
        self.tile_cols, self.tile_rows = int(info[5]), int(info[6])
        self.rebuilt_index = bool(info[7])

    def next_packet(self) -> Packet:
        d = C.POINTER(C.c_uint8)()
        n, ts, k = C.c_size_t(), C.c_int64(), C.c_int()
        _check(self._L.ebiv_reader_next_packet(self._h, C.byref(d), C.byref(n), C.byref(ts), C.byref(k)))
        return Packet(C.string_at(d, n.value), ts.value, bool(k.value))

    NextPacket = next_packet

    def packet(self, i: int) -> Packet:
        d = C.POINTER(C.c_uint8)()
        n, k = C.c_size_t(), C.c_int()
        _check(self._L.ebiv_reader_packet(self._h, int(i), C.byref(d), C.byref(n), C.byref(k)))
        return Packet(C.string_at(d, n.value), self.frame_time(i), bool(k.value))

    def packets(self) -> list[Packet]:
        return [self.packet(i) for i in range(self.frame_count)]

    def index(self) -> list[IndexEntry]:
        out = []
        for i in range(self.frame_count):
            p = self.packet(i)
            out.append(IndexEntry(len(p.data), p.keyframe))
        return out

    def seek(self, t_ns: int) -> int:
        landed = C.c_int64()
        _check(self._L.ebiv_reader_seek(self._h, int(t_ns), C.byref(landed)))
        return landed.value

    Seek = seek

    def duration(self) -> int:
        return int(self._L.ebiv_reader_duration(self._h))

    def frame_time(self, i: int) -> int:
        return int(self._L.ebiv_reader_frame_time(self._h, int(i)))

    def frame_index_at(self, t_ns: int) -> int:
        return int(self._L.ebiv_reader_frame_index_at(self._h, int(t_ns)))

    def video_info(self) -> VideoInfo:
        return VideoInfo(self.width, self.height, self.fps_num / self.fps_den)

    def close(self) -> None:
        self._L.ebiv_reader_close(self._h)

    def __del__(self):
        try:
            if self._h:
                self._L.ebiv_reader_destroy(self._h)
                self._h = None
        except Exception:
            pass

    def __iter__(self):
        while True:
            try:
                yield self.next_packet()
            except EOF:
                return


def NewDemuxer(data: bytes) -> Reader:
    return Reader(data)


def parse_frame_header(pkt: bytes) -> dict:
    info = (C.c_int32 * 6)()
    _check(_native.lib().ebiv_parse_frame_header(pkt, len(pkt), info))
    return {"type": info[0], "coding": info[1], "width": info[2], "height": info[3],
            "golden_override": bool(info[4]), "body_offset": info[5]}


# ---------------------------------------------------------------------------
# Encoder (ebiv/encoder.go)
# ---------------------------------------------------------------------------


@dataclass
class Config:
    width: int
    height: int
    fps_num: int = 30
    fps_den: int = 1
    tile_cols: int = 0
    tile_rows: int = 0


def packed_size(w: int, h: int) -> int:
    return w * h + 2 * ((w + 1) // 2) * ((h + 1) // 2)


class Encoder:
    """EBIV encoder.  Options mirror WithIntra / WithGOP / WithTiles /
    WithAutoTiles / WithAltRef / WithFastEncode."""

    def __init__(self, cfg: Config, intra: int | None = None, gop: int = 1, tiles: tuple[int, int] | None = None,
                 auto_tiles: int = 0, altref: int = 0, fast: bool = False, threads: int = 1,
                 search: str = "diamond", exhaustive_range: int = 16, keep_recon: bool = False,
                 fallback_sad: int = 0):
        L = _native.lib()
        o = _native.EncoderOptions()
        L.ebiv_encoder_default_options(C.byref(o))
        o.width, o.height = cfg.width, cfg.height
        o.fps_num, o.fps_den = cfg.fps_num, cfg.fps_den
        o.tile_cols, o.tile_rows = cfg.tile_cols, cfg.tile_rows
        if tiles is not None:
            o.with_tiles_cols, o.with_tiles_rows = tiles
        if intra is not None:
            o.coded, o.qp = 1, int(intra)
        o.gop = int(gop)
        o.auto_tiles = int(auto_tiles)
        o.altref_window = int(altref)
        o.fast_encode = int(bool(fast))
        o.threads = int(threads)
        o.search = {"diamond": 0, "exhaustive": 1, "proposed": 2}[search]
        o.exhaustive_range = int(exhaustive_range)
        o.keep_recon = int(bool(keep_recon))
        o.proposed_fallback_sad = int(fallback_sad)
        h = C.c_void_p()
        _check(L.ebiv_encoder_create(C.byref(o), C.byref(h)), "NewEncoder")
        self._h, self._L, self.cfg = h, L, cfg

    def write_frame(self, packed: bytes | np.ndarray) -> None:
        b = packed.tobytes() if isinstance(packed, np.ndarray) else bytes(packed)
        _check(self._L.ebiv_encoder_write_frame(self._h, b, len(b)), "WriteFrame")

    WriteFrame = write_frame

    def close(self) -> None:
        _check(self._L.ebiv_encoder_close(self._h), "Close")

    Close = close

    def output(self) -> bytes:
        d = C.POINTER(C.c_uint8)()
        n = C.c_size_t()
        self._L.ebiv_encoder_output(self._h, C.byref(d), C.byref(n))
        return C.string_at(d, n.value)

    def recons(self) -> list[bytes]:
        n = self._L.ebiv_encoder_recon_count(self._h)
        sz = packed_size(self.cfg.width, self.cfg.height)
        buf = (C.c_uint8 * sz)()
        out = []
        for i in range(n):
            _check(self._L.ebiv_encoder_recon(self._h, i, buf, sz))
            out.append(bytes(buf))
        return out

    def sad_evaluations(self) -> int:
        return int(self._L.ebiv_encoder_sad_evaluations(self._h))

    def search_fallbacks(self) -> int:
        return int(self._L.ebiv_encoder_search_fallbacks(self._h))

    def search_seconds(self) -> float:
        """Thread seconds in motion search, summed over tile threads."""
        return float(self._L.ebiv_encoder_search_seconds(self._h))

    def propose_seconds(self) -> float:
        """Wall seconds the proposer spent preparing candidates (search='proposed')."""
        return float(self._L.ebiv_encoder_propose_seconds(self._h))

    def set_candidates(self, mv: np.ndarray) -> None:
        """mv: int16 (frames, mbs, k, 2) quarter-pel candidates for search='proposed'."""
        a = np.ascontiguousarray(mv, dtype=np.int16)
        f, m, k, _ = a.shape
        _check(self._L.ebiv_encoder_set_candidates(self._h, a.ctypes.data_as(C.POINTER(C.c_int16)), f, m, k))
        self._cand = a

    def __del__(self):
        try:
            if self._h:
                self._L.ebiv_encoder_destroy(self._h)
                self._h = None
        except Exception:
            pass


# ---------------------------------------------------------------------------
# Synthetic content
# ---------------------------------------------------------------------------


def synth_frame(w: int, h: int, seed: int) -> bytes:
    """ebiv/harness_test.go:105-129 (gradient, diagonal edge, checker)."""
    buf = (C.c_uint8 * packed_size(w, h))()
    _check(_native.lib().ebiv_synth_frame(w, h, seed, buf, len(buf)))
    return bytes(buf)


def synth_pan(w: int, h: int, seed: int) -> bytes:
    """ebiv/harness_test.go:134-171 (texture panned 2 px/frame)."""
    buf = (C.c_uint8 * packed_size(w, h))()
    _check(_native.lib().ebiv_synth_pan(w, h, seed, buf, len(buf)))
    return bytes(buf)


@dataclass
class SceneSpec:
    width: int = 640
    height: int = 360
    seed: int = 1
    sprites: int = 6
    vel_max_q: int = 16
    integer_vel: bool = True
    pan_max_q: int = 0
    flash_period: int = 0
    flash_start: int = 30
    flash_len: int = 3
    flash_amp: int = 40
    noise_y16: int = 32
    noise_c16: int = 16

    def as_array(self):
        v = [self.width, self.height, self.seed, self.sprites, self.vel_max_q, int(self.integer_vel),
             self.pan_max_q, self.flash_period, self.flash_start, self.flash_len, self.flash_amp,
             self.noise_y16, self.noise_c16]
        return (C.c_int64 * 13)(*v)


class Scene:
    def __init__(self, spec: SceneSpec):
        h = C.c_void_p()
        _check(_native.lib().ebiv_scene_create(spec.as_array(), C.byref(h)))
        self._h, self.spec = h, spec

    def render(self, i: int) -> bytes:
        buf = (C.c_uint8 * packed_size(self.spec.width, self.spec.height))()
        _check(_native.lib().ebiv_scene_render(self._h, int(i), buf, len(buf)))
        return bytes(buf)

    def __del__(self):
        try:
            if self._h:
                _native.lib().ebiv_scene_destroy(self._h)
                self._h = None
        except Exception:
            pass


def encode_scene(spec: SceneSpec, frames: int, qp: int, gop: int, tiles: tuple[int, int], fast: bool = False,
                 threads: int = 1, altref: int = 0) -> bytes:
    """Renders and encodes a sprite scene in one native call."""
    L = _native.lib()
    o = _native.EncoderOptions()
    L.ebiv_encoder_default_options(C.byref(o))
    o.width, o.height = spec.width, spec.height
    o.coded, o.qp, o.gop = 1, qp, gop
    o.with_tiles_cols, o.with_tiles_rows = tiles
    o.fast_encode = int(fast)
    o.threads = threads
    o.altref_window = altref
    d = C.POINTER(C.c_uint8)()
    n = C.c_size_t()
    _check(L.ebiv_encode_scene(spec.as_array(), int(frames), C.byref(o), C.byref(d), C.byref(n)), "encode")
    try:
        return C.string_at(d, n.value)
    finally:
        L.ebiv_free(d)


def encode_key_from_levels(width: int, height: int, qp: int, mode: int, levels: np.ndarray) -> bytes:
    """A one-tile intra key frame packet with chosen levels (include/ebiv_host.h,
    ebiv_encode_key_from_levels): levels has 384 entries per macroblock in
    raster order — sixteen 4x4 luma blocks of 16, then 64 Cb and 64 Cr."""
    L = _native.lib()
    lv = np.ascontiguousarray(levels, dtype=np.int32).ravel()
    d = C.POINTER(C.c_uint8)()
    n = C.c_size_t()
    _check(L.ebiv_encode_key_from_levels(int(width), int(height), int(qp), int(mode),
                                         lv.ctypes.data_as(C.POINTER(C.c_int32)), lv.size, C.byref(d), C.byref(n)),
           "encode_key_from_levels")
    try:
        return C.string_at(d, n.value)
    finally:
        L.ebiv_free(d)

