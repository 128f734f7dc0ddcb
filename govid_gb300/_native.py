"""Loader for the in-tree native library ``govid_gb300/_lib/libebivgpu.so``.

The product path has no fallback: if the library is missing, importing the
decoder raises.  Build it with ``python -m govid_gb300.build`` (or
``__graft_entry__.build()``).
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libebivgpu.so"

_lib = None


class EncoderOptions(C.Structure):
    _fields_ = [
        ("width", C.c_int32), ("height", C.c_int32),
        ("fps_num", C.c_uint32), ("fps_den", C.c_uint32),
        ("tile_cols", C.c_int32), ("tile_rows", C.c_int32),
        ("with_tiles_cols", C.c_int32), ("with_tiles_rows", C.c_int32),
        ("coded", C.c_int32), ("qp", C.c_int32), ("gop", C.c_int32),
        ("auto_tiles", C.c_int32), ("altref_window", C.c_int32),
        ("fast_encode", C.c_int32), ("threads", C.c_int32),
        ("search", C.c_int32), ("exhaustive_range", C.c_int32),
        ("keep_recon", C.c_int32), ("proposed_fallback_sad", C.c_int32),
    ]


class PlaneView(C.Structure):
    _fields_ = [("y", C.c_void_p), ("cb", C.c_void_p), ("cr", C.c_void_p),
                ("y_stride", C.c_int32), ("c_stride", C.c_int32), ("width", C.c_int32), ("height", C.c_int32)]


class ServeOptions(C.Structure):
    _fields_ = [("duration_s", C.c_double), ("frames_per_stream", C.c_int64), ("seek_prob", C.c_double),
                ("seed", C.c_uint64), ("hbm_budget_bytes", C.c_uint64), ("max_frames_per_round", C.c_int32),
                ("ring", C.c_int32), ("record", C.c_int32), ("key_lane", C.c_int32),
                ("start_spread_s", C.c_double), ("decode_ahead", C.c_int32), ("decode_lanes", C.c_int32),
                ("long_key_mbs", C.c_int32), ("key_cache", C.c_int32)]


class ServeStats(C.Structure):
    _fields_ = [(k, C.c_int64) for k in ("requests", "frames", "errors", "seeks", "loops", "rounds",
                                         "admitted_total", "admitted_peak", "waiting_at_end")] + \
               [(k, C.c_double) for k in ("elapsed_s", "latency_p50_ms", "latency_p99_ms", "latency_max_ms",
                                          "latency_mean_ms", "frames_per_s", "kernel_ms", "entropy_ms",
                                          "recon_ms")] + [("key_frames", C.c_int64)] + \
               [("peak_bytes", C.c_uint64), ("ready_at_arrival", C.c_int64), ("unserved", C.c_int64),
                ("seek_latency_p50_ms", C.c_double), ("seek_latency_p99_ms", C.c_double),
                ("main_rounds", C.c_int64), ("side_rounds", C.c_int64), ("main_frames", C.c_int64),
                ("main_round_s", C.c_double), ("idle_s", C.c_double), ("plan_s", C.c_double),
                ("launch_s", C.c_double), ("collect_s", C.c_double), ("key_installs", C.c_int64),
                ("warmed_streams", C.c_int64), ("warmup_s", C.c_double), ("aside_rounds", C.c_int64),
                ("prepare_s", C.c_double), ("follow_rounds", C.c_int64), ("seek_shortcuts", C.c_int64)]


class Frame(C.Structure):
    _fields_ = [
        ("y", C.POINTER(C.c_uint8)), ("cb", C.POINTER(C.c_uint8)), ("cr", C.POINTER(C.c_uint8)),
        ("y_stride", C.c_int32), ("c_stride", C.c_int32),
        ("width", C.c_int32), ("height", C.c_int32),
        ("timestamp_ns", C.c_int64), ("ring_slot", C.c_int32), ("keyframe", C.c_int32),
    ]


class SourceFrame(C.Structure):
    _fields_ = [
        ("handle", C.c_int64),
        ("y", C.POINTER(C.c_uint8)), ("cb", C.POINTER(C.c_uint8)), ("cr", C.POINTER(C.c_uint8)),
        ("y_stride", C.c_int32), ("c_stride", C.c_int32),
        ("width", C.c_int32), ("height", C.c_int32),
        ("timestamp_ns", C.c_int64), ("frame_index", C.c_int64), ("keyframe", C.c_int32),
        ("rgba", C.POINTER(C.c_uint8)),
    ]


def _sig(lib, name, res, *args):
    f = getattr(lib, name)
    f.restype = res
    f.argtypes = list(args)


def lib() -> C.CDLL:
    """Returns the loaded native library, raising if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise ImportError(f"{LIB_PATH} is missing: build the GB300 decoder first (python -m govid_gb300.build)")
    L = C.CDLL(str(LIB_PATH))
    P, S, I, I64, U8P = C.c_void_p, C.c_size_t, C.c_int, C.c_int64, C.POINTER(C.c_uint8)
    PP = C.POINTER(C.c_void_p)
    # decoder
    _sig(L, "ebivgpu_create", I, I, PP)
    _sig(L, "ebivgpu_decode", I, P, C.c_char_p, S, I64, C.POINTER(Frame))
    _sig(L, "ebivgpu_flush", None, P)
    _sig(L, "ebivgpu_destroy", None, P)
    _sig(L, "ebivgpu_frame_rgba", I, P, I, U8P, S)
    _sig(L, "ebivgpu_codec_launches", I64, P)
    _sig(L, "ebivgpu_set_rgba", I, P, I)
    _sig(L, "ebivgpu_frame_rgba_pooled", C.c_void_p, P, I)
    _sig(L, "ebivgpu_status_string", C.c_char_p, I)
    _sig(L, "ebivgpu_device_available", I)
    _sig(L, "ebivgpu_abi_sizes", I, C.POINTER(S), I)
    # batch
    _sig(L, "ebivgpu_batch_create", I, PP)
    _sig(L, "ebivgpu_batch_destroy", None, P)
    _sig(L, "ebivgpu_batch_add_stream", I, P, C.POINTER(C.c_char_p), C.POINTER(S), I, I, C.POINTER(I))
    _sig(L, "ebivgpu_batch_add_streaming", I, P, I, C.POINTER(I))
    _sig(L, "ebivgpu_batch_submit", I, P, I, C.c_char_p, S)
    _sig(L, "ebivgpu_batch_seek", I, P, I, I64)
    _sig(L, "ebivgpu_batch_set_active", I, P, I, I)
    _sig(L, "ebivgpu_batch_remove_stream", I, P, I)
    _sig(L, "ebivgpu_batch_remaining", I64, P, I)
    _sig(L, "ebivgpu_batch_round", I, P, C.POINTER(I))
    _sig(L, "ebivgpu_batch_round_for", I, P, C.POINTER(I), I, C.POINTER(I))
    _sig(L, "ebivgpu_batch_result_count", I, P)
    _sig(L, "ebivgpu_batch_result", I, P, I, C.POINTER(I), C.POINTER(I64), C.POINTER(I), C.POINTER(I))
    _sig(L, "ebivgpu_batch_result_planes", I, P, I, C.POINTER(PlaneView))
    _sig(L, "ebivgpu_batch_result_download", I, P, I, U8P, S)
    _sig(L, "ebivgpu_batch_timing", I, P, I, C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_double))
    _sig(L, "ebivgpu_batch_set_lookahead", I, P, I)
    _sig(L, "ebivgpu_batch_set_pipeline", I, P, I)
    _sig(L, "ebivgpu_batch_set_tuning", I, P, I, I)
    _sig(L, "ebivgpu_batch_reload_stream", I, P, I, C.POINTER(C.c_void_p), C.POINTER(S), I)
    _sig(L, "ebivgpu_batch_result_download_async", I, P, I, C.c_void_p, S)
    _sig(L, "ebivgpu_batch_sync", I, P)
    _sig(L, "ebivgpu_batch_drain", I, P, C.POINTER(I))
    _sig(L, "ebivgpu_batch_launches", I64, P)
    _sig(L, "ebivgpu_batch_device_bytes", C.c_uint64, P)
    _sig(L, "ebivgpu_stream_footprint", C.c_uint64, I, I, I, I)
    # serving
    _sig(L, "ebivgpu_server_create", I, C.POINTER(ServeOptions), PP)
    _sig(L, "ebivgpu_server_stream_footprint", C.c_uint64, C.POINTER(ServeOptions), I, I, C.c_uint64)
    _sig(L, "ebivgpu_server_request_log", I64, P, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, I64)
    _sig(L, "ebivgpu_server_add_stream", I, P, C.POINTER(C.c_char_p), C.POINTER(S), I, C.c_double, I)
    _sig(L, "ebivgpu_server_run", I, P, C.POINTER(ServeStats))
    _sig(L, "ebivgpu_server_frame_hashes", I64, P, C.POINTER(C.c_int32), C.POINTER(I64), C.POINTER(C.c_uint64), I64)
    _sig(L, "ebivgpu_server_destroy", None, P)
    _sig(L, "ebivgpu_frame_hash", C.c_uint64, C.c_char_p, S)
    # learned motion-vector proposer
    F32P, I16P = C.POINTER(C.c_float), C.POINTER(C.c_int16)
    _sig(L, "ebiv_mvnet_create", I, I, I, I, I, C.c_uint64, PP)
    _sig(L, "ebiv_mvnet_destroy", None, P)
    _sig(L, "ebiv_mvnet_param_count", I)
    _sig(L, "ebiv_mvnet_get_params", I, P, F32P)
    _sig(L, "ebiv_mvnet_set_params", I, P, F32P)
    _sig(L, "ebiv_mvnet_exhaustive", I, P, U8P, U8P, I, I, I16P, C.POINTER(C.c_int32))
    _sig(L, "ebiv_mvnet_add_pair", I, P, U8P, U8P, I, I16P)
    _sig(L, "ebiv_mvnet_pairs", I, P)
    _sig(L, "ebiv_mvnet_set_input", I, P, I, U8P, U8P, I, I16P)
    _sig(L, "ebiv_mvnet_gather", I, P, C.POINTER(C.c_int32), I)
    _sig(L, "ebiv_mvnet_gradients", I, P, I, F32P, F32P)
    _sig(L, "ebiv_mvnet_train_step", I, P, I, C.c_float, F32P)
    _sig(L, "ebiv_mvnet_head", I, P, I, F32P)
    _sig(L, "ebiv_mvnet_propose", I, P, U8P, U8P, I, I16P)
    _sig(L, "ebiv_encoder_set_mvnet", I, P, P)
    # block analysis
    _sig(L, "ebivgpu_analysis_create", I, PP)
    _sig(L, "ebivgpu_analysis_destroy", None, P)
    _sig(L, "ebivgpu_fdct_satd", I, P, C.c_void_p, I, I, C.c_void_p, C.c_void_p, C.POINTER(C.c_double))
    # container ingest
    _sig(L, "ebivgpu_container_open", I, C.c_char_p, S, PP)
    _sig(L, "ebivgpu_container_close", None, P)
    _sig(L, "ebivgpu_container_info", I, P, C.POINTER(C.c_int64))
    _sig(L, "ebivgpu_container_entry", I, P, I, C.POINTER(C.c_uint64), C.POINTER(C.c_uint32), C.POINTER(I))
    _sig(L, "ebivgpu_container_seek", I, P, I64, C.POINTER(I64), C.POINTER(I64))
    _sig(L, "ebivgpu_batch_add_container", I, P, P, I, C.POINTER(I))
    # decode-ahead frame source
    SFP = C.POINTER(SourceFrame)
    _sig(L, "ebivgpu_source_create", I, C.c_char_p, S, I, I, PP)
    _sig(L, "ebivgpu_source_next", I, P, SFP)
    _sig(L, "ebivgpu_source_poll", I, P, SFP, C.POINTER(I))
    _sig(L, "ebivgpu_source_seek", I, P, I64, C.POINTER(I64))
    _sig(L, "ebivgpu_source_release", None, P, I64)
    _sig(L, "ebivgpu_source_close", I, P)
    _sig(L, "ebivgpu_source_destroy", None, P)
    _sig(L, "ebivgpu_source_decoded", I64, P)
    _sig(L, "ebivgpu_source_duration", I64, P)
    _sig(L, "ebivgpu_source_lookahead", I, P)
    # alt-ref temporal filter
    _sig(L, "ebivgpu_altref_create", I, PP)
    _sig(L, "ebivgpu_altref_destroy", None, P)
    _sig(L, "ebivgpu_altref_build", I, P, C.POINTER(C.c_char_p), I, I, I, I, U8P, S, C.POINTER(I))
    _sig(L, "ebivgpu_altref_time", I, P, I, I, C.POINTER(C.c_double))
    _sig(L, "ebivgpu_decode_key_noalloc", I, C.c_char_p, S, C.c_void_p, C.c_int32, S, C.c_void_p, C.c_void_p,
         C.c_int32, S, C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_int32))
    # encoder
    _sig(L, "ebiv_encoder_default_options", None, C.POINTER(EncoderOptions))
    _sig(L, "ebiv_encoder_create", I, C.POINTER(EncoderOptions), PP)
    _sig(L, "ebiv_encoder_write_frame", I, P, C.c_char_p, S)
    _sig(L, "ebiv_encoder_close", I, P)
    _sig(L, "ebiv_encoder_output", I, P, C.POINTER(U8P), C.POINTER(S))
    _sig(L, "ebiv_encoder_recon", I, P, I, U8P, S)
    _sig(L, "ebiv_encoder_recon_count", I, P)
    _sig(L, "ebiv_encoder_sad_evaluations", C.c_uint64, P)
    _sig(L, "ebiv_encoder_search_fallbacks", C.c_uint64, P)
    _sig(L, "ebiv_encoder_search_seconds", C.c_double, P)
    _sig(L, "ebiv_encoder_propose_seconds", C.c_double, P)
    _sig(L, "ebiv_encoder_set_candidates", I, P, C.POINTER(C.c_int16), I, I, I)
    _sig(L, "ebiv_encoder_destroy", None, P)
    # reader
    _sig(L, "ebiv_reader_open", I, C.c_char_p, S, PP)
    _sig(L, "ebiv_reader_info", I, P, C.POINTER(C.c_int64))
    _sig(L, "ebiv_reader_next_packet", I, P, C.POINTER(U8P), C.POINTER(S), C.POINTER(I64), C.POINTER(I))
    _sig(L, "ebiv_reader_packet", I, P, I, C.POINTER(U8P), C.POINTER(S), C.POINTER(I))
    _sig(L, "ebiv_reader_seek", I, P, I64, C.POINTER(I64))
    _sig(L, "ebiv_reader_duration", I64, P)
    _sig(L, "ebiv_reader_frame_time", I64, P, I64)
    _sig(L, "ebiv_reader_frame_index_at", I64, P, I64)
    _sig(L, "ebiv_reader_close", I, P)
    _sig(L, "ebiv_reader_destroy", None, P)
    _sig(L, "ebiv_parse_frame_header", I, C.c_char_p, S, C.POINTER(C.c_int32))
    # synthetic content
    _sig(L, "ebiv_synth_frame", I, I, I, I, U8P, S)
    _sig(L, "ebiv_synth_pan", I, I, I, I, U8P, S)
    _sig(L, "ebiv_scene_create", I, C.POINTER(C.c_int64), PP)
    _sig(L, "ebiv_scene_render", I, P, I, U8P, S)
    _sig(L, "ebiv_scene_destroy", None, P)
    _sig(L, "ebiv_encode_scene", I, C.POINTER(C.c_int64), I, C.POINTER(EncoderOptions), C.POINTER(U8P),
         C.POINTER(S))
    _sig(L, "ebiv_free", None, P)
    _sig(L, "ebiv_encode_key_from_levels", I, I, I, I, I, C.POINTER(C.c_int32), S, C.POINTER(U8P), C.POINTER(S))
    _sig(L, "ebiv_encode_block", I, C.POINTER(C.c_int32), I, I, I, U8P, S, C.POINTER(S), C.POINTER(C.c_uint32),
         U8P)
    _sig(L, "ebiv_encode_tokens", I, C.POINTER(C.c_uint16), I, U8P, S, C.POINTER(S), C.POINTER(C.c_uint32), U8P)
    _lib = L
    return L
