/*
 * ebivgpu — GB300 (sm_103a) EBIV decoder, C-ABI drop-in boundary.
 *
 * These entry points are what a cgo binding of govid's Codec contract calls.
 * Plain pointers and sizes only; no exceptions cross the boundary; every call
 * returns an ebiv status code.
 *
 * Reference interfaces replaced (govid, paths relative to its root):
 *   ebivgpu_create   <- ebiv.NewCodec(WithFrameRing(n))  ebiv/codec.go:48-64
 *   ebivgpu_decode   <- (*ebiv.Codec).Decode(govid.Packet) ebiv/codec.go:70-111
 *                       via govid.Codec.Decode             govid.go:41-44
 *   ebivgpu_flush    <- (*ebiv.Codec).Flush()              ebiv/codec.go:115-117
 *   ebivgpu_destroy  <- (garbage collection of the Codec)
 *   ebivgpu_frame_rgba <- govid.Frame.ConvertRGBA / RGBA   frame.go:72-91
 *   ebivgpu_set_rgba / ebivgpu_frame_rgba_pooled
 *                    <- govid.WithRGBA (pooled conversion)  source.go:61-74,131-150
 *   ebivgpu_batch_*  <- many independent Codec.Decode call chains at once
 *   ebivgpu_altref_* <- (*ebiv.Encoder).buildAltRef        ebiv/encoder.go:326-407
 *   ebivgpu_fdct_satd <- forwardDCT / satd                ebiv/transform.go:44-119
 *   ebivgpu_source_* <- govid asyncSource (NewAsyncPlayer's decode-ahead
 *                       frame source)                     source.go:84-266
 *   ebivgpu_container_* <- ebiv.NewDemuxer index load, Reader.Seek
 *                                                       ebiv/reader.go:32-160,222-238
 *                       (no single reference counterpart; the reference runs
 *                       one Codec per stream)
 */
#ifndef EBIVGPU_H
#define EBIVGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes: one per ebiv error sentinel (ebiv/format.go:110-119), plus
 * the boundary's own. */
enum {
  EBIV_OK = 0,
  EBIV_ERR_CORRUPT = 1,      /* ebiv.ErrCorrupt */
  EBIV_ERR_NOKEYFRAME = 2,   /* ebiv.ErrNoKeyframe */
  EBIV_ERR_DIMENSIONS = 3,   /* ebiv.ErrDimensions */
  EBIV_ERR_UNSUPPORTED = 4,  /* ebiv.ErrUnsupported */
  EBIV_ERR_VERSION = 5,      /* ebiv.ErrVersion */
  EBIV_ERR_BADMAGIC = 6,     /* ebiv.ErrBadMagic */
  EBIV_ERR_CONFIG = 7,       /* ebiv.ErrConfig */
  EBIV_ERR_WRITER_CLOSED = 8,/* ebiv.ErrWriterClosed */
  EBIV_ERR_EOF = 9,          /* io.EOF from a demuxer */
  EBIV_ERR_IO = 10,
  EBIV_ERR_DEVICE = 11,      /* CUDA failure or no usable GPU */
  EBIV_ERR_ARG = 12,         /* invalid argument at the boundary */
  EBIV_ERR_TOO_LARGE = 13    /* frame or packet beyond ebivgpu_decode_key_noalloc's fixed scratch */
};

typedef struct ebivgpu_codec ebivgpu_codec;

/* A decoded frame: host-visible 4:2:0 planes owned by the codec's ring
 * (valid for `ring` further decodes, as in ebiv/codec.go:15-22), strides
 * aligned to 64 bytes (ebiv/geometry.go:22-49). */
typedef struct {
  const uint8_t* y;
  const uint8_t* cb;
  const uint8_t* cr;
  int32_t y_stride, c_stride;
  int32_t width, height;
  int64_t timestamp_ns;
  int32_t ring_slot;
  int32_t keyframe;
} ebivgpu_frame;

/* Creates a codec on the current CUDA device; ring >= 2 (else 3). */
int ebivgpu_create(int ring, ebivgpu_codec** out);
/* Decodes one packet.  The packet bytes are consumed before return, so the
 * caller may reuse them (govid.Packet.Data aliases a reused buffer,
 * ebiv/reader.go:186-188). */
int ebivgpu_decode(ebivgpu_codec* c, const uint8_t* pkt, size_t n, int64_t ts_ns, ebivgpu_frame* out);
void ebivgpu_flush(ebivgpu_codec* c);
void ebivgpu_destroy(ebivgpu_codec* c);
/* YCbCr -> RGBA (BT.601 fixed point, frame.go:8-67) of the frame in ring
 * slot `slot`, computed on the GPU; dst holds width*height*4 bytes. */
int ebivgpu_frame_rgba(ebivgpu_codec* c, int slot, uint8_t* dst, size_t cap);
/* WithRGBA (source.go:61-74): with enable != 0 every later successful
 * decode also converts the frame to RGBA on the GPU (BT.601 fixed point,
 * frame.go:8-67), from the frame's device planes in the same decode round,
 * into a pinned buffer pooled per ring slot.  ebivgpu_frame_rgba_pooled
 * returns that buffer (width*height*4 bytes) for the frame in ring slot
 * `slot`, or NULL when the slot's frame was decoded without it.  The buffer
 * lives as long as the frame: ring-size further decodes (with a ring of 3 or
 * more, past govid's "second frame change" lifetime of WithRGBA buffers). */
int ebivgpu_set_rgba(ebivgpu_codec* c, int enable);
const uint8_t* ebivgpu_frame_rgba_pooled(ebivgpu_codec* c, int slot);
/* Kernel launches this codec has issued (for launch accounting). */
int64_t ebivgpu_codec_launches(ebivgpu_codec* c);
const char* ebivgpu_status_string(int status);

/* ---- Batched decode of many independent streams --------------------------
 * A batch holds streams whose packets are resident in HBM (add_stream) or fed
 * one packet per round (add_streaming + submit).  Each round decodes the next
 * packet of every active stream with one set of kernel launches; decoded
 * frames stay in the stream's device frame pool (valid for `ring` further
 * frames of that stream). */
typedef struct ebivgpu_batch ebivgpu_batch;
typedef struct {
  const uint8_t* y;   /* device pointers */
  const uint8_t* cb;
  const uint8_t* cr;
  int32_t y_stride, c_stride;
  int32_t width, height;
} ebivgpu_plane_view;

int ebivgpu_batch_create(ebivgpu_batch** out);
void ebivgpu_batch_destroy(ebivgpu_batch* b);
int ebivgpu_batch_add_stream(ebivgpu_batch* b, const uint8_t* const* pkts, const size_t* lens, int n, int ring,
                             int* stream_id);
int ebivgpu_batch_add_streaming(ebivgpu_batch* b, int ring, int* stream_id);
int ebivgpu_batch_submit(ebivgpu_batch* b, int stream_id, const uint8_t* pkt, size_t n);
/* Repositions a resident stream at a packet index (seek to a key frame). */
int ebivgpu_batch_seek(ebivgpu_batch* b, int stream_id, int64_t packet_index);
int ebivgpu_batch_set_active(ebivgpu_batch* b, int stream_id, int active);
int ebivgpu_batch_remove_stream(ebivgpu_batch* b, int stream_id);
int64_t ebivgpu_batch_remaining(ebivgpu_batch* b, int stream_id);
/* One round over every active stream; *frames = frames attempted. */
int ebivgpu_batch_round(ebivgpu_batch* b, int* frames);
int ebivgpu_batch_round_for(ebivgpu_batch* b, const int* stream_ids, int count, int* frames);
int ebivgpu_batch_result_count(ebivgpu_batch* b);
int ebivgpu_batch_result(ebivgpu_batch* b, int i, int* stream_id, int64_t* frame_index, int* status, int* keyframe);
int ebivgpu_batch_result_planes(ebivgpu_batch* b, int i, ebivgpu_plane_view* out);
int ebivgpu_batch_result_download(ebivgpu_batch* b, int i, uint8_t* packed, size_t cap);
/* enable: 1 on (resets counters), 0 off, -1 read only. */
int ebivgpu_batch_timing(ebivgpu_batch* b, int enable, double* kernel_ms, double* entropy_ms, double* recon_ms);
/* Frames per resident stream per round (default 1).  Entropy decoding of
 * later frames needs no pixels of earlier ones, so a round decodes all their
 * tiles in one launch and reconstructs the frames in order.  Set it before
 * adding streams. */
int ebivgpu_batch_set_lookahead(ebivgpu_batch* b, int frames);
/* Pipelined rounds (set before adding streams; resident streams only).
 * depth 1: each ebivgpu_batch_round starts the new round's entropy stage,
 * collects the round in flight and returns ITS results, so one round's
 * entropy overlaps the previous round's reconstruction.  depth D (2 or 3):
 * rounds are planned D calls ahead of their results, so a round's entropy
 * stage has the D previous rounds' reconstruction to run under.  depth 0:
 * the synchronous rounds.  ebivgpu_batch_drain collects every round in
 * flight.  Results and frame order per stream are those of the synchronous
 * rounds. */
int ebivgpu_batch_set_pipeline(ebivgpu_batch* b, int depth);
/* Launch shapes, the knobs the autotuner (govid_gb300/autotune.py) searches:
 * the most entropy launches a pipelined round splits its frames into (1 to
 * 4, default 4) and the warps per CTA of the intra stage (4, 8 or 16; 0, the
 * default, picks by the tile count).  Results do not depend on them. */
int ebivgpu_batch_set_tuning(ebivgpu_batch* b, int entropy_groups, int intra_warps);
/* Replaces a resident stream's packets with a new clip of the same size
 * (starting with a key frame) and rewinds it; its frame pool is kept.  No
 * round may be in flight (drain first); the copies from pkts (pinned memory
 * makes them asynchronous) complete before the next round's decode.  The
 * pkts buffers must stay unchanged until ebivgpu_batch_sync returns (or the
 * batch is destroyed). */
int ebivgpu_batch_reload_stream(ebivgpu_batch* b, int stream_id, const uint8_t* const* pkts, const size_t* lens,
                                int n);
/* Queues a result's packed-plane copy to host memory without waiting;
 * ebivgpu_batch_sync waits for every queued copy and for the copies of the
 * last ebivgpu_batch_reload_stream.  A result's frame stays
 * valid until `ring` newer frames of its stream are returned. */
int ebivgpu_batch_result_download_async(ebivgpu_batch* b, int index, uint8_t* packed, size_t cap);
int ebivgpu_batch_sync(ebivgpu_batch* b);
int ebivgpu_batch_drain(ebivgpu_batch* b, int* frames);
int64_t ebivgpu_batch_launches(ebivgpu_batch* b);
uint64_t ebivgpu_batch_device_bytes(ebivgpu_batch* b);
/* HBM bytes one stream of this geometry holds (frame pool + scratch). */
uint64_t ebivgpu_stream_footprint(int width, int height, int ring, int lookahead);
/* ---- Serving loop --------------------------------------------------------
 * Continuous batching of per-frame requests from many streams: each stream
 * issues requests as a Poisson process at its frame rate; a decode thread
 * keeps every admitted stream up to decode_ahead frames ahead of its
 * requests, all streams' next frames (max_frames_per_round each) in shared
 * rounds, key frames with long entropy chains on a side lane; decode_lanes
 * such threads, each with its own engine, split the streams; requests are
 * served in order as their frames are ready (latency: arrival to hand-out,
 * zero wait when the frame was decoded before it was asked for); seeks go
 * to key frames (frames decoded for the old position are dropped), looping
 * streams continue from their first frame; streams are admitted while their
 * HBM footprints fit the budget and release it when they finish.  No single
 * reference counterpart: the reference serves one Player per stream, each
 * an AsyncPlayer decoding ahead (player.go, source.go). */
typedef struct ebivgpu_server ebivgpu_server;
typedef struct {
  double duration_s;           /* requests arrive during this many seconds */
  int64_t frames_per_stream;   /* requests per stream at most */
  double seek_prob;            /* fraction of requests that are seeks */
  uint64_t seed;
  uint64_t hbm_budget_bytes;   /* admission cap on frame state */
  int32_t max_frames_per_round;/* per stream, when it fell behind */
  int32_t ring;
  int32_t record;              /* hash every delivered frame (testing) */
  int32_t key_lane;            /* side lanes for key frames with long entropy chains beside the main rounds (0 = none, 1-4) */
  double start_spread_s;       /* streams admitted at start begin uniformly within this many seconds */
  int32_t decode_ahead;        /* frames decoded ahead of each stream's requests (0: twice max_frames_per_round) */
  int32_t decode_lanes;        /* engines decoding side by side, each with its own thread and side lane (0: 1) */
  int32_t long_key_mbs;        /* key frames whose largest tile has more macroblocks use the side lanes (0: 1500) */
  int32_t key_cache;           /* streams with such key frames: 1 keep each decoded key frame (image, golden,
                                  table history) and install it at a seek or when reached again instead of
                                  decoding it, and fill the caches in the background on side lanes nobody
                                  waits on; 2 also decode all of them at admission, before the stream's
                                  requests start (for the streams admitted at start, before the request
                                  clock starts: a preparation step reported as prepare_s); 3 as 2 for every
                                  stream (0: off) */
} ebivgpu_serve_options;
typedef struct {
  int64_t requests, frames, errors, seeks, loops, rounds;
  int64_t admitted_total, admitted_peak, waiting_at_end;
  double elapsed_s, latency_p50_ms, latency_p99_ms, latency_max_ms, latency_mean_ms, frames_per_s, kernel_ms;
  double entropy_ms, recon_ms; /* kernel_ms split: entropy stage, reconstruction stages */
  int64_t key_frames;          /* key frames decoded (stream starts, seeks, loops) */
  uint64_t peak_bytes;
  int64_t ready_at_arrival;    /* requests whose frame was decoded before they arrived */
  int64_t unserved;            /* requests past the end of a clip that does not loop */
  double seek_latency_p50_ms, seek_latency_p99_ms; /* requests that were seeks */
  int64_t main_rounds, side_rounds, main_frames;    /* rounds of the decode thread, frames of main rounds */
  double main_round_s, idle_s;  /* decode threads: time inside main rounds, time with nothing to decode */
  double plan_s, launch_s, collect_s; /* main rounds: host planning, launches, waiting for the GPU */
  int64_t key_installs, warmed_streams; /* key frames served from the key cache; streams warmed at admission */
  double warmup_s;             /* summed admission-to-first-request time of the warmed streams */
  int64_t aside_rounds;        /* side-lane rounds that filled key caches in the background */
  double prepare_s;            /* key_cache 2: key frames of the streams admitted at start, before the first request */
  int64_t follow_rounds;       /* side rounds that decoded the frame after an installed seek target */
  int64_t seek_shortcuts;      /* seeks answered at once from a stream whose key frames are all cached */
} ebivgpu_serve_stats;
int ebivgpu_server_create(const ebivgpu_serve_options* o, ebivgpu_server** out);
int ebivgpu_server_add_stream(ebivgpu_server* s, const uint8_t* const* pkts, const size_t* lens, int n, double fps,
                              int loop);
int ebivgpu_server_run(ebivgpu_server* s, ebivgpu_serve_stats* out);
/* (stream index in add order, frame index, FNV-1a of the packed planes) per
 * delivered frame when record was set; returns the total count. */
int64_t ebivgpu_server_frame_hashes(ebivgpu_server* s, int32_t* stream, int64_t* frame, uint64_t* hash, int64_t cap);
/* Every delivered request in delivery order: arrival time (s from the start
 * of the request clock), latency (ms), stream (add order), frame index, and
 * whether it was a seek; any array may be NULL; returns the total count. */
int64_t ebivgpu_server_request_log(ebivgpu_server* s, double* arrival_s, double* latency_ms, int32_t* stream,
                                   int64_t* frame, int32_t* seek, int64_t cap);
void ebivgpu_server_destroy(ebivgpu_server* s);
/* FNV-1a 64 of a buffer (the hash the server records). */
uint64_t ebivgpu_frame_hash(const uint8_t* packed, size_t n);
/* The HBM footprint a server with options o admits a stream of this geometry
 * by: its frame pool and decode slots, plus packet_bytes of resident packets
 * (each packet rounded up to 16 bytes); a stream with a key cache adds two
 * frame images per key frame. */
uint64_t ebivgpu_server_stream_footprint(const ebivgpu_serve_options* o, int width, int height, uint64_t packet_bytes);

/* ---- Key-frame decode without device allocation ---------------------------
 * No reference counterpart: govid allocates its frame buffers on first use
 * (ebiv/codec.go:129-153).  This entry point is for callers that must not
 * allocate device memory on their decode path: a presentation thread with a
 * frame deadline (cudaMalloc/cudaFree can synchronise the device), or a
 * process whose device memory is fixed at start-up.
 *
 * Decodes one key-frame packet, as the first frame of a fresh stream (the
 * result and status equal ebivgpu_decode's on a new codec), into the caller's
 * device planes.  All scratch is one static device array of
 * EBIVGPU_NOALLOC_SCRATCH_BYTES (8,490,496) bytes per device, held by every
 * device that loads the library until the process exits, so frames are
 * limited to EBIVGPU_NOALLOC_MAX_MBS macroblocks
 * (1280x720) and packets to EBIVGPU_NOALLOC_MAX_PACKET bytes; larger ones
 * return EBIV_ERR_TOO_LARGE.  The planes must cover the macroblock-aligned
 * frame: y_stride >= 16*ceil(W/16) and y_cap >= y_stride*16*ceil(H/16);
 * c_stride >= 8*ceil(W/16) and c_cap >= c_stride*8*ceil(H/16).  Bytes beyond
 * the visible W x H are scratch.  With y == NULL the call only reports W and H.
 * Runs on cuda_stream (a cudaStream_t; NULL = the legacy default stream) and
 * returns when the frame is decoded.  Inter frames return EBIV_ERR_NOKEYFRAME;
 * a key frame coded as inter (it would predict from a new codec's zeroed
 * references; the encoder never writes one) returns EBIV_ERR_UNSUPPORTED.
 *
 * The first call on a device resolves the scratch's address and uploads the
 * decoder's constant tables; make it before any stream capture.  Calls that
 * overlap in time on one device share the scratch and race: serialise them.
 * A CUDA error already pending in the calling thread makes the call return
 * EBIV_ERR_DEVICE before it launches anything, leaving that error in place. */
#define EBIVGPU_NOALLOC_MAX_MBS 3600
#define EBIVGPU_NOALLOC_MAX_PACKET (2u << 20)
#define EBIVGPU_NOALLOC_SCRATCH_BYTES 8490496u
int ebivgpu_decode_key_noalloc(const uint8_t* pkt, size_t n, uint8_t* y, int32_t y_stride, size_t y_cap, uint8_t* cb,
                               uint8_t* cr, int32_t c_stride, size_t c_cap, void* cuda_stream, int32_t* width,
                               int32_t* height);

/* ---- Container ingest on the GPU -------------------------------------------
 * Replaces ebiv.NewDemuxer's index load and Reader.Seek
 *   ebiv/reader.go:32-160 (readIndex / scanFrames), ebiv/reader.go:222-238
 * for a decode that reads the container in place.
 *
 * ebivgpu_container_open copies the container once into pinned host memory
 * mapped into the device, checks the file header (ebiv/format.go:230-265),
 * and builds the frame index on the GPU: the footer's CRC-checked index, or
 * a scan of the frame records when the footer does not validate (statuses as
 * NewDemuxer's).  info6: width, height, fps_num, fps_den, frames, index
 * rebuilt by scanning (0/1).  ebivgpu_container_entry: frame i's payload
 * offset in the container, payload size, key flag; EBIV_ERR_IO for an index
 * entry whose payload lies outside the container (an offset near 2^64 passes
 * validateEntry's wrapping sum, ebiv/reader.go:115-123, and the reference's
 * NextPacket then fails, reader.go:203-205).  ebivgpu_container_seek
 * resolves Seek(t) on the GPU: the last key frame at or before the frame
 * shown at t (frameIndexAt, ebiv/format.go:263-275) and its time; a frame
 * rate so hostile that frameIndexAt's correction walk does not settle within
 * 2^20 steps returns EBIV_ERR_CORRUPT.  ebivgpu_batch_add_container adds a
 * resident batch stream that decodes straight from the pinned bytes: no
 * packet is copied into HBM, the kernels read them over the host link; the
 * container must outlive the stream, and one with an unreadable entry is
 * refused (EBIV_ERR_IO). */
typedef struct ebivgpu_container ebivgpu_container;
int ebivgpu_container_open(const uint8_t* data, size_t n, ebivgpu_container** out);
void ebivgpu_container_close(ebivgpu_container* c);
int ebivgpu_container_info(ebivgpu_container* c, int64_t* info6);
int ebivgpu_container_entry(ebivgpu_container* c, int i, uint64_t* payload_offset, uint32_t* size, int* keyframe);
int ebivgpu_container_seek(ebivgpu_container* c, int64_t t_ns, int64_t* frame, int64_t* landed_ns);
int ebivgpu_batch_add_container(ebivgpu_batch* b, ebivgpu_container* c, int ring, int* stream_id);

/* ---- Alt-ref temporal filter on the GPU ------------------------------------
 * Replaces (*ebiv.Encoder).buildAltRef   ebiv/encoder.go:326-407
 * (the encoder's golden-override image of a GOP, built when WithAltRef is on).
 *
 * frames: count host pointers to tightly packed 4:2:0 frames (Y W*H, Cb and
 * Cr CW*CH each), the GOP in order; the first min(window, count) are
 * filtered.  On success *accepted is the number of (frame, block) pairs that
 * agreed with the GOP head; 0 means no alt-ref (the reference returns nil:
 * window below 3 frames, or nothing agreed) and out is left untouched;
 * otherwise out receives the packed image (cap >= W*H + 2*CW*CH).  The
 * handle keeps its device buffers between calls (one caller at a time). */
typedef struct ebivgpu_altref ebivgpu_altref;
int ebivgpu_altref_create(ebivgpu_altref** out);
void ebivgpu_altref_destroy(ebivgpu_altref* a);
int ebivgpu_altref_build(ebivgpu_altref* a, const uint8_t* const* frames, int count, int width, int height,
                         int window, uint8_t* out, size_t cap, int* accepted);
/* Mean device time (CUDA events) of the filter kernel over reps runs on the
 * frames of the last ebivgpu_altref_build call, already resident. */
int ebivgpu_altref_time(ebivgpu_altref* a, int window, int reps, double* kernel_ms);

/* ---- The encoder's block analysis on the GPU -------------------------------
 * Replaces forwardDCT and satd   ebiv/transform.go:44-119
 * over a batch of blocks (the inner loops of the encoder's rate-distortion
 * search).  residuals: count row-major n x n int32 blocks (n = 4, 8, 16) in
 * host memory; coeffs (count*n*n int32) receives each block's forward DCT
 * and satd (count int64) its Hadamard cost; either may be NULL.  kernel_ms
 * (optional) receives the kernel's device time.  One caller at a time per
 * handle. */
typedef struct ebivgpu_analysis ebivgpu_analysis;
int ebivgpu_analysis_create(ebivgpu_analysis** out);
void ebivgpu_analysis_destroy(ebivgpu_analysis* a);
int ebivgpu_fdct_satd(ebivgpu_analysis* a, const int32_t* residuals, int n, int count, int32_t* coeffs, int64_t* satd,
                      double* kernel_ms);

/* ---- Decode-ahead frame source (govid.NewAsyncPlayer) -----------------------
 * Replaces asyncSource   source.go:84-266 (newAsyncSource, run, next, poll,
 * seek, release, close), the frame source of NewAsyncPlayer(d, c, depth,
 * WithRGBA)   player.go:40-57, with its demuxer (ebiv.NewDemuxer,
 * ebiv/reader.go:32-258) and codec (ebiv.NewCodec, ebiv/codec.go:48-192).
 *
 * The source copies the container, keeps its packets resident on the GPU
 * and decodes ahead of the consumer on a native worker thread: frames are
 * decoded min(depth, 32) at a time in pipelined rounds, copied to pinned
 * host memory (with EBIVGPU_SOURCE_RGBA also converted to RGBA on the GPU,
 * BT.601 fixed point, frame.go:8-67) and queued, up to depth frames.
 *
 * next blocks until a frame or a terminal status is available; poll returns
 * at once (*ready 0: nothing yet).  A status other than EBIV_OK is
 * EBIV_ERR_EOF at the end of the stream or the decode error of the next
 * frame; the worker then parks until a seek (readNextFrame's error,
 * source.go:164-170), and later calls return the same status.  After close,
 * next and poll return EBIV_ERR_EOF.  seek: a new generation (frames decoded
 * before it are never returned), the stream repositioned at the last key
 * frame at or before t (Seek, ebiv/reader.go:222-238), *landed_ns its time.
 * A returned frame's planes (strides width and (width+1)/2) and RGBA stay
 * valid until ebivgpu_source_release(handle).  A consumer holding so many
 * frames that none can be decoded (more than depth + lookahead + 4) gets
 * EBIV_ERR_ARG from next and poll rather than a wait that never ends (the
 * worker resumes at the next release).  close returns once
 * the worker has stopped; destroy frees everything, returned frames
 * included.  ebivgpu_source_decoded counts frames the worker has decoded. */
#define EBIVGPU_SOURCE_RGBA 1
typedef struct ebivgpu_source ebivgpu_source;
typedef struct {
  int64_t handle;
  const uint8_t* y;
  const uint8_t* cb;
  const uint8_t* cr;
  int32_t y_stride, c_stride;
  int32_t width, height;
  int64_t timestamp_ns;
  int64_t frame_index;
  int32_t keyframe;
  const uint8_t* rgba; /* width*height*4 bytes with EBIVGPU_SOURCE_RGBA, else NULL */
} ebivgpu_source_frame;
int ebivgpu_source_create(const uint8_t* container, size_t n, int depth, int flags, ebivgpu_source** out);
int ebivgpu_source_next(ebivgpu_source* s, ebivgpu_source_frame* f);
int ebivgpu_source_poll(ebivgpu_source* s, ebivgpu_source_frame* f, int* ready);
int ebivgpu_source_seek(ebivgpu_source* s, int64_t t_ns, int64_t* landed_ns);
void ebivgpu_source_release(ebivgpu_source* s, int64_t handle);
int ebivgpu_source_close(ebivgpu_source* s);
void ebivgpu_source_destroy(ebivgpu_source* s);
int64_t ebivgpu_source_decoded(ebivgpu_source* s);
int64_t ebivgpu_source_duration(ebivgpu_source* s);
int ebivgpu_source_lookahead(ebivgpu_source* s);

/* sizeof of the public structs, for bindings to check their layouts:
 * ebivgpu_frame, ebivgpu_plane_view, ebivgpu_serve_options,
 * ebivgpu_serve_stats, ebivgpu_source_frame (the first n); returns 5. */
int ebivgpu_abi_sizes(size_t* sizes, int n);

/* Non-zero when a CUDA device is usable from this process. */
int ebivgpu_device_available(void);

#ifdef __cplusplus
}
#endif
#endif
