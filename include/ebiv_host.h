/*
 * EBIV host tools C-ABI: the encoder, the container demuxer and the seeded
 * synthetic content generators that feed the GB300 decoder.  Plain pointers
 * and sizes only; every call returns an ebiv status code (see ebivgpu.h).
 *
 * Reference interfaces replaced (govid, paths relative to its root):
 *   ebiv_encoder_*  <- ebiv.NewEncoder / (*Encoder).WriteFrame / Close
 *                      (ebiv/encoder.go:128-176, 447-452) with the options
 *                      WithIntra/WithGOP/WithTiles/WithAutoTiles/WithAltRef/
 *                      WithFastEncode (ebiv/encoder.go:50-124)
 *   ebiv_reader_*   <- ebiv.NewDemuxer / (*Reader).NextPacket / Seek /
 *                      Duration / VideoInfo / Index (ebiv/reader.go:32-258),
 *                      the govid.Demuxer contract (govid.go:32-38)
 *   ebiv_synth_*    <- the test harness generators synthFrame / synthPan
 *                      (ebiv/harness_test.go:105-171) and the sprite scenes
 *                      of the decode workloads
 */
#ifndef EBIV_HOST_H
#define EBIV_HOST_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ebiv_encoder ebiv_encoder;
typedef struct ebiv_reader ebiv_reader;
typedef struct ebiv_scene ebiv_scene;

/* Encoder options.  coded=0 writes lossless raw key frames (the reference's
 * default); with_tiles_cols/rows < 0 means WithTiles was not given. */
typedef struct {
  int32_t width, height;
  uint32_t fps_num, fps_den;
  int32_t tile_cols, tile_rows;           /* Config.TileCols / TileRows */
  int32_t with_tiles_cols, with_tiles_rows;
  int32_t coded;                          /* WithIntra */
  int32_t qp;
  int32_t gop;                            /* WithGOP */
  int32_t auto_tiles;                     /* WithAutoTiles */
  int32_t altref_window;                  /* WithAltRef */
  int32_t fast_encode;                    /* WithFastEncode */
  int32_t threads;                        /* host threads for tile fan-out */
  int32_t search;                         /* 0 diamond, 1 exhaustive, 2 proposed */
  int32_t exhaustive_range;               /* full-pel radius for search=1 */
  int32_t keep_recon;                     /* keep reconstructions */
  int32_t proposed_fallback_sad;          /* search=2: exhaustive when best SAD per 256 px exceeds this (0 never) */
} ebiv_encoder_options;

void ebiv_encoder_default_options(ebiv_encoder_options* o);
int ebiv_encoder_create(const ebiv_encoder_options* o, ebiv_encoder** out);
/* Frame as tightly packed planes: Y (w*h), Cb, Cr ((w+1)/2 * (h+1)/2 each). */
int ebiv_encoder_write_frame(ebiv_encoder* e, const uint8_t* packed, size_t n);
int ebiv_encoder_close(ebiv_encoder* e);
/* Container bytes written so far (complete after close). */
int ebiv_encoder_output(ebiv_encoder* e, const uint8_t** data, size_t* n);
int ebiv_encoder_recon(ebiv_encoder* e, int index, uint8_t* packed, size_t cap);
int ebiv_encoder_recon_count(ebiv_encoder* e);
uint64_t ebiv_encoder_sad_evaluations(ebiv_encoder* e);
/* Proposed searches (search=2) the exhaustive search decided. */
uint64_t ebiv_encoder_search_fallbacks(ebiv_encoder* e);
/* Thread seconds spent in motion search (summed over tile threads) and wall
 * seconds of the proposer's per-frame preparation (search=2). */
double ebiv_encoder_search_seconds(ebiv_encoder* e);
double ebiv_encoder_propose_seconds(ebiv_encoder* e);
/* Installs candidate motion vectors per macroblock for search=2: a table of
 * frames*mbs*k (x,y) int16 pairs in quarter pixels, frame-major, consumed in
 * inter-frame order. */
int ebiv_encoder_set_candidates(ebiv_encoder* e, const int16_t* mv, int frames, int mbs, int k);
void ebiv_encoder_destroy(ebiv_encoder* e);

/* Demuxer over an in-memory container (the bytes are copied). */
int ebiv_reader_open(const uint8_t* data, size_t n, ebiv_reader** out);
/* width, height, fps_num, fps_den, frame count, tile cols, tile rows, rebuilt */
int ebiv_reader_info(ebiv_reader* r, int64_t* info8);
/* NextPacket: *data stays valid until the reader is destroyed. */
int ebiv_reader_next_packet(ebiv_reader* r, const uint8_t** data, size_t* n, int64_t* ts_ns, int* keyframe);
/* ebiv_reader_next_packet and ebiv_reader_packet return EBIV_ERR_IO for an
 * index entry whose payload position, int64(Offset) + 8, is negative (an
 * offset near 2^64 passes validateEntry's wrapping sum, ebiv/reader.go:115-123;
 * the reference's seek then fails, reader.go:203-205); next_packet stays on
 * that entry. */
int ebiv_reader_packet(ebiv_reader* r, int index, const uint8_t** data, size_t* n, int* keyframe);
int ebiv_reader_seek(ebiv_reader* r, int64_t t_ns, int64_t* landed_ns);
int64_t ebiv_reader_duration(ebiv_reader* r);
int64_t ebiv_reader_frame_time(ebiv_reader* r, int64_t i);
/* frameIndexAt (ebiv/format.go:263-275); -1 for a frame rate so hostile that
 * its correction walk does not settle within 2^20 steps, where
 * ebiv_reader_seek returns EBIV_ERR_CORRUPT. */
int64_t ebiv_reader_frame_index_at(ebiv_reader* r, int64_t t_ns);
int ebiv_reader_close(ebiv_reader* r);
void ebiv_reader_destroy(ebiv_reader* r);

/* parseFrameHeader: info[0]=type, [1]=coding, [2]=width, [3]=height,
 * [4]=golden override, [5]=body offset. */
int ebiv_parse_frame_header(const uint8_t* pkt, size_t n, int32_t* info6);

/* Synthetic content into tightly packed planes. */
int ebiv_synth_frame(int w, int h, int seed, uint8_t* packed, size_t cap);
int ebiv_synth_pan(int w, int h, int seed, uint8_t* packed, size_t cap);
/* spec: width, height, seed, sprites, vel_max_q, integer_vel, pan_max_q,
 * flash_period, flash_start, flash_len, flash_amp, noise_y16, noise_c16 */
int ebiv_scene_create(const int64_t* spec13, ebiv_scene** out);
int ebiv_scene_render(ebiv_scene* s, int frame, uint8_t* packed, size_t cap);
void ebiv_scene_destroy(ebiv_scene* s);

/* Encodes `frames` frames of a sprite scene in one call (renders and encodes
 * on the host; threads parallelise tile encoding). */
int ebiv_encode_scene(const int64_t* spec13, int frames, const ebiv_encoder_options* o, uint8_t** out, size_t* n);
void ebiv_free(void* p);

/* Codes one n x n block of levels as the encoder codes a residual block:
 * sign-data hiding (ebiv/residual.go:134-180, levels are adjusted in place),
 * token grammar (ebiv/residual.go:30-75) and rANS (ebiv/rans.go:186-214)
 * with tables normalized from the block's own tokens.  freqs receives 16
 * entries per context (72 contexts), used one flag per context. */
int ebiv_encode_block(int32_t* levels, int n, int plane, int tx_idx, uint8_t* stream, size_t cap, size_t* len,
                      uint32_t* freqs, uint8_t* used);
/* One packet: a one-tile intra key frame of w x h whose macroblocks (raster
 * order) take their levels from `levels` — sixteen 4x4 luma blocks of 16
 * levels, then 64 Cb and 64 Cr levels, 384 per macroblock — all blocks with
 * intra mode `mode` (the token grammar of decodeLumaMB/decodeChromaMB,
 * ebiv/decode_intra.go:121-187, tables from the frame's own counts).  For
 * test streams with chosen coefficients.  *out is freed with ebiv_free. */
int ebiv_encode_key_from_levels(int w, int h, int qp, int mode, const int32_t* levels, size_t nlevels, uint8_t** out,
                                size_t* n);
/* rANS-codes `count` (context, symbol) pairs with tables normalized from
 * their own counts (ebiv/rans.go:46-85, 186-214). */
int ebiv_encode_tokens(const uint16_t* pairs, int count, uint8_t* stream, size_t cap, size_t* len, uint32_t* freqs,
                       uint8_t* used);

#ifdef __cplusplus
}
#endif
#endif
