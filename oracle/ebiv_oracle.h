/*
 * TEST INFRASTRUCTURE — the CPU oracle for the EBIV decode path.
 *
 * A line-faithful C++ restatement of govid's pure-Go EBIV decoder
 * (ebiv/codec.go, ebiv/decode_intra.go, ebiv/decode_inter.go, ebiv/rans.go,
 * ebiv/residual.go, ebiv/mv.go, ebiv/quant.go, ebiv/transform.go,
 * ebiv/predict.go, ebiv/motioncomp.go, ebiv/frame.go, ebiv/format.go) and of
 * govid's YCbCr->RGBA conversion (frame.go:8-67).
 *
 * Only the test suite, the smoke check and the benchmark's CPU-baseline leg
 * use this library, and only as the checker: the product decode path never
 * links or calls it.  Parity status: pinned against the reference's
 * known-answer tests restated in tests/ (sign-data-hiding vectors, rANS and
 * transform properties) and cross-checked against the product encoder's
 * reconstruction; the reference Go decoder cannot run here, so there are no
 * golden decoded planes produced by the reference itself.
 */
#ifndef EBIV_ORACLE_H
#define EBIV_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes, one per ebiv error sentinel (ebiv/format.go:110-119). */
enum {
  EO_OK = 0,
  EO_ERR_CORRUPT = 1,
  EO_ERR_NOKEYFRAME = 2,
  EO_ERR_DIMENSIONS = 3,
  EO_ERR_UNSUPPORTED = 4,
  EO_ERR_ARG = 100
};

typedef struct eo_codec eo_codec;

/* NewCodec(WithFrameRing(ring)) — ebiv/codec.go:48-64.  threads > 1 spreads
 * tiles over a worker pool the way ebiv/pool.go does. */
eo_codec* eo_codec_create(int ring, int threads);
void eo_codec_destroy(eo_codec* c);

/* Codec.Decode — ebiv/codec.go:70-111.  On success *slot receives the ring
 * index of the decoded image and *w, *h the stream geometry. */
int eo_codec_decode(eo_codec* c, const uint8_t* pkt, size_t n, int* slot, int* w, int* h);

/* Codec.Flush — ebiv/codec.go:115-117. */
void eo_codec_flush(eo_codec* c);
/* Test statistic: intra residual samples outside [-32768, 32767] that every
 * codec of the process has reconstructed (reset != 0 clears the count). */
long eo_wide_residuals(int reset);

/* Copies ring image `slot` out as tightly packed Y, Cb, Cr planes. */
int eo_codec_ring_image(eo_codec* c, int slot, uint8_t* packed, size_t cap);

/* Copies the padded work/ref/golden reference planes (0=ref, 1=golden) out,
 * packed Y then Cb then Cr at padded sizes; used by side-effect tests. */
int eo_codec_reference(eo_codec* c, int which, uint8_t* packed, size_t cap);

/* Decodes a whole packet sequence, writing each frame's packed planes to
 * out + i*frame_bytes.  statuses[i] receives each frame's status. */
int eo_decode_sequence(const uint8_t* const* pkts, const size_t* lens, int n,
                       int threads, uint8_t* out, size_t frame_bytes, int* statuses);

/* Decodes `nstreams` independent packet sequences with `threads` workers,
 * streams spread over workers (tiles serial within a stream).  Returns the
 * number of frames decoded without error; outputs are discarded (timing). */
long eo_decode_streams(const uint8_t* const* const* pkts, const size_t* const* lens,
                       const int* nframes, int nstreams, int threads);

/* convertYCbCr420ToRGBA — frame.go:8-67, on tightly packed planes. */
void eo_rgba(const uint8_t* y, const uint8_t* cb, const uint8_t* cr, int w, int h,
             uint8_t* dst);

/* Unit entry points for property tests. */
void eo_inverse_dct(const int32_t* src, int32_t* dst, int n);
void eo_zigzag(int n, int* order);
int eo_dct_matrix(int n, int32_t* out);
int eo_quant_steps(int qp, int32_t* dc, int32_t* ac);

/* Decodes one block of coefficient tokens from a rANS stream whose tables
 * are given as frequency vectors (freqs[c*16 + s], used[c]).  Returns the
 * decoder error status; levels receive the row-major block. */
int eo_decode_block(const uint8_t* stream, size_t n, const uint32_t* freqs,
                    const uint8_t* used, int plane, int tx_idx, int bn, int32_t* levels);

/* Decodes `count` symbols from the given contexts (ctxs[i]) — a raw rANS
 * round-trip probe.  Returns the decoder status. */
int eo_decode_symbols(const uint8_t* stream, size_t n, const uint32_t* freqs,
                      const uint8_t* used, const int* ctxs, int count, int* syms);

#ifdef __cplusplus
}
#endif
#endif
