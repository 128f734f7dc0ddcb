/* Learned motion-vector proposer for the EBIV encoder's inter search
 * (govid_gb300/csrc/mvnet_kernels.cu).  No reference counterpart: govid's
 * encoder searches with a diamond (ebiv/encode_inter.go:381-419); this net
 * proposes the candidates the encoder's search=2 mode evaluates instead.
 *
 * A 4-layer 3x3 conv net (2 -> 32 -> 32 -> 32 -> 34 channels, ReLU between)
 * on quarter-resolution luma of the current and reference frames; BF16
 * activations, FP32 accumulation, gradients and Adam state; trained on the
 * GPU against exhaustive full-pel SAD search labels. */
#ifndef EBIV_MVNET_H
#define EBIV_MVNET_H

#include <stddef.h>
#include <stdint.h>

#include "ebiv_host.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ebiv_mvnet ebiv_mvnet;

#define EBIV_MVNET_PARAMS 28930 /* FP32 parameters: per layer weights [out][in][3][3], then bias */
#define EBIV_MVNET_TOPK 8       /* candidates per 16x16 macroblock */

/* One net for frames whose padded luma is pad_width x pad_height (multiples
 * of 16).  max_batch frame pairs per training step; max_pairs examples in
 * the device-resident training set (0 for inference). */
int ebiv_mvnet_create(int max_batch, int pad_width, int pad_height, int max_pairs, uint64_t seed, ebiv_mvnet** out);
void ebiv_mvnet_destroy(ebiv_mvnet* n);
int ebiv_mvnet_param_count(void);
int ebiv_mvnet_get_params(ebiv_mvnet* n, float* out);
int ebiv_mvnet_set_params(ebiv_mvnet* n, const float* in); /* also resets the Adam state */
/* Exhaustive full-pel SAD search (|dx|,|dy| <= range <= 16) per macroblock of
 * the padded luma planes (stride >= pad_width): best (dx, dy) in full pels
 * and its SAD.  Ties prefer the zero vector, then raster order. */
int ebiv_mvnet_exhaustive(ebiv_mvnet* n, const uint8_t* cur, const uint8_t* ref, int stride, int range, int16_t* mv,
                          int32_t* sad);
/* Training set and batches: labels are full-pel (dx, dy) per macroblock. */
int ebiv_mvnet_add_pair(ebiv_mvnet* n, const uint8_t* cur, const uint8_t* ref, int stride, const int16_t* labels);
int ebiv_mvnet_pairs(ebiv_mvnet* n);
int ebiv_mvnet_set_input(ebiv_mvnet* n, int slot, const uint8_t* cur, const uint8_t* ref, int stride,
                         const int16_t* labels);
int ebiv_mvnet_gather(ebiv_mvnet* n, const int32_t* idx, int batch);
/* Forward, loss and backward over batch slots 0..batch-1.  stats3 = mean
 * loss, top-1 rate, top-8 rate.  gradients() returns the parameter gradients
 * without updating; train_step() applies one Adam step with rate lr. */
int ebiv_mvnet_gradients(ebiv_mvnet* n, int batch, float* grads, float* stats3);
int ebiv_mvnet_train_step(ebiv_mvnet* n, int batch, float lr, float* stats3);
/* Head logits of slots 0..batch-1, [batch][34][pad_height/4][pad_width/4]. */
int ebiv_mvnet_head(ebiv_mvnet* n, int batch, float* out);
/* Top-8 candidates per macroblock for one frame pair, [mbs][8][2] full pels. */
int ebiv_mvnet_propose(ebiv_mvnet* n, const uint8_t* cur, const uint8_t* ref, int stride, int16_t* cand);
/* Makes the net the candidate source of an encoder created with search=2;
 * the net must outlive the encode and match its padded size. */
int ebiv_encoder_set_mvnet(ebiv_encoder* e, ebiv_mvnet* n);

#ifdef __cplusplus
}
#endif

#endif
