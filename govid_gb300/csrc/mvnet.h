// Learned motion-vector proposer (see mvnet_kernels.cu): the net's device
// state, its training entry points and the encoder's candidate source.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "encoder.h"

struct __nv_bfloat16;

namespace ebiv {
namespace mvnet {
constexpr int kInCh = 2;     // current and reference luma, quarter resolution
constexpr int kHidden = 32;  // channels of the three hidden layers
constexpr int kLayers = 4;   // 3x3 convolutions
constexpr int kRange = 16;   // full-pel displacement range of the proposals
constexpr int kBins = 17;    // per axis: -16, -14, ..., 16 full pels
constexpr int kHeadCh = 2 * kBins;
constexpr int kTopK = 8;     // candidates per macroblock
constexpr int kParams = (kHidden * kInCh * 9 + kHidden) + 2 * (kHidden * kHidden * 9 + kHidden) +
                        (kHeadCh * kHidden * 9 + kHeadCh);
}  // namespace mvnet

// One net instance for frames of one padded luma size (multiples of 16).
class MvNet {
 public:
  ~MvNet();
  // maxBatch: frame pairs per training step; maxPairs: capacity of the
  // device-resident training set (0 for inference only).
  int init(int maxBatch, int padW, int padH, int maxPairs, uint64_t seed);
  int setParams(const float* p);  // FP32 master parameters; resets Adam
  int getParams(float* p) const;
  // Best full-pel vector per macroblock by exhaustive SAD search in +-range.
  int exhaustive(const uint8_t* cur, const uint8_t* ref, int stride, int range, int16_t* mv, int32_t* sad);
  // Appends a (current, reference, labels) example to the training set.
  int addPair(const uint8_t* cur, const uint8_t* ref, int stride, const int16_t* labels);
  // Places one example directly in batch slot `slot` (labels may be null).
  int setInput(int slot, const uint8_t* cur, const uint8_t* ref, int stride, const int16_t* labels);
  // Fills batch slots 0..batch-1 with training-set examples idx[0..batch-1].
  int gather(const int* idx, int batch);
  // Forward + loss + backward on slots 0..batch-1 without an update; grads
  // gets the parameter gradients (may be null); stats = loss, top-1, top-8.
  int gradients(int batch, float* grads, float* stats);
  int trainStep(int batch, float lr, float* stats);  // forward, backward, Adam
  int headOutput(int batch, float* out);             // head logits [batch][34][h][w]
  int propose(int16_t* cand);                        // slot 0: [mbs][8][2] full pels
  int width() const { return W_; }
  int height() const { return H_; }
  int macroblocks() const { return mbs_; }
  int pairs() const { return pairs_; }

 private:
  int uploadPair(const uint8_t* cur, const uint8_t* ref, int stride, __nv_bfloat16* dst);
  void forward(int batch);
  void backward(int batch);
  int lossAndGrad(int batch, bool grad, float* stats);

  int B_ = 0, W_ = 0, H_ = 0, w_ = 0, h_ = 0, mbs_ = 0, maxPairs_ = 0, pairs_ = 0, step_ = 0;
  cudaStream_t stream_ = nullptr;
  std::vector<void*> allocs_;
  float *params_ = nullptr, *grads_ = nullptr, *adamM_ = nullptr, *adamV_ = nullptr;
  __nv_bfloat16 *pbf_ = nullptr, *wT_ = nullptr, *x0_ = nullptr;
  __nv_bfloat16* act_[mvnet::kLayers - 1] = {};
  float* gAct_[mvnet::kLayers - 1] = {};
  float *head_ = nullptr, *gHead_ = nullptr, *stats_ = nullptr;
  int16_t *labels_ = nullptr, *cand_ = nullptr, *mvs_ = nullptr, *dataLab_ = nullptr;
  int* idx_ = nullptr;
  int32_t* sads_ = nullptr;
  uint8_t* planes_ = nullptr;
  __nv_bfloat16* data_ = nullptr;
};

// The encoder's candidate source: runs the net on the frame pair once per
// inter frame and hands each macroblock its top-8 vectors.
class NetProposer : public MVProposer {
 public:
  explicit NetProposer(MvNet* net) : net_(net) {}
  void prepare(const uint8_t* src, const uint8_t* ref, int padW, int padH) override;
  int candidates(int mbx, int mby, MotionVector* out, int max) const override;
  bool ready() const { return ok_; }

 private:
  MvNet* net_;
  std::vector<int16_t> cand_;
  int mbCols_ = 1;
  bool ok_ = false;
};

}  // namespace ebiv
