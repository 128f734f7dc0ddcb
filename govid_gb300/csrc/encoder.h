// EBIV encoder (host C++).  It produces plain EBIV v4 bitstreams with the
// reference encoder's rate-distortion decisions (ebiv/encoder.go,
// ebiv/encode_intra.go, ebiv/encode_inter.go, ebiv/quant.go, ebiv/rans.go,
// ebiv/residual.go, ebiv/mv.go) and writes the container (ebiv/writer.go).
// It feeds the GPU decoder's tests and benchmarks and hosts the motion-vector
// proposal hook used by the learned inter search.
#pragma once

#include <cstdint>
#include <functional>
#include <memory>
#include <vector>

#include "ebiv_format.h"

namespace ebiv {

// A 4:2:0 image with tightly packed planes (strides W and CW).
struct PackedImage {
  int W = 0, H = 0, CW = 0, CH = 0;
  std::vector<uint8_t> Y, Cb, Cr;
  void alloc(int w, int h) {
    W = w;
    H = h;
    CW = (w + 1) / 2;
    CH = (h + 1) / 2;
    Y.assign((size_t)W * H, 0);
    Cb.assign((size_t)CW * CH, 0);
    Cr.assign((size_t)CW * CH, 0);
  }
};

struct MotionVector {
  int16_t x = 0, y = 0;
};

// Candidate motion vectors for one 16x16 macroblock, supplied by an external
// proposer (the learned inter search).  When a proposer is installed the
// encoder evaluates these candidates (plus the predictor and zero) with the
// same SAD and sub-pel refinement the diamond search uses, instead of walking
// the diamond.
struct MVProposer {
  virtual ~MVProposer() = default;
  // Called once per inter frame before its tiles encode.  src and ref are the
  // padded luma planes (stride = padded width).
  virtual void prepare(const uint8_t* src, const uint8_t* ref, int padW, int padH) = 0;
  // Writes up to max candidates for macroblock (mbx, mby); returns the count.
  virtual int candidates(int mbx, int mby, MotionVector* out, int max) const = 0;
};

enum class SearchMode { Diamond = 0, Exhaustive = 1, Proposed = 2 };

struct EncoderOptions {
  int width = 0, height = 0;
  uint32_t fpsNum = 30, fpsDen = 1;
  int tileCols = 0, tileRows = 0;  // Config.TileCols/TileRows (file header)
  int withTilesCols = -1;          // WithTiles(cols, rows); -1 = not given
  int withTilesRows = -1;
  bool coded = false;              // WithIntra
  int qp = 20;
  int gop = 1;                     // WithGOP
  int autoTiles = 0;               // WithAutoTiles
  int altRefWindow = 0;            // WithAltRef
  bool fastEncode = false;         // WithFastEncode
  int threads = 1;                 // host threads for tile fan-out
  SearchMode search = SearchMode::Diamond;
  int exhaustiveRange = 16;        // full-pel search radius for Exhaustive
  int proposedFallbackSAD = 0;     // Proposed: exhaustive search when the best SAD per 256 px exceeds this (0 = never)
  bool keepRecon = false;          // keep each written frame's reconstruction
};

class Encoder {
 public:
  explicit Encoder(const EncoderOptions& o);
  ~Encoder();
  int status() const { return status_; }
  int writeFrame(const PackedImage& img);
  int close();
  const std::vector<uint8_t>& output() const { return out_; }
  void setProposer(MVProposer* p) { proposer_ = p; }
  // Motion search statistics accumulated over the encode (SAD evaluations).
  uint64_t sadEvaluations() const;
  uint64_t searchFallbacks() const;  // proposed searches handed to the exhaustive search
  double searchSeconds() const;      // thread seconds in motion search (summed over tile threads)
  double proposeSeconds() const;     // wall seconds of the proposer's per-frame preparation
  int frameCount() const { return accepted_; }
  // Reconstructions (visible region) of the frames written so far, in
  // container order, when keepRecon was set.
  const std::vector<PackedImage>& recons() const { return recons_; }

 private:
  struct Impl;
  std::unique_ptr<Impl> impl_;
  EncoderOptions opt_;
  std::vector<uint8_t> out_;
  int status_ = kOK;
  int accepted_ = 0;
  MVProposer* proposer_ = nullptr;
  std::vector<PackedImage> recons_;
  int flushGOP();
  void keep(const void* frame);
  int gridCols() const;
  int gridRows() const;
};

// Single-block and token-stream coding hooks (see encoder.cpp).
int encodeBlockStream(int32_t* levels, int n, int plane, int txIdx, std::vector<uint8_t>* stream,
                      std::vector<uint32_t>* freqs, std::vector<uint8_t>* used);
int encodeKeyFromLevels(int w, int h, int qp, int mode, const int32_t* levels, size_t nlevels,
                        std::vector<uint8_t>* pkt);
int encodeTokenStream(const uint16_t* pairs, int count, std::vector<uint8_t>* stream, std::vector<uint32_t>* freqs,
                      std::vector<uint8_t>* used);

}  // namespace ebiv
