// Single-stream GB300 EBIV codec (host side): the govid.Codec contract on top
// of the multi-stream engine with one streaming stream.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "container.h"
#include "ebiv_format.h"
#include "engine.h"

namespace ebiv {

struct DecodedFrame {
  const uint8_t* y = nullptr;
  const uint8_t* cb = nullptr;
  const uint8_t* cr = nullptr;
  int yStride = 0, cStride = 0, width = 0, height = 0, slot = -1;
  bool keyframe = false;
};

int ensureDeviceTables();

class GpuCodec {
 public:
  explicit GpuCodec(int ring);
  ~GpuCodec();
  int init();
  int decode(const uint8_t* pkt, size_t n, DecodedFrame* out);
  void flush();
  int rgba(int slot, uint8_t* dst, size_t cap);
  // WithRGBA (source.go:61-74): every later decode also produces the frame's
  // RGBA, kept in a pinned buffer per ring slot (valid as long as the frame).
  int setRGBA(bool on);
  const uint8_t* pooledRGBA(int slot) const;
  int ensureRGBA();
  int64_t launches() const { return eng_.launches() + extraLaunches_; }
  // Padded reference planes (0 = last reference, 1 = golden), packed.
  int copyReference(int which, uint8_t* dst, size_t cap);

 private:
  int ringSize_;
  Engine eng_;
  int sid_ = -1;
  Geometry geo_;
  bool ready_ = false;
  std::vector<uint8_t*> ring_;  // pinned host images, 64-byte aligned strides
  int next_ = 0;
  uint8_t* dRGBA_ = nullptr;
  size_t rgbaCap_ = 0;
  bool rgbaOn_ = false;
  std::vector<uint8_t*> rgbaRing_;  // pinned W*H*4 per ring slot (WithRGBA)
  std::vector<char> rgbaValid_;     // slot holds the RGBA of its current frame
  int64_t extraLaunches_ = 0;
  std::vector<RoundResult> results_;
};

}  // namespace ebiv
