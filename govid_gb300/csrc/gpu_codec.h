// Single-stream GB300 EBIV codec (host side).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "container.h"
#include "ebiv_format.h"
#include "payload.h"

namespace ebiv {

// Three padded device frame buffers: work, last reference, golden.
struct DeviceFrameSet {
  uint8_t* buf[3] = {nullptr, nullptr, nullptr};
  uint8_t* y[3] = {nullptr, nullptr, nullptr};
  uint8_t* cb[3] = {nullptr, nullptr, nullptr};
  uint8_t* cr[3] = {nullptr, nullptr, nullptr};
  size_t bytesPerFrame = 0;
  bool alloc(const Geometry& g);
  void release();
};

struct DecodedFrame {
  const uint8_t* y = nullptr;
  const uint8_t* cb = nullptr;
  const uint8_t* cr = nullptr;
  int yStride = 0, cStride = 0, width = 0, height = 0, slot = -1;
  bool keyframe = false;
};

int ensureDeviceTables();
size_t alignUp(size_t v, size_t a);

class GpuCodec {
 public:
  explicit GpuCodec(int ring);
  ~GpuCodec();
  int init();
  int decode(const uint8_t* pkt, size_t n, DecodedFrame* out);
  void flush();
  int rgba(int slot, uint8_t* dst, size_t cap);
  int64_t launches() const { return launches_; }
  const Geometry& geometry() const { return geo_; }
  // Device copy of the padded reference planes (0 = last reference,
  // 1 = golden), for side-effect checks.
  int copyReference(int which, uint8_t* dst, size_t cap);

 private:
  int configure(int w, int h);
  int ensureStage(size_t bytes);
  int runPayload(const uint8_t* pkt, size_t n, const PayloadPlan& plan, int rec, int ref, int gold, bool inter);
  int decodeCoded(const uint8_t* pkt, size_t n, const FrameHeader& fh, uint8_t* img);

  int ringSize_;
  cudaStream_t stream_ = nullptr;
  Geometry geo_;
  bool ready_ = false;
  std::vector<uint8_t*> ring_;
  int next_ = 0;
  DeviceFrameSet frames_;
  int work_ = 0, ref_ = 1, golden_ = 2, lastWork_ = -1;
  TableHistory hist_;
  uint8_t* dStage_ = nullptr;
  uint8_t* hStage_ = nullptr;
  size_t stageCap_ = 0;
  void* dRec_ = nullptr;
  uint32_t* dCoef_ = nullptr;
  int16_t* dMV_ = nullptr;
  void* dTileStat_ = nullptr;
  uint8_t* dRGBA_ = nullptr;
  size_t rgbaCap_ = 0;
  int64_t launches_ = 0;
};

}  // namespace ebiv
