// Single-stream GB300 EBIV codec: the govid.Codec contract (Decode / Flush,
// ebiv/codec.go:70-192) over the engine (engine.h) with one streaming stream.
// Each Decode plans the payload on the host, uploads the packet with the
// frame descriptors in one copy, runs the entropy / inter / intra kernels and
// copies the visible planes into the codec's host ring image; the ring cursor
// follows the reference (it advances before decoding, Flush resets it).
#include <cuda_runtime.h>

#include <cstring>
#include <memory>
#include <mutex>
#include <vector>

#include "../../include/ebivgpu.h"
#include "container.h"
#include "gpu_codec.h"
#include "gpu_types.h"
#include "payload.h"

namespace ebiv {

int uploadCodingTables(const int* scan4, const int* scan8, const int* scan16, const int32_t* dct);
void launchRGBA(const uint8_t* y, const uint8_t* cb, const uint8_t* cr, int ys, int cs, int w, int h, uint8_t* dst,
                cudaStream_t s);

int ensureDeviceTables() {
  static std::mutex mu;
  static bool done[64] = {false};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return kErrDevice;
  std::lock_guard<std::mutex> g(mu);
  if (done[dev]) return kOK;
  const CodingTables& t = codingTables();
  int32_t dct[3 * 256];
  std::memset(dct, 0, sizeof(dct));
  for (int k = 0; k < 3; k++) std::memcpy(dct + k * 256, t.dct[k], sizeof(int32_t) * kLumaTx[k] * kLumaTx[k]);
  const int st = uploadCodingTables(t.scan[0], t.scan[1], t.scan[2], dct);
  if (st == kOK) done[dev] = true;
  return st;
}

// ---------------------------------------------------------------------------
GpuCodec::GpuCodec(int ring) : ringSize_(ring >= 2 ? ring : 3) {}

GpuCodec::~GpuCodec() {
  cudaStreamSynchronize(eng_.stream());
  for (uint8_t* p : ring_)
    if (p) cudaFreeHost(p);
  for (uint8_t* p : rgbaRing_)
    if (p) cudaFreeHost(p);
  if (dRGBA_) cudaFree(dRGBA_);
}

int GpuCodec::init() {
  const int st = eng_.init();
  if (st) return st;
  return eng_.addStreamingStream(2, &sid_);
}

// Codec.Decode — ebiv/codec.go:70-111.  The header checks that precede the
// ring advance run here; everything else runs in the engine.
int GpuCodec::decode(const uint8_t* pkt, size_t n, DecodedFrame* out) {
  FrameHeader fh;
  int st = parseFrameHeader(pkt, n, &fh);
  if (st) return st;
  if (fh.type == kFrameKey) {
    if ((int64_t)fh.width * fh.height > kMaxDecodePixels) return kErrUnsupported;
    if (ready_ && (fh.width != geo_.W || fh.height != geo_.H)) return kErrDimensions;
    if (!ready_) {
      geo_ = Geometry::of(fh.width, fh.height);
      const size_t img = (size_t)geo_.YStride * geo_.H + 2 * (size_t)geo_.CStride * geo_.CH;
      ring_.assign((size_t)ringSize_, nullptr);
      for (auto& p : ring_) {
        if (cudaMallocHost(&p, img) != cudaSuccess) return kErrDevice;
        std::memset(p, 0, img);
      }
      ready_ = true;
      next_ = 0;
    }
  } else if (!ready_) {
    return kErrNoKeyframe;
  }
  const int slot = next_;
  next_ = (next_ + 1) % (int)ring_.size();
  st = eng_.submit(sid_, pkt, n);
  if (st) return st;
  // The frame is copied into its ring image behind the reconstruction, with
  // one wait for both.  A failed decode leaves the slot's bytes undefined; the
  // slot's previous frame was already out of its validity window (a frame
  // stays valid for ring-size further decodes, ebiv/codec.go:15-22).
  uint8_t* img = ring_[(size_t)slot];
  uint8_t* Y = img;
  uint8_t* Cb = img + (size_t)geo_.YStride * geo_.H;
  uint8_t* Cr = Cb + (size_t)geo_.CStride * geo_.CH;
  uint8_t* rgbaHost = nullptr;
  if ((size_t)slot < rgbaValid_.size()) rgbaValid_[(size_t)slot] = 0;  // the slot's frame changes
  if (rgbaOn_) {
    st = ensureRGBA();
    if (st) return st;
    rgbaHost = rgbaRing_[(size_t)slot];
    rgbaValid_[(size_t)slot] = 0;
  }
  results_.clear();
  eng_.decodeInto(sid_, Y, geo_.YStride, Cb, Cr, geo_.CStride, &results_, rgbaHost ? dRGBA_ : nullptr, rgbaHost);
  if (results_.size() != 1) return kErrDevice;
  const RoundResult& r = results_[0];
  if (r.status) return r.status;
  if (rgbaHost) rgbaValid_[(size_t)slot] = 1;
  out->y = Y;
  out->cb = Cb;
  out->cr = Cr;
  out->yStride = geo_.YStride;
  out->cStride = geo_.CStride;
  out->width = geo_.W;
  out->height = geo_.H;
  out->slot = slot;
  out->keyframe = fh.type == kFrameKey;
  return kOK;
}

void GpuCodec::flush() { next_ = 0; }

int GpuCodec::setRGBA(bool on) {
  rgbaOn_ = on;
  return kOK;
}

// The device conversion buffer and the per-slot pinned pool, sized on the
// first use after the stream's key frame fixed the geometry.
int GpuCodec::ensureRGBA() {
  const size_t need = (size_t)geo_.W * geo_.H * 4;
  if (rgbaCap_ < need) {
    if (dRGBA_) cudaFree(dRGBA_);
    dRGBA_ = nullptr;
    rgbaCap_ = 0;
    if (cudaMalloc(&dRGBA_, need) != cudaSuccess) return kErrDevice;
    rgbaCap_ = need;
  }
  if (rgbaRing_.size() != ring_.size()) {
    for (uint8_t* p : rgbaRing_)
      if (p) cudaFreeHost(p);
    rgbaRing_.assign(ring_.size(), nullptr);
    rgbaValid_.assign(ring_.size(), 0);
    for (auto& p : rgbaRing_)
      if (cudaMallocHost(&p, need) != cudaSuccess) return kErrDevice;
  }
  return kOK;
}

const uint8_t* GpuCodec::pooledRGBA(int slot) const {
  if (!rgbaOn_ || slot < 0 || slot >= (int)rgbaRing_.size() || !rgbaValid_[(size_t)slot]) return nullptr;
  return rgbaRing_[(size_t)slot];
}

int GpuCodec::rgba(int slot, uint8_t* dst, size_t cap) {
  if (!ready_ || slot < 0 || slot >= (int)ring_.size()) return kErrArg;
  const size_t need = (size_t)geo_.W * geo_.H * 4;
  if (cap < need) return kErrArg;
  if (rgbaCap_ < need) {
    if (dRGBA_) cudaFree(dRGBA_);
    dRGBA_ = nullptr;
    rgbaCap_ = 0;
    if (cudaMalloc(&dRGBA_, need) != cudaSuccess) return kErrDevice;
    rgbaCap_ = need;
  }
  const uint8_t* img = ring_[(size_t)slot];
  const uint8_t* Y = img;
  const uint8_t* Cb = img + (size_t)geo_.YStride * geo_.H;
  const uint8_t* Cr = Cb + (size_t)geo_.CStride * geo_.CH;
  // The ring image lives in pinned host memory, which the GPU reads directly.
  launchRGBA(Y, Cb, Cr, geo_.YStride, geo_.CStride, geo_.W, geo_.H, dRGBA_, eng_.stream());
  extraLaunches_++;
  if (cudaMemcpyAsync(dst, dRGBA_, need, cudaMemcpyDeviceToHost, eng_.stream()) != cudaSuccess) return kErrDevice;
  if (cudaStreamSynchronize(eng_.stream()) != cudaSuccess) return kErrDevice;
  return cudaGetLastError() == cudaSuccess ? kOK : kErrDevice;
}

int GpuCodec::copyReference(int which, uint8_t* dst, size_t cap) { return eng_.copyReference(sid_, which, dst, cap); }

}  // namespace ebiv

// ---------------------------------------------------------------------------
// C-ABI
// ---------------------------------------------------------------------------
using namespace ebiv;

struct ebivgpu_codec {
  std::unique_ptr<GpuCodec> c;
};

extern "C" {

int ebivgpu_abi_sizes(size_t* sizes, int n) {
  const size_t v[] = {sizeof(ebivgpu_frame), sizeof(ebivgpu_plane_view), sizeof(ebivgpu_serve_options),
                      sizeof(ebivgpu_serve_stats), sizeof(ebivgpu_source_frame)};
  const int k = (int)(sizeof(v) / sizeof(v[0]));
  for (int i = 0; i < n && i < k && sizes; i++) sizes[i] = v[i];
  return k;
}

int ebivgpu_device_available(void) {
  int n = 0;
  return cudaGetDeviceCount(&n) == cudaSuccess && n > 0 ? 1 : 0;
}

int ebivgpu_create(int ring, ebivgpu_codec** out) {
  if (!out) return kErrArg;
  *out = nullptr;
  if (!ebivgpu_device_available()) return kErrDevice;
  ebivgpu_codec* h = new (std::nothrow) ebivgpu_codec();
  if (!h) return kErrDevice;
  h->c.reset(new GpuCodec(ring));
  const int st = h->c->init();
  if (st) {
    delete h;
    return st;
  }
  *out = h;
  return kOK;
}

int ebivgpu_decode(ebivgpu_codec* h, const uint8_t* pkt, size_t n, int64_t ts, ebivgpu_frame* out) {
  if (!h || (!pkt && n) || !out) return kErrArg;
  DecodedFrame f;
  const int st = h->c->decode(pkt, n, &f);
  if (st) return st;
  out->y = f.y;
  out->cb = f.cb;
  out->cr = f.cr;
  out->y_stride = f.yStride;
  out->c_stride = f.cStride;
  out->width = f.width;
  out->height = f.height;
  out->timestamp_ns = ts;
  out->ring_slot = f.slot;
  out->keyframe = f.keyframe ? 1 : 0;
  return kOK;
}

void ebivgpu_flush(ebivgpu_codec* h) {
  if (h) h->c->flush();
}

void ebivgpu_destroy(ebivgpu_codec* h) { delete h; }

int ebivgpu_frame_rgba(ebivgpu_codec* h, int slot, uint8_t* dst, size_t cap) {
  if (!h || !dst) return kErrArg;
  return h->c->rgba(slot, dst, cap);
}

int64_t ebivgpu_codec_launches(ebivgpu_codec* h) { return h ? h->c->launches() : 0; }

int ebivgpu_set_rgba(ebivgpu_codec* h, int enable) { return h ? h->c->setRGBA(enable != 0) : kErrArg; }

const uint8_t* ebivgpu_frame_rgba_pooled(ebivgpu_codec* h, int slot) { return h ? h->c->pooledRGBA(slot) : nullptr; }

const char* ebivgpu_status_string(int s) {
  switch (s) {
    case kOK: return "ok";
    case kErrCorrupt: return "ebiv: corrupt stream";
    case kErrNoKeyframe: return "ebiv: inter frame before any key frame";
    case kErrDimensions: return "ebiv: frame dimensions do not match the stream";
    case kErrUnsupported: return "ebiv: unsupported stream feature";
    case kErrVersion: return "ebiv: unsupported format version";
    case kErrBadMagic: return "ebiv: not an EBIV file";
    case kErrConfig: return "ebiv: invalid configuration";
    case kErrWriterClosed: return "ebiv: writer is closed";
    case kErrEOF: return "EOF";
    case kErrIO: return "i/o error";
    case kErrDevice: return "ebivgpu: CUDA device error";
    case kErrArg: return "ebivgpu: invalid argument";
    case kErrTooLarge:
      return "ebivgpu: frame exceeds the no-allocation scratch (at most 3600 macroblocks and a 2 MiB packet)";
    default: return "unknown status";
  }
}

}  // extern "C"

