// Single-stream GB300 EBIV codec: the govid.Codec contract (Decode / Flush,
// ebiv/codec.go:70-192) on one CUDA stream.
//
// Per coded frame the host plans the payload (tables, tile ranges), uploads
// one staging block (descriptor + tables + tiles + packet) with a single copy,
// and launches stage A (entropy), B1 (inter reconstruction) and B2 (intra
// wavefront).  Reference-frame semantics follow the reference exactly:
// decode into `work`; on success a key frame fills golden (override payload
// or a copy), the visible region goes to the ring image, and work/ref swap.
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
void launchEntropy(const FrameDesc* frames, const int2* jobs, int njobs, cudaStream_t s);
void launchInter(const FrameDesc* frames, int nframes, int maxMBs, cudaStream_t s);
void launchIntra(const FrameDesc* frames, const int2* jobs, int njobs, cudaStream_t s);
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

size_t alignUp(size_t v, size_t a) { return (v + a - 1) / a * a; }

bool DeviceFrameSet::alloc(const Geometry& g) {
  const size_t ySize = (size_t)g.padW() * g.padH(), cSize = (size_t)g.padCW() * g.padCH();
  bytesPerFrame = ySize + 2 * cSize;
  for (int i = 0; i < 3; i++) {
    if (cudaMalloc(&buf[i], bytesPerFrame) != cudaSuccess) return false;
    cudaMemset(buf[i], 0, bytesPerFrame);
    y[i] = buf[i];
    cb[i] = buf[i] + ySize;
    cr[i] = buf[i] + ySize + cSize;
  }
  return true;
}
void DeviceFrameSet::release() {
  for (int i = 0; i < 3; i++)
    if (buf[i]) cudaFree(buf[i]);
  std::memset(buf, 0, sizeof(buf));
}

// ---------------------------------------------------------------------------
GpuCodec::GpuCodec(int ring) : ringSize_(ring >= 2 ? ring : 3) {}

GpuCodec::~GpuCodec() {
  if (stream_) cudaStreamSynchronize(stream_);
  frames_.release();
  for (uint8_t* p : ring_)
    if (p) cudaFreeHost(p);
  if (dStage_) cudaFree(dStage_);
  if (hStage_) cudaFreeHost(hStage_);
  if (dRec_) cudaFree(dRec_);
  if (dCoef_) cudaFree(dCoef_);
  if (dMV_) cudaFree(dMV_);
  if (dTileStat_) cudaFree(dTileStat_);
  if (dRGBA_) cudaFree(dRGBA_);
  if (stream_) cudaStreamDestroy(stream_);
}

int GpuCodec::init() {
  if (cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking) != cudaSuccess) return kErrDevice;
  return ensureDeviceTables();
}

// configure — ebiv/codec.go:129-153
int GpuCodec::configure(int w, int h) {
  if ((int64_t)w * h > kMaxDecodePixels) return kErrUnsupported;
  if (ready_) return (w != geo_.W || h != geo_.H) ? kErrDimensions : kOK;
  geo_ = Geometry::of(w, h);
  ring_.assign((size_t)ringSize_, nullptr);
  const size_t img = (size_t)geo_.YStride * geo_.H + 2 * (size_t)geo_.CStride * geo_.CH;
  for (auto& p : ring_) {
    if (cudaMallocHost(&p, img) != cudaSuccess) return kErrDevice;
    std::memset(p, 0, img);
  }
  if (!frames_.alloc(geo_)) return kErrDevice;
  work_ = 0;
  ref_ = 1;
  golden_ = 2;
  const size_t mbs = (size_t)geo_.mbCols * geo_.mbRows;
  if (cudaMalloc(&dRec_, mbs * sizeof(MBRec)) != cudaSuccess) return kErrDevice;
  if (cudaMalloc(&dCoef_, mbs * kCoefPerMB * sizeof(uint32_t)) != cudaSuccess) return kErrDevice;
  if (cudaMalloc(&dMV_, mbs * 2 * sizeof(int16_t)) != cudaSuccess) return kErrDevice;
  if (cudaMalloc(&dTileStat_, mbs * sizeof(TileStat)) != cudaSuccess) return kErrDevice;
  next_ = 0;
  ready_ = true;
  return kOK;
}

int GpuCodec::ensureStage(size_t bytes) {
  if (bytes <= stageCap_) return kOK;
  size_t cap = alignUp(bytes + bytes / 2, 1 << 20);
  if (dStage_) cudaFree(dStage_);
  if (hStage_) cudaFreeHost(hStage_);
  dStage_ = nullptr;
  hStage_ = nullptr;
  stageCap_ = 0;
  if (cudaMalloc(&dStage_, cap) != cudaSuccess) return kErrDevice;
  if (cudaMallocHost(&hStage_, cap) != cudaSuccess) return kErrDevice;
  stageCap_ = cap;
  return kOK;
}

// Uploads and launches one planned payload; returns the device status.
int GpuCodec::runPayload(const uint8_t* pkt, size_t n, const PayloadPlan& plan, int rec, int ref, int gold,
                         bool inter) {
  const int T = (int)plan.tiles.size();
  const size_t oDesc = 0;
  const size_t oStatus = alignUp(oDesc + sizeof(FrameDesc), 64);
  const size_t oTables = alignUp(oStatus + sizeof(int32_t), 64);
  const size_t oTiles = alignUp(oTables + sizeof(DeviceTables), 64);
  const size_t oJobs = alignUp(oTiles + sizeof(TileRange) * (size_t)T, 64);
  const size_t oPkt = alignUp(oJobs + sizeof(int2) * (size_t)T, 256);
  const size_t total = oPkt + n;
  int st = ensureStage(total);
  if (st) return st;
  uint8_t* h = hStage_;
  uint8_t* d = dStage_;
  FrameDesc fd;
  std::memset(&fd, 0, sizeof(fd));
  fd.rec[0] = frames_.y[rec];
  fd.rec[1] = frames_.cb[rec];
  fd.rec[2] = frames_.cr[rec];
  fd.ref[0] = frames_.y[ref];
  fd.ref[1] = frames_.cb[ref];
  fd.ref[2] = frames_.cr[ref];
  fd.gold[0] = frames_.y[gold];
  fd.gold[1] = frames_.cb[gold];
  fd.gold[2] = frames_.cr[gold];
  fd.strideY = geo_.padW();
  fd.strideC = geo_.padCW();
  fd.padW = geo_.padW();
  fd.padH = geo_.padH();
  fd.padCW = geo_.padCW();
  fd.padCH = geo_.padCH();
  fd.mbCols = geo_.mbCols;
  fd.mbRows = geo_.mbRows;
  fd.inter = inter ? 1 : 0;
  const Quant q = quantFor(plan.qp);
  fd.qdc = q.dc;
  fd.qac = q.ac;
  fd.tileCount = T;
  fd.pkt = d + oPkt;
  fd.tables = reinterpret_cast<const DeviceTables*>(d + oTables);
  fd.tiles = reinterpret_cast<const TileRange*>(d + oTiles);
  fd.mbrec = static_cast<MBRec*>(dRec_);
  fd.coef = dCoef_;
  fd.mvgrid = dMV_;
  fd.tileStat = static_cast<TileStat*>(dTileStat_);
  fd.status = reinterpret_cast<int32_t*>(d + oStatus);
  fd.gate = nullptr;
  std::memcpy(h + oDesc, &fd, sizeof(fd));
  const int32_t zero = 0;
  std::memcpy(h + oStatus, &zero, sizeof(zero));
  std::memcpy(h + oTables, &plan.tables, sizeof(DeviceTables));
  std::memcpy(h + oTiles, plan.tiles.data(), sizeof(TileRange) * (size_t)T);
  int2* jobs = reinterpret_cast<int2*>(h + oJobs);
  for (int t = 0; t < T; t++) jobs[t] = make_int2(0, t);
  std::memcpy(h + oPkt, pkt, n);
  if (cudaMemcpyAsync(d, h, total, cudaMemcpyHostToDevice, stream_) != cudaSuccess) return kErrDevice;
  const FrameDesc* dfd = reinterpret_cast<const FrameDesc*>(d + oDesc);
  const int2* djobs = reinterpret_cast<const int2*>(d + oJobs);
  launchEntropy(dfd, djobs, T, stream_);
  launches_++;
  if (inter) {
    launchInter(dfd, 1, geo_.mbCols * geo_.mbRows, stream_);
    launches_++;
  }
  launchIntra(dfd, djobs, T, stream_);
  launches_++;
  int32_t status = 0;
  if (cudaMemcpyAsync(&status, d + oStatus, sizeof(status), cudaMemcpyDeviceToHost, stream_) != cudaSuccess)
    return kErrDevice;
  if (cudaStreamSynchronize(stream_) != cudaSuccess) return kErrDevice;
  if (cudaGetLastError() != cudaSuccess) return kErrDevice;
  return status;
}

// Codec.Decode — ebiv/codec.go:70-111
int GpuCodec::decode(const uint8_t* pkt, size_t n, DecodedFrame* out) {
  FrameHeader fh;
  int st = parseFrameHeader(pkt, n, &fh);
  if (st) return st;
  if (fh.type == kFrameKey) {
    st = configure(fh.width, fh.height);
    if (st) return st;
  } else if (!ready_) {
    return kErrNoKeyframe;
  }
  const int slot = next_;
  next_ = (next_ + 1) % (int)ring_.size();
  uint8_t* img = ring_[(size_t)slot];
  const uint8_t* body = pkt + fh.bodyOffset;
  const size_t blen = n - fh.bodyOffset;
  switch (fh.coding) {
    case kCodingRaw: {  // decodeRaw — ebiv/codec.go:195-207
      if (blen != geo_.packedSize()) return kErrCorrupt;
      uint8_t* Y = img;
      uint8_t* Cb = img + (size_t)geo_.YStride * geo_.H;
      uint8_t* Cr = Cb + (size_t)geo_.CStride * geo_.CH;
      for (int y = 0; y < geo_.H; y++) std::memcpy(Y + (size_t)y * geo_.YStride, body + (size_t)y * geo_.W, geo_.W);
      const size_t ys = (size_t)geo_.W * geo_.H, cs = (size_t)geo_.CW * geo_.CH;
      for (int y = 0; y < geo_.CH; y++) {
        std::memcpy(Cb + (size_t)y * geo_.CStride, body + ys + (size_t)y * geo_.CW, geo_.CW);
        std::memcpy(Cr + (size_t)y * geo_.CStride, body + ys + cs + (size_t)y * geo_.CW, geo_.CW);
      }
      break;
    }
    case kCodingIntra:
    case kCodingInter:
      st = decodeCoded(pkt, n, fh, img);
      if (st) return st;
      break;
    default:
      return kErrUnsupported;
  }
  out->y = img;
  out->cb = img + (size_t)geo_.YStride * geo_.H;
  out->cr = out->cb + (size_t)geo_.CStride * geo_.CH;
  out->yStride = geo_.YStride;
  out->cStride = geo_.CStride;
  out->width = geo_.W;
  out->height = geo_.H;
  out->slot = slot;
  out->keyframe = fh.type == kFrameKey;
  return kOK;
}

// Codec.decodeCoded — ebiv/codec.go:162-192
int GpuCodec::decodeCoded(const uint8_t* pkt, size_t n, const FrameHeader& fh, uint8_t* img) {
  const bool inter = fh.coding == kCodingInter;
  const bool key = fh.type == kFrameKey;
  size_t bodyOff = fh.bodyOffset, bodyLen = n - fh.bodyOffset;
  size_t ovOff = 0, ovLen = 0;
  if (fh.goldenOverride) {
    int k;
    const uint64_t keyLen = getUvarint(pkt + bodyOff, bodyLen, &k);
    if (k <= 0 || keyLen > (uint64_t)(bodyLen - (size_t)k)) return kErrCorrupt;
    ovOff = bodyOff + (size_t)k + (size_t)keyLen;
    ovLen = bodyLen - (size_t)k - (size_t)keyLen;
    bodyOff += (size_t)k;
    bodyLen = (size_t)keyLen;
  }
  PayloadPlan plan;
  int st = planPayload(pkt, bodyOff, bodyLen, key, geo_.mbCols, geo_.mbRows, hist_, &plan);
  if (st) return st;
  st = runPayload(pkt, n, plan, work_, ref_, golden_, inter);
  if (st) return st;
  if (key) {
    if (fh.goldenOverride) {
      st = planPayload(pkt, ovOff, ovLen, false, geo_.mbCols, geo_.mbRows, hist_, &plan);
      if (st) return st;
      st = runPayload(pkt, n, plan, golden_, work_, work_, true);
      if (st) return st;
    } else {
      if (cudaMemcpyAsync(frames_.buf[golden_], frames_.buf[work_], frames_.bytesPerFrame, cudaMemcpyDeviceToDevice,
                          stream_) != cudaSuccess)
        return kErrDevice;
    }
  }
  // storeImage — ebiv/frame.go:67-77
  uint8_t* Y = img;
  uint8_t* Cb = img + (size_t)geo_.YStride * geo_.H;
  uint8_t* Cr = Cb + (size_t)geo_.CStride * geo_.CH;
  if (cudaMemcpy2DAsync(Y, geo_.YStride, frames_.y[work_], geo_.padW(), geo_.W, geo_.H, cudaMemcpyDeviceToHost,
                        stream_) != cudaSuccess ||
      cudaMemcpy2DAsync(Cb, geo_.CStride, frames_.cb[work_], geo_.padCW(), geo_.CW, geo_.CH, cudaMemcpyDeviceToHost,
                        stream_) != cudaSuccess ||
      cudaMemcpy2DAsync(Cr, geo_.CStride, frames_.cr[work_], geo_.padCW(), geo_.CW, geo_.CH, cudaMemcpyDeviceToHost,
                        stream_) != cudaSuccess)
    return kErrDevice;
  if (cudaStreamSynchronize(stream_) != cudaSuccess) return kErrDevice;
  lastWork_ = work_;
  std::swap(work_, ref_);
  return kOK;
}

void GpuCodec::flush() { next_ = 0; }

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
  launchRGBA(Y, Cb, Cr, geo_.YStride, geo_.CStride, geo_.W, geo_.H, dRGBA_, stream_);
  launches_++;
  if (cudaMemcpyAsync(dst, dRGBA_, need, cudaMemcpyDeviceToHost, stream_) != cudaSuccess) return kErrDevice;
  if (cudaStreamSynchronize(stream_) != cudaSuccess) return kErrDevice;
  return cudaGetLastError() == cudaSuccess ? kOK : kErrDevice;
}

}  // namespace ebiv

// ---------------------------------------------------------------------------
// C-ABI
// ---------------------------------------------------------------------------
using namespace ebiv;

struct ebivgpu_codec {
  std::unique_ptr<GpuCodec> c;
};

extern "C" {

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
    default: return "unknown status";
  }
}

}  // extern "C"

namespace ebiv {
int GpuCodec::copyReference(int which, uint8_t* dst, size_t cap) {
  if (!ready_ || cap < frames_.bytesPerFrame) return kErrArg;
  const int idx = which == 0 ? ref_ : golden_;
  if (cudaMemcpyAsync(dst, frames_.buf[idx], frames_.bytesPerFrame, cudaMemcpyDeviceToHost, stream_) != cudaSuccess)
    return kErrDevice;
  return cudaStreamSynchronize(stream_) == cudaSuccess ? kOK : kErrDevice;
}
}  // namespace ebiv
