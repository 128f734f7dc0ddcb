// Key-frame decode with no device allocation.
//
// ebivgpu_decode_key_noalloc decodes one key-frame packet, as the first frame
// of a fresh stream, into planes the caller owns.  All decoder scratch (frame
// descriptors, coding tables, tile ranges, macroblock records, sparse levels,
// intra lists, the packet bytes) lives in one file-scope device array of fixed
// size, so the call never allocates device memory: it is for callers that
// must not call cudaMalloc/cudaFree on their decode path — a presentation
// thread with a frame deadline (allocation can synchronise the device), a
// process whose device memory is fixed at start-up (a late allocation can
// fail mid-stream), or a caller that has reserved all remaining memory.
//
// The kernels are the ones the stateful codec runs (entropy, then intra
// reconstruction; the golden-override payload of an alt-ref key packet gets
// the entropy pass only, which alone decides its status).  No buffer of the
// scratch has to start at zero except the two per-payload status words, which
// every call uploads as zero.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <mutex>
#include <vector>

#include "container.h"
#include "ebiv_format.h"
#include "gpu_codec.h"
#include "gpu_types.h"
#include "payload.h"
#include "../../include/ebivgpu.h"

namespace ebiv {

void launchEntropy(const FrameDesc* frames, const int4* jobs, int njobs, int* next, int maxTileMBs, cudaStream_t s);
void launchInter(const FrameDesc* frames, int nframes, int maxMBs, int phase, cudaStream_t s);
void launchIntra(const FrameDesc* frames, const int2* jobs, int njobs, int maxTileMBs, int maxTileKeys, int warps,
                 cudaStream_t s);

namespace {

constexpr int kNAMaxMBs = EBIVGPU_NOALLOC_MAX_MBS;
constexpr size_t kNAMaxPacket = EBIVGPU_NOALLOC_MAX_PACKET;

constexpr size_t a256(size_t v) { return (v + 255) & ~size_t(255); }
// Scratch layout; index 0 of each pair is the key payload, 1 the override.
constexpr size_t kOffDesc = 0;
constexpr size_t kOffStatus = a256(kOffDesc + 2 * sizeof(FrameDesc));
constexpr size_t kOffTables = a256(kOffStatus + 2 * sizeof(int32_t));
constexpr size_t kOffTiles = a256(kOffTables + 2 * sizeof(DeviceTables));
constexpr size_t kOffJobs = a256(kOffTiles + 2 * (size_t)kNAMaxMBs * sizeof(TileRange));
constexpr size_t kNAMaxEJobs = (kNAMaxMBs + kEntropyTilesPerJob - 1) / kEntropyTilesPerJob;
constexpr size_t kOffEJobs = a256(kOffJobs + 2 * (size_t)kNAMaxMBs * sizeof(int2));
constexpr size_t kOffRec = a256(kOffEJobs + 2 * kNAMaxEJobs * sizeof(int4));  // end of the uploaded head
constexpr size_t kOffCoef = a256(kOffRec + (size_t)kNAMaxMBs * sizeof(MBRec));
constexpr size_t kOffMV = a256(kOffCoef + (size_t)kNAMaxMBs * kCoefPerMB * sizeof(uint32_t));
constexpr size_t kOffLV = a256(kOffMV + (size_t)kNAMaxMBs * 2 * sizeof(int16_t));
constexpr size_t kOffIntra = a256(kOffLV + (size_t)kNAMaxMBs * sizeof(int16_t));
constexpr size_t kOffTS = a256(kOffIntra + 2 * (size_t)kNAMaxMBs * sizeof(uint32_t));
constexpr size_t kOffPkt = a256(kOffTS + (size_t)kNAMaxMBs * sizeof(TileStat));
constexpr size_t kNABytes = a256(kOffPkt + kNAMaxPacket);
static_assert(kNABytes == EBIVGPU_NOALLOC_SCRATCH_BYTES, "the header states the scratch size");
static_assert(kNABytes < (16u << 20), "the no-allocation scratch stays modest");

}  // namespace
}  // namespace ebiv

// The scratch: one per device, in the module's static device memory.
static __device__ __align__(256) unsigned char gNoAllocScratch[ebiv::kNABytes];

namespace ebiv {
namespace {

// First call on a device: resolve the scratch address and upload the
// constant coding tables.  Both are plain symbol operations.
int noAllocSetup(uint8_t** out) {
  static std::mutex mu;
  static uint8_t* addr[64] = {nullptr};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return kErrDevice;
  std::lock_guard<std::mutex> g(mu);
  if (!addr[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, gNoAllocScratch) != cudaSuccess || !p) return kErrDevice;
    const int st = ensureDeviceTables();
    if (st) return st;
    addr[dev] = static_cast<uint8_t*>(p);
  }
  *out = addr[dev];
  return kOK;
}

void fillDesc(FrameDesc& fd, uint8_t* d, int which, const Geometry& g, const PayloadPlan& plan, bool inter,
              uint8_t* y, uint8_t* cb, uint8_t* cr, int ys, int cs) {
  std::memset(&fd, 0, sizeof(fd));
  fd.rec[0] = y;
  fd.rec[1] = cb;
  fd.rec[2] = cr;
  for (int p = 0; p < 3; p++) fd.ref[p] = fd.gold[p] = fd.rec[p];  // read only by inter reconstruction
  fd.strideY = ys;
  fd.strideC = cs;
  fd.padW = g.padW();
  fd.padH = g.padH();
  fd.padCW = g.padCW();
  fd.padCH = g.padCH();
  fd.mbCols = g.mbCols;
  fd.mbRows = g.mbRows;
  fd.inter = inter ? 1 : 0;
  const Quant q = quantFor(plan.qp);
  fd.qdc = q.dc;
  fd.qac = q.ac;
  fd.tileCount = (int)plan.tiles.size();
  fd.pkt = d + kOffPkt;
  fd.tables = reinterpret_cast<const DeviceTables*>(d + kOffTables) + which;
  fd.tiles = reinterpret_cast<const TileRange*>(d + kOffTiles) + (size_t)which * kNAMaxMBs;
  fd.mbrec = reinterpret_cast<MBRec*>(d + kOffRec);
  fd.coef = reinterpret_cast<uint32_t*>(d + kOffCoef);
  fd.mvgrid = reinterpret_cast<int16_t*>(d + kOffMV);
  fd.lvgrid = reinterpret_cast<int16_t*>(d + kOffLV);
  fd.intraList = reinterpret_cast<uint32_t*>(d + kOffIntra);
  fd.intraSorted = fd.intraList + (size_t)g.mbCols * g.mbRows;
  fd.tileStat = reinterpret_cast<TileStat*>(d + kOffTS);
  fd.status = reinterpret_cast<int32_t*>(d + kOffStatus) + which;
  fd.gate = nullptr;
}

}  // namespace
}  // namespace ebiv

using namespace ebiv;

extern "C" int ebivgpu_decode_key_noalloc(const uint8_t* pkt, size_t n, uint8_t* y, int32_t y_stride, size_t y_cap,
                                          uint8_t* cb, uint8_t* cr, int32_t c_stride, size_t c_cap, void* cuda_stream,
                                          int32_t* width, int32_t* height) {
  if (!pkt && n) return kErrArg;
  // Header checks in the order a fresh codec makes them (ebiv/codec.go:70-100).
  FrameHeader fh;
  int st = parseFrameHeader(pkt, n, &fh);
  if (st) return st;
  if (fh.type != kFrameKey) return kErrNoKeyframe;
  if ((int64_t)fh.width * fh.height > kMaxDecodePixels) return kErrUnsupported;
  const Geometry g = Geometry::of(fh.width, fh.height);
  if (width) *width = g.W;
  if (height) *height = g.H;
  const size_t mbs = (size_t)g.mbCols * g.mbRows;
  if (mbs > (size_t)kNAMaxMBs || n > kNAMaxPacket) return kErrTooLarge;
  if (!y) return kOK;  // dimensions only
  if (!cb || !cr || y_stride < g.padW() || c_stride < g.padCW() || y_cap < (size_t)y_stride * g.padH() ||
      c_cap < (size_t)c_stride * g.padCH())
    return kErrArg;
  cudaStream_t s = static_cast<cudaStream_t>(cuda_stream);

  if (fh.coding == kCodingRaw) {  // decodeRaw — ebiv/codec.go:195-207
    if (n - fh.bodyOffset != g.packedSize()) return kErrCorrupt;
    const uint8_t* body = pkt + fh.bodyOffset;
    const size_t ys = (size_t)g.W * g.H, csz = (size_t)g.CW * g.CH;
    if (cudaMemcpy2DAsync(y, (size_t)y_stride, body, g.W, g.W, g.H, cudaMemcpyHostToDevice, s) ||
        cudaMemcpy2DAsync(cb, (size_t)c_stride, body + ys, g.CW, g.CW, g.CH, cudaMemcpyHostToDevice, s) ||
        cudaMemcpy2DAsync(cr, (size_t)c_stride, body + ys + csz, g.CW, g.CW, g.CH, cudaMemcpyHostToDevice, s) ||
        cudaStreamSynchronize(s))
      return kErrDevice;
    return kOK;
  }
  if (fh.coding != kCodingIntra && fh.coding != kCodingInter) return kErrUnsupported;
  // A key frame coded as inter predicts from a fresh codec's zeroed reference
  // buffers; the scratch holds no reference planes, so it is refused.
  if (fh.coding == kCodingInter) return kErrUnsupported;

  // Plan the key payload and, for an alt-ref packet, the override that
  // follows it (the same splitting as the stateful codec).
  size_t bodyOff = fh.bodyOffset, bodyLen = n - fh.bodyOffset, ovOff = 0, ovLen = 0;
  if (fh.goldenOverride) {
    int k;
    const uint64_t keyLen = getUvarint(pkt + bodyOff, bodyLen, &k);
    if (k <= 0 || keyLen > (uint64_t)(bodyLen - (size_t)k)) return kErrCorrupt;
    ovOff = bodyOff + (size_t)k + (size_t)keyLen;
    ovLen = bodyLen - (size_t)k - (size_t)keyLen;
    bodyOff += (size_t)k;
    bodyLen = (size_t)keyLen;
  }
  TableHistory hist;
  PayloadPlan plan[2];
  st = planPayload(pkt, bodyOff, bodyLen, true, g.mbCols, g.mbRows, hist, &plan[0]);
  if (st) return st;
  int ovPlan = kOK;
  if (fh.goldenOverride) ovPlan = planPayload(pkt, ovOff, ovLen, false, g.mbCols, g.mbRows, hist, &plan[1]);
  const bool withOv = fh.goldenOverride && ovPlan == kOK;

  // An error left pending by earlier work of the caller is not this call's:
  // fail before launching, without clearing it, so launch errors below are ours.
  if (cudaPeekAtLastError() != cudaSuccess) return kErrDevice;
  uint8_t* d = nullptr;
  st = noAllocSetup(&d);
  if (st) return st;

  // Head of the scratch (descriptors, zeroed statuses, tables, tiles, jobs),
  // staged on the host and uploaded in one copy.
  std::vector<uint8_t> head(kOffRec, 0);
  const int payloads = withOv ? 2 : 1;
  for (int w = 0; w < payloads; w++) {
    const PayloadPlan& p = plan[w];
    FrameDesc fd;
    fillDesc(fd, d, w, g, p, w == 1, y, cb, cr, y_stride, c_stride);
    std::memcpy(head.data() + kOffDesc + w * sizeof(FrameDesc), &fd, sizeof(fd));
    std::memcpy(head.data() + kOffTables + w * sizeof(DeviceTables), &p.tables, sizeof(DeviceTables));
    TileRange* tr = reinterpret_cast<TileRange*>(head.data() + kOffTiles) + (size_t)w * kNAMaxMBs;
    int2* jb = reinterpret_cast<int2*>(head.data() + kOffJobs) + (size_t)w * kNAMaxMBs;
    for (size_t t = 0; t < p.tiles.size(); t++) {
      tr[t] = p.tiles[t];
      jb[t] = make_int2(w, (int)t);
    }
    int4* ej = reinterpret_cast<int4*>(head.data() + kOffEJobs) + (size_t)w * kNAMaxEJobs;
    const int nt = (int)p.tiles.size();
    for (int t0 = 0; t0 < nt; t0 += kEntropyTilesPerJob)
      ej[t0 / kEntropyTilesPerJob] = make_int4(w, t0, std::min(kEntropyTilesPerJob, nt - t0), 0);
  }
  int32_t status[2] = {0, 0};
  if (cudaMemcpyAsync(d, head.data(), head.size(), cudaMemcpyHostToDevice, s) != cudaSuccess ||
      cudaMemcpyAsync(d + kOffPkt, pkt, n, cudaMemcpyHostToDevice, s) != cudaSuccess)
    return kErrDevice;
  const FrameDesc* dd = reinterpret_cast<const FrameDesc*>(d + kOffDesc);
  const int2* dj = reinterpret_cast<const int2*>(d + kOffJobs);
  const int4* de = reinterpret_cast<const int4*>(d + kOffEJobs);
  const int nt0 = (int)plan[0].tiles.size();
  auto groups = [](int nt) { return (nt + kEntropyTilesPerJob - 1) / kEntropyTilesPerJob; };
  int maxTile = 0, maxKeys = 0;
  for (const TileRange& t : plan[0].tiles) {
    const int w = t.mbX1 - t.mbX0, h = t.mbY1 - t.mbY0;
    maxTile = std::max(maxTile, w * h);
    maxKeys = std::max(maxKeys, 4 * (w - 1) + 11 * (h - 1) + 1);
  }
  // Each launch is checked where it is made.
  launchEntropy(dd, de, groups(nt0), nullptr, (int)mbs, s);
  if (cudaGetLastError() != cudaSuccess) return kErrDevice;
  launchInter(dd, 1, (int)mbs, 0, s);  // the intra macroblocks' residuals
  if (cudaGetLastError() != cudaSuccess) return kErrDevice;
  launchIntra(dd, dj, nt0, maxTile, maxKeys, 0, s);
  if (cudaGetLastError() != cudaSuccess) return kErrDevice;
  if (withOv) {  // after the key's reconstruction, which reads the records it overwrites
    launchEntropy(dd, de + kNAMaxEJobs, groups((int)plan[1].tiles.size()), nullptr, (int)mbs, s);
    if (cudaGetLastError() != cudaSuccess) return kErrDevice;
  }
  if (cudaMemcpyAsync(status, d + kOffStatus, sizeof(status), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return kErrDevice;
  // Status order of the stateful codec: the key's own, then the override's plan, then its decode.
  if (status[0]) return status[0];
  if (fh.goldenOverride && ovPlan) return ovPlan;
  return withOv ? status[1] : kOK;
}
