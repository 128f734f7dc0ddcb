// Multi-stream decode engine (see engine.h) and its C-ABI.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <new>

#include "../../include/ebivgpu.h"
#include "container.h"
#include "engine.h"
#include "gpu_codec.h"

namespace ebiv {

void launchEntropy(const FrameDesc* frames, const int2* jobs, int njobs, cudaStream_t s);
void launchInter(const FrameDesc* frames, int nframes, int maxMBs, cudaStream_t s);
void launchIntra(const FrameDesc* frames, const int2* jobs, int njobs, cudaStream_t s);

namespace {
inline size_t al(size_t v, size_t a) { return (v + a - 1) / a * a; }
inline int stride64(int w) { return (w + 63) & ~63; }
}  // namespace

struct Engine::Stream {
  int id = -1;
  bool active = true;
  bool resident = false;
  int ring = 3;
  Geometry geo;
  int strideY = 0, strideC = 0;
  size_t yBytes = 0, cBytes = 0, bufBytes = 0;
  bool ready = false;
  std::vector<uint8_t*> pool;
  std::vector<int> outputs;  // FIFO of buffer indices, oldest first
  int ref = -1, golden = -1;
  TableHistory hist;
  // Resident packets: host copies (for planning) and one device block.
  std::vector<std::vector<uint8_t>> hostPkts;
  uint8_t* dPkts = nullptr;
  std::vector<size_t> dOff;
  int64_t next = 0;
  // Streaming: the submitted packet awaiting its round.
  std::vector<uint8_t> pendingPkt;
  bool pending = false;
  // Per-frame scratch.
  MBRec* dRec = nullptr;
  uint32_t* dCoef = nullptr;
  int16_t* dMV = nullptr;
  TileStat* dTileStat = nullptr;
  TileStat* dTileStatOv = nullptr;
  size_t mbs = 0;
  size_t bytes = 0;

  uint8_t* plane(int b, int k) const {
    return pool[(size_t)b] + (k == 0 ? 0 : yBytes + (size_t)(k - 1) * cBytes);
  }
  void release() {
    for (auto p : pool) cudaFree(p);
    pool.clear();
    if (dPkts) cudaFree(dPkts);
    if (dRec) cudaFree(dRec);
    if (dCoef) cudaFree(dCoef);
    if (dMV) cudaFree(dMV);
    if (dTileStat) cudaFree(dTileStat);
    if (dTileStatOv) cudaFree(dTileStatOv);
    dPkts = nullptr;
    dRec = nullptr;
    dCoef = nullptr;
    dMV = nullptr;
    dTileStat = dTileStatOv = nullptr;
  }
};

struct Engine::Job {
  int stream = -1;
  int64_t pktIndex = -1;
  const uint8_t* hPkt = nullptr;  // host bytes (planning)
  const uint8_t* dPkt = nullptr;  // device bytes (kernels); null => staged this round
  size_t n = 0;
  FrameHeader fh;
  int status = kOK;  // host-side result when the frame never reaches the GPU
  bool gpu = false;  // frame has kernels this round
  int work = -1, ovBuf = -1;
  bool hasOv = false;
  int ovPlanStatus = kOK;
  PayloadPlan main, ov;
  TableHistory ovHist;
  int mainDesc = -1, ovDesc = -1;
  size_t stageOff = 0;  // for streamed packets: offset in the staging block
};

Engine::Engine() {}

Engine::~Engine() {
  if (stream_) cudaStreamSynchronize(stream_);
  for (auto& s : streams_)
    if (s) s->release();
  if (dStage_) cudaFree(dStage_);
  if (hStage_) cudaFreeHost(hStage_);
  for (auto& e : ev_)
    if (e) cudaEventDestroy(e);
  if (ownStream_ && stream_) cudaStreamDestroy(stream_);
}

int Engine::init(cudaStream_t s) {
  if (s) {
    stream_ = s;
  } else {
    if (cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking) != cudaSuccess) return kErrDevice;
    ownStream_ = true;
  }
  for (auto& e : ev_)
    if (cudaEventCreate(&e) != cudaSuccess) return kErrDevice;
  return ensureDeviceTables();
}

size_t Engine::footprint(int w, int h, int ring) {
  const Geometry g = Geometry::of(w, h);
  const size_t yb = (size_t)stride64(g.padW()) * g.padH(), cb = (size_t)stride64(g.padCW()) * g.padCH();
  const size_t mbs = (size_t)g.mbCols * g.mbRows;
  return (size_t)(ring + 4) * (yb + 2 * cb) + mbs * (sizeof(MBRec) + kCoefPerMB * 4 + 4 + 2 * sizeof(TileStat));
}

int Engine::addResidentStream(const uint8_t* const* pkts, const size_t* lens, int n, int ring, int* id) {
  std::unique_ptr<Stream> s(new (std::nothrow) Stream());
  if (!s) return kErrArg;
  s->resident = true;
  s->ring = ring >= 2 ? ring : 3;
  size_t total = 0;
  s->hostPkts.resize((size_t)n);
  s->dOff.resize((size_t)n);
  for (int i = 0; i < n; i++) {
    s->hostPkts[(size_t)i].assign(pkts[i], pkts[i] + lens[i]);
    s->dOff[(size_t)i] = total;
    total += al(lens[i], 16);
  }
  if (cudaMalloc(&s->dPkts, total ? total : 16) != cudaSuccess) return kErrDevice;
  for (int i = 0; i < n; i++)
    if (lens[i] && cudaMemcpy(s->dPkts + s->dOff[(size_t)i], pkts[i], lens[i], cudaMemcpyHostToDevice) != cudaSuccess)
      return kErrDevice;
  s->bytes += total;
  deviceBytes_ += total;
  s->id = (int)streams_.size();
  *id = s->id;
  streams_.push_back(std::move(s));
  return kOK;
}

int Engine::addStreamingStream(int ring, int* id) {
  std::unique_ptr<Stream> s(new (std::nothrow) Stream());
  if (!s) return kErrArg;
  s->ring = ring >= 2 ? ring : 3;
  s->id = (int)streams_.size();
  *id = s->id;
  streams_.push_back(std::move(s));
  return kOK;
}

int Engine::submit(int id, const uint8_t* pkt, size_t n) {
  if (id < 0 || id >= (int)streams_.size() || !streams_[(size_t)id] || streams_[(size_t)id]->resident) return kErrArg;
  Stream& s = *streams_[(size_t)id];
  s.pendingPkt.assign(pkt, pkt + n);
  s.pending = true;
  return kOK;
}

int Engine::seekStream(int id, int64_t index) {
  if (id < 0 || id >= (int)streams_.size() || !streams_[(size_t)id]) return kErrArg;
  Stream& s = *streams_[(size_t)id];
  if (!s.resident || index < 0 || index > (int64_t)s.hostPkts.size()) return kErrArg;
  s.next = index;
  return kOK;
}

int64_t Engine::remaining(int id) const {
  if (id < 0 || id >= (int)streams_.size() || !streams_[(size_t)id]) return 0;
  const Stream& s = *streams_[(size_t)id];
  return s.resident ? (int64_t)s.hostPkts.size() - s.next : (s.pending ? 1 : 0);
}

int Engine::setActive(int id, bool active) {
  if (id < 0 || id >= (int)streams_.size() || !streams_[(size_t)id]) return kErrArg;
  streams_[(size_t)id]->active = active;
  return kOK;
}

int Engine::removeStream(int id) {
  if (id < 0 || id >= (int)streams_.size() || !streams_[(size_t)id]) return kErrArg;
  cudaStreamSynchronize(stream_);
  deviceBytes_ -= streams_[(size_t)id]->bytes;
  streams_[(size_t)id]->release();
  streams_[(size_t)id].reset();
  return kOK;
}

// configure — ebiv/codec.go:129-153
int Engine::configure(Stream& s, int w, int h) {
  if ((int64_t)w * h > kMaxDecodePixels) return kErrUnsupported;
  if (s.ready) return (w != s.geo.W || h != s.geo.H) ? kErrDimensions : kOK;
  s.geo = Geometry::of(w, h);
  s.strideY = stride64(s.geo.padW());
  s.strideC = stride64(s.geo.padCW());
  s.yBytes = (size_t)s.strideY * s.geo.padH();
  s.cBytes = (size_t)s.strideC * s.geo.padCH();
  s.bufBytes = s.yBytes + 2 * s.cBytes;
  const int P = s.ring + 4;
  for (int i = 0; i < P; i++) {
    uint8_t* p = nullptr;
    if (cudaMalloc(&p, s.bufBytes) != cudaSuccess) return kErrDevice;
    if (cudaMemsetAsync(p, 0, s.bufBytes, stream_) != cudaSuccess) return kErrDevice;
    s.pool.push_back(p);
  }
  // The reference allocates zeroed work/ref/golden buffers at configure.
  s.ref = 0;
  s.golden = 1;
  s.mbs = (size_t)s.geo.mbCols * s.geo.mbRows;
  if (cudaMalloc(&s.dRec, s.mbs * sizeof(MBRec)) != cudaSuccess) return kErrDevice;
  if (cudaMalloc(&s.dCoef, s.mbs * kCoefPerMB * sizeof(uint32_t)) != cudaSuccess) return kErrDevice;
  if (cudaMalloc(&s.dMV, s.mbs * 2 * sizeof(int16_t)) != cudaSuccess) return kErrDevice;
  if (cudaMalloc(&s.dTileStat, s.mbs * sizeof(TileStat)) != cudaSuccess) return kErrDevice;
  if (cudaMalloc(&s.dTileStatOv, s.mbs * sizeof(TileStat)) != cudaSuccess) return kErrDevice;
  const size_t b = (size_t)P * s.bufBytes + s.mbs * (sizeof(MBRec) + kCoefPerMB * 4 + 4 + 2 * sizeof(TileStat));
  s.bytes += b;
  deviceBytes_ += b;
  s.ready = true;
  return kOK;
}

int Engine::takeFree(Stream& s) {
  std::vector<char> used(s.pool.size(), 0);
  if (s.ref >= 0) used[(size_t)s.ref] = 1;
  if (s.golden >= 0) used[(size_t)s.golden] = 1;
  for (int b : s.outputs) used[(size_t)b] = 1;
  for (size_t i = 0; i < s.pool.size(); i++)
    if (!used[i]) return (int)i;
  return -1;
}

int Engine::ensureStage(size_t bytes) {
  if (bytes <= stageCap_) return kOK;
  const size_t cap = al(bytes + bytes / 2, 1 << 20);
  if (dStage_) {
    cudaStreamSynchronize(stream_);
    cudaFree(dStage_);
  }
  if (hStage_) cudaFreeHost(hStage_);
  dStage_ = nullptr;
  hStage_ = nullptr;
  stageCap_ = 0;
  if (cudaMalloc(&dStage_, cap) != cudaSuccess) return kErrDevice;
  if (cudaMallocHost(&hStage_, cap) != cudaSuccess) return kErrDevice;
  stageCap_ = cap;
  return kOK;
}

// Host half of Codec.Decode for one packet: header, configure, raw frames,
// payload planning.  Leaves j.gpu set when kernels must run.
int Engine::planFrame(Stream& s, Job& j, std::vector<RoundResult>* results) {
  (void)results;
  j.status = parseFrameHeader(j.hPkt, j.n, &j.fh);
  if (j.status) return j.status;
  if (j.fh.type == kFrameKey) {
    j.status = configure(s, j.fh.width, j.fh.height);
    if (j.status) return j.status;
  } else if (!s.ready) {
    return j.status = kErrNoKeyframe;
  }
  const FrameHeader& fh = j.fh;
  if (fh.coding == kCodingRaw) {  // decodeRaw — ebiv/codec.go:195-207
    const size_t blen = j.n - fh.bodyOffset;
    if (blen != s.geo.packedSize()) return j.status = kErrCorrupt;
    j.work = takeFree(s);
    if (j.work < 0) return j.status = kErrDevice;
    return kOK;  // scattered by the round, no kernels
  }
  if (fh.coding != kCodingIntra && fh.coding != kCodingInter) return j.status = kErrUnsupported;
  const bool key = fh.type == kFrameKey;
  size_t bodyOff = fh.bodyOffset, bodyLen = j.n - fh.bodyOffset, ovOff = 0, ovLen = 0;
  if (fh.goldenOverride) {
    int k;
    const uint64_t keyLen = getUvarint(j.hPkt + bodyOff, bodyLen, &k);
    if (k <= 0 || keyLen > (uint64_t)(bodyLen - (size_t)k)) return j.status = kErrCorrupt;
    ovOff = bodyOff + (size_t)k + (size_t)keyLen;
    ovLen = bodyLen - (size_t)k - (size_t)keyLen;
    bodyOff += (size_t)k;
    bodyLen = (size_t)keyLen;
  }
  j.status = planPayload(j.hPkt, bodyOff, bodyLen, key, s.geo.mbCols, s.geo.mbRows, s.hist, &j.main);
  if (j.status) return j.status;
  j.work = takeFree(s);
  if (j.work < 0) return j.status = kErrDevice;
  if (key && fh.goldenOverride) {
    j.hasOv = true;
    j.ovHist = s.hist;
    j.ovPlanStatus = planPayload(j.hPkt, ovOff, ovLen, false, s.geo.mbCols, s.geo.mbRows, j.ovHist, &j.ov);
    if (j.ovPlanStatus == kOK) {
      // The override decodes over a copy of the current golden so that a
      // failing override leaves the same partial image the reference's
      // in-place decode does.
      std::vector<char> used(s.pool.size(), 0);
      for (size_t i = 0; i < s.pool.size(); i++) {
        if ((int)i == s.ref || (int)i == s.golden || (int)i == j.work) used[i] = 1;
      }
      for (int b : s.outputs) used[(size_t)b] = 1;
      for (size_t i = 0; i < s.pool.size(); i++)
        if (!used[i]) {
          j.ovBuf = (int)i;
          break;
        }
      if (j.ovBuf < 0) return j.status = kErrDevice;
      if (cudaMemcpyAsync(s.pool[(size_t)j.ovBuf], s.pool[(size_t)s.golden], s.bufBytes, cudaMemcpyDeviceToDevice,
                          stream_) != cudaSuccess)
        return j.status = kErrDevice;
    }
  }
  j.gpu = true;
  return kOK;
}

void Engine::finishFrame(Stream& s, Job& j, const int32_t* st, std::vector<RoundResult>* results) {
  RoundResult r;
  r.stream = s.id;
  r.frameIndex = j.pktIndex;
  r.keyframe = j.fh.type == kFrameKey;
  int status = j.status;
  int out = -1;
  if (status == kOK && j.fh.coding == kCodingRaw) {
    out = j.work;
  } else if (status == kOK && j.gpu) {
    status = st[j.mainDesc];
    if (status == kOK) {
      const bool key = j.fh.type == kFrameKey;
      if (key && j.hasOv) {
        s.hist = j.ovHist;  // the override's tables were parsed (ebiv/codec.go:177-183)
        if (j.ovPlanStatus != kOK) {
          status = j.ovPlanStatus;
        } else {
          s.golden = j.ovBuf;  // written in place over golden, even on failure
          status = st[j.ovDesc];
        }
      } else if (key) {
        s.golden = j.work;
      }
      if (status == kOK) {
        s.ref = j.work;
        out = j.work;
      }
    }
  }
  if (out >= 0) {
    s.outputs.push_back(out);
    while ((int)s.outputs.size() > s.ring) s.outputs.erase(s.outputs.begin());
    r.view.y = s.plane(out, 0);
    r.view.cb = s.plane(out, 1);
    r.view.cr = s.plane(out, 2);
    r.view.yStride = s.strideY;
    r.view.cStride = s.strideC;
    r.view.width = s.geo.W;
    r.view.height = s.geo.H;
    r.view.buffer = out;
  }
  r.status = status;
  if (results) results->push_back(r);
}

int Engine::round(std::vector<RoundResult>* results) {
  std::vector<int> ids;
  for (auto& s : streams_)
    if (s && s->active && ((s->resident && s->next < (int64_t)s->hostPkts.size()) || (!s->resident && s->pending)))
      ids.push_back(s->id);
  return roundFor(ids, results);
}

int Engine::roundFor(const std::vector<int>& ids, std::vector<RoundResult>* results) {
  std::vector<Job> jobs;
  jobs.reserve(ids.size());
  size_t streamedBytes = 0;
  for (int id : ids) {
    if (id < 0 || id >= (int)streams_.size() || !streams_[(size_t)id]) continue;
    Stream& s = *streams_[(size_t)id];
    Job j;
    j.stream = id;
    if (s.resident) {
      if (s.next >= (int64_t)s.hostPkts.size()) continue;
      j.pktIndex = s.next;
      j.hPkt = s.hostPkts[(size_t)s.next].data();
      j.n = s.hostPkts[(size_t)s.next].size();
      j.dPkt = s.dPkts + s.dOff[(size_t)s.next];
      s.next++;
    } else {
      if (!s.pending) continue;
      j.hPkt = s.pendingPkt.data();
      j.n = s.pendingPkt.size();
      j.pktIndex = s.next++;
    }
    planFrame(s, j, results);
    if (j.status == kOK && j.gpu && !s.resident) {
      j.stageOff = streamedBytes;
      streamedBytes += al(j.n, 16);
    }
    jobs.push_back(std::move(j));
  }
  // Raw frames: scatter the packed planes into their pool buffer.
  for (Job& j : jobs) {
    if (j.status != kOK || j.fh.coding != kCodingRaw) continue;
    Stream& s = *streams_[(size_t)j.stream];
    const Geometry& g = s.geo;
    const uint8_t* body = j.hPkt + j.fh.bodyOffset;
    const size_t ys = (size_t)g.W * g.H, cs = (size_t)g.CW * g.CH;
    if (cudaMemcpy2DAsync(s.plane(j.work, 0), s.strideY, body, g.W, g.W, g.H, cudaMemcpyHostToDevice, stream_) ||
        cudaMemcpy2DAsync(s.plane(j.work, 1), s.strideC, body + ys, g.CW, g.CW, g.CH, cudaMemcpyHostToDevice,
                          stream_) ||
        cudaMemcpy2DAsync(s.plane(j.work, 2), s.strideC, body + ys + cs, g.CW, g.CW, g.CH, cudaMemcpyHostToDevice,
                          stream_))
      j.status = kErrDevice;
  }
  // Lay out the staging block: descriptors, statuses, tables, tiles, jobs,
  // streamed packet bytes.
  int nMain = 0, nOv = 0, tMain = 0, tOv = 0, maxMBs = 0, maxMBsOv = 0;
  for (Job& j : jobs) {
    if (j.status != kOK || !j.gpu) continue;
    const Stream& s = *streams_[(size_t)j.stream];
    j.mainDesc = nMain++;
    tMain += (int)j.main.tiles.size();
    if (j.main.tiles.size() && j.fh.coding == kCodingInter) maxMBs = std::max(maxMBs, (int)s.mbs);
    if (j.hasOv && j.ovPlanStatus == kOK) {
      nOv++;
      tOv += (int)j.ov.tiles.size();
      maxMBsOv = std::max(maxMBsOv, (int)s.mbs);
    }
  }
  {
    int k = 0;
    for (Job& j : jobs)
      if (j.status == kOK && j.gpu && j.hasOv && j.ovPlanStatus == kOK) j.ovDesc = nMain + k++;
  }
  const int nDesc = nMain + nOv;
  std::vector<int32_t> statuses((size_t)std::max(nDesc, 1), 0);
  if (nDesc > 0) {
    const size_t oDesc = 0;
    const size_t oStat = al(oDesc + sizeof(FrameDesc) * nDesc, 64);
    const size_t oTab = al(oStat + sizeof(int32_t) * nDesc, 64);
    const size_t oTiles = al(oTab + sizeof(DeviceTables) * nDesc, 64);
    const size_t oJobs = al(oTiles + sizeof(TileRange) * (size_t)(tMain + tOv), 64);
    const size_t oPkt = al(oJobs + sizeof(int2) * (size_t)(tMain + tOv), 256);
    const size_t total = oPkt + streamedBytes;
    if (ensureStage(total)) return -1;
    uint8_t* h = hStage_;
    uint8_t* d = dStage_;
    FrameDesc* hd = reinterpret_cast<FrameDesc*>(h + oDesc);
    int32_t* hs = reinterpret_cast<int32_t*>(h + oStat);
    DeviceTables* ht = reinterpret_cast<DeviceTables*>(h + oTab);
    TileRange* hr = reinterpret_cast<TileRange*>(h + oTiles);
    int2* hj = reinterpret_cast<int2*>(h + oJobs);
    int tileCur = 0;
    auto fill = [&](Job& j, const PayloadPlan& plan, int di, int rec, int ref, int gold, bool inter, int gateDesc,
                    TileStat* ts) {
      const Stream& s = *streams_[(size_t)j.stream];
      FrameDesc& fd = hd[di];
      std::memset(&fd, 0, sizeof(fd));
      for (int k = 0; k < 3; k++) {
        fd.rec[k] = s.plane(rec, k);
        fd.ref[k] = s.plane(ref, k);
        fd.gold[k] = s.plane(gold, k);
      }
      fd.strideY = s.strideY;
      fd.strideC = s.strideC;
      fd.padW = s.geo.padW();
      fd.padH = s.geo.padH();
      fd.padCW = s.geo.padCW();
      fd.padCH = s.geo.padCH();
      fd.mbCols = s.geo.mbCols;
      fd.mbRows = s.geo.mbRows;
      fd.inter = inter ? 1 : 0;
      const Quant q = quantFor(plan.qp);
      fd.qdc = q.dc;
      fd.qac = q.ac;
      fd.tileCount = (int)plan.tiles.size();
      fd.pkt = j.dPkt ? j.dPkt : d + oPkt + j.stageOff;
      fd.tables = reinterpret_cast<const DeviceTables*>(d + oTab) + di;
      fd.tiles = reinterpret_cast<const TileRange*>(d + oTiles) + tileCur;
      fd.mbrec = s.dRec;
      fd.coef = s.dCoef;
      fd.mvgrid = s.dMV;
      fd.tileStat = ts;
      fd.status = reinterpret_cast<int32_t*>(d + oStat) + di;
      fd.gate = gateDesc >= 0 ? reinterpret_cast<const int32_t*>(d + oStat) + gateDesc : nullptr;
      hs[di] = 0;
      ht[di] = plan.tables;
      for (size_t t = 0; t < plan.tiles.size(); t++) {
        hr[tileCur + t] = plan.tiles[t];
        hj[tileCur + t] = make_int2(di, (int)t);
      }
      tileCur += (int)plan.tiles.size();
    };
    for (Job& j : jobs) {
      if (j.status != kOK || !j.gpu) continue;
      Stream& s = *streams_[(size_t)j.stream];
      fill(j, j.main, j.mainDesc, j.work, s.ref, s.golden, j.fh.coding == kCodingInter, -1, s.dTileStat);
      if (!s.resident) std::memcpy(h + oPkt + j.stageOff, j.hPkt, j.n);
    }
    for (Job& j : jobs) {
      if (j.status != kOK || !j.gpu || j.ovDesc < 0) continue;
      Stream& s = *streams_[(size_t)j.stream];
      fill(j, j.ov, j.ovDesc, j.ovBuf, j.work, j.work, true, j.mainDesc, s.dTileStatOv);
    }
    if (cudaMemcpyAsync(d, h, total, cudaMemcpyHostToDevice, stream_) != cudaSuccess) return -1;
    const FrameDesc* dd = reinterpret_cast<const FrameDesc*>(d + oDesc);
    const int2* dj = reinterpret_cast<const int2*>(d + oJobs);
    if (timing_) cudaEventRecord(ev_[0], stream_);
    launchEntropy(dd, dj, tMain, stream_);
    if (timing_) cudaEventRecord(ev_[1], stream_);
    if (maxMBs > 0) {
      launchInter(dd, nMain, maxMBs, stream_);
      launches_++;
    }
    launchIntra(dd, dj, tMain, stream_);
    launches_ += 2;
    if (nOv > 0) {
      // Override tile jobs index descriptors absolutely; the inter kernel
      // takes its frame from blockIdx.y, so it gets the override sub-array.
      launchEntropy(dd, dj + tMain, tOv, stream_);
      launchInter(dd + nMain, nOv, maxMBsOv, stream_);
      launchIntra(dd, dj + tMain, tOv, stream_);
      launches_ += 3;
    }
    if (timing_) cudaEventRecord(ev_[2], stream_);
    if (cudaMemcpyAsync(statuses.data(), d + oStat, sizeof(int32_t) * nDesc, cudaMemcpyDeviceToHost, stream_) !=
        cudaSuccess)
      return -1;
  }
  if (cudaStreamSynchronize(stream_) != cudaSuccess || cudaGetLastError() != cudaSuccess) {
    for (Job& j : jobs)
      if (j.status == kOK) j.status = kErrDevice;
  }
  if (timing_ && nDesc > 0) {
    float a = 0, b = 0;
    cudaEventElapsedTime(&a, ev_[0], ev_[1]);
    cudaEventElapsedTime(&b, ev_[1], ev_[2]);
    entropyMs_ += a;
    reconMs_ += b;
    kernelMs_ += a + b;
  }
  for (Job& j : jobs) {
    Stream& s = *streams_[(size_t)j.stream];
    if (!s.resident) s.pending = false;
    finishFrame(s, j, statuses.data(), results);
  }
  return (int)jobs.size();
}

int Engine::downloadFrame(const EngineFrameView& v, uint8_t* packed, size_t cap) {
  const int cw = (v.width + 1) / 2, ch = (v.height + 1) / 2;
  const size_t need = (size_t)v.width * v.height + 2 * (size_t)cw * ch;
  if (!v.y || cap < need) return kErrArg;
  uint8_t* y = packed;
  uint8_t* cb = packed + (size_t)v.width * v.height;
  uint8_t* cr = cb + (size_t)cw * ch;
  if (cudaMemcpy2DAsync(y, v.width, v.y, v.yStride, v.width, v.height, cudaMemcpyDeviceToHost, stream_) ||
      cudaMemcpy2DAsync(cb, cw, v.cb, v.cStride, cw, ch, cudaMemcpyDeviceToHost, stream_) ||
      cudaMemcpy2DAsync(cr, cw, v.cr, v.cStride, cw, ch, cudaMemcpyDeviceToHost, stream_))
    return kErrDevice;
  return cudaStreamSynchronize(stream_) == cudaSuccess ? kOK : kErrDevice;
}

int Engine::downloadStrided(const EngineFrameView& v, uint8_t* y, int ys, uint8_t* cb, uint8_t* cr, int cs) {
  const int cw = (v.width + 1) / 2, ch = (v.height + 1) / 2;
  if (cudaMemcpy2DAsync(y, ys, v.y, v.yStride, v.width, v.height, cudaMemcpyDeviceToHost, stream_) ||
      cudaMemcpy2DAsync(cb, cs, v.cb, v.cStride, cw, ch, cudaMemcpyDeviceToHost, stream_) ||
      cudaMemcpy2DAsync(cr, cs, v.cr, v.cStride, cw, ch, cudaMemcpyDeviceToHost, stream_))
    return kErrDevice;
  return kOK;
}

int Engine::copyReference(int id, int which, uint8_t* dst, size_t cap) {
  if (id < 0 || id >= (int)streams_.size() || !streams_[(size_t)id]) return kErrArg;
  Stream& s = *streams_[(size_t)id];
  if (!s.ready) return kErrArg;
  // Packed padded planes (Y then Cb then Cr at padded widths).
  const Geometry& g = s.geo;
  const size_t need = (size_t)g.padW() * g.padH() + 2 * (size_t)g.padCW() * g.padCH();
  if (cap < need) return kErrArg;
  const int b = which == 0 ? s.ref : s.golden;
  uint8_t* cb = dst + (size_t)g.padW() * g.padH();
  uint8_t* cr = cb + (size_t)g.padCW() * g.padCH();
  if (cudaMemcpy2DAsync(dst, g.padW(), s.plane(b, 0), s.strideY, g.padW(), g.padH(), cudaMemcpyDeviceToHost,
                        stream_) ||
      cudaMemcpy2DAsync(cb, g.padCW(), s.plane(b, 1), s.strideC, g.padCW(), g.padCH(), cudaMemcpyDeviceToHost,
                        stream_) ||
      cudaMemcpy2DAsync(cr, g.padCW(), s.plane(b, 2), s.strideC, g.padCW(), g.padCH(), cudaMemcpyDeviceToHost,
                        stream_))
    return kErrDevice;
  return cudaStreamSynchronize(stream_) == cudaSuccess ? kOK : kErrDevice;
}

}  // namespace ebiv

// ---------------------------------------------------------------------------
// C-ABI: batched decode of many independent streams
// ---------------------------------------------------------------------------
using namespace ebiv;

struct ebivgpu_batch {
  Engine e;
  std::vector<RoundResult> last;
};

extern "C" {

int ebivgpu_batch_create(ebivgpu_batch** out) {
  if (!out) return kErrArg;
  *out = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n <= 0) return kErrDevice;
  ebivgpu_batch* b = new (std::nothrow) ebivgpu_batch();
  if (!b) return kErrDevice;
  const int st = b->e.init();
  if (st) {
    delete b;
    return st;
  }
  *out = b;
  return kOK;
}

void ebivgpu_batch_destroy(ebivgpu_batch* b) { delete b; }

int ebivgpu_batch_add_stream(ebivgpu_batch* b, const uint8_t* const* pkts, const size_t* lens, int n, int ring,
                             int* stream_id) {
  if (!b || (!pkts && n) || !stream_id || n < 0) return kErrArg;
  return b->e.addResidentStream(pkts, lens, n, ring, stream_id);
}

int ebivgpu_batch_add_streaming(ebivgpu_batch* b, int ring, int* stream_id) {
  if (!b || !stream_id) return kErrArg;
  return b->e.addStreamingStream(ring, stream_id);
}

int ebivgpu_batch_submit(ebivgpu_batch* b, int stream_id, const uint8_t* pkt, size_t n) {
  if (!b || (!pkt && n)) return kErrArg;
  return b->e.submit(stream_id, pkt, n);
}

int ebivgpu_batch_seek(ebivgpu_batch* b, int stream_id, int64_t packet_index) {
  return b ? b->e.seekStream(stream_id, packet_index) : kErrArg;
}

int ebivgpu_batch_set_active(ebivgpu_batch* b, int stream_id, int active) {
  return b ? b->e.setActive(stream_id, active != 0) : kErrArg;
}

int ebivgpu_batch_remove_stream(ebivgpu_batch* b, int stream_id) { return b ? b->e.removeStream(stream_id) : kErrArg; }

int64_t ebivgpu_batch_remaining(ebivgpu_batch* b, int stream_id) { return b ? b->e.remaining(stream_id) : 0; }

int ebivgpu_batch_round(ebivgpu_batch* b, int* frames) {
  if (!b) return kErrArg;
  b->last.clear();
  const int n = b->e.round(&b->last);
  if (frames) *frames = n < 0 ? 0 : n;
  return n < 0 ? kErrDevice : kOK;
}

int ebivgpu_batch_round_for(ebivgpu_batch* b, const int* ids, int count, int* frames) {
  if (!b || (!ids && count)) return kErrArg;
  b->last.clear();
  std::vector<int> v(ids, ids + count);
  const int n = b->e.roundFor(v, &b->last);
  if (frames) *frames = n < 0 ? 0 : n;
  return n < 0 ? kErrDevice : kOK;
}

int ebivgpu_batch_result_count(ebivgpu_batch* b) { return b ? (int)b->last.size() : 0; }

int ebivgpu_batch_result(ebivgpu_batch* b, int i, int* stream_id, int64_t* frame_index, int* status, int* keyframe) {
  if (!b || i < 0 || i >= (int)b->last.size()) return kErrArg;
  const RoundResult& r = b->last[(size_t)i];
  if (stream_id) *stream_id = r.stream;
  if (frame_index) *frame_index = r.frameIndex;
  if (status) *status = r.status;
  if (keyframe) *keyframe = r.keyframe ? 1 : 0;
  return kOK;
}

int ebivgpu_batch_result_planes(ebivgpu_batch* b, int i, ebivgpu_plane_view* out) {
  if (!b || !out || i < 0 || i >= (int)b->last.size()) return kErrArg;
  const RoundResult& r = b->last[(size_t)i];
  if (r.status != kOK) return r.status;
  out->y = r.view.y;
  out->cb = r.view.cb;
  out->cr = r.view.cr;
  out->y_stride = r.view.yStride;
  out->c_stride = r.view.cStride;
  out->width = r.view.width;
  out->height = r.view.height;
  return kOK;
}

int ebivgpu_batch_result_download(ebivgpu_batch* b, int i, uint8_t* packed, size_t cap) {
  if (!b || i < 0 || i >= (int)b->last.size()) return kErrArg;
  const RoundResult& r = b->last[(size_t)i];
  if (r.status != kOK) return r.status;
  return b->e.downloadFrame(r.view, packed, cap);
}

int ebivgpu_batch_timing(ebivgpu_batch* b, int enable, double* kernel_ms, double* entropy_ms, double* recon_ms) {
  if (!b) return kErrArg;
  if (enable >= 0) {
    b->e.enableTiming(enable != 0);
    b->e.resetTiming();
  }
  if (kernel_ms) *kernel_ms = b->e.kernelMillis();
  if (entropy_ms) *entropy_ms = b->e.entropyMillis();
  if (recon_ms) *recon_ms = b->e.reconMillis();
  return kOK;
}

int64_t ebivgpu_batch_launches(ebivgpu_batch* b) { return b ? b->e.launches() : 0; }
uint64_t ebivgpu_batch_device_bytes(ebivgpu_batch* b) { return b ? (uint64_t)b->e.deviceBytes() : 0; }
uint64_t ebivgpu_stream_footprint(int w, int h, int ring) { return (uint64_t)Engine::footprint(w, h, ring); }

}  // extern "C"
