// Multi-stream decode engine (see engine.h) and its C-ABI.
#include <cuda_runtime.h>

#include <algorithm>
#include <map>
#include <chrono>
#include <cstring>
#include <new>

#include "../../include/ebivgpu.h"
#include "container.h"
#include "engine.h"
#include "gpu_codec.h"

namespace ebiv {

void launchEntropy(const FrameDesc* frames, const int4* jobs, int njobs, int* next, int maxTileMBs, cudaStream_t s);
void launchInter(const FrameDesc* frames, int nframes, int maxMBs, int phase, cudaStream_t s);
void launchIntra(const FrameDesc* frames, const int2* jobs, int njobs, int maxTileMBs, int maxTileKeys, int warps,
                 cudaStream_t s);
void launchRGBA(const uint8_t* y, const uint8_t* cb, const uint8_t* cr, int ys, int cs, int w, int h, uint8_t* dst,
                cudaStream_t s);

namespace {
inline size_t al(size_t v, size_t a) { return (v + a - 1) / a * a; }
inline int stride64(int w) { return (w + 63) & ~63; }
}  // namespace

// Per-frame scratch in HBM for one in-flight frame of a stream.
struct Slot {
  MBRec* rec = nullptr;
  uint32_t* coef = nullptr;
  int16_t* mv = nullptr;
  int16_t* lv = nullptr;
  uint32_t* intra = nullptr;  // intra list, then the level-sorted copy
  TileStat* ts = nullptr;
  // per macroblock: whether its inter prediction waits for the previous
  // frame's intra stage; then two intra progress bytes (large tiles)
  uint8_t* dep = nullptr;
  uint8_t* symLog = nullptr;   // the entropy stage's symbol log, kSymPerMB bytes per macroblock
  uint32_t* symOff = nullptr;  // per macroblock: its first symbol in its tile's log
  bool alloc(size_t mbs) {
    return cudaMalloc(&dep, 3 * mbs) == cudaSuccess && cudaMalloc(&rec, mbs * sizeof(MBRec)) == cudaSuccess &&
           cudaMalloc(&coef, mbs * kCoefPerMB * sizeof(uint32_t)) == cudaSuccess &&
           cudaMalloc(&mv, mbs * 2 * sizeof(int16_t)) == cudaSuccess &&
           cudaMalloc(&lv, mbs * sizeof(int16_t)) == cudaSuccess &&
           cudaMalloc(&intra, 2 * mbs * sizeof(uint32_t)) == cudaSuccess &&
           cudaMalloc(&ts, mbs * sizeof(TileStat)) == cudaSuccess &&
           cudaMalloc(&symLog, mbs * kSymPerMB) == cudaSuccess &&
           cudaMalloc(&symOff, mbs * sizeof(uint32_t)) == cudaSuccess;
  }
  void release() {
    cudaFree(dep);
    cudaFree(rec);
    cudaFree(coef);
    cudaFree(mv);
    cudaFree(lv);
    cudaFree(intra);
    cudaFree(ts);
    cudaFree(symLog);
    cudaFree(symOff);
  }
  static size_t bytes(size_t mbs) {
    return mbs * (sizeof(MBRec) + kCoefPerMB * 4 + 4 + 2 + 8 + sizeof(TileStat) + 3 + kSymPerMB + 4);
  }
};

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
  std::vector<int> outputs;  // FIFO of committed output buffers, oldest first
  int ref = -1, golden = -1;
  TableHistory hist;
  // Resident packets: per packet its host bytes (for planning) and its
  // offset in one device block.  A copied stream owns both (hostBlock, and
  // dPkts allocated by the engine); a container stream views a pinned,
  // device-mapped container, which the kernels read in place.
  std::vector<uint8_t> hostBlock;
  std::vector<const uint8_t*> hostPkt;
  std::vector<size_t> pktLen;
  uint8_t* dPkts = nullptr;
  size_t dPktsCap = 0;
  bool ownsPkts = true;
  std::vector<size_t> dOff;
  size_t packets() const { return hostPkt.size(); }
  // Copies n packets into hostBlock at 16-byte aligned offsets (dOff); returns the block size.
  size_t copyPackets(const uint8_t* const* pkts, const size_t* lens, int n) {
    size_t total = 0;
    dOff.resize((size_t)n);
    pktLen.resize((size_t)n);
    for (int i = 0; i < n; i++) {
      dOff[(size_t)i] = total;
      pktLen[(size_t)i] = lens[i];
      total += (lens[i] + 15) & ~(size_t)15;
    }
    hostBlock.assign(total ? total : 16, 0);
    hostPkt.resize((size_t)n);
    for (int i = 0; i < n; i++) {
      if (lens[i]) std::memcpy(hostBlock.data() + dOff[(size_t)i], pkts[i], lens[i]);
      hostPkt[(size_t)i] = hostBlock.data() + dOff[(size_t)i];
    }
    return total;
  }
  int64_t next = 0;
  // Streaming: the submitted packet awaiting its round.
  std::vector<uint8_t> pendingPkt;
  bool pending = false;
  std::vector<Slot> slots;
  size_t mbs = 0;
  size_t bytes = 0;
  // Pipelined rounds: references after the newest planned round (valid while
  // hasProv), pool buffers claimed per round parity, and an epoch bumped at
  // every rollback (jobs planned under an older epoch are discarded).
  bool hasProv = false;
  int pRef = -1, pGolden = -1;
  int64_t lastRound = 0;
  int64_t epoch = 0;
  std::vector<int> roundBufs[Engine::kParities];  // by round parity (the last: side lane)
  bool inSide = false;            // a side round holds this stream
  // Key-frame cache: per key frame decoded while caching is on, its image,
  // the golden image after it (only when an alt-ref override made them
  // differ) and the table history after it.  A key frame resets the table
  // history and every reference, so these are the whole decoder state after
  // it (ebiv/codec.go:155-191).
  struct CachedKey {
    uint8_t* img = nullptr;
    uint8_t* golden = nullptr;
    TableHistory hist;
  };
  bool cacheKeys = false;
  std::map<int64_t, CachedKey> keyCache;
  size_t cacheBytes = 0;
  bool inAside = false;  // a side-lane round decodes one of its key frames into the cache

  uint8_t* plane(int b, int k) const {
    return pool[(size_t)b] + (k == 0 ? 0 : yBytes + (size_t)(k - 1) * cBytes);
  }
  void release() {
    for (auto p : pool) cudaFree(p);
    pool.clear();
    for (auto& kv : keyCache) {
      cudaFree(kv.second.img);
      if (kv.second.golden) cudaFree(kv.second.golden);
    }
    keyCache.clear();
    for (auto& sl : slots) sl.release();
    slots.clear();
    if (dPkts && ownsPkts) cudaFree(dPkts);
    dPkts = nullptr;
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
  int ref = -1, golden = -1;  // references the frame decodes against
  bool hasOv = false;
  int ovPlanStatus = kOK;
  PayloadPlan main, ov;
  TableHistory hMain;    // table history after the main payload was planned
  TableHistory hBefore;  // table history before this frame was planned
  TableHistory hAfter;   // table history after this frame (and its override) was planned
  int step = 0, slot = -1;
  int mainDesc = -1, ovDesc = -1;
  int gateDesc = -1;  // descriptor whose status gates this frame (-1: none)
  size_t stageOff = 0;
  int64_t epoch = 0;  // the stream's epoch when planned
};

struct Engine::StepInfo {
  int mainFirst = 0, mainCount = 0, ovFirst = 0, ovCount = 0;
  int jobFirst = 0, jobCount = 0, ovJobFirst = 0, ovJobCount = 0;
  int maxMBs = 0, maxOvMBs = 0;  // largest frame of the step (macroblocks)
  bool hasPrev = false;  // a frame of the step follows a frame of the same round (two inter phases)
};

struct Engine::Round {
  int64_t id = 0;
  int parity = 0;
  std::vector<Job> jobs;
  std::vector<std::vector<int>> chains;  // per stream, indices into jobs in decode order
  std::vector<StepInfo> steps;
  int nDesc = 0, nTiles = 0, nEJobs = 0;
  int maxTileMBs = 0;   // largest tile of the round's frames (macroblocks)
  int maxTileKeys = 0;  // largest intra wavefront key range of those tiles
  int groups = 1, stepsPerGroup = 1;  // entropy launches (groups of consecutive steps)
  size_t oDesc = 0, oStat = 0, oJobs = 0, oEJobs = 0;
  bool launched = false;  // entropy launched; statuses pending
  bool reconLaunched = false;
  bool aside = false;     // key frames decoded only into their streams' key caches
  void noteTile(const TileRange& t) {
    const int w = t.mbX1 - t.mbX0, h = t.mbY1 - t.mbY0;
    maxTileMBs = std::max(maxTileMBs, w * h);
    maxTileKeys = std::max(maxTileKeys, 4 * (w - 1) + 11 * (h - 1) + 1);
  }
  void clear() {
    jobs.clear();
    chains.clear();
    steps.clear();
    nDesc = nTiles = nEJobs = maxTileMBs = maxTileKeys = 0;
    groups = stepsPerGroup = 1;
    launched = false;
    aside = false;
  }
};

Engine::Engine() : rounds_(new Round[kParities]) {}

Engine::~Engine() {
  if (streamE_) cudaStreamSynchronize(streamE_);
  if (stream_) cudaStreamSynchronize(stream_);
  for (auto& s : streams_)
    if (s) s->release();
  for (int l = 0; l < kSideLanes; l++) {
    if (streamES_[l]) cudaStreamSynchronize(streamES_[l]);
    if (streamRS_[l]) cudaStreamSynchronize(streamRS_[l]);
  }
  for (int p = 0; p < kParities; p++) {
    if (dStage_[p]) cudaFree(dStage_[p]);
    if (hStage_[p]) cudaFreeHost(hStage_[p]);
    if (hStatus_[p]) cudaFreeHost(hStatus_[p]);
    for (auto& e : ev_[p])
      if (e) cudaEventDestroy(e);
  }
  if (dOne_) cudaFree(dOne_);
  for (auto& e : sideDone_)
    if (e) cudaEventDestroy(e);
  if (mainDone_) cudaEventDestroy(mainDone_);
  if (streamC_) {
    cudaStreamSynchronize(streamC_);
    cudaStreamDestroy(streamC_);
  }
  if (copyDone_) cudaEventDestroy(copyDone_);
  if (reloadDone_) {
    cudaEventSynchronize(reloadDone_);
    cudaEventDestroy(reloadDone_);
  }
  if (streamB_) {
    cudaStreamSynchronize(streamB_);
    cudaStreamDestroy(streamB_);
  }
  for (int p = 0; p < kMainParities; p++)
    for (int k = 0; k < kMaxSteps; k++) {
      if (stepA_[p][k]) cudaEventDestroy(stepA_[p][k]);
      if (stepB_[p][k]) cudaEventDestroy(stepB_[p][k]);
    }
  for (auto& sg : streamEG_)
    if (sg) {
      cudaStreamSynchronize(sg);
      cudaStreamDestroy(sg);
    }
  for (int p = 0; p < kMainParities; p++) {
    if (evUp_[p]) cudaEventDestroy(evUp_[p]);
    for (auto& e : evGroup_[p])
      if (e) cudaEventDestroy(e);
  }
  for (int l = 0; l < kSideLanes; l++) {
    if (streamES_[l]) cudaStreamDestroy(streamES_[l]);
    if (streamRS_[l]) cudaStreamDestroy(streamRS_[l]);
  }
  if (ownStreamE_ && streamE_) cudaStreamDestroy(streamE_);
  if (ownStream_ && stream_) cudaStreamDestroy(stream_);
}

int Engine::init(cudaStream_t s) {
  if (s) {
    stream_ = s;
  } else {
    if (cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking) != cudaSuccess) return kErrDevice;
    ownStream_ = true;
  }
  for (auto& row : ev_)
    for (auto& e : row)
      if (cudaEventCreate(&e) != cudaSuccess) return kErrDevice;
  if (cudaStreamCreateWithFlags(&streamB_, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&streamC_, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&copyDone_, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&reloadDone_, cudaEventDisableTiming) != cudaSuccess)
    return kErrDevice;
  for (int p = 0; p < kMainParities; p++) {
    if (cudaEventCreateWithFlags(&evUp_[p], cudaEventDisableTiming) != cudaSuccess) return kErrDevice;
    for (auto& e : evGroup_[p])  // timed: the entropy time of a grouped round ends at its last group
      if (cudaEventCreate(&e) != cudaSuccess) return kErrDevice;
  }
  for (int p = 0; p < kMainParities; p++)
    for (int k = 0; k < kMaxSteps; k++)
      if (cudaEventCreateWithFlags(&stepA_[p][k], cudaEventDisableTiming) != cudaSuccess ||
          cudaEventCreateWithFlags(&stepB_[p][k], cudaEventDisableTiming) != cudaSuccess)
        return kErrDevice;
  int32_t one = 1;
  if (cudaMalloc(&dOne_, sizeof(int32_t)) != cudaSuccess ||
      cudaMemcpy(dOne_, &one, sizeof(one), cudaMemcpyHostToDevice) != cudaSuccess)
    return kErrDevice;
  return ensureDeviceTables();
}

int Engine::setLookahead(int k) {
  if (k < 1 || k > 64) return kErrArg;
  for (auto& s : streams_)
    if (s && s->ready) return kErrArg;  // pools are sized at configure
  lookahead_ = k;
  return kOK;
}

// Frame buffers per stream: the ring's outputs plus a round's, the two
// references, and the buffers a round claims; a pipelined engine of depth D
// holds D more rounds' worth of claims.
int Engine::poolSize(int ring, int k, int depth, bool side) {
  // A stream is in one side round at a time: its frames and an override.
  return ring + (2 + depth) * k + 3 + depth + (side ? kSideFrames + 1 : 0);
}

size_t Engine::footprint(int w, int h, int ring, int lookahead, int depth, int sideLanes) {
  const bool side = sideLanes > 0;
  const Geometry g = Geometry::of(w, h);
  const size_t yb = (size_t)stride64(g.padW()) * g.padH(), cb = (size_t)stride64(g.padCW()) * g.padCH();
  const size_t mbs = (size_t)g.mbCols * g.mbRows;
  return (size_t)poolSize(ring, lookahead, depth, side) * (yb + 2 * cb) +
         ((size_t)(depth + 1) * (lookahead + 1) +
          (size_t)(std::min(kSideFrames, lookahead) + 1) * (size_t)(side ? sideLanes : 0)) *
             Slot::bytes(mbs);
}

int Engine::addResidentStream(const uint8_t* const* pkts, const size_t* lens, int n, int ring, int* id) {
  std::unique_ptr<Stream> s(new (std::nothrow) Stream());
  if (!s) return kErrArg;
  s->resident = true;
  s->ring = ring >= 2 ? ring : 3;
  const size_t total = s->copyPackets(pkts, lens, n);
  if (cudaMalloc(&s->dPkts, total ? total : 16) != cudaSuccess) return kErrDevice;
  s->dPktsCap = total ? total : 16;
  if (total && cudaMemcpy(s->dPkts, s->hostBlock.data(), total, cudaMemcpyHostToDevice) != cudaSuccess)
    return kErrDevice;
  s->bytes += s->dPktsCap;
  deviceBytes_ += s->dPktsCap;
  s->id = (int)streams_.size();
  *id = s->id;
  streams_.push_back(std::move(s));
  return kOK;
}

int Engine::addContainerStream(const uint8_t* hostBase, const uint8_t* devBase, const uint64_t* off,
                               const uint32_t* pktLen, int n, int ring, int* id) {
  if (!hostBase || !devBase || (n && (!off || !pktLen)) || n < 0 || !id) return kErrArg;
  std::unique_ptr<Stream> s(new (std::nothrow) Stream());
  if (!s) return kErrArg;
  s->resident = true;
  s->ownsPkts = false;
  s->ring = ring >= 2 ? ring : 3;
  s->hostPkt.resize((size_t)n);
  s->pktLen.resize((size_t)n);
  s->dOff.resize((size_t)n);
  for (int i = 0; i < n; i++) {
    s->hostPkt[(size_t)i] = hostBase + off[i];
    s->pktLen[(size_t)i] = pktLen[i];
    s->dOff[(size_t)i] = (size_t)off[i];
  }
  s->dPkts = const_cast<uint8_t*>(devBase);
  s->id = (int)streams_.size();
  *id = s->id;
  streams_.push_back(std::move(s));
  return kOK;
}

// Replaces a resident stream's packets (a new clip on the same stream: it
// starts with a key frame of the stream's size) and rewinds it, keeping its
// frame pool.  The copies run on the entropy stream, ahead of the next
// round's entropy stage, the only reader of packet bytes.
int Engine::reloadStream(int id, const uint8_t* const* pkts, const size_t* lens, int n) {
  if (id < 0 || id >= (int)streams_.size() || !streams_[(size_t)id] || n < 0) return kErrArg;
  if (!pipe_.empty()) return kErrArg;  // drain() first
  Stream& s = *streams_[(size_t)id];
  if (!s.resident || !s.ownsPkts) return kErrArg;
  const size_t total = s.copyPackets(pkts, lens, n);  // host copies for planning
  cudaStream_t se = entropyStream();
  if (total > s.dPktsCap) {
    if (cudaStreamSynchronize(se) != cudaSuccess) return kErrDevice;
    cudaFree(s.dPkts);
    s.bytes -= s.dPktsCap;
    deviceBytes_ -= s.dPktsCap;
    s.dPkts = nullptr;
    s.dPktsCap = 0;
    if (cudaMalloc(&s.dPkts, total) != cudaSuccess) return kErrDevice;
    s.dPktsCap = total;
    s.bytes += total;
    deviceBytes_ += total;
  }
  for (int i = 0; i < n; i++)
    if (lens[i] &&
        cudaMemcpyAsync(s.dPkts + s.dOff[(size_t)i], pkts[i], lens[i], cudaMemcpyHostToDevice, se) != cudaSuccess)
      return kErrDevice;
  // syncCopies() waits for this event: after it the caller may reuse pkts.
  if (cudaEventRecord(reloadDone_, se) != cudaSuccess) return kErrDevice;
  reloadPending_ = true;
  s.next = 0;
  s.hasProv = false;
  s.epoch++;
  return kOK;
}

int Engine::downloadFrameAsync(const EngineFrameView& v, uint8_t* packed, size_t cap) {
  const int cw = (v.width + 1) / 2, ch = (v.height + 1) / 2;
  const size_t need = (size_t)v.width * v.height + 2 * (size_t)cw * ch;
  if (!v.y || cap < need) return kErrArg;
  uint8_t* y = packed;
  uint8_t* cb = packed + (size_t)v.width * v.height;
  uint8_t* cr = cb + (size_t)cw * ch;
  // A returned frame is complete (its round was collected), so the copy waits
  // for nothing; device work of later rounds waits for copyDone_.
  if (cudaMemcpy2DAsync(y, v.width, v.y, v.yStride, v.width, v.height, cudaMemcpyDeviceToHost, streamC_) ||
      cudaMemcpy2DAsync(cb, cw, v.cb, v.cStride, cw, ch, cudaMemcpyDeviceToHost, streamC_) ||
      cudaMemcpy2DAsync(cr, cw, v.cr, v.cStride, cw, ch, cudaMemcpyDeviceToHost, streamC_) ||
      cudaEventRecord(copyDone_, streamC_))
    return kErrDevice;
  copiesPending_ = true;
  return kOK;
}

int Engine::convertFrameAsync(const EngineFrameView& v, uint8_t* rgbaDev, uint8_t* rgbaHost) {
  if (!v.y || !rgbaDev || !rgbaHost) return kErrArg;
  launchRGBA(v.y, v.cb, v.cr, v.yStride, v.cStride, v.width, v.height, rgbaDev, streamC_);
  launches_++;
  if (cudaGetLastError() != cudaSuccess ||
      cudaMemcpyAsync(rgbaHost, rgbaDev, (size_t)v.width * v.height * 4, cudaMemcpyDeviceToHost, streamC_) ||
      cudaEventRecord(copyDone_, streamC_))
    return kErrDevice;
  copiesPending_ = true;
  return kOK;
}

int Engine::syncCopies() {
  if (cudaStreamSynchronize(streamC_) != cudaSuccess) return kErrDevice;
  copiesPending_ = false;
  if (reloadPending_ && cudaEventSynchronize(reloadDone_) != cudaSuccess) return kErrDevice;
  reloadPending_ = false;
  return kOK;
}

int Engine::addStreamingStream(int ring, int* id) {
  if (pipeDepth_) return kErrArg;  // pipelined rounds keep packets resident
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
  if (!s.resident || index < 0 || index > (int64_t)s.packets()) return kErrArg;
  s.next = index;
  return kOK;
}

int64_t Engine::remaining(int id) const {
  if (id < 0 || id >= (int)streams_.size() || !streams_[(size_t)id]) return 0;
  const Stream& s = *streams_[(size_t)id];
  return s.resident ? (int64_t)s.packets() - s.next : (s.pending ? 1 : 0);
}

int Engine::setActive(int id, bool active) {
  if (id < 0 || id >= (int)streams_.size() || !streams_[(size_t)id]) return kErrArg;
  streams_[(size_t)id]->active = active;
  return kOK;
}

int Engine::removeStream(int id) {
  if (id < 0 || id >= (int)streams_.size() || !streams_[(size_t)id]) return kErrArg;
  if (streamE_) cudaStreamSynchronize(streamE_);
  for (int l = 0; l < kSideLanes; l++) {
    if (streamES_[l]) cudaStreamSynchronize(streamES_[l]);
    if (streamRS_[l]) cudaStreamSynchronize(streamRS_[l]);
  }
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
  const int k = s.resident ? lookahead_ : 1;
  const int P = poolSize(s.ring, k, pipeDepth_, side_);
  cudaStream_t zs = planStream_ ? planStream_ : stream_;
  for (int i = 0; i < P; i++) {
    uint8_t* p = nullptr;
    if (cudaMalloc(&p, s.bufBytes) != cudaSuccess) return kErrDevice;
    if (cudaMemsetAsync(p, 0, s.bufBytes, zs) != cudaSuccess) return kErrDevice;
    s.pool.push_back(p);
  }
  // The reference allocates zeroed work/ref/golden buffers at configure.
  s.ref = 0;
  s.golden = 1;
  s.mbs = (size_t)s.geo.mbCols * s.geo.mbRows;
  // Slots: one per frame step and one for an override, per round parity.
  // Job slots index lookahead_ + 1 per parity; streaming streams use slot 0
  // and the override slot.
  const int perParity = lookahead_ + 1;
  s.slots.resize((size_t)slotSets() * perParity);
  size_t nSlots = 0;
  for (size_t i = 0; i < s.slots.size(); i++) {
    const int within = (int)(i % (size_t)perParity);
    const bool sideSet = (int)(i / (size_t)perParity) >= mainSets();
    if (within < (sideSet ? std::min(kSideFrames, k) : k) || within == perParity - 1) {
      if (!s.slots[i].alloc(s.mbs)) return kErrDevice;
      nSlots++;
    }
  }
  const size_t b = (size_t)P * s.bufBytes + nSlots * Slot::bytes(s.mbs);
  s.bytes += b;
  deviceBytes_ += b;
  s.ready = true;
  return kOK;
}

// Staging for round parity P (host pinned + device).  The other parity's
// round may be in flight; it never touches these buffers.
int Engine::ensureStage(int P, size_t bytes) {
  if (bytes <= stageCap_[P]) return kOK;
  const size_t cap = al(bytes + bytes / 2, 1 << 20);
  if (dStage_[P]) cudaFree(dStage_[P]);  // synchronises the device
  if (hStage_[P]) cudaFreeHost(hStage_[P]);
  dStage_[P] = nullptr;
  hStage_[P] = nullptr;
  stageCap_[P] = 0;
  if (cudaMalloc(&dStage_[P], cap) != cudaSuccess) return kErrDevice;
  if (cudaMallocHost(&hStage_[P], cap) != cudaSuccess) return kErrDevice;
  stageCap_[P] = cap;
  return kOK;
}

// Pinned host words the round's frame statuses are read back into.
int Engine::ensureStatus(int P, int n) {
  if (n <= statusCap_[P]) return kOK;
  const int cap = std::max(n * 2, 256);
  if (hStatus_[P]) cudaFreeHost(hStatus_[P]);
  hStatus_[P] = nullptr;
  statusCap_[P] = 0;
  if (cudaMallocHost(&hStatus_[P], sizeof(int32_t) * (size_t)cap) != cudaSuccess) return kErrDevice;
  statusCap_[P] = cap;
  return kOK;
}

// A pool buffer outside `busy` (the committed references and outputs plus
// everything the round has already claimed).
static int freeBuffer(size_t poolSize, const std::vector<char>& busy) {
  for (size_t i = 0; i < poolSize; i++)
    if (!busy[i]) return (int)i;
  return -1;
}

// Host half of Codec.Decode for one packet: header, configure, raw frames,
// payload planning (ebiv/codec.go:70-192).  ref/golden are the references the
// frame decodes against; busy marks pool buffers it must not claim.
int Engine::planFrame(Stream& s, Job& j, std::vector<char>& busy) {
  j.status = parseFrameHeader(j.hPkt, j.n, &j.fh);
  if (j.status) return j.status;
  if (j.fh.type == kFrameKey) {
    const bool first = !s.ready;
    j.status = configure(s, j.fh.width, j.fh.height);
    if (j.status) return j.status;
    if (first) {
      busy.assign(s.pool.size(), 0);
      busy[(size_t)s.ref] = busy[(size_t)s.golden] = 1;
      j.ref = s.ref;
      j.golden = s.golden;
    }
  } else if (!s.ready) {
    return j.status = kErrNoKeyframe;
  }
  const FrameHeader& fh = j.fh;
  if (fh.coding == kCodingRaw) {  // decodeRaw — ebiv/codec.go:195-207
    if (j.n - fh.bodyOffset != s.geo.packedSize()) return j.status = kErrCorrupt;
    j.work = freeBuffer(s.pool.size(), busy);
    if (j.work < 0) return j.status = kErrDevice;
    busy[(size_t)j.work] = 1;
    return kOK;
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
  j.hMain = s.hist;
  j.work = freeBuffer(s.pool.size(), busy);
  if (j.work < 0) return j.status = kErrDevice;
  busy[(size_t)j.work] = 1;
  if (key && fh.goldenOverride) {
    j.hasOv = true;
    // The override's tables chain after the key's (ebiv/codec.go:177-183);
    // s.hist holds them speculatively until the key's own decode is known.
    j.ovPlanStatus = planPayload(j.hPkt, ovOff, ovLen, false, s.geo.mbCols, s.geo.mbRows, s.hist, &j.ov);
    if (j.ovPlanStatus == kOK) {
      // The override decodes over a copy of the current golden so that a
      // failing override leaves the same partial image the reference's
      // in-place decode does.
      j.ovBuf = freeBuffer(s.pool.size(), busy);
      if (j.ovBuf < 0) return j.status = kErrDevice;
      busy[(size_t)j.ovBuf] = 1;
      if (cudaMemcpyAsync(s.pool[(size_t)j.ovBuf], s.pool[(size_t)j.golden], s.bufBytes, cudaMemcpyDeviceToDevice,
                          planStream_) != cudaSuccess)
        return j.status = kErrDevice;
    }
  }
  j.gpu = true;
  return kOK;
}

int Engine::finishFrame(Stream& s, Job& j, const int32_t* st, std::vector<RoundResult>* results) {
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
    const bool key = j.fh.type == kFrameKey;
    if (status != kOK) {
      if (j.hasOv) s.hist = j.hMain;  // the override's tables were never parsed
    } else if (key && j.hasOv) {
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
  if (out >= 0 && r.keyframe && s.cacheKeys && j.fh.coding != kCodingRaw)
    cacheKey(s, j.pktIndex, out, s.golden, j.hAfter);
  if (out >= 0) {
    s.outputs.push_back(out);
    const int cap = s.ring + (s.resident ? lookahead_ : 1);
    while ((int)s.outputs.size() > cap) s.outputs.erase(s.outputs.begin());
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
  return status;
}

int Engine::round(std::vector<RoundResult>* results) {
  std::vector<int> ids;
  for (auto& s : streams_)
    if (s && s->active && ((s->resident && s->next < (int64_t)s->packets()) || (!s->resident && s->pending)))
      ids.push_back(s->id);
  return roundFor(ids, results);
}

// ---------------------------------------------------------------------------
// A round: plan + entropy launch, reconstruction launch, collect.  Run back
// to back (the synchronous engine) or overlapped with the neighbouring rounds
// (the pipelined engine: round N+1 is planned and its entropy stage runs on
// the entropy stream while round N reconstructs on the engine's stream; round
// N+1's reconstruction is launched once round N has been collected, so a
// stream whose round-N chain failed has its round-N+1 frames skipped and
// re-planned).
// ---------------------------------------------------------------------------
int Engine::setPipelined(int depth) {
  if (depth < 0 || depth > kMaxDepth) return kErrArg;
  for (auto& s : streams_)
    if (s) return kErrArg;  // pool and slot counts depend on it
  const bool on = depth > 0;
  if (on && !streamE_) {
    if (cudaStreamCreateWithFlags(&streamE_, cudaStreamNonBlocking) != cudaSuccess) return kErrDevice;
    ownStreamE_ = true;
  }
  for (auto& sg : streamEG_)
    if (on && !sg && cudaStreamCreateWithFlags(&sg, cudaStreamNonBlocking) != cudaSuccess) return kErrDevice;
  pipeDepth_ = depth;
  return kOK;
}

int Engine::planRound(const std::vector<int>& ids, const std::vector<int>* maxFrames, Round& R) {
  R.clear();
  R.id = ++roundSeq_;
  const int P = R.parity;
  std::vector<Job>& jobs = R.jobs;
  jobs.reserve(ids.size() * (size_t)lookahead_);
  size_t streamedBytes = 0;
  cudaStream_t se = entropyStream(P);
  cudaStream_t sr = reconStream(P);
  planStream_ = sr;
  // Frame-buffer writes of this round (raw frames, override copies, the
  // reconstruction) come after every queued download.
  if (copiesPending_ && cudaStreamWaitEvent(sr, copyDone_, 0) != cudaSuccess) return -1;
  for (size_t ii = 0; ii < ids.size(); ii++) {
    const int id = ids[ii];
    if (id < 0 || id >= (int)streams_.size() || !streams_[(size_t)id]) continue;
    Stream& s = *streams_[(size_t)id];
    // A stream in the side lane stays out of main rounds; the side lane takes
    // only streams with no round in flight.
    if (isSide(P) ? (s.inSide || s.hasProv || s.inAside) : s.inSide) continue;
    std::vector<int> chain;
    std::vector<char> busy;
    // Start from the provisional references after the stream's in-flight
    // round, when it has one.
    int provRef = s.hasProv ? s.pRef : s.ref, provGolden = s.hasProv ? s.pGolden : s.golden;
    busy.assign(s.pool.size(), 0);
    if (provRef >= 0) busy[(size_t)provRef] = 1;
    if (provGolden >= 0) busy[(size_t)provGolden] = 1;
    for (int b : s.outputs) busy[(size_t)b] = 1;
    for (int q = 0; q < kParities; q++)
      if (q != P)
        for (int b : s.roundBufs[q]) busy[(size_t)b] = 1;
    s.roundBufs[P].clear();
    int k = s.resident ? lookahead_ : 1;
    if (maxFrames && ii < maxFrames->size()) k = std::max(0, std::min(k, (*maxFrames)[ii]));
    const int slotBase = slotSet(P) * (lookahead_ + 1);
    int lastGpu = -1;  // job index of the chain's last GPU frame
    for (int step = 0; step < k; step++) {
      Job j;
      j.stream = id;
      j.step = step;
      j.epoch = s.epoch;
      if (s.resident) {
        if (s.next >= (int64_t)s.packets()) break;
        j.pktIndex = s.next;
        j.hPkt = s.hostPkt[(size_t)s.next];
        j.n = s.pktLen[(size_t)s.next];
        j.dPkt = s.dPkts + s.dOff[(size_t)s.next];
        s.next++;
      } else {
        if (!s.pending) break;
        j.hPkt = s.pendingPkt.data();
        j.n = s.pendingPkt.size();
        j.pktIndex = s.next++;
        s.pending = false;
      }
      j.ref = provRef;
      j.golden = provGolden;
      j.slot = slotBase + step;
      j.hBefore = s.hist;
      planFrame(s, j, busy);
      j.hAfter = s.hist;
      // (configure may have allocated the pool: references start as the zeroed buffers)
      if (j.ref < 0) j.ref = s.ref;
      if (j.golden < 0) j.golden = s.golden;
      if (j.work >= 0) s.roundBufs[P].push_back(j.work);
      if (j.ovBuf >= 0) s.roundBufs[P].push_back(j.ovBuf);
      if (j.status == kOK && j.gpu) {
        j.gateDesc = lastGpu;  // resolved to a descriptor index below
        if (!s.resident) {
          j.stageOff = streamedBytes;
          streamedBytes += al(j.n, 16);
        }
        provRef = j.work;
        if (j.fh.type == kFrameKey) provGolden = (j.hasOv && j.ovPlanStatus == kOK) ? j.ovBuf : j.work;
        lastGpu = (int)jobs.size();
      }
      const bool stop = j.hasOv;  // an override's outcome decides golden: end the chain here
      chain.push_back((int)jobs.size());
      jobs.push_back(std::move(j));
      if (stop) break;
    }
    if (!chain.empty()) {
      R.chains.push_back(std::move(chain));
      s.pRef = provRef;
      s.pGolden = provGolden;
      s.hasProv = true;
      s.lastRound = R.id;
      if (isSide(P)) s.inSide = true;
    }
  }
  // Raw frames: scatter the packed planes into their pool buffer (engine
  // stream: after the previous round's reconstruction, before this one's).
  for (Job& j : jobs) {
    if (j.status != kOK || j.fh.coding != kCodingRaw) continue;
    Stream& s = *streams_[(size_t)j.stream];
    const Geometry& g = s.geo;
    const uint8_t* body = j.hPkt + j.fh.bodyOffset;
    const size_t ys = (size_t)g.W * g.H, cs = (size_t)g.CW * g.CH;
    if (cudaMemcpy2DAsync(s.plane(j.work, 0), s.strideY, body, g.W, g.W, g.H, cudaMemcpyHostToDevice, sr) ||
        cudaMemcpy2DAsync(s.plane(j.work, 1), s.strideC, body + ys, g.CW, g.CW, g.CH, cudaMemcpyHostToDevice, sr) ||
        cudaMemcpy2DAsync(s.plane(j.work, 2), s.strideC, body + ys + cs, g.CW, g.CW, g.CH, cudaMemcpyHostToDevice,
                          sr))
      j.status = kErrDevice;
  }
  // ---- descriptors grouped by step: [main step 0][ov step 0][main step 1]... --
  int maxStep = -1;
  for (const Job& j : jobs)
    if (j.status == kOK && j.gpu) maxStep = std::max(maxStep, j.step);
  R.steps.assign((size_t)(maxStep + 1), StepInfo{});
  int nDesc = 0, nTiles = 0;
  for (int st = 0; st <= maxStep; st++) {
    StepInfo& si = R.steps[(size_t)st];
    si.mainFirst = nDesc;
    si.jobFirst = nTiles;
    for (Job& j : jobs) {
      if (j.status != kOK || !j.gpu || j.step != st) continue;
      j.mainDesc = nDesc++;
      si.mainCount++;
      nTiles += (int)j.main.tiles.size();
      si.jobCount += (int)j.main.tiles.size();
      si.maxMBs = std::max(si.maxMBs, (int)streams_[(size_t)j.stream]->mbs);
      for (const TileRange& t : j.main.tiles) R.noteTile(t);
    }
    si.ovFirst = nDesc;
    si.ovJobFirst = nTiles;
    for (Job& j : jobs) {
      if (j.status != kOK || !j.gpu || j.step != st || !j.hasOv || j.ovPlanStatus != kOK) continue;
      j.ovDesc = nDesc++;
      si.ovCount++;
      nTiles += (int)j.ov.tiles.size();
      si.ovJobCount += (int)j.ov.tiles.size();
      si.maxOvMBs = std::max(si.maxOvMBs, (int)streams_[(size_t)j.stream]->mbs);
      for (const TileRange& t : j.ov.tiles) R.noteTile(t);
    }
  }
  R.nDesc = nDesc;
  R.nTiles = nTiles;
  if (nDesc == 0) return kOK;
  // Entropy jobs: groups of up to kEntropyTilesPerJob tiles of one frame.
  std::vector<int> tilesOf((size_t)nDesc, 0);
  for (const Job& j : jobs) {
    if (j.mainDesc >= 0) tilesOf[(size_t)j.mainDesc] = (int)j.main.tiles.size();
    if (j.ovDesc >= 0) tilesOf[(size_t)j.ovDesc] = (int)j.ov.tiles.size();
  }
  int nEJobs = 0;
  for (int t : tilesOf) nEJobs += (t + kEntropyTilesPerJob - 1) / kEntropyTilesPerJob;
  R.nEJobs = nEJobs;
  // Pipelined main rounds decode their steps' tiles in up to kEntropyGroups
  // launches of consecutive steps on separate streams, so a step's
  // reconstruction waits only for its own group: the long chains of a large
  // frame late in the round do not hold back the steps before it.
  const int nsteps = (int)R.steps.size();
  R.groups = (!isSide(P) && pipeDepth_ && streamEG_[0] && nsteps > 1) ? std::min(entropyGroups_, nsteps) : 1;
  R.stepsPerGroup = (nsteps + R.groups - 1) / R.groups;
  R.groups = (nsteps + R.stepsPerGroup - 1) / R.stepsPerGroup;
  R.oDesc = 0;
  R.oStat = al(R.oDesc + sizeof(FrameDesc) * nDesc, 64);
  const size_t oTab = al(R.oStat + sizeof(int32_t) * nDesc, 64);
  const size_t oTiles = al(oTab + sizeof(DeviceTables) * nDesc, 64);
  R.oJobs = al(oTiles + sizeof(TileRange) * (size_t)nTiles, 64);
  R.oEJobs = al(R.oJobs + sizeof(int2) * (size_t)nTiles, 64);
  const size_t oQueue = al(R.oEJobs + sizeof(int4) * (size_t)nEJobs, 64);  // entropy job counters, 64 B apart
  const size_t oPkt = al(oQueue + 64 * (size_t)R.groups, 256);
  const size_t total = oPkt + streamedBytes;
  if (ensureStage(P, total) || ensureStatus(P, nDesc)) return -1;
  uint8_t* h = hStage_[P];
  uint8_t* d = dStage_[P];
  FrameDesc* hd = reinterpret_cast<FrameDesc*>(h + R.oDesc);
  int32_t* hs = reinterpret_cast<int32_t*>(h + R.oStat);
  DeviceTables* ht = reinterpret_cast<DeviceTables*>(h + oTab);
  TileRange* hr = reinterpret_cast<TileRange*>(h + oTiles);
  int2* hj = reinterpret_cast<int2*>(h + R.oJobs);
  // Tile jobs are laid out in descriptor order, so each descriptor's tiles
  // and each step's job ranges are contiguous.
  std::vector<int> tileFirst((size_t)nDesc, 0);
  {
    int acc = 0;
    for (int di = 0; di < nDesc; di++) {
      tileFirst[(size_t)di] = acc;
      acc += tilesOf[(size_t)di];
    }
  }
  std::vector<const PayloadPlan*> planOf((size_t)nDesc, nullptr);
  auto fill = [&](const Job& j, const PayloadPlan& plan, int di, int rec, int ref, int gold, bool inter, int gateDesc,
                  const Slot& sl, const Job* prev) {
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
    const int tf = tileFirst[(size_t)di];
    fd.tiles = reinterpret_cast<const TileRange*>(d + oTiles) + tf;
    fd.mbrec = sl.rec;
    fd.coef = sl.coef;
    fd.mvgrid = sl.mv;
    fd.lvgrid = sl.lv;
    fd.intraList = sl.intra;
    fd.intraSorted = sl.intra + s.mbs;
    fd.tileStat = sl.ts;
    fd.symLog = sl.symLog;
    fd.symOff = sl.symOff;
    fd.symPerMB = kSymPerMB;
    fd.status = reinterpret_cast<int32_t*>(d + R.oStat) + di;
    fd.gate = gateDesc >= 0 ? reinterpret_cast<const int32_t*>(d + R.oStat) + gateDesc : nullptr;
    fd.dep = sl.dep;
    fd.prevRec = nullptr;
    fd.prevKey = 0;
    if (prev) {  // the previous frame of the chain, reconstructed one step earlier in this round
      const Stream& ps = *streams_[(size_t)prev->stream];
      fd.prevRec = ps.slots[(size_t)prev->slot].rec;
      fd.prevKey = prev->fh.type == kFrameKey ? 1 : 0;
    }
    hs[di] = 0;
    ht[di] = plan.tables;
    for (size_t t = 0; t < plan.tiles.size(); t++) {
      hr[tf + t] = plan.tiles[t];
      hj[tf + t] = make_int2(di, (int)t);
    }
    planOf[(size_t)di] = &plan;
  };
  for (Job& j : jobs) {
    if (j.mainDesc < 0) continue;
    Stream& s = *streams_[(size_t)j.stream];
    const int gate = j.gateDesc >= 0 ? jobs[(size_t)j.gateDesc].mainDesc : -1;
    const int ovSlot = slotSet(P) * (lookahead_ + 1) + lookahead_;
    const Job* prev = j.gateDesc >= 0 ? &jobs[(size_t)j.gateDesc] : nullptr;
    fill(j, j.main, j.mainDesc, j.work, j.ref, j.golden, j.fh.coding == kCodingInter, gate, s.slots[(size_t)j.slot],
         prev);
    if (prev && j.fh.coding == kCodingInter) R.steps[(size_t)j.step].hasPrev = true;
    if (!s.resident) std::memcpy(h + oPkt + j.stageOff, j.hPkt, j.n);
    if (j.ovDesc >= 0)
      fill(j, j.ov, j.ovDesc, j.ovBuf, j.work, j.work, true, j.mainDesc, s.slots[(size_t)ovSlot], nullptr);
  }
  {
    // Each intra launch takes its tiles largest first, so a large tile never
    // starts in a late wave.
    auto tileMBs = [&](const int2& jb) {
      const TileRange& t = planOf[(size_t)jb.x]->tiles[(size_t)jb.y];
      return (int)(t.mbX1 - t.mbX0) * (int)(t.mbY1 - t.mbY0);
    };
    auto larger = [&](const int2& a, const int2& b) { return tileMBs(a) > tileMBs(b); };
    for (const StepInfo& si : R.steps) {
      std::stable_sort(hj + si.jobFirst, hj + si.jobFirst + si.jobCount, larger);
      std::stable_sort(hj + si.ovJobFirst, hj + si.ovJobFirst + si.ovJobCount, larger);
    }
  }
  int groupFirst[kEntropyGroups + 1] = {0};
  {
    // By group, then longest tile first, so the slowest chains start in the
    // first wave.
    std::vector<int> groupOf((size_t)nDesc, 0);
    for (int st = 0; st < nsteps; st++) {
      const StepInfo& si = R.steps[(size_t)st];
      for (int di = si.mainFirst; di < si.mainFirst + si.mainCount; di++) groupOf[(size_t)di] = st / R.stepsPerGroup;
      for (int di = si.ovFirst; di < si.ovFirst + si.ovCount; di++) groupOf[(size_t)di] = st / R.stepsPerGroup;
    }
    struct EJob {
      int group;
      uint32_t longest;
      int4 job;
    };
    std::vector<EJob> ej;
    ej.reserve((size_t)nEJobs);
    for (int di = 0; di < nDesc; di++) {
      for (int t0 = 0; t0 < tilesOf[(size_t)di]; t0 += kEntropyTilesPerJob) {
        const int nt = std::min(kEntropyTilesPerJob, tilesOf[(size_t)di] - t0);
        uint32_t longest = 0;
        for (int t = t0; t < t0 + nt; t++) longest = std::max(longest, planOf[(size_t)di]->tiles[(size_t)t].length);
        ej.push_back({groupOf[(size_t)di], longest, make_int4(di, t0, nt, 0)});
      }
    }
    std::stable_sort(ej.begin(), ej.end(), [](const EJob& a, const EJob& b) {
      return a.group != b.group ? a.group < b.group : a.longest > b.longest;
    });
    int4* he = reinterpret_cast<int4*>(h + R.oEJobs);
    for (size_t k = 0; k < ej.size(); k++) {
      he[k] = ej[k].job;
      groupFirst[ej[k].group + 1] = (int)k + 1;
    }
    for (int g = 1; g <= R.groups; g++) groupFirst[g] = std::max(groupFirst[g], groupFirst[g - 1]);
    for (int g = 0; g < R.groups; g++) *reinterpret_cast<int32_t*>(h + oQueue + 64 * (size_t)g) = 0;
  }
  if (cudaMemcpyAsync(d, h, total, cudaMemcpyHostToDevice, se) != cudaSuccess) return -1;
  const FrameDesc* dd = reinterpret_cast<const FrameDesc*>(d + R.oDesc);
  const int4* de = reinterpret_cast<const int4*>(d + R.oEJobs);
  if (timing_) cudaEventRecord(ev_[P][0], se);
  if (R.groups == 1) {
    launchEntropy(dd, de, nEJobs, reinterpret_cast<int32_t*>(d + oQueue), R.maxTileMBs, se);
    launches_++;
    cudaEventRecord(ev_[P][1], se);  // entropy done
  } else {
    // The entropy stream carries only the staging copy; the groups run on
    // pool streams after it.
    if (cudaEventRecord(evUp_[P], se) != cudaSuccess) return -1;
    for (int g = 0; g < R.groups; g++) {
      cudaStream_t sg = streamEG_[nextEG_];
      nextEG_ = (nextEG_ + 1) % kEntropyStreams;
      if (cudaStreamWaitEvent(sg, evUp_[P], 0) != cudaSuccess) return -1;
      launchEntropy(dd, de + groupFirst[g], groupFirst[g + 1] - groupFirst[g],
                    reinterpret_cast<int32_t*>(d + oQueue + 64 * (size_t)g), R.maxTileMBs, sg);
      launches_++;
      if (cudaEventRecord(evGroup_[P][g], sg) != cudaSuccess) return -1;
    }
  }
  R.launched = true;
  planStream_ = nullptr;
  return kOK;
}

int Engine::launchRecon(Round& R) {
  if (!R.launched) return kOK;
  const int P = R.parity;
  cudaStream_t sr = reconStream(P);
  uint8_t* h = hStage_[P];
  uint8_t* d = dStage_[P];
  // Frames of streams rolled back since planning: point their gate at a word
  // that is always set, so the reconstruction skips them.
  for (Job& j : R.jobs) {
    const Stream* s = j.stream >= 0 && j.stream < (int)streams_.size() ? streams_[(size_t)j.stream].get() : nullptr;
    if (s && j.epoch == s->epoch) continue;
    for (int di : {j.mainDesc, j.ovDesc}) {
      if (di < 0) continue;
      FrameDesc* hd = reinterpret_cast<FrameDesc*>(h + R.oDesc) + di;
      hd->gate = dOne_;
      FrameDesc* ddi = reinterpret_cast<FrameDesc*>(d + R.oDesc) + di;
      if (cudaMemcpyAsync(&ddi->gate, &hd->gate, sizeof(hd->gate), cudaMemcpyHostToDevice, sr) != cudaSuccess)
        return -1;
    }
  }
  // A step's reconstruction waits for its entropy group (the whole entropy
  // stage when the round has one group).
  const bool grouped = R.groups > 1;
  auto entropyDone = [&](int st) { return grouped ? evGroup_[P][st / R.stepsPerGroup] : ev_[P][1]; };
  if (cudaStreamWaitEvent(sr, entropyDone(0), 0) != cudaSuccess) return -1;
  if (copiesPending_ && cudaStreamWaitEvent(sr, copyDone_, 0) != cudaSuccess) return -1;
  int groupA = 0, groupB = -1;
  const FrameDesc* dd = reinterpret_cast<const FrameDesc*>(d + R.oDesc);
  const int2* dj = reinterpret_cast<const int2*>(d + R.oJobs);
  if (timing_) cudaEventRecord(ev_[P][2], sr);
  // Per step: inter phase 0 (macroblocks independent of the previous step's
  // intra stage), inter phase 1 (the rest), intra.  On main rounds phase 0 of
  // step s+1 runs on a second stream beside step s's intra stage: it waits
  // for step s's inter pixels (event A) and step s+1's phase 1 waits for it
  // (event B).
  const int nsteps = (int)R.steps.size();
  const bool split = !isSide(P) && streamB_ && nsteps > 1 && nsteps <= kMaxSteps;
  for (int st = 0; st < nsteps; st++) {
    const StepInfo& si = R.steps[(size_t)st];
    if (grouped && st / R.stepsPerGroup != groupA) {
      groupA = st / R.stepsPerGroup;
      if (cudaStreamWaitEvent(sr, entropyDone(st), 0) != cudaSuccess) return -1;
    }
    if (split && st > 0) {
      if (cudaStreamWaitEvent(sr, stepB_[P][st], 0) != cudaSuccess) return -1;
    } else if (si.maxMBs > 0) {
      launchInter(dd + si.mainFirst, si.mainCount, si.maxMBs, 0, sr);
      launches_++;
    }
    if (si.maxMBs > 0 && si.hasPrev) {
      launchInter(dd + si.mainFirst, si.mainCount, si.maxMBs, 1, sr);
      launches_++;
    }
    if (split && st + 1 < nsteps) {
      const StepInfo& nx = R.steps[(size_t)st + 1];
      if (cudaEventRecord(stepA_[P][st], sr) != cudaSuccess ||
          cudaStreamWaitEvent(streamB_, stepA_[P][st], 0) != cudaSuccess)
        return -1;
      const int gB = grouped ? (st + 1) / R.stepsPerGroup : 0;
      if (gB != groupB) {
        groupB = gB;
        if (cudaStreamWaitEvent(streamB_, entropyDone(st + 1), 0) != cudaSuccess) return -1;
      }
      if (nx.maxMBs > 0) {
        launchInter(dd + nx.mainFirst, nx.mainCount, nx.maxMBs, 0, streamB_);
        launches_++;
      }
      if (cudaEventRecord(stepB_[P][st + 1], streamB_) != cudaSuccess) return -1;
    }
    if (si.jobCount > 0) {
      launchIntra(dd, dj + si.jobFirst, si.jobCount, R.maxTileMBs, R.maxTileKeys, intraWarps_, sr);
      launches_++;
    }
    if (si.ovCount > 0) {
      launchInter(dd + si.ovFirst, si.ovCount, si.maxOvMBs, 0, sr);
      launchIntra(dd, dj + si.ovJobFirst, si.ovJobCount, R.maxTileMBs, R.maxTileKeys, intraWarps_, sr);
      launches_ += 2;
    }
  }
  if (timing_) cudaEventRecord(ev_[P][3], sr);
  if (cudaMemcpyAsync(hStatus_[P], d + R.oStat, sizeof(int32_t) * R.nDesc, cudaMemcpyDeviceToHost, sr) !=
      cudaSuccess)
    return -1;
  return kOK;
}

int Engine::collectRound(Round& R, std::vector<RoundResult>* results) {
  const int P = R.parity;
  const bool gpu = R.nDesc > 0;
  std::vector<int32_t> statuses((size_t)std::max(R.nDesc, 1), 0);
  if (cudaStreamSynchronize(reconStream(P)) != cudaSuccess || cudaGetLastError() != cudaSuccess) {
    for (Job& j : R.jobs)
      if (j.status == kOK) j.status = kErrDevice;
  } else if (gpu) {
    std::memcpy(statuses.data(), hStatus_[P], sizeof(int32_t) * R.nDesc);
  }
  if (timing_ && gpu) {
    float a = 0, b = 0;
    if (R.groups > 1) {  // entropy time: until the last group is done
      for (int g = 0; g < R.groups; g++) {
        float t = 0;
        cudaEventElapsedTime(&t, ev_[P][0], evGroup_[P][g]);
        a = std::max(a, t);
      }
    } else {
      cudaEventElapsedTime(&a, ev_[P][0], ev_[P][1]);
    }
    cudaEventElapsedTime(&b, ev_[P][2], ev_[P][3]);
    entropyMs_ += a;
    reconMs_ += b;
    kernelMs_ += a + b;
  }
  if (R.aside) {  // key frames into the caches; the streams' state is untouched
    for (const Job& j : R.jobs) {
      if (j.stream < 0 || j.stream >= (int)streams_.size() || !streams_[(size_t)j.stream]) continue;
      Stream& s = *streams_[(size_t)j.stream];
      s.roundBufs[P].clear();
      s.inAside = false;
      const bool ok = j.status == kOK && j.gpu && j.mainDesc >= 0 && statuses[(size_t)j.mainDesc] == kOK &&
                      j.fh.type == kFrameKey && j.work >= 0 &&
                      (!j.hasOv || (j.ovPlanStatus == kOK && j.ovDesc >= 0 && statuses[(size_t)j.ovDesc] == kOK));
      if (ok) cacheKey(s, j.pktIndex, j.work, j.hasOv ? j.ovBuf : j.work, j.hAfter);
    }
    R.clear();
    return 0;
  }
  // ---- commit each stream's chain in order; roll back at the first skipped frame
  int attempted = 0;
  for (const auto& chain : R.chains) {
    const int id = R.jobs[(size_t)chain[0]].stream;
    if (id < 0 || id >= (int)streams_.size() || !streams_[(size_t)id]) continue;  // removed meanwhile
    Stream& s = *streams_[(size_t)id];
    s.roundBufs[P].clear();
    if (isSide(P)) s.inSide = false;
    if (R.jobs[(size_t)chain[0]].epoch != s.epoch) continue;  // planned before a rollback: discarded
    // A newer round of this stream was planned on top of this chain's
    // outcome; commit this chain as if it were the newest.
    const bool newer = s.lastRound > R.id;
    TableHistory newest;
    if (newer) {
      newest = s.hist;
      s.hist = R.jobs[(size_t)chain.back()].hAfter;
    }
    bool rolledBack = false, failed = false;
    for (size_t c = 0; c < chain.size(); c++) {
      Job& j = R.jobs[(size_t)chain[c]];
      if (j.mainDesc >= 0 && statuses[(size_t)j.mainDesc] == kSkipped) {
        // The frame this one depended on failed: re-plan from here with the
        // table history as it stood before this frame was planned; anything
        // planned after it is discarded.
        s.hist = j.hBefore;
        s.next = j.pktIndex;
        rolledBack = true;
        break;
      }
      failed = finishFrame(s, j, statuses.data(), results) != kOK || failed;
      attempted++;
    }
    if (rolledBack || (newer && failed)) {
      // The newer round assumed this chain's frames succeeded: discard it and
      // continue after this chain.
      if (!rolledBack) s.next = R.jobs[(size_t)chain.back()].pktIndex + 1;
      s.epoch++;
      s.hasProv = false;
    } else if (newer) {
      s.hist = newest;
    }
    if (s.lastRound == R.id) s.hasProv = false;  // no later round holds provisional state
  }
  R.clear();
  return attempted;
}

int Engine::roundFor(const std::vector<int>& ids, std::vector<RoundResult>* results,
                     const std::vector<int>* maxFrames) {
  if (!pipeDepth_) {
    Round& R = rounds_[0];
    R.parity = 0;
    const auto t0 = std::chrono::steady_clock::now();
    const bool failed = planRound(ids, maxFrames, R) != 0;
    const auto t1 = std::chrono::steady_clock::now();
    if (failed || launchRecon(R)) {
      for (Job& j : R.jobs)
        if (j.status == kOK) j.status = kErrDevice;
      R.nDesc = 0;
      collectRound(R, results);
      return -1;
    }
    const auto t2 = std::chrono::steady_clock::now();
    const int n = collectRound(R, results);
    const auto t3 = std::chrono::steady_clock::now();
    planSec_ += std::chrono::duration<double>(t1 - t0).count();
    launchSec_ += std::chrono::duration<double>(t2 - t1).count();
    collectSec_ += std::chrono::duration<double>(t3 - t2).count();
    return n;
  }
  // Pipelined: plan this round and start its entropy stage; when more than
  // depth rounds are in flight, collect the oldest (whose results this call
  // returns); then launch the reconstruction of the oldest round not yet
  // reconstructing (its predecessor has been collected).
  int p = 0;
  for (bool used = true; used; p++) {
    used = false;
    for (int q : pipe_) used = used || q == p;
    if (!used) break;
  }
  Round& R = rounds_[p];
  R.parity = p;
  R.reconLaunched = false;
  int failed = planRound(ids, maxFrames, R) ? p : -1;
  pipe_.push_back(p);
  int n = 0;
  if ((int)pipe_.size() > pipeDepth_ && rounds_[pipe_.front()].reconLaunched) {
    n = collectRound(rounds_[pipe_.front()], results);
    pipe_.erase(pipe_.begin());
  }
  Round& F = rounds_[pipe_.front()];
  if (!F.reconLaunched) {
    if (failed != F.parity && launchRecon(F)) failed = F.parity;
    F.reconLaunched = true;
  }
  if (failed >= 0) {  // a device call failed: finish every round in flight
    for (int q : pipe_) {
      Round& X = rounds_[q];
      if (q == failed) {
        for (Job& j : X.jobs)
          if (j.status == kOK) j.status = kErrDevice;
        X.nDesc = 0;
      }
      if (!X.reconLaunched && q != failed) launchRecon(X);
      n += collectRound(X, results);
    }
    pipe_.clear();
    return -1;
  }
  return n;
}

int Engine::decodeInto(int id, uint8_t* y, int ys, uint8_t* cb, uint8_t* cr, int cs,
                       std::vector<RoundResult>* results, uint8_t* rgbaDev, uint8_t* rgbaHost) {
  if (pipeDepth_ || id < 0 || id >= (int)streams_.size() || !streams_[(size_t)id]) return kErrArg;
  Round& R = rounds_[0];
  R.parity = 0;
  bool failed = planRound({id}, nullptr, R) || launchRecon(R);
  if (!failed && R.jobs.size() == 1 && R.jobs[0].status == kOK && R.jobs[0].work >= 0) {
    const Stream& s = *streams_[(size_t)id];
    const int b = R.jobs[0].work, w = s.geo.W, h = s.geo.H, cw = (w + 1) / 2, ch = (h + 1) / 2;
    failed = cudaMemcpy2DAsync(y, ys, s.plane(b, 0), s.strideY, w, h, cudaMemcpyDeviceToHost, stream_) ||
             cudaMemcpy2DAsync(cb, cs, s.plane(b, 1), s.strideC, cw, ch, cudaMemcpyDeviceToHost, stream_) ||
             cudaMemcpy2DAsync(cr, cs, s.plane(b, 2), s.strideC, cw, ch, cudaMemcpyDeviceToHost, stream_);
    if (!failed && rgbaDev && rgbaHost) {
      launchRGBA(s.plane(b, 0), s.plane(b, 1), s.plane(b, 2), s.strideY, s.strideC, w, h, rgbaDev, stream_);
      launches_++;
      failed = cudaGetLastError() != cudaSuccess ||
               cudaMemcpyAsync(rgbaHost, rgbaDev, (size_t)w * h * 4, cudaMemcpyDeviceToHost, stream_) != cudaSuccess;
    }
  }
  if (failed) {
    for (Job& j : R.jobs)
      if (j.status == kOK) j.status = kErrDevice;
    R.nDesc = 0;
    collectRound(R, results);
    return -1;
  }
  return collectRound(R, results);
}

int Engine::enableSideLane(int lanes) {
  for (auto& s : streams_)
    if (s) return kErrArg;  // pool and slot counts depend on it
  if (lanes < 1 || lanes > kSideLanes) return kErrArg;
  sideLanes_ = lanes;
  for (int l = 0; l < lanes; l++) {
    if (!streamES_[l] && cudaStreamCreateWithFlags(&streamES_[l], cudaStreamNonBlocking) != cudaSuccess)
      return kErrDevice;
    if (!streamRS_[l] && cudaStreamCreateWithFlags(&streamRS_[l], cudaStreamNonBlocking) != cudaSuccess)
      return kErrDevice;
    if (!sideDone_[l] && cudaEventCreateWithFlags(&sideDone_[l], cudaEventDisableTiming) != cudaSuccess)
      return kErrDevice;
  }
  side_ = true;
  return kOK;
}

int Engine::freeSideLane() const {
  if (!side_) return -1;
  for (int l = 0; l < sideLanes_; l++)
    if (!sideInflight_[l]) return l;
  return -1;
}

int Engine::freeSideLanes() const {
  int n = 0;
  for (int l = 0; l < sideLanes_; l++) n += sideInflight_[l] ? 0 : 1;
  return n;
}

bool Engine::anySideBusy() const {
  for (bool b : sideInflight_)
    if (b) return true;
  return false;
}

int Engine::launchSide(int lane, const std::vector<int>& ids, const std::vector<int>* frames) {
  if (!side_ || lane < 0 || lane >= sideLanes_ || sideInflight_[lane]) return kErrArg;
  Round& R = rounds_[kSide + lane];
  R.parity = kSide + lane;
  // Frames per stream: the lane's slot set holds min(kSideFrames, lookahead).
  const int cap = std::min(kSideFrames, lookahead_);
  std::vector<int> n(ids.size(), 1);
  if (frames)
    for (size_t i = 0; i < n.size() && i < frames->size(); i++) n[i] = std::max(1, std::min(cap, (*frames)[i]));
  if (planRound(ids, &n, R) || launchRecon(R)) {
    for (Job& j : R.jobs)
      if (j.status == kOK) j.status = kErrDevice;
    R.nDesc = 0;
  }
  if (cudaEventRecord(sideDone_[lane], streamRS_[lane]) != cudaSuccess) return kErrDevice;
  sideInflight_[lane] = true;
  return kOK;
}

bool Engine::sideReady(int lane) {
  return sideBusy(lane) && cudaEventQuery(sideDone_[lane]) != cudaErrorNotReady;
}

int Engine::collectSide(int lane, std::vector<RoundResult>* results) {
  if (!sideBusy(lane)) return 0;
  const int n = collectRound(rounds_[kSide + lane], results);
  sideInflight_[lane] = false;
  return n;
}

int Engine::drain(std::vector<RoundResult>* results) {
  int n = 0;
  while (!pipe_.empty()) {
    Round& R = rounds_[pipe_.front()];
    if (!R.reconLaunched && launchRecon(R)) {
      for (Job& j : R.jobs)
        if (j.status == kOK) j.status = kErrDevice;
      R.nDesc = 0;
    }
    R.reconLaunched = true;
    n += collectRound(R, results);
    pipe_.erase(pipe_.begin());
  }
  return n;
}

// Copies a decoded key frame (pool buffer img; golden when an override made
// it differ) and the table history after it into the stream's key cache.
// Both images are complete (their round was collected) and no device work
// of a later round writes them before these copies return.
void Engine::cacheKey(Stream& s, int64_t index, int img, int golden, const TableHistory& hist) {
  if (s.keyCache.count(index)) return;
  Stream::CachedKey ck;
  const bool og = golden != img;
  if (cudaMalloc(&ck.img, s.bufBytes) == cudaSuccess &&
      cudaMemcpy(ck.img, s.pool[(size_t)img], s.bufBytes, cudaMemcpyDeviceToDevice) == cudaSuccess &&
      (!og || (cudaMalloc(&ck.golden, s.bufBytes) == cudaSuccess &&
               cudaMemcpy(ck.golden, s.pool[(size_t)golden], s.bufBytes, cudaMemcpyDeviceToDevice) ==
                   cudaSuccess))) {
    ck.hist = hist;
    const size_t b = s.bufBytes * (og ? 2 : 1);
    s.cacheBytes += b;
    deviceBytes_ += b;
    s.keyCache[index] = ck;
  } else {
    if (ck.img) cudaFree(ck.img);
    if (ck.golden) cudaFree(ck.golden);
    cudaGetLastError();  // the cache is an optimisation: a failed copy leaves the key uncached
  }
}

int Engine::launchAside(int lane, const std::vector<int>& ids, const std::vector<int64_t>& keys) {
  if (!side_ || lane < 0 || lane >= sideLanes_ || sideInflight_[lane] || ids.size() != keys.size()) return kErrArg;
  struct Saved {
    int64_t next;
    TableHistory hist;
    bool hasProv;
    int pRef, pGolden;
    int64_t lastRound;
  };
  std::vector<int> use;
  std::vector<Saved> saved;
  for (size_t i = 0; i < ids.size(); i++) {
    const int id = ids[i];
    if (id < 0 || id >= (int)streams_.size() || !streams_[(size_t)id]) continue;
    Stream& s = *streams_[(size_t)id];
    if (!s.resident || !s.ready || !s.cacheKeys || s.inSide || s.inAside || s.hasProv || keys[i] < 0 ||
        keys[i] >= (int64_t)s.packets() || s.keyCache.count(keys[i]))
      continue;
    saved.push_back({s.next, s.hist, s.hasProv, s.pRef, s.pGolden, s.lastRound});
    use.push_back(id);
    s.next = keys[i];
  }
  if (use.empty()) return kErrArg;
  Round& R = rounds_[kSide + lane];
  R.parity = kSide + lane;
  const std::vector<int> one(use.size(), 1);
  const int planned = planRound(use, &one, R);
  R.aside = true;
  // Planning moved the streams as if they had decoded the key frame; their
  // own decode resumes exactly where it was.
  for (size_t i = 0; i < use.size(); i++) {
    Stream& s = *streams_[(size_t)use[i]];
    s.next = saved[i].next;
    s.hist = saved[i].hist;
    s.hasProv = saved[i].hasProv;
    s.pRef = saved[i].pRef;
    s.pGolden = saved[i].pGolden;
    s.lastRound = saved[i].lastRound;
    s.inSide = false;
    s.inAside = true;
  }
  if (planned || launchRecon(R)) {
    for (Job& j : R.jobs)
      if (j.status == kOK) j.status = kErrDevice;
    R.nDesc = 0;
  }
  if (cudaEventRecord(sideDone_[lane], streamRS_[lane]) != cudaSuccess) return kErrDevice;
  sideInflight_[lane] = true;
  return kOK;
}

bool Engine::inAside(int id) const {
  return id >= 0 && id < (int)streams_.size() && streams_[(size_t)id] && streams_[(size_t)id]->inAside;
}

int Engine::setKeyCache(int id, bool on) {
  if (id < 0 || id >= (int)streams_.size() || !streams_[(size_t)id] || !streams_[(size_t)id]->resident)
    return kErrArg;
  streams_[(size_t)id]->cacheKeys = on;
  return kOK;
}

bool Engine::keyCached(int id, int64_t index) const {
  if (id < 0 || id >= (int)streams_.size() || !streams_[(size_t)id]) return false;
  return streams_[(size_t)id]->keyCache.count(index) != 0;
}

size_t Engine::keyCacheBytes(int id) const {
  if (id < 0 || id >= (int)streams_.size() || !streams_[(size_t)id]) return 0;
  return streams_[(size_t)id]->cacheBytes;
}

int Engine::launchMain(const std::vector<int>& ids, const std::vector<int>* maxFrames) {
  if (pipeDepth_ || mainInflight_) return kErrArg;
  if (!mainDone_ && cudaEventCreateWithFlags(&mainDone_, cudaEventDisableTiming) != cudaSuccess) return kErrDevice;
  Round& R = rounds_[0];
  R.parity = 0;
  const bool failed = planRound(ids, maxFrames, R) != 0 || launchRecon(R) != 0;
  if (failed) {
    for (Job& j : R.jobs)
      if (j.status == kOK) j.status = kErrDevice;
    R.nDesc = 0;
  }
  if (cudaEventRecord(mainDone_, reconStream(0)) != cudaSuccess) return kErrDevice;
  mainInflight_ = true;
  return failed ? -1 : kOK;
}

bool Engine::mainReady() { return mainInflight_ && cudaEventQuery(mainDone_) != cudaErrorNotReady; }

int Engine::collectMain(std::vector<RoundResult>* results) {
  if (!mainInflight_) return 0;
  const int n = collectRound(rounds_[0], results);
  mainInflight_ = false;
  return n;
}

int Engine::installKey(int id, int64_t index, std::vector<RoundResult>* results) {
  if (id < 0 || id >= (int)streams_.size() || !streams_[(size_t)id] || pipeDepth_) return kErrArg;
  Stream& s = *streams_[(size_t)id];
  const auto it = s.keyCache.find(index);
  if (it == s.keyCache.end() || s.inSide || !s.ready) return kErrArg;
  // A main round in flight may hold this stream: its frames there are
  // discarded at collection (the stream's epoch moves on) and its buffers
  // stay untouched until then.
  bool inMain = false;
  for (int q = 0; q < kSide; q++) inMain = inMain || !s.roundBufs[q].empty();
  if (s.hasProv && !inMain) return kErrArg;
  std::vector<char> busy(s.pool.size(), 0);
  if (s.ref >= 0) busy[(size_t)s.ref] = 1;
  if (s.golden >= 0) busy[(size_t)s.golden] = 1;
  for (int b : s.outputs) busy[(size_t)b] = 1;
  for (const auto& rb : s.roundBufs)  // an aside round's buffer
    for (int b2 : rb) busy[(size_t)b2] = 1;
  const int b = freeBuffer(s.pool.size(), busy);
  if (b < 0) return kErrDevice;
  busy[(size_t)b] = 1;
  int g = b;
  if (it->second.golden) {
    g = freeBuffer(s.pool.size(), busy);
    if (g < 0) return kErrDevice;
  }
  if (cudaMemcpy(s.pool[(size_t)b], it->second.img, s.bufBytes, cudaMemcpyDeviceToDevice) != cudaSuccess ||
      (g != b && cudaMemcpy(s.pool[(size_t)g], it->second.golden, s.bufBytes, cudaMemcpyDeviceToDevice) !=
                     cudaSuccess))
    return kErrDevice;
  // The state Decode leaves after this key frame: references, table history,
  // the next packet, and the frame as the newest output.
  if (inMain) {
    s.epoch++;
    s.hasProv = false;
  }
  s.ref = b;
  s.golden = g;
  s.hist = it->second.hist;
  s.next = index + 1;
  s.outputs.push_back(b);
  const int cap = s.ring + (s.resident ? lookahead_ : 1);
  while ((int)s.outputs.size() > cap) s.outputs.erase(s.outputs.begin());
  RoundResult r;
  r.stream = s.id;
  r.frameIndex = index;
  r.keyframe = true;
  r.status = kOK;
  r.view.y = s.plane(b, 0);
  r.view.cb = s.plane(b, 1);
  r.view.cr = s.plane(b, 2);
  r.view.yStride = s.strideY;
  r.view.cStride = s.strideC;
  r.view.width = s.geo.W;
  r.view.height = s.geo.H;
  r.view.buffer = b;
  if (results) results->push_back(r);
  return kOK;
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

namespace ebiv {
Engine* batchEngine(ebivgpu_batch* b) { return b ? &b->e : nullptr; }
}  // namespace ebiv

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

int ebivgpu_batch_result_download_async(ebivgpu_batch* b, int i, uint8_t* packed, size_t cap) {
  if (!b || i < 0 || i >= (int)b->last.size()) return kErrArg;
  const RoundResult& r = b->last[(size_t)i];
  if (r.status != kOK) return r.status;
  return b->e.downloadFrameAsync(r.view, packed, cap);
}

int ebivgpu_batch_sync(ebivgpu_batch* b) {
  if (!b) return kErrArg;
  return b->e.syncCopies();
}

int ebivgpu_batch_reload_stream(ebivgpu_batch* b, int stream_id, const uint8_t* const* pkts, const size_t* lens,
                                int n) {
  if (!b || (!pkts && n) || (!lens && n)) return kErrArg;
  return b->e.reloadStream(stream_id, pkts, lens, n);
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

int ebivgpu_batch_set_lookahead(ebivgpu_batch* b, int frames) { return b ? b->e.setLookahead(frames) : kErrArg; }

int ebivgpu_batch_set_pipeline(ebivgpu_batch* b, int depth) { return b ? b->e.setPipelined(depth) : kErrArg; }

int ebivgpu_batch_set_tuning(ebivgpu_batch* b, int entropy_groups, int intra_warps) {
  return b ? b->e.setTuning(entropy_groups, intra_warps) : kErrArg;
}

int ebivgpu_batch_drain(ebivgpu_batch* b, int* frames) {
  if (!b) return kErrArg;
  b->last.clear();
  const int n = b->e.drain(&b->last);
  if (frames) *frames = n < 0 ? 0 : n;
  return n < 0 ? kErrDevice : kOK;
}

int64_t ebivgpu_batch_launches(ebivgpu_batch* b) { return b ? b->e.launches() : 0; }
uint64_t ebivgpu_batch_device_bytes(ebivgpu_batch* b) { return b ? (uint64_t)b->e.deviceBytes() : 0; }
uint64_t ebivgpu_stream_footprint(int w, int h, int ring, int lookahead) {
  return (uint64_t)Engine::footprint(w, h, ring, lookahead < 1 ? 1 : lookahead);
}

}  // extern "C"
