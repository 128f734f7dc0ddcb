// Serving loop over the decode engine: continuous batching of per-frame
// requests from many streams, HBM-budget admission, seeks and looping, with
// per-request latency.
//
// Each stream issues frame requests as a Poisson process at its frame rate.
// A decode thread keeps every admitted stream a few frames ahead of its
// requests (govid's AsyncPlayer keeps `depth` frames ready the same way,
// source.go:84-187), batching all streams' next frames into shared rounds;
// requests are served in order from the decoded frames as they arrive.  A
// seek request moves the stream to a key frame (ebiv/reader.go:222-238
// semantics: decoding restarts there exactly, from the stream's key-frame
// cache when it holds that frame); a looping stream continues from its first
// frame at the end.  Streams are admitted while the sum of their HBM
// footprints (frame pool, scratch, packets, key caches) fits the budget; a
// finished stream releases its memory when a waiting stream needs it.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cmath>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <new>
#include <random>
#include <set>
#include <thread>
#include <vector>

#include "../../include/ebivgpu.h"
#include "container.h"
#include "engine.h"

namespace ebiv {

namespace {
double nowSec() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}
uint64_t fnv1a(const uint8_t* p, size_t n, uint64_t h = 1469598103934665603ull) {
  for (size_t i = 0; i < n; i++) {
    h ^= p[i];
    h *= 1099511628211ull;
  }
  return h;
}
}  // namespace

struct ServeOptionsC {
  double duration = 10;       // seconds during which requests arrive
  int64_t framesPerStream = 600;
  double seekProb = 0.05;
  uint64_t seed = 1;
  uint64_t hbmBudget = 120ull << 30;
  int maxFramesPerRound = 4;  // frames of one stream per round (the engine's lookahead)
  int ring = 3;
  int record = 0;
  int keyLane = 1;  // side lanes for long key frames (0: none; at most Engine::kSideLanes)
  double startSpread = 0;  // streams admitted at start begin at a uniform offset in [0, startSpread) s
  int decodeAhead = 0;     // frames decoded ahead of each stream's requests (0: twice the lookahead)
  int lanes = 0;           // decode lanes (engines with their own thread and side lane); 0: 1
  int longKeyMBs = 0;      // key frames whose largest tile has more macroblocks go to a side lane (0: 1500)
  int keyCache = 0;        // 1 long-key streams cache key frames as decoded, 2 also decode them at admission, 3 every stream as 2
};

struct ServeStatsC {
  int64_t requests = 0, frames = 0, errors = 0, seeks = 0, loops = 0, rounds = 0;
  int64_t admittedTotal = 0, admittedPeak = 0, waitingAtEnd = 0;
  double elapsed = 0, p50 = 0, p99 = 0, pmax = 0, mean = 0, framesPerSec = 0, kernelMs = 0, entropyMs = 0, reconMs = 0;
  int64_t keyFrames = 0;
  uint64_t peakBytes = 0;
  int64_t readyAtArrival = 0, unserved = 0;
  double seekP50 = 0, seekP99 = 0;
  int64_t mainRounds = 0, sideRounds = 0, mainFrames = 0;
  int64_t keyInstalls = 0, warmedStreams = 0, asideRounds = 0, followRounds = 0, seekShortcuts = 0;
  double warmupSec = 0;  // admission to first request of streams that decoded their key frames first
  double prepareSec = 0;  // key_cache 2: key frames of the streams admitted at start, before the first request
  double mainRoundSec = 0, idleSec = 0;  // decode thread: inside main rounds, waiting for work
  double planSec = 0, launchSec = 0, collectSec = 0;  // inside main rounds: host planning, launches, wait
};

// Threads: one decode thread per decode lane (an engine of its own; one by
// default) and one request thread.
//
// * A decode thread keeps every stream of its lane up to `decodeAhead` frames
//   ahead of its requests, in main rounds of up to `maxFramesPerRound` frames
//   per stream (their entropy stages in one launch). It launches a main round
//   and collects it when the GPU is done, handling seeks and side rounds
//   meanwhile.
// * Key frames whose tiles carry long entropy chains go to the engine's side
//   lanes, so they never hold up a main round. So do the frames after a seek
//   target, which need to arrive within a frame interval.
// * With a key cache, a stream keeps its decoded key frames (image, golden,
//   table history) and installs one at a seek instead of decoding it; key
//   frames may be decoded into the caches ahead of time (at admission, or in
//   side rounds nobody waits on).
// * A decode thread also admits streams (HBM budget) and removes finished
//   ones when a waiting stream needs the memory.
// * The request thread generates each stream's Poisson requests, serves them
//   in order from the decoded frames, and applies seeks: a new epoch drops the
//   frames decoded for the old position, and decoding restarts at the key
//   frame. A stream whose key frames are all cached has its seek answered from
//   the cache at once.
//
// A request's latency runs from its arrival to the moment its frame is
// decoded and handed out: zero wait when the frame was ready before it was
// asked for.
class Server {
 public:
  explicit Server(const ServeOptionsC& o) : opt_(o), rng_(o.seed) {
    lookahead_ = std::max(1, opt_.maxFramesPerRound);
    ahead_ = opt_.decodeAhead > 0 ? opt_.decodeAhead : 2 * lookahead_;
    ahead_ = std::max(ahead_, lookahead_);
  }
  int init() {
    const int n = opt_.lanes > 0 ? std::min(opt_.lanes, 16) : 1;
    for (int i = 0; i < n; i++) {
      std::unique_ptr<Lane> L(new (std::nothrow) Lane());
      if (!L) return kErrDevice;
      int st = L->eng.setLookahead(lookahead_);
      if (st) return st;
      st = L->eng.init();
      if (st) return st;
      if (opt_.keyLane && (st = L->eng.enableSideLane(sideLanes()))) return st;
      L->eng.enableTiming(true);
      L->index = i;
      lanes_.push_back(std::move(L));
    }
    return kOK;
  }

  int addStream(const uint8_t* const* pkts, const size_t* lens, int n, double fps, bool loop) {
    if (n <= 0 || fps <= 0) return kErrArg;
    std::unique_ptr<Spec> sp(new (std::nothrow) Spec());
    if (!sp) return kErrArg;
    sp->pkts.resize((size_t)n);
    for (int i = 0; i < n; i++) sp->pkts[(size_t)i].assign(pkts[i], pkts[i] + lens[i]);
    FrameHeader fh;
    if (parseFrameHeader(sp->pkts[0].data(), sp->pkts[0].size(), &fh) || fh.type != kFrameKey) return kErrCorrupt;
    sp->w = fh.width;
    sp->h = fh.height;
    for (int i = 0; i < n; i++) {
      FrameHeader f;
      if (parseFrameHeader(sp->pkts[(size_t)i].data(), sp->pkts[(size_t)i].size(), &f) == kOK && f.type == kFrameKey)
        sp->keys.push_back(i);
    }
    sp->longKey = opt_.keyLane && maxTileMBs(sp->pkts[0], fh) > (opt_.longKeyMBs > 0 ? opt_.longKeyMBs : kLongKeyMBs);
    sp->fps = fps;
    sp->loop = loop;
    sp->footprint = Engine::footprint(sp->w, sp->h, ringOf(), lookahead_, 0, sideLanes());
    if (cachesKeys(*sp)) {  // one image per key frame (two when an override changed golden)
      const Geometry g = Geometry::of(sp->w, sp->h);
      auto s64 = [](int w) { return (size_t)((w + 63) & ~63); };  // the engine's 64-byte row stride
      const size_t img = s64(g.padW()) * g.padH() + 2 * s64(g.padCW()) * g.padCH();
      sp->footprint += 2 * img * sp->keys.size();
    }
    for (auto& p : sp->pkts) sp->footprint += (p.size() + 15) / 16 * 16;
    specs_.push_back(std::move(sp));
    return kOK;
  }

  int run(ServeStatsC* out) {
    for (size_t i = 0; i < specs_.size(); i++) waiting_.push_back((int)i);
    if (cudaGetDevice(&device_) != cudaSuccess) return kErrDevice;
    t0_ = nowSec();
    {
      std::lock_guard<std::mutex> lk(mu_);
      admit(nullptr, true);
    }
    std::vector<std::thread> dec;
    for (auto& L : lanes_) {
      Lane* lp = L.get();
      dec.emplace_back([this, lp] { decodeLoop(*lp); });
    }
    if (opt_.keyCache > 1) {
      // Preparation (key_cache 2): the streams admitted at start decode their
      // key frames into their caches before any request; the request clock
      // starts afterwards, so their requests begin as if admitted now.
      // Every stream also fills its decode-ahead before the clock starts, as a
      // player buffers before it starts playback.
      std::unique_lock<std::mutex> lk(mu_);
      for (;;) {
        bool busy = false;
        for (auto& sp : specs_) {
          if (!sp->admitted) continue;
          const int64_t left = (int64_t)sp->pkts.size();
          busy = busy || sp->warming || (int64_t)sp->ready.size() < std::min<int64_t>(ahead_, left);
        }
        if (!busy || stop_) break;
        cvRequest_.wait_for(lk, std::chrono::milliseconds(1));
      }
      const double shift = nowSec() - t0_;
      st_.prepareSec = shift;
      t0_ += shift;
      for (auto& sp : specs_) {
        if (!sp->admitted) continue;
        sp->admittedAt = 0;
        sp->startAt = opt_.startSpread > 0 ? std::uniform_real_distribution<double>(0, opt_.startSpread)(rng_) : 0;
        for (Ready& rd : sp->ready) rd.at -= shift;  // decoded before the clock started
      }
      st_.warmupSec = 0;
    }
    requestLoop();
    {
      std::lock_guard<std::mutex> lk(mu_);
      stop_ = true;
    }
    cvDecode_.notify_all();
    for (auto& t : dec) t.join();
    ServeStatsC st = st_;
    st.elapsed = endTime_;
    st.waitingAtEnd = (int64_t)waiting_.size();
    auto pctl = [](std::vector<double>& v, double q) {
      if (v.empty()) return 0.0;
      std::sort(v.begin(), v.end());
      return v[(size_t)std::min<double>(v.size() - 1, std::floor(q * (v.size() - 1)))] * 1000;
    };
    std::vector<double> lat = lat_;
    latencies_ = lat;
    if (!lat.empty()) {
      st.p50 = pctl(lat, 0.5);
      st.p99 = pctl(lat, 0.99);
      st.pmax = lat.back() * 1000;
      double sum = 0;
      for (double v : lat) sum += v;
      st.mean = sum / lat.size() * 1000;
    }
    st.seekP50 = pctl(seekLat_, 0.5);
    st.seekP99 = pctl(seekLat_, 0.99);
    st.framesPerSec = st.elapsed > 0 ? st.frames / st.elapsed : 0;
    for (auto& L : lanes_) {
      st.kernelMs += L->eng.kernelMillis();
      st.entropyMs += L->eng.entropyMillis();
      st.reconMs += L->eng.reconMillis();
    }
    *out = st;
    return decodeStatus_;
  }

  const std::vector<double>& latencies() const { return latencies_; }
  struct Hash {
    int stream;
    int64_t frame;
    uint64_t hash;
  };
  const std::vector<Hash>& hashes() const { return hashes_; }

 private:
  // A key frame whose largest tile has more macroblocks than this takes
  // longer to entropy-decode (about 4.6 us per macroblock on one warp) than
  // a round of the longest inter chains in a mixed set of streams, so it
  // goes to the side lane.
  static constexpr int kLongKeyMBs = 1500;

  struct Request {
    double arrival = 0;
    int64_t seekTo = -1;
  };
  struct Ready {
    int64_t frame = -1;
    int status = kOK;
    bool keyframe = false;
    uint64_t hash = 0;
    double at = 0;  // when it was decoded
  };
  struct Spec {
    std::vector<std::vector<uint8_t>> pkts;
    std::vector<int64_t> keys;
    int w = 0, h = 0;
    double fps = 30;
    bool loop = false, longKey = false;
    uint64_t footprint = 0;
    // shared (mu_)
    int lane = -1, engineId = -1;
    bool admitted = false, done = false, finished = false;
    double startAt = 0;
    uint64_t epoch = 0;       // bumped by a seek
    int64_t seekTarget = 0;   // where the newest epoch starts
    std::deque<Ready> ready;  // decoded frames of the current epoch, in order
    int inflight = 0;         // frames in a round of the current epoch
    // request thread
    bool started = false;
    double nextArrival = 0;
    int64_t issued = 0, consumePos = 0;
    std::deque<Request> queue;
    bool warming = false;     // decoding its key frames into the cache before its requests start
    bool noInstall = false;   // an install failed: this stream decodes its key frames
    int warmRounds = 0;       // side rounds spent warming its key cache
    bool keysCached = false;  // every key frame is in its key cache (seeks are answered from it at once)
    bool inMain = false;      // frames of it are in the main round in flight
    double admittedAt = 0;
    // decode thread
    uint64_t decEpoch = 0;
    bool inSide = false;
  };

  // A decode lane: an engine (with its own CUDA streams and side lane), the
  // streams admitted to it and the thread that drives it.  Lanes run side
  // by side on the GPU, so a long key frame holds up only its own lane's
  // side round and its rounds only its own streams.
  struct Lane {
    Engine eng;
    int index = 0;
    std::vector<int> admitted;  // spec indices
    std::vector<int> specOf;    // engine stream id -> spec index
    std::vector<std::pair<int, uint64_t>> sidePlanned[Engine::kSideLanes];
    std::vector<std::pair<int, uint64_t>> mainPlanned;  // (spec, epoch) of the main round in flight
    double mainLaunchedAt = 0;
  };

  int ringOf() const { return std::max(opt_.ring, ahead_ + 2); }
  // Streams that keep a key cache: those with long key frames (key_cache 1
  // and 2), every stream (key_cache 3).
  bool cachesKeys(const Spec& sp) const { return opt_.keyCache >= 3 || (sp.longKey && opt_.keyCache > 0); }
  int sideLanes() const { return opt_.keyLane > 0 ? std::min(opt_.keyLane, Engine::kSideLanes) : 0; }

  // The largest tile of a key frame's coded payload: frame header, then the
  // override length when present, qp, tile columns, tile rows
  // (ebiv/frame.go:224-236), split as tileGrid does.
  static int maxTileMBs(const std::vector<uint8_t>& pkt, const FrameHeader& fh) {
    const Geometry g = Geometry::of(fh.width, fh.height);
    size_t p = fh.bodyOffset;
    auto uv = [&](uint64_t* v) {
      *v = 0;
      for (int sh = 0; p < pkt.size() && sh < 64; sh += 7) {
        const uint8_t c = pkt[p++];
        *v |= (uint64_t)(c & 0x7F) << sh;
        if (c < 0x80) return true;
      }
      return false;
    };
    uint64_t skip = 0, cols = 1, rows = 1;
    if (fh.coding != kCodingIntra) return g.mbCols * g.mbRows;
    if (fh.goldenOverride && !uv(&skip)) return g.mbCols * g.mbRows;
    p++;  // qp
    if (!uv(&cols) || !uv(&rows)) return g.mbCols * g.mbRows;
    const TileGrid grid(g.mbCols, g.mbRows, (int)std::min<uint64_t>(cols, 1 << 16),
                        (int)std::min<uint64_t>(rows, 1 << 16));
    int m = 0;
    for (int t = 0; t < grid.count(); t++) {
      int x0, x1, y0, y1;
      grid.bounds(t, &x0, &x1, &y0, &y1);
      m = std::max(m, (x1 - x0) * (y1 - y0));
    }
    return m;
  }

  bool isKey(const Spec& sp, int64_t i) const { return std::binary_search(sp.keys.begin(), sp.keys.end(), i); }
  double now() const { return nowSec() - t0_; }

  // Admits waiting streams while their footprints fit (mu_ held): into
  // `only` (a lane whose stream finished), or round-robin over the lanes at
  // start.
  void admit(Lane* only, bool initial) {
    while (!waiting_.empty() && used_ + specs_[(size_t)waiting_.front()]->footprint <= opt_.hbmBudget) {
      const int si = waiting_.front();
      Spec& sp = *specs_[(size_t)si];
      Lane& L = only ? *only : *lanes_[(size_t)(nextLane_++ % lanes_.size())];
      std::vector<const uint8_t*> ptrs;
      std::vector<size_t> lens;
      for (auto& p : sp.pkts) {
        ptrs.push_back(p.data());
        lens.push_back(p.size());
      }
      if (L.eng.addResidentStream(ptrs.data(), lens.data(), (int)ptrs.size(), ringOf(), &sp.engineId)) break;
      waiting_.pop_front();
      sp.lane = L.index;
      if ((int)L.specOf.size() <= sp.engineId) L.specOf.resize((size_t)sp.engineId + 1, -1);
      L.specOf[(size_t)sp.engineId] = si;
      if (cachesKeys(sp)) {
        L.eng.setKeyCache(sp.engineId, true);
        sp.warming = opt_.keyCache > 1;
      }
      sp.admittedAt = now();
      sp.startAt = now();
      if (initial && opt_.startSpread > 0)
        sp.startAt += std::uniform_real_distribution<double>(0, opt_.startSpread)(rng_);
      sp.admitted = true;
      used_ += sp.footprint;
      L.admitted.push_back(si);
      admittedCount_++;
      st_.admittedTotal++;
      st_.admittedPeak = std::max<int64_t>(st_.admittedPeak, admittedCount_);
      st_.peakBytes = std::max<uint64_t>(st_.peakBytes, used_);
    }
  }

  // Publishes a round's results (mu_ held): frames of a stream's current
  // epoch join its ready list; the rest are dropped.
  void publish(const Lane& L, const std::vector<RoundResult>& rs, const std::vector<uint64_t>& hashes,
               const std::vector<std::pair<int, uint64_t>>& planned) {
    const double t = now();
    for (size_t i = 0; i < rs.size(); i++) {
      const RoundResult& r = rs[i];
      const int si = r.stream >= 0 && r.stream < (int)L.specOf.size() ? L.specOf[(size_t)r.stream] : -1;
      if (si < 0) continue;
      Spec& sp = *specs_[(size_t)si];
      uint64_t ep = ~0ull;
      for (const auto& pl : planned)
        if (pl.first == si) ep = pl.second;
      if (ep != sp.epoch || sp.warming) continue;
      Ready rd;
      rd.frame = r.frameIndex;
      rd.status = r.status;
      rd.keyframe = r.keyframe;
      rd.hash = i < hashes.size() ? hashes[i] : 0;
      rd.at = t;
      sp.ready.push_back(rd);
    }
    for (const auto& pl : planned) {
      Spec& sp = *specs_[(size_t)pl.first];
      if (pl.second == sp.epoch) sp.inflight = 0;
    }
  }

  void hashResults(Lane& L, const std::vector<RoundResult>& rs, std::vector<uint64_t>* out) {
    out->assign(rs.size(), 0);
    if (!opt_.record) return;
    std::vector<uint8_t> buf;
    for (size_t i = 0; i < rs.size(); i++) {
      const RoundResult& r = rs[i];
      if (r.status != kOK) continue;
      const int cw = (r.view.width + 1) / 2, ch = (r.view.height + 1) / 2;
      buf.resize((size_t)r.view.width * r.view.height + 2 * (size_t)cw * ch);
      if (L.eng.downloadFrame(r.view, buf.data(), buf.size()) == kOK) (*out)[i] = fnv1a(buf.data(), buf.size());
    }
  }

  // Collects the main round when its work is done (decode thread).
  bool collectMainIfReady(Lane& L, std::vector<RoundResult>& res, std::vector<uint64_t>& hashes) {
    if (!L.eng.mainBusy() || !L.eng.mainReady()) return false;
    res.clear();
    const double c0 = nowSec();
    L.eng.collectMain(&res);
    const double c1 = nowSec();
    hashResults(L, res, &hashes);
    std::lock_guard<std::mutex> lk(mu_);
    st_.rounds++;
    st_.mainRounds++;
    st_.mainFrames += (int64_t)res.size();
    st_.mainRoundSec += c1 - L.mainLaunchedAt;
    st_.collectSec += c1 - c0;
    publish(L, res, hashes, L.mainPlanned);
    for (const auto& pl : L.mainPlanned) specs_[(size_t)pl.first]->inMain = false;
    L.mainPlanned.clear();
    cvRequest_.notify_all();
    return true;
  }

  void decodeLoop(Lane& L) {
    cudaSetDevice(device_);
    std::vector<RoundResult> res;
    std::vector<uint64_t> hashes;
    for (;;) {
      collectMainIfReady(L, res, hashes);
      std::vector<int> ids, counts, kids, reposition;
      std::vector<int64_t> repoTo;
      std::vector<std::pair<int, uint64_t>> planned;
      std::vector<std::pair<int, int64_t>> installs;  // (spec, key frame) served from the key cache
      std::vector<char> installSeek;                   // the install answers a seek
      std::set<int> followIds;                         // engine ids of follow-up side frames
      std::vector<int> asideIds;
      std::vector<int64_t> asideKeys;
      int sideLane = -1;
      {
        std::unique_lock<std::mutex> lk(mu_);
        if (stop_) break;
        // Finished streams leave; waiting ones come in.
        bool removed = false;
        // Finished streams free their memory only when a waiting stream needs
        // it (freeing synchronises the device, which would stall every lane).
        for (size_t k = 0; k < L.admitted.size() && !waiting_.empty();) {
          Spec& sp = *specs_[(size_t)L.admitted[k]];
          if (sp.finished && !sp.inSide && !sp.inMain && !L.eng.inAside(sp.engineId)) {
            L.eng.removeStream(sp.engineId);
            used_ -= sp.footprint;
            sp.done = true;
            L.admitted.erase(L.admitted.begin() + (long)k);
            admittedCount_--;
            removed = true;
          } else {
            k++;
          }
        }
        if (removed) admit(&L, false);
        sideLane = L.eng.freeSideLane();  // the long key frames found now go there
        const bool mainFree = !L.eng.mainBusy();
        for (int si : L.admitted) {
          Spec& sp = *specs_[(size_t)si];
          if (sp.inSide || sp.finished) continue;
          if (sp.warming && !sp.inMain) {
            // Admission: each key frame once through a side lane into the
            // cache, then back to the first frame and the requests start.
            int64_t want = -1;
            for (int64_t k : sp.keys)
              if (!L.eng.keyCached(sp.engineId, k)) {
                want = k;
                break;
              }
            const int64_t at = (int64_t)sp.pkts.size() - L.eng.remaining(sp.engineId);
            if (want >= 0 && sp.warmRounds > (int)sp.keys.size() + 2) {  // a key frame that will not cache
              want = -1;
              sp.noInstall = true;
            }
            if (want < 0) {
              sp.warming = false;
              sp.keysCached = !sp.noInstall;
              reposition.push_back(sp.engineId);
              repoTo.push_back(0);
              sp.startAt = now();
              st_.warmedStreams++;
              st_.warmupSec += sp.startAt - sp.admittedAt;
            } else if (at != want) {
              reposition.push_back(sp.engineId);
              repoTo.push_back(want);
            } else if (sideLane >= 0 && kids.size() < 64) {
              kids.push_back(sp.engineId);
              sp.inSide = true;
              sp.warmRounds++;
              L.sidePlanned[sideLane].push_back({si, sp.epoch});
            }
            continue;
          }
          int64_t pos = -1;  // where the stream decodes next (after a reposition made below)
          if (sp.decEpoch != sp.epoch) {  // a seek: restart at its key frame
            if (!sp.noInstall && L.eng.keyCached(sp.engineId, sp.seekTarget)) {
              // (even while the main round in flight holds the stream: its
              // frames there are discarded)
              sp.decEpoch = sp.epoch;
              installs.push_back({si, sp.seekTarget});
              installSeek.push_back(1);
              sp.inflight = 1;
              continue;
            }
            if (sp.inMain) continue;  // once the round in flight is collected
            sp.decEpoch = sp.epoch;
            reposition.push_back(sp.engineId);  // applied before this pass launches anything
            repoTo.push_back(sp.seekTarget);
            pos = sp.seekTarget;
          }
          if (sp.inMain || sp.warming) continue;  // its frames are in the main round in flight
          const int room = ahead_ - (int)sp.ready.size() - sp.inflight;
          if (room <= 0) continue;
          if (pos < 0) pos = (int64_t)sp.pkts.size() - L.eng.remaining(sp.engineId);
          if (pos >= (int64_t)sp.pkts.size()) {
            if (!sp.loop) continue;
            reposition.push_back(sp.engineId);  // looping: on from the first frame
            repoTo.push_back(0);
            st_.loops++;
            pos = 0;
          }
          if (sp.longKey && !sp.noInstall && isKey(sp, pos) && L.eng.keyCached(sp.engineId, pos)) {
            installs.push_back({si, pos});
            installSeek.push_back(0);
            sp.inflight = 1;
            continue;
          }
          if (sp.longKey && isKey(sp, pos)) {
            // (A stream whose key frame is being decoded into its cache waits
            // for that round instead.)
            if (sideLane >= 0 && kids.size() < 64 && !L.eng.inAside(sp.engineId)) {
              kids.push_back(sp.engineId);
              sp.inSide = true;
              sp.inflight = 1;
              L.sidePlanned[sideLane].push_back({si, sp.epoch});
            }
            continue;
          }
          if (!mainFree) continue;
          int n = std::min(room, lookahead_);
          n = (int)std::min<int64_t>(n, (int64_t)sp.pkts.size() - pos);
          if (sp.longKey) {  // stop before the next long key frame
            const auto nk = std::upper_bound(sp.keys.begin(), sp.keys.end(), pos);
            if (nk != sp.keys.end()) n = (int)std::min<int64_t>(n, *nk - pos);
          }
          ids.push_back(sp.engineId);
          counts.push_back(n);
          sp.inflight = n;
          sp.inMain = true;
          planned.push_back({si, sp.epoch});
        }
        // A side lane nobody waits on fills key caches in the background (one
        // lane stays free for key frames a stream waits for): for up to 16
        // streams, the first key frame not yet cached after where each stream
        // decodes now.
        // (Only when no main round runs: the background rounds would slow it.)
        if (opt_.keyCache > 0 && mainFree && kids.empty() && sideLane >= 0 && L.eng.freeSideLanes() >= 2) {
          for (int si : L.admitted) {
            if (asideIds.size() >= 16) break;
            Spec& sp = *specs_[(size_t)si];
            if (!cachesKeys(sp) || sp.warming || sp.inSide || sp.inMain || sp.finished || sp.noInstall ||
                L.eng.inAside(sp.engineId))
              continue;
            const int64_t at = (int64_t)sp.pkts.size() - L.eng.remaining(sp.engineId);
            int64_t want = -1;
            for (size_t q = 0; q < sp.keys.size() && want < 0; q++) {
              const int64_t k = sp.keys[(std::upper_bound(sp.keys.begin(), sp.keys.end(), at) - sp.keys.begin() + q) %
                                        sp.keys.size()];
              if (!L.eng.keyCached(sp.engineId, k)) want = k;
            }
            if (want < 0) continue;
            asideIds.push_back(sp.engineId);
            asideKeys.push_back(want);
          }
        }
        if (ids.empty() && kids.empty() && reposition.empty() && installs.empty() && asideIds.empty()) {
          const bool gpuBusy = L.eng.mainBusy() || L.eng.anySideBusy();
          const double w0 = nowSec();
          // GPU work in flight: poll it often; none: wait for requests.
          cvDecode_.wait_for(lk, std::chrono::microseconds(gpuBusy ? 50 : 500));
          if (!gpuBusy) st_.idleSec += nowSec() - w0;
          if (!gpuBusy) continue;
        }
      }
      for (size_t k = 0; k < reposition.size(); k++) L.eng.seekStream(reposition[k], repoTo[k]);
      if (!installs.empty()) {
        res.clear();
        for (const auto& in : installs) {
          const int id = specs_[(size_t)in.first]->engineId;
          if (L.eng.installKey(id, in.second, &res) != kOK) {  // not installable: decode key frames from now on
            L.eng.seekStream(id, in.second);
            std::lock_guard<std::mutex> lk(mu_);
            specs_[(size_t)in.first]->inflight = 0;
            specs_[(size_t)in.first]->noInstall = true;
          }
        }
        hashResults(L, res, &hashes);
        std::lock_guard<std::mutex> lk(mu_);
        st_.keyInstalls += (int64_t)res.size();
        std::vector<std::pair<int, uint64_t>> pl;
        for (const auto& in : installs) pl.push_back({in.first, specs_[(size_t)in.first]->decEpoch});
        publish(L, res, hashes, pl);
        // The frame after an installed seek target goes to a side round now
        // rather than to the next main round: the requests that follow a
        // seek arrive within a frame interval.
        for (size_t q = 0; q < installs.size(); q++) {
          Spec& sp = *specs_[(size_t)installs[q].first];
          if (!installSeek[q] || sideLane < 0 || !asideIds.empty() || kids.size() >= 64 || sp.inSide || sp.noInstall ||
              sp.epoch != sp.decEpoch || L.eng.inAside(sp.engineId) ||
              L.eng.remaining(sp.engineId) <= 0 ||
              (sp.longKey && (isKey(sp, installs[q].second + 1) || isKey(sp, installs[q].second + 2))))
            continue;
          kids.push_back(sp.engineId);
          sp.inSide = true;
          sp.inflight = (int)std::min<int64_t>(Engine::kSideFrames, L.eng.remaining(sp.engineId));
          L.sidePlanned[sideLane].push_back({installs[q].first, sp.epoch});
          st_.followRounds++;
          followIds.insert(sp.engineId);
        }
        cvRequest_.notify_all();
      }
      if (!asideIds.empty() && L.eng.launchAside(sideLane, asideIds, asideKeys) == kOK) {
        std::lock_guard<std::mutex> lk(mu_);
        st_.asideRounds++;
      }
      std::vector<int> kframes(kids.size(), 1);  // long key frames: one; frames after a seek: two
      for (size_t q = 0; q < kids.size(); q++)
        if (followIds.count(kids[q])) kframes[q] = Engine::kSideFrames;
      if (!kids.empty() && L.eng.launchSide(sideLane, kids, &kframes)) {
        std::lock_guard<std::mutex> lk(mu_);
        decodeStatus_ = kErrDevice;
        stop_ = true;
        cvRequest_.notify_all();
        break;
      }
      if (!ids.empty()) {
        const double r0 = nowSec();
        const int rc = L.eng.launchMain(ids, &counts);
        const double r1 = nowSec();
        std::lock_guard<std::mutex> lk(mu_);
        L.mainPlanned = planned;
        L.mainLaunchedAt = r0;
        st_.planSec += r1 - r0;
        if (rc != kOK && !L.eng.mainBusy()) {
          decodeStatus_ = kErrDevice;
          stop_ = true;
          cvRequest_.notify_all();
          break;
        }
      }
      for (int l = 0; l < Engine::kSideLanes; l++) {
        if (!L.eng.sideReady(l)) continue;
        res.clear();
        L.eng.collectSide(l, &res);
        hashResults(L, res, &hashes);
        std::lock_guard<std::mutex> lk(mu_);
        st_.rounds++;
        st_.sideRounds++;
        publish(L, res, hashes, L.sidePlanned[l]);
        for (const auto& pl : L.sidePlanned[l]) specs_[(size_t)pl.first]->inSide = false;
        L.sidePlanned[l].clear();
        cvRequest_.notify_all();
      }
    }
    if (L.eng.mainBusy()) {
      res.clear();
      L.eng.collectMain(&res);
    }
    for (int l = 0; l < Engine::kSideLanes; l++) {
      res.clear();
      L.eng.collectSide(l, &res);
    }
  }

  // Serves the head requests of a stream from its ready frames (mu_ held).
  void serve(Spec& sp, int si, double t) {
    while (!sp.queue.empty()) {
      Request& head = sp.queue.front();
      if (head.seekTo >= 0) {  // Seek: a new epoch at the key frame
        sp.epoch++;
        sp.seekTarget = head.seekTo;
        sp.ready.clear();
        sp.inflight = 0;
        sp.consumePos = head.seekTo;
        if (sp.keysCached && !opt_.record) {
          // The key frame's image is already in the stream's key cache: the
          // request is answered now (the decode thread installs the same
          // image as the stream's state, and its copy of the frame is
          // dropped). Record runs take the install path, which they hash.
          Ready rd;
          rd.frame = head.seekTo;
          rd.keyframe = true;
          rd.at = t;
          sp.ready.push_back(rd);
          st_.seekShortcuts++;
        }
        head.seekTo = -2;  // applied; the request wants the key frame
        st_.seeks++;
        cvDecode_.notify_all();
      }
      if (sp.consumePos >= (int64_t)sp.pkts.size()) {
        if (!sp.loop) {  // the clip ended: the remaining requests cannot be served
          st_.unserved += (int64_t)sp.queue.size();
          sp.queue.clear();
          return;
        }
        sp.consumePos = 0;
      }
      while (!sp.ready.empty() && sp.ready.front().frame != sp.consumePos) sp.ready.pop_front();
      if (sp.ready.empty()) return;
      const Ready rd = sp.ready.front();
      sp.ready.pop_front();
      const bool wasSeek = head.seekTo == -2;
      const double arrival = head.arrival;
      sp.queue.pop_front();
      sp.consumePos++;
      cvDecode_.notify_all();
      if (rd.status != kOK) {
        st_.errors++;
        continue;
      }
      st_.frames++;
      if (rd.keyframe) st_.keyFrames++;
      const double l = std::max(0.0, std::max(t, rd.at) - arrival);
      lat_.push_back(l);
      log_.push_back({arrival, l, si, rd.frame, wasSeek});
      if (wasSeek) seekLat_.push_back(l);
      if (rd.at <= arrival) st_.readyAtArrival++;
      if (opt_.record) hashes_.push_back({si, rd.frame, rd.hash});
    }
  }

  void requestLoop() {
    std::unique_lock<std::mutex> lk(mu_);
    for (;;) {
      if (stop_) break;
      const double t = now();
      double nextT = 1e30;
      bool live = !waiting_.empty() && (admittedCount_ > 0 || t <= opt_.duration);
      for (size_t si = 0; si < specs_.size(); si++) {
        Spec& sp = *specs_[si];
        if (!sp.admitted || sp.done || sp.finished) continue;
        live = true;
        if (sp.warming) continue;
        if (!sp.started) {
          sp.started = true;
          sp.nextArrival = sp.startAt;
        }
        while (sp.nextArrival <= t && sp.nextArrival <= opt_.duration && sp.issued < opt_.framesPerStream) {
          Request r;
          r.arrival = sp.nextArrival;
          if (sp.issued > 0 && std::uniform_real_distribution<double>(0, 1)(rng_) < opt_.seekProb && !sp.keys.empty())
            r.seekTo = sp.keys[std::uniform_int_distribution<size_t>(0, sp.keys.size() - 1)(rng_)];
          sp.queue.push_back(r);
          sp.issued++;
          st_.requests++;
          sp.nextArrival += std::exponential_distribution<double>(sp.fps)(rng_);
        }
        serve(sp, (int)si, t);
        const bool noMore = sp.issued >= opt_.framesPerStream || sp.nextArrival > opt_.duration;
        if (noMore && sp.queue.empty()) {
          sp.finished = true;  // the decode thread removes it and admits the next
          cvDecode_.notify_all();
          continue;
        }
        if (!noMore) nextT = std::min(nextT, sp.nextArrival);
      }
      if (!live) break;
      const double wait = std::min(nextT - now(), 0.002);
      if (wait > 0) cvRequest_.wait_for(lk, std::chrono::duration<double>(wait));
    }
    endTime_ = now();
  }

  ServeOptionsC opt_;
  int lookahead_ = 1, ahead_ = 2;
  std::vector<std::unique_ptr<Lane>> lanes_;
  std::mt19937_64 rng_;
  std::vector<std::unique_ptr<Spec>> specs_;
  std::mutex mu_;
  std::condition_variable cvDecode_, cvRequest_;
  std::deque<int> waiting_;
  int64_t admittedCount_ = 0;
  size_t nextLane_ = 0;
  uint64_t used_ = 0;
  bool stop_ = false;
  int decodeStatus_ = kOK;
  int device_ = 0;
  double t0_ = 0, endTime_ = 0;
  ServeStatsC st_;
  std::vector<double> lat_, seekLat_, latencies_;

 public:
  struct LogEntry {
    double arrival, latency;
    int stream;
    int64_t frame;
    bool seek;
  };
  const std::vector<LogEntry>& requestLog() const { return log_; }

 private:
  std::vector<LogEntry> log_;
  std::vector<Hash> hashes_;
};

}  // namespace ebiv

using namespace ebiv;

struct ebivgpu_server {
  std::unique_ptr<Server> s;
};

extern "C" {

int ebivgpu_server_create(const ebivgpu_serve_options* o, ebivgpu_server** out) {
  if (!o || !out) return kErrArg;
  *out = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n <= 0) return kErrDevice;
  ServeOptionsC c;
  c.duration = o->duration_s;
  c.framesPerStream = o->frames_per_stream;
  c.seekProb = o->seek_prob;
  c.seed = o->seed;
  c.hbmBudget = o->hbm_budget_bytes;
  c.maxFramesPerRound = o->max_frames_per_round > 0 ? o->max_frames_per_round : 1;
  c.ring = o->ring >= 2 ? o->ring : 3;
  c.record = o->record;
  c.keyLane = o->key_lane;
  c.startSpread = o->start_spread_s > 0 ? o->start_spread_s : 0;
  c.decodeAhead = o->decode_ahead > 0 ? o->decode_ahead : 0;
  c.lanes = o->decode_lanes > 0 ? o->decode_lanes : 0;
  c.longKeyMBs = o->long_key_mbs > 0 ? o->long_key_mbs : 0;
  c.keyCache = o->key_cache > 0 ? o->key_cache : 0;
  ebivgpu_server* h = new (std::nothrow) ebivgpu_server();
  if (!h) return kErrDevice;
  h->s.reset(new Server(c));
  const int st = h->s->init();
  if (st) {
    delete h;
    return st;
  }
  *out = h;
  return kOK;
}

int ebivgpu_server_add_stream(ebivgpu_server* h, const uint8_t* const* pkts, const size_t* lens, int n, double fps,
                              int loop) {
  if (!h || !pkts || !lens) return kErrArg;
  return h->s->addStream(pkts, lens, n, fps, loop != 0);
}

int ebivgpu_server_run(ebivgpu_server* h, ebivgpu_serve_stats* out) {
  if (!h || !out) return kErrArg;
  ServeStatsC st;
  const int r = h->s->run(&st);
  out->requests = st.requests;
  out->frames = st.frames;
  out->errors = st.errors;
  out->seeks = st.seeks;
  out->loops = st.loops;
  out->rounds = st.rounds;
  out->admitted_total = st.admittedTotal;
  out->admitted_peak = st.admittedPeak;
  out->waiting_at_end = st.waitingAtEnd;
  out->elapsed_s = st.elapsed;
  out->latency_p50_ms = st.p50;
  out->latency_p99_ms = st.p99;
  out->latency_max_ms = st.pmax;
  out->latency_mean_ms = st.mean;
  out->frames_per_s = st.framesPerSec;
  out->kernel_ms = st.kernelMs;
  out->entropy_ms = st.entropyMs;
  out->recon_ms = st.reconMs;
  out->key_frames = st.keyFrames;
  out->peak_bytes = st.peakBytes;
  out->ready_at_arrival = st.readyAtArrival;
  out->unserved = st.unserved;
  out->seek_latency_p50_ms = st.seekP50;
  out->seek_latency_p99_ms = st.seekP99;
  out->main_rounds = st.mainRounds;
  out->side_rounds = st.sideRounds;
  out->main_frames = st.mainFrames;
  out->main_round_s = st.mainRoundSec;
  out->idle_s = st.idleSec;
  out->plan_s = st.planSec;
  out->launch_s = st.launchSec;
  out->collect_s = st.collectSec;
  out->key_installs = st.keyInstalls;
  out->warmed_streams = st.warmedStreams;
  out->warmup_s = st.warmupSec;
  out->aside_rounds = st.asideRounds;
  out->prepare_s = st.prepareSec;
  out->follow_rounds = st.followRounds;
  out->seek_shortcuts = st.seekShortcuts;
  return r;
}

int64_t ebivgpu_server_frame_hashes(ebivgpu_server* h, int32_t* stream, int64_t* frame, uint64_t* hash, int64_t cap) {
  if (!h) return 0;
  const auto& v = h->s->hashes();
  const int64_t n = std::min<int64_t>(cap, (int64_t)v.size());
  for (int64_t i = 0; i < n; i++) {
    stream[i] = v[(size_t)i].stream;
    frame[i] = v[(size_t)i].frame;
    hash[i] = v[(size_t)i].hash;
  }
  return (int64_t)v.size();
}

int64_t ebivgpu_server_request_log(ebivgpu_server* h, double* arrival_s, double* latency_ms, int32_t* stream,
                                   int64_t* frame, int32_t* seek, int64_t cap) {
  if (!h) return 0;
  const auto& v = h->s->requestLog();
  const int64_t n = std::min<int64_t>(cap, (int64_t)v.size());
  for (int64_t i = 0; i < n; i++) {
    const auto& e = v[(size_t)i];
    if (arrival_s) arrival_s[i] = e.arrival;
    if (latency_ms) latency_ms[i] = e.latency * 1000;
    if (stream) stream[i] = e.stream;
    if (frame) frame[i] = e.frame;
    if (seek) seek[i] = e.seek ? 1 : 0;
  }
  return (int64_t)v.size();
}

void ebivgpu_server_destroy(ebivgpu_server* h) { delete h; }

uint64_t ebivgpu_frame_hash(const uint8_t* packed, size_t n) { return fnv1a(packed, n); }

uint64_t ebivgpu_server_stream_footprint(const ebivgpu_serve_options* o, int width, int height, uint64_t packet_bytes) {
  if (!o || width <= 0 || height <= 0) return 0;
  const int lookahead = std::max(1, (int)o->max_frames_per_round);
  const int ahead = std::max(o->decode_ahead > 0 ? (int)o->decode_ahead : 2 * lookahead, lookahead);
  const int ring = std::max(o->ring >= 2 ? (int)o->ring : 3, ahead + 2);
  const int side = o->key_lane > 0 ? std::min((int)o->key_lane, Engine::kSideLanes) : 0;
  return Engine::footprint(width, height, ring, lookahead, 0, side) + packet_bytes;  // without a key cache
}

}  // extern "C"
