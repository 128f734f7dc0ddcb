// Serving loop over the decode engine: continuous batching of per-frame
// requests from many streams, HBM-budget admission, seeks and looping, with
// per-request latency.
//
// Each stream issues frame requests as a Poisson process at its frame rate.
// A round decodes, for every admitted stream with queued requests, the run
// of requested frames at its head (one frame for a stream that keeps up, a
// few for one that fell behind — the engine's per-stream lookahead), all in
// one set of kernel launches; requests that arrive while a round runs join
// the next one.  A seek request moves the stream to a key frame
// (ebiv/reader.go:222-238 semantics: decoding restarts there exactly); a
// looping stream seeks back to its first frame at the end.  Streams are
// admitted while the sum of their HBM footprints (frame pool + scratch)
// fits the budget; a finished stream releases its memory and the next
// waiting stream is admitted.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <deque>
#include <memory>
#include <new>
#include <random>
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
  int maxFramesPerRound = 4;
  int ring = 3;
  int record = 0;
  int keyLane = 1;  // key frames decode on the engine's side lane
  double startSpread = 0;  // streams admitted at start begin at a uniform offset in [0, startSpread) s
};

struct ServeStatsC {
  int64_t requests = 0, frames = 0, errors = 0, seeks = 0, loops = 0, rounds = 0;
  int64_t admittedTotal = 0, admittedPeak = 0, waitingAtEnd = 0;
  double elapsed = 0, p50 = 0, p99 = 0, pmax = 0, mean = 0, framesPerSec = 0, kernelMs = 0, entropyMs = 0, reconMs = 0;
  int64_t keyFrames = 0;
  uint64_t peakBytes = 0;
};

class Server {
 public:
  explicit Server(const ServeOptionsC& o) : opt_(o), rng_(o.seed) {}
  int init() {
    int st = eng_.setLookahead(std::max(1, opt_.maxFramesPerRound));
    if (st) return st;
    st = eng_.init();
    if (st) return st;
    if (opt_.keyLane && (st = eng_.enableSideLane())) return st;
    eng_.enableTiming(true);
    return kOK;
  }

  int addStream(const uint8_t* const* pkts, const size_t* lens, int n, double fps, bool loop) {
    if (n <= 0 || fps <= 0) return kErrArg;
    Spec sp;
    sp.pkts.resize((size_t)n);
    for (int i = 0; i < n; i++) sp.pkts[(size_t)i].assign(pkts[i], pkts[i] + lens[i]);
    FrameHeader fh;
    if (parseFrameHeader(sp.pkts[0].data(), sp.pkts[0].size(), &fh) || fh.type != kFrameKey) return kErrCorrupt;
    sp.w = fh.width;
    sp.h = fh.height;
    for (int i = 0; i < n; i++) {
      FrameHeader f;
      if (parseFrameHeader(sp.pkts[(size_t)i].data(), sp.pkts[(size_t)i].size(), &f) == kOK && f.type == kFrameKey)
        sp.keys.push_back(i);
    }
    sp.fps = fps;
    sp.loop = loop;
    sp.footprint = Engine::footprint(sp.w, sp.h, opt_.ring, std::max(1, opt_.maxFramesPerRound), false,
                                     opt_.keyLane != 0) +
                   [&] {
                     size_t b = 0;
                     for (auto& p : sp.pkts) b += (p.size() + 15) / 16 * 16;
                     return b;
                   }();
    specs_.push_back(std::move(sp));
    return kOK;
  }

  int run(ServeStatsC* out) {
    std::deque<int> waiting;
    for (size_t i = 0; i < specs_.size(); i++) waiting.push_back((int)i);
    std::vector<int> admitted;  // spec indices
    std::vector<int> specOf;    // engine stream id -> spec index
    uint64_t used = 0;
    ServeStatsC st;
    const double t0 = nowSec();
    auto admit = [&] {
      while (!waiting.empty() && used + specs_[(size_t)waiting.front()].footprint <= opt_.hbmBudget) {
        const int si = waiting.front();
        waiting.pop_front();
        Spec& sp = specs_[(size_t)si];
        std::vector<const uint8_t*> ptrs;
        std::vector<size_t> lens;
        for (auto& p : sp.pkts) {
          ptrs.push_back(p.data());
          lens.push_back(p.size());
        }
        if (eng_.addResidentStream(ptrs.data(), lens.data(), (int)ptrs.size(), opt_.ring, &sp.engineId)) break;
        if ((int)specOf.size() <= sp.engineId) specOf.resize((size_t)sp.engineId + 1, -1);
        specOf[(size_t)sp.engineId] = si;
        sp.nextArrival = nowSec() - t0;
        if (opt_.startSpread > 0 && st.rounds == 0)
          sp.nextArrival += std::uniform_real_distribution<double>(0, opt_.startSpread)(rng_);
        sp.pos = 0;
        used += sp.footprint;
        admitted.push_back(si);
        st.admittedTotal++;
        st.admittedPeak = std::max<int64_t>(st.admittedPeak, (int64_t)admitted.size());
        st.peakBytes = std::max<uint64_t>(st.peakBytes, used);
      }
    };
    admit();
    std::vector<double> lat;
    // Each result answers the head request of its stream.
    auto deliver = [&](const std::vector<RoundResult>& rs, double done) {
      for (const RoundResult& r : rs) {
        const int si = r.stream >= 0 && r.stream < (int)specOf.size() ? specOf[(size_t)r.stream] : -1;
        if (si < 0) continue;
        Spec& sp = specs_[(size_t)si];
        if (sp.queue.empty()) continue;
        const Request req = sp.queue.front();
        sp.queue.pop_front();
        sp.pos = r.frameIndex + 1;
        if (r.status != kOK) {
          st.errors++;
          continue;
        }
        st.frames++;
        if (r.keyframe) st.keyFrames++;
        lat.push_back(done - req.arrival);
        if (opt_.record) {
          const int cw = (r.view.width + 1) / 2, ch = (r.view.height + 1) / 2;
          std::vector<uint8_t> buf((size_t)r.view.width * r.view.height + 2 * (size_t)cw * ch);
          eng_.downloadFrame(r.view, buf.data(), buf.size());
          hashes_.push_back({si, r.frameIndex, fnv1a(buf.data(), buf.size())});
        }
      }
    };
    // Applies the head request's seek and the clip end (loop, or drop the
    // requests of a finished clip); false when there is nothing to decode.
    auto prepareHead = [&](Spec& sp) -> bool {
      if (sp.queue.empty()) return false;
      Request& head = sp.queue.front();
      if (head.seekTo >= 0) {
        eng_.seekStream(sp.engineId, head.seekTo);
        sp.pos = head.seekTo;
        head.seekTo = -1;
        st.seeks++;
      }
      if (sp.pos >= (int64_t)sp.pkts.size()) {
        if (!sp.loop) {
          sp.queue.clear();  // the clip ended: the remaining requests cannot be served
          return false;
        }
        eng_.seekStream(sp.engineId, 0);
        sp.pos = 0;
        st.loops++;
      }
      return true;
    };
    auto isKey = [](const Spec& sp, int64_t i) { return std::binary_search(sp.keys.begin(), sp.keys.end(), i); };
    std::vector<RoundResult> res;
    std::vector<int> sideSpecs;
    for (;;) {
      const double now = nowSec() - t0;
      // Arrivals up to now.
      for (int si : admitted) {
        Spec& sp = specs_[(size_t)si];
        while (sp.nextArrival <= now && sp.nextArrival <= opt_.duration && sp.issued < opt_.framesPerStream &&
               !sp.done) {
          Request r;
          r.arrival = sp.nextArrival;
          if (std::uniform_real_distribution<double>(0, 1)(rng_) < opt_.seekProb && !sp.keys.empty()) {
            r.seekTo = sp.keys[std::uniform_int_distribution<size_t>(0, sp.keys.size() - 1)(rng_)];
          }
          sp.queue.push_back(r);
          sp.issued++;
          st.requests++;
          sp.nextArrival += std::exponential_distribution<double>(sp.fps)(rng_);
        }
      }
      // Key lane: collect a finished side round, then send every stream whose
      // next frame is a key frame (start, seek, loop, GOP boundary) to it, so
      // no main round waits for a key frame's long entropy chains.
      if (opt_.keyLane && eng_.sideBusy() && eng_.sideReady()) {
        res.clear();
        eng_.collectSide(&res);
        deliver(res, nowSec() - t0);
        for (int si : sideSpecs) specs_[(size_t)si].inSide = false;
        sideSpecs.clear();
        st.rounds++;
      }
      if (opt_.keyLane && !eng_.sideBusy()) {
        std::vector<int> kids, kcap;
        for (int si : admitted) {
          Spec& sp = specs_[(size_t)si];
          if (sp.inSide || !prepareHead(sp) || !isKey(sp, sp.pos)) continue;
          kids.push_back(sp.engineId);
          kcap.push_back(1);
          sideSpecs.push_back(si);
          sp.inSide = true;
        }
        if (!kids.empty() && eng_.launchSide(kids, &kcap)) return kErrDevice;
      }
      // Main round: each stream's run of plain requests at its queue head,
      // ending before a seek and (with the key lane) before a key frame.
      std::vector<int> ids, counts;
      for (int si : admitted) {
        Spec& sp = specs_[(size_t)si];
        if (sp.inSide || !prepareHead(sp)) continue;
        if (opt_.keyLane && isKey(sp, sp.pos)) continue;  // waits for the key lane
        int n = 0;
        for (const Request& r : sp.queue) {
          if (n > 0 && r.seekTo >= 0) break;
          if (++n >= opt_.maxFramesPerRound) break;
        }
        n = (int)std::min<int64_t>(n, (int64_t)sp.pkts.size() - sp.pos);
        if (opt_.keyLane) {
          const auto nk = std::upper_bound(sp.keys.begin(), sp.keys.end(), sp.pos);
          if (nk != sp.keys.end()) n = (int)std::min<int64_t>(n, *nk - sp.pos);
        }
        ids.push_back(sp.engineId);
        counts.push_back(n);
      }
      if (ids.empty()) {
        // Finished streams release their memory; admit waiting ones.
        bool changed = false;
        for (size_t k = 0; k < admitted.size();) {
          Spec& sp = specs_[(size_t)admitted[k]];
          const bool ended = !sp.inSide && sp.queue.empty() &&
                             (sp.issued >= opt_.framesPerStream || sp.nextArrival > opt_.duration ||
                              (!sp.loop && sp.pos >= (int64_t)sp.pkts.size()));
          if (ended) {
            eng_.removeStream(sp.engineId);
            used -= sp.footprint;
            sp.done = true;
            admitted.erase(admitted.begin() + (long)k);
            changed = true;
          } else {
            k++;
          }
        }
        if (changed) admit();
        if (admitted.empty() && waiting.empty()) break;
        if (now > opt_.duration && admitted.empty()) break;
        double nextT = 1e30;
        for (int si : admitted) nextT = std::min(nextT, specs_[(size_t)si].nextArrival);
        if (nextT > opt_.duration + 1 && waiting.empty() && !eng_.sideBusy()) {
          bool pending = false;
          for (int si : admitted) pending |= !specs_[(size_t)si].queue.empty();
          if (!pending) break;
        }
        double wait = nextT - (nowSec() - t0);
        if (eng_.sideBusy()) wait = std::min(wait, 0.0002);  // poll the key lane
        if (wait > 0) std::this_thread::sleep_for(std::chrono::duration<double>(std::min(wait, 0.005)));
        continue;
      }
      res.clear();
      eng_.roundFor(ids, &res, &counts);
      st.rounds++;
      deliver(res, nowSec() - t0);
    }
    if (eng_.sideBusy()) {
      res.clear();
      eng_.collectSide(&res);
      deliver(res, nowSec() - t0);
    }
    st.elapsed = nowSec() - t0;
    st.waitingAtEnd = (int64_t)waiting.size();
    std::sort(lat.begin(), lat.end());
    latencies_ = lat;
    if (!lat.empty()) {
      st.p50 = lat[lat.size() / 2] * 1000;
      st.p99 = lat[(size_t)std::min<double>(lat.size() - 1, std::floor(0.99 * (lat.size() - 1)))] * 1000;
      st.pmax = lat.back() * 1000;
      double s = 0;
      for (double v : lat) s += v;
      st.mean = s / lat.size() * 1000;
    }
    st.framesPerSec = st.elapsed > 0 ? st.frames / st.elapsed : 0;
    st.kernelMs = eng_.kernelMillis();
    st.entropyMs = eng_.entropyMillis();
    st.reconMs = eng_.reconMillis();
    *out = st;
    return kOK;
  }

  const std::vector<double>& latencies() const { return latencies_; }
  struct Hash {
    int stream;
    int64_t frame;
    uint64_t hash;
  };
  const std::vector<Hash>& hashes() const { return hashes_; }

 private:
  struct Request {
    double arrival = 0;
    int64_t seekTo = -1;
  };
  struct Spec {
    std::vector<std::vector<uint8_t>> pkts;
    std::vector<int64_t> keys;
    int w = 0, h = 0;
    double fps = 30;
    bool loop = false;
    uint64_t footprint = 0;
    int engineId = -1;
    double nextArrival = 0;
    int64_t issued = 0;
    int64_t pos = 0;
    bool done = false;
    bool inSide = false;  // its key frame is on the side lane
    std::deque<Request> queue;
  };
  ServeOptionsC opt_;
  Engine eng_;
  std::mt19937_64 rng_;
  std::vector<Spec> specs_;
  std::vector<RoundResult> results_;
  std::vector<double> latencies_;
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

void ebivgpu_server_destroy(ebivgpu_server* h) { delete h; }

uint64_t ebivgpu_frame_hash(const uint8_t* packed, size_t n) { return fnv1a(packed, n); }

}  // extern "C"
