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
    sp.footprint = Engine::footprint(sp.w, sp.h, opt_.ring, std::max(1, opt_.maxFramesPerRound)) +
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
        sp.nextArrival = nowSec() - t0;
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
      // Build the round: each stream's run of plain requests at its head.
      std::vector<int> ids, counts, owners;
      for (int si : admitted) {
        Spec& sp = specs_[(size_t)si];
        if (sp.queue.empty()) continue;
        Request& head = sp.queue.front();
        if (head.seekTo >= 0) {
          eng_.seekStream(sp.engineId, head.seekTo);
          sp.pos = head.seekTo;
          head.seekTo = -1;
          st.seeks++;
        }
        if (sp.pos >= (int64_t)sp.pkts.size()) {
          if (sp.loop) {
            eng_.seekStream(sp.engineId, 0);
            sp.pos = 0;
            st.loops++;
          } else {
            // The clip ended: the remaining requests cannot be served.
            sp.queue.clear();
            continue;
          }
        }
        int n = 0;
        for (const Request& r : sp.queue) {
          if (n > 0 && r.seekTo >= 0) break;
          if (++n >= opt_.maxFramesPerRound) break;
        }
        n = std::min<int64_t>(n, (int64_t)sp.pkts.size() - sp.pos);
        ids.push_back(sp.engineId);
        counts.push_back(n);
        owners.push_back(si);
      }
      if (ids.empty()) {
        // Finished streams release their memory; admit waiting ones.
        bool changed = false;
        for (size_t k = 0; k < admitted.size();) {
          Spec& sp = specs_[(size_t)admitted[k]];
          const bool ended = sp.queue.empty() && (sp.issued >= opt_.framesPerStream || sp.nextArrival > opt_.duration ||
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
        if (nextT > opt_.duration + 1 && waiting.empty()) {
          bool pending = false;
          for (int si : admitted) pending |= !specs_[(size_t)si].queue.empty();
          if (!pending) break;
        }
        const double wait = nextT - (nowSec() - t0);
        if (wait > 0) std::this_thread::sleep_for(std::chrono::duration<double>(std::min(wait, 0.005)));
        continue;
      }
      results_.clear();
      eng_.roundFor(ids, &results_, &counts);
      const double done = nowSec() - t0;
      st.rounds++;
      for (const RoundResult& r : results_) {
        int si = -1;
        for (size_t k = 0; k < ids.size(); k++)
          if (ids[k] == r.stream) si = owners[k];
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
