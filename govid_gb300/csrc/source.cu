// Decode-ahead frame source: govid's asyncSource (source.go:84-266), the
// frame source behind govid.NewAsyncPlayer (player.go:40-57), on the GPU.
//
// The reference keeps one goroutine decoding the next frame (demuxer
// NextPacket, then Codec.Decode) into a channel of `depth` frames, with a
// seek generation so frames decoded before a seek never reach the player,
// and parks the goroutine after an error or end of stream until a seek.
// Here one native worker thread does the same with the batch engine: the
// stream's packets are resident in HBM, frames are decoded `lookahead` at a
// time (their entropy stages in one launch, the reconstructions in order)
// in pipelined rounds, and each decoded frame is copied into a pinned host
// slot (with WithRGBA also converted on the device and copied), then queued.
//
// Differences from the reference, all invisible to govid's Player:
//   * frames are decoded in rounds, so up to depth + 2 * lookahead frames
//     are decoded ahead of the consumer (the reference: depth + 1);
//   * a frame's planes (and RGBA) stay valid until the consumer releases it
//     (the Player releases the retired frame at every change and the queued
//     next frame at a seek, player.go:142-144,178-180); the reference ties
//     only the RGBA buffers to release and lets the codec's ring bound the
//     planes (ebiv/codec.go:15-22);
//   * next() and poll() on a parked source whose last entry (end of stream
//     or the error) was already taken return that status again instead of
//     blocking or reporting "not ready";
//   * a consumer holding so many frames that none can be decoded (more than
//     depth + lookahead + 4) gets kErrArg from next() and poll() instead of
//     waiting forever;
//   * a seek the demuxer refuses (a frame rate whose frameIndexAt walk does
//     not settle) changes nothing; the reference has already started a new
//     generation then, dropping the queued frames;
//   * the packets are read at open, so a container whose index holds an
//     entry NextPacket cannot read (an offset that wraps validateEntry's sum
//     to a negative position, ebiv/reader.go:115-123,203-205) is refused
//     there with kErrIO; the reference plays up to that frame.
#include <cuda_runtime.h>

#include <condition_variable>
#include <cstdint>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <new>
#include <thread>
#include <vector>

#include "../../include/ebivgpu.h"
#include "container.h"
#include "ebiv_format.h"
#include "engine.h"

namespace ebiv {
namespace {

// A pinned host buffer for one decoded frame: packed planes, then RGBA.
struct HostSlot {
  uint8_t* planes = nullptr;
  size_t planesCap = 0;
  uint8_t* rgba = nullptr;
  size_t rgbaCap = 0;
  uint32_t use = 0;  // bumped at every hand-out: the handle's check word
  bool free = true;
  int width = 0, height = 0;
  int64_t frameIndex = -1;
  bool keyframe = false;
};

// One queued result: a frame in a slot, or a terminal status (slot -1).
struct Entry {
  int slot = -1;
  int status = kOK;
  uint64_t gen = 0;
};

int grow(uint8_t** p, size_t* cap, size_t need) {
  if (*cap >= need) return kOK;
  if (*p) cudaFreeHost(*p);
  *p = nullptr;
  *cap = 0;
  if (cudaHostAlloc(reinterpret_cast<void**>(p), need, cudaHostAllocDefault) != cudaSuccess) {
    *p = nullptr;
    return kErrDevice;
  }
  *cap = need;
  return kOK;
}

}  // namespace

class Source {
 public:
  ~Source() {
    close();
    std::vector<RoundResult> tmp;
    if (engineReady_) engine_.drain(&tmp);
    if (dRGBA_) cudaFree(dRGBA_);
    for (HostSlot& s : slots_) {
      if (s.planes) cudaFreeHost(s.planes);
      if (s.rgba) cudaFreeHost(s.rgba);
    }
  }

  int open(const uint8_t* data, size_t n, int depth, int flags) {
    if (depth < 1) depth = 1;  // newAsyncSource, source.go:113-115
    depth_ = depth;
    rgba_ = (flags & EBIVGPU_SOURCE_RGBA) != 0;
    if (int st = reader_.open(data, n)) return st;
    if (reader_.frameCount() == 0) return kErrEOF;
    // Every container error is reported before the GPU is touched.
    std::vector<const uint8_t*> pk((size_t)reader_.frameCount());
    std::vector<size_t> len(pk.size());
    for (int i = 0; i < reader_.frameCount(); i++)
      if (int st = reader_.packet(i, &pk[(size_t)i], &len[(size_t)i])) return st;
    if (cudaGetDevice(&device_) != cudaSuccess) return kErrDevice;
    lookahead_ = depth < kMaxLookahead ? depth : kMaxLookahead;
    if (int st = engine_.init()) return st;
    engineReady_ = true;
    if (engine_.setLookahead(lookahead_) || engine_.setPipelined(kPipeline)) return kErrArg;
    if (int st = engine_.addResidentStream(pk.data(), len.data(), (int)pk.size(), 3, &sid_)) return st;
    slots_.resize((size_t)(depth_ + 2 * lookahead_ + kConsumerFrames));
    for (size_t i = 0; i < slots_.size(); i++) freeList_.push_back((int)i);
    worker_ = std::thread([this] { run(); });
    return kOK;
  }

  // next (source.go:196-210) when block, else poll (source.go:212-224).
  int take(bool block, ebivgpu_source_frame* f, int* ready) {
    std::unique_lock<std::mutex> lk(mu_);
    for (;;) {
      if (closing_) {
        if (ready) *ready = 1;
        return kErrEOF;  // source.go:206-208
      }
      while (!queue_.empty()) {
        const Entry e = queue_.front();
        queue_.pop_front();
        cvWork_.notify_all();
        if (e.gen != gen_) {  // decoded for an earlier seek generation
          if (e.slot >= 0) freeSlot(e.slot);
          continue;
        }
        if (e.slot < 0) {
          terminal_ = e.status;
          terminalTaken_ = true;
          if (ready) *ready = 1;
          return e.status;
        }
        HostSlot& s = slots_[(size_t)e.slot];
        s.use++;
        fill(e.slot, s, f);
        if (ready) *ready = 1;
        return kOK;
      }
      if (parked_ && terminalTaken_) {
        if (ready) *ready = 1;
        return terminal_;
      }
      if (!parked_ && !busy_ && engineGen_ == gen_ && (int)freeList_.size() < lookahead_) {
        // Nothing queued and no frame can be decoded until the consumer
        // releases one: waiting would never end.
        if (ready) *ready = 1;
        return kErrArg;
      }
      if (!block) {
        if (ready) *ready = 0;
        return kOK;
      }
      cvReady_.wait(lk);
    }
  }

  // seek (source.go:226-248): a new generation, the demuxer repositioned at
  // the last key frame at or before t, the codec flushed, queued frames
  // dropped, a parked worker woken.
  int seek(int64_t t, int64_t* landed) {
    std::lock_guard<std::mutex> lk(mu_);
    int64_t at = 0;
    if (int st = reader_.seek(t, &at)) return st;  // a refused seek changes nothing
    gen_++;
    target_ = reader_.position();
    parked_ = false;
    terminalTaken_ = false;
    terminal_ = kOK;
    for (const Entry& e : queue_)
      if (e.slot >= 0) freeSlot(e.slot);
    queue_.clear();
    cvWork_.notify_all();
    if (landed) *landed = at;
    return kOK;
  }

  // release (source.go:131-150): the frame's buffers go back to the pool.
  void release(int64_t handle) {
    const int slot = (int)(handle & 0xFFFFFFFF);
    const uint32_t use = (uint32_t)((uint64_t)handle >> 32);
    std::lock_guard<std::mutex> lk(mu_);
    if (slot < 0 || slot >= (int)slots_.size()) return;
    HostSlot& s = slots_[(size_t)slot];
    if (s.free || s.use != use) return;  // stale or repeated release
    freeSlot(slot);
    cvWork_.notify_all();
  }

  // close (source.go:250-254): returns once the worker has stopped.
  void close() {
    {
      std::lock_guard<std::mutex> lk(mu_);
      closing_ = true;
    }
    cvWork_.notify_all();
    cvReady_.notify_all();
    if (worker_.joinable()) worker_.join();
  }

  int64_t decoded() {
    std::lock_guard<std::mutex> lk(mu_);
    return decoded_;
  }
  int64_t duration() const { return reader_.duration(); }
  int lookahead() const { return lookahead_; }

 private:
  static constexpr int kMaxLookahead = 32;
  static constexpr int kPipeline = 2;
  // Frames the consumer may hold besides the queue before decoding waits for
  // a release (govid's Player holds the current, next and retired frames).
  static constexpr int kConsumerFrames = 4;

  void freeSlot(int i) {
    slots_[(size_t)i].free = true;
    freeList_.push_back(i);
  }

  void fill(int i, const HostSlot& s, ebivgpu_source_frame* f) const {
    const int cw = (s.width + 1) / 2, ch = (s.height + 1) / 2;
    f->handle = (int64_t)(((uint64_t)s.use << 32) | (uint32_t)i);
    f->y = s.planes;
    f->cb = s.planes + (size_t)s.width * s.height;
    f->cr = f->cb + (size_t)cw * ch;
    f->y_stride = s.width;
    f->c_stride = cw;
    f->width = s.width;
    f->height = s.height;
    f->timestamp_ns = reader_.header().frameTime(s.frameIndex);
    f->frame_index = s.frameIndex;
    f->keyframe = s.keyframe ? 1 : 0;
    f->rgba = rgba_ ? s.rgba : nullptr;
  }

  // Room for one more round: the queue below depth and a slot for each frame
  // the round can return.
  bool canDecode() const { return (int)queue_.size() < depth_ && (int)freeList_.size() >= lookahead_; }

  void park(int status, uint64_t gen) {
    Entry e;
    e.status = status;
    e.gen = gen;
    queue_.push_back(e);
    parked_ = true;
    cvReady_.notify_all();
  }

  // run (source.go:152-187).
  void run() {
    cudaSetDevice(device_);
    std::vector<RoundResult> res;
    std::vector<int> claimed;
    std::unique_lock<std::mutex> lk(mu_);
    for (;;) {
      cvWork_.wait(lk, [&] { return closing_ || (!parked_ && (engineGen_ != gen_ || canDecode())); });
      if (closing_) break;
      if (engineGen_ != gen_) {  // a seek: drop the rounds in flight, rewind the stream
        const uint64_t g = gen_;
        const int64_t target = target_;
        busy_ = true;
        lk.unlock();
        res.clear();
        engine_.drain(&res);
        pending_ = 0;
        const int st = engine_.seekStream(sid_, target);
        lk.lock();
        busy_ = false;
        engineGen_ = g;
        if (st && g == gen_) park(st, g);
        cvReady_.notify_all();
        continue;
      }
      const uint64_t g = gen_;
      claimed.clear();
      for (int k = 0; k < lookahead_; k++) {
        claimed.push_back(freeList_.back());
        freeList_.pop_back();
        slots_[(size_t)claimed.back()].free = false;
      }
      busy_ = true;
      lk.unlock();

      res.clear();
      int status = kOK;
      bool ended = false;
      const int64_t before = engine_.remaining(sid_);
      if (before > 0 || pending_ > 0) {
        // Rounds of a pipelined engine come back `kPipeline` calls after
        // they were planned; at the end of the stream empty rounds push the
        // last ones out.  (Frames are re-planned only after a failure, which
        // parks the source, so planned minus returned is what is in flight.)
        if (engine_.round(&res) < 0) status = kErrDevice;
        pending_ += (before - engine_.remaining(sid_)) - (int64_t)res.size();
      } else {
        ended = true;  // readNextFrame: NextPacket returned io.EOF
      }
      // Copy every frame up to the first failure; one wait for all of them.
      size_t used = 0;
      int failAt = -1;
      for (size_t i = 0; i < res.size() && failAt < 0 && status == kOK; i++) {
        const RoundResult& r = res[i];
        if (r.status != kOK) {
          failAt = (int)i;
          break;
        }
        HostSlot& s = slots_[(size_t)claimed[used]];
        const EngineFrameView& v = r.view;
        const size_t need = (size_t)v.width * v.height + 2 * (size_t)((v.width + 1) / 2) * ((v.height + 1) / 2);
        int st = grow(&s.planes, &s.planesCap, need);
        if (!st) st = engine_.downloadFrameAsync(v, s.planes, s.planesCap);
        if (!st && rgba_) {
          const size_t rb = (size_t)v.width * v.height * 4;
          st = grow(&s.rgba, &s.rgbaCap, rb);
          if (!st && rgbaDevCap_ < rb) {
            if (dRGBA_) cudaFree(dRGBA_);
            dRGBA_ = nullptr;
            rgbaDevCap_ = 0;
            if (cudaMalloc(reinterpret_cast<void**>(&dRGBA_), rb) != cudaSuccess) st = kErrDevice;
            else rgbaDevCap_ = rb;
          }
          if (!st) st = engine_.convertFrameAsync(v, dRGBA_, s.rgba);
        }
        if (st) {
          status = st;
          break;
        }
        s.width = v.width;
        s.height = v.height;
        s.frameIndex = r.frameIndex;
        s.keyframe = r.keyframe;
        used++;
      }
      if (engine_.syncCopies() != kOK && status == kOK) status = kErrDevice;

      lk.lock();
      busy_ = false;
      decoded_ += (int64_t)res.size();
      const bool current = g == gen_ && !closing_;
      for (size_t k = 0; k < claimed.size(); k++) {
        if (current && k < used && status == kOK) {
          Entry e;
          e.slot = claimed[k];
          e.gen = g;
          queue_.push_back(e);
        } else {
          freeSlot(claimed[k]);
        }
      }
      if (current) {
        if (status != kOK) park(status, g);
        else if (failAt >= 0) park(res[(size_t)failAt].status, g);
        else if (ended) park(kErrEOF, g);
      }
      cvReady_.notify_all();
    }
  }

  Reader reader_;
  Engine engine_;
  bool engineReady_ = false;
  int sid_ = -1;
  int device_ = 0;
  int64_t pending_ = 0;  // worker only: frames planned and not yet returned
  int depth_ = 1, lookahead_ = 1;
  bool rgba_ = false;
  uint8_t* dRGBA_ = nullptr;
  size_t rgbaDevCap_ = 0;

  std::mutex mu_;  // guards everything below
  std::condition_variable cvWork_, cvReady_;
  std::vector<HostSlot> slots_;  // sized at open, never reallocated
  std::vector<int> freeList_;
  std::deque<Entry> queue_;
  uint64_t gen_ = 0, engineGen_ = 0;
  int64_t target_ = 0;
  bool parked_ = false, closing_ = false;
  bool busy_ = false;  // the worker is decoding (it will queue or free its slots)
  bool terminalTaken_ = false;
  int terminal_ = kOK;
  int64_t decoded_ = 0;
  std::thread worker_;
};

}  // namespace ebiv

struct ebivgpu_source {
  ebiv::Source src;
};

extern "C" {

int ebivgpu_source_create(const uint8_t* container, size_t n, int depth, int flags, ebivgpu_source** out) {
  if (!out || (!container && n)) return EBIV_ERR_ARG;
  *out = nullptr;
  if (flags & ~EBIVGPU_SOURCE_RGBA) return EBIV_ERR_ARG;
  ebivgpu_source* s = new (std::nothrow) ebivgpu_source();
  if (!s) return EBIV_ERR_DEVICE;
  if (int st = s->src.open(container, n, depth, flags)) {
    delete s;
    return st;
  }
  *out = s;
  return EBIV_OK;
}

int ebivgpu_source_next(ebivgpu_source* s, ebivgpu_source_frame* f) {
  if (!s || !f) return EBIV_ERR_ARG;
  return s->src.take(true, f, nullptr);
}

int ebivgpu_source_poll(ebivgpu_source* s, ebivgpu_source_frame* f, int* ready) {
  if (!s || !f || !ready) return EBIV_ERR_ARG;
  return s->src.take(false, f, ready);
}

int ebivgpu_source_seek(ebivgpu_source* s, int64_t t_ns, int64_t* landed_ns) {
  if (!s) return EBIV_ERR_ARG;
  return s->src.seek(t_ns, landed_ns);
}

void ebivgpu_source_release(ebivgpu_source* s, int64_t handle) {
  if (s) s->src.release(handle);
}

int ebivgpu_source_close(ebivgpu_source* s) {
  if (!s) return EBIV_ERR_ARG;
  s->src.close();
  return EBIV_OK;
}

int64_t ebivgpu_source_decoded(ebivgpu_source* s) { return s ? s->src.decoded() : 0; }
int64_t ebivgpu_source_duration(ebivgpu_source* s) { return s ? s->src.duration() : 0; }
int ebivgpu_source_lookahead(ebivgpu_source* s) { return s ? s->src.lookahead() : 0; }

void ebivgpu_source_destroy(ebivgpu_source* s) { delete s; }

}  // extern "C"
