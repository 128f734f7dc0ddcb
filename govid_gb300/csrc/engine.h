// Multi-stream GB300 EBIV decode engine.
//
// Each stream owns a pool of padded frame buffers in HBM.  A frame decodes
// straight into a free pool buffer, which then *is* the decoded output (the
// visible region at a 64-byte aligned stride), the next frame's last
// reference, and — for a key frame — the golden reference.  Reference and
// golden are therefore aliases, never copies.  A buffer returns to the free
// list once it is neither the last reference, the golden reference, nor one
// of the stream's `ring` most recent outputs (ebiv/codec.go:15-22).
//
// A round decodes the next packet of every active stream: the host plans each
// coded payload (ebiv/frame.go:242-274, ebiv/rans.go:396-471), uploads one
// block of descriptors, and launches the entropy, inter and intra kernels once
// for all streams' tiles and macroblocks.  Reference-side effects follow
// ebiv/codec.go:70-192 exactly, including on errors.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <memory>
#include <vector>

#include "ebiv_format.h"
#include "gpu_types.h"
#include "payload.h"

namespace ebiv {

struct EngineFrameView {
  const uint8_t* y = nullptr;  // device pointers into the pool buffer
  const uint8_t* cb = nullptr;
  const uint8_t* cr = nullptr;
  int yStride = 0, cStride = 0, width = 0, height = 0;
  int buffer = -1;
};

struct RoundResult {
  int stream = -1;
  int status = kOK;
  int64_t frameIndex = -1;  // packet index within the stream
  bool keyframe = false;
  EngineFrameView view;     // valid when status == kOK
};

class Engine {
 public:
  Engine();
  ~Engine();
  int init(cudaStream_t s = nullptr);
  cudaStream_t stream() const { return stream_; }

  // A stream whose packets are all resident in HBM (uploaded here).
  int addResidentStream(const uint8_t* const* pkts, const size_t* lens, int n, int ring, int* id);
  // A resident stream that decodes in place from a container in pinned,
  // device-mapped host memory: packet i is pktLen[i] bytes at offset off[i]
  // of the container (hostBase for planning, devBase for the kernels).  No
  // packet is copied; the container must outlive the stream.
  int addContainerStream(const uint8_t* hostBase, const uint8_t* devBase, const uint64_t* off, const uint32_t* pktLen,
                         int n, int ring, int* id);
  // A stream fed one packet per round through submit().
  int addStreamingStream(int ring, int* id);
  // Frames per resident stream decoded per round (entropy of all of them in
  // one launch, reconstruction in dependency order).  Set before the streams
  // see their first key frame.
  int setLookahead(int k);
  int lookahead() const { return lookahead_; }
  int submit(int id, const uint8_t* pkt, size_t n);
  // Rewinds a resident stream to packet `index` (the caller seeks to a key
  // frame); Flush semantics: only the output cursor resets.
  int seekStream(int id, int64_t index);
  int streams() const { return (int)streams_.size(); }
  int64_t remaining(int id) const;
  // Marks a stream inactive (it keeps its buffers until removed).
  int setActive(int id, bool active);
  int removeStream(int id);

  // Decodes one packet for every active stream with work; returns the number
  // of frames attempted.  Results (one per attempted frame) are appended.
  int round(std::vector<RoundResult>* results);
  // Same, for an explicit subset of streams; maxFrames (optional, parallel
  // to ids) caps each stream's frames this round below the lookahead.
  int roundFor(const std::vector<int>& ids, std::vector<RoundResult>* results,
               const std::vector<int>* maxFrames = nullptr);
  // The Codec contract's round (synchronous engine, one streaming stream):
  // decodes the stream's pending packet and copies the frame's visible planes
  // to host memory (y, cb, cr at strides ys, cs) behind the reconstruction on
  // the same CUDA stream, so the round ends with one wait.  The copy is made
  // whatever the frame's status; the caller hands the planes out only when
  // the result's status is 0.
  // With rgbaDev (W*H*4 bytes of device memory) and rgbaHost non-null, the
  // frame is also converted to RGBA on the device (convertYCbCr420ToRGBA,
  // frame.go:8-67) from its device planes and copied to rgbaHost, in the
  // same round and behind the same single wait.
  int decodeInto(int id, uint8_t* y, int ys, uint8_t* cb, uint8_t* cr, int cs, std::vector<RoundResult>* results,
                 uint8_t* rgbaDev = nullptr, uint8_t* rgbaHost = nullptr);
  // Launch shapes (the autotuner's knobs; any time): the most entropy
  // launches a pipelined round splits its steps into (1 to 4), and the warps
  // per CTA of the intra stage (4, 8, 16; 0 picks by the tile count).
  int setTuning(int entropyGroups, int intraWarps) {
    if (entropyGroups < 1 || entropyGroups > kEntropyGroups ||
        (intraWarps != 0 && intraWarps != 4 && intraWarps != 8 && intraWarps != 16))
      return kErrArg;
    entropyGroups_ = entropyGroups;
    intraWarps_ = intraWarps;
    return kOK;
  }
  // Pipelined rounds (set before adding streams; resident streams only):
  // each round() plans a round and starts its entropy stage on a second CUDA
  // stream, collects the round in flight (whose results it returns) and then
  // launches the new round's reconstruction, so one round's entropy overlaps
  // the previous round's reconstruction.  drain() collects the last round.
  // depth D keeps D rounds in flight: a round's entropy stage starts D - 1
  // round() calls before its reconstruction, and its results come back D
  // calls after it was planned.  depth 0 is the synchronous engine; at most
  // kMaxDepth.
  int setPipelined(int depth);
  bool pipelined() const { return pipeDepth_ > 0; }
  int pipeDepth() const { return pipeDepth_; }
  int drain(std::vector<RoundResult>* results);
  // Side lanes (enabled before adding streams): rounds of one or two frames
  // for each of a few streams (the serving loop sends key frames with long
  // entropy chains there, and the frames after a seek), each lane on its own
  // pair of CUDA streams next to the main rounds and the other lanes,
  // collected when done.  A stream in a
  // side round is left out of main rounds until collected; the caller sends
  // a stream to a side lane only between its main rounds.
  static constexpr int kSideLanes = 4;
  static constexpr int kSideFrames = 4;  // frames of one stream a side round decodes at most
  int enableSideLane(int lanes = 1);  // 1 to kSideLanes
  int sideLanes() const { return sideLanes_; }
  int freeSideLane() const;  // a lane with no round in flight, or -1
  int freeSideLanes() const;  // how many lanes have no round in flight
  int launchSide(int lane, const std::vector<int>& ids, const std::vector<int>* frames = nullptr);
  bool sideBusy(int lane) const { return lane >= 0 && lane < kSideLanes && sideInflight_[lane]; }
  bool anySideBusy() const;
  bool sideReady(int lane);  // the lane's round is complete
  int collectSide(int lane, std::vector<RoundResult>* results);

  // Key-frame cache of a resident stream (serving): with it on, every key
  // frame the stream decodes keeps a copy of its image (and of the golden
  // image when an override changed it) and of the table history after it.
  // installKey puts the stream in the state decoding that key frame leaves
  // (references, table history, next packet) without decoding it, and
  // returns the frame as a result; the stream must have no round in flight.
  // The synchronous engine's round in two halves (serving): launchMain plans
  // and launches it, mainReady() says when its work is done, collectMain
  // returns its results.  While it runs, installKey may take a stream of the
  // round (the round's frames of that stream are then discarded) and side
  // rounds run beside it.
  int launchMain(const std::vector<int>& ids, const std::vector<int>* maxFrames);
  bool mainBusy() const { return mainInflight_; }
  bool mainReady();
  int collectMain(std::vector<RoundResult>* results);
  int setKeyCache(int id, bool on);
  bool keyCached(int id, int64_t index) const;
  size_t keyCacheBytes(int id) const;
  int installKey(int id, int64_t index, std::vector<RoundResult>* results);
  // A side-lane round that decodes key frame keys[i] of stream ids[i] only
  // into that stream's key cache: the stream keeps decoding in main rounds
  // meanwhile, its state untouched (collectSide returns no result for it).
  int launchAside(int lane, const std::vector<int>& ids, const std::vector<int64_t>& keys);
  bool inAside(int id) const;

  int downloadFrame(const EngineFrameView& v, uint8_t* packed, size_t cap);
  // Queues the copy on the engine's copy stream, beside the reconstruction;
  // complete after syncCopies().  Later rounds' device work waits for it
  // before touching frame buffers.
  int downloadFrameAsync(const EngineFrameView& v, uint8_t* packed, size_t cap);
  // Also on the copy stream: the frame's RGBA (convertYCbCr420ToRGBA,
  // frame.go:8-67) into rgbaDev (W*H*4 bytes of device memory), then copied
  // to rgbaHost.  Conversions queued one after another may share rgbaDev.
  int convertFrameAsync(const EngineFrameView& v, uint8_t* rgbaDev, uint8_t* rgbaHost);
  int syncCopies();
  // New packets for a resident stream (its frame pool is kept); no round may
  // be in flight.
  int reloadStream(int id, const uint8_t* const* pkts, const size_t* lens, int n);
  int downloadStrided(const EngineFrameView& v, uint8_t* y, int ys, uint8_t* cb, uint8_t* cr, int cs);
  int copyReference(int id, int which, uint8_t* dst, size_t cap);
  int64_t launches() const { return launches_; }
  size_t deviceBytes() const { return deviceBytes_; }
  // Per-stream HBM footprint (pool + scratch) for a geometry.
  static size_t footprint(int w, int h, int ring, int lookahead, int depth = 0, int sideLanes = 0);
  static int poolSize(int ring, int lookahead, int depth, bool side = false);

  // Kernel-time accounting: CUDA events recorded around each round's
  // kernels on the engine's stream.
  void enableTiming(bool on) { timing_ = on; }
  double kernelMillis() const { return kernelMs_; }
  // Host time of synchronous rounds: planning (headers, tables, descriptors,
  // the staging upload and the entropy launch), the reconstruction launches,
  // and the wait for the round to finish.
  double planSeconds() const { return planSec_; }
  double launchSeconds() const { return launchSec_; }
  double collectSeconds() const { return collectSec_; }
  double entropyMillis() const { return entropyMs_; }
  double reconMillis() const { return reconMs_; }
  void resetTiming() { kernelMs_ = entropyMs_ = reconMs_ = 0; }

 private:
  struct Stream;
  struct Job;
  struct StepInfo;
  struct Round;
  int configure(Stream& s, int w, int h);
  int planFrame(Stream& s, Job& j, std::vector<char>& busy);
  int finishFrame(Stream& s, Job& j, const int32_t* statuses, std::vector<RoundResult>* results);
  int ensureStage(int parity, size_t bytes);
  int ensureStatus(int parity, int n);
  int planRound(const std::vector<int>& ids, const std::vector<int>* maxFrames, Round& r);
  int launchRecon(Round& r);
  int collectRound(Round& r, std::vector<RoundResult>* results);
  void cacheKey(Stream& s, int64_t index, int img, int golden, const TableHistory& hist);
  // Streams of a round by parity: 0/1 main (pipelined rounds alternate), 2 side.
  static bool isSide(int parity) { return parity >= kSide; }
  cudaStream_t entropyStream(int parity = 0) const {
    return isSide(parity) ? streamES_[parity - kSide] : (pipeDepth_ ? streamE_ : stream_);
  }
  cudaStream_t reconStream(int parity = 0) const { return isSide(parity) ? streamRS_[parity - kSide] : stream_; }
  int mainSets() const { return pipeDepth_ + 1; }
  // Slot sets: one per main parity in use (lookahead + 1 slots), then one
  // per side lane (a frame slot and the override slot).
  int slotSet(int parity) const { return isSide(parity) ? mainSets() + (parity - kSide) : parity; }
  int slotSets() const { return mainSets() + (side_ ? sideLanes_ : 0); }
  static constexpr int kMaxDepth = 3;
  static constexpr int kMainParities = kMaxDepth + 1;  // main rounds in flight at most
  static constexpr int kSide = kMainParities;           // parities kSide.. are the side lanes
  static constexpr int kParities = kMainParities + kSideLanes;

  cudaStream_t stream_ = nullptr;   // reconstruction, copies, status read-back
  cudaStream_t streamE_ = nullptr;  // entropy stage of pipelined rounds
  cudaStream_t streamES_[kSideLanes] = {}, streamRS_[kSideLanes] = {};  // side lanes: entropy, reconstruction
  cudaStream_t planStream_ = nullptr;  // reconstruction stream of the round being planned
  cudaEvent_t sideDone_[kSideLanes] = {};
  // Copy stream of downloadFrameAsync and the event after its last copy.
  cudaStream_t streamC_ = nullptr;
  cudaEvent_t copyDone_ = nullptr;
  bool copiesPending_ = false;
  cudaEvent_t reloadDone_ = nullptr;  // the last reloadStream's host-to-device copies
  bool reloadPending_ = false;
  // Entropy groups of pipelined main rounds: a pool of streams the groups
  // take in turn (so the groups of consecutive rounds run side by side), the
  // staging-upload event and one completion event per group.
  static constexpr int kEntropyGroups = 4;
  int entropyGroups_ = kEntropyGroups;
  int intraWarps_ = 0;
  static constexpr int kEntropyStreams = 2 * kEntropyGroups;
  cudaStream_t streamEG_[kEntropyStreams] = {};
  int nextEG_ = 0;
  cudaEvent_t evUp_[kMainParities] = {};
  cudaEvent_t evGroup_[kMainParities][kEntropyGroups] = {};
  // Second reconstruction stream of main rounds and its per-step events.
  static constexpr int kMaxSteps = 65;
  cudaStream_t streamB_ = nullptr;
  cudaEvent_t stepA_[kMainParities][kMaxSteps] = {};
  cudaEvent_t stepB_[kMainParities][kMaxSteps] = {};
  bool ownStream_ = false, ownStreamE_ = false;
  int pipeDepth_ = 0;
  bool side_ = false;
  int sideLanes_ = 0;
  bool mainInflight_ = false;
  cudaEvent_t mainDone_ = nullptr;
  bool sideInflight_[kSideLanes] = {};
  std::vector<std::unique_ptr<Stream>> streams_;
  std::unique_ptr<Round[]> rounds_;  // by parity
  std::vector<int> pipe_;  // parities of the main rounds in flight, oldest first
  int64_t roundSeq_ = 0;
  uint8_t* dStage_[kParities] = {};
  uint8_t* hStage_[kParities] = {};
  size_t stageCap_[kParities] = {};
  int32_t* hStatus_[kParities] = {};
  int statusCap_[kParities] = {};
  int32_t* dOne_ = nullptr;  // constant 1: the gate of discarded frames
  int64_t launches_ = 0;
  int lookahead_ = 1;
  size_t deviceBytes_ = 0;
  bool timing_ = false;
  cudaEvent_t ev_[kParities][4] = {};
  double kernelMs_ = 0, entropyMs_ = 0, reconMs_ = 0;
  double planSec_ = 0, launchSec_ = 0, collectSec_ = 0;
};

}  // namespace ebiv
