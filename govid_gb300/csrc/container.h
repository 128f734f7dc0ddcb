// EBIV container demuxer (host C++), the Demuxer half of the drop-in
// boundary: it parses the file header, loads the CRC-checked frame index from
// the footer or rebuilds it by scanning frame records, and hands out packets
// (ebiv/reader.go:20-258, ebiv/format.go:186-328).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "ebiv_format.h"

namespace ebiv {

struct FileHeader {
  uint16_t version = 0;
  int width = 0, height = 0;
  uint32_t fpsNum = 0, fpsDen = 0;
  uint8_t chroma = 0, depth = 0, colorRange = 0, colorPrimaries = 0;
  uint16_t tileCols = 0, tileRows = 0;
  uint32_t flags = 0;
  // frameTime — ebiv/format.go:250-253
  // (Go int64 arithmetic: the products wrap modulo 2^64 before dividing.)
  int64_t frameTime(int64_t i) const {
    const int64_t p = (int64_t)((uint64_t)i * (uint64_t)fpsDen * 1000000000ull);
    return p / (int64_t)fpsNum;
  }
  // -1 when the correction walk needs kSeekWalkLimit steps or more.
  int64_t frameIndexAt(int64_t t) const;
  static constexpr int kSeekWalkLimit = 1 << 20;
};

struct IndexEntry {
  uint64_t offset = 0;
  uint32_t size = 0;
  bool keyframe = false;
  // Where the payload is read: offset + the record header, in Go's wrapping
  // int64 (ebiv/reader.go:203).  validateEntry's uint64 sum can wrap, so an
  // index entry may carry an offset near 2^64: the reference then seeks to a
  // negative position and NextPacket fails (kErrIO here), or, for the eight
  // offsets that wrap to 0..7, reads from there.
  int64_t payloadAt() const { return (int64_t)(offset + 8u); }
  bool readable() const { return payloadAt() >= 0; }
};

// Parsed per-packet header (ebiv/format.go:333-409).
struct FrameHeader {
  int type = 0, coding = 0;
  int width = 0, height = 0;
  bool goldenOverride = false;
  size_t bodyOffset = 0;
};
int parseFrameHeader(const uint8_t* b, size_t n, FrameHeader* out);

// The reader holds the whole container in memory (the caller's bytes are
// copied once), so packets are stable views into it.
class Reader {
 public:
  int open(const uint8_t* data, size_t n);
  const FileHeader& header() const { return hdr_; }
  const std::vector<IndexEntry>& index() const { return index_; }
  int frameCount() const { return (int)index_.size(); }
  // NextPacket — returns kErrEOF at the end, kErrIO (without advancing) for
  // an entry whose payload position is negative.
  int nextPacket(const uint8_t** data, size_t* n, int64_t* ts, bool* key);
  // Packet i without moving the read position (kErrIO when unreadable).
  int packet(int i, const uint8_t** data, size_t* n) const;
  // Seek — positions at the last key frame at or before t; returns its time.
  int seek(int64_t t, int64_t* landed);
  int keyframeBefore(int i) const;
  int64_t duration() const { return hdr_.frameTime((int64_t)index_.size()); }
  void close() { closed_ = true; }
  int position() const { return next_; }
  bool rebuiltIndex() const { return rebuilt_; }

 private:
  int readIndex();
  int scanFrames();
  std::vector<uint8_t> data_;
  FileHeader hdr_;
  std::vector<IndexEntry> index_;
  int next_ = 0;
  bool closed_ = false;
  bool rebuilt_ = false;
};

}  // namespace ebiv
