// EBIV container demuxer: ebiv/reader.go and ebiv/format.go restated in C++.
#include "container.h"

#include <cstring>

namespace ebiv {

// frameIndexAt — ebiv/format.go:263-275.  The estimate is within a frame of
// the answer unless t * fpsNum wraps (Go int64 arithmetic), where the
// reference's correction walk can run for ~2^63 steps; a walk that needs
// 2^20 steps or more gives -1 instead, as the GPU seek does.
int64_t FileHeader::frameIndexAt(int64_t t) const {
  if (t <= 0) return 0;
  const int64_t num = (int64_t)((uint64_t)t * (uint64_t)fpsNum);
  const int64_t den = (int64_t)((uint64_t)fpsDen * 1000000000ull);
  int64_t i = num / den;
  int steps = 0;
  while (frameTime(i + 1) <= t)
    if (++steps >= kSeekWalkLimit) return -1;
    else i++;
  while (i > 0 && frameTime(i) > t)
    if (++steps >= kSeekWalkLimit) return -1;
    else i--;
  return i;
}

// parseFrameHeader — ebiv/format.go:376-409
int parseFrameHeader(const uint8_t* b, size_t n, FrameHeader* f) {
  *f = FrameHeader{};
  if (n < 1) return kErrCorrupt;
  f->type = b[0] & 0x03;
  f->coding = (b[0] >> 2) & 0x07;
  f->goldenOverride = (b[0] & (1 << 5)) != 0;
  if (f->type != kFrameKey && f->type != kFrameInter) return kErrCorrupt;
  if (f->goldenOverride && f->type != kFrameKey) return kErrCorrupt;
  if (f->type != kFrameKey) {
    f->bodyOffset = 1;
    return kOK;
  }
  if (n < 6) return kErrCorrupt;
  f->width = rd16(b + 1);
  f->height = rd16(b + 3);
  if (f->width == 0 || f->height == 0) return kErrCorrupt;
  if ((b[5] >> 4) != 0) return kErrUnsupported;
  if ((b[5] & 0x0f) != 0) return kErrUnsupported;
  f->bodyOffset = 6;
  return kOK;
}

// NewDemuxer + FileHeader.unmarshal — ebiv/reader.go:32-61, format.go:208-247
int Reader::open(const uint8_t* data, size_t n) {
  data_.assign(data, data + n);
  index_.clear();
  next_ = 0;
  closed_ = false;
  rebuilt_ = false;
  if (n < (size_t)kFileHeaderSize) return kErrBadMagic;
  const uint8_t* b = data_.data();
  if (std::memcmp(b, "EBIV", 4) != 0) return kErrBadMagic;
  hdr_.version = rd16(b + 4);
  if (hdr_.version != kVersion) return kErrVersion;
  if (rd16(b + 6) != kFileHeaderSize) return kErrCorrupt;
  const uint32_t w = rd32(b + 8), h = rd32(b + 12);
  if (w == 0 || w > 65535 || h == 0 || h > 65535) return kErrCorrupt;
  hdr_.width = (int)w;
  hdr_.height = (int)h;
  hdr_.fpsNum = rd32(b + 16);
  hdr_.fpsDen = rd32(b + 20);
  if (hdr_.fpsNum == 0 || hdr_.fpsDen == 0) return kErrCorrupt;
  hdr_.chroma = b[28];
  hdr_.depth = b[29];
  hdr_.colorRange = b[30];
  hdr_.colorPrimaries = b[31];
  if (hdr_.chroma != 0 || hdr_.depth != 0) return kErrUnsupported;
  hdr_.tileCols = rd16(b + 32);
  hdr_.tileRows = rd16(b + 34);
  hdr_.flags = rd32(b + 36);
  if (readIndex() == kOK) return kOK;
  index_.clear();
  const int st = scanFrames();
  if (st == kOK) rebuilt_ = true;
  return st;
}

// readIndex + validateEntry — ebiv/reader.go:65-121
int Reader::readIndex() {
  const int64_t size = (int64_t)data_.size();
  if (size < kFileHeaderSize + kFooterSize) return kErrCorrupt;
  const uint8_t* footer = data_.data() + size - kFooterSize;
  if (std::memcmp(footer + 16, "EBIX", 4) != 0) return kErrCorrupt;
  const uint64_t offset = rd64(footer);
  const uint32_t count = rd32(footer + 8);
  const uint32_t want = rd32(footer + 12);
  // An offset past the file fails in the reference too (the bounds check, or
  // the seek to a wrapped negative position); checking it first keeps the sum
  // below from overflowing.
  if (offset < (uint64_t)kFileHeaderSize || offset > (uint64_t)size) return kErrCorrupt;
  const int64_t end = (int64_t)offset + (int64_t)count * kIndexEntrySize;
  if (end != size - kFooterSize) return kErrCorrupt;
  const uint8_t* buf = data_.data() + offset;
  if (crc32IEEE(buf, (size_t)count * kIndexEntrySize) != want) return kErrCorrupt;
  index_.resize(count);
  for (uint32_t i = 0; i < count; i++) {
    const uint8_t* p = buf + (size_t)i * kIndexEntrySize;
    IndexEntry& e = index_[i];
    e.offset = rd64(p);
    e.size = rd32(p + 8);
    e.keyframe = (rd32(p + 12) & 1) != 0;
    if (e.offset < (uint64_t)kFileHeaderSize || e.size == 0 || e.size > kMaxFrameSize) return kErrCorrupt;
    if (e.offset + kFrameRecordSize + (uint64_t)e.size > offset) return kErrCorrupt;
  }
  if (count > 0 && !index_[0].keyframe) return kErrCorrupt;
  return kOK;
}

// scanFrames — ebiv/reader.go:126-160
int Reader::scanFrames() {
  const int64_t size = (int64_t)data_.size();
  int64_t off = kFileHeaderSize;
  while (off + kFrameRecordSize <= size) {
    const uint8_t* rec = data_.data() + off;
    if (rd16(rec) != kFrameSync) break;
    const bool key = (rd16(rec + 2) & 1) != 0;
    const uint32_t payload = rd32(rec + 4);
    if (payload == 0 || payload > kMaxFrameSize) break;
    const int64_t end = off + kFrameRecordSize + (int64_t)payload;
    if (end > size) break;
    index_.push_back({(uint64_t)off, payload, key});
    off = end;
  }
  if (index_.empty()) return kErrCorrupt;
  if (!index_[0].keyframe) return kErrCorrupt;
  return kOK;
}

// NextPacket — ebiv/reader.go:189-217
int Reader::nextPacket(const uint8_t** data, size_t* n, int64_t* ts, bool* key) {
  if (closed_ || next_ >= (int)index_.size()) return kErrEOF;
  const IndexEntry& e = index_[(size_t)next_];
  if (!e.readable()) return kErrIO;  // reader.go:203-205: the seek fails, next stays
  *data = data_.data() + e.payloadAt();
  *n = e.size;
  if (ts) *ts = hdr_.frameTime(next_);
  if (key) *key = e.keyframe;
  next_++;
  return kOK;
}

int Reader::packet(int i, const uint8_t** data, size_t* n) const {
  if (i < 0 || i >= (int)index_.size()) return kErrArg;
  const IndexEntry& e = index_[(size_t)i];
  if (!e.readable()) return kErrIO;
  *data = data_.data() + e.payloadAt();
  *n = e.size;
  return kOK;
}

// Seek / keyframeBefore — ebiv/reader.go:222-258
int Reader::seek(int64_t t, int64_t* landed) {
  if (closed_ || index_.empty()) return kErrEOF;
  int64_t target = hdr_.frameIndexAt(t);
  if (target < 0) return kErrCorrupt;  // a frame rate the walk cannot settle
  if (target >= (int64_t)index_.size()) target = (int64_t)index_.size() - 1;
  target = keyframeBefore((int)target);
  next_ = (int)target;
  if (landed) *landed = hdr_.frameTime(target);
  return kOK;
}

int Reader::keyframeBefore(int i) const {
  if (i >= (int)index_.size()) i = (int)index_.size() - 1;
  while (i > 0 && !index_[(size_t)i].keyframe) i--;
  return i;
}

}  // namespace ebiv
