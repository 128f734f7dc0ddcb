// Host-side fuzz harness for the EBIV demuxer (govid_gb300/csrc/container.cpp,
// the Demuxer half of the drop-in boundary: NewDemuxer, readIndex,
// scanFrames, NextPacket; ebiv/reader.go:32-217).
//
// For each container it opens a Reader and prints one line: the status, and
// when it opened, the frame count, whether the index was rebuilt by scanning,
// and per frame the payload position (-1 when NextPacket cannot read it), the
// size, the key flag and the CRC-32 of the bytes packet(i) hands out
// (every view read in full, so an out-of-range one fails under
// AddressSanitizer); nextPacket must hand out the same views up to the first
// unreadable entry and stay there.  The test that drives it compares every
// line with the oracle's demuxer.
//
// Input (binary, little endian): u32 containers; per container u32 length,
// bytes.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

#include "container.h"

using namespace ebiv;

namespace {

void run(const uint8_t* data, size_t n) {
  Reader r;
  const int st = r.open(data, n);
  std::printf("%d", st);
  if (st) {
    std::printf("\n");
    return;
  }
  std::printf(" %d %d", r.frameCount(), r.rebuiltIndex() ? 1 : 0);
  // Every frame through packet(i): the view must be the container's bytes at
  // the payload position.
  int firstUnreadable = -1;
  for (int i = 0; i < r.frameCount(); i++) {
    const IndexEntry& e = r.index()[(size_t)i];
    const uint8_t* a = nullptr;
    size_t an = 0;
    const int pst = r.packet(i, &a, &an);
    if (pst == kErrIO) {
      if (e.readable()) {
        std::printf(" mismatch\n");
        return;
      }
      if (firstUnreadable < 0) firstUnreadable = i;
      std::printf(" -1:%u:%d", e.size, e.keyframe ? 1 : 0);
      continue;
    }
    const int64_t at = e.payloadAt();
    if (pst != kOK || an != e.size || at < 0 || (uint64_t)at + an > n || std::memcmp(a, data + at, an) != 0) {
      std::printf(" mismatch\n");
      return;
    }
    std::printf(" %lld:%zu:%d:%08x", (long long)at, an, e.keyframe ? 1 : 0, crc32IEEE(a, an));
  }
  // NextPacket from the start: the same views up to the first unreadable
  // entry, where it fails and stays (ebiv/reader.go:189-217), else EOF.
  const int stop = firstUnreadable < 0 ? r.frameCount() : firstUnreadable;
  for (int i = 0; i <= stop; i++) {
    const uint8_t* b = nullptr;
    size_t bn = 0;
    int64_t ts = 0;
    bool key = false;
    const int nst = r.nextPacket(&b, &bn, &ts, &key);
    const uint8_t* a = nullptr;
    size_t an = 0;
    const bool ok = i < stop ? (nst == kOK && r.packet(i, &a, &an) == kOK && a == b && an == bn &&
                                key == r.index()[(size_t)i].keyframe && ts == r.header().frameTime(i))
                             : (nst == (firstUnreadable < 0 ? kErrEOF : kErrIO) && r.position() == stop);
    if (!ok) {
      std::printf(" next-mismatch\n");
      return;
    }
  }
  std::printf("\n");
}

}  // namespace

int main(int argc, char** argv) {
  if (argc != 2) {
    std::fprintf(stderr, "usage: %s containers.bin\n", argv[0]);
    return 2;
  }
  FILE* f = std::fopen(argv[1], "rb");
  if (!f) return 2;
  std::vector<uint8_t> data;
  uint8_t buf[1 << 16];
  size_t k;
  while ((k = std::fread(buf, 1, sizeof(buf), f)) > 0) data.insert(data.end(), buf, buf + k);
  std::fclose(f);
  size_t at = 0;
  auto take32 = [&](uint32_t* v) {
    if (data.size() - at < 4) return false;
    std::memcpy(v, data.data() + at, 4);
    at += 4;
    return true;
  };
  uint32_t nc;
  if (!take32(&nc)) return 2;
  for (uint32_t c = 0; c < nc; c++) {
    uint32_t len;
    if (!take32(&len) || data.size() - at < len) return 2;
    // A copy of exactly the container's bytes, so a read past its end is
    // caught (the reader copies it once more).
    std::vector<uint8_t> one(data.begin() + (long)at, data.begin() + (long)at + len);
    at += len;
    run(one.data(), one.size());
  }
  return 0;
}
