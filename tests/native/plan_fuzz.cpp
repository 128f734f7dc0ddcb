// Host-side fuzz harness for the GPU decoder's packet planning.
//
// Every byte range, macroblock bound and table the decode kernels read comes
// from the host planner (govid_gb300/csrc/payload.cpp, container.cpp), so the
// kernels' safety on hostile input rests on these invariants of each plan the
// planner accepts:
//   * every tile's bytes lie inside the packet;
//   * the tiles are the clamped grid (ebiv/frame.go:87-111), in order, their
//     macroblock bounds inside the frame, mbBase their running sum;
//   * the qp indexes the quantizer table;
//   * every used table is a non-decreasing run of starts ending at kM at the
//     alphabet size, padded with 0xFFFF.
// Built with AddressSanitizer and UBSan by the test that drives it, so an out
// of bounds read or an overflow in the planner itself fails too.
//
// The harness replays the Codec contract's host steps per packet exactly as
// GpuCodec::decode and Engine::planFrame run them (header checks, geometry,
// raw length, the golden-override split, main and override plans, and the
// table-history rollback of a failed main decode) and checks, against the
// oracle's status for the same packet: whatever the host rejects, the oracle
// rejects with the same status.  A packet the host accepts may still fail in
// the kernels (rANS errors), which the oracle reports; the harness takes the
// oracle's status as that outcome.  One outcome is ambiguous from the status
// alone: a key frame with an override whose main plan passed and whose
// override plan failed with the same status the oracle reports (a failing main
// decode rolls the table history back, a failing override plan does not), so a
// stream's comparison ends there.
//
// Input (binary, little endian): u32 streams; per stream u32 packets; per
// packet u32 length, i32 oracle status, bytes.  Output: one summary line.
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "container.h"
#include "payload.h"

using namespace ebiv;

namespace {

struct Input {
  const uint8_t* p;
  size_t n;
  size_t at = 0;
  bool take(void* dst, size_t k) {
    if (n - at < k) return false;
    std::memcpy(dst, p + at, k);
    at += k;
    return true;
  }
};

[[noreturn]] void violated(const char* what, int stream, int pkt) {
  std::fprintf(stderr, "invariant violated: %s (stream %d, packet %d)\n", what, stream, pkt);
  std::exit(3);
}

void checkPlan(const PayloadPlan& p, size_t pktLen, const Geometry& g, int stream, int pkt) {
  if (p.qp < 0 || p.qp > kMaxQP) violated("qp out of range", stream, pkt);
  const TileGrid grid(g.mbCols, g.mbRows, p.tileCols, p.tileRows);
  if ((int)p.tiles.size() != grid.count()) violated("tile count differs from the clamped grid", stream, pkt);
  uint32_t base = 0;
  for (int i = 0; i < grid.count(); i++) {
    const TileRange& t = p.tiles[(size_t)i];
    if ((uint64_t)t.offset + t.length > pktLen) violated("tile bytes outside the packet", stream, pkt);
    int x0, x1, y0, y1;
    grid.bounds(i, &x0, &x1, &y0, &y1);
    if (t.mbX0 != x0 || t.mbX1 != x1 || t.mbY0 != y0 || t.mbY1 != y1) violated("tile bounds", stream, pkt);
    if (!(x0 < x1 && x1 <= g.mbCols && y0 < y1 && y1 <= g.mbRows)) violated("tile outside the frame", stream, pkt);
    if (t.mbBase != base) violated("mbBase", stream, pkt);
    base += (uint32_t)((x1 - x0) * (y1 - y0));
  }
  if (base != (uint32_t)(g.mbCols * g.mbRows)) violated("tiles do not cover the frame", stream, pkt);
  for (int c = 0; c < kNumContexts; c++) {
    if (!p.tables.used[c]) continue;
    const int a = alphabetSize(c);
    const uint16_t* s = p.tables.start[c];
    if (s[0] != 0) violated("table does not start at 0", stream, pkt);
    for (int k = 1; k <= a; k++)
      if (s[k] < s[k - 1]) violated("table starts decrease", stream, pkt);
    if (s[a] != kM) violated("table does not end at kM", stream, pkt);
    for (int k = a + 1; k < 17; k++)
      if (s[k] != 0xFFFF) violated("table padding", stream, pkt);
  }
}

struct Counts {
  long streams = 0, packets = 0, compared = 0, hostRejects = 0, kernelRejects = 0, accepted = 0, ambiguous = 0;
};

// One stream through the Codec contract's host steps.
bool runStream(int sidx, const std::vector<std::vector<uint8_t>>& pk, const std::vector<int32_t>& oracle, Counts* c) {
  bool ready = false;
  Geometry geo;
  TableHistory hist;
  PayloadPlan main, ov;
  for (size_t i = 0; i < pk.size(); i++) {
    const uint8_t* b = pk[i].data();
    const size_t n = pk[i].size();
    const int want = oracle[i];
    c->packets++;
    c->compared++;
    // GpuCodec::decode's checks before the engine.
    FrameHeader fh;
    int st = parseFrameHeader(b, n, &fh);
    if (!st && fh.type == kFrameKey) {
      if ((int64_t)fh.width * fh.height > kMaxDecodePixels) st = kErrUnsupported;
      else if (ready && (fh.width != geo.W || fh.height != geo.H)) st = kErrDimensions;
      else if (!ready) {
        geo = Geometry::of(fh.width, fh.height);
        ready = true;
      }
    } else if (!st && !ready) {
      st = kErrNoKeyframe;
    }
    // Engine::planFrame.
    bool hasOv = false, planned = false;
    int ovStatus = kOK;
    TableHistory hMain;
    if (!st && fh.coding == kCodingRaw) {
      if (n - fh.bodyOffset != geo.packedSize()) st = kErrCorrupt;
    } else if (!st && fh.coding != kCodingIntra && fh.coding != kCodingInter) {
      st = kErrUnsupported;
    } else if (!st) {
      const bool key = fh.type == kFrameKey;
      size_t bodyOff = fh.bodyOffset, bodyLen = n - fh.bodyOffset, ovOff = 0, ovLen = 0;
      if (fh.goldenOverride) {
        int k;
        const uint64_t keyLen = getUvarint(b + bodyOff, bodyLen, &k);
        if (k <= 0 || keyLen > (uint64_t)(bodyLen - (size_t)k)) st = kErrCorrupt;
        else {
          ovOff = bodyOff + (size_t)k + (size_t)keyLen;
          ovLen = bodyLen - (size_t)k - (size_t)keyLen;
          bodyOff += (size_t)k;
          bodyLen = (size_t)keyLen;
        }
      }
      if (!st) st = planPayload(b, bodyOff, bodyLen, key, geo.mbCols, geo.mbRows, hist, &main);
      if (!st) {
        checkPlan(main, n, geo, sidx, (int)i);
        planned = true;
        hMain = hist;
        if (key && fh.goldenOverride) {
          hasOv = true;
          ovStatus = planPayload(b, ovOff, ovLen, false, geo.mbCols, geo.mbRows, hist, &ov);
          if (ovStatus == kOK) checkPlan(ov, n, geo, sidx, (int)i);
        }
      }
    }
    if (st) {
      c->hostRejects++;
      if (want != st) {
        std::fprintf(stderr, "stream %d packet %zu: host rejects with %d, oracle says %d\n", sidx, i, st, want);
        return false;
      }
      continue;
    }
    if (!planned) {  // a raw frame
      if (want != kOK) {
        std::fprintf(stderr, "stream %d packet %zu: raw frame accepted, oracle says %d\n", sidx, i, want);
        return false;
      }
      c->accepted++;
      continue;
    }
    if (want == kOK) {
      if (hasOv && ovStatus != kOK) {
        std::fprintf(stderr, "stream %d packet %zu: override plan fails with %d, oracle decodes\n", sidx, i, ovStatus);
        return false;
      }
      c->accepted++;
      continue;
    }
    // The host accepted; the oracle failed.
    if (hasOv && ovStatus != kOK && ovStatus == want) {
      c->ambiguous++;
      return true;  // main decode failure or override plan failure: the history differs
    }
    c->kernelRejects++;
    if (hasOv) hist = hMain;  // the failed main decode never reached the override's tables
  }
  return true;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc != 2) {
    std::fprintf(stderr, "usage: %s streams.bin\n", argv[0]);
    return 2;
  }
  FILE* f = std::fopen(argv[1], "rb");
  if (!f) return 2;
  std::vector<uint8_t> data;
  uint8_t buf[1 << 16];
  size_t k;
  while ((k = std::fread(buf, 1, sizeof(buf), f)) > 0) data.insert(data.end(), buf, buf + k);
  std::fclose(f);
  Input in{data.data(), data.size()};
  uint32_t ns;
  if (!in.take(&ns, 4)) return 2;
  Counts c;
  int bad = 0;
  for (uint32_t s = 0; s < ns; s++) {
    uint32_t np;
    if (!in.take(&np, 4)) return 2;
    std::vector<std::vector<uint8_t>> pk(np);
    std::vector<int32_t> oracle(np);
    for (uint32_t i = 0; i < np; i++) {
      uint32_t len;
      if (!in.take(&len, 4) || !in.take(&oracle[i], 4) || in.n - in.at < len) return 2;
      pk[i].assign(in.p + in.at, in.p + in.at + len);
      in.at += len;
    }
    c.streams++;
    if (!runStream((int)s, pk, oracle, &c)) bad++;
  }
  std::printf("streams %ld packets %ld compared %ld host_rejects %ld kernel_rejects %ld accepted %ld ambiguous %ld mismatches %d\n",
              c.streams, c.packets, c.compared, c.hostRejects, c.kernelRejects, c.accepted, c.ambiguous, bad);
  return bad ? 1 : 0;
}
