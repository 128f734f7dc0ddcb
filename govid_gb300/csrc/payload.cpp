#include "payload.h"

#include <cstring>

namespace ebiv {

namespace {
// Builds the kernel form of one table.  Returns false when the frequencies
// do not describe a usable table: a sum other than kM, or a prefix sum past
// kM (a uint32 sum that wrapped; the reference would fault filling its
// reverse map, this decoder reports ErrCorrupt).
bool buildStarts(const uint32_t* f, int n, uint16_t* start) {
  uint32_t cum = 0;
  bool wrapped = false;
  for (int s = 0; s < n; s++) {
    if ((uint64_t)cum + f[s] > kM) wrapped = true;
    start[s] = (uint16_t)(cum > kM ? kM : cum);
    cum += f[s];
  }
  for (int s = n; s < 17; s++) start[s] = s == n ? (uint16_t)kM : (uint16_t)0xFFFF;
  return cum == kM && !wrapped;
}
}  // namespace

int planPayload(const uint8_t* base, size_t bodyOffset, size_t len, bool key, int mbCols, int mbRows,
                TableHistory& hist, PayloadPlan* plan) {
  const uint8_t* body = base + bodyOffset;
  // parseCodedHeader — ebiv/frame.go:197-220
  if (len < 1) return kErrCorrupt;
  const int qp = body[0];
  size_t pos = 1;
  int n;
  const uint64_t cols = getUvarint(body + pos, len - pos, &n);
  if (n <= 0) return kErrCorrupt;
  pos += (size_t)n;
  const uint64_t rows = getUvarint(body + pos, len - pos, &n);
  if (n <= 0) return kErrCorrupt;
  pos += (size_t)n;
  if (qp > kMaxQP || cols == 0 || rows == 0 || cols > 65535 || rows > 65535) return kErrCorrupt;
  plan->qp = qp;
  plan->tileCols = (int)cols;
  plan->tileRows = (int)rows;
  const uint64_t tablesLen = getUvarint(body + pos, len - pos, &n);
  if (n <= 0 || tablesLen > (uint64_t)(len - pos - (size_t)n)) return kErrCorrupt;
  pos += (size_t)n;

  // parseTablesInto — ebiv/rans.go:396-471
  DeviceTables& t = plan->tables;
  if (key)
    for (int c = 0; c < kNumContexts; c++) hist.e[c].len = 0;
  const uint8_t* tb = body + pos;
  const size_t tlen = (size_t)tablesLen;
  size_t tp = 0;
  for (int c = 0; c < kNumContexts; c++) {
    if (tp >= tlen) return kErrCorrupt;
    const uint8_t mode = tb[tp++];
    if (c == ctxBypass && mode != 0) return kErrCorrupt;
    const int asz = alphabetSize(c);
    TableHistory::Entry& h = hist.e[c];
    const bool haveRef = h.len == asz;
    t.used[c] = 0;
    switch (mode) {
      case 0:
        break;
      case 1:
        if (key || !haveRef) return kErrCorrupt;
        if (!buildStarts(h.v, asz, t.start[c])) return kErrCorrupt;
        t.used[c] = 1;
        break;
      case 2:
        if (!h.alloc) {
          std::memset(h.v, 0, sizeof(h.v));
          h.alloc = true;
        }
        h.len = asz;
        for (int s = 0; s < asz; s++) {
          const uint64_t v = getUvarint(tb + tp, tlen - tp, &n);
          if (n <= 0) return kErrCorrupt;
          tp += (size_t)n;
          h.v[s] = (uint32_t)v;
        }
        if (!buildStarts(h.v, asz, t.start[c])) return kErrCorrupt;
        t.used[c] = 1;
        break;
      case 3:
        if (key || !haveRef) return kErrCorrupt;
        for (int s = 0; s < asz; s++) {
          const int64_t v = getVarint(tb + tp, tlen - tp, &n);
          if (n <= 0) return kErrCorrupt;
          tp += (size_t)n;
          const int64_t nv = (int64_t)h.v[s] + v;
          if (nv < 0 || nv > (int64_t)kM) return kErrCorrupt;
          h.v[s] = (uint32_t)nv;
        }
        if (!buildStarts(h.v, asz, t.start[c])) return kErrCorrupt;
        t.used[c] = 1;
        break;
      default:
        return kErrCorrupt;
    }
  }
  // installBypass — ebiv/rans.go:317-322
  {
    const uint32_t bypass[2] = {kM / 2, kM / 2};
    buildStarts(bypass, 2, t.start[ctxBypass]);
    t.used[ctxBypass] = 1;
  }
  if (tp != tlen) return kErrCorrupt;
  pos += tlen;

  const uint64_t want = cols * rows;
  plan->tiles.clear();
  while (plan->tiles.size() < want) {
    const uint64_t tl = getUvarint(body + pos, len - pos, &n);
    if (n <= 0 || tl > (uint64_t)(len - pos - (size_t)n)) return kErrCorrupt;
    pos += (size_t)n;
    TileRange r;
    r.offset = (uint32_t)(bodyOffset + pos);
    r.length = (uint32_t)tl;
    r.mbX0 = r.mbX1 = r.mbY0 = r.mbY1 = 0;
    r.mbBase = 0;
    plan->tiles.push_back(r);
    pos += (size_t)tl;
  }
  // decodeCoded's grid check — ebiv/decode_intra.go:60-63
  const TileGrid grid(mbCols, mbRows, (int)cols, (int)rows);
  if ((uint64_t)grid.count() != plan->tiles.size()) return kErrCorrupt;
  uint32_t mbBase = 0;
  for (int i = 0; i < grid.count(); i++) {
    int x0, x1, y0, y1;
    grid.bounds(i, &x0, &x1, &y0, &y1);
    plan->tiles[(size_t)i].mbBase = mbBase;
    mbBase += (uint32_t)((x1 - x0) * (y1 - y0));
    plan->tiles[(size_t)i].mbX0 = (uint16_t)x0;
    plan->tiles[(size_t)i].mbX1 = (uint16_t)x1;
    plan->tiles[(size_t)i].mbY0 = (uint16_t)y0;
    plan->tiles[(size_t)i].mbY1 = (uint16_t)y1;
  }
  return kOK;
}

}  // namespace ebiv
