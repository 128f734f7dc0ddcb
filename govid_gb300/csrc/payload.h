// Host-side planning of one coded EBIV payload for the GPU decoder: the coded
// header, the per-context frequency tables (resolved against the stream's
// table history) and the tile byte ranges.  This is the serial, byte-sized
// part of decode (ebiv/frame.go:197-274, ebiv/rans.go:396-471); the kernels
// receive its result as a compact descriptor.
#pragma once

#include <cstdint>
#include <vector>

#include "ebiv_format.h"

namespace ebiv {

// Last shipped frequency vector per context, with Go slice semantics: a key
// frame truncates to length zero but keeps the backing values, which a later
// full table that fails part-way leaves partly overwritten.
struct TableHistory {
  struct Entry {
    int len = 0;
    bool alloc = false;
    uint32_t v[16] = {0};
  };
  Entry e[kNumContexts];
};

// Cumulative starts per context as the kernels consume them: start[c][s] for
// s < alphabet, then kM, padded to 17 entries with 0xFFFF so the lane-wise
// ballot lookup never selects a symbol past the alphabet.
struct DeviceTables {
  uint16_t start[kNumContexts][17];
  uint8_t used[kNumContexts];
  uint8_t pad[8];
};

struct TileRange {
  uint32_t offset;  // byte offset within the packet
  uint32_t length;
  uint16_t mbX0, mbX1, mbY0, mbY1;
  uint32_t mbBase;  // macroblocks in the tiles before this one (tile order)
};

struct PayloadPlan {
  int qp = 0;
  int tileCols = 0, tileRows = 0;
  std::vector<TileRange> tiles;
  DeviceTables tables;
};

// Parses a coded payload located at body[0..len) (offsets recorded relative
// to `base`, the start of the packet).  Updates `hist` exactly as the
// reference does, including on failure.  mbCols/mbRows give the stream's
// macroblock grid for the tile-count check.
int planPayload(const uint8_t* base, size_t bodyOffset, size_t len, bool key, int mbCols, int mbRows,
                TableHistory& hist, PayloadPlan* plan);

}  // namespace ebiv
