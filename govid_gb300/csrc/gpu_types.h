// Device-side data layout of the GB300 EBIV decoder, shared by the kernels
// and the host orchestration.
//
// HBM layout per stream:
//   * three padded frame buffers (work / last-reference / golden), each the
//     luma plane (mbCols*16 x mbRows*16) followed by Cb and Cr
//     (mbCols*8 x mbRows*8), rows contiguous, stride = padded width;
//   * per decode slot: the packet bytes, a FrameDesc, the resolved rANS
//     tables, the tile ranges, one 48-byte MBRec per macroblock, a fixed
//     408-word coefficient region per macroblock and the motion-vector grid.
#pragma once

#include <cstdint>

#include "payload.h"

namespace ebiv {

// Per-macroblock output of the entropy stage.
enum : uint8_t { kRecSkip = 0, kRecInter = 1, kRecIntra = 2, kRecNone = 0xFF };

struct alignas(16) MBRec {
  uint8_t mode;    // kRecSkip / kRecInter / kRecIntra / kRecNone
  uint8_t ref;     // refLast / refGolden
  uint8_t part;    // partition shape
  uint8_t cbp;     // coded-block pattern (inter)
  uint8_t tx;      // luma transform index
  uint8_t cmode;   // chroma intra mode
  uint8_t pad0, pad1;
  int16_t mv[4][2];       // per-partition vectors, quarter pel
  uint8_t lmode[16];      // luma intra mode per transform block (raster)
  uint32_t nzmask;        // bit k: luma block k has coefficients; 16: Cb; 17: Cr
  uint32_t wmask;         // bit k: luma block k written; 16: Cb; 17: Cr
};
static_assert(sizeof(MBRec) == 48, "MBRec layout");

// Coefficient region per macroblock, in 32-bit words: each block has its
// nonzero count followed by entries packing (row-major position in bits 0-7,
// signed level in bits 8-31).  Luma block k of an n x n transform starts at
// k*(n*n+1); Cb at kCoefCb, Cr at kCoefCr.
constexpr int kCoefCb = 272;
constexpr int kCoefCr = 337;
constexpr int kCoefPerMB = 408;
constexpr uint32_t kWriteAll = 0x3FFFFu;

// The entropy kernel decodes up to this many tiles of one frame per CTA
// (one warp each), sharing the frame's symbol tables.  A job is
// int4{descriptor, first tile, tile count, 0}.
constexpr int kEntropyTilesPerJob = 4;

// Bytes of symbol log per macroblock in a decode slot (the entropy stage's
// symbol path; a tile whose symbols do not fit takes the full chain, which
// decodes it a second time).  Key frames coded at q18 average about 80
// symbols per macroblock and more in textured areas, and the chain also
// reserves room for a whole block before decoding it, so the log holds 192.
constexpr int kSymPerMB = 192;

struct TileStat {
  int32_t err;         // 0 or an ebiv status
  int32_t intraCount;  // intra macroblocks reconstructed in this tile
  int32_t done;        // macroblocks the tile's chain reached (raster order)
  int32_t errAt;       // symbol path: log index of the failing symbol (or none); -1: full chain
};

// Intra list entries hold the frame macroblock index in bits 0-17.
constexpr int32_t kSkipped = 1000;
constexpr int kLevelShift = 18;
constexpr uint32_t kIndexMask = (1u << kLevelShift) - 1;

struct FrameDesc {
  // Planes (padded).  ref/gold may alias rec's siblings; never rec itself.
  uint8_t* rec[3];
  const uint8_t* ref[3];
  const uint8_t* gold[3];
  int32_t strideY, strideC;  // = padded widths
  int32_t padW, padH, padCW, padCH;
  int32_t mbCols, mbRows;
  int32_t inter;
  int32_t qdc, qac;
  int32_t tileCount;
  int32_t pad;
  const uint8_t* pkt;
  const DeviceTables* tables;
  const TileRange* tiles;
  MBRec* mbrec;
  uint32_t* coef;
  int16_t* mvgrid;      // 2 x int16 per macroblock (wide-tile fallback rows)
  int16_t* lvgrid;      // 1 x int16 per macroblock (wide-tile fallback rows)
  uint32_t* intraList;  // per tile at mbBase: intra macroblocks, raster order
  uint32_t* intraSorted;// per tile at mbBase: the same grouped by level
  TileStat* tileStat;
  int32_t* status;      // frame status, written by the commit step
  // Status of the frame this one depends on (the previous frame of the
  // stream decoded in the same round).  When it is nonzero the reconstruction
  // kernels skip this frame and mark it kSkipped; the host re-plans it.
  const int32_t* gate;
  // Records of that previous frame while its intra stage may still be
  // running (null when it is complete), and whether it was a key frame
  // (then every macroblock of this frame waits for it).  Inter
  // reconstruction runs in two phases: macroblocks whose prediction reads
  // no intra macroblock of the previous frame, then the rest (marked in dep).
  const MBRec* prevRec;
  int32_t prevKey;
  int32_t pad2;
  uint8_t* dep;
  // Symbol path of the entropy stage (null symLog: every tile takes the full
  // chain): a log of symPerMB bytes per macroblock, tile t's at
  // tiles[t].mbBase * symPerMB, and per macroblock the index of its first
  // symbol in its tile's log (at mbBase + raster index within the tile).
  uint8_t* symLog;
  uint32_t* symOff;
  int32_t symPerMB;
  int32_t pad3;
};

}  // namespace ebiv
