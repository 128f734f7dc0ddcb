// EBIV bitstream constants and small shared helpers for the host side of the
// GB300 decoder and the EBIV encoder.  The constants restate the reference's
// coding model (ebiv/model.go:20-213, ebiv/rans.go:20-25, ebiv/quant.go:19-51,
// ebiv/transform.go:15-40, ebiv/scan.go:17-35) and are identical by necessity:
// they define the bitstream.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace ebiv {

constexpr int kScaleBits = 12;
constexpr uint32_t kM = 1u << kScaleBits;  // rANS frequency total
constexpr uint32_t kLower = 1u << 23;      // normalized interval lower bound
constexpr int kStates = 4;                 // interleaved rANS states

constexpr int kMB = 16;       // luma macroblock
constexpr int kCMB = 8;       // chroma block per macroblock
constexpr int kDCPred = 128;  // neutral prediction
constexpr int kMaxLevels = 256;
constexpr int kLumaTx[3] = {4, 8, 16};

enum IntraMode { modeDC, modeV, modeH, modeTM, modeD45, modeD27, modeD23, modeD135, modeD117, modeD113, kNumIntraModes };
enum MBMode { mbSkip, mbInter, mbIntra, kNumMBModes };
enum RefSel { refLast, refGolden, kNumRefs };
enum CBPBits { cbpLuma = 1, cbpCb = 2, cbpCr = 4, kNumCBP = 8 };
enum PartMode { partWhole, part16x8, part8x16, part8x8, kNumPartModes };
enum Token { tZero, tOne, tTwo, tThree, tFour, tEscape, tEOB, kNumTokens };
constexpr int kNumMVClasses = 16, kNumEscClasses = 16;

enum Ctx {
  ctxTxSize, ctxLumaMode, ctxChromaMode, ctxMBMode, ctxRef, ctxPart, ctxCBP, ctxSign,
  ctxEscClass, ctxMVClassX, ctxMVClassY, ctxBypass, ctxTokenBase
};
constexpr int kNumBands = 5, kNumPrevClass = 3;
constexpr int kLumaTokenCtx = 3 * kNumBands * kNumPrevClass;
constexpr int kChromaTokenCtx = kNumBands * kNumPrevClass;
constexpr int kNumContexts = ctxTokenBase + kLumaTokenCtx + kChromaTokenCtx;  // 72
constexpr int kPlaneLuma = 0, kPlaneChroma = 1;
constexpr int kSDHMinSpan = 4;
constexpr int kMVClampRange = 4096;
constexpr int kMaxQP = 63;
constexpr int64_t kMaxDecodePixels = 8192LL * 4320LL;

// Container sizes (ebiv/format.go:28-46).
constexpr int kVersion = 4;
constexpr int kFileHeaderSize = 48;
constexpr int kFrameRecordSize = 8;
constexpr int kIndexEntrySize = 16;
constexpr int kFooterSize = 20;
constexpr uint32_t kMaxFrameSize = 256u << 20;
constexpr uint16_t kFrameSync = 0xEB17;

// Coding modes / frame types (ebiv/format.go:62-95).
enum { kFrameKey = 0, kFrameInter = 1 };
enum { kCodingRaw = 0, kCodingIntra = 1, kCodingInter = 2 };

// Status codes shared with the C-ABI (one per ebiv error sentinel,
// ebiv/format.go:110-119).
enum Status {
  kOK = 0,
  kErrCorrupt = 1,
  kErrNoKeyframe = 2,
  kErrDimensions = 3,
  kErrUnsupported = 4,
  kErrVersion = 5,
  kErrBadMagic = 6,
  kErrConfig = 7,
  kErrWriterClosed = 8,
  kErrEOF = 9,
  kErrIO = 10,
  kErrDevice = 11,
  kErrArg = 12,
  kErrTooLarge = 13,  // beyond the fixed scratch of ebivgpu_decode_key_noalloc
};

struct Rect4 {
  int x, y, w, h;
};
inline const Rect4* partRects(int part) {
  static const Rect4 r[4][4] = {
      {{0, 0, 16, 16}, {0, 0, 0, 0}, {0, 0, 0, 0}, {0, 0, 0, 0}},
      {{0, 0, 16, 8}, {0, 8, 16, 8}, {0, 0, 0, 0}, {0, 0, 0, 0}},
      {{0, 0, 8, 16}, {8, 0, 8, 16}, {0, 0, 0, 0}, {0, 0, 0, 0}},
      {{0, 0, 8, 8}, {8, 0, 8, 8}, {0, 8, 8, 8}, {8, 8, 8, 8}},
  };
  return r[part];
}
constexpr int kPartCount[4] = {1, 2, 2, 4};

inline int alphabetSize(int c) {
  switch (c) {
    case ctxTxSize: return 3;
    case ctxLumaMode:
    case ctxChromaMode: return kNumIntraModes;
    case ctxMBMode: return kNumMBModes;
    case ctxRef: return kNumRefs;
    case ctxPart: return kNumPartModes;
    case ctxCBP: return kNumCBP;
    case ctxSign: return 2;
    case ctxEscClass: return kNumEscClasses;
    case ctxMVClassX:
    case ctxMVClassY: return kNumMVClasses;
    case ctxBypass: return 2;
    default: return kNumTokens;
  }
}

inline int tokenCtx(int plane, int txIdx, int band, int prevClass) {
  if (plane == kPlaneLuma) return ctxTokenBase + (txIdx * kNumBands + band) * kNumPrevClass + prevClass;
  return ctxTokenBase + kLumaTokenCtx + band * kNumPrevClass + prevClass;
}
inline int bandOf(int i) { return i == 0 ? 0 : i <= 2 ? 1 : i <= 8 ? 2 : i <= 20 ? 3 : 4; }
inline int classForMag(int mag) { return mag <= 0 ? 0 : (mag == 1 ? 1 : 2); }
inline uint8_t clampByte(int32_t v) { return v < 0 ? 0 : (v > 255 ? 255 : (uint8_t)v); }
inline int32_t wrapAdd(int32_t a, int32_t b) { return (int32_t)((uint32_t)a + (uint32_t)b); }
inline int32_t wrapMul(int32_t a, int32_t b) { return (int32_t)((uint32_t)a * (uint32_t)b); }
inline int txIndexOf(int n) { return n == 4 ? 0 : (n == 8 ? 1 : 2); }
inline int bitLen(uint64_t v) {
  int n = 0;
  while (v) {
    n++;
    v >>= 1;
  }
  return n;
}

// Scan orders, DCT matrices and quantizer steps, built once.
struct CodingTables {
  int scan[3][256];
  int32_t dct[3][256];
  int32_t quantStep[kMaxQP + 1];
  CodingTables() {
    for (int t = 0; t < 3; t++) {
      const int n = kLumaTx[t];
      int k = 0;
      // Diagonal zigzag: even diagonals run up-right, odd ones down-left.
      for (int d = 0; d < 2 * n - 1; d++) {
        if ((d & 1) == 0) {
          for (int y = d < n - 1 ? d : n - 1; y >= 0 && d - y < n; y--) scan[t][k++] = y * n + (d - y);
        } else {
          for (int x = d < n - 1 ? d : n - 1; x >= 0 && d - x < n; x--) scan[t][k++] = (d - x) * n + x;
        }
      }
      // Orthonormal DCT-II basis scaled by 2^13 and rounded half away from 0.
      for (int kk = 0; kk < n; kk++) {
        const double alpha = kk == 0 ? std::sqrt(1.0 / (double)n) : std::sqrt(2.0 / (double)n);
        for (int i = 0; i < n; i++) {
          const double c = alpha * std::cos((2.0 * (double)i + 1.0) * (double)kk * M_PI / (2.0 * (double)n));
          dct[t][kk * n + i] = (int32_t)std::round(c * 8192.0);
        }
      }
    }
    for (int qp = 0; qp <= kMaxQP; qp++) {
      double step = std::round(std::pow(2.0, (double)qp / 6.0));
      quantStep[qp] = (int32_t)(step < 1 ? 1 : step);
    }
  }
};
const CodingTables& codingTables();

struct Quant {
  int32_t dc = 1, ac = 1;
};
inline Quant quantFor(int qp) {
  if (qp < 0) qp = 0;
  if (qp > kMaxQP) qp = kMaxQP;
  Quant q;
  q.ac = codingTables().quantStep[qp];
  q.dc = qp >= 6 ? codingTables().quantStep[qp - 6] : q.ac;
  return q;
}

// Unsigned LEB128 with encoding/binary's 10-byte limit and overflow rule.
inline uint64_t getUvarint(const uint8_t* b, size_t len, int* n) {
  uint64_t x = 0;
  unsigned s = 0;
  for (size_t i = 0; i < len; i++) {
    if (i == 10) {
      *n = -(int)(i + 1);
      return 0;
    }
    const uint8_t c = b[i];
    if (c < 0x80) {
      if (i == 9 && c > 1) {
        *n = -(int)(i + 1);
        return 0;
      }
      *n = (int)i + 1;
      return x | (uint64_t)c << s;
    }
    x |= (uint64_t)(c & 0x7f) << s;
    s += 7;
  }
  *n = 0;
  return 0;
}
inline int64_t getVarint(const uint8_t* b, size_t len, int* n) {
  const uint64_t ux = getUvarint(b, len, n);
  int64_t x = (int64_t)(ux >> 1);
  if (ux & 1) x = ~x;
  return x;
}
inline void putUvarint(std::vector<uint8_t>& out, uint64_t v) {
  while (v >= 0x80) {
    out.push_back((uint8_t)(v | 0x80));
    v >>= 7;
  }
  out.push_back((uint8_t)v);
}
inline void putVarint(std::vector<uint8_t>& out, int64_t v) {
  uint64_t ux = (uint64_t)v << 1;
  if (v < 0) ux = ~ux;
  putUvarint(out, ux);
}

// Stream geometry with 64-byte aligned output strides (ebiv/geometry.go:22-49).
struct Geometry {
  int W = 0, H = 0, CW = 0, CH = 0, YStride = 0, CStride = 0;
  int mbCols = 0, mbRows = 0;
  static Geometry of(int w, int h) {
    Geometry g;
    g.W = w;
    g.H = h;
    g.CW = (w + 1) / 2;
    g.CH = (h + 1) / 2;
    g.YStride = (w + 63) & ~63;
    g.CStride = (g.CW + 63) & ~63;
    g.mbCols = (w + kMB - 1) / kMB;
    g.mbRows = (h + kMB - 1) / kMB;
    return g;
  }
  int padW() const { return mbCols * kMB; }
  int padH() const { return mbRows * kMB; }
  int padCW() const { return mbCols * kCMB; }
  int padCH() const { return mbRows * kCMB; }
  size_t packedSize() const { return (size_t)W * H + 2 * (size_t)CW * CH; }
};

// Tile partition of the macroblock grid (ebiv/frame.go:87-111,170-177).
struct TileGrid {
  int cols = 1, rows = 1;
  std::vector<int> colEdges, rowEdges;
  TileGrid() = default;
  TileGrid(int mbCols, int mbRows, int c, int r) {
    if (c < 1) c = 1;
    if (r < 1) r = 1;
    cols = c < mbCols ? c : mbCols;
    rows = r < mbRows ? r : mbRows;
    for (int i = 0; i <= cols; i++) colEdges.push_back((int)((int64_t)mbCols * i / cols));
    for (int i = 0; i <= rows; i++) rowEdges.push_back((int)((int64_t)mbRows * i / rows));
  }
  int count() const { return cols * rows; }
  void bounds(int idx, int* x0, int* x1, int* y0, int* y1) const {
    const int tc = idx % cols, tr = idx / cols;
    *x0 = colEdges[tc];
    *x1 = colEdges[tc + 1];
    *y0 = rowEdges[tr];
    *y1 = rowEdges[tr + 1];
  }
};

inline uint16_t rd16(const uint8_t* p) { return (uint16_t)(p[0] | p[1] << 8); }
inline uint32_t rd32(const uint8_t* p) { return (uint32_t)p[0] | (uint32_t)p[1] << 8 | (uint32_t)p[2] << 16 | (uint32_t)p[3] << 24; }
inline uint64_t rd64(const uint8_t* p) { return (uint64_t)rd32(p) | (uint64_t)rd32(p + 4) << 32; }
inline void wr16(uint8_t* p, uint16_t v) {
  p[0] = (uint8_t)v;
  p[1] = (uint8_t)(v >> 8);
}
inline void wr32(uint8_t* p, uint32_t v) {
  for (int i = 0; i < 4; i++) p[i] = (uint8_t)(v >> (8 * i));
}
inline void wr64(uint8_t* p, uint64_t v) {
  for (int i = 0; i < 8; i++) p[i] = (uint8_t)(v >> (8 * i));
}
uint32_t crc32IEEE(const uint8_t* data, size_t n);

}  // namespace ebiv
