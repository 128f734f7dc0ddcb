// TEST INFRASTRUCTURE — CPU oracle for the EBIV decode path.
//
// A line-faithful restatement of govid's pure-Go EBIV decoder, used only by
// the tests, the smoke check and the benchmark's CPU-baseline leg as the
// checker.  Every function cites the reference function it follows
// (paths relative to the govid project root).  Go's integer semantics are kept
// exactly: truncating division, arithmetic right shift, modular int32 wrap
// where Go converts int64->int32 or adds int32 values, int16 motion vectors.
//
// Where the reference would hit a Go runtime panic on hostile input (slice
// bounds on lengths that overflow int, rANS tables whose uint32 frequency sum
// wraps to 4096), this restatement reports ErrCorrupt instead.
#include "ebiv_oracle.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <functional>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

namespace eo {

// ---- ebiv/model.go:20-152 --------------------------------------------------
constexpr int kScaleBits = 12;
constexpr uint32_t kM = 1u << kScaleBits;
constexpr uint32_t kLower = 1u << 23;
constexpr int kStates = 4;
constexpr int mbSize = 16, chromaMB = 8, dcPred = 128, maxLevels = 256;
constexpr int lumaTx[3] = {4, 8, 16};
enum { modeDC, modeV, modeH, modeTM, modeD45, modeD27, modeD23, modeD135, modeD117, modeD113, numIntraModes };
enum { mbSkip, mbInter, mbIntra, numMBModes };
enum { refLast, refGolden, numRefs };
enum { cbpLuma = 1, cbpCb = 2, cbpCr = 4, numCBP = 8 };
enum { partWhole, part16x8, part8x16, part8x8, numPartModes };
enum { tZero, tOne, tTwo, tThree, tFour, tEscape, tEOB, numTokens };
constexpr int numMVClasses = 16, numEscClasses = 16;
enum {
  ctxTxSize, ctxLumaMode, ctxChromaMode, ctxMBMode, ctxRef, ctxPart, ctxCBP, ctxSign,
  ctxEscClass, ctxMVClassX, ctxMVClassY, ctxBypass, ctxTokenBase
};
constexpr int numBands = 5, numPrevClass = 3;
constexpr int lumaTokenCtx = 3 * numBands * numPrevClass;
constexpr int chromaTokenCtx = numBands * numPrevClass;
constexpr int numContexts = ctxTokenBase + lumaTokenCtx + chromaTokenCtx;  // 72
constexpr int planeLuma = 0, planeChroma = 1;
constexpr int sdhMinSpan = 4;  // ebiv/residual.go:21
constexpr int mvClampRange = 4096;  // ebiv/motioncomp.go:19
constexpr int maxQP = 63;
constexpr int64_t maxDecodePixels = 8192LL * 4320LL;  // ebiv/codec.go:123

// partRects — ebiv/model.go:91-96
struct Rect4 { int x, y, w, h; };
static const Rect4 kPartRects[4][4] = {
    {{0, 0, 16, 16}},
    {{0, 0, 16, 8}, {0, 8, 16, 8}},
    {{0, 0, 8, 16}, {8, 0, 8, 16}},
    {{0, 0, 8, 8}, {8, 0, 8, 8}, {0, 8, 8, 8}, {8, 8, 8, 8}},
};
static const int kPartCount[4] = {1, 2, 2, 4};

// alphabetSizes — ebiv/model.go:195-213
static int alphabetSize(int c) {
  switch (c) {
    case ctxTxSize: return 3;
    case ctxLumaMode: case ctxChromaMode: return numIntraModes;
    case ctxMBMode: return numMBModes;
    case ctxRef: return numRefs;
    case ctxPart: return numPartModes;
    case ctxCBP: return numCBP;
    case ctxSign: return 2;
    case ctxEscClass: return numEscClasses;
    case ctxMVClassX: case ctxMVClassY: return numMVClasses;
    case ctxBypass: return 2;
    default: return numTokens;
  }
}

// tokenCtx — ebiv/model.go:156-161
static inline int tokenCtx(int plane, int txIdx, int band, int prevClass) {
  if (plane == planeLuma) return ctxTokenBase + (txIdx * numBands + band) * numPrevClass + prevClass;
  return ctxTokenBase + lumaTokenCtx + band * numPrevClass + prevClass;
}
// bandOf — ebiv/model.go:165-178
static inline int bandOf(int i) {
  if (i == 0) return 0;
  if (i <= 2) return 1;
  if (i <= 8) return 2;
  if (i <= 20) return 3;
  return 4;
}
// classForMag — ebiv/model.go:182-191
static inline int classForMag(int mag) { return mag <= 0 ? 0 : (mag == 1 ? 1 : 2); }
// clampByte — ebiv/model.go:222-230
static inline uint8_t clampByte(int32_t v) { return v < 0 ? 0 : (v > 255 ? 255 : (uint8_t)v); }
// Go int32 addition wraps modulo 2^32.
static inline int32_t add32(int32_t a, int32_t b) { return (int32_t)((uint32_t)a + (uint32_t)b); }
static inline int32_t mul32(int32_t a, int32_t b) { return (int32_t)((uint32_t)a * (uint32_t)b); }

// ---- scan tables: ebiv/scan.go:17-35 ---------------------------------------
struct Tables {
  int scan[3][256];
  int32_t dct[3][256];
  int32_t quantStep[maxQP + 1];
  Tables() {
    for (int t = 0; t < 3; t++) {
      int n = lumaTx[t], k = 0;
      for (int d = 0; d < 2 * n - 1; d++) {
        if (d % 2 == 0) {
          for (int y = std::min(d, n - 1); y >= 0 && d - y < n; y--) scan[t][k++] = y * n + (d - y);
        } else {
          for (int x = std::min(d, n - 1); x >= 0 && d - x < n; x--) scan[t][k++] = (d - x) * n + x;
        }
      }
      // buildDCTMatrix — ebiv/transform.go:27-40
      for (int kk = 0; kk < n; kk++) {
        double alpha = std::sqrt(2.0 / (double)n);
        if (kk == 0) alpha = std::sqrt(1.0 / (double)n);
        for (int i = 0; i < n; i++) {
          double c = alpha * std::cos((2.0 * (double)i + 1.0) * (double)kk * M_PI / (2.0 * (double)n));
          dct[t][kk * n + i] = (int32_t)std::round(c * (double)(1 << 13));
        }
      }
    }
    // quantStep — ebiv/quant.go:19-29
    for (int qp = 0; qp <= maxQP; qp++) {
      double step = std::round(std::pow(2.0, (double)qp / 6.0));
      if (step < 1) step = 1;
      quantStep[qp] = (int32_t)step;
    }
  }
};
static const Tables& T() {
  static Tables t;
  return t;
}
static inline int txIndexOf(int n) { return n == 4 ? 0 : (n == 8 ? 1 : 2); }

// ---- varints (encoding/binary Uvarint / Varint semantics) ------------------
static inline uint64_t uvarint(const uint8_t* b, size_t len, int* n) {
  uint64_t x = 0;
  unsigned s = 0;
  for (size_t i = 0; i < len; i++) {
    if (i == 10) { *n = -(int)(i + 1); return 0; }
    uint8_t c = b[i];
    if (c < 0x80) {
      if (i == 9 && c > 1) { *n = -(int)(i + 1); return 0; }
      *n = (int)i + 1;
      return x | (uint64_t)c << s;
    }
    x |= (uint64_t)(c & 0x7f) << s;
    s += 7;
  }
  *n = 0;
  return 0;
}
static inline int64_t varint(const uint8_t* b, size_t len, int* n) {
  uint64_t ux = uvarint(b, len, n);
  int64_t x = (int64_t)(ux >> 1);
  if (ux & 1) x = ~x;
  return x;
}

// ---- rANS tables: ebiv/rans.go:36-148 --------------------------------------
struct RansTable {
  uint32_t start[16];
  uint32_t freq[16];
  int n = 0;
  bool used = false;
  uint16_t slot2sym[kM];
};

// buildTableInto (decode form) — ebiv/rans.go:120-148.  Returns false when the
// reference would panic filling slot2sym (frequency prefix sum past ransM).
static bool buildTableInto(RansTable& t, const uint32_t* freq, int n) {
  t.used = false;
  t.n = n;
  uint32_t cum = 0;
  bool wrapped = false;
  for (int s = 0; s < n; s++) {
    t.start[s] = cum;
    t.freq[s] = freq[s];
    uint64_t next = (uint64_t)cum + freq[s];
    if (next > kM) wrapped = true;
    cum += freq[s];
  }
  if (cum != kM) return true;  // unused context
  if (wrapped) return false;   // Go: index out of range in the slot2sym fill
  t.used = true;
  for (int s = 0; s < n; s++)
    for (uint32_t k = 0; k < freq[s]; k++) t.slot2sym[t.start[s] + k] = (uint16_t)s;
  return true;
}

// prevFreqs entry with Go slice semantics: length plus a retained backing
// array, so a key frame's wipe (len 0) keeps the old values for growFreqs.
struct PrevFreq {
  int len = 0;
  bool alloc = false;
  uint32_t v[16] = {0};
};

// ---- rANS decoder: ebiv/rans.go:222-310 ------------------------------------
struct RansDecoder {
  const uint8_t* buf = nullptr;
  int64_t pos = 0;
  const RansTable* tables = nullptr;
  uint32_t state[kStates] = {0};
  uint64_t counter = 0;
  int err = EO_OK;

  int reset(const uint8_t* b, int64_t len, const RansTable* t) {
    if (len < kStates * 4) return EO_ERR_CORRUPT;
    buf = b;
    pos = len;
    tables = t;
    counter = 0;
    err = EO_OK;
    for (int i = kStates - 1; i >= 0; i--) state[i] = pop32();
    return EO_OK;
  }
  uint8_t pop() { return buf[--pos]; }
  uint32_t pop32() {
    uint32_t a = pop(), b = pop(), c = pop(), e = pop();
    return a << 24 | b << 16 | c << 8 | e;
  }
  void fail(int e) {
    if (err == EO_OK) err = e;
  }
  int decode(int ctx) {
    if (err != EO_OK) return 0;
    const RansTable& t = tables[ctx];
    if (!t.used) {
      fail(EO_ERR_CORRUPT);
      return 0;
    }
    int i = (int)(counter & (kStates - 1));
    counter++;
    uint32_t x = state[i];
    uint32_t slot = x & (kM - 1);
    int sym = t.slot2sym[slot];
    x = t.freq[sym] * (x >> kScaleBits) + slot - t.start[sym];
    if (x < kLower) {
      int64_t p = pos;
      while (x < kLower) {
        if (p == 0) {
          pos = 0;
          fail(EO_ERR_CORRUPT);
          return 0;
        }
        p--;
        x = (x << 8) | (uint32_t)buf[p];
      }
      pos = p;
    }
    state[i] = x;
    return sym;
  }
  // getRawBits — ebiv/mv.go:75-81
  uint32_t getRawBits(int n) {
    uint32_t v = 0;
    for (int i = 0; i < n; i++) v = v << 1 | (uint32_t)decode(ctxBypass);
    return v;
  }
  // getClassValue — ebiv/mv.go:95-108
  uint32_t getClassValue(int classCtx, int maxClass) {
    int cls = decode(classCtx);
    if (cls < 0 || cls >= maxClass) {
      fail(EO_ERR_CORRUPT);
      return 0;
    }
    if (cls == 0) return 0;
    if (cls == 1) return 1;
    return (1u << (cls - 1)) | getRawBits(cls - 1);
  }
  // getMVComponent / zigzagDecode — ebiv/mv.go:116-118, motioncomp.go:410-412
  int getMVComponent(int classCtx) {
    uint32_t u = getClassValue(classCtx, numMVClasses);
    return (int)(u >> 1) ^ -(int)(u & 1);
  }
  int getEscapeValue() { return (int)getClassValue(ctxEscClass, numEscClasses); }
};

// parseTablesInto — ebiv/rans.go:396-471
static int parseTablesInto(RansTable* tables, PrevFreq* prev, const uint8_t* b, size_t blen,
                           bool key, size_t* consumed) {
  if (key)
    for (int c = 0; c < numContexts; c++) prev[c].len = 0;
  size_t pos = 0;
  for (int c = 0; c < numContexts; c++) {
    if (pos >= blen) return EO_ERR_CORRUPT;
    uint8_t mode = b[pos++];
    if (c == ctxBypass && mode != 0) return EO_ERR_CORRUPT;
    int asz = alphabetSize(c);
    bool haveRef = prev[c].len == asz;
    switch (mode) {
      case 0:  // tblUnused
        tables[c].used = false;
        break;
      case 1:  // tblSame
        if (key || !haveRef) return EO_ERR_CORRUPT;
        if (!buildTableInto(tables[c], prev[c].v, asz)) return EO_ERR_CORRUPT;
        if (!tables[c].used) return EO_ERR_CORRUPT;
        break;
      case 2: {  // tblFull — growFreqs keeps the backing array
        PrevFreq& p = prev[c];
        if (!p.alloc) {
          std::memset(p.v, 0, sizeof(p.v));
          p.alloc = true;
        }
        p.len = asz;
        for (int s = 0; s < asz; s++) {
          int n;
          uint64_t v = uvarint(b + pos, blen - pos, &n);
          if (n <= 0) return EO_ERR_CORRUPT;
          pos += (size_t)n;
          p.v[s] = (uint32_t)v;
        }
        if (!buildTableInto(tables[c], p.v, asz)) return EO_ERR_CORRUPT;
        if (!tables[c].used) return EO_ERR_CORRUPT;
        break;
      }
      case 3: {  // tblDelta
        if (key || !haveRef) return EO_ERR_CORRUPT;
        PrevFreq& p = prev[c];
        for (int s = 0; s < asz; s++) {
          int n;
          int64_t v = varint(b + pos, blen - pos, &n);
          if (n <= 0) return EO_ERR_CORRUPT;
          pos += (size_t)n;
          int64_t nv = (int64_t)p.v[s] + v;
          if (nv < 0 || nv > (int64_t)kM) return EO_ERR_CORRUPT;
          p.v[s] = (uint32_t)nv;
        }
        if (!buildTableInto(tables[c], p.v, asz)) return EO_ERR_CORRUPT;
        if (!tables[c].used) return EO_ERR_CORRUPT;
        break;
      }
      default:
        return EO_ERR_CORRUPT;
    }
  }
  // installBypass — ebiv/rans.go:317-322
  static const uint32_t bypass[2] = {kM / 2, kM / 2};
  buildTableInto(tables[ctxBypass], bypass, 2);
  *consumed = pos;
  return EO_OK;
}

// ---- planes: ebiv/predict.go:15-24, ebiv/frame.go:19-37 --------------------
struct PlaneView {
  uint8_t* data = nullptr;
  int stride = 0, w = 0, h = 0;
  inline uint8_t at(int x, int y) const { return data[(size_t)y * stride + x]; }
};
struct FrameBuf {
  std::vector<uint8_t> ybuf, cbbuf, crbuf;
  PlaneView y, cb, cr;
  int mbCols = 0, mbRows = 0;
  void init(int W, int H) {
    mbCols = (W + mbSize - 1) / mbSize;
    mbRows = (H + mbSize - 1) / mbSize;
    int pw = mbCols * mbSize, ph = mbRows * mbSize, cw = mbCols * chromaMB, ch = mbRows * chromaMB;
    ybuf.assign((size_t)pw * ph, 0);
    cbbuf.assign((size_t)cw * ch, 0);
    crbuf.assign((size_t)cw * ch, 0);
    y = {ybuf.data(), pw, pw, ph};
    cb = {cbbuf.data(), cw, cw, ch};
    cr = {crbuf.data(), cw, cw, ch};
  }
  void copyFrom(const FrameBuf& s) {  // ebiv/frame.go:42-46
    ybuf = s.ybuf;
    cbbuf = s.cbbuf;
    crbuf = s.crbuf;
    y.data = ybuf.data();
    cb.data = cbbuf.data();
    cr.data = crbuf.data();
  }
};

// ---- geometry: ebiv/geometry.go:22-49 --------------------------------------
struct Geometry {
  int W = 0, H = 0, CW = 0, CH = 0, YStride = 0, CStride = 0;
};
static Geometry geometryFor(int w, int h) {
  Geometry g;
  g.W = w;
  g.H = h;
  g.CW = (w + 1) / 2;
  g.CH = (h + 1) / 2;
  g.YStride = (w + 63) & ~63;
  g.CStride = (g.CW + 63) & ~63;
  return g;
}
struct Image {
  std::vector<uint8_t> Y, Cb, Cr;
};

// ---- tile grid: ebiv/frame.go:80-177 ---------------------------------------
struct TileBounds {
  int mbX0, mbX1, mbY0, mbY1;
};
struct TileGrid {
  int cols = 1, rows = 1;
  std::vector<int> colEdges, rowEdges;
  TileGrid(int mbCols, int mbRows, int c, int r) {
    if (c < 1) c = 1;
    if (r < 1) r = 1;
    cols = std::min(c, mbCols);
    rows = std::min(r, mbRows);
    for (int i = 0; i <= cols; i++) colEdges.push_back((int)((int64_t)mbCols * i / cols));
    for (int i = 0; i <= rows; i++) rowEdges.push_back((int)((int64_t)mbRows * i / rows));
  }
  int count() const { return cols * rows; }
  TileBounds bounds(int idx) const {
    int tc = idx % cols, tr = idx / cols;
    return {colEdges[tc], colEdges[tc + 1], rowEdges[tr], rowEdges[tr + 1]};
  }
};

// ---- transform: ebiv/transform.go:129-194 ----------------------------------
static void inverseDCT(const int32_t* src, int32_t* dst, int n) {
  int maxR = -1, maxC = -1;
  for (int r = 0; r < n; r++)
    for (int c = 0; c < n; c++)
      if (src[r * n + c] != 0) {
        if (r > maxR) maxR = r;
        if (c > maxC) maxC = c;
      }
  if (maxR < 0) {
    for (int i = 0; i < n * n; i++) dst[i] = 0;
    return;
  }
  const int64_t round = 1LL << 12;
  const int32_t* c = T().dct[txIndexOf(n)];
  if (maxR == 0 && maxC == 0) {
    int64_t d0 = c[0];
    int64_t col = (d0 * (int64_t)src[0] + round) >> 13;
    int32_t val = (int32_t)((d0 * col + round) >> 13);
    for (int i = 0; i < n * n; i++) dst[i] = val;
    return;
  }
  int32_t tmp[maxLevels];
  for (int i = 0; i < n; i++)
    for (int l = 0; l <= maxC; l++) {
      int64_t acc = 0;
      for (int k = 0; k <= maxR; k++) acc += (int64_t)c[k * n + i] * (int64_t)src[k * n + l];
      tmp[i * n + l] = (int32_t)((acc + round) >> 13);
    }
  for (int i = 0; i < n; i++)
    for (int m = 0; m < n; m++) {
      int64_t acc = 0;
      for (int l = 0; l <= maxC; l++) acc += (int64_t)c[l * n + m] * (int64_t)tmp[i * n + l];
      dst[i * n + m] = (int32_t)((acc + round) >> 13);
    }
}

// ---- quantizer: ebiv/quant.go:38-80 ----------------------------------------
struct Quantizer {
  int32_t dc = 1, ac = 1;
};
static Quantizer newQuantizer(int qp) {
  if (qp < 0) qp = 0;
  if (qp > maxQP) qp = maxQP;
  Quantizer q;
  q.ac = T().quantStep[qp];
  q.dc = q.ac;
  if (qp >= 6) q.dc = T().quantStep[qp - 6];
  return q;
}

// ---- residual: ebiv/residual.go:79-126 -------------------------------------
static void decodeBlock(RansDecoder& d, int plane, int txIdx, int32_t* levels, int n) {
  const int* scan = T().scan[txIndexOf(n)];
  int total = n * n;
  int first = -1, last = -1;
  int32_t sumAbs = 0;
  int prevClass = 0;
  for (int i = 0; i < total; i++) {
    int ctx = tokenCtx(plane, txIdx, bandOf(i), prevClass);
    int t = d.decode(ctx);
    if (t == tEOB) break;
    if (t == tZero) {
      levels[scan[i]] = 0;
      prevClass = 0;
      continue;
    }
    int mag;
    if (t == tEscape) {
      mag = 5 + d.getEscapeValue();
      prevClass = 2;
    } else {
      mag = t - tZero;
      prevClass = classForMag(mag);
    }
    sumAbs = add32(sumAbs, (int32_t)mag);
    if (first < 0) {
      first = i;
    } else if (d.decode(ctxSign) == 1) {
      mag = -mag;
    }
    levels[scan[i]] = (int32_t)mag;
    last = i;
  }
  if (first < 0) return;
  bool neg;
  if (last - first >= sdhMinSpan) {
    neg = (sumAbs & 1) == 1;
  } else {
    neg = d.decode(ctxSign) == 1;
  }
  if (neg) levels[scan[first]] = -levels[scan[first]];
}

// ---- intra prediction: ebiv/predict.go:30-219 -------------------------------
struct AngMode {
  int angle, invAngle;
  bool vertical;
};
static const AngMode kAng[numIntraModes] = {
    {0, 0, false}, {0, 0, false}, {0, 0, false}, {0, 0, false},
    {32, 0, true}, {13, 0, true}, {-13, -630, true},
    {32, 0, false}, {13, 0, false}, {-13, -630, false},
};

static bool aboveRightAvailable(int x0, int y0, int n, int tileTopPx, int tileRightPx, int mbTopPx,
                                int mbRightPx) {
  if (y0 <= tileTopPx || x0 + 2 * n > tileRightPx) return false;
  if (y0 == mbTopPx) return true;
  return x0 + 2 * n <= mbRightPx;
}

static void substituteRefs(int32_t* ref, const bool* avail, int len) {
  int first = -1;
  for (int i = 0; i < len; i++)
    if (avail[i]) {
      first = i;
      break;
    }
  if (first < 0) {
    for (int i = 0; i < len; i++) ref[i] = dcPred;
    return;
  }
  for (int i = 0; i < first; i++) ref[i] = ref[first];
  for (int i = first + 1; i < len; i++)
    if (!avail[i]) ref[i] = ref[i - 1];
}

static void angularPredict(const int32_t* ref, int corner, int n, const AngMode& m, int32_t* pred) {
  int32_t ext[3 * mbSize + 2] = {0};
  int off = n;
  if (m.vertical) {
    for (int k = 0; k <= 2 * n; k++) ext[off + k] = ref[corner + k];
  } else {
    for (int k = 0; k <= 2 * n; k++) ext[off + k] = ref[corner - k];
  }
  if (m.angle < 0) {
    int low = (n * m.angle) >> 5;
    for (int x = -1; x >= low; x--) {
      int idx = (x * m.invAngle + 128) >> 8;
      ext[off + x] = m.vertical ? ref[corner - idx] : ref[corner + idx];
    }
  }
  for (int a = 0; a < n; a++) {
    int pos = (a + 1) * m.angle;
    int idx = pos >> 5;
    int fact = pos & 31;
    for (int b = 0; b < n; b++) {
      int32_t s0 = ext[off + b + idx + 1];
      int32_t s1 = ext[off + b + idx + 2];
      int32_t v = ((32 - fact) * s0 + fact * s1 + 16) >> 5;
      if (m.vertical)
        pred[a * n + b] = v;
      else
        pred[b * n + a] = v;
    }
  }
}

static void predictIntra(const PlaneView& p, int x0, int y0, int n, int mode, bool avAbove,
                         bool avLeft, bool avAboveRight, int32_t* pred) {
  int32_t ref[4 * mbSize + 1] = {0};
  bool avail[4 * mbSize + 1] = {false};
  int corner = 2 * n;
  for (int i = 0; i < 2 * n; i++) {
    int row = 2 * n - 1 - i;
    if (avLeft && row < n) {
      ref[i] = p.at(x0 - 1, y0 + row);
      avail[i] = true;
    }
  }
  if (avAbove && avLeft) {
    ref[corner] = p.at(x0 - 1, y0 - 1);
    avail[corner] = true;
  }
  for (int j = 0; j < 2 * n; j++) {
    if (avAbove && (j < n || avAboveRight)) {
      ref[corner + 1 + j] = p.at(x0 + j, y0 - 1);
      avail[corner + 1 + j] = true;
    }
  }
  substituteRefs(ref, avail, 4 * n + 1);
  auto topOf = [&](int x) { return ref[corner + 1 + x]; };
  auto leftOf = [&](int y) { return ref[corner - 1 - y]; };
  switch (mode) {
    case modeV:
      for (int r = 0; r < n; r++)
        for (int c = 0; c < n; c++) pred[r * n + c] = topOf(c);
      break;
    case modeH:
      for (int r = 0; r < n; r++) {
        int32_t v = leftOf(r);
        for (int c = 0; c < n; c++) pred[r * n + c] = v;
      }
      break;
    case modeTM: {
      int32_t crn = ref[corner];
      for (int r = 0; r < n; r++) {
        int32_t l = leftOf(r);
        for (int c = 0; c < n; c++) pred[r * n + c] = clampByte(topOf(c) + l - crn);
      }
      break;
    }
    case modeDC: {
      int32_t sum = 0;
      for (int i = 0; i < n; i++) sum += topOf(i) + leftOf(i);
      int32_t dc = (sum + n) / (2 * n);
      for (int i = 0; i < n * n; i++) pred[i] = dc;
      break;
    }
    default:
      angularPredict(ref, corner, n, kAng[mode], pred);
  }
}

// Test statistic (no counterpart in the reference): intra residual samples
// outside the 16-bit range reconstructed so far, so a test can show that its
// corpus reaches the GPU decoder's wide-residual path.
static std::atomic<long> gWideResiduals{0};

// reconstruct — ebiv/predict.go:209-219
static void reconstruct(const PlaneView& p, int x0, int y0, int n, const int32_t* pred,
                        const int32_t* residual) {
  long wide = 0;
  for (int r = 0; r < n; r++) {
    uint8_t* dst = p.data + (size_t)(y0 + r) * p.stride + x0;
    for (int c = 0; c < n; c++) {
      const int32_t v = residual[r * n + c];
      wide += (v < -32768 || v > 32767) ? 1 : 0;
      dst[c] = clampByte(add32(pred[r * n + c], v));
    }
  }
  if (wide) gWideResiduals += wide;
}

// ---- motion compensation: ebiv/motioncomp.go -------------------------------
struct MV {
  int16_t x = 0, y = 0;
};
static const int32_t kLumaTaps[4][4] = {{0, 64, 0, 0}, {-6, 55, 18, -3}, {-8, 40, 40, -8}, {-3, 18, 55, -6}};
static inline int clampCoord(int v, int hi) { return v < 0 ? 0 : (v >= hi ? hi - 1 : v); }

// lumaSubpel — ebiv/motioncomp.go:49-78
static int32_t lumaSubpel(const PlaneView& ref, int px, int py, int fx, int fy) {
  auto g = [&](int x, int y) -> int32_t { return ref.at(clampCoord(x, ref.w), clampCoord(y, ref.h)); };
  if (fx == 0 && fy == 0) return g(px, py);
  if (fy == 0) {
    const int32_t* t = kLumaTaps[fx];
    int32_t v = t[0] * g(px - 1, py) + t[1] * g(px, py) + t[2] * g(px + 1, py) + t[3] * g(px + 2, py);
    return clampByte((v + 32) >> 6);
  }
  if (fx == 0) {
    const int32_t* t = kLumaTaps[fy];
    int32_t v = t[0] * g(px, py - 1) + t[1] * g(px, py) + t[2] * g(px, py + 1) + t[3] * g(px, py + 2);
    return clampByte((v + 32) >> 6);
  }
  const int32_t* tx = kLumaTaps[fx];
  int32_t h[4];
  for (int k = 0; k < 4; k++) {
    int yy = py - 1 + k;
    h[k] = tx[0] * g(px - 1, yy) + tx[1] * g(px, yy) + tx[2] * g(px + 1, yy) + tx[3] * g(px + 2, yy);
  }
  const int32_t* ty = kLumaTaps[fy];
  int32_t v = ty[0] * h[0] + ty[1] * h[1] + ty[2] * h[2] + ty[3] * h[3];
  return clampByte((v + (1 << 11)) >> 12);
}

// chromaSubpel — ebiv/motioncomp.go:82-97
static int32_t chromaSubpel(const PlaneView& ref, int px, int py, int fx, int fy) {
  auto g = [&](int x, int y) -> int32_t { return ref.at(clampCoord(x, ref.w), clampCoord(y, ref.h)); };
  if (fx == 0 && fy == 0) return g(px, py);
  int32_t a = g(px, py), b = g(px + 1, py), c = g(px, py + 1), d = g(px + 1, py + 1);
  int32_t v = (8 - fx) * (8 - fy) * a + fx * (8 - fy) * b + (8 - fx) * fy * c + fx * fy * d;
  return (v + 32) >> 6;
}

static bool interiorLuma(const PlaneView& ref, int srcX, int srcY, int fx, int fy, int pw, int ph) {
  if (fx == 0 && fy == 0) return srcX >= 0 && srcY >= 0 && srcX + pw <= ref.w && srcY + ph <= ref.h;
  return srcX - 1 >= 0 && srcY - 1 >= 0 && srcX + pw + 2 <= ref.w && srcY + ph + 2 <= ref.h;
}

// mcLuma + mcLumaInterior — ebiv/motioncomp.go:112-185.  The interior path
// computes the same filter without clamped coordinates.
static void mcLuma(const PlaneView& ref, int srcX, int srcY, int fx, int fy, int pw, int ph,
                   int32_t* out, int dstX, int dstY, int dstStride) {
  if (!interiorLuma(ref, srcX, srcY, fx, fy, pw, ph)) {
    for (int r = 0; r < ph; r++)
      for (int c = 0; c < pw; c++)
        out[(dstY + r) * dstStride + dstX + c] = lumaSubpel(ref, srcX + c, srcY + r, fx, fy);
    return;
  }
  const uint8_t* data = ref.data;
  int stride = ref.stride;
  for (int r = 0; r < ph; r++) {
    int32_t* dst = out + (dstY + r) * dstStride + dstX;
    for (int c = 0; c < pw; c++) {
      size_t b = (size_t)(srcY + r) * stride + srcX + c;
      int32_t v;
      if (fx == 0 && fy == 0) {
        v = data[b];
      } else if (fy == 0) {
        const int32_t* t = kLumaTaps[fx];
        v = clampByte((t[0] * data[b - 1] + t[1] * data[b] + t[2] * data[b + 1] + t[3] * data[b + 2] + 32) >> 6);
      } else if (fx == 0) {
        const int32_t* t = kLumaTaps[fy];
        v = clampByte((t[0] * data[b - stride] + t[1] * data[b] + t[2] * data[b + stride] +
                       t[3] * data[b + 2 * stride] + 32) >> 6);
      } else {
        const int32_t *tx = kLumaTaps[fx], *ty = kLumaTaps[fy];
        int32_t h[4];
        for (int k = 0; k < 4; k++) {
          size_t bb = (size_t)(srcY + r - 1 + k) * stride + srcX + c;
          h[k] = tx[0] * data[bb - 1] + tx[1] * data[bb] + tx[2] * data[bb + 1] + tx[3] * data[bb + 2];
        }
        v = clampByte((ty[0] * h[0] + ty[1] * h[1] + ty[2] * h[2] + ty[3] * h[3] + (1 << 11)) >> 12);
      }
      dst[c] = v;
    }
  }
}

// mcChroma — ebiv/motioncomp.go:214-256
static void mcChroma(const PlaneView& ref, int srcX, int srcY, int fx, int fy, int pw, int ph,
                     int32_t* out, int dstX, int dstY, int dstStride) {
  bool interior = srcX >= 0 && srcY >= 0 && srcX + pw + 1 <= ref.w && srcY + ph + 1 <= ref.h;
  if (fx == 0 && fy == 0) interior = srcX >= 0 && srcY >= 0 && srcX + pw <= ref.w && srcY + ph <= ref.h;
  if (!interior) {
    for (int r = 0; r < ph; r++)
      for (int c = 0; c < pw; c++)
        out[(dstY + r) * dstStride + dstX + c] = chromaSubpel(ref, srcX + c, srcY + r, fx, fy);
    return;
  }
  const uint8_t* data = ref.data;
  int stride = ref.stride;
  int32_t w00 = (8 - fx) * (8 - fy), w01 = fx * (8 - fy), w10 = (8 - fx) * fy, w11 = fx * fy;
  for (int r = 0; r < ph; r++)
    for (int c = 0; c < pw; c++) {
      size_t b = (size_t)(srcY + r) * stride + srcX + c;
      int32_t v;
      if (fx == 0 && fy == 0)
        v = data[b];
      else
        v = (w00 * data[b] + w01 * data[b + 1] + w10 * data[b + stride] + w11 * data[b + stride + 1] + 32) >> 6;
      out[(dstY + r) * dstStride + dstX + c] = v;
    }
}

// mcLumaByte / mcChromaByte — ebiv/motioncomp.go:265-368: the int32 path
// followed by a clamped byte store (the reference states they are identical).
static void mcLumaByte(const PlaneView& ref, int srcX, int srcY, int fx, int fy, int pw, int ph,
                       const PlaneView& dst, int dstX, int dstY) {
  int32_t tmp[256];
  mcLuma(ref, srcX, srcY, fx, fy, pw, ph, tmp, 0, 0, pw);
  for (int r = 0; r < ph; r++)
    for (int c = 0; c < pw; c++) dst.data[(size_t)(dstY + r) * dst.stride + dstX + c] = clampByte(tmp[r * pw + c]);
}
static void mcChromaByte(const PlaneView& ref, int srcX, int srcY, int fx, int fy, int pw, int ph,
                         const PlaneView& dst, int dstX, int dstY) {
  int32_t tmp[64];
  mcChroma(ref, srcX, srcY, fx, fy, pw, ph, tmp, 0, 0, pw);
  for (int r = 0; r < ph; r++)
    for (int c = 0; c < pw; c++) dst.data[(size_t)(dstY + r) * dst.stride + dstX + c] = clampByte(tmp[r * pw + c]);
}

static inline int16_t clampMV(int v) {  // ebiv/motioncomp.go:394-402
  if (v < -mvClampRange) v = -mvClampRange;
  if (v > mvClampRange) v = mvClampRange;
  return (int16_t)v;
}

// ---- MV prediction: ebiv/mv.go:21-65 ---------------------------------------
static inline int16_t median3(int16_t a, int16_t b, int16_t c) {
  if (a > b) std::swap(a, b);
  if (b > c) b = c;
  if (a > b) b = a;
  return b;
}
static MV predictMV(const MV* mv, int stride, int mbx, int mby, const TileBounds& b) {
  MV a, bv, c;
  bool aOK = mbx > b.mbX0, bOK = mby > b.mbY0, cOK = false;
  if (aOK) a = mv[mby * stride + mbx - 1];
  if (bOK) {
    bv = mv[(mby - 1) * stride + mbx];
    if (mbx + 1 < b.mbX1) {
      c = mv[(mby - 1) * stride + mbx + 1];
      cOK = true;
    } else if (aOK) {
      c = mv[(mby - 1) * stride + mbx - 1];
      cOK = true;
    }
  }
  if (!aOK && !bOK && !cOK) return MV{};
  if (aOK && !bOK && !cOK) return a;
  if (!aOK && bOK && !cOK) return bv;
  MV r;
  r.x = median3(a.x, bv.x, c.x);
  r.y = median3(a.y, bv.y, c.y);
  return r;
}

// ---- tile decoder: ebiv/decode_intra.go, ebiv/decode_inter.go --------------
struct BlockScratch {
  int32_t pred[maxLevels], levels[maxLevels], coeffs[maxLevels], recon[maxLevels];
};
struct TileDecoder {
  RansDecoder dec;
  FrameBuf* rec = nullptr;
  FrameBuf* ref = nullptr;
  FrameBuf* golden = nullptr;
  Quantizer q;
  bool inter = false;
  MV* mv = nullptr;
  int mvStride = 0;
  BlockScratch sc;

  void dequantize(int n) {  // ebiv/quant.go:72-80
    for (int i = 0; i < n * n; i++) sc.coeffs[i] = mul32(sc.levels[i], i == 0 ? q.dc : q.ac);
  }

  // decodeTile — ebiv/decode_intra.go:121-135
  void decodeTile(const TileBounds& b) {
    for (int mby = b.mbY0; mby < b.mbY1; mby++)
      for (int mbx = b.mbX0; mbx < b.mbX1; mbx++) {
        if (inter) {
          decodeInterMB(mbx, mby, b);
        } else {
          decodeLumaMB(mbx, mby, b);
          decodeChromaMB(mbx, mby, b);
        }
        if (dec.err != EO_OK) return;
      }
  }

  // decodeLumaMB — ebiv/decode_intra.go:137-157
  void decodeLumaMB(int mbx, int mby, const TileBounds& b) {
    int txIdx = dec.decode(ctxTxSize);
    if (txIdx < 0 || txIdx >= 3) {
      dec.fail(EO_ERR_CORRUPT);
      return;
    }
    int n = lumaTx[txIdx];
    int tileLeft = b.mbX0 * mbSize, tileTop = b.mbY0 * mbSize, tileRight = b.mbX1 * mbSize;
    int mbTop = mby * mbSize, mbRight = (mbx + 1) * mbSize;
    for (int by = 0; by < mbSize; by += n)
      for (int bx = 0; bx < mbSize; bx += n) {
        int x0 = mbx * mbSize + bx, y0 = mby * mbSize + by;
        int mode = dec.decode(ctxLumaMode);
        bool avAR = aboveRightAvailable(x0, y0, n, tileTop, tileRight, mbTop, mbRight);
        reconBlock(planeLuma, txIdx, rec->y, x0, y0, n, mode, y0 > tileTop, x0 > tileLeft, avAR);
      }
  }

  // decodeChromaMB — ebiv/decode_intra.go:159-167
  void decodeChromaMB(int mbx, int mby, const TileBounds& b) {
    int tileLeft = b.mbX0 * chromaMB, tileTop = b.mbY0 * chromaMB;
    int x0 = mbx * chromaMB, y0 = mby * chromaMB;
    int mode = dec.decode(ctxChromaMode);
    reconBlock(planeChroma, 0, rec->cb, x0, y0, chromaMB, mode, y0 > tileTop, x0 > tileLeft, false);
    reconBlock(planeChroma, 0, rec->cr, x0, y0, chromaMB, mode, y0 > tileTop, x0 > tileLeft, false);
  }

  // reconBlock — ebiv/decode_intra.go:170-187
  void reconBlock(int plane, int txIdx, const PlaneView& p, int x0, int y0, int n, int mode,
                  bool avAbove, bool avLeft, bool avAR) {
    if (mode < 0 || mode >= numIntraModes) {
      dec.fail(EO_ERR_CORRUPT);
      return;
    }
    for (int i = 0; i < n * n; i++) sc.levels[i] = 0;
    decodeBlock(dec, plane, txIdx, sc.levels, n);
    if (dec.err != EO_OK) return;
    dequantize(n);
    inverseDCT(sc.coeffs, sc.recon, n);
    predictIntra(p, x0, y0, n, mode, avAbove, avLeft, avAR, sc.pred);
    reconstruct(p, x0, y0, n, sc.pred, sc.recon);
  }

  // decodeInterMB — ebiv/decode_inter.go:8-62
  void decodeInterMB(int mbx, int mby, const TileBounds& b) {
    int mode = dec.decode(ctxMBMode);
    int idx = mby * mvStride + mbx;
    switch (mode) {
      case mbSkip: {
        MV m = predictMV(mv, mvStride, mbx, mby, b);
        mv[idx] = m;
        reconMCMB(mbx, mby, m);
        break;
      }
      case mbIntra:
        decodeLumaMB(mbx, mby, b);
        decodeChromaMB(mbx, mby, b);
        mv[idx] = MV{};
        break;
      case mbInter: {
        int refSel = dec.decode(ctxRef);
        if (refSel < 0 || refSel >= numRefs) {
          dec.fail(EO_ERR_CORRUPT);
          return;
        }
        FrameBuf* r = ref;
        MV pred = predictMV(mv, mvStride, mbx, mby, b);
        if (refSel == refGolden) {
          r = golden;
          pred = MV{};
        }
        int part = dec.decode(ctxPart);
        if (part < 0 || part >= numPartModes) {
          dec.fail(EO_ERR_CORRUPT);
          return;
        }
        MV mvs[4];
        for (int i = 0; i < kPartCount[part]; i++) {
          MV pp = i > 0 ? mvs[0] : pred;
          int dx = dec.getMVComponent(ctxMVClassX);
          mvs[i].x = clampMV((int)pp.x + dx);
          int dy = dec.getMVComponent(ctxMVClassY);
          mvs[i].y = clampMV((int)pp.y + dy);
        }
        if (dec.err != EO_OK) return;
        mv[idx] = refSel == refGolden ? MV{} : mvs[0];
        reconInterMB(r, mbx, mby, part, mvs);
        break;
      }
      default:
        dec.fail(EO_ERR_CORRUPT);
    }
  }

  // reconMCMB — ebiv/decode_inter.go:66-71
  void reconMCMB(int mbx, int mby, MV m) {
    mcLumaByte(ref->y, mbx * mbSize + (m.x >> 2), mby * mbSize + (m.y >> 2), m.x & 3, m.y & 3, mbSize, mbSize,
               rec->y, mbx * mbSize, mby * mbSize);
    int cx = mbx * chromaMB, cy = mby * chromaMB;
    mcChromaByte(ref->cb, cx + (m.x >> 3), cy + (m.y >> 3), m.x & 7, m.y & 7, chromaMB, chromaMB, rec->cb, cx, cy);
    mcChromaByte(ref->cr, cx + (m.x >> 3), cy + (m.y >> 3), m.x & 7, m.y & 7, chromaMB, chromaMB, rec->cr, cx, cy);
  }

  // reconInterMB — ebiv/decode_inter.go:73-118
  void reconInterMB(FrameBuf* r, int mbx, int mby, int part, const MV* mvs) {
    int cbp = dec.decode(ctxCBP);
    if (cbp < 0 || cbp >= numCBP || dec.err != EO_OK) {
      dec.fail(EO_ERR_CORRUPT);
      return;
    }
    const Rect4* rects = kPartRects[part];
    int np = kPartCount[part];
    if (cbp & cbpLuma) {
      int32_t mcY[256];
      for (int i = 0; i < np; i++) {
        const Rect4& rc = rects[i];
        mcLuma(r->y, mbx * mbSize + rc.x + (mvs[i].x >> 2), mby * mbSize + rc.y + (mvs[i].y >> 2), mvs[i].x & 3,
               mvs[i].y & 3, rc.w, rc.h, mcY, rc.x, rc.y, mbSize);
      }
      int txIdx = dec.decode(ctxTxSize);
      if (txIdx < 0 || txIdx >= 3) {
        dec.fail(EO_ERR_CORRUPT);
        return;
      }
      int n = lumaTx[txIdx];
      for (int by = 0; by < mbSize; by += n)
        for (int bx = 0; bx < mbSize; bx += n) {
          for (int rr = 0; rr < n; rr++)
            for (int cc = 0; cc < n; cc++) sc.pred[rr * n + cc] = mcY[(by + rr) * mbSize + bx + cc];
          reconResidual(planeLuma, txIdx, rec->y, mbx * mbSize + bx, mby * mbSize + by, n);
          if (dec.err != EO_OK) return;
        }
    } else {
      for (int i = 0; i < np; i++) {
        const Rect4& rc = rects[i];
        mcLumaByte(r->y, mbx * mbSize + rc.x + (mvs[i].x >> 2), mby * mbSize + rc.y + (mvs[i].y >> 2), mvs[i].x & 3,
                   mvs[i].y & 3, rc.w, rc.h, rec->y, mbx * mbSize + rc.x, mby * mbSize + rc.y);
      }
    }
    int cx = mbx * chromaMB, cy = mby * chromaMB;
    reconInterChroma(cx, cy, rects, np, mvs, r->cb, rec->cb, (cbp & cbpCb) != 0);
    reconInterChroma(cx, cy, rects, np, mvs, r->cr, rec->cr, (cbp & cbpCr) != 0);
  }

  // reconInterChroma — ebiv/decode_inter.go:123-136
  void reconInterChroma(int cx, int cy, const Rect4* rects, int np, const MV* mvs, const PlaneView& r,
                        const PlaneView& p, bool coded) {
    if (coded) {
      int32_t mc[64];
      for (int i = 0; i < np; i++) {
        const Rect4& rc = rects[i];
        int cpx = rc.x / 2, cpy = rc.y / 2, cpw = rc.w / 2, cph = rc.h / 2;
        mcChroma(r, cx + cpx + (mvs[i].x >> 3), cy + cpy + (mvs[i].y >> 3), mvs[i].x & 7, mvs[i].y & 7, cpw, cph, mc,
                 cpx, cpy, chromaMB);
      }
      std::memcpy(sc.pred, mc, sizeof(mc));
      reconResidual(planeChroma, 0, p, cx, cy, chromaMB);
      return;
    }
    for (int i = 0; i < np; i++) {
      const Rect4& rc = rects[i];
      int cpx = rc.x / 2, cpy = rc.y / 2, cpw = rc.w / 2, cph = rc.h / 2;
      mcChromaByte(r, cx + cpx + (mvs[i].x >> 3), cy + cpy + (mvs[i].y >> 3), mvs[i].x & 7, mvs[i].y & 7, cpw, cph, p,
                   cx + cpx, cy + cpy);
    }
  }

  // reconResidual — ebiv/decode_inter.go:140-152
  void reconResidual(int plane, int txIdx, const PlaneView& p, int x0, int y0, int n) {
    for (int i = 0; i < n * n; i++) sc.levels[i] = 0;
    decodeBlock(dec, plane, txIdx, sc.levels, n);
    if (dec.err != EO_OK) return;
    dequantize(n);
    inverseDCT(sc.coeffs, sc.recon, n);
    reconstruct(p, x0, y0, n, sc.pred, sc.recon);
  }
};

// ---- worker pool: ebiv/pool.go:19-72 ---------------------------------------
// A fixed set of workers shared by every frame of a codec; run() hands out
// item indices and blocks until all have finished.
class Pool {
 public:
  explicit Pool(int n) {
    for (int i = 0; i < n; i++) workers_.emplace_back([this] { loop(); });
  }
  ~Pool() {
    {
      std::lock_guard<std::mutex> g(mu_);
      stop_ = true;
    }
    cv_.notify_all();
    for (auto& t : workers_) t.join();
  }
  // run — ebiv/pool.go:58-72: a single item runs inline on the caller.
  void run(int count, const std::function<void(int)>& fn) {
    if (count <= 0) return;
    if (count == 1 || workers_.empty()) {
      for (int i = 0; i < count; i++) fn(i);
      return;
    }
    std::unique_lock<std::mutex> lk(mu_);
    job_ = &fn;
    next_ = 0;
    count_ = count;
    done_ = 0;
    gen_++;
    cv_.notify_all();
    done_cv_.wait(lk, [&] { return done_ == count_; });
    job_ = nullptr;
  }

 private:
  void loop() {
    uint64_t seen = 0;
    std::unique_lock<std::mutex> lk(mu_);
    for (;;) {
      cv_.wait(lk, [&] { return stop_ || gen_ != seen; });
      if (stop_) return;
      seen = gen_;
      while (job_ && next_ < count_) {
        int i = next_++;
        const std::function<void(int)>* f = job_;
        lk.unlock();
        (*f)(i);
        lk.lock();
        if (++done_ == count_) done_cv_.notify_all();
      }
    }
  }
  std::vector<std::thread> workers_;
  std::mutex mu_;
  std::condition_variable cv_, done_cv_;
  const std::function<void(int)>* job_ = nullptr;
  int next_ = 0, count_ = 0, done_ = 0;
  uint64_t gen_ = 0;
  bool stop_ = false;
};

// ---- decode state + codec: ebiv/decode_intra.go:28-94, ebiv/codec.go -------
struct DecodeState {
  std::vector<RansTable> tables;
  std::vector<PrevFreq> prevFreqs;
  std::vector<MV> mv;
  std::vector<std::unique_ptr<TileDecoder>> tds;
  DecodeState() : tables(numContexts), prevFreqs(numContexts) {}

  // parsePayload + decodeCoded — ebiv/frame.go:242-274, decode_intra.go:55-94
  int decodeCoded(FrameBuf* rec, FrameBuf* ref, FrameBuf* golden, const uint8_t* body, size_t blen,
                  bool inter, bool key, Pool* pool) {
    // parseCodedHeader — ebiv/frame.go:197-220
    if (blen < 1) return EO_ERR_CORRUPT;
    int qp = body[0];
    size_t pos = 1;
    int n;
    uint64_t cols = uvarint(body + pos, blen - pos, &n);
    if (n <= 0) return EO_ERR_CORRUPT;
    pos += (size_t)n;
    uint64_t rows = uvarint(body + pos, blen - pos, &n);
    if (n <= 0) return EO_ERR_CORRUPT;
    pos += (size_t)n;
    if (qp > maxQP || cols == 0 || rows == 0 || cols > 65535 || rows > 65535) return EO_ERR_CORRUPT;
    uint64_t tablesLen = uvarint(body + pos, blen - pos, &n);
    if (n <= 0 || tablesLen > (uint64_t)(blen - pos - (size_t)n)) return EO_ERR_CORRUPT;
    pos += (size_t)n;
    size_t consumed = 0;
    int st = parseTablesInto(tables.data(), prevFreqs.data(), body + pos, (size_t)tablesLen, key, &consumed);
    if (st != EO_OK) return st;
    if (consumed != tablesLen) return EO_ERR_CORRUPT;
    pos += (size_t)tablesLen;
    uint64_t want = cols * rows;
    std::vector<std::pair<const uint8_t*, size_t>> tiles;
    while (tiles.size() < want) {
      uint64_t tl = uvarint(body + pos, blen - pos, &n);
      if (n <= 0 || tl > (uint64_t)(blen - pos - (size_t)n)) return EO_ERR_CORRUPT;
      pos += (size_t)n;
      tiles.emplace_back(body + pos, (size_t)tl);
      pos += (size_t)tl;
    }
    TileGrid grid(rec->mbCols, rec->mbRows, (int)cols, (int)rows);
    if ((uint64_t)grid.count() != tiles.size()) return EO_ERR_CORRUPT;
    Quantizer q = newQuantizer(qp);
    int nMB = rec->mbCols * rec->mbRows;
    mv.assign((size_t)nMB, MV{});
    while (tds.size() < tiles.size()) tds.emplace_back(new TileDecoder());
    std::vector<int> errs(tiles.size(), EO_OK);
    auto work = [&](int i) {
      TileDecoder* td = tds[(size_t)i].get();
      td->rec = rec;
      td->ref = ref;
      td->golden = golden;
      td->q = q;
      td->inter = inter;
      td->mv = mv.data();
      td->mvStride = rec->mbCols;
      int e = td->dec.reset(tiles[(size_t)i].first, (int64_t)tiles[(size_t)i].second, tables.data());
      if (e != EO_OK) {
        errs[(size_t)i] = e;
        return;
      }
      td->decodeTile(grid.bounds(i));
      errs[(size_t)i] = td->dec.err;
    };
    if (pool)
      pool->run((int)tiles.size(), work);
    else
      for (int i = 0; i < (int)tiles.size(); i++) work(i);
    for (int e : errs)
      if (e != EO_OK) return e;
    return EO_OK;
  }
};

}  // namespace eo

using namespace eo;

struct eo_codec {
  int ringSize = 3;
  Geometry geo;
  bool ready = false;
  std::vector<Image> ring;
  int next = 0;
  std::unique_ptr<FrameBuf> work, ref, golden;
  std::unique_ptr<DecodeState> dec;
  std::unique_ptr<Pool> pool;

  // configure — ebiv/codec.go:129-153
  int configure(int w, int h) {
    if ((int64_t)w * h > maxDecodePixels) return EO_ERR_UNSUPPORTED;
    if (ready) {
      if (w != geo.W || h != geo.H) return EO_ERR_DIMENSIONS;
      return EO_OK;
    }
    geo = geometryFor(w, h);
    ring.assign((size_t)ringSize, Image{});
    for (auto& im : ring) {
      im.Y.assign((size_t)geo.YStride * geo.H, 0);
      im.Cb.assign((size_t)geo.CStride * geo.CH, 0);
      im.Cr.assign((size_t)geo.CStride * geo.CH, 0);
    }
    work.reset(new FrameBuf());
    ref.reset(new FrameBuf());
    golden.reset(new FrameBuf());
    work->init(w, h);
    ref->init(w, h);
    golden->init(w, h);
    dec.reset(new DecodeState());
    next = 0;
    ready = true;
    return EO_OK;
  }

  // storeImage — ebiv/frame.go:67-77
  void store(Image& img) {
    for (int y = 0; y < geo.H; y++) std::memcpy(&img.Y[(size_t)y * geo.YStride], work->y.data + (size_t)y * work->y.stride, geo.W);
    for (int y = 0; y < geo.CH; y++) {
      std::memcpy(&img.Cb[(size_t)y * geo.CStride], work->cb.data + (size_t)y * work->cb.stride, geo.CW);
      std::memcpy(&img.Cr[(size_t)y * geo.CStride], work->cr.data + (size_t)y * work->cr.stride, geo.CW);
    }
  }

  // Codec.Decode — ebiv/codec.go:70-111 (with parseFrameHeader, format.go:376-409)
  int decode(const uint8_t* b, size_t n, int* slot) {
    if (n < 1) return EO_ERR_CORRUPT;
    int type = b[0] & 0x03, coding = (b[0] >> 2) & 0x07;
    bool hasOverride = (b[0] & (1 << 5)) != 0;
    if (type != 0 && type != 1) return EO_ERR_CORRUPT;
    if (hasOverride && type != 0) return EO_ERR_CORRUPT;
    const uint8_t* body = b + 1;
    size_t blen = n - 1;
    int W = 0, H = 0;
    if (type == 0) {
      if (n < 6) return EO_ERR_CORRUPT;
      W = b[1] | (b[2] << 8);
      H = b[3] | (b[4] << 8);
      if (W == 0 || H == 0) return EO_ERR_CORRUPT;
      if ((b[5] >> 4) != 0) return EO_ERR_UNSUPPORTED;
      if ((b[5] & 0x0f) != 0) return EO_ERR_UNSUPPORTED;
      body = b + 6;
      blen = n - 6;
      int e = configure(W, H);
      if (e != EO_OK) return e;
    } else if (!ready) {
      return EO_ERR_NOKEYFRAME;
    }
    int s = next;
    next++;
    if (next == (int)ring.size()) next = 0;
    Image& img = ring[(size_t)s];
    int st;
    switch (coding) {
      case 0:
        st = decodeRaw(img, body, blen);
        break;
      case 1:
      case 2:
        st = decodeCoded(img, coding == 2, type == 0, hasOverride, body, blen);
        break;
      default:
        return EO_ERR_UNSUPPORTED;
    }
    if (st != EO_OK) return st;
    *slot = s;
    return EO_OK;
  }

  // Codec.decodeCoded — ebiv/codec.go:162-192
  int decodeCoded(Image& dst, bool inter, bool key, bool hasOverride, const uint8_t* body, size_t blen) {
    const uint8_t* ov = nullptr;
    size_t ovLen = 0;
    if (hasOverride) {
      int n;
      uint64_t keyLen = uvarint(body, blen, &n);
      if (n <= 0 || keyLen > (uint64_t)(blen - (size_t)n)) return EO_ERR_CORRUPT;
      ov = body + n + keyLen;
      ovLen = blen - (size_t)n - (size_t)keyLen;
      body = body + n;
      blen = (size_t)keyLen;
    }
    int e = dec->decodeCoded(work.get(), ref.get(), golden.get(), body, blen, inter, key, pool.get());
    if (e != EO_OK) return e;
    if (key) {
      if (hasOverride) {
        e = dec->decodeCoded(golden.get(), work.get(), work.get(), ov, ovLen, true, false, pool.get());
        if (e != EO_OK) return e;
      } else {
        golden->copyFrom(*work);
      }
    }
    store(dst);
    std::swap(work, ref);
    return EO_OK;
  }

  // Codec.decodeRaw — ebiv/codec.go:195-207
  int decodeRaw(Image& dst, const uint8_t* body, size_t blen) {
    size_t ySize = (size_t)geo.W * geo.H, cSize = (size_t)geo.CW * geo.CH;
    if (blen != ySize + 2 * cSize) return EO_ERR_CORRUPT;
    for (int y = 0; y < geo.H; y++) std::memcpy(&dst.Y[(size_t)y * geo.YStride], body + (size_t)y * geo.W, geo.W);
    for (int y = 0; y < geo.CH; y++) {
      std::memcpy(&dst.Cb[(size_t)y * geo.CStride], body + ySize + (size_t)y * geo.CW, geo.CW);
      std::memcpy(&dst.Cr[(size_t)y * geo.CStride], body + ySize + cSize + (size_t)y * geo.CW, geo.CW);
    }
    return EO_OK;
  }

  size_t packedSize() const { return (size_t)geo.W * geo.H + 2 * (size_t)geo.CW * geo.CH; }
  void pack(const Image& im, uint8_t* out) const {
    size_t o = 0;
    for (int y = 0; y < geo.H; y++, o += geo.W) std::memcpy(out + o, &im.Y[(size_t)y * geo.YStride], geo.W);
    for (int y = 0; y < geo.CH; y++, o += geo.CW) std::memcpy(out + o, &im.Cb[(size_t)y * geo.CStride], geo.CW);
    for (int y = 0; y < geo.CH; y++, o += geo.CW) std::memcpy(out + o, &im.Cr[(size_t)y * geo.CStride], geo.CW);
  }
};

extern "C" {

eo_codec* eo_codec_create(int ring, int threads) {
  eo_codec* c = new eo_codec();
  if (ring >= 2) c->ringSize = ring;
  if (threads > 1) c->pool.reset(new Pool(threads));
  return c;
}
void eo_codec_destroy(eo_codec* c) { delete c; }

int eo_codec_decode(eo_codec* c, const uint8_t* pkt, size_t n, int* slot, int* w, int* h) {
  if (!c) return EO_ERR_ARG;
  int s = -1;
  int st = c->decode(pkt, n, &s);
  if (slot) *slot = s;
  if (w) *w = c->geo.W;
  if (h) *h = c->geo.H;
  return st;
}

long eo_wide_residuals(int reset) {
  return reset ? gWideResiduals.exchange(0) : gWideResiduals.load();
}

void eo_codec_flush(eo_codec* c) {
  if (c) c->next = 0;
}

int eo_codec_ring_image(eo_codec* c, int slot, uint8_t* packed, size_t cap) {
  if (!c || !c->ready || slot < 0 || slot >= (int)c->ring.size() || cap < c->packedSize()) return EO_ERR_ARG;
  c->pack(c->ring[(size_t)slot], packed);
  return EO_OK;
}

int eo_codec_reference(eo_codec* c, int which, uint8_t* packed, size_t cap) {
  if (!c || !c->ready) return EO_ERR_ARG;
  FrameBuf* f = which == 0 ? c->ref.get() : c->golden.get();
  size_t need = f->ybuf.size() + f->cbbuf.size() + f->crbuf.size();
  if (cap < need) return EO_ERR_ARG;
  std::memcpy(packed, f->ybuf.data(), f->ybuf.size());
  std::memcpy(packed + f->ybuf.size(), f->cbbuf.data(), f->cbbuf.size());
  std::memcpy(packed + f->ybuf.size() + f->cbbuf.size(), f->crbuf.data(), f->crbuf.size());
  return EO_OK;
}

int eo_decode_sequence(const uint8_t* const* pkts, const size_t* lens, int n, int threads, uint8_t* out,
                       size_t frame_bytes, int* statuses) {
  eo_codec* c = eo_codec_create(3, threads);
  int bad = 0;
  for (int i = 0; i < n; i++) {
    int slot = -1;
    int st = c->decode(pkts[i], lens[i], &slot);
    statuses[i] = st;
    if (st == EO_OK && out && c->packedSize() <= frame_bytes)
      c->pack(c->ring[(size_t)slot], out + (size_t)i * frame_bytes);
    if (st != EO_OK) bad++;
  }
  delete c;
  return bad;
}

long eo_decode_streams(const uint8_t* const* const* pkts, const size_t* const* lens, const int* nframes, int nstreams,
                       int threads) {
  std::atomic<int> nextStream{0};
  std::atomic<long> ok{0};
  auto worker = [&] {
    for (;;) {
      int s = nextStream.fetch_add(1);
      if (s >= nstreams) return;
      eo_codec c;
      long good = 0;
      for (int i = 0; i < nframes[s]; i++) {
        int slot;
        if (c.decode(pkts[s][i], lens[s][i], &slot) == EO_OK) good++;
      }
      ok += good;
    }
  };
  if (threads < 1) threads = 1;
  std::vector<std::thread> ts;
  for (int t = 0; t < threads; t++) ts.emplace_back(worker);
  for (auto& t : ts) t.join();
  return ok.load();
}

void eo_rgba(const uint8_t* y, const uint8_t* cb, const uint8_t* cr, int w, int h, uint8_t* dst) {
  // convertYCbCr420ToRGBA — frame.go:8-67 on packed planes (strides w, (w+1)/2)
  int cw = (w + 1) / 2;
  size_t di = 0;
  for (int row = 0; row < h; row++) {
    const uint8_t* yr = y + (size_t)row * w;
    size_t ci = (size_t)(row / 2) * cw;
    for (int col = 0; col < w; col++) {
      int32_t yy1 = (int32_t)yr[col] * 0x10101;
      int32_t cb1 = (int32_t)cb[ci + col / 2] - 128;
      int32_t cr1 = (int32_t)cr[ci + col / 2] - 128;
      int32_t r = yy1 + 91881 * cr1;
      int32_t g = yy1 - 22554 * cb1 - 46802 * cr1;
      int32_t b = yy1 + 116130 * cb1;
      r = r < 0 ? 0 : (r > 0xff0000 ? 0xff0000 : r);
      g = g < 0 ? 0 : (g > 0xff0000 ? 0xff0000 : g);
      b = b < 0 ? 0 : (b > 0xff0000 ? 0xff0000 : b);
      dst[di] = (uint8_t)(r >> 16);
      dst[di + 1] = (uint8_t)(g >> 16);
      dst[di + 2] = (uint8_t)(b >> 16);
      dst[di + 3] = 0xff;
      di += 4;
    }
  }
}

void eo_inverse_dct(const int32_t* src, int32_t* dst, int n) { inverseDCT(src, dst, n); }

void eo_zigzag(int n, int* order) {
  const int* s = T().scan[txIndexOf(n)];
  for (int i = 0; i < n * n; i++) order[i] = s[i];
}

int eo_dct_matrix(int n, int32_t* out) {
  if (n != 4 && n != 8 && n != 16) return EO_ERR_ARG;
  std::memcpy(out, T().dct[txIndexOf(n)], sizeof(int32_t) * n * n);
  return EO_OK;
}

int eo_quant_steps(int qp, int32_t* dc, int32_t* ac) {
  Quantizer q = newQuantizer(qp);
  *dc = q.dc;
  *ac = q.ac;
  return EO_OK;
}

static void buildProbeTables(std::vector<RansTable>& tables, const uint32_t* freqs, const uint8_t* used) {
  for (int c = 0; c < numContexts; c++) {
    tables[(size_t)c].used = false;
    if (c == ctxBypass || !used[c]) continue;
    buildTableInto(tables[(size_t)c], freqs + c * 16, alphabetSize(c));
  }
  static const uint32_t bypass[2] = {kM / 2, kM / 2};
  buildTableInto(tables[ctxBypass], bypass, 2);
}

int eo_decode_block(const uint8_t* stream, size_t n, const uint32_t* freqs, const uint8_t* used, int plane,
                    int tx_idx, int bn, int32_t* levels) {
  std::vector<RansTable> tables(numContexts);
  buildProbeTables(tables, freqs, used);
  RansDecoder d;
  int e = d.reset(stream, (int64_t)n, tables.data());
  if (e != EO_OK) return e;
  for (int i = 0; i < bn * bn; i++) levels[i] = 0;
  decodeBlock(d, plane, tx_idx, levels, bn);
  return d.err;
}

int eo_decode_symbols(const uint8_t* stream, size_t n, const uint32_t* freqs, const uint8_t* used, const int* ctxs,
                      int count, int* syms) {
  std::vector<RansTable> tables(numContexts);
  buildProbeTables(tables, freqs, used);
  RansDecoder d;
  int e = d.reset(stream, (int64_t)n, tables.data());
  if (e != EO_OK) return e;
  for (int i = 0; i < count; i++) syms[i] = d.decode(ctxs[i]);
  return d.err;
}

}  // extern "C"
