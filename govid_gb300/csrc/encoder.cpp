// EBIV encoder: rate-distortion intra/inter coding, two-pass real-cost RDOQ,
// static-table rANS and the container writer.  Each routine cites the
// reference routine whose decisions it reproduces; the decisions must match
// for the encoded sizes the reference pins (ebiv/regression_test.go:15-39).
//
// Build note: compiled with -ffp-contract=off so the RDOQ cost arithmetic is
// evaluated as separate IEEE-754 multiplies and adds on every host.
#include "encoder.h"

#include <algorithm>
#include <chrono>
#include <atomic>
#include <cmath>
#include <cstring>

#include "thread_pool.h"

namespace ebiv {

const CodingTables& codingTables() {
  static CodingTables t;
  return t;
}

uint32_t crc32IEEE(const uint8_t* data, size_t n) {
  static uint32_t table[256];
  static bool init = [] {
    for (uint32_t i = 0; i < 256; i++) {
      uint32_t c = i;
      for (int k = 0; k < 8; k++) c = (c & 1) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
      table[i] = c;
    }
    return true;
  }();
  (void)init;
  uint32_t c = 0xFFFFFFFFu;
  for (size_t i = 0; i < n; i++) c = table[(c ^ data[i]) & 0xff] ^ (c >> 8);
  return c ^ 0xFFFFFFFFu;
}

namespace {

// ---------------------------------------------------------------------------
// Planes and padded frame buffers (ebiv/predict.go:15-24, ebiv/frame.go:19-64)
// ---------------------------------------------------------------------------
struct Plane {
  uint8_t* d = nullptr;
  int stride = 0, w = 0, h = 0;
  inline uint8_t at(int x, int y) const { return d[(size_t)y * stride + x]; }
  inline void set(int x, int y, uint8_t v) const { d[(size_t)y * stride + x] = v; }
};

struct Frame {
  std::vector<uint8_t> yb, cbb, crb;
  Plane y, cb, cr;
  int mbCols = 0, mbRows = 0;
  explicit Frame(const Geometry& g) {
    mbCols = g.mbCols;
    mbRows = g.mbRows;
    yb.assign((size_t)g.padW() * g.padH(), 0);
    cbb.assign((size_t)g.padCW() * g.padCH(), 0);
    crb.assign((size_t)g.padCW() * g.padCH(), 0);
    y = {yb.data(), g.padW(), g.padW(), g.padH()};
    cb = {cbb.data(), g.padCW(), g.padCW(), g.padCH()};
    cr = {crb.data(), g.padCW(), g.padCW(), g.padCH()};
  }
};

// Edge replication into the padding (loadImage/loadPlane, ebiv/frame.go:50-64).
void loadPlane(const Plane& dst, const uint8_t* src, int sStride, int vw, int vh) {
  for (int y = 0; y < dst.h; y++) {
    const int sy = std::min(y, vh - 1);
    uint8_t* row = dst.d + (size_t)y * dst.stride;
    for (int x = 0; x < dst.w; x++) row[x] = src[(size_t)sy * sStride + std::min(x, vw - 1)];
  }
}
void loadImage(Frame& f, const PackedImage& img) {
  loadPlane(f.y, img.Y.data(), img.W, img.W, img.H);
  loadPlane(f.cb, img.Cb.data(), img.CW, img.CW, img.CH);
  loadPlane(f.cr, img.Cr.data(), img.CW, img.CW, img.CH);
}

// ---------------------------------------------------------------------------
// Entropy layer, encoder half (ebiv/rans.go:46-214, 339-389)
// ---------------------------------------------------------------------------
struct Tok {
  uint16_t ctx, sym;
};
struct TokStream {
  std::vector<Tok> toks;
  inline void put(int ctx, int sym) { toks.push_back({(uint16_t)ctx, (uint16_t)sym}); }
};

using Freqs = std::vector<uint32_t>;  // empty == context unused

int largestReducible(const Freqs& f) {
  int best = -1;
  for (int s = 0; s < (int)f.size(); s++)
    if (f[s] > 1 && (best < 0 || f[s] > f[best])) best = s;
  if (best < 0)
    for (int s = 0; s < (int)f.size(); s++)
      if (f[s] > 0) return s;
  return best;
}

// normalizeFreqs — ebiv/rans.go:46-85
Freqs normalizeFreqs(const std::vector<uint32_t>& counts) {
  uint64_t total = 0;
  for (uint32_t c : counts) total += c;
  if (total == 0) return {};
  Freqs freq(counts.size(), 0);
  uint32_t used = 0;
  int largest = 0;
  for (int s = 0; s < (int)counts.size(); s++) {
    if (counts[s] == 0) continue;
    uint32_t f = (uint32_t)((uint64_t)counts[s] * kM / total);
    if (f == 0) f = 1;
    freq[s] = f;
    used += f;
    if (freq[s] > freq[largest]) largest = s;
  }
  while (used > kM) {
    freq[largestReducible(freq)]--;
    used--;
  }
  if (used < kM) freq[largest] += kM - used;
  return freq;
}

struct EncSym {
  uint32_t start = 0, freq = 0;
};
struct EncTable {
  std::vector<EncSym> enc;
  bool used = false;
};
EncTable buildEncTable(const Freqs& freq, int size) {
  EncTable t;
  t.enc.assign((size_t)size, EncSym{});
  uint32_t cum = 0;
  for (int s = 0; s < (int)freq.size(); s++) {
    t.enc[s] = {cum, freq[s]};
    cum += freq[s];
  }
  t.used = cum == kM;
  return t;
}

// ransEncode — ebiv/rans.go:186-214
std::vector<uint8_t> ransEncode(const std::vector<Tok>& toks, const std::vector<EncTable>& tables) {
  std::vector<uint8_t> st;
  st.reserve(toks.size() / 2 + 16);
  uint32_t state[kStates];
  for (int i = 0; i < kStates; i++) state[i] = kLower;
  for (int64_t j = (int64_t)toks.size() - 1; j >= 0; j--) {
    const Tok& t = toks[(size_t)j];
    const EncSym s = tables[t.ctx].enc[t.sym];
    uint32_t x = state[j % kStates];
    const uint32_t xmax = ((kLower >> kScaleBits) << 8) * s.freq;
    while (x >= xmax) {
      st.push_back((uint8_t)x);
      x >>= 8;
    }
    state[j % kStates] = ((x / s.freq) << kScaleBits) + (x % s.freq) + s.start;
  }
  for (int i = 0; i < kStates; i++)
    for (int k = 0; k < 4; k++) st.push_back((uint8_t)(state[i] >> (8 * k)));
  return st;
}

// serializeTables — ebiv/rans.go:339-377
std::vector<uint8_t> serializeTables(const std::vector<Freqs>& freqs, const std::vector<Freqs>* prev) {
  std::vector<uint8_t> out;
  for (int c = 0; c < kNumContexts; c++) {
    const Freqs& f = freqs[c];
    if (c == ctxBypass || f.empty()) {
      out.push_back(0);
      continue;
    }
    const Freqs* pf = (prev && !(*prev)[c].empty()) ? &(*prev)[c] : nullptr;
    if (pf && *pf == f) {
      out.push_back(1);
      continue;
    }
    std::vector<uint8_t> full;
    for (uint32_t v : f) putUvarint(full, v);
    if (pf) {
      std::vector<uint8_t> delta;
      for (size_t s = 0; s < f.size(); s++) putVarint(delta, (int64_t)f[s] - (int64_t)(*pf)[s]);
      if (delta.size() < full.size()) {
        out.push_back(3);
        out.insert(out.end(), delta.begin(), delta.end());
        continue;
      }
    }
    out.push_back(2);
    out.insert(out.end(), full.begin(), full.end());
  }
  return out;
}

// ---------------------------------------------------------------------------
// Transforms and quantization (ebiv/transform.go:44-194, ebiv/quant.go)
// ---------------------------------------------------------------------------
// forwardDCT — ebiv/transform.go:44-79.  Encoder inputs are residuals of
// two bytes (|v| <= 255), so both passes fit in int32 exactly: the column
// sums stay below 255 * 46341 and the row sums below 1443 * 46341.
template <int N>
void forwardDCTN(const int32_t* src, int32_t* dst) {
  const int32_t* c = codingTables().dct[N == 4 ? 0 : (N == 8 ? 1 : 2)];
  int32_t acc[N * N];
  int32_t tmp[N * N];
  for (int k = 0; k < N * N; k++) acc[k] = 0;
  for (int i = 0; i < N; i++) {
    const int32_t* srow = src + i * N;
    for (int k = 0; k < N; k++) {
      const int32_t cki = c[k * N + i];
      int32_t* arow = acc + k * N;
      for (int j = 0; j < N; j++) arow[j] += cki * srow[j];
    }
  }
  for (int k = 0; k < N * N; k++) tmp[k] = (acc[k] + 4096) >> 13;
  for (int k = 0; k < N; k++) {
    const int32_t* trow = tmp + k * N;
    for (int l = 0; l < N; l++) {
      const int32_t* crow = c + l * N;
      int32_t a = 0;
      for (int j = 0; j < N; j++) a += crow[j] * trow[j];
      dst[k * N + l] = (a + 4096) >> 13;
    }
  }
}
void forwardDCT(const int32_t* src, int32_t* dst, int n) {
  if (n == 4)
    forwardDCTN<4>(src, dst);
  else if (n == 8)
    forwardDCTN<8>(src, dst);
  else
    forwardDCTN<16>(src, dst);
}

void inverseDCT(const int32_t* src, int32_t* dst, int n) {
  int maxR = -1, maxC = -1;
  for (int r = 0; r < n; r++)
    for (int cc = 0; cc < n; cc++)
      if (src[r * n + cc] != 0) {
        maxR = std::max(maxR, r);
        maxC = std::max(maxC, cc);
      }
  if (maxR < 0) {
    std::fill(dst, dst + n * n, 0);
    return;
  }
  const int32_t* c = codingTables().dct[txIndexOf(n)];
  const int64_t round = 1LL << 12;
  if (maxR == 0 && maxC == 0) {
    const int64_t d0 = c[0];
    const int64_t col = (d0 * (int64_t)src[0] + round) >> 13;
    std::fill(dst, dst + n * n, (int32_t)((d0 * col + round) >> 13));
    return;
  }
  int32_t tmp[kMaxLevels];
  for (int i = 0; i < n; i++)
    for (int l = 0; l <= maxC; l++) {
      int64_t a = 0;
      for (int k = 0; k <= maxR; k++) a += (int64_t)c[k * n + i] * (int64_t)src[k * n + l];
      tmp[i * n + l] = (int32_t)((a + round) >> 13);
    }
  for (int i = 0; i < n; i++)
    for (int m = 0; m < n; m++) {
      int64_t a = 0;
      for (int l = 0; l <= maxC; l++) a += (int64_t)c[l * n + m] * (int64_t)tmp[i * n + l];
      dst[i * n + m] = (int32_t)((a + round) >> 13);
    }
}

// satd / fwht — ebiv/transform.go:86-119, unrolled per block size.
template <int N>
inline void fwhtRows(int32_t* t) {
  for (int r = 0; r < N; r++) {
    int32_t* a = t + r * N;
    for (int span = 1; span < N; span <<= 1)
      for (int i = 0; i < N; i += span << 1)
        for (int j = i; j < i + span; j++) {
          const int32_t x = a[j], y = a[j + span];
          a[j] = x + y;
          a[j + span] = x - y;
        }
  }
}
template <int N>
int64_t satdN(const int32_t* residual) {
  int32_t t[N * N];
  for (int i = 0; i < N * N; i++) t[i] = residual[i];
  fwhtRows<N>(t);
  // Columns: the same butterflies applied to whole rows at once.
  for (int span = 1; span < N; span <<= 1)
    for (int i = 0; i < N; i += span << 1)
      for (int j = i; j < i + span; j++) {
        int32_t* x = t + j * N;
        int32_t* y = t + (j + span) * N;
        for (int c = 0; c < N; c++) {
          const int32_t a = x[c], b = y[c];
          x[c] = a + b;
          y[c] = a - b;
        }
      }
  int64_t s = 0;
  for (int i = 0; i < N * N; i++) s += t[i] < 0 ? -(int64_t)t[i] : t[i];
  return s;
}
int64_t satd(const int32_t* residual, int n) {
  return n == 4 ? satdN<4>(residual) : (n == 8 ? satdN<8>(residual) : satdN<16>(residual));
}

using CostModel = std::vector<std::vector<double>>;

// coeffRate — ebiv/quant.go:396-402
double coeffRate(int m, int ctx, const CostModel& cost) {
  if (m <= 4) return cost[ctx][tZero + m];
  const int v = m - 5;
  const int len = bitLen((uint64_t)v);
  return cost[ctx][tEscape] + cost[ctxEscClass][len] + (double)std::max(0, len - 1);
}

struct Quantizer {
  Quant q;
  // quantize — dead zone, ebiv/quant.go:55-69
  void quantize(const int32_t* coeffs, int32_t* levels, int n) const {
    for (int i = 0; i < n * n; i++) {
      const int32_t step = i == 0 ? q.dc : q.ac;
      const int32_t c = coeffs[i];
      levels[i] = c >= 0 ? (c * 8 + 3 * step) / (step * 8) : -((-c * 8 + 3 * step) / (step * 8));
    }
  }
  void dequantize(const int32_t* levels, int32_t* coeffs, int n) const {
    for (int i = 0; i < n * n; i++) coeffs[i] = wrapMul(levels[i], i == 0 ? q.dc : q.ac);
  }
  // quantizeRDOQ — ebiv/quant.go:102-198
  void quantizeRDOQ(const int32_t* coeffs, int32_t* levels, int n, int plane, int txIdx, double lambda,
                    const CostModel& cost) const {
    const int* scan = codingTables().scan[txIndexOf(n)];
    const int total = n * n;
    const double signBits = (cost[ctxSign][0] + cost[ctxSign][1]) * 0.5;
    int ctxScan[kMaxLevels];
    int32_t lvlScan[kMaxLevels];
    double dScan[kMaxLevels], rNZScan[kMaxLevels];
    int prevClass = 0;
    for (int si = 0; si < total; si++) {
      const int nat = scan[si];
      const double step = nat == 0 ? (double)q.dc : (double)q.ac;
      const int32_t c = coeffs[nat];
      const double ac = (double)(c < 0 ? -c : c);
      const int ctx = tokenCtx(plane, txIdx, bandOf(si), prevClass);
      ctxScan[si] = ctx;
      const int l0 = (int)((ac + step / 2) / step);
      int bestMag = 0;
      double bestD = ac * ac;
      double bestCost = bestD;
      double bestR = 0.0;
      const int cands[2] = {l0 - 1, l0};
      for (int cand : cands) {
        if (cand < 1) continue;
        double d = ac - (double)cand * step;
        d *= d;
        const double r = coeffRate(cand, ctx, cost) + signBits;
        const double lr = lambda * r;
        const double cst = d + lr;
        if (cst < bestCost) {
          bestCost = cst;
          bestMag = cand;
          bestD = d;
          bestR = r;
        }
      }
      dScan[si] = bestD;
      rNZScan[si] = bestR;
      if (bestMag > 0) {
        lvlScan[si] = c < 0 ? -bestMag : bestMag;
        prevClass = classForMag(bestMag);
      } else {
        lvlScan[si] = 0;
        prevClass = 0;
      }
    }
    double suffixEnergy[kMaxLevels + 1];
    suffixEnergy[total] = 0;
    for (int i = total - 1; i >= 0; i--) {
      const double c = (double)coeffs[scan[i]];
      const double cc = c * c;
      suffixEnergy[i] = suffixEnergy[i + 1] + cc;
    }
    int lastNZ = -1;
    for (int si = 0; si < total; si++)
      if (lvlScan[si] != 0) lastNZ = si;
    int bestT = -1;
    const double eob0 = lambda * cost[ctxScan[0]][tEOB];
    double bestCost = suffixEnergy[0] + eob0;
    double prefD = 0.0, prefR = 0.0;
    for (int t = 0; t <= lastNZ; t++) {
      prefD += dScan[t];
      if (lvlScan[t] != 0)
        prefR += rNZScan[t];
      else
        prefR += cost[ctxScan[t]][tZero];
      const double eob = t < total - 1 ? cost[ctxScan[t + 1]][tEOB] : 0.0;
      const double rate = lambda * (prefR + eob);
      const double cst = (prefD + suffixEnergy[t + 1]) + rate;
      if (cst < bestCost) {
        bestCost = cst;
        bestT = t;
      }
    }
    for (int si = 0; si < total; si++) levels[scan[si]] = si <= bestT ? lvlScan[si] : 0;
  }
};

// ---------------------------------------------------------------------------
// Residual token grammar, encoder half (ebiv/residual.go:30-180, ebiv/mv.go)
// ---------------------------------------------------------------------------
inline int signBit(int32_t c) { return c < 0 ? 1 : 0; }
inline int32_t iabs(int32_t v) { return v < 0 ? -v : v; }

void putRawBits(TokStream& s, uint64_t v, int n) {
  for (int i = n - 1; i >= 0; i--) s.put(ctxBypass, (int)((v >> i) & 1));
}
void putClassValue(TokStream& s, int classCtx, uint64_t v) {
  const int cls = bitLen(v);
  s.put(classCtx, cls);
  if (cls > 1) putRawBits(s, v - (1ull << (cls - 1)), cls - 1);
}
// The left shift is taken on the unsigned value: shifting a negative signed
// value left is undefined before C++20; the bits are the same.
inline uint64_t zigzagEncode(int64_t v) { return ((uint64_t)v << 1) ^ (uint64_t)(v >> 31); }
void putMVComponent(TokStream& s, int classCtx, int delta) { putClassValue(s, classCtx, zigzagEncode(delta)); }

// encodeBlock — ebiv/residual.go:30-75
bool encodeBlock(TokStream& s, int plane, int txIdx, const int32_t* levels, int n) {
  const int* scan = codingTables().scan[txIndexOf(n)];
  const int total = n * n;
  int first = -1, last = -1;
  for (int i = 0; i < total; i++)
    if (levels[scan[i]] != 0) {
      if (first < 0) first = i;
      last = i;
    }
  int prevClass = 0;
  for (int i = 0; i <= last; i++) {
    const int32_t c = levels[scan[i]];
    const int ctx = tokenCtx(plane, txIdx, bandOf(i), prevClass);
    const int mag = iabs(c);
    if (mag == 0) {
      s.put(ctx, tZero);
      prevClass = 0;
    } else if (mag <= 4) {
      s.put(ctx, tZero + mag);
      prevClass = classForMag(mag);
    } else {
      s.put(ctx, tEscape);
      putClassValue(s, ctxEscClass, (uint64_t)(mag - 5));
      prevClass = 2;
    }
    if (mag != 0 && i != first) s.put(ctxSign, signBit(c));
  }
  if (last < total - 1) s.put(tokenCtx(plane, txIdx, bandOf(last + 1), prevClass), tEOB);
  if (first >= 0 && last - first < kSDHMinSpan) s.put(ctxSign, signBit(levels[scan[first]]));
  return last < 0;
}

// applySignDataHiding — ebiv/residual.go:134-180
void applySignDataHiding(int32_t* levels, int n) {
  const int* scan = codingTables().scan[txIndexOf(n)];
  const int total = n * n;
  int first = -1, last = -1;
  int32_t sum = 0;
  for (int i = 0; i < total; i++) {
    const int32_t v = iabs(levels[scan[i]]);
    if (v != 0) {
      if (first < 0) first = i;
      last = i;
      sum += v;
    }
  }
  if (first < 0 || last - first < kSDHMinSpan) return;
  if ((int)(sum & 1) == signBit(levels[scan[first]])) return;
  for (int i = last; i >= first; i--) {
    const int32_t v = levels[scan[i]];
    if (iabs(v) > 1) {
      levels[scan[i]] = v > 0 ? v - 1 : v + 1;
      return;
    }
  }
  for (int i = first + 1; i < last; i++)
    if (levels[scan[i]] == 0) {
      levels[scan[i]] = 1;
      return;
    }
  if (levels[scan[first + 1]] > 0)
    levels[scan[first + 1]]++;
  else
    levels[scan[first + 1]]--;
}

// ---------------------------------------------------------------------------
// Intra prediction (ebiv/predict.go:26-219)
// ---------------------------------------------------------------------------
struct AngMode {
  int angle, invAngle;
  bool vertical;
};
const AngMode kAngModes[kNumIntraModes] = {
    {0, 0, false}, {0, 0, false}, {0, 0, false}, {0, 0, false}, {32, 0, true},
    {13, 0, true}, {-13, -630, true}, {32, 0, false}, {13, 0, false}, {-13, -630, false},
};

bool aboveRightAvailable(int x0, int y0, int n, int tileTopPx, int tileRightPx, int mbTopPx, int mbRightPx) {
  if (y0 <= tileTopPx || x0 + 2 * n > tileRightPx) return false;
  if (y0 == mbTopPx) return true;
  return x0 + 2 * n <= mbRightPx;
}

void predictIntra(const Plane& p, int x0, int y0, int n, int mode, bool avAbove, bool avLeft, bool avAR,
                  int32_t* pred) {
  int32_t ref[4 * kMB + 1];
  bool avail[4 * kMB + 1];
  const int len = 4 * n + 1;
  for (int i = 0; i < len; i++) {
    ref[i] = 0;
    avail[i] = false;
  }
  const int corner = 2 * n;
  if (avLeft)
    for (int i = n; i < 2 * n; i++) {  // rows 0..n-1 of the left column
      ref[i] = p.at(x0 - 1, y0 + (2 * n - 1 - i));
      avail[i] = true;
    }
  if (avAbove && avLeft) {
    ref[corner] = p.at(x0 - 1, y0 - 1);
    avail[corner] = true;
  }
  if (avAbove) {
    const int cnt = avAR ? 2 * n : n;
    for (int j = 0; j < cnt; j++) {
      ref[corner + 1 + j] = p.at(x0 + j, y0 - 1);
      avail[corner + 1 + j] = true;
    }
  }
  // substituteRefs — HEVC-style gap fill
  int first = -1;
  for (int i = 0; i < len; i++)
    if (avail[i]) {
      first = i;
      break;
    }
  if (first < 0) {
    for (int i = 0; i < len; i++) ref[i] = kDCPred;
  } else {
    for (int i = 0; i < first; i++) ref[i] = ref[first];
    for (int i = first + 1; i < len; i++)
      if (!avail[i]) ref[i] = ref[i - 1];
  }
  const int32_t* top = ref + corner + 1;
  switch (mode) {
    case modeV:
      for (int r = 0; r < n; r++)
        for (int c = 0; c < n; c++) pred[r * n + c] = top[c];
      return;
    case modeH:
      for (int r = 0; r < n; r++)
        for (int c = 0; c < n; c++) pred[r * n + c] = ref[corner - 1 - r];
      return;
    case modeTM: {
      const int32_t crn = ref[corner];
      for (int r = 0; r < n; r++)
        for (int c = 0; c < n; c++) pred[r * n + c] = clampByte(top[c] + ref[corner - 1 - r] - crn);
      return;
    }
    case modeDC: {
      int32_t sum = 0;
      for (int i = 0; i < n; i++) sum += top[i] + ref[corner - 1 - i];
      const int32_t dc = (sum + n) / (2 * n);
      for (int i = 0; i < n * n; i++) pred[i] = dc;
      return;
    }
    default:
      break;
  }
  const AngMode& m = kAngModes[mode];
  int32_t ext[3 * kMB + 2];
  std::memset(ext, 0, sizeof(ext));
  const int off = n;
  for (int k = 0; k <= 2 * n; k++) ext[off + k] = m.vertical ? ref[corner + k] : ref[corner - k];
  if (m.angle < 0) {
    const int low = (n * m.angle) >> 5;
    for (int x = -1; x >= low; x--) {
      const int idx = (x * m.invAngle + 128) >> 8;
      ext[off + x] = m.vertical ? ref[corner - idx] : ref[corner + idx];
    }
  }
  for (int a = 0; a < n; a++) {
    const int pos = (a + 1) * m.angle;
    const int idx = pos >> 5, fact = pos & 31;
    for (int b = 0; b < n; b++) {
      const int32_t v = ((32 - fact) * ext[off + b + idx + 1] + fact * ext[off + b + idx + 2] + 16) >> 5;
      if (m.vertical)
        pred[a * n + b] = v;
      else
        pred[b * n + a] = v;
    }
  }
}

// ---------------------------------------------------------------------------
// Motion compensation (ebiv/motioncomp.go:30-256)
// ---------------------------------------------------------------------------
const int32_t kTaps[4][4] = {{0, 64, 0, 0}, {-6, 55, 18, -3}, {-8, 40, 40, -8}, {-3, 18, 55, -6}};
inline int clampC(int v, int hi) { return v < 0 ? 0 : (v >= hi ? hi - 1 : v); }

// One luma prediction sample at integer position (px,py) plus quarter-pel
// phase (fx,fy), reading a clamped reference.
inline int32_t lumaSample(const Plane& r, int px, int py, int fx, int fy) {
  auto g = [&](int x, int y) -> int32_t { return r.at(clampC(x, r.w), clampC(y, r.h)); };
  if (fx == 0 && fy == 0) return g(px, py);
  if (fy == 0) {
    const int32_t* t = kTaps[fx];
    return clampByte((t[0] * g(px - 1, py) + t[1] * g(px, py) + t[2] * g(px + 1, py) + t[3] * g(px + 2, py) + 32) >> 6);
  }
  if (fx == 0) {
    const int32_t* t = kTaps[fy];
    return clampByte((t[0] * g(px, py - 1) + t[1] * g(px, py) + t[2] * g(px, py + 1) + t[3] * g(px, py + 2) + 32) >> 6);
  }
  const int32_t *tx = kTaps[fx], *ty = kTaps[fy];
  int32_t h[4];
  for (int k = 0; k < 4; k++) {
    const int yy = py - 1 + k;
    h[k] = tx[0] * g(px - 1, yy) + tx[1] * g(px, yy) + tx[2] * g(px + 1, yy) + tx[3] * g(px + 2, yy);
  }
  return clampByte((ty[0] * h[0] + ty[1] * h[1] + ty[2] * h[2] + ty[3] * h[3] + 2048) >> 12);
}

void mcLuma(const Plane& r, int srcX, int srcY, int fx, int fy, int pw, int ph, int32_t* out, int dstX, int dstY,
            int dstStride) {
  const bool interior = (fx == 0 && fy == 0)
                            ? (srcX >= 0 && srcY >= 0 && srcX + pw <= r.w && srcY + ph <= r.h)
                            : (srcX - 1 >= 0 && srcY - 1 >= 0 && srcX + pw + 2 <= r.w && srcY + ph + 2 <= r.h);
  if (!interior) {
    for (int y = 0; y < ph; y++)
      for (int x = 0; x < pw; x++) out[(dstY + y) * dstStride + dstX + x] = lumaSample(r, srcX + x, srcY + y, fx, fy);
    return;
  }
  const int st = r.stride;
  for (int y = 0; y < ph; y++) {
    const uint8_t* s = r.d + (size_t)(srcY + y) * st + srcX;
    int32_t* o = out + (dstY + y) * dstStride + dstX;
    if (fx == 0 && fy == 0) {
      for (int x = 0; x < pw; x++) o[x] = s[x];
    } else if (fy == 0) {
      const int32_t* t = kTaps[fx];
      for (int x = 0; x < pw; x++)
        o[x] = clampByte((t[0] * s[x - 1] + t[1] * s[x] + t[2] * s[x + 1] + t[3] * s[x + 2] + 32) >> 6);
    } else if (fx == 0) {
      const int32_t* t = kTaps[fy];
      for (int x = 0; x < pw; x++)
        o[x] = clampByte((t[0] * s[x - st] + t[1] * s[x] + t[2] * s[x + st] + t[3] * s[x + 2 * st] + 32) >> 6);
    } else {
      // Separable: four horizontally filtered rows, then the vertical taps.
      const int32_t *tx = kTaps[fx], *ty = kTaps[fy];
      int32_t h[4][16];
      for (int k = 0; k < 4; k++) {
        const uint8_t* q = s + (k - 1) * st;
        for (int x = 0; x < pw; x++) h[k][x] = tx[0] * q[x - 1] + tx[1] * q[x] + tx[2] * q[x + 1] + tx[3] * q[x + 2];
      }
      for (int x = 0; x < pw; x++)
        o[x] = clampByte((ty[0] * h[0][x] + ty[1] * h[1][x] + ty[2] * h[2][x] + ty[3] * h[3][x] + 2048) >> 12);
    }
  }
}

void mcChroma(const Plane& r, int srcX, int srcY, int fx, int fy, int pw, int ph, int32_t* out, int dstX, int dstY,
              int dstStride) {
  for (int y = 0; y < ph; y++)
    for (int x = 0; x < pw; x++) {
      const int px = srcX + x, py = srcY + y;
      int32_t v;
      auto g = [&](int xx, int yy) -> int32_t { return r.at(clampC(xx, r.w), clampC(yy, r.h)); };
      if (fx == 0 && fy == 0) {
        v = g(px, py);
      } else {
        v = ((8 - fx) * (8 - fy) * g(px, py) + fx * (8 - fy) * g(px + 1, py) + (8 - fx) * fy * g(px, py + 1) +
             fx * fy * g(px + 1, py + 1) + 32) >> 6;
      }
      out[(dstY + y) * dstStride + dstX + x] = v;
    }
}

inline int16_t clampMV(int v) { return (int16_t)(v < -kMVClampRange ? -kMVClampRange : (v > kMVClampRange ? kMVClampRange : v)); }

inline int16_t median3(int16_t a, int16_t b, int16_t c) {
  if (a > b) std::swap(a, b);
  if (b > c) b = c;
  if (a > b) b = a;
  return b;
}

struct TileB {
  int x0, x1, y0, y1;
};

// predictMV — ebiv/mv.go:21-52
MotionVector predictMV(const MotionVector* mv, int stride, int mbx, int mby, const TileB& b) {
  MotionVector a, bv, c;
  const bool aOK = mbx > b.x0, bOK = mby > b.y0;
  bool cOK = false;
  if (aOK) a = mv[mby * stride + mbx - 1];
  if (bOK) {
    bv = mv[(mby - 1) * stride + mbx];
    if (mbx + 1 < b.x1) {
      c = mv[(mby - 1) * stride + mbx + 1];
      cOK = true;
    } else if (aOK) {
      c = mv[(mby - 1) * stride + mbx - 1];
      cOK = true;
    }
  }
  if (!aOK && !bOK && !cOK) return MotionVector{};
  if (aOK && !bOK && !cOK) return a;
  if (!aOK && bOK && !cOK) return bv;
  MotionVector r;
  r.x = median3(a.x, bv.x, c.x);
  r.y = median3(a.y, bv.y, c.y);
  return r;
}

// ---------------------------------------------------------------------------
// Frame encoder (ebiv/encode_intra.go:33-447, ebiv/encode_inter.go)
// ---------------------------------------------------------------------------
struct MBSearchCache {
  MotionVector last[kNumPartModes][4];
  MotionVector golden;
  bool trySubs = false, tryGolden = false;
};

struct BlockScratch {
  int32_t pred[kMaxLevels], residual[kMaxLevels], coeffs[kMaxLevels], levels[kMaxLevels], recon[kMaxLevels];
};

// estimateBits — ebiv/encode_intra.go:421-447
int estimateBits(const std::vector<Tok>& toks) {
  int bits = 0;
  for (const Tok& t : toks) {
    if (t.ctx >= ctxTokenBase) {
      switch (t.sym) {
        case tEOB: bits += 2; break;
        case tZero: bits += 1; break;
        case tEscape: bits += 6; break;
        default: bits += 4;
      }
    } else if (t.ctx == ctxSign || t.ctx == ctxBypass) {
      bits++;
    } else if (t.ctx == ctxMVClassX || t.ctx == ctxMVClassY || t.ctx == ctxEscClass) {
      bits += 3;
    } else if (t.ctx == ctxMBMode || t.ctx == ctxCBP) {
      bits += 2;
    } else {
      bits += 3;
    }
  }
  return bits;
}

struct FrameEncoder;

struct TileEncoder {
  FrameEncoder* fe;
  BlockScratch sc;
  TokStream lumaToks, cbToks, crToks;
  uint64_t sadCount = 0;
  uint64_t fallbacks = 0;  // proposed searches decided by the exhaustive search
  uint64_t searchNs = 0;   // thread time spent in motion search
  explicit TileEncoder(FrameEncoder* f) : fe(f) {}

  int rdBits(const std::vector<Tok>& toks) const;
  void encodeIntraTile(TokStream& s, const TileB& b);
  void encodeInterTile(TokStream& s, const TileB& b);
  void encodeLumaMB(TokStream& s, int mbx, int mby, const TileB& b);
  int64_t lumaMBCost(int mbx, int mby, const TileB& b, int txIdx);
  int64_t codeLumaMB(TokStream& s, int mbx, int mby, const TileB& b, int txIdx);
  void encodeChromaMB(TokStream& s, int mbx, int mby, const TileB& b);
  int64_t codeBlock(TokStream& s, int plane, int txIdx, const Plane& src, const Plane& rec, int x0, int y0, int n,
                    int mode, bool avAbove, bool avLeft, bool avAR);
  int64_t codeResidual(TokStream& s, int plane, int txIdx, const Plane& src, const Plane& rec, int x0, int y0, int n);
  int chooseIntraMode(const Plane& src, const Plane& rec, int x0, int y0, int n, bool avAbove, bool avLeft, bool avAR);
  int64_t predErr(const Plane& src, const Plane& rec, int x0, int y0, int n, int mode, bool avAbove, bool avLeft,
                  bool avAR);
  void encodeInterMB(TokStream& s, int mbx, int mby, const TileB& b);
  int64_t codeLumaMBBest(TokStream& s, int mbx, int mby, const TileB& b);
  int64_t encodeChromaMBTo(TokStream& s, int mbx, int mby, const TileB& b);
  int64_t mcMBSSE(const Frame* ref, int mbx, int mby, MotionVector mv);
  void reconMC(int mbx, int mby, MotionVector mv);
  int64_t codeInterMB(TokStream& s, const Frame* ref, int mbx, int mby, int part, const MotionVector* mvs,
                      MotionVector pred);
  int64_t codeInterLuma(TokStream& s, int mbx, int mby, const int32_t* mc, int txIdx);
  MotionVector searchMVRect(const Frame* ref, int mbx, int mby, int px, int py, int pw, int ph, MotionVector pred);
  MotionVector searchExhaustive(const Frame* ref, int mbx, int mby, int px, int py, int pw, int ph, MotionVector pred);
  MotionVector searchProposed(const Frame* ref, int mbx, int mby, int px, int py, int pw, int ph, MotionVector pred);
  MotionVector search(const Frame* ref, int mbx, int mby, int px, int py, int pw, int ph, MotionVector pred);
  MotionVector searchOnce(const Frame* ref, int mbx, int mby, int px, int py, int pw, int ph, MotionVector pred);
  int64_t rectSAD(const Frame* ref, int mbx, int mby, int px, int py, int pw, int ph, MotionVector mv);
};

struct FrameEncoder {
  Geometry g;
  std::unique_ptr<Frame> src, rec;
  const Frame* ref = nullptr;
  const Frame* golden = nullptr;
  Quantizer q;
  TileGrid grid;
  std::vector<TokStream> streams;
  std::vector<std::vector<uint32_t>> counts;
  int64_t lambda = 0;
  double lambdaF = 0;
  CostModel rdoq;  // empty in pass 1
  bool haveRDOQ = false;
  std::vector<MotionVector> mv;
  int mvStride = 0;
  std::vector<MBSearchCache> mvSearch;
  WorkerPool* pool = nullptr;
  SearchMode search = SearchMode::Diamond;
  int exhaustiveRange = 16;
  int fallbackSAD = 0;
  const MVProposer* proposer = nullptr;
  std::atomic<uint64_t> sadCount{0};
  std::atomic<uint64_t> fallbacks{0};
  std::atomic<uint64_t> searchNs{0};

  // newFrameEncoder — ebiv/encode_intra.go:89-118
  FrameEncoder(const Geometry& geo, const PackedImage& img, const Frame* r, const Frame* gold, int qp, int tc, int tr)
      : g(geo), ref(r), golden(gold) {
    src.reset(new Frame(g));
    loadImage(*src, img);
    rec.reset(new Frame(g));
    q.q = quantFor(qp);
    grid = TileGrid(g.mbCols, g.mbRows, tc, tr);
    mv.assign((size_t)g.mbCols * g.mbRows, MotionVector{});
    mvStride = g.mbCols;
    const int64_t qac = q.q.ac;
    lambda = qac * qac / 6;
    lambdaF = (double)lambda;
    if (ref) mvSearch.assign((size_t)g.mbCols * g.mbRows, MBSearchCache{});
    counts.resize(kNumContexts);
    for (int c = 0; c < kNumContexts; c++) counts[c].assign((size_t)alphabetSize(c), 0);
  }

  void encodeTilesParallel(bool inter) {
    streams.assign((size_t)grid.count(), TokStream{});
    auto fn = [&](int i) {
      TileEncoder te(this);
      TileB b;
      grid.bounds(i, &b.x0, &b.x1, &b.y0, &b.y1);
      if (inter)
        te.encodeInterTile(streams[(size_t)i], b);
      else
        te.encodeIntraTile(streams[(size_t)i], b);
      sadCount += te.sadCount;
      fallbacks += te.fallbacks;
      searchNs += te.searchNs;
    };
    if (pool)
      pool->run(grid.count(), fn);
    else
      for (int i = 0; i < grid.count(); i++) fn(i);
  }

  // encode — ebiv/encode_intra.go:187-195
  void encode(bool inter, bool twoPass) {
    encodeTilesParallel(inter);
    if (!twoPass) return;
    rdoq = measureCosts();
    haveRDOQ = true;
    rec.reset(new Frame(g));  // resetForPass2
    streams.clear();
    for (auto& c : counts) std::fill(c.begin(), c.end(), 0u);
    std::fill(mv.begin(), mv.end(), MotionVector{});
    encodeTilesParallel(inter);
  }

  // measureCosts — ebiv/encode_intra.go:200-227
  CostModel measureCosts() const {
    std::vector<std::vector<uint32_t>> cnt(kNumContexts);
    for (int c = 0; c < kNumContexts; c++) cnt[c].assign((size_t)alphabetSize(c), 0);
    for (const auto& s : streams)
      for (const Tok& t : s.toks) cnt[t.ctx][t.sym]++;
    CostModel cost(kNumContexts);
    for (int c = 0; c < kNumContexts; c++) {
      const Freqs f = normalizeFreqs(cnt[c]);
      cost[c].assign((size_t)alphabetSize(c), 0.0);
      for (int s = 0; s < alphabetSize(c); s++) {
        const uint32_t fv = f.empty() ? 0 : f[s];
        cost[c][s] = fv == 0 ? 20.0 : std::log2((double)kM / (double)fv);
      }
    }
    return cost;
  }

  // finish — ebiv/encode_intra.go:144-168
  std::vector<uint8_t> finish(int qp, const std::vector<Freqs>* prev, std::vector<Freqs>* freqsOut) {
    for (const auto& s : streams)
      for (const Tok& t : s.toks) counts[t.ctx][t.sym]++;
    std::vector<Freqs> freqs(kNumContexts);
    std::vector<EncTable> tables(kNumContexts);
    for (int c = 0; c < kNumContexts; c++) {
      if (c == ctxBypass) continue;
      freqs[c] = normalizeFreqs(counts[c]);
      tables[c] = buildEncTable(freqs[c].empty() ? Freqs((size_t)alphabetSize(c), 0) : freqs[c], alphabetSize(c));
    }
    tables[ctxBypass] = buildEncTable(Freqs{kM / 2, kM / 2}, 2);
    const std::vector<uint8_t> tableBytes = serializeTables(freqs, prev);
    std::vector<std::vector<uint8_t>> tiles(streams.size());
    auto enc = [&](int i) { tiles[(size_t)i] = ransEncode(streams[(size_t)i].toks, tables); };
    if (pool)
      pool->run((int)streams.size(), enc);
    else
      for (int i = 0; i < (int)streams.size(); i++) enc(i);
    // assemblePayload — ebiv/frame.go:224-236
    std::vector<uint8_t> out;
    out.push_back((uint8_t)qp);
    putUvarint(out, (uint64_t)grid.cols);
    putUvarint(out, (uint64_t)grid.rows);
    putUvarint(out, tableBytes.size());
    out.insert(out.end(), tableBytes.begin(), tableBytes.end());
    for (const auto& t : tiles) {
      putUvarint(out, t.size());
      out.insert(out.end(), t.begin(), t.end());
    }
    *freqsOut = std::move(freqs);
    return out;
  }
};

int TileEncoder::rdBits(const std::vector<Tok>& toks) const {
  if (fe->haveRDOQ) {
    double b = 0;
    for (const Tok& t : toks) b += fe->rdoq[t.ctx][t.sym];
    return (int)(b + 0.5);
  }
  return estimateBits(toks);
}

void TileEncoder::encodeIntraTile(TokStream& s, const TileB& b) {
  for (int mby = b.y0; mby < b.y1; mby++)
    for (int mbx = b.x0; mbx < b.x1; mbx++) {
      encodeLumaMB(s, mbx, mby, b);
      encodeChromaMB(s, mbx, mby, b);
    }
}

// encodeLumaMB — ebiv/encode_intra.go:264-274
void TileEncoder::encodeLumaMB(TokStream& s, int mbx, int mby, const TileB& b) {
  int bestTx = 0;
  int64_t bestCost = int64_t(1) << 62;
  for (int tx = 0; tx < 3; tx++) {
    const int64_t c = lumaMBCost(mbx, mby, b, tx);
    if (c < bestCost) {
      bestCost = c;
      bestTx = tx;
    }
  }
  s.put(ctxTxSize, bestTx);
  codeLumaMB(s, mbx, mby, b, bestTx);
}

int64_t TileEncoder::lumaMBCost(int mbx, int mby, const TileB& b, int txIdx) {
  TokStream trial;
  const int64_t sse = codeLumaMB(trial, mbx, mby, b, txIdx);
  return sse + fe->lambda * (int64_t)rdBits(trial.toks);
}

// codeLumaMB — ebiv/encode_intra.go:288-309
int64_t TileEncoder::codeLumaMB(TokStream& s, int mbx, int mby, const TileB& b, int txIdx) {
  const int n = kLumaTx[txIdx];
  const int tileLeft = b.x0 * kMB, tileTop = b.y0 * kMB, tileRight = b.x1 * kMB;
  const int mbTop = mby * kMB, mbRight = (mbx + 1) * kMB;
  int64_t sse = 0;
  for (int by = 0; by < kMB; by += n)
    for (int bx = 0; bx < kMB; bx += n) {
      const int x0 = mbx * kMB + bx, y0 = mby * kMB + by;
      const bool avAbove = y0 > tileTop, avLeft = x0 > tileLeft;
      const bool avAR = aboveRightAvailable(x0, y0, n, tileTop, tileRight, mbTop, mbRight);
      const int mode = chooseIntraMode(fe->src->y, fe->rec->y, x0, y0, n, avAbove, avLeft, avAR);
      s.put(ctxLumaMode, mode);
      sse += codeBlock(s, kPlaneLuma, txIdx, fe->src->y, fe->rec->y, x0, y0, n, mode, avAbove, avLeft, avAR);
    }
  return sse;
}

// encodeChromaMB — ebiv/encode_intra.go:311-334
void TileEncoder::encodeChromaMB(TokStream& s, int mbx, int mby, const TileB& b) {
  const int tileLeft = b.x0 * kCMB, tileTop = b.y0 * kCMB;
  const int x0 = mbx * kCMB, y0 = mby * kCMB;
  const bool avAbove = y0 > tileTop, avLeft = x0 > tileLeft;
  int best = modeDC;
  int64_t bestErr = int64_t(1) << 62;
  for (int mode = 0; mode < kNumIntraModes; mode++) {
    const int64_t e = predErr(fe->src->cb, fe->rec->cb, x0, y0, kCMB, mode, avAbove, avLeft, false) +
                      predErr(fe->src->cr, fe->rec->cr, x0, y0, kCMB, mode, avAbove, avLeft, false);
    if (e < bestErr) {
      bestErr = e;
      best = mode;
    }
  }
  s.put(ctxChromaMode, best);
  codeBlock(s, kPlaneChroma, 0, fe->src->cb, fe->rec->cb, x0, y0, kCMB, best, avAbove, avLeft, false);
  codeBlock(s, kPlaneChroma, 0, fe->src->cr, fe->rec->cr, x0, y0, kCMB, best, avAbove, avLeft, false);
}

int64_t TileEncoder::codeBlock(TokStream& s, int plane, int txIdx, const Plane& src, const Plane& rec, int x0, int y0,
                               int n, int mode, bool avAbove, bool avLeft, bool avAR) {
  predictIntra(rec, x0, y0, n, mode, avAbove, avLeft, avAR, sc.pred);
  return codeResidual(s, plane, txIdx, src, rec, x0, y0, n);
}

// codeResidual — ebiv/encode_intra.go:346-376
int64_t TileEncoder::codeResidual(TokStream& s, int plane, int txIdx, const Plane& src, const Plane& rec, int x0,
                                  int y0, int n) {
  for (int r = 0; r < n; r++)
    for (int c = 0; c < n; c++) sc.residual[r * n + c] = (int32_t)src.at(x0 + c, y0 + r) - sc.pred[r * n + c];
  forwardDCT(sc.residual, sc.coeffs, n);
  if (fe->haveRDOQ)
    fe->q.quantizeRDOQ(sc.coeffs, sc.levels, n, plane, txIdx, fe->lambdaF, fe->rdoq);
  else
    fe->q.quantize(sc.coeffs, sc.levels, n);
  applySignDataHiding(sc.levels, n);
  encodeBlock(s, plane, txIdx, sc.levels, n);
  fe->q.dequantize(sc.levels, sc.coeffs, n);
  inverseDCT(sc.coeffs, sc.recon, n);
  int64_t sse = 0;
  for (int r = 0; r < n; r++)
    for (int c = 0; c < n; c++) {
      const int32_t rv = clampByte(wrapAdd(sc.pred[r * n + c], sc.recon[r * n + c]));
      rec.set(x0 + c, y0 + r, (uint8_t)rv);
      const int64_t d = (int64_t)rv - (int64_t)src.at(x0 + c, y0 + r);
      sse += d * d;
    }
  return sse;
}

int TileEncoder::chooseIntraMode(const Plane& src, const Plane& rec, int x0, int y0, int n, bool avAbove, bool avLeft,
                                 bool avAR) {
  int best = modeDC;
  int64_t bestErr = int64_t(1) << 62;
  for (int mode = 0; mode < kNumIntraModes; mode++) {
    const int64_t e = predErr(src, rec, x0, y0, n, mode, avAbove, avLeft, avAR);
    if (e < bestErr) {
      bestErr = e;
      best = mode;
    }
  }
  return best;
}

int64_t TileEncoder::predErr(const Plane& src, const Plane& rec, int x0, int y0, int n, int mode, bool avAbove,
                             bool avLeft, bool avAR) {
  predictIntra(rec, x0, y0, n, mode, avAbove, avLeft, avAR, sc.pred);
  for (int r = 0; r < n; r++)
    for (int c = 0; c < n; c++) sc.residual[r * n + c] = (int32_t)src.at(x0 + c, y0 + r) - sc.pred[r * n + c];
  return satd(sc.residual, n);
}

void TileEncoder::encodeInterTile(TokStream& s, const TileB& b) {
  for (int mby = b.y0; mby < b.y1; mby++)
    for (int mbx = b.x0; mbx < b.x1; mbx++) encodeInterMB(s, mbx, mby, b);
}

// encodeInterMB — ebiv/encode_inter.go:37-163
void TileEncoder::encodeInterMB(TokStream& s, int mbx, int mby, const TileB& b) {
  const int idx = mby * fe->mvStride + mbx;
  const int64_t lambda = fe->lambda;
  const MotionVector pred = predictMV(fe->mv.data(), fe->mvStride, mbx, mby, b);
  const int64_t skipSSE = mcMBSSE(fe->ref, mbx, mby, pred);
  const int64_t skipCost = skipSSE + lambda * 2;
  if (skipSSE <= lambda * 8) {
    s.put(ctxMBMode, mbSkip);
    reconMC(mbx, mby, pred);
    fe->mv[idx] = pred;
    return;
  }
  MBSearchCache& cache = fe->mvSearch[idx];
  const bool pass2 = fe->haveRDOQ;
  int bestPart = partWhole;
  MotionVector bestMVs[4];
  if (!pass2) cache.last[partWhole][0] = search(fe->ref, mbx, mby, 0, 0, kMB, kMB, pred);
  bestMVs[0] = cache.last[partWhole][0];
  int64_t bestInterCost;
  {
    TokStream trial;
    const int64_t sse = codeInterMB(trial, fe->ref, mbx, mby, partWhole, bestMVs, pred);
    bestInterCost = sse + lambda * (int64_t)(rdBits(trial.toks) + 3);
  }
  if (!pass2) {
    const int64_t wholeSAD = rectSAD(fe->ref, mbx, mby, 0, 0, kMB, kMB, bestMVs[0]);
    cache.trySubs = wholeSAD > 2 * kMB * kMB;
    cache.tryGolden = fe->golden != nullptr && rectSAD(fe->golden, mbx, mby, 0, 0, kMB, kMB, MotionVector{}) < wholeSAD;
    if (cache.tryGolden) cache.golden = search(fe->golden, mbx, mby, 0, 0, kMB, kMB, MotionVector{});
  }
  if (cache.trySubs) {
    for (int part = partWhole + 1; part < kNumPartModes; part++) {
      const Rect4* rects = partRects(part);
      MotionVector mvs[4];
      for (int i = 0; i < kPartCount[part]; i++) {
        if (pass2) {
          mvs[i] = cache.last[part][i];
          continue;
        }
        const MotionVector pp = i > 0 ? mvs[0] : pred;
        mvs[i] = search(fe->ref, mbx, mby, rects[i].x, rects[i].y, rects[i].w, rects[i].h, pp);
        cache.last[part][i] = mvs[i];
      }
      TokStream trial;
      const int64_t sse = codeInterMB(trial, fe->ref, mbx, mby, part, mvs, pred);
      const int64_t cost = sse + lambda * (int64_t)(rdBits(trial.toks) + 3);
      if (cost < bestInterCost) {
        bestInterCost = cost;
        bestPart = part;
        for (int k = 0; k < 4; k++) bestMVs[k] = mvs[k];
      }
    }
  }
  int64_t goldenCost = int64_t(1) << 62;
  MotionVector goldenMV;
  if (cache.tryGolden) {
    const MotionVector gmv = cache.golden;
    TokStream trial;
    const int64_t sse = codeInterMB(trial, fe->golden, mbx, mby, partWhole, &gmv, MotionVector{});
    goldenCost = sse + lambda * (int64_t)(rdBits(trial.toks) + 3);
    goldenMV = gmv;
  }
  int64_t intraCost = int64_t(1) << 62;
  if (bestInterCost > lambda * 32) {
    TokStream intraTok;
    const int64_t intraSSE = codeLumaMBBest(intraTok, mbx, mby, b) + encodeChromaMBTo(intraTok, mbx, mby, b);
    intraCost = intraSSE + lambda * (int64_t)(rdBits(intraTok.toks) + 2);
  }
  if (skipCost <= bestInterCost && skipCost <= intraCost && skipCost <= goldenCost) {
    s.put(ctxMBMode, mbSkip);
    reconMC(mbx, mby, pred);
    fe->mv[idx] = pred;
  } else if (goldenCost < bestInterCost && goldenCost <= intraCost) {
    s.put(ctxMBMode, mbInter);
    s.put(ctxRef, refGolden);
    codeInterMB(s, fe->golden, mbx, mby, partWhole, &goldenMV, MotionVector{});
    fe->mv[idx] = MotionVector{};
  } else if (bestInterCost <= intraCost) {
    s.put(ctxMBMode, mbInter);
    s.put(ctxRef, refLast);
    codeInterMB(s, fe->ref, mbx, mby, bestPart, bestMVs, pred);
    fe->mv[idx] = bestMVs[0];
  } else {
    s.put(ctxMBMode, mbIntra);
    encodeLumaMB(s, mbx, mby, b);
    encodeChromaMB(s, mbx, mby, b);
    fe->mv[idx] = MotionVector{};
  }
}

int64_t TileEncoder::codeLumaMBBest(TokStream& s, int mbx, int mby, const TileB& b) {
  int bestTx = 0;
  int64_t bestCost = int64_t(1) << 62;
  for (int tx = 0; tx < 3; tx++) {
    const int64_t c = lumaMBCost(mbx, mby, b, tx);
    if (c < bestCost) {
      bestCost = c;
      bestTx = tx;
    }
  }
  s.put(ctxTxSize, bestTx);
  return codeLumaMB(s, mbx, mby, b, bestTx);
}

int64_t TileEncoder::encodeChromaMBTo(TokStream& s, int mbx, int mby, const TileB& b) {
  encodeChromaMB(s, mbx, mby, b);
  const int x0 = mbx * kCMB, y0 = mby * kCMB;
  int64_t sse = 0;
  for (int r = 0; r < kCMB; r++)
    for (int c = 0; c < kCMB; c++) {
      int64_t d = (int64_t)fe->src->cb.at(x0 + c, y0 + r) - fe->rec->cb.at(x0 + c, y0 + r);
      sse += d * d;
    }
  for (int r = 0; r < kCMB; r++)
    for (int c = 0; c < kCMB; c++) {
      int64_t d = (int64_t)fe->src->cr.at(x0 + c, y0 + r) - fe->rec->cr.at(x0 + c, y0 + r);
      sse += d * d;
    }
  return sse;
}

// mcMBSSE — ebiv/encode_inter.go:202-231
int64_t TileEncoder::mcMBSSE(const Frame* ref, int mbx, int mby, MotionVector mv) {
  int32_t mcY[256];
  mcLuma(ref->y, mbx * kMB + (mv.x >> 2), mby * kMB + (mv.y >> 2), mv.x & 3, mv.y & 3, kMB, kMB, mcY, 0, 0, kMB);
  int64_t sse = 0;
  const int x0 = mbx * kMB, y0 = mby * kMB;
  for (int r = 0; r < kMB; r++)
    for (int c = 0; c < kMB; c++) {
      const int64_t d = (int64_t)fe->src->y.at(x0 + c, y0 + r) - mcY[r * kMB + c];
      sse += d * d;
    }
  int32_t mcC[64];
  const int cx = mbx * kCMB, cy = mby * kCMB;
  mcChroma(ref->cb, cx + (mv.x >> 3), cy + (mv.y >> 3), mv.x & 7, mv.y & 7, kCMB, kCMB, mcC, 0, 0, kCMB);
  for (int r = 0; r < kCMB; r++)
    for (int c = 0; c < kCMB; c++) {
      const int64_t d = (int64_t)fe->src->cb.at(cx + c, cy + r) - mcC[r * kCMB + c];
      sse += d * d;
    }
  mcChroma(ref->cr, cx + (mv.x >> 3), cy + (mv.y >> 3), mv.x & 7, mv.y & 7, kCMB, kCMB, mcC, 0, 0, kCMB);
  for (int r = 0; r < kCMB; r++)
    for (int c = 0; c < kCMB; c++) {
      const int64_t d = (int64_t)fe->src->cr.at(cx + c, cy + r) - mcC[r * kCMB + c];
      sse += d * d;
    }
  return sse;
}

// reconMC / writeMC — ebiv/encode_inter.go:235-260
void TileEncoder::reconMC(int mbx, int mby, MotionVector mv) {
  int32_t mcY[256];
  mcLuma(fe->ref->y, mbx * kMB + (mv.x >> 2), mby * kMB + (mv.y >> 2), mv.x & 3, mv.y & 3, kMB, kMB, mcY, 0, 0, kMB);
  for (int r = 0; r < kMB; r++)
    for (int c = 0; c < kMB; c++) fe->rec->y.set(mbx * kMB + c, mby * kMB + r, clampByte(mcY[r * kMB + c]));
  int32_t mcC[64];
  const int cx = mbx * kCMB, cy = mby * kCMB;
  mcChroma(fe->ref->cb, cx + (mv.x >> 3), cy + (mv.y >> 3), mv.x & 7, mv.y & 7, kCMB, kCMB, mcC, 0, 0, kCMB);
  for (int r = 0; r < kCMB; r++)
    for (int c = 0; c < kCMB; c++) fe->rec->cb.set(cx + c, cy + r, clampByte(mcC[r * kCMB + c]));
  mcChroma(fe->ref->cr, cx + (mv.x >> 3), cy + (mv.y >> 3), mv.x & 7, mv.y & 7, kCMB, kCMB, mcC, 0, 0, kCMB);
  for (int r = 0; r < kCMB; r++)
    for (int c = 0; c < kCMB; c++) fe->rec->cr.set(cx + c, cy + r, clampByte(mcC[r * kCMB + c]));
}

// allZeroBlocks — ebiv/encode_inter.go:346-353
bool allZeroBlocks(const TokStream& s) {
  for (const Tok& t : s.toks)
    if (t.sym != tEOB || (int)t.ctx < ctxTokenBase) return false;
  return true;
}

// codeInterMB — ebiv/encode_inter.go:267-342
int64_t TileEncoder::codeInterMB(TokStream& s, const Frame* ref, int mbx, int mby, int part, const MotionVector* mvs,
                                 MotionVector pred) {
  const Rect4* rects = partRects(part);
  const int np = kPartCount[part];
  s.put(ctxPart, part);
  for (int i = 0; i < np; i++) {
    const MotionVector pp = i > 0 ? mvs[0] : pred;
    putMVComponent(s, ctxMVClassX, (int)mvs[i].x - (int)pp.x);
    putMVComponent(s, ctxMVClassY, (int)mvs[i].y - (int)pp.y);
  }
  int32_t mcY[256];
  for (int i = 0; i < np; i++) {
    const Rect4& rc = rects[i];
    mcLuma(ref->y, mbx * kMB + rc.x + (mvs[i].x >> 2), mby * kMB + rc.y + (mvs[i].y >> 2), mvs[i].x & 3,
           mvs[i].y & 3, rc.w, rc.h, mcY, rc.x, rc.y, kMB);
  }
  const int cx = mbx * kCMB, cy = mby * kCMB;
  int32_t mcCb[64], mcCr[64];
  for (int i = 0; i < np; i++) {
    const Rect4& rc = rects[i];
    const int cpx = rc.x / 2, cpy = rc.y / 2, cpw = rc.w / 2, cph = rc.h / 2;
    mcChroma(ref->cb, cx + cpx + (mvs[i].x >> 3), cy + cpy + (mvs[i].y >> 3), mvs[i].x & 7, mvs[i].y & 7, cpw, cph,
             mcCb, cpx, cpy, kCMB);
    mcChroma(ref->cr, cx + cpx + (mvs[i].x >> 3), cy + cpy + (mvs[i].y >> 3), mvs[i].x & 7, mvs[i].y & 7, cpw, cph,
             mcCr, cpx, cpy, kCMB);
  }
  int bestTx = 0;
  int64_t bestCost = int64_t(1) << 62;
  for (int tx = 0; tx < 3; tx++) {
    TokStream trial;
    const int64_t sse = codeInterLuma(trial, mbx, mby, mcY, tx);
    const int64_t cost = sse + fe->lambda * (int64_t)rdBits(trial.toks);
    if (cost < bestCost) {
      bestCost = cost;
      bestTx = tx;
    }
  }
  lumaToks.toks.clear();
  int64_t sse = codeInterLuma(lumaToks, mbx, mby, mcY, bestTx);
  const bool lumaZero = allZeroBlocks(lumaToks);
  cbToks.toks.clear();
  std::memcpy(sc.pred, mcCb, sizeof(mcCb));
  sse += codeResidual(cbToks, kPlaneChroma, 0, fe->src->cb, fe->rec->cb, cx, cy, kCMB);
  const bool cbZero = allZeroBlocks(cbToks);
  crToks.toks.clear();
  std::memcpy(sc.pred, mcCr, sizeof(mcCr));
  sse += codeResidual(crToks, kPlaneChroma, 0, fe->src->cr, fe->rec->cr, cx, cy, kCMB);
  const bool crZero = allZeroBlocks(crToks);
  int cbp = 0;
  if (!lumaZero) cbp |= cbpLuma;
  if (!cbZero) cbp |= cbpCb;
  if (!crZero) cbp |= cbpCr;
  s.put(ctxCBP, cbp);
  if (!lumaZero) {
    s.put(ctxTxSize, bestTx);
    s.toks.insert(s.toks.end(), lumaToks.toks.begin(), lumaToks.toks.end());
  }
  if (!cbZero) s.toks.insert(s.toks.end(), cbToks.toks.begin(), cbToks.toks.end());
  if (!crZero) s.toks.insert(s.toks.end(), crToks.toks.begin(), crToks.toks.end());
  return sse;
}

int64_t TileEncoder::codeInterLuma(TokStream& s, int mbx, int mby, const int32_t* mc, int txIdx) {
  const int n = kLumaTx[txIdx];
  int64_t sse = 0;
  for (int by = 0; by < kMB; by += n)
    for (int bx = 0; bx < kMB; bx += n) {
      for (int r = 0; r < n; r++)
        for (int c = 0; c < n; c++) sc.pred[r * n + c] = mc[(by + r) * kMB + bx + c];
      sse += codeResidual(s, kPlaneLuma, txIdx, fe->src->y, fe->rec->y, mbx * kMB + bx, mby * kMB + by, n);
    }
  return sse;
}

MotionVector TileEncoder::search(const Frame* ref, int mbx, int mby, int px, int py, int pw, int ph,
                                 MotionVector pred) {
  const auto t0 = std::chrono::steady_clock::now();
  const MotionVector m = searchOnce(ref, mbx, mby, px, py, pw, ph, pred);
  searchNs += (uint64_t)std::chrono::duration_cast<std::chrono::nanoseconds>(std::chrono::steady_clock::now() - t0)
                  .count();
  return m;
}

MotionVector TileEncoder::searchOnce(const Frame* ref, int mbx, int mby, int px, int py, int pw, int ph,
                                     MotionVector pred) {
  switch (fe->search) {
    case SearchMode::Exhaustive:
      return searchExhaustive(ref, mbx, mby, px, py, pw, ph, pred);
    case SearchMode::Proposed:
      if (fe->proposer && ref == fe->ref) return searchProposed(ref, mbx, mby, px, py, pw, ph, pred);
      return searchMVRect(ref, mbx, mby, px, py, pw, ph, pred);
    default:
      return searchMVRect(ref, mbx, mby, px, py, pw, ph, pred);
  }
}

// searchMVRect — ebiv/encode_inter.go:381-419 (diamond + half/quarter refine)
MotionVector TileEncoder::searchMVRect(const Frame* ref, int mbx, int mby, int px, int py, int pw, int ph,
                                       MotionVector pred) {
  MotionVector best;
  int64_t bestSAD = rectSAD(ref, mbx, mby, px, py, pw, ph, best);
  auto consider = [&](MotionVector m) {
    const int64_t sad = rectSAD(ref, mbx, mby, px, py, pw, ph, m);
    if (sad < bestSAD) {
      bestSAD = sad;
      best = m;
      return true;
    }
    return false;
  };
  consider(pred);
  for (int step = 16; step >= 1; step >>= 1) {
    for (;;) {
      const int cx = best.x, cy = best.y;
      const bool moved = consider({clampMV(cx + step * 4), clampMV(cy)}) ||
                         consider({clampMV(cx - step * 4), clampMV(cy)}) ||
                         consider({clampMV(cx), clampMV(cy + step * 4)}) ||
                         consider({clampMV(cx), clampMV(cy - step * 4)});
      if (!moved) break;
    }
  }
  const int subs[2] = {2, 1};
  for (int sub : subs) {
    const int bx = best.x, by = best.y;
    for (int dy = -1; dy <= 1; dy++)
      for (int dx = -1; dx <= 1; dx++) consider({clampMV(bx + dx * sub), clampMV(by + dy * sub)});
  }
  return best;
}

// Exhaustive full-pel search over +-range pixels around zero and the
// predictor, then the same half/quarter-pel refinement as the diamond.  It is
// the reference search the learned proposer is trained and evaluated against.
MotionVector TileEncoder::searchExhaustive(const Frame* ref, int mbx, int mby, int px, int py, int pw, int ph,
                                           MotionVector pred) {
  MotionVector best;
  int64_t bestSAD = rectSAD(ref, mbx, mby, px, py, pw, ph, best);
  auto consider = [&](MotionVector m) {
    const int64_t sad = rectSAD(ref, mbx, mby, px, py, pw, ph, m);
    if (sad < bestSAD) {
      bestSAD = sad;
      best = m;
    }
  };
  consider(pred);
  const int R = fe->exhaustiveRange;
  for (int dy = -R; dy <= R; dy++)
    for (int dx = -R; dx <= R; dx++) consider({clampMV(dx * 4), clampMV(dy * 4)});
  const int subs[2] = {2, 1};
  for (int sub : subs) {
    const int bx = best.x, by = best.y;
    for (int dy = -1; dy <= 1; dy++)
      for (int dx = -1; dx <= 1; dx++) consider({clampMV(bx + dx * sub), clampMV(by + dy * sub)});
  }
  return best;
}

// Candidate search: zero, the predictor and the proposer's full-pel
// candidates for the macroblock (used for every partition of it), each
// candidate with its one-pixel full-pel neighbourhood (the proposals are
// 2-pixel bins), a one-pixel polish around the best, then the same
// half/quarter-pel refinement as the diamond.  When the best SAD stays above
// fallbackSAD per 256 pixels the exhaustive search decides instead.
MotionVector TileEncoder::searchProposed(const Frame* ref, int mbx, int mby, int px, int py, int pw, int ph,
                                         MotionVector pred) {
  MotionVector best;
  int64_t bestSAD = rectSAD(ref, mbx, mby, px, py, pw, ph, best);
  auto consider = [&](MotionVector m) {
    const int64_t sad = rectSAD(ref, mbx, mby, px, py, pw, ph, m);
    if (sad < bestSAD) {
      bestSAD = sad;
      best = m;
    }
  };
  consider(pred);
  MotionVector cands[32];
  const int nc = fe->proposer->candidates(mbx, mby, cands, 32);
  // Neighbourhoods of adjacent bins overlap: evaluate each position once.
  uint32_t seen[9 * 32];
  int nSeen = 0;
  for (int i = 0; i < nc; i++) {
    const int cx = cands[i].x & ~3, cy = cands[i].y & ~3;
    for (int dy = -1; dy <= 1; dy++)
      for (int dx = -1; dx <= 1; dx++) {
        const MotionVector m{clampMV(cx + dx * 4), clampMV(cy + dy * 4)};
        const uint32_t key = (uint32_t)(uint16_t)m.x | ((uint32_t)(uint16_t)m.y << 16);
        bool dup = false;
        for (int k = 0; k < nSeen && !dup; k++) dup = seen[k] == key;
        if (dup) continue;
        seen[nSeen++] = key;
        consider(m);
      }
  }
  {
    const int bx = best.x & ~3, by = best.y & ~3;
    for (int dy = -1; dy <= 1; dy++)
      for (int dx = -1; dx <= 1; dx++) consider({clampMV(bx + dx * 4), clampMV(by + dy * 4)});
  }
  if (fe->fallbackSAD > 0 && bestSAD * 256 > (int64_t)fe->fallbackSAD * pw * ph) {
    fallbacks++;
    return searchExhaustive(ref, mbx, mby, px, py, pw, ph, pred);
  }
  const int subs[2] = {2, 1};
  for (int sub : subs) {
    const int bx = best.x, by = best.y;
    for (int dy = -1; dy <= 1; dy++)
      for (int dx = -1; dx <= 1; dx++) consider({clampMV(bx + dx * sub), clampMV(by + dy * sub)});
  }
  return best;
}

// rectSAD — ebiv/encode_inter.go:421-454
int64_t TileEncoder::rectSAD(const Frame* ref, int mbx, int mby, int px, int py, int pw, int ph, MotionVector mv) {
  sadCount++;
  if ((mv.x & 3) == 0 && (mv.y & 3) == 0) {
    const int srcX = mbx * kMB + px + (mv.x >> 2), srcY = mby * kMB + py + (mv.y >> 2);
    if (srcX >= 0 && srcY >= 0 && srcX + pw <= ref->y.w && srcY + ph <= ref->y.h) {
      const int x0 = mbx * kMB + px, y0 = mby * kMB + py;
      int64_t sad = 0;
      for (int r = 0; r < ph; r++) {
        const uint8_t* a = fe->src->y.d + (size_t)(y0 + r) * fe->src->y.stride + x0;
        const uint8_t* bb = ref->y.d + (size_t)(srcY + r) * ref->y.stride + srcX;
        int32_t rs = 0;
        for (int c = 0; c < pw; c++) rs += std::abs((int32_t)a[c] - (int32_t)bb[c]);
        sad += rs;
      }
      return sad;
    }
  }
  int32_t mc[256];
  mcLuma(ref->y, mbx * kMB + px + (mv.x >> 2), mby * kMB + py + (mv.y >> 2), mv.x & 3, mv.y & 3, pw, ph, mc, px, py,
         kMB);
  int64_t sad = 0;
  const int x0 = mbx * kMB, y0 = mby * kMB;
  for (int r = 0; r < ph; r++)
    for (int c = 0; c < pw; c++)
      sad += std::abs((int32_t)fe->src->y.at(x0 + px + c, y0 + py + r) - mc[(py + r) * kMB + px + c]);
  return sad;
}

}  // namespace

// ---------------------------------------------------------------------------
// GOP-level encoder (ebiv/encoder.go) and container writer (ebiv/writer.go)
// ---------------------------------------------------------------------------
struct Encoder::Impl {
  Geometry geo;
  std::unique_ptr<WorkerPool> pool;
  std::shared_ptr<Frame> ref, golden;
  std::vector<Freqs> prevFreqs;
  std::vector<uint8_t> prevY;
  bool havePrevY = false;
  std::vector<PackedImage> pending;
  std::vector<uint8_t> buf;
  // writer state
  std::vector<uint8_t>* out = nullptr;
  struct Entry {
    uint64_t off;
    uint32_t size;
    bool key;
  };
  std::vector<Entry> index;
  uint64_t off = 0;
  bool closed = false;
  int err = kOK;
  uint64_t sads = 0;
  uint64_t fallbacks = 0;
  uint64_t searchNs = 0;   // summed thread time in motion search
  uint64_t proposeNs = 0;  // wall time of the proposer's per-frame preparation

  int writeFrame(const std::vector<uint8_t>& payload, bool key) {  // Writer.WriteFrame
    if (err) return err;
    if (closed) return kErrWriterClosed;
    if (payload.empty() || payload.size() > kMaxFrameSize) return err = kErrConfig;
    if (index.empty() && !key) return err = kErrConfig;
    uint8_t rec[kFrameRecordSize];
    wr16(rec, kFrameSync);
    wr16(rec + 2, key ? 1 : 0);
    wr32(rec + 4, (uint32_t)payload.size());
    out->insert(out->end(), rec, rec + kFrameRecordSize);
    out->insert(out->end(), payload.begin(), payload.end());
    index.push_back({off, (uint32_t)payload.size(), key});
    off += kFrameRecordSize + payload.size();
    return kOK;
  }
};

Encoder::Encoder(const EncoderOptions& o) : impl_(new Impl()), opt_(o) {
  // Config.validate — ebiv/format.go:138-149
  if (o.width <= 0 || o.width > 65535 || o.height <= 0 || o.height > 65535 || o.fpsNum == 0 || o.fpsDen == 0 ||
      o.tileCols < 0 || o.tileCols > 65535 || o.tileRows < 0 || o.tileRows > 65535) {
    status_ = kErrConfig;
    return;
  }
  Impl& m = *impl_;
  m.geo = Geometry::of(o.width, o.height);
  m.out = &out_;
  if (o.threads > 1) m.pool.reset(new WorkerPool(o.threads));
  if (opt_.gop < 1) opt_.gop = 1;
  // FileHeader.marshal — ebiv/format.go:186-204
  uint8_t h[kFileHeaderSize];
  std::memset(h, 0, sizeof(h));
  h[0] = 'E';
  h[1] = 'B';
  h[2] = 'I';
  h[3] = 'V';
  wr16(h + 4, kVersion);
  wr16(h + 6, kFileHeaderSize);
  wr32(h + 8, (uint32_t)o.width);
  wr32(h + 12, (uint32_t)o.height);
  wr32(h + 16, o.fpsNum);
  wr32(h + 20, o.fpsDen);
  wr16(h + 32, (uint16_t)o.tileCols);
  wr16(h + 34, (uint16_t)o.tileRows);
  out_.assign(h, h + kFileHeaderSize);
  m.off = kFileHeaderSize;
}

Encoder::~Encoder() = default;

uint64_t Encoder::sadEvaluations() const { return impl_->sads; }
uint64_t Encoder::searchFallbacks() const { return impl_->fallbacks; }
double Encoder::searchSeconds() const { return (double)impl_->searchNs * 1e-9; }
double Encoder::proposeSeconds() const { return (double)impl_->proposeNs * 1e-9; }

namespace {
std::vector<uint8_t> frameHeaderBytes(int type, int coding, const Geometry& g, bool override_) {
  std::vector<uint8_t> b;
  uint8_t x = (uint8_t)((type & 0x03) | ((coding & 0x07) << 2));
  if (override_) x |= 1 << 5;
  b.push_back(x);
  if (type == kFrameKey) {
    b.push_back((uint8_t)g.W);
    b.push_back((uint8_t)(g.W >> 8));
    b.push_back((uint8_t)g.H);
    b.push_back((uint8_t)(g.H >> 8));
    b.push_back(0);  // Chroma420<<4 | depth8
  }
  return b;
}

// buildAltRef — ebiv/encoder.go:328-407
bool buildAltRef(const Geometry& g, const std::vector<PackedImage>& frames, int window, PackedImage* out) {
  const int n = std::min(window, (int)frames.size());
  if (n < 3) return false;
  const int w = g.W, h = g.H, cw = g.CW, ch = g.CH;
  const PackedImage& target = frames[0];
  std::vector<uint32_t> sumY((size_t)w * h, 0), sumCb((size_t)cw * ch, 0), sumCr((size_t)cw * ch, 0);
  std::vector<uint16_t> cntY((size_t)w * h, 0), cntC((size_t)cw * ch, 0);
  auto acc = [](std::vector<uint32_t>& sum, std::vector<uint16_t>* cnt, const std::vector<uint8_t>& src, int stride,
                int x0, int y0, int x1, int y1, int pw) {
    for (int y = y0; y < y1; y++)
      for (int x = x0; x < x1; x++) {
        sum[(size_t)y * pw + x] += src[(size_t)y * stride + x];
        if (cnt) (*cnt)[(size_t)y * pw + x]++;
      }
  };
  acc(sumY, &cntY, target.Y, w, 0, 0, w, h, w);
  acc(sumCb, &cntC, target.Cb, cw, 0, 0, cw, ch, cw);
  acc(sumCr, nullptr, target.Cr, cw, 0, 0, cw, ch, cw);
  int accepted = 0;
  for (int j = 1; j < n; j++) {
    const PackedImage& f = frames[(size_t)j];
    for (int by = 0; by < h; by += kMB) {
      const int bh = std::min(kMB, h - by);
      for (int bx = 0; bx < w; bx += kMB) {
        const int bw = std::min(kMB, w - bx);
        int64_t sad = 0;
        for (int y = by; y < by + bh; y++)
          for (int x = bx; x < bx + bw; x++)
            sad += std::abs((int32_t)target.Y[(size_t)y * w + x] - (int32_t)f.Y[(size_t)y * w + x]);
        if (sad > (int64_t)bw * bh * 6) continue;
        accepted++;
        acc(sumY, &cntY, f.Y, w, bx, by, bx + bw, by + bh, w);
        const int cx0 = bx / 2, cy0 = by / 2, cx1 = std::min(cw, (bx + bw + 1) / 2), cy1 = std::min(ch, (by + bh + 1) / 2);
        acc(sumCb, &cntC, f.Cb, cw, cx0, cy0, cx1, cy1, cw);
        acc(sumCr, nullptr, f.Cr, cw, cx0, cy0, cx1, cy1, cw);
      }
    }
  }
  if (accepted == 0) return false;
  out->alloc(w, h);
  for (size_t i = 0; i < out->Y.size(); i++) {
    const uint32_t c = cntY[i];
    out->Y[i] = (uint8_t)((sumY[i] + c / 2) / c);
  }
  for (size_t i = 0; i < out->Cb.size(); i++) {
    const uint32_t c = cntC[i];
    out->Cb[i] = (uint8_t)((sumCb[i] + c / 2) / c);
    out->Cr[i] = (uint8_t)((sumCr[i] + c / 2) / c);
  }
  return true;
}

int autoTileGrid(int mbCols, int mbRows, int workers, int* rows) {
  const int target = std::min(workers, 16);
  if (target < 2 || mbCols * mbRows < 2 * 16 * 16) {
    *rows = 1;
    return 1;
  }
  const int maxCols = std::max(1, mbCols / 16), maxRows = std::max(1, mbRows / 16);
  int cols = (int)std::round(std::sqrt((double)target * (double)mbCols / (double)mbRows));
  cols = std::min(std::max(cols, 1), maxCols);
  *rows = std::min(std::max((target + cols - 1) / cols, 1), maxRows);
  return cols;
}
}  // namespace

int Encoder::writeFrame(const PackedImage& img) {
  if (status_ != kOK) return status_;
  Impl& m = *impl_;
  if (img.W != m.geo.W || img.H != m.geo.H) return kErrDimensions;
  if (!opt_.coded) {
    // writeRaw — ebiv/encoder.go:178-187
    std::vector<uint8_t> b = frameHeaderBytes(kFrameKey, kCodingRaw, m.geo, false);
    b.insert(b.end(), img.Y.begin(), img.Y.end());
    b.insert(b.end(), img.Cb.begin(), img.Cb.end());
    b.insert(b.end(), img.Cr.begin(), img.Cr.end());
    return m.writeFrame(b, true);
  }
  // sceneCut — ebiv/encoder.go:208-227 (always evaluated, records prevY)
  const int w = m.geo.W, h = m.geo.H;
  const bool first = !m.havePrevY;
  int64_t sad = 0;
  if (!first)
    for (size_t i = 0; i < (size_t)w * h; i++) sad += std::abs((int32_t)img.Y[i] - (int32_t)m.prevY[i]);
  m.prevY = img.Y;
  m.havePrevY = true;
  const bool cut = !first && sad > (int64_t)w * h * 28;
  if (cut && m.pending.size() >= 8) {
    int e = flushGOP();
    if (e) return e;
  }
  m.pending.push_back(img);
  if ((int)m.pending.size() >= opt_.gop) {
    int e = flushGOP();
    if (e) return e;
  }
  accepted_++;
  return kOK;
}

int Encoder::gridCols() const { return opt_.withTilesCols >= 0 ? opt_.withTilesCols : opt_.tileCols; }
int Encoder::gridRows() const { return opt_.withTilesRows >= 0 ? opt_.withTilesRows : opt_.tileRows; }

// flushGOP — ebiv/encoder.go:250-306
int Encoder::flushGOP() {
  Impl& m = *impl_;
  if (m.pending.empty()) return kOK;
  std::vector<PackedImage> frames;
  frames.swap(m.pending);
  // Encoder.tileGrid — ebiv/encoder.go:422-432
  int cols = gridCols(), rows = gridRows();
  if (!(cols > 1 || rows > 1) && opt_.autoTiles > 1) cols = autoTileGrid(m.geo.mbCols, m.geo.mbRows, opt_.autoTiles, &rows);
  PackedImage alt;
  const bool haveAlt = buildAltRef(m.geo, frames, opt_.altRefWindow, &alt);
  auto runFrame = [&](const PackedImage& img, const Frame* ref, const Frame* gold, bool inter,
                      const std::vector<Freqs>* prev, std::vector<Freqs>* freqs, std::shared_ptr<Frame>* rec) {
    FrameEncoder fe(m.geo, img, ref, gold, opt_.qp, cols, rows);
    fe.pool = m.pool.get();
    fe.search = opt_.search;
    fe.exhaustiveRange = opt_.exhaustiveRange;
    fe.fallbackSAD = opt_.proposedFallbackSAD;
    fe.proposer = proposer_;
    if (inter && proposer_ && opt_.search == SearchMode::Proposed) {
      const auto t0 = std::chrono::steady_clock::now();
      proposer_->prepare(fe.src->yb.data(), ref->yb.data(), m.geo.padW(), m.geo.padH());
      m.proposeNs += (uint64_t)std::chrono::duration_cast<std::chrono::nanoseconds>(std::chrono::steady_clock::now() - t0)
                         .count();
    }
    fe.encode(inter, !opt_.fastEncode);
    std::vector<uint8_t> payload = fe.finish(opt_.qp, prev, freqs);
    m.sads += fe.sadCount.load();
    m.fallbacks += fe.fallbacks.load();
    m.searchNs += fe.searchNs.load();
    rec->reset(fe.rec.release());
    return payload;
  };
  auto merge = [&](const std::vector<Freqs>& f) {
    for (int c = 0; c < kNumContexts; c++)
      if (!f[c].empty()) m.prevFreqs[c] = f[c];
  };
  std::vector<Freqs> freqs;
  std::shared_ptr<Frame> rec;
  std::vector<uint8_t> payload = runFrame(frames[0], nullptr, nullptr, false, nullptr, &freqs, &rec);
  m.prevFreqs.assign(kNumContexts, Freqs{});
  merge(freqs);
  m.ref = rec;
  m.golden = rec;
  std::vector<uint8_t> b = frameHeaderBytes(kFrameKey, kCodingIntra, m.geo, haveAlt);
  if (haveAlt) {
    std::vector<Freqs> ovFreqs;
    std::shared_ptr<Frame> ovRec;
    std::vector<uint8_t> ov = runFrame(alt, rec.get(), nullptr, true, &m.prevFreqs, &ovFreqs, &ovRec);
    merge(ovFreqs);
    m.golden = ovRec;
    putUvarint(b, payload.size());
    b.insert(b.end(), payload.begin(), payload.end());
    b.insert(b.end(), ov.begin(), ov.end());
  } else {
    b.insert(b.end(), payload.begin(), payload.end());
  }
  int e = m.writeFrame(b, true);
  if (e) return e;
  keep(rec.get());
  for (size_t i = 1; i < frames.size(); i++) {
    std::vector<Freqs> f;
    std::shared_ptr<Frame> r;
    std::vector<uint8_t> p = runFrame(frames[i], m.ref.get(), m.golden.get(), true, &m.prevFreqs, &f, &r);
    merge(f);
    m.ref = r;
    std::vector<uint8_t> fb = frameHeaderBytes(kFrameInter, kCodingInter, m.geo, false);
    fb.insert(fb.end(), p.begin(), p.end());
    e = m.writeFrame(fb, false);
    if (e) return e;
    keep(r.get());
  }
  return kOK;
}

void Encoder::keep(const void* frame) {
  if (!opt_.keepRecon) return;
  const Frame* f = static_cast<const Frame*>(frame);
  const Geometry& g = impl_->geo;
  PackedImage im;
  im.alloc(g.W, g.H);
  for (int y = 0; y < g.H; y++) std::memcpy(&im.Y[(size_t)y * g.W], f->y.d + (size_t)y * f->y.stride, g.W);
  for (int y = 0; y < g.CH; y++) {
    std::memcpy(&im.Cb[(size_t)y * g.CW], f->cb.d + (size_t)y * f->cb.stride, g.CW);
    std::memcpy(&im.Cr[(size_t)y * g.CW], f->cr.d + (size_t)y * f->cr.stride, g.CW);
  }
  recons_.push_back(std::move(im));
}

// Encoder.Close + Writer.Close — ebiv/encoder.go:447-452, ebiv/writer.go:92-119
int Encoder::close() {
  if (status_ != kOK) return status_;
  Impl& m = *impl_;
  if (m.closed) return m.err;
  int e = flushGOP();
  if (e) return e;
  m.closed = true;
  if (m.err) return m.err;
  const uint64_t indexOffset = m.off;
  std::vector<uint8_t> idx(m.index.size() * kIndexEntrySize);
  for (size_t i = 0; i < m.index.size(); i++) {
    uint8_t* p = idx.data() + i * kIndexEntrySize;
    wr64(p, m.index[i].off);
    wr32(p + 8, m.index[i].size);
    wr32(p + 12, m.index[i].key ? 1 : 0);
  }
  out_.insert(out_.end(), idx.begin(), idx.end());
  uint8_t footer[kFooterSize];
  wr64(footer, indexOffset);
  wr32(footer + 8, (uint32_t)m.index.size());
  wr32(footer + 12, crc32IEEE(idx.data(), idx.size()));
  footer[16] = 'E';
  footer[17] = 'B';
  footer[18] = 'I';
  footer[19] = 'X';
  out_.insert(out_.end(), footer, footer + kFooterSize);
  return kOK;
}


// Encodes one block of levels the way the encoder codes a residual block:
// sign-data hiding (ebiv/residual.go:134-180), the token grammar
// (ebiv/residual.go:30-75), per-context tables normalized from the block's
// own token counts (ebiv/rans.go:46-85) and the interleaved rANS coder
// (ebiv/rans.go:186-214).  Returns the adjusted levels, the stream and the
// frequency tables (16 entries per context).
int encodeBlockStream(int32_t* levels, int n, int plane, int txIdx, std::vector<uint8_t>* stream,
                      std::vector<uint32_t>* freqs, std::vector<uint8_t>* used) {
  if (n != 4 && n != 8 && n != 16) return kErrArg;
  applySignDataHiding(levels, n);
  TokStream ts;
  encodeBlock(ts, plane, txIdx, levels, n);
  return encodeTokenStream(ts.toks.data() ? reinterpret_cast<const uint16_t*>(ts.toks.data()) : nullptr,
                           (int)ts.toks.size(), stream, freqs, used);
}

// A one-tile intra key frame built from chosen levels: every macroblock
// codes its luma as sixteen 4x4 blocks (16 levels each, raster order within
// the macroblock) and its chroma as one 8x8 Cb and one 8x8 Cr block (64
// levels each), all with intra mode `mode`; tokens follow the grammar of
// decodeLumaMB/decodeChromaMB (ebiv/decode_intra.go:121-187) after sign-data
// hiding, tables are normalized from the frame's own counts, and the packet
// is header + assemblePayload (ebiv/frame.go:224-236).  It makes test
// streams with coefficients no real source produces.
int encodeKeyFromLevels(int w, int h, int qp, int mode, const int32_t* levels, size_t nlevels,
                        std::vector<uint8_t>* pkt) {
  if (w <= 0 || h <= 0 || qp < 0 || qp > 255 || mode < 0 || mode >= kNumIntraModes) return kErrArg;
  const Geometry g = Geometry::of(w, h);
  const size_t perMB = 16 * 16 + 2 * 64;
  if (nlevels != perMB * (size_t)g.mbCols * g.mbRows) return kErrArg;
  TokStream ts;
  int32_t lv[64];
  const int32_t* src = levels;
  for (int m = 0; m < g.mbCols * g.mbRows; m++) {
    ts.put(ctxTxSize, 0);
    for (int k = 0; k < 16; k++, src += 16) {
      ts.put(ctxLumaMode, mode);
      std::memcpy(lv, src, 16 * sizeof(int32_t));
      applySignDataHiding(lv, 4);
      encodeBlock(ts, kPlaneLuma, 0, lv, 4);
    }
    ts.put(ctxChromaMode, mode);
    for (int c = 0; c < 2; c++, src += 64) {
      std::memcpy(lv, src, 64 * sizeof(int32_t));
      applySignDataHiding(lv, 8);
      encodeBlock(ts, kPlaneChroma, 0, lv, 8);
    }
  }
  std::vector<std::vector<uint32_t>> counts(kNumContexts);
  for (int c = 0; c < kNumContexts; c++) counts[c].assign((size_t)alphabetSize(c), 0);
  for (const Tok& t : ts.toks) counts[t.ctx][t.sym]++;
  std::vector<Freqs> freqs(kNumContexts);
  std::vector<EncTable> tables(kNumContexts);
  for (int c = 0; c < kNumContexts; c++) {
    if (c == ctxBypass) continue;
    freqs[c] = normalizeFreqs(counts[c]);
    tables[c] = buildEncTable(freqs[c].empty() ? Freqs((size_t)alphabetSize(c), 0) : freqs[c], alphabetSize(c));
  }
  tables[ctxBypass] = buildEncTable(Freqs{kM / 2, kM / 2}, 2);
  const std::vector<uint8_t> tableBytes = serializeTables(freqs, nullptr);
  const std::vector<uint8_t> tile = ransEncode(ts.toks, tables);
  *pkt = frameHeaderBytes(kFrameKey, kCodingIntra, g, false);
  pkt->push_back((uint8_t)qp);
  putUvarint(*pkt, 1);
  putUvarint(*pkt, 1);
  putUvarint(*pkt, tableBytes.size());
  pkt->insert(pkt->end(), tableBytes.begin(), tableBytes.end());
  putUvarint(*pkt, tile.size());
  pkt->insert(pkt->end(), tile.begin(), tile.end());
  return kOK;
}

// rANS-encodes a (context, symbol) token list with tables normalized from its
// own counts; the bypass context is the fixed uniform table.
int encodeTokenStream(const uint16_t* pairs, int count, std::vector<uint8_t>* stream, std::vector<uint32_t>* freqs,
                      std::vector<uint8_t>* used) {
  std::vector<Tok> toks((size_t)count);
  for (int i = 0; i < count; i++) toks[(size_t)i] = {pairs[2 * i], pairs[2 * i + 1]};
  std::vector<std::vector<uint32_t>> counts(kNumContexts);
  for (int c = 0; c < kNumContexts; c++) counts[c].assign((size_t)alphabetSize(c), 0);
  for (const Tok& t : toks) {
    if (t.ctx >= kNumContexts || t.sym >= alphabetSize(t.ctx)) return kErrArg;
    counts[t.ctx][t.sym]++;
  }
  std::vector<EncTable> tables(kNumContexts);
  freqs->assign((size_t)kNumContexts * 16, 0);
  used->assign((size_t)kNumContexts, 0);
  for (int c = 0; c < kNumContexts; c++) {
    if (c == ctxBypass) continue;
    const Freqs f = normalizeFreqs(counts[c]);
    tables[c] = buildEncTable(f.empty() ? Freqs((size_t)alphabetSize(c), 0) : f, alphabetSize(c));
    if (!f.empty()) {
      (*used)[(size_t)c] = 1;
      for (size_t s = 0; s < f.size(); s++) (*freqs)[(size_t)c * 16 + s] = f[s];
    }
  }
  tables[ctxBypass] = buildEncTable(Freqs{kM / 2, kM / 2}, 2);
  *stream = ransEncode(toks, tables);
  return kOK;
}
}  // namespace ebiv
