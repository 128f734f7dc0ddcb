// GB300 (sm_103a) EBIV decode kernels.
//
// Stage A  kEntropy   one warp per tile, up to four tiles of one frame per
//                     CTA sharing the frame's symbol tables: the tile's
//                     4-state interleaved rANS chain (ebiv/rans.go:270-304)
//                     drives the macroblock grammar
//                     (ebiv/decode_intra.go:121-167, ebiv/decode_inter.go:8-62,
//                     ebiv/residual.go:79-126, ebiv/mv.go) and emits one
//                     MBRec per macroblock plus sparse levels.  The warp runs
//                     the chain in lockstep; a symbol costs one shared-memory
//                     lookup (slot bucket -> symbol, start, frequency) except
//                     in the few buckets a symbol boundary crosses.
// Stage B1 kInterRecon one warp per macroblock of an inter frame: motion
//                     compensation (ebiv/motioncomp.go) from the last or
//                     golden reference plus dequantized inverse DCT residual
//                     (ebiv/quant.go:72-80, ebiv/transform.go:129-194).
// Stage B2 kIntraRecon one CTA per tile: intra macroblocks reconstructed along
//                     their true dependencies only, a dataflow schedule over
//                     the 4x4-block diagonal steps (ebiv/predict.go:50-219).
//
// Waits are __syncwarp/__syncthreads barriers inside one CTA, and in
// kIntraRecon polls of progress bytes written by warps of the same CTA, each
// bounded (IntraSync); no kernel spins on memory written by another CTA.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>

#include "gpu_types.h"

namespace ebiv {
namespace dev {

constexpr unsigned kFull = 0xffffffffu;

// Per transform size and scan position: row-major index (bits 0-7) and the
// offset of the position's band in the symbol-table rows,
// bandOf(i) * kNumPrevClass * 64 (bits 8-19).  One entry past each scan is
// zero, so the next position's entry can always be loaded.
__constant__ uint32_t cScanRow[3][257];
// 2^13-scaled DCT-II basis, [k*n + i], per transform size.  Global memory:
// the transforms read it with a different index in every lane, which the
// L1 path serves in one pass and the constant cache would serialise.
__device__ int32_t gDct[3][256];
__constant__ int32_t cTaps[4][4] = {{0, 64, 0, 0}, {-6, 55, 18, -3}, {-8, 40, 40, -8}, {-3, 18, 55, -6}};

__device__ __forceinline__ int tokenCtx(int plane, int txIdx, int band, int prevClass) {
  return plane == kPlaneLuma ? ctxTokenBase + (txIdx * kNumBands + band) * kNumPrevClass + prevClass
                             : ctxTokenBase + kLumaTokenCtx + band * kNumPrevClass + prevClass;
}
__device__ __forceinline__ int clampByteD(int32_t v) { return v < 0 ? 0 : (v > 255 ? 255 : v); }
__device__ __forceinline__ int32_t wadd(int32_t a, int32_t b) { return (int32_t)((uint32_t)a + (uint32_t)b); }
__device__ __forceinline__ int32_t wmul(int32_t a, int32_t b) { return (int32_t)((uint32_t)a * (uint32_t)b); }
__device__ __forceinline__ int clampC(int v, int hi) { return v < 0 ? 0 : (v >= hi ? hi - 1 : v); }
__device__ __forceinline__ int16_t clampMV(int v) {
  return (int16_t)(v < -kMVClampRange ? -kMVClampRange : (v > kMVClampRange ? kMVClampRange : v));
}

// ---------------------------------------------------------------------------
// Stage A: entropy decode
// ---------------------------------------------------------------------------
// Symbol tables, built once per CTA for the frame whose tiles the CTA
// decodes.  bucket[c*64+b] describes the symbol s of context c whose range
// holds slot b*64: start (bits 0-11), frequency (12-24), s (25-28), a flag
// (29) when a later symbol starts inside the bucket (the decoder then walks
// sym[]), and a flag (30) for an unused context, whose entry decodes as the
// identity so the chain stays well defined after the error.  sym[c*16+s]
// packs start | frequency << 16 for the walk.
constexpr uint32_t kBImpure = 1u << 29, kBUnused = 1u << 30;
struct EntropyTables {
  uint32_t bucket[kNumContexts * 64];
  uint32_t sym[kNumContexts * 16];
};
constexpr int kRowMax = 128;  // tiles at most this many macroblocks wide pass vector rows in shared memory
struct WarpRows {
  uint32_t mv[2][kRowMax];  // packed vectors of a pass's last row, by pass parity
};

__device__ __forceinline__ void buildTables(EntropyTables& T, const DeviceTables& src, int tid, int nthreads) {
  for (int i = tid; i < kNumContexts * 16; i += nthreads) {
    const int c = i >> 4, sidx = i & 15;
    const uint32_t st = src.start[c][sidx], nx = src.start[c][sidx + 1];
    T.sym[i] = (st == 0xFFFFu || nx == 0xFFFFu) ? 0xFFFFu : (st | ((nx - st) << 16));
  }
  for (int i = tid; i < kNumContexts * 64; i += nthreads) T.bucket[i] = (kM << 12) | kBUnused;
  __syncthreads();
  // Each (context, symbol) pair fills the buckets whose first slot it covers.
  for (int i = tid; i < kNumContexts * 16; i += nthreads) {
    const int c = i >> 4, sidx = i & 15;
    if (!src.used[c]) continue;
    const uint32_t st = src.start[c][sidx], nx = src.start[c][sidx + 1];
    if (st == 0xFFFFu || nx == 0xFFFFu || nx <= st) continue;
    for (uint32_t b = (st + 63) >> 6; b < 64 && (b << 6) < nx; b++)
      T.bucket[c * 64 + b] = st | ((nx - st) << 12) | ((uint32_t)sidx << 25) | (nx < ((b + 1) << 6) ? kBImpure : 0u);
  }
  __syncthreads();
}

// Symbol-log bookkeeping of the symbol path.  kNoError: no failing symbol;
// kFullChain (in TileStat::errAt): the tile was decoded by the full chain;
// kOverflow: internal status of a symbol chain whose log ran out of room
// (never reported: the tile is decoded again by the full chain).  A
// macroblock header takes at most 125 symbols (mode, reference, partition,
// four vectors of two class-coded components of up to 15 symbols each,
// pattern, transform size).
constexpr int32_t kNoError = 0x7FFFFFFF;
constexpr int32_t kFullChain = -1;
constexpr int32_t kOverflow = -100;
constexpr int kMBHeaderSymbols = 128;

// A tile's rANS decoder (ebiv/rans.go:222-304).  All fields are warp-uniform;
// the two next stream bytes are prefetched so renormalisation rarely waits.
// After the first error every symbol decodes as 0.  With kLog every symbol
// the decoder returns while no error is pending (the failing one included,
// as 0) is appended to a symbol log, and errAt is the failing one's index.
template <bool kLog>
struct ChainT {
  const uint8_t* buf;
  int32_t pos;
  uint32_t x0, x1, x2, x3;  // states in use order: x0 decodes the next symbol
  uint32_t b1, b2;          // buf[pos-1], buf[pos-2] when present
  int32_t err;
  const EntropyTables* t;
  uint8_t* log;   // kLog: the tile's symbol log
  int32_t n;      // kLog: symbols logged
  int32_t errAt;  // kLog: index of the failing symbol (kNoError: none)
  int32_t cap;    // kLog: the log's capacity
  int32_t lane;   // kLog: the lane that writes the log

  __device__ __forceinline__ uint32_t byteAt(int i) const { return i >= 0 ? (uint32_t)__ldg(buf + i) : 0u; }
  __device__ __forceinline__ int logged(int s) {
    if (kLog) {
      if (lane == 0) log[n] = (uint8_t)s;
      n++;
    }
    return s;
  }
  __device__ __forceinline__ int fail(int e) {
    err = e;
    if (kLog) errAt = n;
    return logged(0);
  }

  // The next symbol of the context whose bucket row starts at word row
  // (context * 64).
  __device__ __forceinline__ int symAt(int row) {
    if (err) return 0;
    const uint32_t x = x0;
    const uint32_t slot = x & (kM - 1);
    const uint32_t e = t->bucket[row + (int)(slot >> 6)];
    int s = (int)((e >> 25) & 15u);
    uint32_t start = e & 0xFFFu, freq = (e >> 12) & 0x1FFFu;
    if (e & (kBImpure | kBUnused)) {
      if (e & kBUnused) return fail(kErrCorrupt);  // symbol decoded from an unused context
      while (slot >= start + freq) {
        const uint32_t w = t->sym[(row >> 2) + (++s)];
        start = w & 0xFFFFu;
        freq = w >> 16;
      }
    }
    uint32_t xn = freq * (x >> kScaleBits) + slot - start;
    if (xn < kLower) {
      if (pos >= 2 && xn >= (kLower >> 16)) {
        if (xn < (kLower >> 8)) {  // two bytes
          xn = (xn << 16) | (b1 << 8) | b2;
          pos -= 2;
          b1 = byteAt(pos - 1);
          b2 = byteAt(pos - 2);
        } else {  // one byte
          xn = (xn << 8) | b1;
          pos -= 1;
          b1 = b2;
          b2 = byteAt(pos - 2);
        }
      } else {
        while (xn < kLower) {
          if (pos == 0) return fail(kErrCorrupt);  // stream underrun
          pos--;
          xn = (xn << 8) | b1;
          b1 = b2;
          b2 = byteAt(pos - 2);
        }
      }
    }
    x0 = x1;
    x1 = x2;
    x2 = x3;
    x3 = xn;
    return logged(s);
  }
  __device__ __forceinline__ int sym(int ctx) { return symAt(ctx << 6); }
  // Whether the log has room for `need` more symbols; when it has not, the
  // chain stops with kOverflow.
  __device__ __forceinline__ bool room(int need) {
    if (!kLog || n + need <= cap) return true;
    err = kOverflow;
    return false;
  }
  // Initialises the four states from the end of the tile's bytes
  // (ransDecoder.reset, ebiv/rans.go:236-250); false when the stream is too short.
  __device__ __forceinline__ bool reset(const uint8_t* b, uint32_t len, const EntropyTables* tables) {
    buf = b;
    pos = (int32_t)len;
    err = 0;
    t = tables;
    n = 0;
    errAt = kNoError;
    if (len < (uint32_t)(kStates * 4)) {
      err = kErrCorrupt;
      return false;
    }
    uint32_t st[4];
#pragma unroll
    for (int i = kStates - 1; i >= 0; i--) {
      st[i] = byteAt(pos - 1) << 24 | byteAt(pos - 2) << 16 | byteAt(pos - 3) << 8 | byteAt(pos - 4);
      pos -= 4;
    }
    x0 = st[0];
    x1 = st[1];
    x2 = st[2];
    x3 = st[3];
    b1 = byteAt(pos - 1);
    b2 = byteAt(pos - 2);
    return true;
  }
};

// Replays a tile's symbol log from one macroblock's first symbol: the same
// values, and the same error state at every point, as the chain that wrote
// the log (a symbol past the failing one is never read: it decodes as 0).
struct Replay {
  const uint8_t* log;
  int32_t k;      // index of the next symbol in the tile's log
  int32_t errAt;  // index of the failing symbol, or kNoError
  int32_t end;    // the log's capacity: reads stay inside it
  int32_t err;
  __device__ __forceinline__ int symAt(int) {
    if (err) return 0;
    if (k >= end) {  // unreachable while replay and chain agree; keeps every read in bounds
      err = kErrCorrupt;
      return 0;
    }
    const int s = log[k];
    k++;
    if (k > errAt) err = kErrCorrupt;
    return s;
  }
  __device__ __forceinline__ int sym(int) { return symAt(0); }
  __device__ __forceinline__ bool room(int) const { return true; }
};

// getRawBits / getClassValue / getMVComponent — ebiv/mv.go:75-128.
template <class S>
__device__ __forceinline__ uint32_t rawBits(S& d, int n) {
  uint32_t v = 0;
  for (int i = 0; i < n; i++) v = v << 1 | (uint32_t)d.sym(ctxBypass);
  return v;
}
template <class S>
__device__ __forceinline__ uint32_t classValue(S& d, int classCtx) {
  const int cls = d.sym(classCtx);
  if (cls <= 1) return (uint32_t)cls;
  return (1u << (cls - 1)) | rawBits(d, cls - 1);
}
template <class S>
__device__ __forceinline__ int mvComponent(S& d, int classCtx) {
  const uint32_t u = classValue(d, classCtx);
  return (int)(u >> 1) ^ -(int)(u & 1);
}

// decodeBlock (ebiv/residual.go:79-126).  With kOut the block's nonzero
// levels are written as packed entries after a count word (by lane 0);
// without it only the symbols are decoded (the chain of the symbol path:
// everything that decides which symbol comes next, nothing else).  row is
// the bucket row of the block's token contexts at band 0 and previous class
// 0 (context * 64); the band and previous class add their row offsets.
// Returns the count.
template <bool kOut, class S>
__device__ __forceinline__ int entropyBlock(S& d, int row, int sz, uint32_t* region, int lane) {
  const uint32_t* sb = cScanRow[sz];
  const int total = 16 << (2 * sz);
  int first = -1, last = -1, count = 0;
  int32_t sumAbs = 0;
  int pc = 0;  // previous class * 64
  uint32_t firstPos = 0;
  int32_t firstMag = 0;
  uint32_t cur = sb[0];
  for (int i = 0; i < total; i++) {
    const uint32_t nxt = sb[i + 1];  // next position's entry, loaded early (the table is padded)
    const int t = d.symAt(row + (int)(cur >> 8) + pc);
    if (t == tEOB) break;
    if (t == tZero) {
      pc = 0;
      cur = nxt;
      continue;
    }
    int mag;
    if (t == tEscape) {
      mag = 5 + (int)classValue(d, ctxEscClass);
      pc = 2 * 64;
    } else {
      mag = t;
      pc = t == tOne ? 64 : 2 * 64;
    }
    sumAbs = wadd(sumAbs, mag);
    const uint32_t pos = cur & 0xFFu;
    if (first < 0) {
      first = i;
      firstPos = pos;
      firstMag = mag;
    } else {
      if (d.symAt(ctxSign << 6) == 1) mag = -mag;
      if (kOut && lane == 0) region[1 + count] = pos | ((uint32_t)mag << 8);
    }
    count++;
    last = i;
    cur = nxt;
  }
  if (first >= 0) {
    const bool neg = (last - first >= kSDHMinSpan) ? (sumAbs & 1) == 1 : d.symAt(ctxSign << 6) == 1;
    if (kOut && lane == 0) region[1] = firstPos | ((uint32_t)(neg ? -firstMag : firstMag) << 8);
  }
  if (kOut && lane == 0) region[0] = (uint32_t)count;
  return count;
}

__device__ __forceinline__ int16_t median3(int16_t a, int16_t b, int16_t c) {
  if (a > b) {
    const int16_t t = a;
    a = b;
    b = t;
  }
  if (b > c) b = c;
  if (a > b) b = a;
  return b;
}
__device__ __forceinline__ uint32_t packMV(int x, int y) { return (uint32_t)(uint16_t)x | ((uint32_t)(uint16_t)y << 16); }
__device__ __forceinline__ int mvX(uint32_t v) { return (int16_t)(v & 0xFFFFu); }
__device__ __forceinline__ int mvY(uint32_t v) { return (int16_t)(v >> 16); }

// The macroblock record being assembled, in registers (see MBRec: word 0
// mode|ref<<8|part<<16|cbp<<24, 1 tx|cmode<<8, 2-5 vectors, 6-9 luma modes,
// 10 nzmask, 11 wmask).
struct Rec {
  uint32_t w0, w1, mv0, mv1, mv2, mv3, lm0, lm1, lm2, lm3, nz, wm;
  __device__ __forceinline__ void clear() { w0 = w1 = mv0 = mv1 = mv2 = mv3 = lm0 = lm1 = lm2 = lm3 = nz = wm = 0; }
  __device__ __forceinline__ void lumaMode(int k, uint32_t m) {
    const uint32_t v = m << ((k & 3) * 8);
    const int w = k >> 2;
    if (w == 0) lm0 |= v;
    else if (w == 1) lm1 |= v;
    else if (w == 2) lm2 |= v;
    else lm3 |= v;
  }
  __device__ __forceinline__ void setMV(int i, uint32_t v) {
    if (i == 0) mv0 = v;
    else if (i == 1) mv1 = v;
    else if (i == 2) mv2 = v;
    else mv3 = v;
  }
  // One thread stores the whole 48-byte record.
  __device__ __forceinline__ void storeAll(MBRec* dst) const {
    uint4* q = reinterpret_cast<uint4*>(dst);
    q[0] = make_uint4(w0, w1, mv0, mv1);
    q[1] = make_uint4(mv2, mv3, lm0, lm1);
    q[2] = make_uint4(lm2, lm3, nz, wm);
  }
  // Lanes 0-2 store the 48-byte record as three 16-byte words.
  __device__ __forceinline__ void store(MBRec* dst, int lane) const {
    uint4 v;
    if (lane == 0) v = make_uint4(w0, w1, mv0, mv1);
    else if (lane == 1) v = make_uint4(mv2, mv3, lm0, lm1);
    else v = make_uint4(lm2, lm3, nz, wm);
    if (lane < 3) reinterpret_cast<uint4*>(dst)[lane] = v;
  }
};

// Neighbourhood of the macroblock being decoded: availability within the
// tile, the left neighbour's vector/level (registers) and the row above.
struct Nbr {
  bool aOK, bOK, arOK;
  uint32_t mvA, mvB, mvC;  // left, above, above-right (or above-left)
  bool cOK;
};

// predictMV — ebiv/mv.go:21-52 (neighbours within the tile).  The median of
// three runs on both packed 16-bit components at once: median(a, b, c) =
// max(min(a, b), min(max(a, b), c)); unavailable neighbours are zero.
__device__ __forceinline__ uint32_t predictMV(const Nbr& n) {
  if (!n.aOK && !n.bOK && !n.cOK) return 0;
  if (n.aOK && !n.bOK && !n.cOK) return n.mvA;
  if (!n.aOK && n.bOK && !n.cOK) return n.mvB;
  const uint32_t lo = __vmins2(n.mvA, n.mvB), hi = __vmaxs2(n.mvA, n.mvB);
  return __vmaxs2(lo, __vmins2(hi, n.mvC));
}

// The coded blocks of one macroblock in bitstream order: nLuma luma blocks
// (each preceded by its intra mode when intra), then Cb (preceded by the
// chroma intra mode when intra) and Cr when present.
struct BlockPlan {
  int nLuma, tx;
  bool intra, cb, cr;
};

// The block loop of a macroblock.  Returns how many blocks completed before
// an error; *nzOut gets the nonzero mask (bit k luma block k, 16 Cb, 17 Cr).
// A logging chain first checks that its log has room for the block's
// largest possible symbol count (mode, 17 per coefficient, the hidden sign).
template <bool kOut, class S>
__device__ __forceinline__ int entropyBlocks(S& d, Rec& r, const BlockPlan& p, uint32_t* coef, int lane,
                                             uint32_t* nzOut) {
  const int nEnt = p.nLuma + (p.cb ? 1 : 0) + (p.cr ? 1 : 0);
  const int bw = (16 << (2 * p.tx)) + 1;  // words per luma block region
  const int lumaRow = (ctxTokenBase + p.tx * kNumBands * kNumPrevClass) << 6;
  int done = 0;
  uint32_t nz = 0;
#pragma unroll 1
  for (int e = 0; e < nEnt; e++) {
    int row, sz;
    uint32_t* region;
    uint32_t bit;
    if (e < p.nLuma) {
      sz = p.tx;
      if (!d.room(2 + 17 * (16 << (2 * sz)))) break;
      if (p.intra) r.lumaMode(e, (uint32_t)d.sym(ctxLumaMode));
      row = lumaRow;
      region = coef + e * bw;
      bit = 1u << e;
    } else {
      sz = 1;
      if (!d.room(2 + 17 * 64)) break;
      const bool isCb = p.cb && e == p.nLuma;
      if (isCb && p.intra) r.w1 |= (uint32_t)d.sym(ctxChromaMode) << 8;
      row = (ctxTokenBase + kLumaTokenCtx) << 6;
      region = coef + (isCb ? kCoefCb : kCoefCr);
      bit = isCb ? (1u << 16) : (1u << 17);
    }
    const int cnt = entropyBlock<kOut>(d, row, sz, region, lane);
    if (d.err) break;
    if (cnt) nz |= bit;
    done++;
  }
  *nzOut = nz;
  return done;
}

// Intra macroblock header (decodeLumaMB, ebiv/decode_intra.go:137-150): the
// transform size; the blocks follow.
template <class S>
__device__ __forceinline__ void intraHeader(S& d, Rec& r, BlockPlan* p) {
  int tx = d.sym(ctxTxSize);
  if (tx >= 3) tx = 0;  // alphabet size 3: unreachable
  r.w0 = kRecIntra;
  r.w1 = (uint32_t)tx;
  p->tx = tx;
  p->nLuma = 16 >> (2 * tx);
  p->intra = p->cb = p->cr = true;
}

// Inter-frame macroblock header after the mode (decodeInterMB,
// ebiv/decode_inter.go:8-62): reference, partition, vector deltas,
// coded-block pattern, transform size.  The vectors are stored as deltas
// (x, y as int16) in the record; predictVectors turns them into vectors
// (no context depends on a vector, so the chain never needs them).  Returns
// 1 when the blocks of *p follow, 0 when the macroblock ends here (an error).
template <class S>
__device__ __forceinline__ int interHeader(S& d, Rec& r, int mode, BlockPlan* p, bool* intra) {
  if (mode == mbIntra) {
    *intra = true;
    intraHeader(d, r, p);
    return d.err ? 0 : 1;
  }
  if (mode != mbInter) {
    d.err = kErrCorrupt;
    return 0;
  }
  const int refSel = d.sym(ctxRef);
  int part = d.sym(ctxPart);
  if (part >= kNumPartModes) part = 0;  // alphabet size 4: unreachable
  const int np = part == partWhole ? 1 : (part == part8x8 ? 4 : 2);
#pragma unroll 1
  for (int i = 0; i < np; i++) {
    const int dx = mvComponent(d, ctxMVClassX);
    const int dy = mvComponent(d, ctxMVClassY);
    r.setMV(i, packMV(dx, dy));
  }
  if (d.err) return 0;
  const int cbp = d.sym(ctxCBP);
  r.w0 = kRecInter | ((uint32_t)refSel << 8) | ((uint32_t)part << 16) | ((uint32_t)cbp << 24);
  if (d.err) return 0;
  int tx = 0, nb = 0;
  if (cbp & cbpLuma) {
    tx = d.sym(ctxTxSize);
    if (tx >= 3) tx = 0;
    if (d.err) return 0;
    r.w1 = (uint32_t)tx;
    nb = 16 >> (2 * tx);
  }
  p->tx = tx;
  p->nLuma = nb;
  p->intra = false;
  p->cb = (cbp & cbpCb) != 0;
  p->cr = (cbp & cbpCr) != 0;
  return 1;
}

// Write mask after the blocks (decodeLumaMB/decodeChromaMB and
// reconInterMB, ebiv/decode_intra.go:150-187, ebiv/decode_inter.go:63-118):
// an intra macroblock keeps the blocks completed before an error; an inter
// macroblock whose coded luma failed writes only the luma blocks decoded.
__device__ __forceinline__ uint32_t writeMask(const BlockPlan& p, int done) {
  const int nb = p.nLuma;
  if (p.intra) {
    uint32_t w = (1u << min(done, nb)) - 1;
    if (done > nb) w |= 1u << 16;
    if (done > nb + 1) w |= 1u << 17;
    return w;
  }
  if (done < nb) return (1u << done) - 1;
  const int cbEntry = p.cb ? nb : -1;
  const int crEntry = p.cr ? nb + (p.cb ? 1 : 0) : -1;
  uint32_t w = 0xFFFFu;  // coded luma complete, or motion-compensated luma
  if (cbEntry < 0 || done > cbEntry) w |= 1u << 16;
  if (crEntry < 0 || done > crEntry) w |= 1u << 17;
  return w;
}

// Vector prediction over a tile whose chain is done (predictMV,
// ebiv/mv.go:21-52, neighbours inside the tile; decodeInterMB's use of it,
// ebiv/decode_inter.go:8-62).  A macroblock's vector needs the final
// vectors of its left, above and above-right (or above-left) neighbours, so
// the tile runs as a wavefront: in a pass of 32 rows lane k takes row k and,
// at step t, column t - 2k.  The left neighbour is the lane's own result of
// the step before; the row above comes from lane k-1 by shuffle (its
// results of the last three steps are columns x-1, x, x+1), and for lane 0
// from the previous pass's last row (shared memory; the frame's vector grid
// for tiles wider than kRowMax).  A skip macroblock takes the prediction;
// an inter one adds its deltas (partition 0 to the prediction, zero for the
// golden reference; later partitions to partition 0), clamped as the chain
// would have.  Records past `done` are not touched.
__device__ void predictVectors(const FrameDesc* fp, int tile, int done, WarpRows& rows, int lane) {
  const int mbCols = fp->mbCols;
  MBRec* const recs = fp->mbrec;
  uint32_t* const gmv = reinterpret_cast<uint32_t*>(fp->mvgrid);
  const TileRange tr = fp->tiles[tile];
  const int x0 = tr.mbX0, y0 = tr.mbY0, tw = tr.mbX1 - x0, th = tr.mbY1 - y0;
  const bool wide = tw > kRowMax;
  for (int p0 = 0, pass = 0; p0 < th; p0 += 32, pass++) {
    const int ry = p0 + lane;
    const int nrows = min(32, th - p0);
    const int steps = tw + 2 * (nrows - 1);
    const bool lastRowOfPass = lane == 31 && p0 + 32 < th;
    const uint32_t* upRow = wide ? gmv + (size_t)(y0 + p0 - 1) * mbCols + x0 : rows.mv[(pass + 1) & 1];
    uint32_t* nextUp = wide ? gmv + (size_t)(y0 + p0 + 31) * mbCols + x0 : rows.mv[pass & 1];
    // Records of this lane's row; written by this warp's chain, so read
    // with coherent loads (never through the read-only path).
    MBRec* const rowRec = recs + (size_t)(y0 + min(ry, th - 1)) * mbCols + x0;
    const int rowDone = ry < th ? min(tw, done - ry * tw) : 0;  // columns of this row the chain reached
    uint32_t h1 = 0, h2 = 0, h3 = 0;  // this lane's results of steps t-1, t-2, t-3
    // Record words 0-3 of a step's macroblock, loaded four steps ahead into
    // one of four registers that nothing touches until its step, so the
    // global-memory latency overlaps the steps between.
    auto recAt = [&](int x) {
      return x >= 0 && x < rowDone ? reinterpret_cast<const uint4*>(rowRec + x)[0] : make_uint4(0u, 0u, 0u, 0u);
    };
    auto step = [&](int t, const uint4& cur) {
      const int rx = t - 2 * lane;
      const bool act = t < steps && rx >= 0 && rx < rowDone;
      uint32_t above = __shfl_up_sync(kFull, h2, 1);
      uint32_t ar = __shfl_up_sync(kFull, h1, 1);
      uint32_t al = __shfl_up_sync(kFull, h3, 1);
      uint32_t out = 0;
      if (act) {
        if (lane == 0 && p0 > 0) {
          above = upRow[rx];
          ar = rx + 1 < tw ? upRow[rx + 1] : 0u;
          al = rx > 0 ? upRow[rx - 1] : 0u;
        }
        uint32_t* const rw = reinterpret_cast<uint32_t*>(rowRec + rx);
        const uint32_t w0 = cur.x;
        const int mode = (int)(w0 & 0xFF);
        if (mode == kRecSkip || mode == kRecInter) {
          Nbr n;
          n.aOK = rx > 0;
          n.bOK = ry > 0;
          n.arOK = n.bOK && rx + 1 < tw;
          n.cOK = n.arOK || (n.bOK && n.aOK);
          n.mvA = h1;
          n.mvB = n.bOK ? above : 0u;
          n.mvC = n.cOK ? (n.arOK ? ar : al) : 0u;
          uint32_t pred = predictMV(n);
          if (mode == kRecSkip) {
            rw[2] = pred;
            out = pred;
          } else {
            const bool golden = ((w0 >> 8) & 0xFF) == refGolden;
            const int part = (int)((w0 >> 16) & 0xFF);
            if (golden) pred = 0;
            const uint32_t v0 = packMV(clampMV(mvX(pred) + mvX(cur.z)), clampMV(mvY(pred) + mvY(cur.z)));
            rw[2] = v0;
            if (part != partWhole) {
              rw[3] = packMV(clampMV(mvX(v0) + mvX(cur.w)), clampMV(mvY(v0) + mvY(cur.w)));
              if (part == part8x8) {
                const uint32_t d2 = rw[4], d3 = rw[5];
                rw[4] = packMV(clampMV(mvX(v0) + mvX(d2)), clampMV(mvY(v0) + mvY(d2)));
                rw[5] = packMV(clampMV(mvX(v0) + mvX(d3)), clampMV(mvY(v0) + mvY(d3)));
              }
            }
            out = golden ? 0u : v0;
          }
        }
        if (lastRowOfPass) nextUp[rx] = out;
      }
      h3 = h2;
      h2 = h1;
      h1 = out;
    };
    const int base = -2 * lane;
    uint4 q0 = recAt(base), q1 = recAt(base + 1), q2 = recAt(base + 2), q3 = recAt(base + 3);
    for (int t = 0; t < steps; t += 4) {
      step(t, q0);
      q0 = recAt(base + t + 4);
      step(t + 1, q1);
      q1 = recAt(base + t + 5);
      step(t + 2, q2);
      q2 = recAt(base + t + 6);
      step(t + 3, q3);
      q3 = recAt(base + t + 7);
    }
    __syncwarp();  // the pass's last row is read by the next pass's lane 0
  }
}

constexpr int kEntropyWarps = kEntropyTilesPerJob;

// One macroblock's grammar (decodeInterMB, ebiv/decode_inter.go:8-62;
// decodeLumaMB / decodeChromaMB, ebiv/decode_intra.go:137-187).  With kOut
// the record and the coefficient regions are written: by lanes 0-2 of a
// warp that runs the macroblock together, or, with kThread, all by the one
// thread that runs it.  Returns 1 when the macroblock is intra and written
// (an entry of the tile's intra list).
template <bool kOut, bool kThread, class S>
__device__ __forceinline__ int decodeMB(S& d, int inter, MBRec* rec, uint32_t* coef, int lane) {
  int mode = 0;
  if (inter) {
    mode = d.sym(ctxMBMode);
    if (mode == mbSkip) {
      // Skip macroblock (most of an inter frame): a fixed record whose
      // vector predictVectors fills in; nothing else to decode.
      if (kOut) {
        const uint4 a = make_uint4(kRecSkip, 0u, 0u, 0u), z = make_uint4(0u, 0u, 0u, 0u),
                    c = make_uint4(0u, 0u, 0u, kWriteAll);
        uint4* q = reinterpret_cast<uint4*>(rec);
        if (kThread) {
          q[0] = a;
          q[1] = z;
          q[2] = c;
        } else if (lane < 3) {
          q[lane] = lane == 0 ? a : (lane == 1 ? z : c);
        }
      }
      return 0;
    }
  }
  Rec r;
  r.clear();
  bool intra = !inter;
  uint32_t w = 0;
  BlockPlan p;
  int blocks;
  if (inter) {
    blocks = interHeader(d, r, mode, &p, &intra);
  } else {
    intraHeader(d, r, &p);
    blocks = d.err ? 0 : 1;
  }
  if (blocks) {
    uint32_t nz;
    const int nd = entropyBlocks<kOut>(d, r, p, coef, kThread ? 0 : lane, &nz);
    r.nz = nz;
    w = writeMask(p, nd);
  }
  r.wm = w;
  if (kOut) {
    if (kThread) r.storeAll(rec);
    else r.store(rec, lane);
  }
  return intra && w ? 1 : 0;
}

// The full chain of a tile, by one warp (the frame's tables are in sT): the
// rANS symbols drive the macroblock grammar, and every macroblock reached
// gets its record (inter vectors as deltas), its coefficient regions and,
// when it is intra and written, an entry in the tile's intra list (raster
// order).  Returns the macroblocks reached (all of them unless the chain
// stopped at an error).
__device__ __noinline__ int fullChain(const FrameDesc* fp, int tile, const EntropyTables& sT, int lane) {
  const int mbCols = fp->mbCols;
  const int inter = fp->inter;
  MBRec* const recs = fp->mbrec;
  uint32_t* const coefBase = fp->coef;
  const TileRange tr = fp->tiles[tile];
  uint32_t* const intraList = fp->intraList + tr.mbBase;
  const int x0 = tr.mbX0, x1 = tr.mbX1, y0 = tr.mbY0, y1 = tr.mbY1;
  const int tw = x1 - x0, total = tw * (y1 - y0);
  ChainT<false> d;
  d.reset(fp->pkt + tr.offset, tr.length, &sT);
  d.lane = lane;
  int done = 0, intraCount = 0;
  for (int mby = y0; mby < y1 && !d.err; mby++) {
    for (int mbx = x0; mbx < x1; mbx++) {
      const int idx = mby * mbCols + mbx;
      if (decodeMB<true, false>(d, inter, recs + idx, coefBase + (size_t)idx * kCoefPerMB, lane)) {
        if (lane == 0) intraList[intraCount] = (uint32_t)idx;
        intraCount++;
      }
      done++;
      if (d.err) break;
    }
  }
  // Macroblocks the tile never reached are left untouched by reconstruction.
  for (int k = done + lane; k < total; k += 32) {
    MBRec* r = recs + (size_t)(y0 + k / tw) * mbCols + x0 + k % tw;
    r->mode = kRecNone;
    r->wmask = 0;
  }
  if (lane == 0) {
    TileStat ts;
    ts.err = d.err;
    ts.intraCount = intraCount;
    ts.done = done;
    ts.errAt = kFullChain;
    fp->tileStat[tile] = ts;
    if (d.err) atomicExch(fp->status, kErrCorrupt);
  }
  return done;
}

// The symbol chain of a tile, by one warp: only the rANS decoder and the
// grammar decisions that pick the next context, every symbol appended to
// the tile's log and each macroblock's first symbol index recorded; kParse
// rebuilds the records from the log in parallel.  Returns false when the
// log would overflow (the caller then runs fullChain).
__device__ __forceinline__ bool symbolChain(const FrameDesc* fp, int tile, const EntropyTables& sT, int lane) {
  const int inter = fp->inter;
  const TileRange tr = fp->tiles[tile];
  const int tw = tr.mbX1 - tr.mbX0, total = tw * (tr.mbY1 - tr.mbY0);
  uint32_t* const mbOff = fp->symOff + tr.mbBase;
  ChainT<true> d;
  d.reset(fp->pkt + tr.offset, tr.length, &sT);
  d.lane = lane;
  d.log = fp->symLog + (size_t)tr.mbBase * fp->symPerMB;
  d.cap = total * fp->symPerMB;
  if (d.err) d.errAt = 0;  // too short to initialise: the tile fails at once
  int done = 0;
  for (int k = 0; k < total && !d.err; k++) {
    if (lane == 0) mbOff[k] = (uint32_t)d.n;
    if (!d.room(kMBHeaderSymbols)) break;
    decodeMB<false, false>(d, inter, nullptr, nullptr, lane);
    done++;
  }
  if (d.err == kOverflow) return false;
  if (lane == 0) {
    TileStat* ts = fp->tileStat + tile;
    ts->err = d.err;
    ts->done = done;
    ts->errAt = d.errAt;
    if (d.err) atomicExch(fp->status, kErrCorrupt);
  }
  return true;
}

// Entropy jobs: up to kEntropyWarps tiles of one frame per job, one warp per
// tile, sharing the frame's symbol tables.  A tile runs the symbol chain
// when its frame has a symbol log (the full chain when the log would
// overflow), else the full chain.  With a queue counter the grid is
// persistent: each CTA takes jobs (longest first, as listed) until none are
// left, so a round with more jobs than resident CTAs has no second-wave
// tail; without one, CTA b runs job b.
__global__ void __launch_bounds__(32 * kEntropyWarps, 4) kEntropy(const FrameDesc* frames, const int4* jobs, int njobs,
                                                                   int* next) {
  __shared__ EntropyTables sT;
  __shared__ int sJob;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (;;) {
    if (threadIdx.x == 0) sJob = next ? atomicAdd(next, 1) : (int)blockIdx.x;
    __syncthreads();
    const int jb = sJob;
    if (jb >= njobs) return;  // the same for the whole CTA
    const int4 job = jobs[jb];
    const FrameDesc* fp = frames + job.x;
    buildTables(sT, *fp->tables, threadIdx.x, blockDim.x);
    if (warp < job.z) {
      const int tile = job.y + warp;
      if (!fp->symLog || !symbolChain(fp, tile, sT, lane)) fullChain(fp, tile, sT, lane);
    }
    if (!next) return;
    __syncthreads();  // every warp is done with sT and sJob before the next job
  }
}

// Rebuilds the records of the symbol-path tiles from their logs, one warp
// per macroblock over every macroblock of the launch's tiles (grid.y: job *
// kEntropyTilesPerJob + tile within the job; grid.x * kParseWarps: the
// macroblock's raster index within its tile).  The warp first copies a
// window of the tile's log from the macroblock's first symbol into shared
// memory (aligned 16-byte loads), then replays the macroblock's grammar
// (decodeMB, the warp's lanes writing the record and the coefficient
// regions) reading the window, and past it the log in global memory.  A flag
// per macroblock marks the written intra ones for kTileFinish.
constexpr int kParseWarps = 8;
constexpr int kParseWindow = 512;  // bytes of log per warp in shared memory

struct WindowReplay {
  const uint8_t* win;  // shared: log bytes [w0, w0 + wlen)
  const uint8_t* log;  // global: the tile's log
  int32_t w0, wlen, k, errAt, end, err;
  __device__ __forceinline__ int symAt(int) {
    if (err) return 0;
    if (k >= end) {  // unreachable while replay and chain agree; keeps every read in bounds
      err = kErrCorrupt;
      return 0;
    }
    const int r = k - w0;
    const int s = r < wlen ? win[r] : log[k];
    k++;
    if (k > errAt) err = kErrCorrupt;
    return s;
  }
  __device__ __forceinline__ int sym(int) { return symAt(0); }
  __device__ __forceinline__ bool room(int) const { return true; }
};

__global__ void __launch_bounds__(32 * kParseWarps) kParseMB(const FrameDesc* frames, const int4* jobs, int njobs) {
  __shared__ __align__(16) uint8_t sWin[kParseWarps][kParseWindow];
  const int jb = (int)blockIdx.x / kEntropyTilesPerJob, tj = (int)blockIdx.x % kEntropyTilesPerJob;
  if (jb >= njobs) return;
  const int4 job = jobs[jb];
  if (tj >= job.z) return;
  const FrameDesc* fp = frames + job.x;
  const int tile = job.y + tj;
  const TileStat st = fp->tileStat[tile];
  if (st.errAt == kFullChain) return;
  const TileRange tr = fp->tiles[tile];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int tw = tr.mbX1 - tr.mbX0, total = tw * (tr.mbY1 - tr.mbY0);
  const int k = (int)blockIdx.y * kParseWarps + warp;
  if (k >= total) return;
  const int idx = (tr.mbY0 + k / tw) * fp->mbCols + tr.mbX0 + k % tw;
  MBRec* const rec = fp->mbrec + idx;
  uint8_t* const flags = reinterpret_cast<uint8_t*>(fp->lvgrid) + tr.mbBase;
  if (k >= st.done) {  // never reached: left untouched by reconstruction
    if (lane == 0) {
      rec->mode = kRecNone;
      rec->wmask = 0;
      flags[k] = 0;
    }
    return;
  }
  const uint8_t* const log = fp->symLog + (size_t)tr.mbBase * fp->symPerMB;
  const int end = total * fp->symPerMB;
  const int first = (int)fp->symOff[tr.mbBase + k];
  // The window: the aligned 16-byte blocks from the one holding the first
  // symbol, clipped to the tile's log.
  const int w0 = first & ~15;
  const int wlen = max(0, min(kParseWindow, (end & ~15) - w0));  // whole 16-byte blocks only
  uint8_t* const win = sWin[warp];
  for (int o = lane * 16; o < wlen; o += 32 * 16)
    *reinterpret_cast<uint4*>(win + o) = *reinterpret_cast<const uint4*>(log + w0 + o);
  __syncwarp();
  WindowReplay r;
  r.win = win;
  r.log = log;
  r.w0 = w0;
  r.wlen = wlen;
  r.k = first;
  r.errAt = st.errAt;
  r.end = end;
  r.err = r.k > r.errAt ? kErrCorrupt : 0;
  const int f = decodeMB<true, false>(r, fp->inter, rec, fp->coef + (size_t)idx * kCoefPerMB, lane);
  if (lane == 0) flags[k] = (uint8_t)f;
}

// After kParseMB: per tile (one CTA per tile of a job) the written intra
// macroblocks listed in raster order, and (inter frames) the tile's vector
// wavefront.  Tiles the full chain decoded have their intra list already;
// only the wavefront runs for them.
constexpr int kParseThreads = 128;
__global__ void __launch_bounds__(kParseThreads) kTileFinish(const FrameDesc* frames, const int4* jobs, int njobs) {
  __shared__ WarpRows sR;
  __shared__ int sWarp[kParseThreads / 32];
  const int jb = blockIdx.x;
  if (jb >= njobs) return;
  const int4 job = jobs[jb];
  if ((int)blockIdx.y >= job.z) return;
  const FrameDesc* fp = frames + job.x;
  const int tile = job.y + (int)blockIdx.y;
  const TileRange tr = fp->tiles[tile];
  const TileStat st = fp->tileStat[tile];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int mbCols = fp->mbCols, tw = tr.mbX1 - tr.mbX0;
  const int done = st.done;
  if (st.errAt != kFullChain) {
    const uint8_t* const flags = reinterpret_cast<const uint8_t*>(fp->lvgrid) + tr.mbBase;
    int base = 0;
    for (int k0 = 0; k0 < done; k0 += kParseThreads) {
      const int k = k0 + tid;
      const bool f = k < done && flags[k] != 0;
      const unsigned m = __ballot_sync(kFull, f);
      if (lane == 0) sWarp[warp] = __popc(m);
      __syncthreads();
      int before = base, chunk = 0;
      for (int w2 = 0; w2 < kParseThreads / 32; w2++) {
        if (w2 < warp) before += sWarp[w2];
        chunk += sWarp[w2];
      }
      if (f) {
        const int idx = (tr.mbY0 + k / tw) * mbCols + tr.mbX0 + k % tw;
        fp->intraList[tr.mbBase + before + __popc(m & ((1u << lane) - 1u))] = (uint32_t)idx;
      }
      base += chunk;
      __syncthreads();
    }
    if (tid == 0) fp->tileStat[tile].intraCount = base;
  }
  if (fp->inter && warp == 0) predictVectors(fp, tile, done, sR, lane);
}

// ---------------------------------------------------------------------------
// Dequantization + inverse DCT of a whole macroblock (warp-cooperative)
// ---------------------------------------------------------------------------
// Every coded block of the macroblock at once (ebiv/quant.go:72-80,
// ebiv/transform.go:129-194): bit k of mask selects luma block k of the
// tx-sized grid, bits 16/17 the Cb/Cr 8x8 blocks.  dense and tmp are
// per-warp scratch of 384 words; on return dense holds the luma residual
// (16x16 raster) in words 0-255 and the Cb and Cr residuals (8x8 raster) in
// 256-319 and 320-383, zero at the positions of unselected blocks.
__device__ void mbResidual(const uint32_t* coef, int tx, uint32_t mask, int32_t qdc, int32_t qac, int32_t* dense,
                           int32_t* tmp, int lane) {
  const int n = 4 << tx, nn = n * n, per = 4 >> tx, nb = per * per;
  for (int i = lane; i < 384; i += 32) dense[i] = 0;
  __syncwarp();
  // Scatter the sparse levels (luma block b at dense[b*nn], Cb at 256, Cr at
  // 320).  Lane b reads block b's count; the entries of all blocks are then
  // fetched as one flattened list, up to four per lane in flight.
  const int nEnt = nb + 2;
  int myCount = 0;
  if (lane < nEnt) {
    const bool luma = lane < nb;
    if ((mask >> (luma ? lane : 16 + lane - nb)) & 1)
      myCount = (int)coef[luma ? lane * (nn + 1) : (lane == nb ? kCoefCb : kCoefCr)];
  }
  int incl = myCount;
  for (int o = 1; o < 32; o <<= 1) {
    const int v = __shfl_up_sync(kFull, incl, o);
    if (lane >= o) incl += v;
  }
  const int total = __shfl_sync(kFull, incl, 31);
  const int excl = incl - myCount;
  for (int t0 = 0; t0 < total; t0 += 128) {
    uint32_t val[4];
    int dst[4];
#pragma unroll
    for (int u = 0; u < 4; u++) {
      const int t = t0 + u * 32 + lane;
      int ob = 0, oe = 0;
      for (int b = 0; b < nEnt; b++) {  // owning block: last nonempty block starting at or before t
        const int eb = __shfl_sync(kFull, excl, b), cb = __shfl_sync(kFull, myCount, b);
        if (cb > 0 && eb <= t) {
          ob = b;
          oe = eb;
        }
      }
      const bool luma = ob < nb;
      dst[u] = -1;
      if (t < total) {
        val[u] = coef[(luma ? ob * (nn + 1) : (ob == nb ? kCoefCb : kCoefCr)) + 1 + (t - oe)];
        dst[u] = luma ? ob * nn : 256 + (ob - nb) * 64;
      }
    }
#pragma unroll
    for (int u = 0; u < 4; u++) {
      if (dst[u] < 0) continue;
      const int pos = (int)(val[u] & 0xFF);
      dense[dst[u] + pos] = wmul((int32_t)val[u] >> 8, pos == 0 ? qdc : qac);
    }
  }
  __syncwarp();
  // Columns: tmp[b][i][l] = sum_k c[k][i] * dense[b][k][l].
  for (int o = lane; o < 384; o += 32) {
    const bool luma = o < 256;
    const int bn = luma ? n : 8, base = luma ? (o / nn) * nn : 256 + ((o - 256) >> 6) * 64;
    const int q = o - base, i = q / bn, l = q - i * bn;
    const int32_t* c = gDct[luma ? tx : 1];
    int64_t acc = 0;
    for (int k = 0; k < bn; k++) acc += (int64_t)__ldg(c + k * bn + i) * (int64_t)dense[base + k * bn + l];
    tmp[o] = (int32_t)((acc + 4096) >> 13);
  }
  __syncwarp();
  // Rows: out[i][m] = sum_l c[l][m] * tmp[b][i][l], into dense (read only
  // by the column pass, which is complete).
  for (int o = lane; o < 384; o += 32) {
    const bool luma = o < 256;
    const int bn = luma ? n : 8, base = luma ? (o / nn) * nn : 256 + ((o - 256) >> 6) * 64;
    const int q = o - base, i = q / bn, m = q - i * bn;
    const int32_t* c = gDct[luma ? tx : 1];
    int64_t acc = 0;
    for (int l = 0; l < bn; l++) acc += (int64_t)__ldg(c + l * bn + m) * (int64_t)tmp[base + i * bn + l];
    const int32_t v = (int32_t)((acc + 4096) >> 13);
    if (luma) {
      const int b = o / nn, bx = (b % per) * n, by = (b / per) * n;
      dense[(by + i) * 16 + bx + m] = v;
    } else {
      dense[o] = v;
    }
  }
  __syncwarp();
}

// ---------------------------------------------------------------------------
// Motion compensation samples (clamped form of ebiv/motioncomp.go:49-97)
// ---------------------------------------------------------------------------
// A macroblock's residual between kInterRecon phase 0 and its consumer
// (phase 1, or the intra stage), stored over its coefficient region.  When
// every value fits in 16 bits (any real stream: a coded sample's residual is
// within a few thousand), values go in pairs — word w < 128: luma samples w
// (low half) and w + 128; word 256 + w, w < 64: chroma samples 256 + w and
// 320 + w — and word kResFormatWord is 1: 768 bytes instead of 1536.
// Otherwise (a hostile stream whose int32-wrapped arithmetic made a value no
// 16-bit number reproduces under the reconstruction's wrapping add) the 384
// words are stored as they are and the format word is 0.  Both formats put
// the values the readers load first at the same words.
constexpr int kResFormatWord = kCoefPerMB - 1;
__device__ __forceinline__ int32_t lo16(uint32_t w) { return (int32_t)(int16_t)(w & 0xFFFFu); }
__device__ __forceinline__ int32_t hi16(uint32_t w) { return (int32_t)(int16_t)(w >> 16); }
__device__ __forceinline__ int resWordLo(int w) { return w < 128 ? w : w + 128; }  // w < 192: the low sample
__device__ __forceinline__ void storeResidual(uint32_t* cg, const int32_t* res, int lane) {
  bool fits = true;
  for (int q = lane; q < 384; q += 32) fits = fits && res[q] >= -32768 && res[q] <= 32767;
  fits = __all_sync(kFull, fits);
  if (fits) {
    for (int w = lane; w < 192; w += 32) {
      const int a = resWordLo(w), b = a + (w < 128 ? 128 : 64);
      cg[w < 128 ? w : w + 128] = (uint32_t)(uint16_t)res[a] | ((uint32_t)res[b] << 16);
    }
  } else {
    for (int q = lane; q < 384; q += 32) cg[q] = (uint32_t)res[q];
  }
  if (lane == 0) cg[kResFormatWord] = fits ? 1u : 0u;
}
__device__ __forceinline__ void loadResidual(const uint32_t* cg, int32_t* res, int lane) {
  if (cg[kResFormatWord]) {
    for (int w = lane; w < 192; w += 32) {
      const uint32_t v = cg[w < 128 ? w : w + 128];
      const int a = resWordLo(w);
      res[a] = lo16(v);
      res[a + (w < 128 ? 128 : 64)] = hi16(v);
    }
  } else {
    for (int q = lane; q < 384; q += 32) res[q] = (int32_t)cg[q];
  }
}

__device__ __forceinline__ int lumaSample(const uint8_t* p, int stride, int w, int h, int px, int py, int fx, int fy) {
  auto g = [&](int x, int y) -> int32_t { return __ldg(p + (size_t)clampC(y, h) * stride + clampC(x, w)); };
  if (fx == 0 && fy == 0) return g(px, py);
  if (fy == 0) {
    const int32_t* t = cTaps[fx];
    return clampByteD((t[0] * g(px - 1, py) + t[1] * g(px, py) + t[2] * g(px + 1, py) + t[3] * g(px + 2, py) + 32) >> 6);
  }
  if (fx == 0) {
    const int32_t* t = cTaps[fy];
    return clampByteD((t[0] * g(px, py - 1) + t[1] * g(px, py) + t[2] * g(px, py + 1) + t[3] * g(px, py + 2) + 32) >> 6);
  }
  const int32_t* tx = cTaps[fx];
  const int32_t* ty = cTaps[fy];
  int32_t v = 0;
#pragma unroll
  for (int k = 0; k < 4; k++) {
    const int yy = py - 1 + k;
    v += ty[k] * (tx[0] * g(px - 1, yy) + tx[1] * g(px, yy) + tx[2] * g(px + 1, yy) + tx[3] * g(px + 2, yy));
  }
  return clampByteD((v + 2048) >> 12);
}

__device__ __forceinline__ int chromaSample(const uint8_t* p, int stride, int w, int h, int px, int py, int fx, int fy) {
  auto g = [&](int x, int y) -> int32_t { return __ldg(p + (size_t)clampC(y, h) * stride + clampC(x, w)); };
  if (fx == 0 && fy == 0) return g(px, py);
  const int32_t v = (8 - fx) * (8 - fy) * g(px, py) + fx * (8 - fy) * g(px + 1, py) + (8 - fx) * fy * g(px, py + 1) +
                    fx * fy * g(px + 1, py + 1);
  return (v + 32) >> 6;
}

__device__ __forceinline__ int partIndex(int part, int x, int y) {  // luma coords within the MB
  switch (part) {
    case part16x8: return y >= 8;
    case part8x16: return x >= 8;
    case part8x8: return (y >= 8) * 2 + (x >= 8);
    default: return 0;
  }
}

// ---------------------------------------------------------------------------
// Register copies for the reconstruction kernels.  Their byte stores to the
// planes may alias any other memory as far as the compiler knows, so fields
// read through the descriptor or record pointers would be re-loaded after
// every store; these copies are read once.
// ---------------------------------------------------------------------------
struct ReconView {
  uint8_t* rec[3];
  const uint8_t* ref[3];
  const uint8_t* gold[3];
  int strideY, strideC, padW, padH, padCW, padCH, mbCols;
  int32_t qdc, qac;
  const MBRec* mbrec;
  uint32_t* coef;
  __device__ __forceinline__ void load(const FrameDesc& f) {
    for (int k = 0; k < 3; k++) {
      rec[k] = f.rec[k];
      ref[k] = f.ref[k];
      gold[k] = f.gold[k];
    }
    strideY = f.strideY;
    strideC = f.strideC;
    padW = f.padW;
    padH = f.padH;
    padCW = f.padCW;
    padCH = f.padCH;
    mbCols = f.mbCols;
    qdc = f.qdc;
    qac = f.qac;
    mbrec = f.mbrec;
    coef = f.coef;
  }
};

// A macroblock record as three 16-byte words (see MBRec).
struct RecRegs {
  uint4 a, b, c;  // words 0-3, 4-7, 8-11
  __device__ __forceinline__ void load(const MBRec* p) {
    const uint4* q = reinterpret_cast<const uint4*>(p);
    a = q[0];
    b = q[1];
    c = q[2];
  }
  __device__ __forceinline__ int mode() const { return (int)(a.x & 0xFF); }
  __device__ __forceinline__ int ref() const { return (int)((a.x >> 8) & 0xFF); }
  __device__ __forceinline__ int part() const { return (int)((a.x >> 16) & 0xFF); }
  __device__ __forceinline__ int cbp() const { return (int)(a.x >> 24); }
  __device__ __forceinline__ int tx() const { return (int)(a.y & 0xFF); }
  __device__ __forceinline__ int cmode() const { return (int)((a.y >> 8) & 0xFF); }
  __device__ __forceinline__ uint32_t mv(int i) const { return i == 0 ? a.z : (i == 1 ? a.w : (i == 2 ? b.x : b.y)); }
  __device__ __forceinline__ int lmode(int k) const {
    const uint32_t w = k < 8 ? (k < 4 ? b.z : b.w) : (k < 12 ? c.x : c.y);
    return (int)((w >> ((k & 3) * 8)) & 0xFF);
  }
  __device__ __forceinline__ uint32_t nzmask() const { return c.z; }
  __device__ __forceinline__ uint32_t wmask() const { return c.w; }
};

// ---------------------------------------------------------------------------
// Stage B1: inter macroblock reconstruction
// ---------------------------------------------------------------------------
constexpr int kInterWarps = 4;

struct InterScratch {
  int32_t res[384];  // levels, then residuals (mbResidual)
  int32_t tmp[384];
};

// Reconstruction kernels are launched with programmatic stream
// serialisation, so a grid may start while the previous kernel of the stream
// runs; this wait (a no-op without a prerequisite grid) holds every thread
// until that kernel's results are complete and visible.
__device__ __forceinline__ void waitPreviousGrid() {
#ifdef __CUDA_ARCH__
  asm volatile("griddepcontrol.wait;" ::: "memory");
#endif
}

// Lets the next kernel of the stream be scheduled now: its CTAs start and
// hold in waitPreviousGrid until this grid is complete, so the launch
// latency overlaps this kernel.
__device__ __forceinline__ void allowNextGrid() {
#ifdef __CUDA_ARCH__
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
#endif
}

// Whether inter macroblock (mbx, mby) of f predicts from pixels of an intra
// macroblock of the previous frame (f.prevRec) — a conservative test over
// the bounding box of its vectors' source blocks, widened for the filter
// taps and chroma rounding.  A previous key frame makes every macroblock
// dependent; a golden-reference macroblock reads an older, complete frame.
__device__ __forceinline__ bool interDepends(const FrameDesc& f, const RecRegs& r, int mode, int part, int mbx,
                                             int mby) {
  if (!f.prevRec) return false;
  if (f.prevKey) return true;
  if (mode == kRecInter && r.ref() == refGolden) return false;
  const int np = mode == kRecInter ? (part == partWhole ? 1 : (part == part8x8 ? 4 : 2)) : 1;
  int lo = 1 << 30, hi = -(1 << 30), vlo = 1 << 30, vhi = -(1 << 30);
  for (int i = 0; i < np; i++) {
    const uint32_t m = r.mv(i);
    const int dx = (int16_t)(m & 0xFFFFu) >> 2, dy = (int16_t)(m >> 16) >> 2;
    lo = min(lo, dx);
    hi = max(hi, dx);
    vlo = min(vlo, dy);
    vhi = max(vhi, dy);
  }
  // Samples outside the plane are clamped to its edge: clamp each end of the
  // box on its own, so a box wholly outside still names the edge macroblocks.
  const int x0 = min(max(0, mbx * 16 + lo - 4), f.padW - 1), x1 = min(max(0, mbx * 16 + 15 + hi + 4), f.padW - 1);
  const int y0 = min(max(0, mby * 16 + vlo - 4), f.padH - 1), y1 = min(max(0, mby * 16 + 15 + vhi + 4), f.padH - 1);
  const int bx0 = x0 >> 4, bx1 = x1 >> 4, by0 = y0 >> 4, by1 = y1 >> 4;
  if ((bx1 - bx0 + 1) * (by1 - by0 + 1) > 16) return true;  // wide spread: wait
  for (int by = by0; by <= by1; by++)
    for (int bx = bx0; bx <= bx1; bx++) {
      const MBRec* q = f.prevRec + by * f.mbCols + bx;
      if (q->mode == kRecIntra && q->wmask != 0) return true;
    }
  return false;
}

// phase 0: the macroblocks that do not depend on the previous frame's intra
// stage (all of them when that stage is complete), and the residuals of the
// intra macroblocks; phase 1: the other inter macroblocks.
__global__ void __launch_bounds__(32 * kInterWarps, 6) kInterRecon(const FrameDesc* frames, int phase) {
  allowNextGrid();
  waitPreviousGrid();
  __shared__ InterScratch sS[kInterWarps];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const FrameDesc& f = frames[blockIdx.y];
  if (f.gate && *f.gate) {
    if (threadIdx.x == 0) atomicExch(f.status, kSkipped);
    return;
  }
  const int idx = blockIdx.x * kInterWarps + warp;
  if (idx >= f.mbCols * f.mbRows) return;
  ReconView v;
  v.load(f);
  RecRegs r;
  r.load(v.mbrec + idx);
  const int mode = r.mode();
  const uint32_t wm = r.wmask();
  if (!wm) return;
  InterScratch& S = sS[warp];
  // An intra macroblock's residual needs no pixels: phase 0 computes it and
  // stores it over the macroblock's coefficient region, where the intra
  // stage reads it.
  const bool intra = mode == kRecIntra;
  if (intra ? phase != 0 : (!f.inter || (mode != kRecSkip && mode != kRecInter))) return;
  const int mbx = idx % v.mbCols, mby = idx / v.mbCols;
  const bool golden = mode == kRecInter && r.ref() == refGolden;
  const uint8_t* const* refp = golden ? v.gold : v.ref;
  const int part = mode == kRecInter ? r.part() : partWhole;
  const int cbp = mode == kRecInter ? r.cbp() : 0;
  bool deferred = false;  // phase 0: left to phase 1, whose residual is computed now
  if (intra) {
  } else if (phase == 0) {
    deferred = interDepends(f, r, mode, part, mbx, mby);
    if (lane == 0 && f.prevRec) f.dep[idx] = deferred ? 1 : 0;
  } else if (!f.prevRec || !f.dep[idx]) {
    return;
  }
  const uint32_t nzm = r.nzmask();
  const int tx = r.tx();

  // Residuals of the coded blocks that are written, all at once.  Phase 0
  // computes those of intra and deferred macroblocks and stores them over
  // the coefficient region (off the critical path); phase 1 reads them back.
  uint32_t resMask = intra ? nzm & wm : 0;
  if (cbp & cbpLuma) resMask |= nzm & wm & 0xFFFFu;
  if (cbp & cbpCb) resMask |= nzm & wm & (1u << 16);
  if (cbp & cbpCr) resMask |= nzm & wm & (1u << 17);
  uint32_t* const cg = v.coef + (size_t)idx * kCoefPerMB;
  if (phase == 1) {
    if (resMask) loadResidual(cg, S.res, lane);
    __syncwarp();
  } else if (resMask) {
    mbResidual(cg, tx, resMask, v.qdc, v.qac, S.res, S.tmp, lane);
  }
  if (intra || deferred) {
    if (resMask) storeResidual(cg, S.res, lane);
    return;
  }

  // Luma: lane -> row lane/2, 8 columns.
  {
    const int row = lane >> 1, c0 = (lane & 1) * 8;
    const uint32_t m = r.mv(partIndex(part, c0, row));
    const int mvx = (int16_t)(m & 0xFFFFu), mvy = (int16_t)(m >> 16);
    const int fx = mvx & 3, fy = mvy & 3;
    const int sx = mbx * 16 + c0 + (mvx >> 2), sy = mby * 16 + row + (mvy >> 2);
    int pred[8];
    if (fx == 0 && fy == 0 && sx >= 0 && sy >= 0 && sy < v.padH && sx + 8 <= v.padW && (sx & ~7) + 16 <= v.strideY) {
      // Whole-pel vector with the row segment inside the plane: the samples
      // need no clamping; two aligned 8-byte loads cover them (rows start
      // 64-byte aligned and the loads stay inside the row's stride).
      const uint8_t* rowp = refp[0] + (size_t)sy * v.strideY;
      const int base = sx & ~7, sh = (sx & 7) * 8;
      uint64_t w = __ldg(reinterpret_cast<const unsigned long long*>(rowp + base));
      if (sh) w = (w >> sh) | ((uint64_t)__ldg(reinterpret_cast<const unsigned long long*>(rowp + base + 8)) << (64 - sh));
#pragma unroll
      for (int k = 0; k < 8; k++) pred[k] = (int)((w >> (8 * k)) & 0xFF);
    } else {
#pragma unroll
      for (int k = 0; k < 8; k++) pred[k] = lumaSample(refp[0], v.strideY, v.padW, v.padH, sx + k, sy, fx, fy);
    }
    const int n = 4 << tx, per = 4 >> tx;
    uint8_t* out = v.rec[0] + (size_t)(mby * 16 + row) * v.strideY + mbx * 16 + c0;
    const int blkA = (row / n) * per + c0 / n, blkB = (row / n) * per + (c0 + 7) / n;
    if (((wm >> blkA) & 1) && ((wm >> blkB) & 1)) {
      uint64_t o = 0;  // all eight samples are written: one 8-byte store (out is 8-byte aligned)
#pragma unroll
      for (int k = 0; k < 8; k++) {
        const int val = resMask ? clampByteD(wadd(pred[k], S.res[row * 16 + c0 + k])) : pred[k];
        o |= (uint64_t)(uint32_t)val << (8 * k);
      }
      *reinterpret_cast<unsigned long long*>(out) = o;
    } else {
#pragma unroll
      for (int k = 0; k < 8; k++) {
        const int c = c0 + k;
        const int blk = (row / n) * per + c / n;
        if (!((wm >> blk) & 1)) continue;
        const int val = resMask ? clampByteD(wadd(pred[k], S.res[row * 16 + c])) : pred[k];
        out[k] = (uint8_t)val;
      }
    }
  }
  // Chroma: lane -> row lane/4, 2 columns; Cb then Cr.
#pragma unroll
  for (int pl = 0; pl < 2; pl++) {
    const uint32_t bit = 1u << (16 + pl);
    if (!(wm & bit)) continue;
    const int row = lane >> 2, c0 = (lane & 3) * 2;
    const uint32_t m = r.mv(partIndex(part, c0 * 2, row * 2));
    const int mvx = (int16_t)(m & 0xFFFFu), mvy = (int16_t)(m >> 16);
    const int fx = mvx & 7, fy = mvy & 7;
    const int sx = mbx * 8 + c0 + (mvx >> 3), sy = mby * 8 + row + (mvy >> 3);
    int p0 = chromaSample(refp[1 + pl], v.strideC, v.padCW, v.padCH, sx, sy, fx, fy);
    int p1 = chromaSample(refp[1 + pl], v.strideC, v.padCW, v.padCH, sx + 1, sy, fx, fy);
    if (resMask & bit) {
      p0 = clampByteD(wadd(p0, S.res[256 + pl * 64 + row * 8 + c0]));
      p1 = clampByteD(wadd(p1, S.res[256 + pl * 64 + row * 8 + c0 + 1]));
    }
    uint8_t* out = v.rec[1 + pl] + (size_t)(mby * 8 + row) * v.strideC + mbx * 8 + c0;
    out[0] = (uint8_t)p0;
    out[1] = (uint8_t)p1;
  }
}

// ---------------------------------------------------------------------------
// Stage B2: intra reconstruction wavefront
// ---------------------------------------------------------------------------

// Per-warp scratch of the intra stage.  The macroblock being reconstructed
// lives in a working area in shared memory together with the samples its
// prediction may read: area row 0 is the row above the macroblock (from one
// left of it to 31 right of its left edge: above-left corner, above,
// above-right), column 0 the column to its left; chroma likewise (9 x 9).
constexpr int kAreaW = 48;
struct IntraScratch {
  int32_t ref[2][4 * 16 + 1];  // one reference array per half-warp block
  int32_t res[384];            // the macroblock's residual (computed by kInterRecon phase 0)
  uint8_t areaY[17 * kAreaW];
  uint8_t areaC[2][9 * 16];
};

// The reference sample array of predictIntra after substituteRefs, in
// closed form: ref[0..2n-1] left column bottom-to-top, ref[2n] corner,
// ref[2n+1..4n] top then top-right.  (x0, y0) are the block's coordinates
// in the working area a (row stride as).
__device__ __forceinline__ int32_t refValue(int i, int n, bool avAbove, bool avLeft, bool avAR, const uint8_t* a,
                                            int as, int x0, int y0) {
  // Each entry is one sample of the area: the left column L(r) = (x0-1, y0+r)
  // (rows past n-1 repeat row n-1), the top row Tp(j) = (x0+j, y0-1) (past
  // n-1 without above-right: Tp(n-1)), the corner; a missing side is
  // replaced by the other side's nearest sample, both missing by kDCPred.
  const int corner = 2 * n;
  int ax, ay;
  if (i < corner) {
    ax = avLeft ? x0 - 1 : x0;
    ay = avLeft ? y0 + min(corner - 1 - i, n - 1) : y0 - 1;
  } else if (i == corner) {
    ax = avLeft ? x0 - 1 : x0;
    ay = avAbove ? y0 - 1 : y0;
  } else {
    const int j = i - corner - 1;
    ax = avAbove ? x0 + ((j < n || avAR) ? j : n - 1) : x0 - 1;
    ay = avAbove ? y0 - 1 : y0;
  }
  return (avLeft || avAbove) ? (int32_t)a[ay * as + ax] : kDCPred;
}

// Predicts and reconstructs one n x n block (predictIntra,
// ebiv/predict.go:131-219) at area coordinates (ax, ay) of working area a,
// writing each sample to the area and to plane p at (px, py).  Lanes l of nl
// (a half warp or the whole warp) share the block; every lane of the warp
// calls it, with active false where its half has no block this step, so
// both __syncwarp barriers see the full warp.
__device__ void intraBlock(int32_t* ref, uint8_t* a, int as, int ax, int ay, uint8_t* p, int stride, int px, int py,
                           int n, int mode, bool avAbove, bool avLeft, bool avAR, const int32_t* res, int resStride,
                           int l, int nl, bool active) {
  const int corner = 2 * n;
  if (active)
    for (int i = l; i <= 4 * n; i += nl) ref[i] = refValue(i, n, avAbove, avLeft, avAR, a, as, ax, ay);
  __syncwarp();
  if (!active) {
    __syncwarp();
    return;
  }
  // n is 4, 8 or 16: shifts instead of divisions, and the DC sum's loads
  // issued together (unrolled, predicated past n).
  const int lg = n == 4 ? 2 : (n == 8 ? 3 : 4);
  int32_t dc = 0;
  if (mode == modeDC) {
    int32_t sum = 0;
#pragma unroll
    for (int i = 0; i < 16; i++)
      if (i < n) sum += ref[corner + 1 + i] + ref[corner - 1 - i];
    dc = (sum + n) >> (lg + 1);  // sum >= 0: the division by 2n
  }
  int angle = 0, inv = 0;
  bool vertical = false;
  switch (mode) {
    case modeD45: angle = 32; vertical = true; break;
    case modeD27: angle = 13; vertical = true; break;
    case modeD23: angle = -13; inv = -630; vertical = true; break;
    case modeD135: angle = 32; break;
    case modeD117: angle = 13; break;
    case modeD113: angle = -13; inv = -630; break;
    default: break;
  }
  const int nn = n * n;
  for (int o = l; o < nn; o += nl) {
    const int r = o >> lg, c = o & (n - 1);
    int32_t v;
    switch (mode) {
      case modeV: v = ref[corner + 1 + c]; break;
      case modeH: v = ref[corner - 1 - r]; break;
      case modeTM: v = clampByteD(ref[corner + 1 + c] + ref[corner - 1 - r] - ref[corner]); break;
      case modeDC: v = dc; break;
      default: {
        const int aa = vertical ? r : c, b = vertical ? c : r;
        const int pos = (aa + 1) * angle;
        const int idx = pos >> 5, fact = pos & 31;
        auto ext = [&](int k) -> int32_t {
          if (k >= 0) {
            if (k > 2 * n) return 0;
            return vertical ? ref[corner + k] : ref[corner - k];
          }
          const int t = (k * inv + 128) >> 8;
          return vertical ? ref[corner - t] : ref[corner + t];
        };
        v = ((32 - fact) * ext(b + idx + 1) + fact * ext(b + idx + 2) + 16) >> 5;
      }
    }
    v = res ? clampByteD(wadd(v, res[r * resStride + c])) : clampByteD(v);
    a[(ay + r) * as + ax + c] = (uint8_t)v;  // the block's reference array is already in ref
    p[(size_t)(py + r) * stride + px + c] = (uint8_t)v;
  }
  __syncwarp();
}

// Progress of the intra macroblocks of one tile, shared by the warps of its
// CTA.  luma[m] counts the completed diagonal steps of macroblock m's 4x4
// luma blocks (kLumaDone when the luma is complete, at once for 8x8 and
// 16x16 transforms); chroma[m] is 1 when both chroma blocks are.  Every
// other macroblock of the tile starts complete.  A wait that runs past
// kIntraSpinLimit polls sets abort, which ends every later wait at once;
// the frame is then reported failed.
constexpr int kLumaDone = 10;
constexpr int kIntraSpinLimit = 1 << 20;
struct IntraSync {
  volatile uint8_t* luma;
  volatile uint8_t* chroma;
  volatile int* abort;
  int x0, y0, x1, tw;  // the tile: first column and row, end column, width (macroblocks)
  __device__ __forceinline__ int at(int mbx, int mby) const { return (mby - y0) * tw + (mbx - x0); }
  // Waits until progress word p reaches need (all lanes poll the same word).
  __device__ __forceinline__ void wait(volatile uint8_t* p, int need) const {
    for (int it = 0; *p < need && !*abort; it++) {
      if (it >= kIntraSpinLimit) {
        *abort = 1;
        break;
      }
      __nanosleep(64);
    }
    __threadfence_block();
  }
  // Publishes progress v once every lane's writes so far are visible to the CTA.
  __device__ __forceinline__ void publish(volatile uint8_t* p, int v, int lane) const {
    __threadfence_block();
    __syncwarp();
    if (lane == 0) {
      __threadfence_block();
      *p = (uint8_t)v;
    }
  }
};

// The luma of an intra macroblock.  With 4x4 transforms the blocks run in
// ten diagonal steps (bx + 2*by); step t needs the left neighbour's blocks
// up to step t+3 (its column 3 at rows by), which the macroblock waits for
// step by step, and the row above complete: the above-left and above
// macroblocks done and the above-right one past step 6 (its block (0,3),
// the only one the top-right block reads).  Other transform sizes wait for
// all four neighbours to be done.
__device__ void intraLuma(const ReconView& f, IntraScratch& S, const IntraSync& sy, int mbx, int mby, int lane) {
  const int idx = mby * f.mbCols + mbx;
  RecRegs r;
  r.load(f.mbrec + idx);
  if (r.mode() != kRecIntra) return;
  const uint32_t wm = r.wmask();
  if (!wm) return;
  const uint32_t nzm = r.nzmask();
  const int tx = r.tx(), n = 4 << tx, per = 4 >> tx, nb = per * per;
  const int tileLeft = sy.x0 * 16, tileTop = sy.y0 * 16, tileRight = sy.x1 * 16;
  const int mbLeft = mbx * 16, mbTop = mby * 16, mbRight = mbLeft + 16;
  uint8_t* const Y = f.rec[0];
  const int ys = f.strideY;
  const uint32_t resMask = nzm & wm;
  const uint32_t* rg = f.coef + (size_t)idx * kCoefPerMB;
  const bool up = mbTop > tileTop, left = mbLeft > tileLeft, ar = up && mbRight < tileRight;
  volatile uint8_t* const own = sy.luma + sy.at(mbx, mby);
  volatile uint8_t* const leftP = left ? sy.luma + sy.at(mbx - 1, mby) : nullptr;
  // The residual, the row above and, when the left neighbour is complete,
  // the left column are loaded together (one global latency); otherwise the
  // left column follows the left neighbour's steps.
  const bool lumaRes = (resMask & 0xFFFFu) != 0;
  int32_t rv[8];
  if (lumaRes) {
    // Words lane + 32q (q < 4) hold samples in either format; the format
    // word says whether they are pairs or the second half follows.
    uint32_t w4[4];
#pragma unroll
    for (int q = 0; q < 4; q++) w4[q] = rg[lane + 32 * q];
    if (rg[kResFormatWord]) {
#pragma unroll
      for (int q = 0; q < 4; q++) {
        rv[q] = lo16(w4[q]);
        rv[q + 4] = hi16(w4[q]);
      }
    } else {
#pragma unroll
      for (int q = 0; q < 4; q++) {
        rv[q] = (int32_t)w4[q];
        rv[q + 4] = (int32_t)rg[lane + 32 * (q + 4)];
      }
    }
  }
  if (up) {
    if (left) sy.wait(sy.luma + sy.at(mbx - 1, mby - 1), kLumaDone);
    sy.wait(sy.luma + sy.at(mbx, mby - 1), kLumaDone);
    if (ar) sy.wait(sy.luma + sy.at(mbx + 1, mby - 1), tx == 0 ? 7 : kLumaDone);
  }
  if (left && tx != 0) sy.wait(leftP, kLumaDone);
  // One decision for the whole warp (lane 0's reading of the flag).
  bool leftNow = false;
  if (left) leftNow = __shfl_sync(kFull, *leftP >= kLumaDone ? 1 : 0, 0) != 0;
  if (leftNow) __threadfence_block();
  const int xa = mbLeft - 1 + lane;
  const bool haveA = up && xa >= tileLeft && xa < tileRight;
  const bool haveB = up && lane == 0 && mbLeft + 31 < tileRight;  // area entry 32
  const uint8_t* const rowAbove = Y + (size_t)(mbTop - 1) * ys;
  uint8_t a0 = 0, a1 = 0, lc = 0;
  if (haveA) a0 = rowAbove[xa];
  if (haveB) a1 = rowAbove[mbLeft + 31];
  if (leftNow && lane < 16) lc = Y[(size_t)(mbTop + lane) * ys + mbLeft - 1];
  if (lumaRes)
#pragma unroll
    for (int q = 0; q < 8; q++) S.res[lane + 32 * q] = rv[q];
  if (haveA) S.areaY[lane] = a0;
  if (haveB) S.areaY[32] = a1;
  if (leftNow && lane < 16) S.areaY[(1 + lane) * kAreaW] = lc;
  auto block = [&](int k, int l, int nl, bool active, int half) {
    const int bx = (k & (per - 1)) << (2 + tx), by = (k >> (2 - tx)) << (2 + tx);  // per = 4 >> tx, n = 4 << tx
    const int x0 = mbLeft + bx, y0 = mbTop + by;
    const bool avAbove = y0 > tileTop, avLeft = x0 > tileLeft;
    bool avAR = false;
    if (!(y0 <= tileTop || x0 + 2 * n > tileRight)) avAR = (y0 == mbTop) ? true : (x0 + 2 * n <= mbRight);
    const bool hasRes = (nzm >> k) & 1;
    intraBlock(S.ref[half], S.areaY, kAreaW, 1 + bx, 1 + by, Y, ys, x0, y0, n, active ? r.lmode(k) : 0, avAbove,
               avLeft, avAR, hasRes ? S.res + by * 16 + bx : nullptr, 16, l, nl, active);
  };
  if (tx == 0) {
    // Blocks beyond the first unwritten one (a prefix in raster order) are
    // skipped; each step is published all the same.
    const int half = lane >> 4;
    for (int t = 0; t < 10; t++) {
      if (left && !leftNow && !(t & 1) && t <= 6) {  // left column rows 2t..2t+3, for block (0, t/2)
        sy.wait(leftP, t + 4);
        if (lane < 4) S.areaY[(1 + 2 * t + lane) * kAreaW] = Y[(size_t)(mbTop + 2 * t + lane) * ys + mbLeft - 1];
      }
      __syncwarp();
      int k = -1, seen = 0;
      for (int yy = 0; yy < 4; yy++) {
        const int xx = t - 2 * yy;
        if (xx >= 0 && xx < 4) {
          if (seen == half) k = yy * 4 + xx;
          seen++;
        }
      }
      const bool active = k >= 0 && ((wm >> k) & 1);
      block(active ? k : 0, lane & 15, 16, active, half);
      sy.publish(own, t + 1, lane);
    }
  } else {
    __syncwarp();  // the left column was loaded with the row above
    for (int k = 0; k < nb; k++) {
      if (!((wm >> k) & 1)) break;
      block(k, lane, 32, true, 0);
    }
  }
}

// The chroma of an intra macroblock: waits for the left, above-left and
// above macroblocks' chroma (chroma prediction reads no above-right samples).
__device__ void intraChroma(const ReconView& f, IntraScratch& S, const IntraSync& sy, int mbx, int mby, int lane) {
  const int idx = mby * f.mbCols + mbx;
  RecRegs r;
  r.load(f.mbrec + idx);
  if (r.mode() != kRecIntra) return;
  const uint32_t wm = r.wmask();
  if (!(wm >> 16)) return;
  const uint32_t nzm = r.nzmask();
  const bool up = mby > sy.y0, left = mbx > sy.x0;
  const int cs = f.strideC;
  const uint32_t* rg = f.coef + (size_t)idx * kCoefPerMB;
  const bool chromaRes = ((nzm & wm) >> 16) != 0;
  int32_t rv[4];
  if (chromaRes) {
    const uint32_t a = rg[256 + lane], b = rg[288 + lane];
    if (rg[kResFormatWord]) {
      rv[0] = lo16(a);
      rv[1] = lo16(b);
      rv[2] = hi16(a);
      rv[3] = hi16(b);
    } else {
      rv[0] = (int32_t)a;
      rv[1] = (int32_t)b;
      rv[2] = (int32_t)rg[320 + lane];
      rv[3] = (int32_t)rg[352 + lane];
    }
  }
  if (up) {
    if (left) sy.wait(sy.chroma + sy.at(mbx - 1, mby - 1), 1);
    sy.wait(sy.chroma + sy.at(mbx, mby - 1), 1);
  }
  if (left) sy.wait(sy.chroma + sy.at(mbx - 1, mby), 1);
  const int cl = mbx * 8, ct = mby * 8;
  // Both planes' row above and left column, loaded together.
  const bool haveT = up && lane < 9 && (lane > 0 || left), haveL = left && lane < 8;
  uint8_t t0 = 0, t1 = 0, l0 = 0, l1 = 0;
  if (haveT) {
    t0 = f.rec[1][(size_t)(ct - 1) * cs + cl - 1 + lane];
    t1 = f.rec[2][(size_t)(ct - 1) * cs + cl - 1 + lane];
  }
  if (haveL) {
    l0 = f.rec[1][(size_t)(ct + lane) * cs + cl - 1];
    l1 = f.rec[2][(size_t)(ct + lane) * cs + cl - 1];
  }
  if (chromaRes)
#pragma unroll
    for (int q = 0; q < 4; q++) S.res[256 + lane + 32 * q] = rv[q];
  if (haveT) {
    S.areaC[0][lane] = t0;
    S.areaC[1][lane] = t1;
  }
  if (haveL) {
    S.areaC[0][(1 + lane) * 16] = l0;
    S.areaC[1][(1 + lane) * 16] = l1;
  }
  __syncwarp();
  const int cmode = r.cmode();
  for (int pl = 0; pl < 2; pl++) {
    const uint32_t bit = 1u << (16 + pl);
    if (!(wm & bit)) break;
    const bool hasRes = (nzm & bit) != 0;
    intraBlock(S.ref[0], S.areaC[pl], 16, 1, 1, f.rec[1 + pl], cs, mbx * 8, mby * 8, 8, cmode, up, left, false,
               hasRes ? S.res + 256 + pl * 64 : nullptr, 8, lane, 32, true);
  }
}

// Tiles of up to this many macroblocks keep their progress in shared memory;
// larger ones use the slot's progress bytes in global memory.
constexpr int kIntraFlagMBs = 32768;
// Shared memory for ordering a tile's jobs (key counts, then the ordered list).
constexpr int kIntraSortBytes = 64 * 1024;

// Wavefront key of an intra macroblock at (x, y) of its tile: a 4x4-luma
// macroblock can start 4 diagonal steps after its left neighbour, 7 after
// the above-right one and 11 after the one above (10 steps, then the row
// above is complete), so 4x + 11y orders every job after the jobs it waits
// for and interleaves the rows the way the dependencies allow.
__device__ __forceinline__ int intraKey(int x, int y) { return 4 * x + 11 * y; }

// One CTA of W warps per tile, a dataflow schedule: the warps take the
// tile's intra macroblocks' luma and chroma as jobs in wavefront order
// (intraKey; raster order when the tile's ordering does not fit sortInts)
// and each job waits for exactly the neighbouring samples it predicts from
// (IntraSync).  Either order lists every job after the jobs it waits for, so
// the earliest unfinished job can always proceed.  The residuals were
// computed by kInterRecon phase 0.  Dynamic shared memory: W IntraScratch,
// 2 * flagMBs progress bytes (rounded to 16), sortInts words for the
// ordering.  Few tiles take 16 warps per CTA; many tiles fewer, so that
// several CTAs share an SM.
template <int W>
__global__ void __launch_bounds__(32 * W, 16 / W)
    kIntraRecon(const FrameDesc* frames, const int2* jobs, int njobs, int flagMBs, int sortInts) {
  allowNextGrid();
  extern __shared__ __align__(16) uint8_t sDyn[];
  __shared__ int sNext, sAbort, sWarpTot[W];
  IntraScratch* sS = reinterpret_cast<IntraScratch*>(sDyn);
  const int j = blockIdx.x;
  if (j >= njobs) return;
  // Up to the job loop this kernel reads only what the entropy stage wrote
  // (tile statistics, the intra list), so it runs ahead of the previous
  // kernel's completion; the gate and every pixel are read after the wait.
  const FrameDesc& f = frames[jobs[j].x];
  const int tile = jobs[j].y;
  const int n = f.tileStat[tile].intraCount;
  if (n == 0) {
    waitPreviousGrid();
    if (threadIdx.x == 0 && f.gate && *f.gate) atomicExch(f.status, kSkipped);
    return;
  }
  const TileRange tr = f.tiles[tile];
  const int tw = tr.mbX1 - tr.mbX0, th = tr.mbY1 - tr.mbY0, tmbs = tw * th;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, tid = threadIdx.x;
  uint8_t* flags;
  if (tmbs <= flagMBs) {
    flags = sDyn + sizeof(IntraScratch) * W;
  } else if (f.dep) {
    flags = f.dep + (size_t)f.mbCols * f.mbRows + 2 * (size_t)tr.mbBase;
  } else {
    if (tid == 0) atomicExch(f.status, kErrDevice);
    return;
  }
  IntraSync sy;
  sy.luma = flags;
  sy.chroma = flags + tmbs;
  sy.abort = &sAbort;
  sy.x0 = tr.mbX0;
  sy.y0 = tr.mbY0;
  sy.x1 = tr.mbX1;
  sy.tw = tw;
  const uint32_t* list = f.intraList + tr.mbBase;
  for (int i = tid; i < tmbs; i += blockDim.x) {
    sy.luma[i] = kLumaDone;
    sy.chroma[i] = 1;
  }
  if (tid == 0) {
    sNext = 0;
    sAbort = 0;
  }
  __syncthreads();
  const int mbCols = f.mbCols;
  for (int i = tid; i < n; i += blockDim.x) {
    const int idx = (int)(list[i] & kIndexMask);
    const int m = sy.at(idx % mbCols, idx / mbCols);
    sy.luma[m] = 0;
    sy.chroma[m] = 0;
  }
  __syncthreads();
  // Wavefront order: a counting sort of the list by intraKey in shared memory.
  const uint32_t* order = list;
  const int nkeys = intraKey(tw - 1, th - 1) + 1;
  if (nkeys + n <= sortInts) {
    int* cnt = reinterpret_cast<int*>(sDyn + sizeof(IntraScratch) * W + (((size_t)2 * flagMBs + 15) & ~(size_t)15));
    uint32_t* out = reinterpret_cast<uint32_t*>(cnt + nkeys);
    auto keyOf = [&](uint32_t e) {
      const int idx = (int)(e & kIndexMask);
      return intraKey(idx % mbCols - tr.mbX0, idx / mbCols - tr.mbY0);
    };
    for (int i = tid; i < nkeys; i += blockDim.x) cnt[i] = 0;
    __syncthreads();
    for (int i = tid; i < n; i += blockDim.x) atomicAdd(&cnt[keyOf(list[i])], 1);
    __syncthreads();
    {  // exclusive scan of cnt: per-thread chunks, then warps, then the CTA
      const int per = (nkeys + (int)blockDim.x - 1) / (int)blockDim.x;
      const int b = min(tid * per, nkeys), e = min(b + per, nkeys);
      int run = 0;
      for (int i = b; i < e; i++) run += cnt[i];
      int incl = run;
      for (int o = 1; o < 32; o <<= 1) {
        const int v = __shfl_up_sync(kFull, incl, o);
        if (lane >= o) incl += v;
      }
      if (lane == 31) sWarpTot[warp] = incl;
      __syncthreads();
      if (warp == 0) {
        const int t = lane < W ? sWarpTot[lane] : 0;
        int it = t;
        for (int o = 1; o < 32; o <<= 1) {
          const int v = __shfl_up_sync(kFull, it, o);
          if (lane >= o) it += v;
        }
        if (lane < W) sWarpTot[lane] = it - t;
      }
      __syncthreads();
      int acc = sWarpTot[warp] + incl - run;
      for (int i = b; i < e; i++) {
        const int c = cnt[i];
        cnt[i] = acc;
        acc += c;
      }
    }
    __syncthreads();
    for (int i = tid; i < n; i += blockDim.x) {
      const uint32_t e = list[i];
      out[atomicAdd(&cnt[keyOf(e)], 1)] = e;
    }
    __syncthreads();
    order = out;
  }
  waitPreviousGrid();
  if (f.gate && *f.gate) {
    if (threadIdx.x == 0) atomicExch(f.status, kSkipped);
    return;
  }
  ReconView view;
  view.load(f);
  IntraScratch& S = sS[warp];
  for (;;) {
    int k = 0;
    if (lane == 0) k = atomicAdd(&sNext, 1);
    k = __shfl_sync(kFull, k, 0);
    if (k >= 2 * n) break;
    const int idx = (int)(order[k >> 1] & kIndexMask);
    const int mbx = idx % mbCols, mby = idx / mbCols;
    if (k & 1) {
      intraChroma(view, S, sy, mbx, mby, lane);
      sy.publish(sy.chroma + sy.at(mbx, mby), 1, lane);
    } else {
      intraLuma(view, S, sy, mbx, mby, lane);
      sy.publish(sy.luma + sy.at(mbx, mby), kLumaDone, lane);
    }
    __syncwarp();
  }
  __syncthreads();
  if (tid == 0 && sAbort) atomicExch(f.status, kErrDevice);
}

}  // namespace dev

// ---------------------------------------------------------------------------
// Launch wrappers
// ---------------------------------------------------------------------------
int uploadCodingTables(const int* scan4, const int* scan8, const int* scan16, const int32_t* dct) {
  uint32_t s[3][257];
  std::memset(s, 0, sizeof(s));
  const int* scans[3] = {scan4, scan8, scan16};
  for (int k = 0; k < 3; k++)
    for (int i = 0; i < (16 << (2 * k)); i++) {
      const int band = bandOf(i);
      s[k][i] = (uint32_t)scans[k][i] | ((uint32_t)(band * kNumPrevClass * 64) << 8);
    }
  if (cudaMemcpyToSymbol(dev::cScanRow, s, sizeof(s)) != cudaSuccess) return kErrDevice;
  if (cudaMemcpyToSymbol(dev::gDct, dct, sizeof(int32_t) * 3 * 256) != cudaSuccess) return kErrDevice;
  return kOK;
}

// next: a zeroed device counter for the persistent grid (sized to the CTAs
// the device holds at once), or null for one CTA per job.
void launchEntropy(const FrameDesc* frames, const int4* jobs, int njobs, int* next, int maxTileMBs, cudaStream_t s) {
  if (njobs <= 0) return;
  static int resident[64] = {0};
  int dev = 0;
  cudaGetDevice(&dev);
  int grid = njobs;
  if (next && dev >= 0 && dev < 64) {
    if (!resident[dev]) {
      int perSM = 0, sms = 0;
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, dev::kEntropy, 32 * dev::kEntropyWarps, 0);
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
      resident[dev] = std::max(1, perSM * sms);
    }
    grid = std::min(njobs, resident[dev]);
  }
  dev::kEntropy<<<grid, 32 * dev::kEntropyWarps, 0, s>>>(frames, jobs, njobs, next);
  dev::kParseMB<<<dim3(njobs * kEntropyTilesPerJob, (maxTileMBs + dev::kParseWarps - 1) / dev::kParseWarps),
                  32 * dev::kParseWarps, 0, s>>>(frames, jobs, njobs);
  dev::kTileFinish<<<dim3(njobs, kEntropyTilesPerJob), dev::kParseThreads, 0, s>>>(frames, jobs, njobs);
}

// The reconstruction launches overlap their start with the previous kernel
// of the stream (programmatic dependent launch; the kernels wait for it).
template <class... A>
static void launchDependent(void (*k)(A...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, A... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, k, args...);
}

void launchInter(const FrameDesc* frames, int nframes, int maxMBs, int phase, cudaStream_t s) {
  if (nframes <= 0 || maxMBs <= 0) return;
  dim3 grid((maxMBs + dev::kInterWarps - 1) / dev::kInterWarps, nframes);
  launchDependent(dev::kInterRecon, grid, dim3(32 * dev::kInterWarps), 0, s, frames, phase);
}

template <int W>
static void allowIntraSmem() {
  cudaFuncSetAttribute(dev::kIntraRecon<W>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)(sizeof(dev::IntraScratch) * W + 2 * (size_t)dev::kIntraFlagMBs + dev::kIntraSortBytes));
}

template <int W>
static void launchIntraW(const FrameDesc* frames, const int2* jobs, int njobs, int flagMBs, int sortInts,
                         cudaStream_t s) {
  constexpr size_t kScratch = sizeof(dev::IntraScratch) * W;
  const size_t smem = kScratch + (((size_t)2 * flagMBs + 15) & ~(size_t)15) + 4 * (size_t)sortInts;
  launchDependent(dev::kIntraRecon<W>, dim3(njobs), dim3(32 * W), smem, s, frames, jobs, njobs, flagMBs, sortInts);
}

// maxTileMBs: the largest tile of the launch's frames, in macroblocks;
// maxTileKeys: the largest wavefront key range of its tiles (4*(w-1) +
// 11*(h-1) + 1 for a tile of w x h macroblocks).  warps: the warps per CTA
// (4, 8 or 16; anything else picks by the tile count: 16 up to one CTA per
// SM, 8 up to two, else 4).
void launchIntra(const FrameDesc* frames, const int2* jobs, int njobs, int maxTileMBs, int maxTileKeys, int warps,
                 cudaStream_t s) {
  if (njobs <= 0) return;
  static int sms[64] = {0};
  int d = 0;
  cudaGetDevice(&d);
  bool first = false;
  int nsm = 152;
  if (d >= 0 && d < 64) {
    if (!sms[d]) {
      cudaDeviceGetAttribute(&sms[d], cudaDevAttrMultiProcessorCount, d);
      sms[d] = std::max(1, sms[d]);
      first = true;
    }
    nsm = sms[d];
  }
  if (first) {  // the shared-memory limits of all three, once per device
    allowIntraSmem<16>();
    allowIntraSmem<8>();
    allowIntraSmem<4>();
  }
  const int flagMBs = std::max(1, std::min(maxTileMBs, dev::kIntraFlagMBs));
  int sortInts = std::max(0, maxTileMBs) + std::max(0, maxTileKeys);
  if (4 * (size_t)sortInts > (size_t)dev::kIntraSortBytes) sortInts = 0;  // raster order
  if (warps != 4 && warps != 8 && warps != 16) warps = njobs <= nsm ? 16 : (njobs <= 2 * nsm ? 8 : 4);
  if (warps == 16)
    launchIntraW<16>(frames, jobs, njobs, flagMBs, sortInts, s);
  else if (warps == 8)
    launchIntraW<8>(frames, jobs, njobs, flagMBs, sortInts, s);
  else
    launchIntraW<4>(frames, jobs, njobs, flagMBs, sortInts, s);
}

}  // namespace ebiv
