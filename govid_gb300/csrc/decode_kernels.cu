// GB300 (sm_103a) EBIV decode kernels.
//
// Stage A  kEntropy   one warp per tile: the tile's 4-state interleaved rANS
//                     chain (ebiv/rans.go:270-304) drives the macroblock
//                     grammar (ebiv/decode_intra.go:121-167,
//                     ebiv/decode_inter.go:8-62, ebiv/residual.go:79-126,
//                     ebiv/mv.go) and emits one MBRec per macroblock plus
//                     sparse levels.  The warp runs the chain in lockstep;
//                     the symbol lookup is a 17-lane ballot over the
//                     context's cumulative starts held in shared memory.
// Stage B1 kInterRecon one warp per macroblock of an inter frame: motion
//                     compensation (ebiv/motioncomp.go) from the last or
//                     golden reference plus dequantized inverse DCT residual
//                     (ebiv/quant.go:72-80, ebiv/transform.go:129-194).
// Stage B2 kIntraRecon one CTA per tile: intra macroblocks reconstructed along
//                     their true dependencies only, as a wavefront with a
//                     two-macroblock lag per row (ebiv/predict.go:50-219).
//
// Every wait is a __syncwarp/__syncthreads barrier inside one CTA; no kernel
// spins on memory written by another CTA.
#include <cuda_runtime.h>

#include "gpu_types.h"

namespace ebiv {
namespace dev {

constexpr unsigned kFull = 0xffffffffu;

__constant__ uint8_t cScan[3][256];   // zigzag: scan position -> row-major index
__constant__ int32_t cDct[3][256];    // 2^13-scaled DCT-II basis, [k*n + i]
__constant__ int32_t cTaps[4][4] = {{0, 64, 0, 0}, {-6, 55, 18, -3}, {-8, 40, 40, -8}, {-3, 18, 55, -6}};

__device__ __forceinline__ int bandOf(int i) { return i == 0 ? 0 : i <= 2 ? 1 : i <= 8 ? 2 : i <= 20 ? 3 : 4; }
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
// Per-warp symbol tables.  sym[c*16+s] packs the cumulative start (low 16
// bits) and frequency (high 16) of symbol s in context c.  lut[c*64+b] is the
// symbol whose range holds slot b*64 — the decoder starts there and walks
// forward at most a few entries; 0xFF marks an unused context.
struct WarpTables {
  uint32_t sym[kNumContexts * 16];
  uint8_t lut[kNumContexts * 64];
};
constexpr int kRowMax = 128;  // tiles at most this many macroblocks wide keep their rows in shared memory
struct WarpRows {
  uint32_t mv[2][kRowMax];   // packed motion vectors of the row above / the current row
  int16_t lvl[2][kRowMax];   // intra dependency levels (-1: not intra)
  uint32_t rec[12];          // the macroblock record being assembled
};

__device__ __forceinline__ void buildWarpTables(WarpTables& T, const DeviceTables& src, int lane) {
  for (int i = lane; i < kNumContexts * 16; i += 32) {
    const int c = i >> 4, sidx = i & 15;
    const uint32_t st = src.start[c][sidx], nx = src.start[c][sidx + 1];
    T.sym[i] = (st == 0xFFFFu || nx == 0xFFFFu) ? 0xFFFFu : (st | ((nx - st) << 16));
  }
  for (int i = lane; i < kNumContexts * 64; i += 32) T.lut[i] = 0xFF;
  __syncwarp();
  // Each (context, symbol) pair fills the buckets whose first slot it covers.
  for (int i = lane; i < kNumContexts * 16; i += 32) {
    const int c = i >> 4, sidx = i & 15;
    if (!src.used[c]) continue;
    const uint32_t st = src.start[c][sidx], nx = src.start[c][sidx + 1];
    if (st == 0xFFFFu || nx == 0xFFFFu || nx <= st) continue;
    for (uint32_t b = (st + 63) >> 6; b < 64 && (b << 6) < nx; b++) T.lut[c * 64 + b] = (uint8_t)sidx;
  }
  __syncwarp();
}

// A tile's rANS decoder (ebiv/rans.go:222-304).  All fields are warp-uniform;
// the two next stream bytes are prefetched so renormalisation rarely waits.
struct Chain {
  const uint8_t* buf;
  int32_t pos;
  uint32_t x0, x1, x2, x3;  // states in use order: x0 decodes the next symbol
  uint32_t b1, b2;          // buf[pos-1], buf[pos-2] when present
  int32_t err;
  const WarpTables* t;

  __device__ __forceinline__ uint32_t byteAt(int i) const { return i >= 0 ? (uint32_t)__ldg(buf + i) : 0u; }

  __device__ __forceinline__ int sym(int ctx) {
    if (err) return 0;
    const uint32_t slot = x0 & (kM - 1);
    int s = t->lut[ctx * 64 + (slot >> 6)];
    if (s == 0xFF) {
      err = kErrCorrupt;  // symbol decoded from an unused context
      return 0;
    }
    uint32_t w = t->sym[ctx * 16 + s];
    while (slot >= (w & 0xFFFFu) + (w >> 16)) w = t->sym[ctx * 16 + (++s)];
    uint32_t x = (w >> 16) * (x0 >> kScaleBits) + slot - (w & 0xFFFFu);
    while (x < kLower) {
      if (pos == 0) {
        err = kErrCorrupt;  // stream underrun
        return 0;
      }
      pos--;
      x = (x << 8) | b1;
      b1 = b2;
      b2 = byteAt(pos - 2);
    }
    x0 = x1;
    x1 = x2;
    x2 = x3;
    x3 = x;
    return s;
  }
  __device__ __forceinline__ uint32_t rawBits(int n) {
    uint32_t v = 0;
    for (int i = 0; i < n; i++) v = v << 1 | (uint32_t)sym(ctxBypass);
    return v;
  }
  // getClassValue — ebiv/mv.go:95-108
  __device__ __forceinline__ uint32_t classValue(int classCtx) {
    const int cls = sym(classCtx);
    if (cls <= 1) return (uint32_t)cls;
    return (1u << (cls - 1)) | rawBits(cls - 1);
  }
  __device__ __forceinline__ int mvComponent(int classCtx) {
    const uint32_t u = classValue(classCtx);
    return (int)(u >> 1) ^ -(int)(u & 1);
  }
};

// decodeBlock (ebiv/residual.go:79-126): writes the block's nonzero levels as
// packed entries after a count word; lane 0 stores.  Returns the count.
__device__ __forceinline__ int entropyBlock(Chain& d, int plane, int txIdx, int n, uint32_t* region, int lane) {
  const uint8_t* scan = cScan[n == 4 ? 0 : (n == 8 ? 1 : 2)];  // scan follows the block size
  const int total = n * n;
  const int ctxBase = plane == kPlaneLuma ? ctxTokenBase + txIdx * kNumBands * kNumPrevClass
                                          : ctxTokenBase + kLumaTokenCtx;
  int first = -1, last = -1, count = 0;
  int32_t sumAbs = 0;
  int prevClass = 0;
  uint32_t firstPos = 0;
  int32_t firstMag = 0;
  for (int i = 0; i < total; i++) {
    const int t = d.sym(ctxBase + bandOf(i) * kNumPrevClass + prevClass);
    if (t == tEOB) break;
    if (t == tZero) {
      prevClass = 0;
      continue;
    }
    int mag;
    if (t == tEscape) {
      mag = 5 + (int)d.classValue(ctxEscClass);
      prevClass = 2;
    } else {
      mag = t;
      prevClass = mag == 1 ? 1 : 2;
    }
    sumAbs = wadd(sumAbs, mag);
    const uint32_t pos = scan[i];
    if (first < 0) {
      first = i;
      firstPos = pos;
      firstMag = mag;
    } else {
      if (d.sym(ctxSign) == 1) mag = -mag;
      if (lane == 0) region[1 + count] = pos | ((uint32_t)mag << 8);
    }
    count++;
    last = i;
  }
  if (first >= 0) {
    const bool neg = (last - first >= kSDHMinSpan) ? (sumAbs & 1) == 1 : d.sym(ctxSign) == 1;
    if (lane == 0) region[1] = firstPos | ((uint32_t)(neg ? -firstMag : firstMag) << 8);
  }
  if (lane == 0) region[0] = (uint32_t)count;
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

// Tile context: bounds, neighbour rows, record staging.
struct TileCtx {
  Chain d;
  int lane;
  int x0, x1, y0, y1;  // tile bounds in macroblocks
  int mbCols;
  bool wide;           // rows live in global memory
  WarpRows* rows;
  uint32_t* gmv;       // wide-tile fallback: one packed vector per macroblock
  int16_t* glv;        // wide-tile fallback: one level per macroblock

  __device__ __forceinline__ uint32_t mvAt(int mbx, int mby) const {
    return wide ? gmv[mby * mbCols + mbx] : rows->mv[(mby - y0) & 1][mbx - x0];
  }
  __device__ __forceinline__ int lvAt(int mbx, int mby) const {
    return wide ? glv[mby * mbCols + mbx] : rows->lvl[(mby - y0) & 1][mbx - x0];
  }
  __device__ __forceinline__ void setMV(int mbx, int mby, uint32_t v, int lv) {
    if (lane == 0) {
      if (wide) {
        gmv[mby * mbCols + mbx] = v;
        glv[mby * mbCols + mbx] = (int16_t)lv;
      } else {
        rows->mv[(mby - y0) & 1][mbx - x0] = v;
        rows->lvl[(mby - y0) & 1][mbx - x0] = (int16_t)lv;
      }
    }
  }
  // predictMV — ebiv/mv.go:21-52 (neighbours within the tile)
  __device__ __forceinline__ uint32_t predictMV(int mbx, int mby) const {
    const bool aOK = mbx > x0, bOK = mby > y0;
    uint32_t a = 0, bv = 0, c = 0;
    bool cOK = false;
    if (aOK) a = mvAt(mbx - 1, mby);
    if (bOK) {
      bv = mvAt(mbx, mby - 1);
      if (mbx + 1 < x1) {
        c = mvAt(mbx + 1, mby - 1);
        cOK = true;
      } else if (aOK) {
        c = mvAt(mbx - 1, mby - 1);
        cOK = true;
      }
    }
    if (!aOK && !bOK && !cOK) return 0;
    if (aOK && !bOK && !cOK) return a;
    if (!aOK && bOK && !cOK) return bv;
    return packMV(median3((int16_t)mvX(a), (int16_t)mvX(bv), (int16_t)mvX(c)),
                  median3((int16_t)mvY(a), (int16_t)mvY(bv), (int16_t)mvY(c)));
  }
  // Intra dependency level of an intra macroblock at (mbx, mby).
  __device__ __forceinline__ int intraLevel(int mbx, int mby) const {
    int m = -1;
    if (mbx > x0) m = max(m, lvAt(mbx - 1, mby));
    if (mby > y0) {
      m = max(m, lvAt(mbx, mby - 1));
      if (mbx > x0) m = max(m, lvAt(mbx - 1, mby - 1));
      if (mbx + 1 < x1) m = max(m, lvAt(mbx + 1, mby - 1));
    }
    return m + 1;
  }
};

// Record words (see MBRec): 0 mode|ref<<8|part<<16|cbp<<24, 1 tx|cmode<<8,
// 2-5 mv[0..3], 6-9 luma modes, 10 nzmask, 11 wmask.  Lane 0 writes fields
// into the warp's staging copy; lanes 0-11 store it.
__device__ __forceinline__ void recSet(TileCtx& tc, int word, uint32_t v) {
  if (tc.lane == 0) tc.rows->rec[word] = v;
}
__device__ __forceinline__ void recOr(TileCtx& tc, int word, uint32_t v) {
  if (tc.lane == 0) tc.rows->rec[word] |= v;
}

// The coded blocks of one macroblock, decoded by a single inlined block
// decoder in bitstream order.  kind: 0 luma block preceded by its intra mode,
// 1 luma block, 2 chroma Cb (preceded by the chroma intra mode when intra),
// 3 chroma Cr.
struct BlockList {
  int count;
  int tx;
  bool intra;
  uint8_t kind[18];
};

// Decodes the listed blocks; returns how many completed before an error and
// the nonzero mask (bit k luma block k, 16 Cb, 17 Cr).
__device__ __forceinline__ int entropyBlocks(TileCtx& tc, const BlockList& bl, uint32_t* coef, uint32_t* nzOut) {
  Chain& d = tc.d;
  const int n = 4 << bl.tx;
  uint32_t nz = 0;
  int done = 0;
  int luma = 0;
  for (int e = 0; e < bl.count; e++) {
    const int kind = bl.kind[e];
    int plane = kPlaneLuma, bn = n, txi = bl.tx;
    uint32_t* region;
    uint32_t bit;
    if (kind <= 1) {
      if (kind == 0) recOr(tc, 6 + (luma >> 2), (uint32_t)d.sym(ctxLumaMode) << ((luma & 3) * 8));
      region = coef + luma * (n * n + 1);
      bit = 1u << luma;
      luma++;
    } else {
      if (kind == 2 && bl.intra) recOr(tc, 1, (uint32_t)d.sym(ctxChromaMode) << 8);
      plane = kPlaneChroma;
      bn = 8;
      txi = 0;
      region = coef + (kind == 2 ? kCoefCb : kCoefCr);
      bit = kind == 2 ? (1u << 16) : (1u << 17);
    }
    const int cnt = entropyBlock(d, plane, txi, bn, region, tc.lane);
    if (d.err) break;
    if (cnt) nz |= bit;
    done++;
  }
  *nzOut = nz;
  return done;
}

// Intra macroblock symbols (decodeLumaMB + decodeChromaMB,
// ebiv/decode_intra.go:137-187).  Returns the write mask.
__device__ __forceinline__ uint32_t entropyIntraMB(TileCtx& tc, uint32_t* coef) {
  Chain& d = tc.d;
  int tx = d.sym(ctxTxSize);
  if (tx >= 3) tx = 0;  // alphabet size 3: unreachable
  const int nb = 16 >> (2 * tx);
  BlockList bl;
  bl.tx = tx;
  bl.intra = true;
  bl.count = nb + 2;
  for (int k = 0; k < nb; k++) bl.kind[k] = 0;
  bl.kind[nb] = 2;
  bl.kind[nb + 1] = 3;
  recSet(tc, 0, kRecIntra);
  recSet(tc, 1, (uint32_t)tx);
  uint32_t nz;
  const int done = d.err ? 0 : entropyBlocks(tc, bl, coef, &nz);
  if (d.err && done == 0) nz = 0;
  recSet(tc, 10, nz);
  uint32_t w = (1u << min(done, nb)) - 1;
  if (done > nb) w |= 1u << 16;
  if (done > nb + 1) w |= 1u << 17;
  return w;
}

// Inter-frame macroblock symbols (decodeInterMB + reconInterMB grammar,
// ebiv/decode_inter.go:8-118).  Returns the write mask.
__device__ __forceinline__ uint32_t entropyInterMB(TileCtx& tc, int mbx, int mby, uint32_t* coef, bool* intra) {
  Chain& d = tc.d;
  const int mode = d.sym(ctxMBMode);
  if (mode == mbSkip) {
    const uint32_t p = tc.predictMV(mbx, mby);
    tc.setMV(mbx, mby, p, -1);
    recSet(tc, 0, kRecSkip);
    recSet(tc, 2, p);
    return kWriteAll;
  }
  if (mode == mbIntra) {
    *intra = true;
    return entropyIntraMB(tc, coef);  // the caller records the zero vector and level
  }
  if (mode != mbInter) {
    d.err = kErrCorrupt;
    return 0;
  }
  const int refSel = d.sym(ctxRef);
  uint32_t pred = tc.predictMV(mbx, mby);
  if (refSel == refGolden) pred = 0;
  int part = d.sym(ctxPart);
  if (part >= kNumPartModes) part = 0;  // alphabet size 4: unreachable
  const int np = part == partWhole ? 1 : (part == part8x8 ? 4 : 2);
  uint32_t mv0 = 0;
  for (int i = 0; i < np; i++) {
    const uint32_t pp = i > 0 ? mv0 : pred;
    const int dx = d.mvComponent(ctxMVClassX);
    const int vx = clampMV(mvX(pp) + dx);
    const int dy = d.mvComponent(ctxMVClassY);
    const int vy = clampMV(mvY(pp) + dy);
    const uint32_t v = packMV(vx, vy);
    if (i == 0) mv0 = v;
    recSet(tc, 2 + i, v);
  }
  if (d.err) return 0;
  tc.setMV(mbx, mby, refSel == refGolden ? 0u : mv0, -1);
  const int cbp = d.sym(ctxCBP);
  recSet(tc, 0, kRecInter | ((uint32_t)refSel << 8) | ((uint32_t)part << 16) | ((uint32_t)cbp << 24));
  if (d.err) return 0;
  BlockList bl;
  bl.intra = false;
  bl.tx = 0;
  bl.count = 0;
  int nb = 0;
  if (cbp & cbpLuma) {
    int tx = d.sym(ctxTxSize);
    if (tx >= 3) tx = 0;
    if (d.err) return 0;
    recSet(tc, 1, (uint32_t)tx);
    bl.tx = tx;
    nb = 16 >> (2 * tx);
    for (int k = 0; k < nb; k++) bl.kind[bl.count++] = 1;
  }
  const int cbEntry = (cbp & cbpCb) ? bl.count : -1;
  if (cbp & cbpCb) bl.kind[bl.count++] = 2;
  const int crEntry = (cbp & cbpCr) ? bl.count : -1;
  if (cbp & cbpCr) bl.kind[bl.count++] = 3;
  uint32_t nz = 0;
  const int done = entropyBlocks(tc, bl, coef, &nz);
  recSet(tc, 10, nz);
  if (done < nb) return (1u << done) - 1;  // a coded luma block failed: nothing else is written
  uint32_t w = 0xFFFFu;                    // coded luma complete, or motion-compensated luma
  if (cbEntry < 0 || done > cbEntry) w |= 1u << 16;
  if (crEntry < 0 || done > crEntry) w |= 1u << 17;
  return w;
}

constexpr int kEntropyWarps = 4;

__global__ void __launch_bounds__(32 * kEntropyWarps) kEntropy(const FrameDesc* frames, const int2* jobs, int njobs) {
  __shared__ WarpTables sT[kEntropyWarps];
  __shared__ WarpRows sR[kEntropyWarps];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int j = blockIdx.x * kEntropyWarps + warp;
  if (j >= njobs) return;
  const FrameDesc* fp = frames + jobs[j].x;
  const int tile = jobs[j].y;
  // Descriptor fields into registers: the kernel's global stores cannot alias them then.
  const int mbCols = fp->mbCols;
  const int inter = fp->inter;
  MBRec* const recs = fp->mbrec;
  uint32_t* const coefBase = fp->coef;
  uint32_t* const intraList = fp->intraList;
  TileStat* const tstat = fp->tileStat;
  int32_t* const status = fp->status;
  const TileRange tr = fp->tiles[tile];
  buildWarpTables(sT[warp], *fp->tables, lane);

  TileCtx tc;
  tc.lane = lane;
  tc.x0 = tr.mbX0;
  tc.x1 = tr.mbX1;
  tc.y0 = tr.mbY0;
  tc.y1 = tr.mbY1;
  tc.mbCols = mbCols;
  tc.rows = &sR[warp];
  tc.wide = (tc.x1 - tc.x0) > kRowMax;
  tc.gmv = reinterpret_cast<uint32_t*>(fp->mvgrid);
  tc.glv = fp->lvgrid;
  Chain& d = tc.d;
  d.buf = fp->pkt + tr.offset;
  d.pos = (int32_t)tr.length;
  d.err = 0;
  d.t = &sT[warp];
  const int tw = tc.x1 - tc.x0;
  const int total = tw * (tc.y1 - tc.y0);
  int done = 0, intraCount = 0, maxLevel = -1;
  if (tr.length < (uint32_t)(kStates * 4)) {
    d.err = kErrCorrupt;  // tile stream too short to initialise rANS
  } else {
    uint32_t st[4];
#pragma unroll
    for (int i = kStates - 1; i >= 0; i--) {
      st[i] = d.byteAt(d.pos - 1) << 24 | d.byteAt(d.pos - 2) << 16 | d.byteAt(d.pos - 3) << 8 | d.byteAt(d.pos - 4);
      d.pos -= 4;
    }
    d.x0 = st[0];
    d.x1 = st[1];
    d.x2 = st[2];
    d.x3 = st[3];
    d.b1 = d.byteAt(d.pos - 1);
    d.b2 = d.byteAt(d.pos - 2);
    int mbx = tc.x0, mby = tc.y0;
    for (; done < total; done++) {
      const int idx = mby * mbCols + mbx;
      if (lane < 12) tc.rows->rec[lane] = 0;
      __syncwarp();
      uint32_t* coef = coefBase + (size_t)idx * kCoefPerMB;
      bool intra = !inter;
      uint32_t w;
      if (inter) {
        w = entropyInterMB(tc, mbx, mby, coef, &intra);
      } else {
        w = entropyIntraMB(tc, coef);
      }
      if (intra) {
        const int lv = tc.intraLevel(mbx, mby);
        tc.setMV(mbx, mby, 0u, w ? lv : -1);
        if (w) {
          if (lane == 0) intraList[tr.mbBase + intraCount] = (uint32_t)idx | ((uint32_t)lv << kLevelShift);
          intraCount++;
          maxLevel = max(maxLevel, lv);
        }
      }
      recSet(tc, 11, w);
      __syncwarp();
      if (lane < 12) reinterpret_cast<uint32_t*>(recs + idx)[lane] = tc.rows->rec[lane];
      if (d.err) {
        done++;
        break;
      }
      if (++mbx == tc.x1) {
        mbx = tc.x0;
        mby++;
      }
    }
  }
  // Macroblocks the tile never reached are left untouched by reconstruction.
  for (int k = done + lane; k < total; k += 32) {
    MBRec* r = recs + (size_t)(tc.y0 + k / tw) * mbCols + tc.x0 + k % tw;
    r->mode = kRecNone;
    r->wmask = 0;
  }
  if (lane == 0) {
    TileStat ts;
    ts.err = d.err;
    ts.intraCount = intraCount;
    ts.maxLevel = maxLevel;
    ts.pad = 0;
    tstat[tile] = ts;
    if (d.err) atomicExch(status, kErrCorrupt);
  }
}

// ---------------------------------------------------------------------------
// Dequantization + inverse DCT of one block (warp-cooperative)
// ---------------------------------------------------------------------------
// Writes the n x n residual into out[r*outStride + c].  dense and tmp are
// per-warp shared scratch of n*n words.
__device__ void idctBlock(const uint32_t* region, int n, int32_t qdc, int32_t qac, int32_t* dense, int32_t* tmp,
                          int32_t* out, int outStride, int lane) {
  const int nn = n * n;
  const int tx = n == 4 ? 0 : (n == 8 ? 1 : 2);
  for (int i = lane; i < nn; i += 32) dense[i] = 0;
  __syncwarp();
  const int count = (int)region[0];
  for (int e = lane; e < count; e += 32) {
    const uint32_t v = region[1 + e];
    const int pos = (int)(v & 0xFF);
    const int32_t lvl = (int32_t)v >> 8;
    dense[pos] = wmul(lvl, pos == 0 ? qdc : qac);
  }
  __syncwarp();
  const int32_t* c = cDct[tx];
  for (int o = lane; o < nn; o += 32) {
    const int i = o / n, l = o - i * n;
    int64_t acc = 0;
    for (int k = 0; k < n; k++) acc += (int64_t)c[k * n + i] * (int64_t)dense[k * n + l];
    tmp[o] = (int32_t)((acc + 4096) >> 13);
  }
  __syncwarp();
  for (int o = lane; o < nn; o += 32) {
    const int i = o / n, m = o - i * n;
    int64_t acc = 0;
    for (int l = 0; l < n; l++) acc += (int64_t)c[l * n + m] * (int64_t)tmp[i * n + l];
    out[i * outStride + m] = (int32_t)((acc + 4096) >> 13);
  }
  __syncwarp();
}

// ---------------------------------------------------------------------------
// Motion compensation samples (clamped form of ebiv/motioncomp.go:49-97)
// ---------------------------------------------------------------------------
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
// Stage B1: inter macroblock reconstruction
// ---------------------------------------------------------------------------
constexpr int kInterWarps = 4;

struct InterScratch {
  int32_t res[256];
  int32_t dense[256];
  int32_t tmp[256];
};

__global__ void __launch_bounds__(32 * kInterWarps) kInterRecon(const FrameDesc* frames) {
  __shared__ InterScratch sS[kInterWarps];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const FrameDesc& f = frames[blockIdx.y];
  if (f.gate && *f.gate) {
    if (threadIdx.x == 0) atomicExch(f.status, kSkipped);
    return;
  }
  if (!f.inter) return;
  const int idx = blockIdx.x * kInterWarps + warp;
  if (idx >= f.mbCols * f.mbRows) return;
  const MBRec& r = f.mbrec[idx];
  const int mode = r.mode;
  if (mode != kRecSkip && mode != kRecInter) return;
  const uint32_t wm = r.wmask;
  if (!wm) return;
  InterScratch& S = sS[warp];
  const int mbx = idx % f.mbCols, mby = idx / f.mbCols;
  const bool golden = mode == kRecInter && r.ref == refGolden;
  const uint8_t* const* refp = golden ? f.gold : f.ref;
  const int part = mode == kRecInter ? r.part : partWhole;
  const int cbp = mode == kRecInter ? r.cbp : 0;

  // Luma: lane -> row lane/2, 8 columns.
  {
    const int row = lane >> 1, c0 = (lane & 1) * 8;
    const int pi = partIndex(part, c0, row);
    const int mvx = r.mv[pi][0], mvy = r.mv[pi][1];
    const int fx = mvx & 3, fy = mvy & 3;
    const int sx = mbx * 16 + c0 + (mvx >> 2), sy = mby * 16 + row + (mvy >> 2);
    int pred[8];
#pragma unroll
    for (int k = 0; k < 8; k++) pred[k] = lumaSample(refp[0], f.strideY, f.padW, f.padH, sx + k, sy, fx, fy);
    const bool coded = (cbp & cbpLuma) != 0;
    const int tx = r.tx, n = 4 << tx, per = 4 >> tx;
    if (coded) {
      const int nb = per * per;
      for (int k = 0; k < nb; k++) {
        if (!((wm >> k) & 1)) continue;
        const int bx = (k % per) * n, by = (k / per) * n;
        if ((r.nzmask >> k) & 1) {
          idctBlock(f.coef + (size_t)idx * kCoefPerMB + k * (n * n + 1), n, f.qdc, f.qac, S.dense, S.tmp,
                    S.res + by * 16 + bx, 16, lane);
        } else {
          for (int i = lane; i < n * n; i += 32) S.res[(by + i / n) * 16 + bx + i % n] = 0;
          __syncwarp();
        }
      }
    }
    uint8_t* out = f.rec[0] + (size_t)(mby * 16 + row) * f.strideY + mbx * 16 + c0;
#pragma unroll
    for (int k = 0; k < 8; k++) {
      const int c = c0 + k;
      const int blk = (row / n) * per + c / n;
      if (!((wm >> blk) & 1)) continue;
      const int v = coded ? clampByteD(wadd(pred[k], S.res[row * 16 + c])) : pred[k];
      out[k] = (uint8_t)v;
    }
  }
  __syncwarp();
  // Chroma: lane -> row lane/4, 2 columns; Cb then Cr.
#pragma unroll
  for (int pl = 0; pl < 2; pl++) {
    const uint32_t bit = 1u << (16 + pl);
    if (!(wm & bit)) continue;
    const int row = lane >> 2, c0 = (lane & 3) * 2;
    const int pi = partIndex(part, c0 * 2, row * 2);
    const int mvx = r.mv[pi][0], mvy = r.mv[pi][1];
    const int fx = mvx & 7, fy = mvy & 7;
    const int sx = mbx * 8 + c0 + (mvx >> 3), sy = mby * 8 + row + (mvy >> 3);
    int p0 = chromaSample(refp[1 + pl], f.strideC, f.padCW, f.padCH, sx, sy, fx, fy);
    int p1 = chromaSample(refp[1 + pl], f.strideC, f.padCW, f.padCH, sx + 1, sy, fx, fy);
    const bool coded = (cbp & (cbpCb << pl)) != 0;
    if (coded) {
      if (r.nzmask & bit) {
        idctBlock(f.coef + (size_t)idx * kCoefPerMB + (pl ? kCoefCr : kCoefCb), 8, f.qdc, f.qac, S.dense, S.tmp,
                  S.res, 8, lane);
        p0 = clampByteD(wadd(p0, S.res[row * 8 + c0]));
        p1 = clampByteD(wadd(p1, S.res[row * 8 + c0 + 1]));
        __syncwarp();
      }
    }
    uint8_t* out = f.rec[1 + pl] + (size_t)(mby * 8 + row) * f.strideC + mbx * 8 + c0;
    out[0] = (uint8_t)p0;
    out[1] = (uint8_t)p1;
  }
}

// ---------------------------------------------------------------------------
// Stage B2: intra reconstruction wavefront
// ---------------------------------------------------------------------------
constexpr int kIntraWarps = 8;

struct IntraScratch {
  int32_t ref[4 * 16 + 1];
  int32_t res[256];
  int32_t dense[256];
  int32_t tmp[256];
};

// The reference sample array of predictIntra after substituteRefs, in
// closed form: ref[0..2n-1] left column bottom-to-top, ref[2n] corner,
// ref[2n+1..4n] top then top-right.
__device__ __forceinline__ int32_t refValue(int i, int n, bool avAbove, bool avLeft, bool avAR, const uint8_t* p,
                                            int stride, int x0, int y0) {
  const int corner = 2 * n;
  auto L = [&](int r) -> int32_t { return p[(size_t)(y0 + r) * stride + x0 - 1]; };
  auto Tp = [&](int j) -> int32_t { return p[(size_t)(y0 - 1) * stride + x0 + j]; };
  if (!avLeft && !avAbove) return kDCPred;
  if (i < corner) {
    const int row = 2 * n - 1 - i;
    return avLeft ? L(row < n ? row : n - 1) : Tp(0);
  }
  if (i == corner) {
    if (avLeft && avAbove) return p[(size_t)(y0 - 1) * stride + x0 - 1];
    return avLeft ? L(0) : Tp(0);
  }
  const int j = i - corner - 1;
  if (avAbove) return (j < n || avAR) ? Tp(j) : Tp(n - 1);
  return L(0);
}

// Predicts and reconstructs one n x n block at (x0,y0) of plane p.
__device__ void intraBlock(IntraScratch& S, uint8_t* p, int stride, int x0, int y0, int n, int mode, bool avAbove,
                           bool avLeft, bool avAR, bool hasRes, int lane) {
  const int corner = 2 * n;
  for (int i = lane; i <= 4 * n; i += 32) S.ref[i] = refValue(i, n, avAbove, avLeft, avAR, p, stride, x0, y0);
  __syncwarp();
  int32_t dc = 0;
  if (mode == modeDC) {
    int32_t sum = 0;
    for (int i = 0; i < n; i++) sum += S.ref[corner + 1 + i] + S.ref[corner - 1 - i];
    dc = (sum + n) / (2 * n);
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
  int32_t vals[8];
  int cnt = 0;
  for (int o = lane; o < nn; o += 32, cnt++) {
    const int r = o / n, c = o - r * n;
    int32_t v;
    switch (mode) {
      case modeV: v = S.ref[corner + 1 + c]; break;
      case modeH: v = S.ref[corner - 1 - r]; break;
      case modeTM: v = clampByteD(S.ref[corner + 1 + c] + S.ref[corner - 1 - r] - S.ref[corner]); break;
      case modeDC: v = dc; break;
      default: {
        const int a = vertical ? r : c, b = vertical ? c : r;
        const int pos = (a + 1) * angle;
        const int idx = pos >> 5, fact = pos & 31;
        auto ext = [&](int k) -> int32_t {
          if (k >= 0) {
            if (k > 2 * n) return 0;
            return vertical ? S.ref[corner + k] : S.ref[corner - k];
          }
          const int t = (k * inv + 128) >> 8;
          return vertical ? S.ref[corner - t] : S.ref[corner + t];
        };
        v = ((32 - fact) * ext(b + idx + 1) + fact * ext(b + idx + 2) + 16) >> 5;
      }
    }
    if (hasRes) v = clampByteD(wadd(v, S.res[r * n + c]));
    else v = clampByteD(v);
    vals[cnt] = v;
  }
  __syncwarp();  // every lane has read its neighbours before anyone writes
  cnt = 0;
  for (int o = lane; o < nn; o += 32, cnt++) {
    const int r = o / n, c = o - r * n;
    p[(size_t)(y0 + r) * stride + x0 + c] = (uint8_t)vals[cnt];
  }
  __syncwarp();
}

__device__ void intraMB(const FrameDesc& f, IntraScratch& S, int mbx, int mby, int tx0, int tx1, int ty0, int lane) {
  const int idx = mby * f.mbCols + mbx;
  const MBRec& r = f.mbrec[idx];
  if (r.mode != kRecIntra) return;
  const uint32_t wm = r.wmask;
  if (!wm) return;
  const int tx = r.tx, n = 4 << tx, per = 4 >> tx, nb = per * per;
  const int tileLeft = tx0 * 16, tileTop = ty0 * 16, tileRight = tx1 * 16;
  const int mbTop = mby * 16, mbRight = (mbx + 1) * 16;
  const uint32_t* coef = f.coef + (size_t)idx * kCoefPerMB;
  for (int k = 0; k < nb; k++) {
    if (!((wm >> k) & 1)) break;
    const int x0 = mbx * 16 + (k % per) * n, y0 = mby * 16 + (k / per) * n;
    const bool avAbove = y0 > tileTop, avLeft = x0 > tileLeft;
    bool avAR = false;
    if (!(y0 <= tileTop || x0 + 2 * n > tileRight)) avAR = (y0 == mbTop) ? true : (x0 + 2 * n <= mbRight);
    const bool hasRes = (r.nzmask >> k) & 1;
    if (hasRes) idctBlock(coef + k * (n * n + 1), n, f.qdc, f.qac, S.dense, S.tmp, S.res, n, lane);
    intraBlock(S, f.rec[0], f.strideY, x0, y0, n, r.lmode[k], avAbove, avLeft, avAR, hasRes, lane);
  }
  const int cx0 = mbx * 8, cy0 = mby * 8;
  const bool cAbove = cy0 > ty0 * 8, cLeft = cx0 > tx0 * 8;
  for (int pl = 0; pl < 2; pl++) {
    const uint32_t bit = 1u << (16 + pl);
    if (!(wm & bit)) break;
    const bool hasRes = (r.nzmask & bit) != 0;
    if (hasRes) idctBlock(coef + (pl ? kCoefCr : kCoefCb), 8, f.qdc, f.qac, S.dense, S.tmp, S.res, 8, lane);
    intraBlock(S, f.rec[1 + pl], f.strideC, cx0, cy0, 8, r.cmode, cAbove, cLeft, false, hasRes, lane);
  }
}

constexpr int kLevelBuckets = 2048;

// One CTA per tile.  The tile's intra macroblocks (listed by the entropy
// stage with their dependency levels) are counting-sorted by level, then each
// level is reconstructed in parallel with a CTA barrier between levels.  Key
// frames get the classic wavefront (level = x + 2y); inter frames with a few
// isolated intra macroblocks take one or two levels.
__global__ void __launch_bounds__(32 * kIntraWarps) kIntraRecon(const FrameDesc* frames, const int2* jobs, int njobs) {
  __shared__ IntraScratch sS[kIntraWarps];
  __shared__ int sStart[kLevelBuckets + 1];
  __shared__ int sCur[kLevelBuckets];
  const int j = blockIdx.x;
  if (j >= njobs) return;
  const FrameDesc& f = frames[jobs[j].x];
  if (f.gate && *f.gate) {
    if (threadIdx.x == 0) atomicExch(f.status, kSkipped);
    return;
  }
  const int tile = jobs[j].y;
  const TileStat ts = f.tileStat[tile];
  const int n = ts.intraCount;
  if (n == 0) return;
  const TileRange tr = f.tiles[tile];
  const int L = ts.maxLevel + 1;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, tid = threadIdx.x;
  const uint32_t* list = f.intraList + tr.mbBase;
  uint32_t* sorted = f.intraSorted + tr.mbBase;
  auto runMB = [&](uint32_t e) {
    const int idx = (int)(e & kIndexMask);
    intraMB(f, sS[warp], idx % f.mbCols, idx / f.mbCols, tr.mbX0, tr.mbX1, tr.mbY0, lane);
  };
  if (L <= kLevelBuckets) {
    for (int l = tid; l <= L; l += blockDim.x) sStart[l] = 0;
    __syncthreads();
    for (int i = tid; i < n; i += blockDim.x) atomicAdd(&sStart[(list[i] >> kLevelShift) + 1], 1);
    __syncthreads();
    if (warp == 0) {  // inclusive scan of counts -> exclusive level starts
      const int per = (L + 1 + 31) / 32;
      const int b = lane * per, e = min(b + per, L + 1);
      int run = 0;
      for (int l = b; l < e; l++) run += sStart[l];
      int incl = run;
      for (int o = 1; o < 32; o <<= 1) {
        const int v = __shfl_up_sync(kFull, incl, o);
        if (lane >= o) incl += v;
      }
      int acc = incl - run;
      for (int l = b; l < e; l++) {
        acc += sStart[l];
        sStart[l] = acc;
      }
    }
    __syncthreads();
    for (int l = tid; l < L; l += blockDim.x) sCur[l] = sStart[l];
    __syncthreads();
    for (int i = tid; i < n; i += blockDim.x) {
      const uint32_t e = list[i];
      sorted[atomicAdd(&sCur[e >> kLevelShift], 1)] = e;
    }
    __syncthreads();
    for (int l = 0; l < L; l++) {
      for (int k = sStart[l] + warp; k < sStart[l + 1]; k += kIntraWarps) runMB(sorted[k]);
      __syncthreads();
    }
  } else {
    // Very wide or tall tiles: scan the list once per level.
    for (int l = 0; l < L; l++) {
      for (int i = warp; i < n; i += kIntraWarps)
        if ((int)(list[i] >> kLevelShift) == l) runMB(list[i]);
      __syncthreads();
    }
  }
}

}  // namespace dev

// ---------------------------------------------------------------------------
// Launch wrappers
// ---------------------------------------------------------------------------
int uploadCodingTables(const int* scan4, const int* scan8, const int* scan16, const int32_t* dct) {
  uint8_t s[3][256];
  for (int i = 0; i < 16; i++) s[0][i] = (uint8_t)scan4[i];
  for (int i = 0; i < 64; i++) s[1][i] = (uint8_t)scan8[i];
  for (int i = 0; i < 256; i++) s[2][i] = (uint8_t)scan16[i];
  if (cudaMemcpyToSymbol(dev::cScan, s, sizeof(s)) != cudaSuccess) return kErrDevice;
  if (cudaMemcpyToSymbol(dev::cDct, dct, sizeof(int32_t) * 3 * 256) != cudaSuccess) return kErrDevice;
  return kOK;
}

void launchEntropy(const FrameDesc* frames, const int2* jobs, int njobs, cudaStream_t s) {
  if (njobs <= 0) return;
  const int blocks = (njobs + dev::kEntropyWarps - 1) / dev::kEntropyWarps;
  dev::kEntropy<<<blocks, 32 * dev::kEntropyWarps, 0, s>>>(frames, jobs, njobs);
}

void launchInter(const FrameDesc* frames, int nframes, int maxMBs, cudaStream_t s) {
  if (nframes <= 0 || maxMBs <= 0) return;
  dim3 grid((maxMBs + dev::kInterWarps - 1) / dev::kInterWarps, nframes);
  dev::kInterRecon<<<grid, 32 * dev::kInterWarps, 0, s>>>(frames);
}

void launchIntra(const FrameDesc* frames, const int2* jobs, int njobs, cudaStream_t s) {
  if (njobs <= 0) return;
  dev::kIntraRecon<<<njobs, 32 * dev::kIntraWarps, 0, s>>>(frames, jobs, njobs);
}

}  // namespace ebiv
