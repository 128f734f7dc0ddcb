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
struct WarpTables {
  uint16_t start[kNumContexts * 17];
  uint8_t used[kNumContexts];
};

// A tile's rANS decoder.  Every field is warp-uniform: all 32 lanes hold the
// same values and take the same branches.
struct Chain {
  const uint8_t* buf;
  int32_t pos;
  uint32_t x0, x1, x2, x3;  // states in use order: x0 decodes the next symbol
  int32_t err;
  const WarpTables* t;
  int lane;

  __device__ __forceinline__ int sym(int ctx) {
    if (err) return 0;
    if (!t->used[ctx]) {
      err = kErrCorrupt;
      return 0;
    }
    uint32_t x = x0;
    const uint32_t slot = x & (kM - 1);
    const uint32_t st = lane < 17 ? (uint32_t)t->start[ctx * 17 + lane] : 0xFFFFu;
    const unsigned bal = __ballot_sync(kFull, st <= slot);
    const int s = __popc(bal) - 1;
    const uint32_t s0 = __shfl_sync(kFull, st, s);
    const uint32_t s1 = __shfl_sync(kFull, st, s + 1);
    x = (s1 - s0) * (x >> kScaleBits) + slot - s0;
    while (x < kLower) {
      if (pos == 0) {
        err = kErrCorrupt;
        return 0;
      }
      pos--;
      x = (x << 8) | (uint32_t)__ldg(buf + pos);
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
  __device__ __forceinline__ uint32_t classValue(int classCtx, int maxClass) {
    const int cls = sym(classCtx);
    if (cls < 0 || cls >= maxClass) {
      if (!err) err = kErrCorrupt;
      return 0;
    }
    if (cls == 0) return 0;
    if (cls == 1) return 1;
    return (1u << (cls - 1)) | rawBits(cls - 1);
  }
  __device__ __forceinline__ int mvComponent(int classCtx) {
    const uint32_t u = classValue(classCtx, kNumMVClasses);
    return (int)(u >> 1) ^ -(int)(u & 1);
  }
};

// decodeBlock (ebiv/residual.go:79-126): writes the block's nonzero levels as
// packed entries after a count word.  Returns the nonzero count.
__device__ int entropyBlock(Chain& d, int plane, int txIdx, int n, uint32_t* region) {
  // The scan follows the block size; txIdx only selects luma contexts.
  const uint8_t* scan = cScan[n == 4 ? 0 : (n == 8 ? 1 : 2)];
  const int total = n * n;
  int first = -1, last = -1, count = 0;
  int32_t sumAbs = 0;
  int prevClass = 0;
  uint32_t firstPos = 0;
  int32_t firstMag = 0;
  for (int i = 0; i < total; i++) {
    const int t = d.sym(tokenCtx(plane, txIdx, bandOf(i), prevClass));
    if (t == tEOB) break;
    if (t == tZero) {
      prevClass = 0;
      continue;
    }
    int mag;
    if (t == tEscape) {
      mag = 5 + (int)d.classValue(ctxEscClass, kNumEscClasses);
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
      count++;  // slot 1 is reserved for the first coefficient
    } else {
      if (d.sym(ctxSign) == 1) mag = -mag;
      if (d.lane == 0) region[1 + count] = pos | ((uint32_t)mag << 8);
      count++;
    }
    last = i;
  }
  if (first >= 0) {
    bool neg;
    if (last - first >= kSDHMinSpan)
      neg = (sumAbs & 1) == 1;
    else
      neg = d.sym(ctxSign) == 1;
    const int32_t m = neg ? -firstMag : firstMag;
    if (d.lane == 0) region[1] = firstPos | ((uint32_t)m << 8);
  }
  if (d.lane == 0) region[0] = (uint32_t)count;
  return count;
}

struct TileCtx {
  Chain d;
  const FrameDesc* f;
  int bx0, bx1, by0, by1;  // tile bounds in macroblocks
};

__device__ __forceinline__ short2 loadMV(const FrameDesc& f, int idx) {
  return reinterpret_cast<const short2*>(f.mvgrid)[idx];
}
__device__ __forceinline__ void storeMV(const FrameDesc& f, int idx, short2 v, int lane) {
  if (lane == 0) reinterpret_cast<short2*>(f.mvgrid)[idx] = v;
  __syncwarp();
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
// predictMV — ebiv/mv.go:21-52
__device__ short2 predictMV(const TileCtx& tc, int mbx, int mby) {
  const FrameDesc& f = *tc.f;
  const int stride = f.mbCols;
  short2 a = make_short2(0, 0), bv = make_short2(0, 0), c = make_short2(0, 0);
  const bool aOK = mbx > tc.bx0, bOK = mby > tc.by0;
  bool cOK = false;
  if (aOK) a = loadMV(f, mby * stride + mbx - 1);
  if (bOK) {
    bv = loadMV(f, (mby - 1) * stride + mbx);
    if (mbx + 1 < tc.bx1) {
      c = loadMV(f, (mby - 1) * stride + mbx + 1);
      cOK = true;
    } else if (aOK) {
      c = loadMV(f, (mby - 1) * stride + mbx - 1);
      cOK = true;
    }
  }
  if (!aOK && !bOK && !cOK) return make_short2(0, 0);
  if (aOK && !bOK && !cOK) return a;
  if (!aOK && bOK && !cOK) return bv;
  return make_short2(median3(a.x, bv.x, c.x), median3(a.y, bv.y, c.y));
}

// Intra macroblock symbols (decodeLumaMB + decodeChromaMB).
__device__ void entropyIntraMB(TileCtx& tc, MBRec& r, uint32_t* coef) {
  Chain& d = tc.d;
  int tx = d.sym(ctxTxSize);
  if (tx < 0 || tx >= 3) {
    if (!d.err) d.err = kErrCorrupt;
    tx = 0;
  }
  const int n = 4 << tx;
  const int nb = 16 >> (2 * tx);
  r.mode = kRecIntra;
  r.tx = (uint8_t)tx;
  int done = 0;
  for (int k = 0; k < nb && !d.err; k++) {
    const int mode = d.sym(ctxLumaMode);
    r.lmode[k] = (uint8_t)mode;
    const int cnt = entropyBlock(d, kPlaneLuma, tx, n, coef + k * (n * n + 1));
    if (d.err) break;
    if (cnt) r.nzmask |= 1u << k;
    done++;
  }
  uint32_t w = (1u << done) - 1;
  if (!d.err) {
    r.cmode = (uint8_t)d.sym(ctxChromaMode);
    int cnt = entropyBlock(d, kPlaneChroma, 0, 8, coef + kCoefCb);
    if (!d.err) {
      w |= 1u << 16;
      if (cnt) r.nzmask |= 1u << 16;
      cnt = entropyBlock(d, kPlaneChroma, 0, 8, coef + kCoefCr);
      if (!d.err) {
        w |= 1u << 17;
        if (cnt) r.nzmask |= 1u << 17;
      }
    }
  }
  r.wmask = w;
}

// Inter-frame macroblock symbols (decodeInterMB + reconInterMB grammar).
__device__ void entropyInterMB(TileCtx& tc, int mbx, int mby, MBRec& r, uint32_t* coef, int& intraCount) {
  Chain& d = tc.d;
  const FrameDesc& f = *tc.f;
  const int idx = mby * f.mbCols + mbx;
  const int mode = d.sym(ctxMBMode);
  if (mode == mbSkip) {
    const short2 p = predictMV(tc, mbx, mby);
    storeMV(f, idx, p, d.lane);
    r.mode = kRecSkip;
    r.mv[0][0] = p.x;
    r.mv[0][1] = p.y;
    r.wmask = kWriteAll;
    return;
  }
  if (mode == mbIntra) {
    entropyIntraMB(tc, r, coef);
    storeMV(f, idx, make_short2(0, 0), d.lane);
    if (r.wmask) intraCount++;
    return;
  }
  if (mode != mbInter) {
    if (!d.err) d.err = kErrCorrupt;
    r.mode = kRecNone;
    return;
  }
  const int refSel = d.sym(ctxRef);
  if (refSel < 0 || refSel >= kNumRefs) {
    if (!d.err) d.err = kErrCorrupt;
    r.mode = kRecNone;
    return;
  }
  short2 pred = predictMV(tc, mbx, mby);
  if (refSel == refGolden) pred = make_short2(0, 0);
  const int part = d.sym(ctxPart);
  if (part < 0 || part >= kNumPartModes) {
    if (!d.err) d.err = kErrCorrupt;
    r.mode = kRecNone;
    return;
  }
  const int np = part == partWhole ? 1 : (part == part8x8 ? 4 : 2);
  for (int i = 0; i < np; i++) {
    const int ppx = i > 0 ? r.mv[0][0] : pred.x;
    const int ppy = i > 0 ? r.mv[0][1] : pred.y;
    const int dx = d.mvComponent(ctxMVClassX);
    r.mv[i][0] = clampMV(ppx + dx);
    const int dy = d.mvComponent(ctxMVClassY);
    r.mv[i][1] = clampMV(ppy + dy);
  }
  if (d.err) {
    r.mode = kRecNone;
    return;
  }
  storeMV(f, idx, refSel == refGolden ? make_short2(0, 0) : make_short2(r.mv[0][0], r.mv[0][1]), d.lane);
  r.mode = kRecInter;
  r.ref = (uint8_t)refSel;
  r.part = (uint8_t)part;
  const int cbp = d.sym(ctxCBP);
  if (cbp < 0 || cbp >= kNumCBP || d.err) {
    if (!d.err) d.err = kErrCorrupt;
    r.wmask = 0;
    return;
  }
  r.cbp = (uint8_t)cbp;
  uint32_t w = 0;
  if (cbp & cbpLuma) {
    int tx = d.sym(ctxTxSize);
    if (tx < 0 || tx >= 3) {
      if (!d.err) d.err = kErrCorrupt;
      tx = 0;
    }
    r.tx = (uint8_t)tx;
    const int n = 4 << tx, nb = 16 >> (2 * tx);
    int done = 0;
    for (int k = 0; k < nb && !d.err; k++) {
      const int cnt = entropyBlock(d, kPlaneLuma, tx, n, coef + k * (n * n + 1));
      if (d.err) break;
      if (cnt) r.nzmask |= 1u << k;
      done++;
    }
    if (d.err) {
      r.wmask = (1u << done) - 1;
      return;
    }
    w = 0xFFFFu;
  } else {
    w = 0xFFFFu;  // motion-compensated luma, written directly
  }
  if (cbp & cbpCb) {
    const int cnt = entropyBlock(d, kPlaneChroma, 0, 8, coef + kCoefCb);
    if (!d.err) {
      w |= 1u << 16;
      if (cnt) r.nzmask |= 1u << 16;
    }
  } else {
    w |= 1u << 16;
  }
  if (cbp & cbpCr) {
    if (!d.err) {
      const int cnt = entropyBlock(d, kPlaneChroma, 0, 8, coef + kCoefCr);
      if (!d.err) {
        w |= 1u << 17;
        if (cnt) r.nzmask |= 1u << 17;
      }
    }
  } else {
    w |= 1u << 17;
  }
  r.wmask = w;
}

__device__ __forceinline__ void storeRec(MBRec* dst, const MBRec& r, int lane) {
  const uint32_t* s = reinterpret_cast<const uint32_t*>(&r);
  uint32_t* o = reinterpret_cast<uint32_t*>(dst);
  if (lane < 12) o[lane] = s[lane];
}

constexpr int kEntropyWarps = 4;

__global__ void __launch_bounds__(32 * kEntropyWarps) kEntropy(const FrameDesc* frames, const int2* jobs, int njobs) {
  __shared__ WarpTables sT[kEntropyWarps];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int j = blockIdx.x * kEntropyWarps + warp;
  if (j >= njobs) return;
  const FrameDesc& f = frames[jobs[j].x];
  if (f.gate && *f.gate) return;
  const int tile = jobs[j].y;
  WarpTables& T = sT[warp];
  {
    const uint16_t* src = &f.tables->start[0][0];
    for (int i = lane; i < kNumContexts * 17; i += 32) T.start[i] = src[i];
    for (int i = lane; i < kNumContexts; i += 32) T.used[i] = f.tables->used[i];
  }
  __syncwarp();
  const TileRange tr = f.tiles[tile];
  TileCtx tc;
  tc.f = &f;
  tc.bx0 = tr.mbX0;
  tc.bx1 = tr.mbX1;
  tc.by0 = tr.mbY0;
  tc.by1 = tr.mbY1;
  Chain& d = tc.d;
  d.buf = f.pkt + tr.offset;
  d.pos = (int32_t)tr.length;
  d.err = 0;
  d.t = &T;
  d.lane = lane;
  const int tw = tc.bx1 - tc.bx0;
  const int total = tw * (tc.by1 - tc.by0);
  int done = 0;
  int intraCount = 0;
  if (tr.length < (uint32_t)(kStates * 4)) {
    d.err = kErrCorrupt;
  } else {
    uint32_t st[4];
    for (int i = kStates - 1; i >= 0; i--) {
      const uint32_t a = __ldg(d.buf + d.pos - 1), b = __ldg(d.buf + d.pos - 2), c = __ldg(d.buf + d.pos - 3),
                     e = __ldg(d.buf + d.pos - 4);
      d.pos -= 4;
      st[i] = a << 24 | b << 16 | c << 8 | e;
    }
    d.x0 = st[0];
    d.x1 = st[1];
    d.x2 = st[2];
    d.x3 = st[3];
    for (; done < total; done++) {
      const int mbx = tc.bx0 + done % tw, mby = tc.by0 + done / tw;
      const int idx = mby * f.mbCols + mbx;
      MBRec r;
      {
        uint32_t* z = reinterpret_cast<uint32_t*>(&r);
#pragma unroll
        for (int k = 0; k < 12; k++) z[k] = 0;
      }
      uint32_t* coef = f.coef + (size_t)idx * kCoefPerMB;
      if (f.inter) {
        entropyInterMB(tc, mbx, mby, r, coef, intraCount);
      } else {
        entropyIntraMB(tc, r, coef);
        if (r.wmask) intraCount++;
      }
      storeRec(f.mbrec + idx, r, lane);
      if (d.err) {
        done++;
        break;
      }
    }
  }
  // Macroblocks the tile never reached are left untouched by reconstruction.
  for (int k = done + lane; k < total; k += 32) {
    const int mbx = tc.bx0 + k % tw, mby = tc.by0 + k / tw;
    MBRec* r = f.mbrec + (size_t)mby * f.mbCols + mbx;
    r->mode = kRecNone;
    r->wmask = 0;
  }
  if (lane == 0) {
    f.tileStat[tile].err = d.err;
    f.tileStat[tile].intraCount = intraCount;
    if (d.err) atomicExch(f.status, kErrCorrupt);
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
  if (!f.inter || (f.gate && *f.gate)) return;
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

__global__ void __launch_bounds__(32 * kIntraWarps) kIntraRecon(const FrameDesc* frames, const int2* jobs, int njobs) {
  __shared__ IntraScratch sS[kIntraWarps];
  const int j = blockIdx.x;
  if (j >= njobs) return;
  const FrameDesc& f = frames[jobs[j].x];
  if (f.gate && *f.gate) return;
  const int tile = jobs[j].y;
  if (f.tileStat[tile].intraCount == 0) return;
  const TileRange tr = f.tiles[tile];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int tw = tr.mbX1 - tr.mbX0, th = tr.mbY1 - tr.mbY0;
  const int waves = tw + 2 * (th - 1);
  for (int t = 0; t < waves; t++) {
    // Macroblocks (x, y) of the tile with x + 2y == t.
    int ylo = t - (tw - 1) > 0 ? (t - (tw - 1) + 1) / 2 : 0;
    int yhi = t / 2 < th - 1 ? t / 2 : th - 1;
    for (int y = ylo + warp; y <= yhi; y += kIntraWarps) {
      const int x = t - 2 * y;
      intraMB(f, sS[warp], tr.mbX0 + x, tr.mbY0 + y, tr.mbX0, tr.mbX1, tr.mbY0, lane);
    }
    __syncthreads();
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
