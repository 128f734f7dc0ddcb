// The encoder's alt-ref temporal filter on the GPU: buildAltRef
// (ebiv/encoder.go:326-407), the golden-override image of a GOP.  The GOP
// head is denoised by averaging, per 16x16 luma block, every window frame
// whose block agrees with the head's (luma SAD at most 6 per sample); the
// co-located chroma follows its luma block's decision.  Per sample the
// result is (sum + count/2) / count over the head and the accepted frames.
//
// One warp per 16x16 block: lane l owns luma row l/2, columns 8(l%2)..+8
// (one aligned 8-byte load per frame) and the 2 + 2 chroma samples of chroma
// row l/4, columns 2(l%4)..+2.  Each window frame's block is read once: the
// loaded luma feeds both the SAD (a warp reduction) and, when the block is
// accepted, the sums kept in registers.  The frames sit in device buffers
// padded to whole macroblocks with 64-byte row pitches, so every load is
// aligned and in bounds; samples outside the visible frame are masked.  The
// work is a stream over n frames: HBM-bound, n * 1.5 * W * H bytes read.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <vector>

#include "../../include/ebivgpu.h"
#include "ebiv_format.h"

namespace ebiv {
namespace dev {

struct AltRefPlanes {
  const uint8_t* const* y;   // n device pointers, pitch yp
  const uint8_t* const* cb;  // n device pointers, pitch cp
  const uint8_t* const* cr;
  int n, w, h, cw, ch, yp, cp, mbCols, mbRows;
};

__global__ void __launch_bounds__(256) kAltRef(AltRefPlanes P, uint8_t* oy, uint8_t* ocb, uint8_t* ocr,
                                               int* accepted) {
  const int lane = threadIdx.x & 31;
  const int blk = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (blk >= P.mbCols * P.mbRows) return;
  const int bx = (blk % P.mbCols) * 16, by = (blk / P.mbCols) * 16;
  const int bw = min(16, P.w - bx), bh = min(16, P.h - by);
  const int ry = lane >> 1, rx = (lane & 1) * 8;
  const bool rowOK = ry < bh;
  const size_t yoff = (size_t)(by + ry) * P.yp + bx + rx;
  // Chroma region of the block: [bx/2, min(cw, (bx+bw+1)/2)) x [by/2, ...).
  const int cx0 = bx >> 1, cy0 = by >> 1;
  const int cx1 = min(P.cw, (bx + bw + 1) >> 1), cy1 = min(P.ch, (by + bh + 1) >> 1);
  const int cry = cy0 + (lane >> 2), crx = cx0 + (lane & 3) * 2;
  const bool c0 = cry < cy1 && crx < cx1, c1 = cry < cy1 && crx + 1 < cx1;
  const size_t coff = (size_t)cry * P.cp + crx;

  uint32_t sy[8], sb[2], sr[2];
  uint8_t t8[8];  // the head's luma samples (SAD reference)
  {
    const uint64_t v = *reinterpret_cast<const uint64_t*>(P.y[0] + yoff);
#pragma unroll
    for (int k = 0; k < 8; k++) {
      t8[k] = (uint8_t)(v >> (8 * k));
      sy[k] = t8[k];
    }
    const uint16_t b2 = *reinterpret_cast<const uint16_t*>(P.cb[0] + coff);
    const uint16_t r2 = *reinterpret_cast<const uint16_t*>(P.cr[0] + coff);
    sb[0] = b2 & 0xFF;
    sb[1] = b2 >> 8;
    sr[0] = r2 & 0xFF;
    sr[1] = r2 >> 8;
  }
  int cnt = 1, acc = 0;
  const int64_t limit = (int64_t)bw * bh * 6;
  for (int j = 1; j < P.n; j++) {
    const uint64_t v = *reinterpret_cast<const uint64_t*>(P.y[j] + yoff);
    const uint16_t b2 = *reinterpret_cast<const uint16_t*>(P.cb[j] + coff);
    const uint16_t r2 = *reinterpret_cast<const uint16_t*>(P.cr[j] + coff);
    int sad = 0;
#pragma unroll
    for (int k = 0; k < 8; k++) {
      const int d = (int)((v >> (8 * k)) & 0xFF) - (int)t8[k];
      if (rowOK && rx + k < bw) sad += d < 0 ? -d : d;
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) sad += __shfl_xor_sync(0xffffffffu, sad, o);
    if ((int64_t)sad > limit) continue;  // the same for the whole warp
    cnt++;
    acc++;
#pragma unroll
    for (int k = 0; k < 8; k++) sy[k] += (uint32_t)((v >> (8 * k)) & 0xFF);
    sb[0] += b2 & 0xFF;
    sb[1] += b2 >> 8;
    sr[0] += r2 & 0xFF;
    sr[1] += r2 >> 8;
  }
  const uint32_t c = (uint32_t)cnt, half = c / 2;
  if (rowOK) {
    uint8_t* o = oy + (size_t)(by + ry) * P.w + bx + rx;
#pragma unroll
    for (int k = 0; k < 8; k++)
      if (rx + k < bw) o[k] = (uint8_t)((sy[k] + half) / c);
  }
  if (c0) {
    ocb[(size_t)cry * P.cw + crx] = (uint8_t)((sb[0] + half) / c);
    ocr[(size_t)cry * P.cw + crx] = (uint8_t)((sr[0] + half) / c);
  }
  if (c1) {
    ocb[(size_t)cry * P.cw + crx + 1] = (uint8_t)((sb[1] + half) / c);
    ocr[(size_t)cry * P.cw + crx + 1] = (uint8_t)((sr[1] + half) / c);
  }
  if (lane == 0 && acc) atomicAdd(accepted, acc);
}

}  // namespace dev

// Device state of the filter: n padded frames, the output and the counter,
// grown on demand and reused across calls.
struct AltRefContext {
  int n = 0, w = 0, h = 0;
  uint8_t* frames = nullptr;  // n padded frames
  uint8_t* out = nullptr;     // packed W x H + 2 CW x CH
  int* accepted = nullptr;
  const uint8_t** ptrs = nullptr;  // 3n device pointers
  size_t frameBytes = 0, outBytes = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  int yp = 0, cp = 0, mbCols = 0, mbRows = 0;
  ~AltRefContext() { release(); }
  void release() {
    if (frames) cudaFree(frames);
    if (out) cudaFree(out);
    if (accepted) cudaFree(accepted);
    if (ptrs) cudaFree(ptrs);
    if (stream) cudaStreamDestroy(stream);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    frames = out = nullptr;
    accepted = nullptr;
    ptrs = nullptr;
    stream = nullptr;
    ev0 = ev1 = nullptr;
    n = 0;
  }
  int ensure(int nn, int ww, int hh) {
    if (stream && nn <= n && ww == w && hh == h) return kOK;
    release();
    w = ww;
    h = hh;
    n = nn;
    mbCols = (w + 15) / 16;
    mbRows = (h + 15) / 16;
    yp = (mbCols * 16 + 63) & ~63;
    cp = (mbCols * 8 + 63) & ~63;
    frameBytes = (size_t)yp * mbRows * 16 + 2 * (size_t)cp * mbRows * 8;
    const int cw = (w + 1) / 2, ch = (h + 1) / 2;
    outBytes = (size_t)w * h + 2 * (size_t)cw * ch;
    if (cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&ev0) != cudaSuccess || cudaEventCreate(&ev1) != cudaSuccess ||
        cudaMalloc(&frames, frameBytes * n) != cudaSuccess || cudaMalloc(&out, outBytes) != cudaSuccess ||
        cudaMalloc(&accepted, sizeof(int)) != cudaSuccess || cudaMalloc(&ptrs, 3 * sizeof(uint8_t*) * n) != cudaSuccess)
      return kErrDevice;
    // Zero the padding once: masked lanes read it.
    if (cudaMemset(frames, 0, frameBytes * n) != cudaSuccess) return kErrDevice;
    std::vector<const uint8_t*> p((size_t)3 * n);
    for (int j = 0; j < n; j++) {
      uint8_t* f = frames + frameBytes * j;
      p[(size_t)j] = f;
      p[(size_t)n + j] = f + (size_t)yp * mbRows * 16;
      p[(size_t)2 * n + j] = f + (size_t)yp * mbRows * 16 + (size_t)cp * mbRows * 8;
    }
    if (cudaMemcpy(ptrs, p.data(), p.size() * sizeof(uint8_t*), cudaMemcpyHostToDevice) != cudaSuccess)
      return kErrDevice;
    return kOK;
  }
};

// Runs the filter over frames already in the context's device buffers;
// returns the accepted block count (negative on a device error) and the
// kernel's duration through ms when non-null.
static int runAltRef(AltRefContext& c, int n, float* ms) {
  dev::AltRefPlanes P;
  P.y = c.ptrs;
  P.cb = c.ptrs + c.n;
  P.cr = c.ptrs + 2 * c.n;
  P.n = n;
  P.w = c.w;
  P.h = c.h;
  P.cw = (c.w + 1) / 2;
  P.ch = (c.h + 1) / 2;
  P.yp = c.yp;
  P.cp = c.cp;
  P.mbCols = c.mbCols;
  P.mbRows = c.mbRows;
  const int blocks = c.mbCols * c.mbRows;
  const int cw = P.cw, ch = P.ch;
  if (cudaMemsetAsync(c.accepted, 0, sizeof(int), c.stream) != cudaSuccess) return -1;
  cudaEventRecord(c.ev0, c.stream);
  dev::kAltRef<<<(blocks + 7) / 8, 256, 0, c.stream>>>(P, c.out, c.out + (size_t)c.w * c.h,
                                                       c.out + (size_t)c.w * c.h + (size_t)cw * ch, c.accepted);
  if (cudaGetLastError() != cudaSuccess) return -1;
  cudaEventRecord(c.ev1, c.stream);
  int acc = 0;
  if (cudaMemcpyAsync(&acc, c.accepted, sizeof(int), cudaMemcpyDeviceToHost, c.stream) != cudaSuccess ||
      cudaStreamSynchronize(c.stream) != cudaSuccess)
    return -1;
  if (ms) cudaEventElapsedTime(ms, c.ev0, c.ev1);
  return acc;
}

static int uploadFrames(AltRefContext& c, const uint8_t* const* frames, int n) {
  const int cw = (c.w + 1) / 2, ch = (c.h + 1) / 2;
  for (int j = 0; j < n; j++) {
    uint8_t* f = c.frames + c.frameBytes * j;
    const uint8_t* s = frames[j];
    if (cudaMemcpy2DAsync(f, c.yp, s, c.w, c.w, c.h, cudaMemcpyHostToDevice, c.stream) ||
        cudaMemcpy2DAsync(f + (size_t)c.yp * c.mbRows * 16, c.cp, s + (size_t)c.w * c.h, cw, cw, ch,
                          cudaMemcpyHostToDevice, c.stream) ||
        cudaMemcpy2DAsync(f + (size_t)c.yp * c.mbRows * 16 + (size_t)c.cp * c.mbRows * 8, c.cp,
                          s + (size_t)c.w * c.h + (size_t)cw * ch, cw, cw, ch, cudaMemcpyHostToDevice, c.stream))
      return kErrDevice;
  }
  return kOK;
}

}  // namespace ebiv

using namespace ebiv;

struct ebivgpu_altref {
  AltRefContext c;
};

extern "C" {

int ebivgpu_altref_create(ebivgpu_altref** out) {
  if (!out) return kErrArg;
  *out = new (std::nothrow) ebivgpu_altref();
  return *out ? kOK : kErrArg;
}

void ebivgpu_altref_destroy(ebivgpu_altref* a) { delete a; }

int ebivgpu_altref_build(ebivgpu_altref* a, const uint8_t* const* frames, int count, int width, int height, int window,
                         uint8_t* out, size_t cap, int* accepted) {
  if (!a || !frames || !accepted || width <= 0 || height <= 0 || count < 0) return kErrArg;
  *accepted = 0;
  const int n = std::min(window, count);
  if (n < 3) return kOK;  // window too small: no alt-ref (ebiv/encoder.go:329-331)
  const int cw = (width + 1) / 2, ch = (height + 1) / 2;
  const size_t need = (size_t)width * height + 2 * (size_t)cw * ch;
  if (!out || cap < need) return kErrArg;
  for (int j = 0; j < n; j++)
    if (!frames[j]) return kErrArg;
  AltRefContext& c = a->c;
  int st = c.ensure(n, width, height);
  if (st) return st;
  st = uploadFrames(c, frames, n);
  if (st) return st;
  const int acc = runAltRef(c, n, nullptr);
  if (acc < 0) return kErrDevice;
  *accepted = acc;
  if (acc && (cudaMemcpyAsync(out, c.out, need, cudaMemcpyDeviceToHost, c.stream) != cudaSuccess ||
              cudaStreamSynchronize(c.stream) != cudaSuccess))
    return kErrDevice;
  return kOK;
}

int ebivgpu_altref_time(ebivgpu_altref* a, int window, int reps, double* kernel_ms) {
  if (!a || !kernel_ms || reps <= 0 || !a->c.stream) return kErrArg;
  const int n = std::min(window, a->c.n);
  if (n < 3) return kErrArg;
  double total = 0;
  for (int r = 0; r < reps; r++) {
    float ms = 0;
    if (runAltRef(a->c, n, &ms) < 0) return kErrDevice;
    total += ms;
  }
  *kernel_ms = total / reps;
  return kOK;
}

}  // extern "C"
