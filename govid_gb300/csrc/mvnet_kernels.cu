// Learned motion-vector proposer for the EBIV encoder's inter search.
//
// A 4-layer 3x3 convolutional net on quarter-resolution luma of the current
// and reference frames (2 input channels; 32, 32, 32 hidden channels with
// ReLU; a 34-channel head) proposes motion-vector candidates for every 16x16
// macroblock.  The head's channels are logits over 17 horizontal and 17
// vertical displacement bins of 2 full pixels covering -16..16; they are
// averaged over the macroblock's 4x4 quarter-resolution pixels, and the
// top-8 joint (x, y) bins become the candidates the encoder evaluates
// (ebiv/encode_inter.go:381-419 is the search they replace).
//
// Everything the net computes runs in these hand-written kernels:
// activations are stored in BF16, every product is accumulated in FP32,
// gradients and the Adam state are FP32.  Labels come from an exhaustive
// full-pel SAD search on the GPU (kExhaustive), the search the proposer is
// trained and evaluated against.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <memory>
#include <mutex>
#include <vector>

#include "ebiv_format.h"
#include "mvnet.h"

namespace ebiv {
namespace mvnet {

using bf16 = __nv_bfloat16;

// Parameter layout (FP32 master copy): per layer, weights [Cout][Cin][9]
// then bias [Cout].
__host__ __device__ constexpr int layerCin(int l) { return l == 0 ? kInCh : kHidden; }
__host__ __device__ constexpr int layerCout(int l) { return l == kLayers - 1 ? kHeadCh : kHidden; }
__host__ __device__ constexpr int layerWeights(int l) { return layerCout(l) * layerCin(l) * 9; }
__host__ __device__ constexpr int layerOffset(int l) {
  return l == 0 ? 0 : layerOffset(l - 1) + layerWeights(l - 1) + layerCout(l - 1);
}
static_assert(layerOffset(kLayers) == kParams, "parameter count");

constexpr int kTile = 16;  // spatial tile of the convolution kernels
constexpr int kChunk = 16; // input channels staged in shared memory at a time

// ---------------------------------------------------------------------------
// Quarter-resolution input: 4x4 box average of the padded luma plane,
// normalised to (v - 128) / 64.
// ---------------------------------------------------------------------------
__global__ void kDownsample(const uint8_t* __restrict__ plane, int stride, int h, int w, bf16* __restrict__ out) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
  if (x >= w || y >= h) return;
  const uint8_t* p = plane + (size_t)(y * 4) * stride + x * 4;
  int s = 0;
#pragma unroll
  for (int r = 0; r < 4; r++)
#pragma unroll
    for (int c = 0; c < 4; c++) s += p[(size_t)r * stride + c];
  const int v = (s + 8) >> 4;
  out[(size_t)y * w + x] = __float2bfloat16((float)(v - 128) * (1.0f / 64.0f));
}

__device__ __forceinline__ float toF(bf16 v) { return __bfloat162float(v); }
__device__ __forceinline__ float toF(float v) { return v; }
template <class T>
__device__ __forceinline__ T fromF(float v);
template <>
__device__ __forceinline__ bf16 fromF<bf16>(float v) { return __float2bfloat16(v); }
template <>
__device__ __forceinline__ float fromF<float>(float v) { return v; }

// ---------------------------------------------------------------------------
// 3x3 convolution, zero padding 1, one thread per output pixel and all CO
// output channels in registers.  in [B][CI][h][w], w [CO][CI][9] (BF16),
// out [B][CO][h][w].  bias may be null; relu clamps at zero; mask (same
// shape as out, BF16) zeroes outputs where mask <= 0 (the ReLU derivative
// of the layer below, for the data gradient).
// ---------------------------------------------------------------------------
template <int CO, class TIn, class TOut>
__global__ void __launch_bounds__(kTile* kTile) kConv3x3(const TIn* __restrict__ in, int CI, const bf16* __restrict__ wt,
                                                         const float* __restrict__ bias, TOut* __restrict__ out,
                                                         const bf16* __restrict__ mask, int relu, int h, int w) {
  __shared__ float sIn[kChunk][kTile + 2][kTile + 2];
  __shared__ float sW[CO][kChunk][9];
  const int tx = threadIdx.x % kTile, ty = threadIdx.x / kTile;
  const int x0 = blockIdx.x * kTile, y0 = blockIdx.y * kTile, b = blockIdx.z;
  const int x = x0 + tx, y = y0 + ty;
  float acc[CO];
#pragma unroll
  for (int c = 0; c < CO; c++) acc[c] = 0.f;
  const TIn* inB = in + (size_t)b * CI * h * w;
  for (int c0 = 0; c0 < CI; c0 += kChunk) {
    const int nc = min(kChunk, CI - c0);
    __syncthreads();
    for (int i = threadIdx.x; i < nc * (kTile + 2) * (kTile + 2); i += blockDim.x) {
      const int c = i / ((kTile + 2) * (kTile + 2)), rem = i % ((kTile + 2) * (kTile + 2));
      const int yy = y0 - 1 + rem / (kTile + 2), xx = x0 - 1 + rem % (kTile + 2);
      float v = 0.f;
      if (yy >= 0 && yy < h && xx >= 0 && xx < w) v = toF(inB[((size_t)(c0 + c) * h + yy) * w + xx]);
      sIn[c][rem / (kTile + 2)][rem % (kTile + 2)] = v;
    }
    for (int i = threadIdx.x; i < CO * nc * 9; i += blockDim.x) {
      const int co = i / (nc * 9), rem = i % (nc * 9);
      sW[co][rem / 9][rem % 9] = __bfloat162float(wt[((size_t)co * CI + c0 + rem / 9) * 9 + rem % 9]);
    }
    __syncthreads();
    for (int c = 0; c < nc; c++)
#pragma unroll
      for (int k = 0; k < 9; k++) {
        const float v = sIn[c][ty + k / 3][tx + k % 3];
#pragma unroll
        for (int co = 0; co < CO; co++) acc[co] = fmaf(v, sW[co][c][k], acc[co]);
      }
  }
  if (x >= w || y >= h) return;
  TOut* o = out + (size_t)b * CO * h * w + (size_t)y * w + x;
  const bf16* m = mask ? mask + (size_t)b * CO * h * w + (size_t)y * w + x : nullptr;
#pragma unroll
  for (int co = 0; co < CO; co++) {
    float v = acc[co] + (bias ? bias[co] : 0.f);
    if (relu) v = fmaxf(v, 0.f);
    if (m && !(__bfloat162float(m[(size_t)co * h * w]) > 0.f)) v = 0.f;
    o[(size_t)co * h * w] = fromF<TOut>(v);
  }
}

// Weight gradient: dW[co][ci][k] += sum over pixels of g[co][p] * in[ci][p+k],
// db[co] += sum over pixels of g[co][p].  One CTA per (image, band of tile
// rows); each thread owns nine (co, ci, k) entries per 16x16 channel block
// and accumulates over every tile of the band before one atomic add each.
constexpr int kBand = 2;  // tile rows per CTA
template <int CO>
__global__ void __launch_bounds__(256) kConvWgrad(const bf16* __restrict__ in, int CI, const float* __restrict__ g,
                                                  float* __restrict__ dW, float* __restrict__ db, int h, int w) {
  __shared__ float sIn[kChunk][kTile + 2][kTile + 2];
  __shared__ float sG[kChunk][kTile * kTile];
  const int b = blockIdx.z;
  const int tilesX = (w + kTile - 1) / kTile;
  const int rowT0 = blockIdx.y * kBand;
  const int nCoB = (CO + kChunk - 1) / kChunk, nCiB = (CI + kChunk - 1) / kChunk;
  // entry e = threadIdx.x + 256*j (j < 9) of the (coB, ciB) block: co, ci, k
  for (int coB = 0; coB < nCoB; coB++)
    for (int ciB = 0; ciB < nCiB; ciB++) {
      float acc[9];
#pragma unroll
      for (int j = 0; j < 9; j++) acc[j] = 0.f;
      float accB = 0.f;
      for (int tr = rowT0; tr < rowT0 + kBand; tr++) {
        const int y0 = tr * kTile;
        if (y0 >= h) break;
        for (int tcol = 0; tcol < tilesX; tcol++) {
          const int x0 = tcol * kTile;
          __syncthreads();
          for (int i = threadIdx.x; i < kChunk * (kTile + 2) * (kTile + 2); i += blockDim.x) {
            const int c = i / ((kTile + 2) * (kTile + 2)), rem = i % ((kTile + 2) * (kTile + 2));
            const int yy = y0 - 1 + rem / (kTile + 2), xx = x0 - 1 + rem % (kTile + 2);
            const int ci = ciB * kChunk + c;
            float v = 0.f;
            if (ci < CI && yy >= 0 && yy < h && xx >= 0 && xx < w)
              v = __bfloat162float(in[(((size_t)b * CI + ci) * h + yy) * w + xx]);
            sIn[c][rem / (kTile + 2)][rem % (kTile + 2)] = v;
          }
          for (int i = threadIdx.x; i < kChunk * kTile * kTile; i += blockDim.x) {
            const int c = i / (kTile * kTile), p = i % (kTile * kTile);
            const int yy = y0 + p / kTile, xx = x0 + p % kTile;
            const int co = coB * kChunk + c;
            float v = 0.f;
            if (co < CO && yy < h && xx < w) v = g[(((size_t)b * CO + co) * h + yy) * w + xx];
            sG[c][p] = v;
          }
          __syncthreads();
#pragma unroll
          for (int j = 0; j < 9; j++) {
            const int e = threadIdx.x + 256 * j;  // < 16*16*9 = 2304
            const int c = e / (kChunk * 9), rem = e % (kChunk * 9), ci = rem / 9, k = rem % 9;
            const int ky = k / 3, kx = k % 3;
            float s = 0.f;
            for (int p = 0; p < kTile * kTile; p++) s = fmaf(sG[c][p], sIn[ci][p / kTile + ky][p % kTile + kx], s);
            acc[j] += s;
          }
          if (ciB == 0 && threadIdx.x < kChunk) {
            float s = 0.f;
            for (int p = 0; p < kTile * kTile; p++) s += sG[threadIdx.x][p];
            accB += s;
          }
        }
      }
#pragma unroll
      for (int j = 0; j < 9; j++) {
        const int e = threadIdx.x + 256 * j;
        const int c = e / (kChunk * 9), rem = e % (kChunk * 9), ci = rem / 9, k = rem % 9;
        const int co = coB * kChunk + c, cig = ciB * kChunk + ci;
        if (co < CO && cig < CI) atomicAdd(&dW[((size_t)co * CI + cig) * 9 + k], acc[j]);
      }
      if (ciB == 0 && threadIdx.x < kChunk && coB * kChunk + threadIdx.x < CO)
        atomicAdd(&db[coB * kChunk + threadIdx.x], accB);
    }
}

// Per macroblock: average the head over its 4x4 quarter-resolution pixels,
// softmax per axis; with labels, the cross-entropy loss, its gradient back
// onto the head pixels and top-1 / top-8 hits; otherwise the top-8 joint
// candidates.  One thread per macroblock.
__device__ __forceinline__ int binOf(int d) { return min(kBins - 1, max(0, (d + kRange + 1) >> 1)); }

__global__ void kPoolHead(const float* __restrict__ head, int B, int h, int w, const int16_t* __restrict__ labels,
                          float* __restrict__ gHead, float* __restrict__ stats, int16_t* __restrict__ cand,
                          float invCount) {
  const int mbCols = w / 4, mbRows = h / 4, mbs = mbCols * mbRows;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= B * mbs) return;
  const int b = t / mbs, mb = t % mbs, mx = (mb % mbCols) * 4, my = (mb / mbCols) * 4;
  const float* hb = head + (size_t)b * kHeadCh * h * w;
  float lg[kHeadCh];
  for (int c = 0; c < kHeadCh; c++) {
    float s = 0.f;
    for (int r = 0; r < 4; r++)
      for (int q = 0; q < 4; q++) s += hb[((size_t)c * h + my + r) * w + mx + q];
    lg[c] = s * (1.f / 16.f);
  }
  // log-softmax per axis
  float lse[2];
  for (int a = 0; a < 2; a++) {
    float m = -1e30f;
    for (int k = 0; k < kBins; k++) m = fmaxf(m, lg[a * kBins + k]);
    float s = 0.f;
    for (int k = 0; k < kBins; k++) s += __expf(lg[a * kBins + k] - m);
    lse[a] = m + __logf(s);
  }
  if (labels) {
    const int lb[2] = {binOf(labels[2 * (size_t)t]), binOf(labels[2 * (size_t)t + 1])};
    float loss = 0.f;
    bool top1 = true;
    float* gb = gHead + (size_t)b * kHeadCh * h * w;
    for (int a = 0; a < 2; a++) {
      loss += lse[a] - lg[a * kBins + lb[a]];
      int arg = 0;
      for (int k = 1; k < kBins; k++)
        if (lg[a * kBins + k] > lg[a * kBins + arg]) arg = k;
      top1 = top1 && arg == lb[a];
      for (int k = 0; k < kBins; k++) {
        const float p = __expf(lg[a * kBins + k] - lse[a]);
        const float gv = (p - (k == lb[a] ? 1.f : 0.f)) * invCount * (1.f / 16.f);
        for (int r = 0; r < 4; r++)
          for (int q = 0; q < 4; q++) gb[((size_t)(a * kBins + k) * h + my + r) * w + mx + q] = gv;
      }
    }
    // rank of the labelled joint bin among all joint bins
    const float sLab = lg[lb[0]] + lg[kBins + lb[1]];
    int better = 0;
    for (int kx = 0; kx < kBins; kx++)
      for (int ky = 0; ky < kBins; ky++) better += (lg[kx] + lg[kBins + ky] > sLab) ? 1 : 0;
    atomicAdd(&stats[0], loss * invCount);
    atomicAdd(&stats[1], top1 ? 1.f : 0.f);
    atomicAdd(&stats[2], better < kTopK ? 1.f : 0.f);
  }
  if (cand) {
    // top-4 bins per axis, then the best 8 of their 16 pairs
    int ix[4], iy[4];
    for (int a = 0; a < 2; a++) {
      int* id = a ? iy : ix;
      bool used[kBins];
      for (int k = 0; k < kBins; k++) used[k] = false;
      for (int j = 0; j < 4; j++) {
        int best = -1;
        for (int k = 0; k < kBins; k++)
          if (!used[k] && (best < 0 || lg[a * kBins + k] > lg[a * kBins + best])) best = k;
        used[best] = true;
        id[j] = best;
      }
    }
    bool taken[16];
    for (int j = 0; j < 16; j++) taken[j] = false;
    int16_t* o = cand + (size_t)t * kTopK * 2;
    for (int j = 0; j < kTopK; j++) {
      int best = -1;
      float bs = -1e30f;
      for (int q = 0; q < 16; q++) {
        const float s = lg[ix[q / 4]] + lg[kBins + iy[q % 4]];
        if (!taken[q] && (best < 0 || s > bs)) {  // the first untaken pair even if the logits are not finite
          bs = s;
          best = q;
        }
      }
      taken[best] = true;
      o[2 * j] = (int16_t)(-kRange + 2 * ix[best / 4]);
      o[2 * j + 1] = (int16_t)(-kRange + 2 * iy[best % 4]);
    }
  }
}

// Adam on the FP32 master parameters; refreshes the BF16 weight copy and
// clears the gradients.
__global__ void kAdam(float* __restrict__ p, float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                      bf16* __restrict__ pb, int n, float lr, float b1, float b2, float c1, float c2, float eps) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  const float pi = p[i] - lr * (mi * c1) / (sqrtf(vi * c2) + eps);
  p[i] = pi;
  pb[i] = __float2bfloat16(pi);
  g[i] = 0.f;
}

__global__ void kToBF16(const float* __restrict__ p, bf16* __restrict__ pb, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) pb[i] = __float2bfloat16(p[i]);
}

// Weights of layer l arranged for its data gradient: wT[ci][co][8-k] = w[co][ci][k].
__global__ void kTransposeFlip(const bf16* __restrict__ w, bf16* __restrict__ wT, int CO, int CI) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= CO * CI * 9) return;
  const int co = i / (CI * 9), ci = (i / 9) % CI, k = i % 9;
  wT[((size_t)ci * CO + co) * 9 + (8 - k)] = w[i];
}

__global__ void kGather(const bf16* __restrict__ data, const int* __restrict__ idx, bf16* __restrict__ x, size_t per,
                        const int16_t* __restrict__ lab, int16_t* __restrict__ labOut, int mbs, int B) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < (size_t)B * per) x[i] = data[(size_t)idx[i / per] * per + i % per];
  if (i < (size_t)B * mbs * 2) labOut[i] = lab[(size_t)idx[i / (mbs * 2)] * mbs * 2 + i % (mbs * 2)];
}

// ---------------------------------------------------------------------------
// Exhaustive full-pel SAD search: for every 16x16 macroblock, the vector in
// [-R, R]^2 (full pels) with the smallest SAD between the current block and
// the reference (coordinates clamped to the plane, as motion compensation
// samples them).  Ties go to the zero vector, then to raster order, as the
// encoder's exhaustive search scans.  One CTA per macroblock.
// ---------------------------------------------------------------------------
constexpr int kMaxR = 16;
__global__ void __launch_bounds__(256) kExhaustive(const uint8_t* __restrict__ cur, const uint8_t* __restrict__ ref,
                                                   int stride, int W, int H, int mbCols, int R,
                                                   int16_t* __restrict__ mvOut, int32_t* __restrict__ sadOut) {
  __shared__ uint8_t sCur[16][16];
  __shared__ uint8_t sRef[16 + 2 * kMaxR][16 + 2 * kMaxR];
  __shared__ unsigned long long sBest;
  const int mb = blockIdx.x, mbx = mb % mbCols, mby = mb / mbCols;
  const int x0 = mbx * 16, y0 = mby * 16, span = 16 + 2 * R;
  for (int i = threadIdx.x; i < 256; i += blockDim.x) sCur[i / 16][i % 16] = cur[(size_t)(y0 + i / 16) * stride + x0 + i % 16];
  for (int i = threadIdx.x; i < span * span; i += blockDim.x) {
    const int yy = min(max(y0 - R + i / span, 0), H - 1), xx = min(max(x0 - R + i % span, 0), W - 1);
    sRef[i / span][i % span] = ref[(size_t)yy * stride + xx];
  }
  if (threadIdx.x == 0) sBest = ~0ull;
  __syncthreads();
  const int n = (2 * R + 1) * (2 * R + 1);
  unsigned long long best = ~0ull;
  for (int c = threadIdx.x; c < n; c += blockDim.x) {
    const int dy = c / (2 * R + 1) - R, dx = c % (2 * R + 1) - R;
    int s = 0;
    for (int r = 0; r < 16; r++)
#pragma unroll
      for (int q = 0; q < 16; q++) s += abs((int)sCur[r][q] - (int)sRef[r + dy + R][q + dx + R]);
    const unsigned rank = (dx == 0 && dy == 0) ? 0u : (unsigned)c + 1u;  // zero first, then raster order
    const unsigned long long key = ((unsigned long long)(unsigned)s << 32) | rank;
    best = key < best ? key : best;
  }
  atomicMin(&sBest, best);
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned rank = (unsigned)(sBest & 0xffffffffu);
    int dx = 0, dy = 0;
    if (rank) {
      dy = (int)(rank - 1) / (2 * R + 1) - R;
      dx = (int)(rank - 1) % (2 * R + 1) - R;
    }
    mvOut[2 * mb] = (int16_t)dx;
    mvOut[2 * mb + 1] = (int16_t)dy;
    if (sadOut) sadOut[mb] = (int32_t)(sBest >> 32);
  }
}

}  // namespace mvnet

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
using namespace mvnet;

namespace {
template <class T>
T* dalloc(size_t n, int* st) {
  T* p = nullptr;
  if (cudaMalloc(&p, sizeof(T) * (n ? n : 1)) != cudaSuccess) {
    *st = kErrDevice;
    return nullptr;
  }
  cudaMemset(p, 0, sizeof(T) * (n ? n : 1));
  return p;
}

// Deterministic parameter initialisation (He-uniform weights, zero bias)
// from a counter-based generator.
uint64_t mix64(uint64_t z) {
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}
}  // namespace

MvNet::~MvNet() {
  for (void* p : allocs_) cudaFree(p);
  if (stream_) cudaStreamDestroy(stream_);
}

int MvNet::init(int maxBatch, int padW, int padH, int maxPairs, uint64_t seed) {
  if (maxBatch < 1 || padW < 16 || padH < 16 || (padW & 15) || (padH & 15) || maxPairs < 0) return kErrArg;
  B_ = maxBatch;
  W_ = padW;
  H_ = padH;
  w_ = padW / 4;
  h_ = padH / 4;
  mbs_ = (padW / 16) * (padH / 16);
  maxPairs_ = maxPairs;
  int st = kOK;
  if (cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking) != cudaSuccess) return kErrDevice;
  auto reg = [&](void* p) { allocs_.push_back(p); };
  const size_t plane = (size_t)h_ * w_;
  params_ = dalloc<float>(kParams, &st);
  reg(params_);
  grads_ = dalloc<float>(kParams, &st);
  reg(grads_);
  adamM_ = dalloc<float>(kParams, &st);
  reg(adamM_);
  adamV_ = dalloc<float>(kParams, &st);
  reg(adamV_);
  pbf_ = dalloc<bf16>(kParams, &st);
  reg(pbf_);
  wT_ = dalloc<bf16>(kHidden * kHidden * 9 + kHeadCh * kHidden * 9, &st);
  reg(wT_);
  x0_ = dalloc<bf16>((size_t)B_ * kInCh * plane, &st);
  reg(x0_);
  for (int l = 0; l < kLayers - 1; l++) {
    act_[l] = dalloc<bf16>((size_t)B_ * kHidden * plane, &st);
    reg(act_[l]);
    gAct_[l] = dalloc<float>((size_t)B_ * kHidden * plane, &st);
    reg(gAct_[l]);
  }
  head_ = dalloc<float>((size_t)B_ * kHeadCh * plane, &st);
  reg(head_);
  gHead_ = dalloc<float>((size_t)B_ * kHeadCh * plane, &st);
  reg(gHead_);
  labels_ = dalloc<int16_t>((size_t)B_ * mbs_ * 2, &st);
  reg(labels_);
  cand_ = dalloc<int16_t>((size_t)B_ * mbs_ * kTopK * 2, &st);
  reg(cand_);
  stats_ = dalloc<float>(4, &st);
  reg(stats_);
  idx_ = dalloc<int>(B_, &st);
  reg(idx_);
  planes_ = dalloc<uint8_t>((size_t)2 * W_ * H_, &st);
  reg(planes_);
  mvs_ = dalloc<int16_t>((size_t)mbs_ * 2, &st);
  reg(mvs_);
  sads_ = dalloc<int32_t>(mbs_, &st);
  reg(sads_);
  if (maxPairs_ > 0) {
    data_ = dalloc<bf16>((size_t)maxPairs_ * kInCh * plane, &st);
    reg(data_);
    dataLab_ = dalloc<int16_t>((size_t)maxPairs_ * mbs_ * 2, &st);
    reg(dataLab_);
  }
  if (st) return st;
  std::vector<float> p(kParams, 0.f);
  for (int l = 0; l < kLayers; l++) {
    const float bound = std::sqrt(6.f / (float)(layerCin(l) * 9));
    for (int i = 0; i < layerWeights(l); i++) {
      const uint64_t r = mix64(seed * 0x100000001b3ull + (uint64_t)(layerOffset(l) + i));
      const float u = (float)(r >> 40) * (1.f / 16777216.f);  // [0,1)
      p[(size_t)layerOffset(l) + i] = (2.f * u - 1.f) * bound;
    }
  }
  return setParams(p.data());
}

int MvNet::setParams(const float* p) {
  if (cudaMemcpyAsync(params_, p, sizeof(float) * kParams, cudaMemcpyHostToDevice, stream_) != cudaSuccess)
    return kErrDevice;
  kToBF16<<<(kParams + 255) / 256, 256, 0, stream_>>>(params_, pbf_, kParams);
  cudaMemsetAsync(adamM_, 0, sizeof(float) * kParams, stream_);
  cudaMemsetAsync(adamV_, 0, sizeof(float) * kParams, stream_);
  cudaMemsetAsync(grads_, 0, sizeof(float) * kParams, stream_);
  step_ = 0;
  return cudaStreamSynchronize(stream_) == cudaSuccess ? kOK : kErrDevice;
}

int MvNet::getParams(float* p) const {
  if (cudaMemcpyAsync(p, params_, sizeof(float) * kParams, cudaMemcpyDeviceToHost, stream_) != cudaSuccess)
    return kErrDevice;
  return cudaStreamSynchronize(stream_) == cudaSuccess ? kOK : kErrDevice;
}

int MvNet::uploadPair(const uint8_t* cur, const uint8_t* ref, int stride, bf16* dst) {
  if (cudaMemcpy2DAsync(planes_, W_, cur, stride, W_, H_, cudaMemcpyHostToDevice, stream_) != cudaSuccess ||
      cudaMemcpy2DAsync(planes_ + (size_t)W_ * H_, W_, ref, stride, W_, H_, cudaMemcpyHostToDevice, stream_) !=
          cudaSuccess)
    return kErrDevice;
  const dim3 g((w_ + 127) / 128, h_);
  kDownsample<<<g, 128, 0, stream_>>>(planes_, W_, h_, w_, dst);
  kDownsample<<<g, 128, 0, stream_>>>(planes_ + (size_t)W_ * H_, W_, h_, w_, dst + (size_t)h_ * w_);
  return kOK;
}

int MvNet::exhaustive(const uint8_t* cur, const uint8_t* ref, int stride, int range, int16_t* mv, int32_t* sad) {
  if (range < 0 || range > kMaxR) return kErrArg;
  if (cudaMemcpy2DAsync(planes_, W_, cur, stride, W_, H_, cudaMemcpyHostToDevice, stream_) != cudaSuccess ||
      cudaMemcpy2DAsync(planes_ + (size_t)W_ * H_, W_, ref, stride, W_, H_, cudaMemcpyHostToDevice, stream_) !=
          cudaSuccess)
    return kErrDevice;
  kExhaustive<<<mbs_, 256, 0, stream_>>>(planes_, planes_ + (size_t)W_ * H_, W_, W_, H_, W_ / 16, range, mvs_, sads_);
  if (cudaMemcpyAsync(mv, mvs_, sizeof(int16_t) * 2 * mbs_, cudaMemcpyDeviceToHost, stream_) != cudaSuccess)
    return kErrDevice;
  if (sad && cudaMemcpyAsync(sad, sads_, sizeof(int32_t) * mbs_, cudaMemcpyDeviceToHost, stream_) != cudaSuccess)
    return kErrDevice;
  return cudaStreamSynchronize(stream_) == cudaSuccess ? kOK : kErrDevice;
}

int MvNet::addPair(const uint8_t* cur, const uint8_t* ref, int stride, const int16_t* labels) {
  if (pairs_ >= maxPairs_) return kErrArg;
  const size_t per = (size_t)kInCh * h_ * w_;
  int st = uploadPair(cur, ref, stride, data_ + (size_t)pairs_ * per);
  if (st) return st;
  if (cudaMemcpyAsync(dataLab_ + (size_t)pairs_ * mbs_ * 2, labels, sizeof(int16_t) * mbs_ * 2,
                      cudaMemcpyHostToDevice, stream_) != cudaSuccess)
    return kErrDevice;
  if (cudaStreamSynchronize(stream_) != cudaSuccess) return kErrDevice;
  pairs_++;
  return kOK;
}

int MvNet::setInput(int slot, const uint8_t* cur, const uint8_t* ref, int stride, const int16_t* labels) {
  if (slot < 0 || slot >= B_) return kErrArg;
  int st = uploadPair(cur, ref, stride, x0_ + (size_t)slot * kInCh * h_ * w_);
  if (st) return st;
  if (labels && cudaMemcpyAsync(labels_ + (size_t)slot * mbs_ * 2, labels, sizeof(int16_t) * mbs_ * 2,
                                cudaMemcpyHostToDevice, stream_) != cudaSuccess)
    return kErrDevice;
  return cudaStreamSynchronize(stream_) == cudaSuccess ? kOK : kErrDevice;
}

int MvNet::gather(const int* idx, int batch) {
  if (batch < 1 || batch > B_) return kErrArg;
  for (int i = 0; i < batch; i++)
    if (idx[i] < 0 || idx[i] >= pairs_) return kErrArg;
  if (cudaMemcpyAsync(idx_, idx, sizeof(int) * batch, cudaMemcpyHostToDevice, stream_) != cudaSuccess)
    return kErrDevice;
  const size_t per = (size_t)kInCh * h_ * w_;
  const size_t n = std::max((size_t)batch * per, (size_t)batch * mbs_ * 2);
  kGather<<<(unsigned)((n + 255) / 256), 256, 0, stream_>>>(data_, idx_, x0_, per, dataLab_, labels_, mbs_, batch);
  return kOK;
}

void MvNet::forward(int batch) {
  const dim3 g((w_ + kTile - 1) / kTile, (h_ + kTile - 1) / kTile, batch);
  const int T = kTile * kTile;
  const bf16* W0 = pbf_ + layerOffset(0);
  kConv3x3<kHidden, bf16, bf16><<<g, T, 0, stream_>>>(x0_, kInCh, W0, params_ + layerOffset(0) + layerWeights(0),
                                                      act_[0], nullptr, 1, h_, w_);
  for (int l = 1; l < kLayers - 1; l++)
    kConv3x3<kHidden, bf16, bf16><<<g, T, 0, stream_>>>(act_[l - 1], kHidden, pbf_ + layerOffset(l),
                                                        params_ + layerOffset(l) + layerWeights(l), act_[l], nullptr,
                                                        1, h_, w_);
  const int L = kLayers - 1;
  kConv3x3<kHeadCh, bf16, float><<<g, T, 0, stream_>>>(act_[L - 1], kHidden, pbf_ + layerOffset(L),
                                                       params_ + layerOffset(L) + layerWeights(L), head_, nullptr, 0,
                                                       h_, w_);
}

void MvNet::backward(int batch) {
  const dim3 g((w_ + kTile - 1) / kTile, (h_ + kTile - 1) / kTile, batch);
  const dim3 gw(1, (h_ + kTile * kBand - 1) / (kTile * kBand), batch);
  const int T = kTile * kTile;
  // head: weights, then data gradient onto act[L-1] masked by its ReLU
  const int L = kLayers - 1;
  kConvWgrad<kHeadCh><<<gw, 256, 0, stream_>>>(act_[L - 1], kHidden, gHead_, grads_ + layerOffset(L),
                                               grads_ + layerOffset(L) + layerWeights(L), h_, w_);
  kTransposeFlip<<<(layerWeights(L) + 255) / 256, 256, 0, stream_>>>(pbf_ + layerOffset(L), wT_, kHeadCh, kHidden);
  kConv3x3<kHidden, float, float><<<g, T, 0, stream_>>>(gHead_, kHeadCh, wT_, nullptr, gAct_[L - 1], act_[L - 1], 0,
                                                        h_, w_);
  for (int l = L - 1; l >= 1; l--) {
    kConvWgrad<kHidden><<<gw, 256, 0, stream_>>>(act_[l - 1], kHidden, gAct_[l], grads_ + layerOffset(l),
                                                 grads_ + layerOffset(l) + layerWeights(l), h_, w_);
    kTransposeFlip<<<(layerWeights(l) + 255) / 256, 256, 0, stream_>>>(pbf_ + layerOffset(l), wT_, kHidden, kHidden);
    kConv3x3<kHidden, float, float><<<g, T, 0, stream_>>>(gAct_[l], kHidden, wT_, nullptr, gAct_[l - 1], act_[l - 1],
                                                          0, h_, w_);
  }
  kConvWgrad<kHidden><<<gw, 256, 0, stream_>>>(x0_, kInCh, gAct_[0], grads_ + layerOffset(0),
                                               grads_ + layerOffset(0) + layerWeights(0), h_, w_);
}

int MvNet::lossAndGrad(int batch, bool grad, float* stats) {
  cudaMemsetAsync(stats_, 0, sizeof(float) * 4, stream_);
  forward(batch);
  const int n = batch * mbs_;
  kPoolHead<<<(n + 127) / 128, 128, 0, stream_>>>(head_, batch, h_, w_, labels_, gHead_, stats_, nullptr,
                                                  1.f / (float)n);
  if (grad) backward(batch);
  if (stats) {
    float s[4];
    if (cudaMemcpyAsync(s, stats_, sizeof(s), cudaMemcpyDeviceToHost, stream_) != cudaSuccess) return kErrDevice;
    if (cudaStreamSynchronize(stream_) != cudaSuccess) return kErrDevice;
    stats[0] = s[0];
    stats[1] = s[1] / (float)n;
    stats[2] = s[2] / (float)n;
  }
  return cudaStreamSynchronize(stream_) == cudaSuccess ? kOK : kErrDevice;
}

int MvNet::gradients(int batch, float* grads, float* stats) {
  if (batch < 1 || batch > B_) return kErrArg;
  cudaMemsetAsync(grads_, 0, sizeof(float) * kParams, stream_);
  int st = lossAndGrad(batch, true, stats);
  if (st) return st;
  if (grads && cudaMemcpyAsync(grads, grads_, sizeof(float) * kParams, cudaMemcpyDeviceToHost, stream_) != cudaSuccess)
    return kErrDevice;
  cudaMemsetAsync(grads_, 0, sizeof(float) * kParams, stream_);
  return cudaStreamSynchronize(stream_) == cudaSuccess ? kOK : kErrDevice;
}

int MvNet::trainStep(int batch, float lr, float* stats) {
  if (batch < 1 || batch > B_) return kErrArg;
  int st = lossAndGrad(batch, true, nullptr);
  if (st) return st;
  step_++;
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.f / (1.f - std::pow(b1, (float)step_)), c2 = 1.f / (1.f - std::pow(b2, (float)step_));
  kAdam<<<(kParams + 255) / 256, 256, 0, stream_>>>(params_, grads_, adamM_, adamV_, pbf_, kParams, lr, b1, b2, c1,
                                                    c2, 1e-8f);
  if (stats) {
    float s[4];
    if (cudaMemcpyAsync(s, stats_, sizeof(s), cudaMemcpyDeviceToHost, stream_) != cudaSuccess) return kErrDevice;
    if (cudaStreamSynchronize(stream_) != cudaSuccess) return kErrDevice;
    const float n = (float)(batch * mbs_);
    stats[0] = s[0];
    stats[1] = s[1] / n;
    stats[2] = s[2] / n;
  }
  return cudaStreamSynchronize(stream_) == cudaSuccess ? kOK : kErrDevice;
}

int MvNet::headOutput(int batch, float* out) {
  if (batch < 1 || batch > B_) return kErrArg;
  forward(batch);
  if (cudaMemcpyAsync(out, head_, sizeof(float) * (size_t)batch * kHeadCh * h_ * w_, cudaMemcpyDeviceToHost, stream_) !=
      cudaSuccess)
    return kErrDevice;
  return cudaStreamSynchronize(stream_) == cudaSuccess ? kOK : kErrDevice;
}

int MvNet::propose(int16_t* cand) {
  forward(1);
  kPoolHead<<<(mbs_ + 127) / 128, 128, 0, stream_>>>(head_, 1, h_, w_, nullptr, nullptr, nullptr, cand_, 0.f);
  if (cudaMemcpyAsync(cand, cand_, sizeof(int16_t) * mbs_ * kTopK * 2, cudaMemcpyDeviceToHost, stream_) != cudaSuccess)
    return kErrDevice;
  return cudaStreamSynchronize(stream_) == cudaSuccess ? kOK : kErrDevice;
}

// ---------------------------------------------------------------------------
// The encoder's candidate source
// ---------------------------------------------------------------------------
void NetProposer::prepare(const uint8_t* src, const uint8_t* ref, int padW, int padH) {
  ok_ = false;
  if (!net_ || padW != net_->width() || padH != net_->height()) return;
  if (net_->setInput(0, src, ref, padW, nullptr)) return;
  cand_.resize((size_t)net_->macroblocks() * kTopK * 2);
  if (net_->propose(cand_.data())) return;
  mbCols_ = padW / 16;
  ok_ = true;
}

int NetProposer::candidates(int mbx, int mby, MotionVector* out, int max) const {
  if (!ok_) return 0;
  const int16_t* c = cand_.data() + (size_t)(mby * mbCols_ + mbx) * kTopK * 2;
  const int n = std::min(max, kTopK);
  for (int i = 0; i < n; i++) {
    out[i].x = (int16_t)(c[2 * i] * 4);  // quarter pels
    out[i].y = (int16_t)(c[2 * i + 1] * 4);
  }
  return n;
}

}  // namespace ebiv

// ---------------------------------------------------------------------------
// C-ABI (include/ebiv_mvnet.h)
// ---------------------------------------------------------------------------
#include "../../include/ebiv_mvnet.h"

namespace ebiv {
Encoder* encoderOf(ebiv_encoder* e);
const EncoderOptions* encoderOptionsOf(ebiv_encoder* e);
}  // namespace ebiv

struct ebiv_mvnet {
  ebiv::MvNet net;
  ebiv::NetProposer proposer{&net};
};

extern "C" {

int ebiv_mvnet_create(int max_batch, int pad_width, int pad_height, int max_pairs, uint64_t seed, ebiv_mvnet** out) {
  if (!out) return ebiv::kErrArg;
  *out = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n <= 0) return ebiv::kErrDevice;
  ebiv_mvnet* h = new (std::nothrow) ebiv_mvnet();
  if (!h) return ebiv::kErrDevice;
  const int st = h->net.init(max_batch, pad_width, pad_height, max_pairs, seed);
  if (st) {
    delete h;
    return st;
  }
  *out = h;
  return ebiv::kOK;
}

void ebiv_mvnet_destroy(ebiv_mvnet* n) { delete n; }

int ebiv_mvnet_param_count(void) { return ebiv::mvnet::kParams; }

int ebiv_mvnet_get_params(ebiv_mvnet* n, float* out) { return n && out ? n->net.getParams(out) : ebiv::kErrArg; }

int ebiv_mvnet_set_params(ebiv_mvnet* n, const float* in) { return n && in ? n->net.setParams(in) : ebiv::kErrArg; }

int ebiv_mvnet_exhaustive(ebiv_mvnet* n, const uint8_t* cur, const uint8_t* ref, int stride, int range, int16_t* mv,
                          int32_t* sad) {
  if (!n || !cur || !ref || !mv || stride < n->net.width()) return ebiv::kErrArg;
  return n->net.exhaustive(cur, ref, stride, range, mv, sad);
}

int ebiv_mvnet_add_pair(ebiv_mvnet* n, const uint8_t* cur, const uint8_t* ref, int stride, const int16_t* labels) {
  if (!n || !cur || !ref || !labels || stride < n->net.width()) return ebiv::kErrArg;
  return n->net.addPair(cur, ref, stride, labels);
}

int ebiv_mvnet_pairs(ebiv_mvnet* n) { return n ? n->net.pairs() : 0; }

int ebiv_mvnet_set_input(ebiv_mvnet* n, int slot, const uint8_t* cur, const uint8_t* ref, int stride,
                         const int16_t* labels) {
  if (!n || !cur || !ref || stride < n->net.width()) return ebiv::kErrArg;
  return n->net.setInput(slot, cur, ref, stride, labels);
}

int ebiv_mvnet_gather(ebiv_mvnet* n, const int32_t* idx, int batch) {
  return n && idx ? n->net.gather(idx, batch) : ebiv::kErrArg;
}

int ebiv_mvnet_gradients(ebiv_mvnet* n, int batch, float* grads, float* stats3) {
  return n ? n->net.gradients(batch, grads, stats3) : ebiv::kErrArg;
}

int ebiv_mvnet_train_step(ebiv_mvnet* n, int batch, float lr, float* stats3) {
  return n ? n->net.trainStep(batch, lr, stats3) : ebiv::kErrArg;
}

int ebiv_mvnet_head(ebiv_mvnet* n, int batch, float* out) { return n && out ? n->net.headOutput(batch, out) : ebiv::kErrArg; }

int ebiv_mvnet_propose(ebiv_mvnet* n, const uint8_t* cur, const uint8_t* ref, int stride, int16_t* cand) {
  if (!n || !cur || !ref || !cand || stride < n->net.width()) return ebiv::kErrArg;
  const int st = n->net.setInput(0, cur, ref, stride, nullptr);
  return st ? st : n->net.propose(cand);
}

int ebiv_encoder_set_mvnet(ebiv_encoder* e, ebiv_mvnet* n) {
  ebiv::Encoder* enc = ebiv::encoderOf(e);
  const ebiv::EncoderOptions* o = ebiv::encoderOptionsOf(e);
  if (!enc || !o || !n) return ebiv::kErrArg;
  const ebiv::Geometry g = ebiv::Geometry::of(o->width, o->height);
  if (g.padW() != n->net.width() || g.padH() != n->net.height()) return ebiv::kErrDimensions;
  enc->setProposer(&n->proposer);
  return ebiv::kOK;
}

}  // extern "C"
