// The encoder's block analysis on the GPU: forwardDCT and satd
// (ebiv/transform.go:44-119) over a batch of n x n residual blocks, the inner
// loops of the encoder's rate-distortion search (every intra-mode trial and
// every inter candidate transforms or Hadamard-scores its residual).
//
// One warp per block.  forwardDCT: lane l computes columns pass entries
// tmp[k][j] = round(sum_i C[k][i] * src[i][j]) for k*n+j = l, l+32, ...
// (int64 accumulation, rounding shift by 13, the int32 narrowing of the
// reference), then row pass dst[k][m] = round(sum_j C[m][j] * tmp[k][j]);
// the block, the intermediate and the DCT basis sit in shared memory.  satd:
// the in-place Walsh-Hadamard butterflies of the rows, then the columns
// (int32 arithmetic, wrapping as Go's does), and the sum of absolute values
// (int64) as a warp reduction.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <new>

#include "../../include/ebivgpu.h"
#include "ebiv_format.h"

namespace ebiv {
namespace dev {

constexpr int kAnaWarps = 4;
constexpr int kDCTScaleBits = 13;  // the DCT basis is scaled by 2^13 (ebiv/transform.go:15-40)

__global__ void __launch_bounds__(32 * kAnaWarps) kAnalyze(const int32_t* __restrict__ src, int n, int count,
                                                           const int32_t* __restrict__ basis, int32_t* __restrict__ dst,
                                                           int64_t* __restrict__ satdOut) {
  __shared__ int32_t sC[256];
  __shared__ int32_t sBlk[kAnaWarps][256];
  __shared__ int32_t sTmp[kAnaWarps][256];
  const int nn = n * n;
  for (int i = threadIdx.x; i < nn; i += blockDim.x) sC[i] = basis[i];
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int b = blockIdx.x * kAnaWarps + warp;
  if (b >= count) return;
  const int32_t* s = src + (size_t)b * nn;
  int32_t* blk = sBlk[warp];
  int32_t* tmp = sTmp[warp];
  for (int i = lane; i < nn; i += 32) blk[i] = s[i];
  __syncwarp();
  const int64_t round = 1LL << (kDCTScaleBits - 1);
  if (dst) {
    for (int o = lane; o < nn; o += 32) {
      const int k = o / n, j = o - k * n;
      int64_t acc = 0;
      for (int i = 0; i < n; i++) acc += (int64_t)sC[k * n + i] * (int64_t)blk[i * n + j];
      tmp[o] = (int32_t)((acc + round) >> kDCTScaleBits);
    }
    __syncwarp();
    int32_t* d = dst + (size_t)b * nn;
    for (int o = lane; o < nn; o += 32) {
      const int k = o / n, m = o - k * n;
      int64_t acc = 0;
      for (int j = 0; j < n; j++) acc += (int64_t)sC[m * n + j] * (int64_t)tmp[k * n + j];
      d[o] = (int32_t)((acc + round) >> kDCTScaleBits);
    }
    __syncwarp();
  }
  if (satdOut) {
    // Rows, then columns: one butterfly stage at a time over the whole
    // block, each lane taking pairs (a, a + span) of the stage.
    for (int pass = 0; pass < 2; pass++) {
      for (int span = 1; span < n; span <<= 1) {
        for (int q = lane; q < nn / 2; q += 32) {
          // q-th pair of the stage: line (row or column) q / (n/2), pair q % (n/2) within it
          const int line = q / (n / 2), p = q - line * (n / 2);
          const int grp = p / span, off = p - grp * span;
          const int a = grp * 2 * span + off, c = a + span;  // positions within the line
          const int ia = pass == 0 ? line * n + a : a * n + line;
          const int ic = pass == 0 ? line * n + c : c * n + line;
          const int32_t x = blk[ia], y = blk[ic];
          blk[ia] = (int32_t)((uint32_t)x + (uint32_t)y);
          blk[ic] = (int32_t)((uint32_t)x - (uint32_t)y);
        }
        __syncwarp();
      }
    }
    int64_t sum = 0;
    for (int i = lane; i < nn; i += 32) {
      const int32_t v = blk[i];
      sum += v < 0 ? -(int64_t)v : (int64_t)v;
    }
    for (int o = 16; o; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
    if (lane == 0) satdOut[b] = sum;
  }
}

}  // namespace dev
}  // namespace ebiv

using namespace ebiv;

struct ebivgpu_analysis {
  int32_t* dSrc = nullptr;
  int32_t* dDst = nullptr;
  int64_t* dSatd = nullptr;
  int32_t* dBasis = nullptr;  // the three DCT matrices, 256 words each
  size_t cap = 0;             // blocks of 256 words the buffers hold
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  ~ebivgpu_analysis() {
    if (stream) cudaStreamSynchronize(stream);
    cudaFree(dSrc);
    cudaFree(dDst);
    cudaFree(dSatd);
    cudaFree(dBasis);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    if (stream) cudaStreamDestroy(stream);
  }
};

extern "C" {

int ebivgpu_analysis_create(ebivgpu_analysis** out) {
  if (!out) return kErrArg;
  ebivgpu_analysis* a = new (std::nothrow) ebivgpu_analysis();
  if (!a) return kErrArg;
  const CodingTables& t = codingTables();
  int32_t basis[3 * 256];
  std::memset(basis, 0, sizeof(basis));
  for (int k = 0; k < 3; k++) std::memcpy(basis + 256 * k, t.dct[k], sizeof(int32_t) * kLumaTx[k] * kLumaTx[k]);
  if (cudaStreamCreateWithFlags(&a->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&a->ev0) != cudaSuccess || cudaEventCreate(&a->ev1) != cudaSuccess ||
      cudaMalloc(&a->dBasis, sizeof(basis)) != cudaSuccess ||
      cudaMemcpy(a->dBasis, basis, sizeof(basis), cudaMemcpyHostToDevice) != cudaSuccess) {
    delete a;
    return kErrDevice;
  }
  *out = a;
  return kOK;
}

void ebivgpu_analysis_destroy(ebivgpu_analysis* a) { delete a; }

int ebivgpu_fdct_satd(ebivgpu_analysis* a, const int32_t* residuals, int n, int count, int32_t* coeffs,
                      int64_t* satd, double* kernel_ms) {
  if (!a || (!residuals && count) || count < 0 || (n != 4 && n != 8 && n != 16)) return kErrArg;
  if (count == 0) return kOK;
  const size_t nn = (size_t)n * n;
  if ((size_t)count > a->cap) {
    cudaFree(a->dSrc);
    cudaFree(a->dDst);
    cudaFree(a->dSatd);
    a->dSrc = a->dDst = nullptr;
    a->dSatd = nullptr;
    a->cap = 0;
    if (cudaMalloc(&a->dSrc, (size_t)count * 256 * 4) != cudaSuccess ||
        cudaMalloc(&a->dDst, (size_t)count * 256 * 4) != cudaSuccess ||
        cudaMalloc(&a->dSatd, (size_t)count * 8) != cudaSuccess)
      return kErrDevice;
    a->cap = (size_t)count;
  }
  const int k = n == 4 ? 0 : (n == 8 ? 1 : 2);
  if (cudaMemcpyAsync(a->dSrc, residuals, (size_t)count * nn * 4, cudaMemcpyHostToDevice, a->stream) != cudaSuccess)
    return kErrDevice;
  cudaEventRecord(a->ev0, a->stream);
  dev::kAnalyze<<<(count + dev::kAnaWarps - 1) / dev::kAnaWarps, 32 * dev::kAnaWarps, 0, a->stream>>>(
      a->dSrc, n, count, a->dBasis + 256 * k, coeffs ? a->dDst : nullptr, satd ? a->dSatd : nullptr);
  if (cudaGetLastError() != cudaSuccess) return kErrDevice;
  cudaEventRecord(a->ev1, a->stream);
  if ((coeffs && cudaMemcpyAsync(coeffs, a->dDst, (size_t)count * nn * 4, cudaMemcpyDeviceToHost, a->stream)) ||
      (satd && cudaMemcpyAsync(satd, a->dSatd, (size_t)count * 8, cudaMemcpyDeviceToHost, a->stream)) ||
      cudaStreamSynchronize(a->stream) != cudaSuccess)
    return kErrDevice;
  if (kernel_ms) {
    float ms = 0;
    cudaEventElapsedTime(&ms, a->ev0, a->ev1);
    *kernel_ms = ms;
  }
  return kOK;
}

}  // extern "C"
