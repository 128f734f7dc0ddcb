// YCbCr 4:2:0 -> RGBA, BT.601 fixed point (convertYCbCr420ToRGBA,
// frame.go:8-67; identical to Go's color.YCbCrToRGB).  One thread per pair
// of horizontally adjacent pixels, which share one chroma sample; the 8-byte
// output is written as one aligned store when the row allows it.
#include <cuda_runtime.h>

#include <cstdint>

namespace ebiv {
namespace dev {

__device__ __forceinline__ uint32_t rgbaPixel(int yv, int cb1, int cr1) {
  const int32_t yy1 = yv * 0x10101;
  int32_t r = yy1 + 91881 * cr1;
  int32_t g = yy1 - 22554 * cb1 - 46802 * cr1;
  int32_t b = yy1 + 116130 * cb1;
  r = r < 0 ? 0 : (r > 0xff0000 ? 0xff0000 : r);
  g = g < 0 ? 0 : (g > 0xff0000 ? 0xff0000 : g);
  b = b < 0 ? 0 : (b > 0xff0000 ? 0xff0000 : b);
  return (uint32_t)(r >> 16) | ((uint32_t)(g >> 16) << 8) | ((uint32_t)(b >> 16) << 16) | 0xff000000u;
}

__global__ void kRGBA(const uint8_t* __restrict__ Y, const uint8_t* __restrict__ Cb, const uint8_t* __restrict__ Cr,
                      int ys, int cs, int w, int h, uint8_t* __restrict__ dst) {
  const int cw = (w + 1) / 2;
  const int pair = blockIdx.x * blockDim.x + threadIdx.x;
  const int row = blockIdx.y;
  if (pair >= cw || row >= h) return;
  const int col = pair * 2;
  const int cb1 = (int)Cb[(size_t)(row / 2) * cs + pair] - 128;
  const int cr1 = (int)Cr[(size_t)(row / 2) * cs + pair] - 128;
  const uint8_t* yr = Y + (size_t)row * ys;
  uint32_t* o = reinterpret_cast<uint32_t*>(dst + ((size_t)row * w + col) * 4);
  o[0] = rgbaPixel(yr[col], cb1, cr1);
  if (col + 1 < w) o[1] = rgbaPixel(yr[col + 1], cb1, cr1);
}

}  // namespace dev

void launchRGBA(const uint8_t* y, const uint8_t* cb, const uint8_t* cr, int ys, int cs, int w, int h, uint8_t* dst,
                cudaStream_t s) {
  const int cw = (w + 1) / 2;
  dim3 grid((cw + 127) / 128, h);
  dev::kRGBA<<<grid, 128, 0, s>>>(y, cb, cr, ys, cs, w, h, dst);
}

}  // namespace ebiv
