#include "synth.h"

#include <algorithm>

namespace ebiv {

namespace {
// splitmix64: a counter-based 64-bit mixer.
inline uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
struct Rng {
  uint64_t s;
  explicit Rng(uint64_t seed) : s(seed) {}
  uint64_t next() { return mix64(s++); }
  int uniform(int lo, int hi) { return lo + (int)(next() % (uint64_t)(hi - lo + 1)); }
};
inline uint8_t clamp8(int v) { return (uint8_t)(v < 0 ? 0 : (v > 255 ? 255 : v)); }

// Approximately N(0, sigma^2) integer noise: twelve uniform bytes sum to a
// value with mean 1530 and standard deviation ~256.
inline int noiseSample(uint64_t a, uint64_t b, int sigma16) {
  int sum = 0;
  for (int k = 0; k < 8; k++) sum += (int)((a >> (8 * k)) & 0xff);
  for (int k = 0; k < 4; k++) sum += (int)((b >> (8 * k)) & 0xff);
  const int d = (sum - 1530) * sigma16;  // units of 1/16 * 256
  return d >= 0 ? (d + 2048) / 4096 : -((-d + 2048) / 4096);
}

// Bilinear sample of an 8-bit texture at quarter-pel position (xq, yq).
inline int sampleQ(const uint8_t* t, int w, int h, int64_t xq, int64_t yq, bool wrap) {
  int64_t xi = xq >> 2, yi = yq >> 2;
  const int fx = (int)(xq & 3), fy = (int)(yq & 3);
  auto at = [&](int64_t x, int64_t y) -> int {
    if (wrap) {
      x = ((x % w) + w) % w;
      y = ((y % h) + h) % h;
    } else {
      x = std::min<int64_t>(std::max<int64_t>(x, 0), w - 1);
      y = std::min<int64_t>(std::max<int64_t>(y, 0), h - 1);
    }
    return t[(size_t)y * w + x];
  };
  const int a = at(xi, yi), b = at(xi + 1, yi), c = at(xi, yi + 1), d = at(xi + 1, yi + 1);
  return ((4 - fx) * (4 - fy) * a + fx * (4 - fy) * b + (4 - fx) * fy * c + fx * fy * d + 8) >> 4;
}

// A position bouncing between 0 and span (quarter pixels).
inline int64_t bounce(int64_t p, int64_t span) {
  if (span <= 0) return 0;
  const int64_t period = 2 * span;
  int64_t m = ((p % period) + period) % period;
  return m <= span ? m : period - m;
}
}  // namespace

void synthFrame(PackedImage& img, int w, int h, int seed) {
  img.alloc(w, h);
  for (int y = 0; y < h; y++)
    for (int x = 0; x < w; x++) {
      int v = (x * 3 + y * 5 + seed * 7) & 0xff;
      if (x + y > (w + h) / 2) v = 255 - v;
      if (((x / 4 + y / 4) & 1) == 0) v ^= 0x33;
      img.Y[(size_t)y * w + x] = (uint8_t)v;
    }
  for (int y = 0; y < img.CH; y++)
    for (int x = 0; x < img.CW; x++) {
      img.Cb[(size_t)y * img.CW + x] = (uint8_t)((x * 11 + y * 2 + seed * 3) & 0xff);
      img.Cr[(size_t)y * img.CW + x] = (uint8_t)((255 - x * 2 - y * 13 - seed * 5) & 0xff);
    }
}

void synthPan(PackedImage& img, int w, int h, int seed) {
  img.alloc(w, h);
  const int off = 2 * seed;
  for (int y = 0; y < h; y++)
    for (int x = 0; x < w; x++) {
      const int xx = x + off, yy = y + off;
      int v = (xx * 3 + yy * 2) & 0xff;
      if (((xx / 6 + yy / 6) & 1) == 0) v ^= 0x40;
      img.Y[(size_t)y * w + x] = (uint8_t)v;
    }
  const int coff = seed;
  for (int y = 0; y < img.CH; y++)
    for (int x = 0; x < img.CW; x++) {
      const int xx = x + coff, yy = y + coff;
      img.Cb[(size_t)y * img.CW + x] = (uint8_t)((xx * 5 + yy * 3) & 0xff);
      img.Cr[(size_t)y * img.CW + x] = (uint8_t)((200 - xx * 2 - yy * 4) & 0xff);
    }
}

Scene::Scene(const SceneSpec& s) : spec_(s) {
  Rng rng(mix64(s.seed * 0x2545F4914F6CDD1Dull + 17));
  for (int i = 0; i < s.sprites; i++) {
    Sprite sp;
    sp.w = rng.uniform(32, 96);
    sp.h = rng.uniform(32, 96);
    // Uniform texture on a (w+4)x(h+4) canvas, low-passed by a 5x5 box.
    const int cw = sp.w + 4, ch = sp.h + 4;
    std::vector<uint8_t> raw((size_t)cw * ch);
    for (auto& v : raw) v = (uint8_t)(rng.next() & 0xff);
    sp.tex.resize((size_t)sp.w * sp.h);
    for (int y = 0; y < sp.h; y++)
      for (int x = 0; x < sp.w; x++) {
        int sum = 0;
        for (int dy = 0; dy < 5; dy++)
          for (int dx = 0; dx < 5; dx++) sum += raw[(size_t)(y + dy) * cw + x + dx];
        sp.tex[(size_t)y * sp.w + x] = (uint8_t)((sum + 12) / 25);
      }
    sp.x0q = (int64_t)rng.uniform(0, std::max(0, s.width - sp.w)) * 4;
    sp.y0q = (int64_t)rng.uniform(0, std::max(0, s.height - sp.h)) * 4;
    sp.vxq = rng.uniform(-s.velMaxQ, s.velMaxQ);
    sp.vyq = rng.uniform(-s.velMaxQ, s.velMaxQ);
    if (s.integerVel) {
      sp.vxq = (sp.vxq / 4) * 4;
      sp.vyq = (sp.vyq / 4) * 4;
    }
    sprites_.push_back(std::move(sp));
  }
  if (s.panMaxQ > 0) {
    panXq_ = rng.uniform(-s.panMaxQ, s.panMaxQ);
    panYq_ = rng.uniform(-s.panMaxQ, s.panMaxQ);
    std::vector<uint8_t> raw(256 * 256);
    for (auto& v : raw) v = (uint8_t)(rng.next() & 0xff);
    bgTex_.resize(256 * 256);
    for (int y = 0; y < 256; y++)
      for (int x = 0; x < 256; x++) {
        int sum = 0;
        for (int dy = -3; dy <= 3; dy++)
          for (int dx = -3; dx <= 3; dx++) sum += raw[(size_t)((y + dy) & 255) * 256 + ((x + dx) & 255)];
        bgTex_[(size_t)y * 256 + x] = (uint8_t)((sum + 24) / 49);
      }
  }
}

void Scene::render(int t, PackedImage& out) const {
  const SceneSpec& s = spec_;
  const int W = s.width, H = s.height;
  out.alloc(W, H);
  const int64_t wx = (int64_t)std::max(1, W - 1), hy = (int64_t)std::max(1, H - 1);
  std::vector<int16_t> luma((size_t)W * H);
  for (int y = 0; y < H; y++)
    for (int x = 0; x < W; x++)
      luma[(size_t)y * W + x] = (int16_t)((255 * ((int64_t)x * hy + (int64_t)y * wx)) / (2 * wx * hy));
  if (!bgTex_.empty()) {
    const int64_t px = (int64_t)panXq_ * t, py = (int64_t)panYq_ * t;
    for (int y = 0; y < H; y++)
      for (int x = 0; x < W; x++) {
        const int v = sampleQ(bgTex_.data(), 256, 256, (int64_t)x * 4 + px, (int64_t)y * 4 + py, true);
        int16_t& l = luma[(size_t)y * W + x];
        l = (int16_t)((l + v) / 2);
      }
  }
  for (const Sprite& sp : sprites_) {
    const int64_t spanX = (int64_t)std::max(0, W - sp.w) * 4, spanY = (int64_t)std::max(0, H - sp.h) * 4;
    const int64_t pxq = bounce(sp.x0q + (int64_t)sp.vxq * t, spanX);
    const int64_t pyq = bounce(sp.y0q + (int64_t)sp.vyq * t, spanY);
    const int64_t ox = pxq >> 2, oy = pyq >> 2;
    const int fx = (int)(pxq & 3), fy = (int)(pyq & 3);
    for (int y = 0; y < sp.h; y++) {
      const int64_t Y = oy + y;
      if (Y < 0 || Y >= H) continue;
      for (int x = 0; x < sp.w; x++) {
        const int64_t X = ox + x;
        if (X < 0 || X >= W) continue;
        // Sample the texture shifted back by the sub-pixel fraction.
        const int v = (fx | fy) ? sampleQ(sp.tex.data(), sp.w, sp.h, (int64_t)x * 4 - fx, (int64_t)y * 4 - fy, false)
                                : sp.tex[(size_t)y * sp.w + x];
        luma[(size_t)Y * W + X] = (int16_t)v;
      }
    }
  }
  int flash = 0;
  if (s.flashPeriod > 0) {
    const int ph = t % s.flashPeriod;
    if (ph >= s.flashStart && ph < s.flashStart + s.flashLen) flash = s.flashAmp;
  }
  const uint64_t base = mix64(s.seed ^ ((uint64_t)t * 0x9E3779B97F4A7C15ull));
  for (int y = 0; y < H; y++)
    for (int x = 0; x < W; x++) {
      const uint64_t k = base + ((uint64_t)y * W + x) * 2;
      const int n = s.noiseY16 ? noiseSample(mix64(k), mix64(k + 1), s.noiseY16) : 0;
      out.Y[(size_t)y * W + x] = clamp8(luma[(size_t)y * W + x] + flash + n);
    }
  const int CW = out.CW, CH = out.CH;
  const uint64_t cbase = mix64(base ^ 0xC0FFEEull);
  for (int y = 0; y < CH; y++)
    for (int x = 0; x < CW; x++) {
      const int cb = 96 + (64 * x) / std::max(1, CW) + (16 * y) / std::max(1, CH);
      const int cr = 160 - (48 * y) / std::max(1, CH) + (16 * x) / std::max(1, CW);
      const uint64_t k = cbase + ((uint64_t)y * CW + x) * 4;
      const int n1 = s.noiseC16 ? noiseSample(mix64(k), mix64(k + 1), s.noiseC16) : 0;
      const int n2 = s.noiseC16 ? noiseSample(mix64(k + 2), mix64(k + 3), s.noiseC16) : 0;
      out.Cb[(size_t)y * CW + x] = clamp8(cb + n1);
      out.Cr[(size_t)y * CW + x] = clamp8(cr + n2);
    }
}

}  // namespace ebiv
