// Seeded synthetic 4:2:0 content for the decode workloads and for the
// reference's own test generators.  Everything is integer arithmetic on a
// counter-based generator, so a frame depends only on (spec, seed, index) and
// is identical on every host.
#pragma once

#include <cstdint>
#include <vector>

#include "encoder.h"

namespace ebiv {

// The reference test harness's synthFrame / synthPan (ebiv/harness_test.go:105-171).
void synthFrame(PackedImage& img, int w, int h, int seed);
void synthPan(PackedImage& img, int w, int h, int seed);

// Sprite scene: a horizontal+vertical luma gradient (0..255), textured
// rectangular sprites (32-96 px sides, uniform 8-bit texture low-passed by a
// 5x5 box filter) translating at per-sprite velocities, optional global pan of
// a textured background layer, optional periodic full-frame luma flash, plus
// approximately Gaussian noise (sum of twelve uniforms) clamped to [0,255];
// chroma is a smooth gradient plus noise.
struct SceneSpec {
  int width = 640, height = 360;
  uint64_t seed = 1;
  int sprites = 6;
  int velMaxQ = 16;       // max |velocity| per axis in quarter pixels per frame
  bool integerVel = true; // round velocities to whole pixels
  int panMaxQ = 0;        // max |global pan| per axis, quarter pixels per frame
  int flashPeriod = 0;    // frames between flash starts (0 = none)
  int flashStart = 30;    // first flash frame within each period
  int flashLen = 3;       // frames per flash
  int flashAmp = 40;      // luma added during a flash
  int noiseY16 = 32;      // luma noise sigma in 1/16 units (32 = 2.0)
  int noiseC16 = 16;      // chroma noise sigma in 1/16 units
};

class Scene {
 public:
  explicit Scene(const SceneSpec& s);
  void render(int frame, PackedImage& out) const;
  const SceneSpec& spec() const { return spec_; }

 private:
  struct Sprite {
    int w, h;
    int64_t x0q, y0q;  // start position, quarter pixels
    int vxq, vyq;      // velocity, quarter pixels/frame
    std::vector<uint8_t> tex;
  };
  SceneSpec spec_;
  std::vector<Sprite> sprites_;
  std::vector<uint8_t> bgTex_;  // 256x256 tileable texture for the panned layer
  int panXq_ = 0, panYq_ = 0;
};

}  // namespace ebiv
