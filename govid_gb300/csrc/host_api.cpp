// C-ABI over the host tools: encoder, demuxer, synthetic scenes.
#include <algorithm>
#include <atomic>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <memory>
#include <new>
#include <thread>

#include "../../include/ebiv_host.h"
#include "container.h"
#include "encoder.h"
#include "synth.h"

using namespace ebiv;


struct ebiv_encoder {
  std::unique_ptr<Encoder> enc;
  EncoderOptions opt;
  struct Proposer : MVProposer {
    std::vector<int16_t> mv;
    int frames = 0, mbs = 0, k = 0, mbCols = 1;
    int cur = -1;
    void prepare(const uint8_t*, const uint8_t*, int padW, int) override {
      cur++;
      mbCols = padW / kMB;
    }
    int candidates(int mbx, int mby, MotionVector* out, int max) const override {
      if (cur < 0 || cur >= frames) return 0;
      const int idx = mby * mbCols + mbx;
      if (idx < 0 || idx >= mbs) return 0;
      const int n = k < max ? k : max;
      const int16_t* p = mv.data() + ((size_t)cur * mbs + idx) * k * 2;
      for (int i = 0; i < n; i++) {
        out[i].x = p[2 * i];
        out[i].y = p[2 * i + 1];
      }
      return n;
    }
  } proposer;
};
namespace ebiv {
Encoder* encoderOf(ebiv_encoder* e) { return e ? e->enc.get() : nullptr; }
const EncoderOptions* encoderOptionsOf(ebiv_encoder* e) { return e ? &e->opt : nullptr; }
}  // namespace ebiv

struct ebiv_reader {
  Reader r;
};
struct ebiv_scene {
  std::unique_ptr<Scene> s;
};

namespace {
EncoderOptions toOptions(const ebiv_encoder_options* o) {
  EncoderOptions e;
  e.width = o->width;
  e.height = o->height;
  e.fpsNum = o->fps_num;
  e.fpsDen = o->fps_den;
  e.tileCols = o->tile_cols;
  e.tileRows = o->tile_rows;
  e.withTilesCols = o->with_tiles_cols;
  e.withTilesRows = o->with_tiles_rows;
  e.coded = o->coded != 0;
  e.qp = o->qp;
  if (e.qp < 0) e.qp = 0;
  if (e.qp > kMaxQP) e.qp = kMaxQP;
  e.gop = o->gop >= 1 ? o->gop : 1;
  e.autoTiles = o->auto_tiles;
  e.altRefWindow = o->altref_window >= 0 ? o->altref_window : 0;
  e.fastEncode = o->fast_encode != 0;
  e.threads = o->threads;
  e.search = (SearchMode)o->search;
  e.exhaustiveRange = o->exhaustive_range > 0 ? o->exhaustive_range : 16;
  e.proposedFallbackSAD = o->proposed_fallback_sad > 0 ? o->proposed_fallback_sad : 0;
  e.keepRecon = o->keep_recon != 0;
  return e;
}
SceneSpec toSpec(const int64_t* v) {
  SceneSpec s;
  s.width = (int)v[0];
  s.height = (int)v[1];
  s.seed = (uint64_t)v[2];
  s.sprites = (int)v[3];
  s.velMaxQ = (int)v[4];
  s.integerVel = v[5] != 0;
  s.panMaxQ = (int)v[6];
  s.flashPeriod = (int)v[7];
  s.flashStart = (int)v[8];
  s.flashLen = (int)v[9];
  s.flashAmp = (int)v[10];
  s.noiseY16 = (int)v[11];
  s.noiseC16 = (int)v[12];
  return s;
}
size_t packedBytes(int w, int h) { return (size_t)w * h + 2 * (size_t)((w + 1) / 2) * ((h + 1) / 2); }
void pack(const PackedImage& im, uint8_t* out) {
  std::memcpy(out, im.Y.data(), im.Y.size());
  std::memcpy(out + im.Y.size(), im.Cb.data(), im.Cb.size());
  std::memcpy(out + im.Y.size() + im.Cb.size(), im.Cr.data(), im.Cr.size());
}
void unpack(const uint8_t* in, int w, int h, PackedImage& im) {
  im.alloc(w, h);
  std::memcpy(im.Y.data(), in, im.Y.size());
  std::memcpy(im.Cb.data(), in + im.Y.size(), im.Cb.size());
  std::memcpy(im.Cr.data(), in + im.Y.size() + im.Cb.size(), im.Cr.size());
}
}  // namespace

extern "C" {

void ebiv_encoder_default_options(ebiv_encoder_options* o) {
  std::memset(o, 0, sizeof(*o));
  o->fps_num = 30;
  o->fps_den = 1;
  o->with_tiles_cols = -1;
  o->with_tiles_rows = -1;
  o->qp = 20;
  o->gop = 1;
  o->threads = 1;
  o->exhaustive_range = 16;
}

int ebiv_encoder_create(const ebiv_encoder_options* o, ebiv_encoder** out) {
  if (!o || !out) return kErrArg;
  ebiv_encoder* e = new (std::nothrow) ebiv_encoder();
  if (!e) return kErrArg;
  e->opt = toOptions(o);
  e->enc.reset(new Encoder(e->opt));
  if (e->enc->status() != kOK) {
    const int st = e->enc->status();
    delete e;
    return st;
  }
  *out = e;
  return kOK;
}

int ebiv_encoder_write_frame(ebiv_encoder* e, const uint8_t* packed, size_t n) {
  if (!e || !packed) return kErrArg;
  if (n != packedBytes(e->opt.width, e->opt.height)) return kErrDimensions;
  PackedImage im;
  unpack(packed, e->opt.width, e->opt.height, im);
  return e->enc->writeFrame(im);
}

int ebiv_encoder_close(ebiv_encoder* e) { return e ? e->enc->close() : kErrArg; }

int ebiv_encoder_output(ebiv_encoder* e, const uint8_t** data, size_t* n) {
  if (!e) return kErrArg;
  *data = e->enc->output().data();
  *n = e->enc->output().size();
  return kOK;
}

int ebiv_encoder_recon(ebiv_encoder* e, int index, uint8_t* packed, size_t cap) {
  if (!e) return kErrArg;
  const auto& r = e->enc->recons();
  if (index < 0 || index >= (int)r.size()) return kErrArg;
  if (cap < packedBytes(e->opt.width, e->opt.height)) return kErrArg;
  pack(r[(size_t)index], packed);
  return kOK;
}

int ebiv_encoder_recon_count(ebiv_encoder* e) { return e ? (int)e->enc->recons().size() : 0; }

uint64_t ebiv_encoder_sad_evaluations(ebiv_encoder* e) { return e ? e->enc->sadEvaluations() : 0; }

uint64_t ebiv_encoder_search_fallbacks(ebiv_encoder* e) { return e ? e->enc->searchFallbacks() : 0; }

double ebiv_encoder_search_seconds(ebiv_encoder* e) { return e ? e->enc->searchSeconds() : 0.0; }

double ebiv_encoder_propose_seconds(ebiv_encoder* e) { return e ? e->enc->proposeSeconds() : 0.0; }

int ebiv_encoder_set_candidates(ebiv_encoder* e, const int16_t* mv, int frames, int mbs, int k) {
  if (!e || !mv || frames < 0 || mbs <= 0 || k <= 0) return kErrArg;
  e->proposer.mv.assign(mv, mv + (size_t)frames * mbs * k * 2);
  e->proposer.frames = frames;
  e->proposer.mbs = mbs;
  e->proposer.k = k;
  e->proposer.cur = -1;
  e->enc->setProposer(&e->proposer);
  return kOK;
}

void ebiv_encoder_destroy(ebiv_encoder* e) { delete e; }

int ebiv_reader_open(const uint8_t* data, size_t n, ebiv_reader** out) {
  if (!out || (!data && n)) return kErrArg;
  ebiv_reader* r = new (std::nothrow) ebiv_reader();
  if (!r) return kErrArg;
  const int st = r->r.open(data, n);
  if (st != kOK) {
    delete r;
    return st;
  }
  *out = r;
  return kOK;
}

int ebiv_reader_info(ebiv_reader* r, int64_t* v) {
  if (!r) return kErrArg;
  const FileHeader& h = r->r.header();
  v[0] = h.width;
  v[1] = h.height;
  v[2] = h.fpsNum;
  v[3] = h.fpsDen;
  v[4] = r->r.frameCount();
  v[5] = h.tileCols;
  v[6] = h.tileRows;
  v[7] = r->r.rebuiltIndex() ? 1 : 0;
  return kOK;
}

int ebiv_reader_next_packet(ebiv_reader* r, const uint8_t** data, size_t* n, int64_t* ts, int* key) {
  if (!r) return kErrArg;
  bool k = false;
  const int st = r->r.nextPacket(data, n, ts, &k);
  if (key) *key = k ? 1 : 0;
  return st;
}

int ebiv_reader_packet(ebiv_reader* r, int index, const uint8_t** data, size_t* n, int* key) {
  if (!r) return kErrArg;
  const int st = r->r.packet(index, data, n);
  if (st == kOK && key) *key = r->r.index()[(size_t)index].keyframe ? 1 : 0;
  return st;
}

int ebiv_reader_seek(ebiv_reader* r, int64_t t, int64_t* landed) { return r ? r->r.seek(t, landed) : kErrArg; }
int64_t ebiv_reader_duration(ebiv_reader* r) { return r ? r->r.duration() : 0; }
int64_t ebiv_reader_frame_time(ebiv_reader* r, int64_t i) { return r ? r->r.header().frameTime(i) : 0; }
int64_t ebiv_reader_frame_index_at(ebiv_reader* r, int64_t t) { return r ? r->r.header().frameIndexAt(t) : 0; }
int ebiv_reader_close(ebiv_reader* r) {
  if (!r) return kErrArg;
  r->r.close();
  return kOK;
}
void ebiv_reader_destroy(ebiv_reader* r) { delete r; }

int ebiv_parse_frame_header(const uint8_t* pkt, size_t n, int32_t* info) {
  FrameHeader f;
  const int st = parseFrameHeader(pkt, n, &f);
  info[0] = f.type;
  info[1] = f.coding;
  info[2] = f.width;
  info[3] = f.height;
  info[4] = f.goldenOverride ? 1 : 0;
  info[5] = (int32_t)f.bodyOffset;
  return st;
}

int ebiv_synth_frame(int w, int h, int seed, uint8_t* packed, size_t cap) {
  if (w <= 0 || h <= 0 || cap < packedBytes(w, h)) return kErrArg;
  PackedImage im;
  synthFrame(im, w, h, seed);
  pack(im, packed);
  return kOK;
}

int ebiv_synth_pan(int w, int h, int seed, uint8_t* packed, size_t cap) {
  if (w <= 0 || h <= 0 || cap < packedBytes(w, h)) return kErrArg;
  PackedImage im;
  synthPan(im, w, h, seed);
  pack(im, packed);
  return kOK;
}

int ebiv_scene_create(const int64_t* spec, ebiv_scene** out) {
  if (!spec || !out || spec[0] <= 0 || spec[1] <= 0 || spec[0] > 65535 || spec[1] > 65535) return kErrArg;
  ebiv_scene* s = new (std::nothrow) ebiv_scene();
  if (!s) return kErrArg;
  s->s.reset(new Scene(toSpec(spec)));
  *out = s;
  return kOK;
}

int ebiv_scene_render(ebiv_scene* s, int frame, uint8_t* packed, size_t cap) {
  if (!s) return kErrArg;
  const SceneSpec& sp = s->s->spec();
  if (cap < packedBytes(sp.width, sp.height)) return kErrArg;
  PackedImage im;
  s->s->render(frame, im);
  pack(im, packed);
  return kOK;
}

void ebiv_scene_destroy(ebiv_scene* s) { delete s; }

namespace {

int copyOut(const std::vector<uint8_t>& v, uint8_t** out, size_t* n) {
  *n = v.size();
  *out = (uint8_t*)std::malloc(*n ? *n : 1);
  if (!*out) return kErrArg;
  std::memcpy(*out, v.data(), *n);
  return kOK;
}

// Runs fn(0..count-1) on up to `workers` threads.
void fanOut(int count, int workers, const std::function<void(int)>& fn) {
  std::atomic<int> next{0};
  auto loop = [&] {
    for (int i; (i = next.fetch_add(1)) < count;) fn(i);
  };
  std::vector<std::thread> ts;
  for (int k = 1; k < std::min(workers, count); k++) ts.emplace_back(loop);
  loop();
  for (auto& t : ts) t.join();
}

// The first frame of every GOP the serial encoder would close, from its own
// two rules (Encoder::writeFrame, after ebiv/encoder.go:189-227): a scene cut
// (luma SAD against the previous frame above 28 per pixel) ends a GOP of at
// least 8 pending frames, and a GOP ends when it holds `gop` frames.  The
// per-frame cut tests run in parallel; each worker renders its run of frames
// in order, so every frame is rendered about once.
std::vector<int> gopStarts(const Scene& scene, int frames, int gop, int workers) {
  std::vector<uint8_t> cut((size_t)frames, 0);
  const int runs = std::max(1, std::min(workers * 2, frames));
  fanOut(runs, workers, [&](int r) {
    const int a = (int)((int64_t)frames * r / runs), b = (int)((int64_t)frames * (r + 1) / runs);
    PackedImage prev, cur;
    if (a > 0) scene.render(a - 1, prev);
    for (int i = a; i < b; i++) {
      scene.render(i, cur);
      if (i > 0) {
        int64_t sad = 0;
        for (size_t k = 0; k < cur.Y.size(); k++) sad += std::abs((int32_t)cur.Y[k] - (int32_t)prev.Y[k]);
        cut[i] = sad > (int64_t)cur.W * cur.H * 28;
      }
      std::swap(prev, cur);
    }
  });
  std::vector<int> starts{0};
  int pending = 0;
  for (int i = 0; i < frames; i++) {
    if (i > 0 && cut[i] && pending >= 8) {
      starts.push_back(i);
      pending = 0;
    }
    if (++pending >= gop) {
      if (i + 1 < frames) starts.push_back(i + 1);
      pending = 0;
    }
  }
  return starts;
}

// The frame records of an encoder's container: the bytes between the file
// header and the index.
bool frameRecords(const std::vector<uint8_t>& c, const uint8_t** p, size_t* n) {
  if (c.size() < (size_t)kFileHeaderSize + kFooterSize) return false;
  uint64_t idx = 0;
  for (int k = 7; k >= 0; k--) idx = idx << 8 | c[c.size() - kFooterSize + k];
  if (idx < (uint64_t)kFileHeaderSize || idx > c.size()) return false;
  *p = c.data() + kFileHeaderSize;
  *n = (size_t)idx - kFileHeaderSize;
  return true;
}

}  // namespace

// GOPs are independent in the encoder (each key frame starts from empty
// reference and table state, Encoder::flushGOP), so a clip is encoded GOP by
// GOP on concurrent encoders and the frame records are joined into one
// container: the output equals the serial encoder's byte for byte.  Each GOP
// encoder fans its tiles out over its share of the threads.
int ebiv_encode_scene(const int64_t* spec, int frames, const ebiv_encoder_options* o, uint8_t** out, size_t* n) {
  if (!spec || !o || !out || !n || frames < 0) return kErrArg;
  Scene scene(toSpec(spec));
  const EncoderOptions opt = toOptions(o);
  const int threads = std::max(1, opt.threads);
  const bool gopParallel = opt.coded && !opt.keepRecon && opt.search != SearchMode::Proposed && frames > 1 &&
                           threads > 1;
  if (!gopParallel) {
    Encoder enc(opt);
    if (enc.status() != kOK) return enc.status();
    PackedImage im;
    for (int i = 0; i < frames; i++) {
      scene.render(i, im);
      const int st = enc.writeFrame(im);
      if (st != kOK) return st;
    }
    const int st = enc.close();
    if (st != kOK) return st;
    return copyOut(enc.output(), out, n);
  }
  {
    Encoder probe(opt);
    if (probe.status() != kOK) return probe.status();
  }
  const std::vector<int> starts = gopStarts(scene, frames, opt.gop, threads);
  const int gops = (int)starts.size();
  const int cols = opt.withTilesCols >= 0 ? opt.withTilesCols : opt.tileCols;
  const int rows = opt.withTilesRows >= 0 ? opt.withTilesRows : opt.tileRows;
  const int tiles = std::max(1, std::max(cols, 1) * std::max(rows, 1));
  const int perGop = std::max(1, std::min(threads, tiles));
  const int conc = std::max(1, std::min(gops, threads / perGop));
  EncoderOptions gopOpt = opt;
  gopOpt.threads = perGop;
  std::vector<std::vector<uint8_t>> parts((size_t)gops);
  std::vector<int> status((size_t)gops, kOK);
  fanOut(gops, conc, [&](int g) {
    const int a = starts[g], b = g + 1 < gops ? starts[g + 1] : frames;
    Encoder enc(gopOpt);
    PackedImage im;
    int st = enc.status();
    for (int i = a; i < b && st == kOK; i++) {
      scene.render(i, im);
      st = enc.writeFrame(im);
    }
    if (st == kOK) st = enc.close();
    status[g] = st;
    if (st == kOK) parts[g] = enc.output();
  });
  for (int s : status)
    if (s != kOK) return s;
  // Join: the first part's file header, every part's frame records, then a
  // new index (offsets shifted) and footer (ebiv/writer.go:92-119).
  std::vector<uint8_t> c(parts[0].begin(), parts[0].begin() + kFileHeaderSize);
  for (const auto& part : parts) {
    const uint8_t* p;
    size_t len;
    if (!frameRecords(part, &p, &len)) return kErrConfig;
    c.insert(c.end(), p, p + len);
  }
  const uint64_t indexOffset = c.size();
  std::vector<uint8_t> idx;
  uint32_t count = 0;
  for (size_t off = kFileHeaderSize; off + kFrameRecordSize <= indexOffset; count++) {
    const uint32_t flags = (uint32_t)c[off + 2] | (uint32_t)c[off + 3] << 8;
    const uint32_t size = (uint32_t)c[off + 4] | (uint32_t)c[off + 5] << 8 | (uint32_t)c[off + 6] << 16 |
                          (uint32_t)c[off + 7] << 24;
    uint8_t e[kIndexEntrySize];
    wr64(e, off);
    wr32(e + 8, size);
    wr32(e + 12, flags & 1u);
    idx.insert(idx.end(), e, e + kIndexEntrySize);
    off += kFrameRecordSize + size;
  }
  c.insert(c.end(), idx.begin(), idx.end());
  uint8_t footer[kFooterSize];
  wr64(footer, indexOffset);
  wr32(footer + 8, count);
  wr32(footer + 12, crc32IEEE(idx.data(), idx.size()));
  footer[16] = 'E';
  footer[17] = 'B';
  footer[18] = 'I';
  footer[19] = 'X';
  c.insert(c.end(), footer, footer + kFooterSize);
  return copyOut(c, out, n);
}

void ebiv_free(void* p) { std::free(p); }

int ebiv_encode_block(int32_t* levels, int n, int plane, int tx_idx, uint8_t* stream, size_t cap, size_t* len,
                      uint32_t* freqs, uint8_t* used) {
  std::vector<uint8_t> st, u;
  std::vector<uint32_t> f;
  const int r = encodeBlockStream(levels, n, plane, tx_idx, &st, &f, &u);
  if (r) return r;
  if (st.size() > cap) return kErrArg;
  std::memcpy(stream, st.data(), st.size());
  *len = st.size();
  std::memcpy(freqs, f.data(), f.size() * 4);
  std::memcpy(used, u.data(), u.size());
  return kOK;
}

int ebiv_encode_key_from_levels(int w, int h, int qp, int mode, const int32_t* levels, size_t nlevels, uint8_t** out,
                                size_t* n) {
  if (!levels || !out || !n) return kErrArg;
  std::vector<uint8_t> pkt;
  if (int st = encodeKeyFromLevels(w, h, qp, mode, levels, nlevels, &pkt)) return st;
  return copyOut(pkt, out, n);
}

int ebiv_encode_tokens(const uint16_t* pairs, int count, uint8_t* stream, size_t cap, size_t* len, uint32_t* freqs,
                       uint8_t* used) {
  std::vector<uint8_t> st, u;
  std::vector<uint32_t> f;
  const int r = encodeTokenStream(pairs, count, &st, &f, &u);
  if (r) return r;
  if (st.size() > cap) return kErrArg;
  std::memcpy(stream, st.data(), st.size());
  *len = st.size();
  std::memcpy(freqs, f.data(), f.size() * 4);
  std::memcpy(used, u.data(), u.size());
  return kOK;
}

}  // extern "C"
