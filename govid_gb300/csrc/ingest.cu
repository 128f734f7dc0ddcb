// Container ingest on the GPU: the EBIV demuxer's index and seek
// (ebiv/reader.go:32-258, ebiv/format.go:186-328) run on the device over a
// container held in pinned, device-mapped host memory, which the GPU reads
// in place (no copy into HBM).  A batch stream then decodes straight from
// the same bytes: planning reads them on the host, the kernels on the
// device, and no packet is staged or copied per frame.
//
//   kIndexFooter  readIndex (ebiv/reader.go:65-124): footer magic and
//                 bounds, the CRC-32 (IEEE) of the index table, every entry
//                 validated, the first a key frame.  The CRC runs over 256
//                 chunks in parallel; the chunk CRCs are joined with the
//                 GF(2)-linear map that advances a CRC register over a run of
//                 zero bytes (a 32x32 bit matrix built by 32 threads).
//   kScanFrames   scanFrames (ebiv/reader.go:126-160) when the footer does
//                 not validate: the frame records walked in order (each
//                 record's size gives the next), one thread.
//   kSeek         Seek (ebiv/reader.go:222-238): frameIndexAt
//                 (ebiv/format.go:263-275), clamped to the last frame, then
//                 the last key frame at or before it (a block-wide max).
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <new>
#include <vector>

#include "../../include/ebivgpu.h"
#include "ebiv_format.h"
#include "engine.h"

struct ebivgpu_batch;  // batch.cu
namespace ebiv {
Engine* batchEngine(ebivgpu_batch* b);
}

namespace ebiv {
namespace dev {

constexpr uint32_t kCrcPoly = 0xEDB88320u;  // IEEE, reflected
constexpr int kIngestThreads = 256;

struct IndexOut {
  uint64_t* off;   // payload offset (record offset + 8)
  uint32_t* size;  // payload size
  uint8_t* key;
  int32_t* count;  // frames, or -1 when the index does not validate
  int32_t cap;     // entries the arrays hold
};

__device__ __forceinline__ uint32_t rd32(const uint8_t* p) {
  return (uint32_t)p[0] | (uint32_t)p[1] << 8 | (uint32_t)p[2] << 16 | (uint32_t)p[3] << 24;
}
__device__ __forceinline__ uint64_t rd64(const uint8_t* p) { return (uint64_t)rd32(p) | (uint64_t)rd32(p + 4) << 32; }
__device__ __forceinline__ uint32_t crcByte(const uint32_t* T, uint32_t r, uint32_t b) {
  return T[(r ^ b) & 0xFFu] ^ (r >> 8);
}

__global__ void __launch_bounds__(kIngestThreads) kIndexFooter(const uint8_t* c, uint64_t n, IndexOut out) {
  __shared__ uint32_t T[256];
  __shared__ uint32_t part[kIngestThreads];
  __shared__ uint32_t M[32];  // M[k]: the register 1 << k advanced over `chunk` zero bytes
  __shared__ int ok;
  __shared__ uint64_t sOff;
  __shared__ uint32_t sCount, sWant;
  const int tid = threadIdx.x;
  {  // the byte table of the reflected CRC
    uint32_t r = (uint32_t)tid;
    for (int k = 0; k < 8; k++) r = (r & 1) ? kCrcPoly ^ (r >> 1) : r >> 1;
    T[tid] = r;
  }
  if (tid == 0) {
    ok = 0;
    if (n >= kFileHeaderSize + kFooterSize && c[n - 4] == 'E' && c[n - 3] == 'B' && c[n - 2] == 'I' &&
        c[n - 1] == 'X') {
      const uint8_t* f = c + n - kFooterSize;
      const uint64_t off = rd64(f);
      const uint32_t count = rd32(f + 8);
      const uint64_t end = off + (uint64_t)count * kIndexEntrySize;
      if (off >= (uint64_t)kFileHeaderSize && end == n - kFooterSize && end >= off && (int64_t)count <= out.cap) {
        ok = 1;
        sOff = off;
        sCount = count;
        sWant = rd32(f + 12);
      }
    }
  }
  __syncthreads();
  if (!ok) {
    if (tid == 0) *out.count = -1;
    return;
  }
  const uint64_t off = sOff;
  const uint32_t count = sCount;
  const uint64_t len = (uint64_t)count * kIndexEntrySize;
  const uint64_t chunk = (len + kIngestThreads - 1) / kIngestThreads;
  // Chunk CRC registers from zero, and the zero-run map of a full chunk.
  {
    const uint64_t b = (uint64_t)tid * chunk, e = b + chunk < len ? b + chunk : len;
    uint32_t r = 0;
    for (uint64_t i = b; i < e; i++) r = crcByte(T, r, c[off + i]);
    part[tid] = r;
    if (tid < 32) {
      uint32_t v = 1u << tid;
      for (uint64_t i = 0; i < chunk; i++) v = crcByte(T, v, 0);
      M[tid] = v;
    }
  }
  __syncthreads();
  if (tid == 0) {
    // Register after the whole table: r = advance(r, chunk) ^ part[i] for
    // each full chunk, the last (short) chunk byte by byte.
    uint32_t r = 0xFFFFFFFFu;
    const uint64_t full = chunk ? len / chunk : 0;
    for (uint64_t i = 0; i < full; i++) {
      uint32_t a = 0;
      for (int k = 0; k < 32; k++)
        if ((r >> k) & 1) a ^= M[k];
      r = a ^ part[i];
    }
    for (uint64_t i = full * chunk; i < len; i++) r = crcByte(T, r, c[off + i]);
    ok = (~r == sWant) ? 1 : 0;
  }
  __syncthreads();
  // validateEntry — ebiv/reader.go:115-123; the first entry a key frame.
  for (uint32_t i = tid; i < count && ok; i += kIngestThreads) {
    const uint8_t* p = c + off + (uint64_t)i * kIndexEntrySize;
    const uint64_t eo = rd64(p);
    const uint32_t sz = rd32(p + 8);
    const bool key = (rd32(p + 12) & 1u) != 0;
    const bool valid = eo >= (uint64_t)kFileHeaderSize && sz != 0 && sz <= (uint32_t)kMaxFrameSize &&
                       eo + kFrameRecordSize + sz <= off && (i != 0 || key);
    if (!valid) ok = 0;  // benign race: every writer stores 0
    out.off[i] = eo + kFrameRecordSize;
    out.size[i] = sz;
    out.key[i] = key ? 1 : 0;
  }
  __syncthreads();
  if (tid == 0) *out.count = ok ? (int32_t)count : -1;
}

__global__ void kScanFrames(const uint8_t* c, uint64_t n, IndexOut out) {
  if (threadIdx.x != 0) return;
  uint64_t off = kFileHeaderSize;
  int32_t k = 0;
  while (off + kFrameRecordSize <= n && k < out.cap) {
    const uint8_t* p = c + off;
    const uint32_t sync = (uint32_t)p[0] | (uint32_t)p[1] << 8;
    const uint32_t flags = (uint32_t)p[2] | (uint32_t)p[3] << 8;
    const uint32_t sz = rd32(p + 4);
    if (sync != kFrameSync || sz == 0 || sz > (uint32_t)kMaxFrameSize) break;
    const uint64_t end = off + kFrameRecordSize + sz;
    if (end > n) break;
    out.off[k] = off + kFrameRecordSize;
    out.size[k] = sz;
    out.key[k] = (flags & 1u) ? 1 : 0;
    k++;
    off = end;
  }
  *out.count = (k == 0 || !out.key[0]) ? -1 : k;
}

// frameTime (ebiv/format.go:250-253) with Go's int64 wrap-around.
__device__ __forceinline__ int64_t frameTimeD(int64_t i, uint32_t num, uint32_t den) {
  const int64_t p = (int64_t)((uint64_t)i * (uint64_t)den * 1000000000ull);
  return p / (int64_t)num;
}

// result[0]: the frame index seeked to (or -1 when frameIndexAt's
// correction walk did not settle within 2^20 steps, which only hostile frame
// rates reach); result[1]: its presentation time.
__global__ void __launch_bounds__(kIngestThreads) kSeek(const uint8_t* key, int32_t count, uint32_t num, uint32_t den,
                                                     int64_t t, int64_t* result) {
  __shared__ int64_t sTarget;
  __shared__ int32_t best[kIngestThreads / 32];
  const int tid = threadIdx.x;
  if (tid == 0) {
    int64_t i = 0;
    bool settled = true;
    if (t > 0) {
      const int64_t q = (int64_t)((uint64_t)t * (uint64_t)num), d = (int64_t)((uint64_t)den * 1000000000ull);
      i = q / d;
      int steps = 0;
      while (frameTimeD(i + 1, num, den) <= t && (settled = ++steps < (1 << 20))) i++;
      while (settled && i > 0 && frameTimeD(i, num, den) > t && (settled = ++steps < (1 << 20))) i--;
    }
    if (i >= count) i = count - 1;
    sTarget = settled ? i : -1;
  }
  __syncthreads();
  const int64_t target = sTarget;
  if (target < 0) {
    if (tid == 0) {
      result[0] = -1;
      result[1] = 0;
    }
    return;
  }
  // keyframeBefore: the largest key frame index <= target (index 0 at worst).
  int32_t m = 0;
  for (int64_t i = tid; i <= target; i += kIngestThreads)
    if (key[i]) m = (int32_t)i;
  for (int o = 16; o; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((tid & 31) == 0) best[tid >> 5] = m;
  __syncthreads();
  if (tid == 0) {
    int32_t b = 0;
    for (int w = 0; w < kIngestThreads / 32; w++) b = max(b, best[w]);
    result[0] = b;
    result[1] = frameTimeD(b, num, den);
  }
}

}  // namespace dev
}  // namespace ebiv

using namespace ebiv;

struct ebivgpu_container {
  uint8_t* host = nullptr;        // pinned copy of the container
  const uint8_t* dev = nullptr;   // its device mapping
  size_t n = 0;
  uint32_t fpsNum = 0, fpsDen = 0;
  int width = 0, height = 0;
  int rebuilt = 0;
  uint64_t* dOff = nullptr;
  uint32_t* dSize = nullptr;
  uint8_t* dKey = nullptr;
  int32_t* dCount = nullptr;
  int64_t* dSeek = nullptr;
  cudaStream_t stream = nullptr;
  std::vector<uint64_t> off;  // host copies of the device-built index
  std::vector<uint32_t> size;
  std::vector<uint8_t> key;
  ~ebivgpu_container() {
    if (stream) cudaStreamSynchronize(stream);
    if (host) cudaFreeHost(host);
    cudaFree(dOff);
    cudaFree(dSize);
    cudaFree(dKey);
    cudaFree(dCount);
    cudaFree(dSeek);
    if (stream) cudaStreamDestroy(stream);
  }
};

extern "C" {

int ebivgpu_container_open(const uint8_t* data, size_t n, ebivgpu_container** out) {
  if (!out || (!data && n)) return kErrArg;
  *out = nullptr;
  // FileHeader.unmarshal — ebiv/format.go:230-265 (48 bytes, on the host).
  if (n < (size_t)kFileHeaderSize || std::memcmp(data, "EBIV", 4) != 0) return kErrBadMagic;
  auto r16 = [&](int o) { return (uint32_t)data[o] | (uint32_t)data[o + 1] << 8; };
  auto r32 = [&](int o) { return r16(o) | r16(o + 2) << 16; };
  if (r16(4) != kVersion) return kErrVersion;
  const uint32_t w = r32(8), h = r32(12), fn = r32(16), fd = r32(20);
  if (r16(6) != (uint32_t)kFileHeaderSize || w == 0 || w > 65535 || h == 0 || h > 65535 || fn == 0 || fd == 0)
    return kErrCorrupt;
  if (data[28] != 0 || data[29] != 0) return kErrUnsupported;
  ebivgpu_container* c = new (std::nothrow) ebivgpu_container();
  if (!c) return kErrArg;
  c->n = n;
  c->fpsNum = fn;
  c->fpsDen = fd;
  c->width = (int)w;
  c->height = (int)h;
  // Frames the index may hold: every record takes at least 9 bytes.
  const int32_t cap = (int32_t)std::min<size_t>((n - kFileHeaderSize) / (kFrameRecordSize + 1) + 1, 1u << 30);
  void* dptr = nullptr;
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaHostAlloc(reinterpret_cast<void**>(&c->host), n, cudaHostAllocMapped) != cudaSuccess ||
      cudaHostGetDevicePointer(&dptr, c->host, 0) != cudaSuccess || cudaMalloc(&c->dOff, 8 * (size_t)cap) ||
      cudaMalloc(&c->dSize, 4 * (size_t)cap) || cudaMalloc(&c->dKey, (size_t)cap) || cudaMalloc(&c->dCount, 4) ||
      cudaMalloc(&c->dSeek, 16)) {
    delete c;
    return kErrDevice;
  }
  c->dev = static_cast<const uint8_t*>(dptr);
  std::memcpy(c->host, data, n);
  dev::IndexOut io{c->dOff, c->dSize, c->dKey, c->dCount, cap};
  int32_t count = -1;
  dev::kIndexFooter<<<1, dev::kIngestThreads, 0, c->stream>>>(c->dev, (uint64_t)n, io);
  if (cudaMemcpyAsync(&count, c->dCount, 4, cudaMemcpyDeviceToHost, c->stream) != cudaSuccess ||
      cudaStreamSynchronize(c->stream) != cudaSuccess) {
    delete c;
    return kErrDevice;
  }
  if (count < 0) {  // the footer did not validate: rebuild by scanning
    c->rebuilt = 1;
    dev::kScanFrames<<<1, 32, 0, c->stream>>>(c->dev, (uint64_t)n, io);
    if (cudaMemcpyAsync(&count, c->dCount, 4, cudaMemcpyDeviceToHost, c->stream) != cudaSuccess ||
        cudaStreamSynchronize(c->stream) != cudaSuccess) {
      delete c;
      return kErrDevice;
    }
    if (count < 0) {
      delete c;
      return kErrCorrupt;  // no frames, or the first is not a key frame
    }
  }
  c->off.resize((size_t)count);
  c->size.resize((size_t)count);
  c->key.resize((size_t)count);
  if ((count && (cudaMemcpyAsync(c->off.data(), c->dOff, 8 * (size_t)count, cudaMemcpyDeviceToHost, c->stream) ||
                 cudaMemcpyAsync(c->size.data(), c->dSize, 4 * (size_t)count, cudaMemcpyDeviceToHost, c->stream) ||
                 cudaMemcpyAsync(c->key.data(), c->dKey, (size_t)count, cudaMemcpyDeviceToHost, c->stream))) ||
      cudaStreamSynchronize(c->stream) != cudaSuccess) {
    delete c;
    return kErrDevice;
  }
  *out = c;
  return kOK;
}

void ebivgpu_container_close(ebivgpu_container* c) { delete c; }

int ebivgpu_container_info(ebivgpu_container* c, int64_t* info6) {
  if (!c || !info6) return kErrArg;
  info6[0] = c->width;
  info6[1] = c->height;
  info6[2] = c->fpsNum;
  info6[3] = c->fpsDen;
  info6[4] = (int64_t)c->off.size();
  info6[5] = c->rebuilt;
  return kOK;
}

// An index entry whose payload lies outside the container: validateEntry's
// uint64 sum (ebiv/reader.go:115-123) wraps for offsets near 2^64, and the
// reference then fails NextPacket with a seek to a negative position
// (reader.go:203-205).  Offsets that wrap to 0..7 stay inside the file.
static bool entryReadable(const ebivgpu_container* c, size_t i) {
  return c->off[i] <= c->n && c->size[i] <= c->n - c->off[i];
}

int ebivgpu_container_entry(ebivgpu_container* c, int i, uint64_t* payload_offset, uint32_t* size, int* keyframe) {
  if (!c || i < 0 || i >= (int)c->off.size()) return kErrArg;
  if (!entryReadable(c, (size_t)i)) return kErrIO;
  if (payload_offset) *payload_offset = c->off[(size_t)i];
  if (size) *size = c->size[(size_t)i];
  if (keyframe) *keyframe = c->key[(size_t)i];
  return kOK;
}

int ebivgpu_container_seek(ebivgpu_container* c, int64_t t_ns, int64_t* frame, int64_t* landed_ns) {
  if (!c) return kErrArg;
  if (c->off.empty()) return kErrEOF;
  int64_t r[2] = {0, 0};
  dev::kSeek<<<1, dev::kIngestThreads, 0, c->stream>>>(c->dKey, (int32_t)c->off.size(), c->fpsNum, c->fpsDen, t_ns,
                                                        c->dSeek);
  if (cudaGetLastError() != cudaSuccess ||
      cudaMemcpyAsync(r, c->dSeek, sizeof(r), cudaMemcpyDeviceToHost, c->stream) != cudaSuccess ||
      cudaStreamSynchronize(c->stream) != cudaSuccess)
    return kErrDevice;
  if (r[0] < 0) return kErrCorrupt;
  if (frame) *frame = r[0];
  if (landed_ns) *landed_ns = r[1];
  return kOK;
}

int ebivgpu_batch_add_container(ebivgpu_batch* b, ebivgpu_container* c, int ring, int* stream_id) {
  if (!b || !c || !stream_id) return kErrArg;
  Engine* e = batchEngine(b);
  if (!e) return kErrArg;
  // The stream reads every packet in place, ahead of its frame: a container
  // with an unreadable entry is refused here (the reference reports it when
  // playback reaches that frame).
  for (size_t i = 0; i < c->off.size(); i++)
    if (!entryReadable(c, i)) return kErrIO;
  return e->addContainerStream(c->host, c->dev, c->off.data(), c->size.data(), (int)c->off.size(), ring, stream_id);
}

}  // extern "C"
