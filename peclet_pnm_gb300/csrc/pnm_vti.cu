// VTI ingest (pnm_vti_*): the reference's SDFReader::read_vti (src/sdf_reader.cpp:28-152) for
// ImageData files whose first appended array is raw float32 behind a UInt64 byte count.
//
// Header semantics follow the reference: the first 8 KiB are searched as text; the resolution is
// WholeExtent "x1 x2 y1 y2 z1 z2" -> (x2-x1+1, y2-y1+1, z2-z1+1); Origin and Spacing are the first
// attributes of those names; the array starts after the first '_' that follows
// <AppendedData encoding="raw">, as an 8-byte length in host byte order and the values. A length
// that differs from the resolution's byte count is read byte-wise as far as both allow and the
// remaining bytes are zero, as the reference's zero-initialised buffer leaves them (a length
// larger than the volume is clamped to it rather than written past the buffer).
//
// pnm_read_vti_dev streams the values to device memory through two pinned staging buffers: the
// file read of one chunk overlaps the copy of the previous one.
#include <cuda_runtime.h>

#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <algorithm>
#include <cstring>
#include <string>

#include "pnm_ctx.h"

namespace {

constexpr size_t kHeaderBytes = 8192;
constexpr size_t kChunk = 64ull << 20;  // staging chunk of the device read

// value of attr="..." at its first occurrence, or empty
std::string attribute(const std::string& text, const char* name) {
  const std::string key = std::string(name) + "=\"";
  const size_t p = text.find(key);
  if (p == std::string::npos) return "";
  const size_t b = p + key.size(), e = text.find('"', b);
  if (e == std::string::npos) return "";
  return text.substr(b, e - b);
}

int parse_floats(const std::string& s, float* out, int n) {
  const char* c = s.c_str();
  for (int i = 0; i < n; ++i) {
    char* end = nullptr;
    errno = 0;
    const float v = std::strtof(c, &end);
    if (end == c) return i;
    out[i] = v;
    c = end;
  }
  return n;
}

struct VtiHeader {
  int32_t dims[3];
  float origin[3], spacing[3];
  int64_t offset;  // first value byte
  int64_t bytes;   // the array's byte count from the file
};

int read_header(std::FILE* f, VtiHeader* h, std::string* why) {
  std::string text(kHeaderBytes, '\0');
  const size_t got = std::fread(&text[0], 1, kHeaderBytes, f);
  text.resize(got);
  const std::string ext = attribute(text, "WholeExtent");
  if (ext.empty()) {
    *why = "Could not find WholeExtent in VTI header";
    return PNM_ERR_ARG;
  }
  long long e[6];
  {
    const char* c = ext.c_str();
    for (int i = 0; i < 6; ++i) {
      char* end = nullptr;
      e[i] = std::strtoll(c, &end, 10);
      if (end == c) {
        *why = "malformed WholeExtent in VTI header";
        return PNM_ERR_ARG;
      }
      c = end;
    }
  }
  for (int a = 0; a < 3; ++a) {
    const long long n = e[2 * a + 1] - e[2 * a] + 1;
    if (n < 0 || n > 0x7fffffffll) {
      *why = "WholeExtent out of range";
      return PNM_ERR_SHAPE;
    }
    h->dims[a] = (int32_t)n;
  }
  for (int a = 0; a < 3; ++a) h->origin[a] = h->spacing[a] = 0.0f;
  parse_floats(attribute(text, "Origin"), h->origin, 3);
  parse_floats(attribute(text, "Spacing"), h->spacing, 3);
  const size_t tag = text.find("<AppendedData encoding=\"raw\">");
  if (tag == std::string::npos) {
    *why = "Could not find AppendedData tag";
    return PNM_ERR_ARG;
  }
  const size_t us = text.find('_', tag);
  if (us == std::string::npos) {
    *why = "Could not find binary data marker '_' in first 8KB";
    return PNM_ERR_ARG;
  }
  uint64_t len = 0;
  if (std::fseek(f, (long)(us + 1), SEEK_SET) != 0 || std::fread(&len, 8, 1, f) != 1) {
    *why = "Failed to read data_bytes (UInt64) from file.";
    return PNM_ERR_ARG;
  }
  h->offset = (int64_t)(us + 1 + 8);
  h->bytes = len > (uint64_t)INT64_MAX ? INT64_MAX : (int64_t)len;
  return PNM_OK;
}

thread_local std::string g_vti_error;

int fail(int code, const std::string& why) {
  g_vti_error = why;
  return code;
}

}  // namespace

extern "C" {

const char* pnm_vti_last_error(void) { return g_vti_error.c_str(); }

int pnm_read_vti_header(const char* path, int32_t dims_xyz[3], float origin_xyz[3],
                        float spacing_xyz[3], int64_t* data_bytes) {
  if (!path || !dims_xyz || !origin_xyz || !spacing_xyz) return fail(PNM_ERR_ARG, "null argument");
  std::FILE* f = std::fopen(path, "rb");
  if (!f) return fail(PNM_ERR_ARG, std::string("Could not open file: ") + path);
  VtiHeader h;
  std::string why;
  const int rc = read_header(f, &h, &why);
  std::fclose(f);
  if (rc != PNM_OK) return fail(rc, why);
  for (int a = 0; a < 3; ++a) {
    dims_xyz[a] = h.dims[a];
    origin_xyz[a] = h.origin[a];
    spacing_xyz[a] = h.spacing[a];
  }
  if (data_bytes) *data_bytes = h.bytes;
  return PNM_OK;
}

int pnm_read_vti(const char* path, float* dst, int64_t n) {
  if (!path || (!dst && n > 0) || n < 0) return fail(PNM_ERR_ARG, "null argument");
  std::FILE* f = std::fopen(path, "rb");
  if (!f) return fail(PNM_ERR_ARG, std::string("Could not open file: ") + path);
  VtiHeader h;
  std::string why;
  int rc = read_header(f, &h, &why);
  if (rc == PNM_OK) {
    const int64_t want = std::min<int64_t>(h.bytes, n * 4);
    int64_t got = 0;
    if (std::fseek(f, (long)h.offset, SEEK_SET) == 0)
      got = (int64_t)std::fread(dst, 1, (size_t)want, f);
    if (got < n * 4) std::memset((char*)dst + got, 0, (size_t)(n * 4 - got));
  }
  std::fclose(f);
  return rc == PNM_OK ? PNM_OK : fail(rc, why);
}

int pnm_read_vti_dev(pnm_ctx* ctx, const char* path, float* d_dst, int64_t n) {
  if (!ctx) return fail(PNM_ERR_ARG, "null argument");
  pnm::Ctx& c = ctx->c;
  if (!path || (!d_dst && n > 0) || n < 0) {
    c.last_error = "null argument";
    return fail(PNM_ERR_ARG, c.last_error);
  }
  std::FILE* f = std::fopen(path, "rb");
  if (!f) return fail(PNM_ERR_ARG, std::string("Could not open file: ") + path);
  VtiHeader h;
  std::string why;
  int rc = read_header(f, &h, &why);
  void* stage[2] = {nullptr, nullptr};
  cudaEvent_t done[2] = {nullptr, nullptr};
  auto body = [&]() -> int {
    if (rc != PNM_OK) return fail(rc, why);
    if (cudaSetDevice(c.device) != cudaSuccess) return fail(PNM_ERR_CUDA, "cudaSetDevice");
    if (n > 0) {  // the destination must be device (or managed) memory
      cudaPointerAttributes pa{};
      if (cudaPointerGetAttributes(&pa, d_dst) != cudaSuccess ||
          (pa.type != cudaMemoryTypeDevice && pa.type != cudaMemoryTypeManaged)) {
        cudaGetLastError();
        return fail(PNM_ERR_ARG, "destination is not device memory");
      }
    }
    const int64_t avail = std::min<int64_t>(h.bytes, n * 4);  // bytes
    if (std::fseek(f, (long)h.offset, SEEK_SET) != 0) return fail(PNM_ERR_ARG, "seek failed");
    for (int i = 0; i < 2; ++i)
      if (cudaMallocHost(&stage[i], kChunk) != cudaSuccess ||
          cudaEventCreateWithFlags(&done[i], cudaEventDisableTiming) != cudaSuccess)
        return fail(PNM_ERR_CUDA, "staging buffers");
    int64_t pos = 0;
    for (int k = 0; pos < avail; ++k) {
      const int b = k & 1;
      // the copy that last used this buffer must have drained before it is refilled
      if (k >= 2 && cudaEventSynchronize(done[b]) != cudaSuccess)
        return fail(PNM_ERR_CUDA, "staging copy");
      const int64_t cnt = std::min<int64_t>((int64_t)kChunk, avail - pos);
      const int64_t got = (int64_t)std::fread(stage[b], 1, (size_t)cnt, f);
      if (got > 0 &&
          (cudaMemcpyAsync((char*)d_dst + pos, stage[b], (size_t)got, cudaMemcpyHostToDevice,
                           c.stream) != cudaSuccess ||
           cudaEventRecord(done[b], c.stream) != cudaSuccess))
        return fail(PNM_ERR_CUDA, "staging copy");
      pos += got;
      if (got < cnt) break;  // short file
    }
    if (pos < n * 4 &&
        cudaMemsetAsync((char*)d_dst + pos, 0, (size_t)(n * 4 - pos), c.stream) != cudaSuccess)
      return fail(PNM_ERR_CUDA, "zero fill");
    if (cudaStreamSynchronize(c.stream) != cudaSuccess) return fail(PNM_ERR_CUDA, "sync");
    return PNM_OK;
  };
  const int out = body();
  std::fclose(f);
  // a failed call may leave a staging copy in flight: drain the stream before the buffers go
  if (out != PNM_OK && (stage[0] || stage[1])) cudaStreamSynchronize(c.stream);
  for (int i = 0; i < 2; ++i) {
    if (done[i]) cudaEventDestroy(done[i]);
    if (stage[i]) cudaFreeHost(stage[i]);
  }
  cudaGetLastError();
  if (out != PNM_OK) c.last_error = g_vti_error;
  return out;
}

}  // extern "C"
