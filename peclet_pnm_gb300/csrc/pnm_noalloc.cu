// pnm_extract_pores_noalloc: extract_pores on a device SDF that allocates no device memory.
//
// Who needs it: callers that own every byte of device memory through their own pool allocator
// and cannot let a library call cudaMalloc / cudaFree on its own — host frameworks that run
// under a fixed memory budget (a stray cudaMalloc can fail against it or fragment the pool),
// and long-running serving loops that must not enter the driver allocator while other work is
// in flight (cudaMalloc / cudaFree can implicitly synchronise the device). Such a caller passes
// its device input and output buffers and a stream; the only scratch this entry point uses is
// the file-scope device array below.
//
// Limits and sharing:
//  * at most kNoAllocMaxVoxels voxels per call; larger volumes are rejected with
//    PNM_ERR_SHAPE before any work is queued;
//  * every GPU that loads the library holds the array (~16 MiB) until the process exits;
//  * all calls on a device share the one array, which keeps the last call's contents (the peak
//    bitmap is cleared at the start of every call): two calls whose work overlaps on the GPU —
//    different streams, or host threads racing — corrupt each other's results. Serialise calls
//    per device (one stream, or an event between calls);
//  * the first call on each device looks up the array's device address (cudaGetSymbolAddress,
//    with that device current) and caches it. Under CUDA's lazy module loading (the default
//    since CUDA 12.2) that first call is also when the driver loads this library's kernels on
//    the device and reserves the array, which allocates and may synchronise: make the first call
//    at start-up, before the caller's pool claims the device's memory and before any stream
//    capture (or set CUDA_MODULE_LOADING=EAGER, which loads the module with the context).
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <climits>
#include <cmath>
#include <cstdint>
#include <mutex>

#include "pnm_ctx.h"
#include "pnm_device.cuh"

namespace pnm {
namespace {

constexpr long long kNoAllocMaxVoxels = 1ll << 26;  // 67,108,864 voxels (406^3)
constexpr long long kWords = kNoAllocMaxVoxels / 32;             // peak bitmap words
constexpr long long kScanTmp = kWords / SCAN_TILE + 2;           // scan block partials
constexpr long long kScratchWords = kWords + (kWords + 1) + kScanTmp;

// [peak bitmap: kWords][prefix counts: kWords + 1][scan partials: kScanTmp]
static __device__ __align__(256) uint32_t g_noalloc_scratch[kScratchWords];

constexpr int kMaxDevices = 64;
std::atomic<uint32_t*> g_scratch_addr[kMaxDevices];
std::mutex g_scratch_mu;

// Device address of the scratch array on the current device (looked up once per device).
int scratch_on_current_device(uint32_t** out) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) return PNM_ERR_NO_DEVICE;
  if (dev >= kMaxDevices) return PNM_ERR_INTERNAL;
  uint32_t* p = g_scratch_addr[dev].load(std::memory_order_acquire);
  if (!p) {
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    p = g_scratch_addr[dev].load(std::memory_order_acquire);
    if (!p) {
      const cudaError_t e = cudaGetSymbolAddress((void**)&p, g_noalloc_scratch);
      if (e != cudaSuccess || !p) {
        cudaGetLastError();
        return PNM_ERR_CUDA;
      }
      g_scratch_addr[dev].store(p, std::memory_order_release);
    }
  }
  *out = p;
  return PNM_OK;
}

constexpr int NX = 32, NY = 8, NZ = 8;

// The peak test of the SDF pass on its own (pore_extraction.hpp:85-106): a voxel with
// !(sdf <= 0) is a pore when no periodic neighbour has a larger (value, wrapped index). Bits go
// into the caller-supplied bitmap (here: the static scratch array). One block per 32 x 8 x 8
// tile on a 1-D grid (tile = (bz * tny + by) * tnx + bx), so no shape meets the 65,535 limit of
// a grid's y and z extents.
__global__ void __launch_bounds__(NX* NY)
    k_peak_bits(const float* __restrict__ sdf, Dims d, uint32_t* __restrict__ bits) {
  constexpr int HX = NX + 2, HY = NY + 2, HZ = NZ + 2, NT = NX * NY;
  __shared__ float s[HZ][HY][HX];
  __shared__ int wx[HX], wy[HY], wz[HZ];
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  const int nxy = nx * ny;
  const int tnx = (nx + NX - 1) / NX, tny = (ny + NY - 1) / NY;
  const int tile = (int)blockIdx.x;
  const int X0 = (tile % tnx) * NX, Y0 = ((tile / tnx) % tny) * NY, Z0 = (tile / tnx / tny) * NZ;
  const int t = threadIdx.x;
  if (t < HX) wx[t] = ((X0 - 1 + t) % nx + nx) % nx;
  if (t < HY) wy[t] = ((Y0 - 1 + t) % ny + ny) % ny;
  if (t < HZ) wz[t] = ((Z0 - 1 + t) % nz + nz) % nz;
  __syncthreads();
  for (int i = t; i < HX * HY * HZ; i += NT) {
    const int hx = i % HX, hy = (i / HX) % HY, hz = i / (HX * HY);
    s[hz][hy][hx] = __ldg(&sdf[wz[hz] * nxy + wy[hy] * nx + wx[hx]]);
  }
  __syncthreads();
  const int tx = t % NX, ty = t / NX;
  const int gx = X0 + tx, gy = Y0 + ty;
  if (gx >= nx || gy >= ny) return;
  for (int tz = 0; tz < NZ; ++tz) {
    const int gz = Z0 + tz;
    if (gz >= nz) break;
    const int ci = gz * nxy + gy * nx + gx;
    const float cv = s[tz + 1][ty + 1][tx + 1];
    if (cv <= 0.0f) continue;
    bool peak = true;
    for (int k = 0; k < 27 && peak; ++k) {
      if (k == kSelf) continue;
      const int dz = k / 9 - 1, dy = (k / 3) % 3 - 1, dx = k % 3 - 1;
      const float nv = s[tz + 1 + dz][ty + 1 + dy][tx + 1 + dx];
      if (nv > cv) peak = false;
      else if (nv == cv && wz[tz + 1 + dz] * nxy + wy[ty + 1 + dy] * nx + wx[tx + 1 + dx] > ci)
        peak = false;
    }
    if (peak) atomicOr(&bits[ci >> 5], 1u << (ci & 31));
  }
}

}  // namespace
}  // namespace pnm

extern "C" int pnm_extract_pores_noalloc(const float* d_sdf, int32_t nx, int32_t ny, int32_t nz,
                                         const float origin_xyz[3], const float spacing_xyz[3],
                                         pnm_pore* d_pores, int64_t pore_cap, int64_t* n_pores,
                                         void* stream) {
  using namespace pnm;
  if (!origin_xyz || !spacing_xyz || !n_pores) return PNM_ERR_ARG;
  *n_pores = 0;
  if (nx < 0 || ny < 0 || nz < 0) return PNM_ERR_ARG;
  for (int a = 0; a < 3; ++a)
    if (!(spacing_xyz[a] > 0.0f) || !std::isfinite(spacing_xyz[a])) return PNM_ERR_ARG;
  const Dims d{nx, ny, nz};
  const long long n = d.n();
  if (n == 0) return PNM_OK;
  if (n > kNoAllocMaxVoxels) return PNM_ERR_SHAPE;  // beyond the static scratch
  if (!d_sdf || (!d_pores && pore_cap > 0)) return PNM_ERR_ARG;
  uint32_t* scratch = nullptr;
  const int rc = scratch_on_current_device(&scratch);
  if (rc != PNM_OK) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const long long words = (n + 31) / 32;
  uint32_t* bits = scratch;
  unsigned* pref = scratch + kWords;
  unsigned* part = scratch + kWords + (kWords + 1);
  if (cudaMemsetAsync(bits, 0, words * sizeof(uint32_t), s) != cudaSuccess) {
    cudaGetLastError();
    return PNM_ERR_CUDA;
  }
  // tiles <= 2^26 / 1 (a 1 x 1 x 2^26 volume): within a 1-D grid's 2^31 - 1 blocks
  const long long tiles = (long long)((nx + NX - 1) / NX) * ((ny + NY - 1) / NY) *
                          ((nz + NZ - 1) / NZ);
  k_peak_bits<<<(unsigned)tiles, NX * NY, 0, s>>>(d_sdf, d, bits);
  if (cudaGetLastError() != cudaSuccess) return PNM_ERR_CUDA;
  long long launches = 0;
  exclusive_scan(PopcountOf{bits}, words, pref, part, s, &launches);
  if (cudaGetLastError() != cudaSuccess) return PNM_ERR_CUDA;
  const unsigned egrid = (unsigned)std::min<long long>((words + 255) / 256, 152 * 8);
  const long long cap = std::min<long long>(pore_cap, 1000000);  // max_pores, :77
  launch_pores_emit(d_sdf, d, bits, pref, words, origin_xyz, spacing_xyz, d_pores, cap, egrid, s);
  if (cudaGetLastError() != cudaSuccess) return PNM_ERR_CUDA;
  unsigned total = 0;
  if (cudaMemcpyAsync(&total, pref + words, sizeof(unsigned), cudaMemcpyDeviceToHost, s) !=
          cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess) {
    cudaGetLastError();
    return PNM_ERR_CUDA;
  }
  const int64_t np = std::min<int64_t>(total, 1000000);  // max_pores, pore_extraction.hpp:77
  *n_pores = np;
  return np > pore_cap ? PNM_ERR_CAPACITY : PNM_OK;
}
