// The C ABI of libpnm_gb300.so (include/pnm_gb300.h): context and workspace management, argument
// checks mirroring the reference binding (src/pnm_bindings.cpp), host<->device staging, and the
// sequencing of the device stages. No CPU fallback: without an sm_103 device every entry point
// returns PNM_ERR_NO_DEVICE.
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>

#include "pnm_ctx.h"

namespace pnm {

Status cuda_status(cudaError_t e, const char* what) {
  Status s;
  s.code = PNM_ERR_CUDA;
  s.msg = std::string("CUDA error in ") + what + ": " + cudaGetErrorString(e);
  return s;
}

Status Workspace::get(int slot, size_t bytes, void** out) {
  if (bytes == 0) bytes = 16;
  if (cap[slot] < bytes) {
    if (ptr[slot]) cudaFree(ptr[slot]);
    ptr[slot] = nullptr;
    cap[slot] = 0;
    // grow with headroom so that slightly larger volumes reuse the allocation
    const size_t want = bytes + bytes / 8;
    cudaError_t e = cudaMalloc(&ptr[slot], want);
    if (e != cudaSuccess) {
      cudaGetLastError();
      e = cudaMalloc(&ptr[slot], bytes);
      if (e != cudaSuccess) {
        cudaGetLastError();
        ptr[slot] = nullptr;
        return cuda_status(e, "cudaMalloc(workspace)");
      }
      cap[slot] = bytes;
    } else {
      cap[slot] = want;
    }
  }
  *out = ptr[slot];
  return Status::ok();
}

void Workspace::release() {
  for (size_t i = 0; i < ptr.size(); ++i) {
    if (ptr[i]) cudaFree(ptr[i]);
    ptr[i] = nullptr;
    cap[i] = 0;
  }
}

size_t Workspace::total_bytes() const {
  size_t t = 0;
  for (size_t c : cap) t += c;
  return t;
}

Status Ctx::ensure_copy_events(int n) {
  if (!copy_stream) PNM_CUDA(cudaStreamCreateWithFlags(&copy_stream, cudaStreamNonBlocking));
  while ((int)events.size() < n) {
    cudaEvent_t e;
    PNM_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    events.push_back(e);
  }
  return Status::ok();
}

Status Ctx::ensure_side() {
  if (side_stream) return Status::ok();
  PNM_CUDA(cudaStreamCreateWithFlags(&side_stream, cudaStreamNonBlocking));
  PNM_CUDA(cudaEventCreateWithFlags(&side_fork, cudaEventDisableTiming));
  PNM_CUDA(cudaEventCreateWithFlags(&side_join, cudaEventDisableTiming));
  PNM_CUDA(cudaEventCreate(&side_t0));
  PNM_CUDA(cudaEventCreate(&side_t1));
  PNM_CUDA(cudaMallocHost(&h_side, 16));
  return Status::ok();
}

Status Ctx::join_side() {
  if (!side_pending) return Status::ok();
  PNM_CUDA(cudaStreamWaitEvent(stream, side_join, 0));
  side_pending = false;
  return Status::ok();
}

// The counters reach the host through a kernel's stores to mapped pinned memory: a copy-engine
// transfer would queue behind label slabs already on their way to the host, and the pair stages
// that wait for the pair count would then start only after the whole label download.
__global__ void k_counters_to_host(const unsigned* __restrict__ d, unsigned* h) {
  for (int i = threadIdx.x; i < CNT_COUNT; i += blockDim.x) h[i] = d[i];
}
Status Ctx::read_counters() {
  k_counters_to_host<<<1, 32, 0, stream>>>(d_cnt, h_cnt_dev);
  ++launches;
  PNM_CUDA(cudaGetLastError());
  PNM_CUDA(cudaStreamSynchronize(stream));
  return Status::ok();
}

void Ctx::call_begin() {
  for (double& t : last.stage_ms) t = 0.0;
  side_timed = false;
  tstage.clear();
  open_stages.clear();
}

void Ctx::interval_begin(int id) {
  const size_t k = tstage.size();
  while (tev.size() < 2 * k + 2) {
    cudaEvent_t e;
    if (cudaEventCreate(&e) != cudaSuccess) {
      cudaGetLastError();
      return;
    }
    tev.push_back(e);
  }
  if (cudaEventRecord(tev[2 * k], stream) != cudaSuccess) {
    cudaGetLastError();
    return;
  }
  tstage.push_back(id);
}

void Ctx::interval_end() {
  if (tstage.empty()) return;
  if (cudaEventRecord(tev[2 * (tstage.size() - 1) + 1], stream) != cudaSuccess) cudaGetLastError();
}

void Ctx::stage_begin(int id, const char* name) {
  nvtxRangePushA(name);
  ++nvtx_depth;
  if (!timing) return;
  if (!open_stages.empty()) interval_end();  // pause the enclosing stage
  open_stages.push_back(id);
  interval_begin(id);
}

void Ctx::stage_end() {
  if (timing && !open_stages.empty()) {
    interval_end();
    open_stages.pop_back();
    if (!open_stages.empty()) interval_begin(open_stages.back());  // resume the enclosing one
  }
  if (nvtx_depth > 0) {
    nvtxRangePop();
    --nvtx_depth;
  }
}

void Ctx::stage_collect() {
  if (timing && side_timed) {  // the side stream's interval (it overlaps the main stream's)
    float ms = 0.0f;
    if (cudaEventSynchronize(side_t1) == cudaSuccess &&
        cudaEventElapsedTime(&ms, side_t0, side_t1) == cudaSuccess && side_stage >= 0 &&
        side_stage < PNM_STAGE_COUNT)
      last.stage_ms[side_stage] += ms;
    else
      cudaGetLastError();
    side_timed = false;
  }
  if (!timing || tstage.empty()) return;
  if (cudaEventSynchronize(tev[2 * tstage.size() - 1]) != cudaSuccess) {
    cudaGetLastError();
    tstage.clear();
    return;
  }
  for (size_t k = 0; k < tstage.size(); ++k) {
    float ms = 0.0f;
    if (cudaEventElapsedTime(&ms, tev[2 * k], tev[2 * k + 1]) == cudaSuccess &&
        tstage[k] >= 0 && tstage[k] < PNM_STAGE_COUNT)
      last.stage_ms[tstage[k]] += ms;
    else
      cudaGetLastError();
  }
  tstage.clear();
  open_stages.clear();
}

Status check_dims(Dims d, const float* spacing, bool need_spacing) {
  if (d.nx < 0 || d.ny < 0 || d.nz < 0) return Status{PNM_ERR_ARG, "dims must be non-negative"};
  // voxel ids, labels and the first-appearance sentinel are int32 (get_idx returns int,
  // pore_extraction.hpp:59-64)
  if (d.n() > (long long)INT_MAX - 8)
    return Status{PNM_ERR_SHAPE, "volume too large: nx*ny*nz must be < 2^31 - 8"};
  if (need_spacing) {
    if (!spacing) return Status{PNM_ERR_ARG, "spacing is null"};
    for (int a = 0; a < 3; ++a)
      if (!(spacing[a] > 0.0f) || !std::isfinite(spacing[a]))
        return Status{PNM_ERR_ARG, "spacing must be finite and positive"};
  }
  return Status::ok();
}

}  // namespace pnm

using pnm::Ctx;
using pnm::Dims;
using pnm::Status;

namespace {

int finish(pnm_ctx* ctx, Status s) {
  ++ctx->c.calls;
  ctx->c.stage_collect();
  if (!s.good()) ctx->c.last_error = s.msg;
  return s.code;
}

Status enter(Ctx& c) {
  const cudaError_t e = cudaSetDevice(c.device);
  if (e != cudaSuccess) return pnm::cuda_status(e, "cudaSetDevice");
  c.call_begin();
  return Status::ok();
}

template <class T>
T* host_dup(const T* src, size_t count) {
  T* p = static_cast<T*>(std::malloc(sizeof(T) * (count ? count : 1)));
  if (p && count) std::memcpy(p, src, sizeof(T) * count);
  return p;
}

// Waits for the context's host copies when the call's scope ends (early returns included), so
// no copy still reads or writes a caller's host buffer after the call returns.
struct CopyDrain {
  Ctx& c;
  ~CopyDrain() {
    if (c.copy_stream) cudaStreamSynchronize(c.copy_stream);
  }
};

Status upload_sdf(Ctx& c, const float* sdf, Dims d, const float** d_sdf) {
  float* buf = nullptr;
  PNM_TRY(c.buf(pnm::S_SDF, d.n(), &buf));
  PNM_CUDA(cudaMemcpyAsync(buf, sdf, d.n() * sizeof(float), cudaMemcpyHostToDevice, c.stream));
  *d_sdf = buf;
  return Status::ok();
}

constexpr int64_t kMaxPores = 1000000;  // pore_extraction.hpp:77

Status do_pores(Ctx& c, const float* d_sdf, Dims d, const float* org, const float* spc,
                pnm_pore* d_out, int64_t cap, int64_t* n) {
  pnm::SegState st;
  PNM_TRY(pnm::run_sdf_pass(c, d_sdf, d, spc, &st));
  return pnm::run_pores(c, st, org, spc, d_out, cap, n);
}

void record(Ctx& c, const pnm::SegState& st, int64_t n_pores, int64_t n_pairs) {
  c.last.voxels = st.d.n();
  c.last.ccl_edges = st.n_edges;
  c.last.flood_sweeps = st.flood_sweeps;
  c.last.n_pore_labels = st.n_pore_labels;
  c.last.n_solid_labels = st.n_solid_labels;
  c.last.n_pores = n_pores;
  c.last.n_pairs = n_pairs;
}

Status do_network(Ctx& c, const float* d_sdf, Dims d, const float* org, const float* spc,
                  pnm_pore* d_pores, int64_t pore_cap, int64_t* n_pores, int32_t* d_seg,
                  bool want_pairs, int32_t** d_pairs, int64_t* n_pairs,
                  pnm::HostXfer* xfer = nullptr) {
  pnm::SegState st;
  // the pore records need the SDF pass alone: they run on the side stream meanwhile; the
  // caller's stream joins it however the call ends, so later work there is ordered after it
  struct SideJoin {
    Ctx& c;
    ~SideJoin() { (void)c.join_side(); }
  } side_join{c};
  const std::function<Status()> pores = [&]() {
    return pnm::run_pores_side(c, st, org, spc, d_pores, pore_cap);
  };
  PNM_TRY(pnm::run_segmentation(c, d_sdf, d, spc, &st, false, xfer, d_pores ? &pores : nullptr));
  if (d_pores) PNM_TRY(pnm::side_pores_count(c, n_pores));
  PNM_TRY(pnm::run_seg_and_topology(c, st, d_seg, want_pairs, d_pairs, n_pairs, xfer));
  record(c, st, d_pores ? *n_pores : 0, want_pairs ? *n_pairs : 0);
  return Status::ok();
}

}  // namespace

extern "C" {

const char* pnm_execution_space(void) { return "CudaGB300(sm_103a)"; }

void pnm_free(void* p) { std::free(p); }

int pnm_ctx_create(int device, pnm_ctx** out) {
  if (!out) return PNM_ERR_ARG;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return PNM_ERR_NO_DEVICE;
  }
  if (device < 0 && cudaGetDevice(&device) != cudaSuccess) return PNM_ERR_NO_DEVICE;
  if (device >= ndev) return PNM_ERR_NO_DEVICE;
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return PNM_ERR_NO_DEVICE;
  if (prop.major != 10 || prop.minor != 3) return PNM_ERR_NO_DEVICE;  // built for sm_103a only
  auto* ctx = new (std::nothrow) pnm_ctx();
  if (!ctx) return PNM_ERR_INTERNAL;
  Ctx& c = ctx->c;
  c.device = device;
  c.sm_count = prop.multiProcessorCount;
  if (cudaSetDevice(device) != cudaSuccess ||
      cudaStreamCreateWithFlags(&c.own_stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaMalloc(&c.d_cnt, pnm::CNT_COUNT * sizeof(unsigned)) != cudaSuccess ||
      cudaHostAlloc(&c.h_cnt, pnm::CNT_COUNT * sizeof(unsigned), cudaHostAllocMapped) !=
          cudaSuccess ||
      cudaHostGetDevicePointer(&c.h_cnt_dev, c.h_cnt, 0) != cudaSuccess) {
    cudaGetLastError();
    delete ctx;
    return PNM_ERR_CUDA;
  }
  c.stream = c.own_stream;
  *out = ctx;
  return PNM_OK;
}

void pnm_ctx_destroy(pnm_ctx* ctx) {
  if (!ctx) return;
  Ctx& c = ctx->c;
  cudaSetDevice(c.device);
  cudaStreamSynchronize(c.stream);
  c.ws.release();
  if (c.d_cnt) cudaFree(c.d_cnt);
  if (c.h_cnt) cudaFreeHost(c.h_cnt);
  if (c.copy_stream) {
    cudaStreamSynchronize(c.copy_stream);
    cudaStreamDestroy(c.copy_stream);
  }
  for (cudaEvent_t e : c.events) cudaEventDestroy(e);
  for (cudaEvent_t e : c.tev) cudaEventDestroy(e);
  if (c.side_stream) {
    cudaStreamSynchronize(c.side_stream);
    cudaStreamDestroy(c.side_stream);
    for (cudaEvent_t e : {c.side_fork, c.side_join, c.side_t0, c.side_t1})
      if (e) cudaEventDestroy(e);
    if (c.h_side) cudaFreeHost(c.h_side);
  }
  if (c.own_stream) cudaStreamDestroy(c.own_stream);
  delete ctx;
}

const char* pnm_last_error(const pnm_ctx* ctx) { return ctx ? ctx->c.last_error.c_str() : ""; }

int pnm_ctx_get_stats(const pnm_ctx* ctx, pnm_stats* out) {
  if (!ctx || !out) return PNM_ERR_ARG;
  *out = ctx->c.last;
  out->launches = ctx->c.launches;
  out->calls = ctx->c.calls;
  out->workspace_bytes = (int64_t)ctx->c.ws.total_bytes();
  return PNM_OK;
}

int pnm_ctx_set_timing(pnm_ctx* ctx, int32_t on) {
  if (!ctx) return PNM_ERR_ARG;
  ctx->c.timing = on != 0;
  return PNM_OK;
}

int pnm_ctx_set_wait_limit(pnm_ctx* ctx, int64_t limit_ns, int32_t extra_arrivals) {
  if (!ctx || limit_ns < 1 || limit_ns > 60000000000ll || extra_arrivals < 0) return PNM_ERR_ARG;
  ctx->c.wait_ns = (unsigned long long)limit_ns;
  ctx->c.wait_extra = (unsigned)extra_arrivals;
  return PNM_OK;
}

int pnm_ctx_set_stream(pnm_ctx* ctx, void* stream) {
  if (!ctx) return PNM_ERR_ARG;
  ctx->c.stream = stream ? static_cast<cudaStream_t>(stream) : ctx->c.own_stream;
  return PNM_OK;
}

int pnm_ctx_trim(pnm_ctx* ctx) {
  if (!ctx) return PNM_ERR_ARG;
  cudaSetDevice(ctx->c.device);
  cudaStreamSynchronize(ctx->c.stream);
  ctx->c.ws.release();
  return PNM_OK;
}

int pnm_extract_pores(pnm_ctx* ctx, const float* sdf, int32_t nx, int32_t ny, int32_t nz,
                      const float origin_xyz[3], const float spacing_xyz[3], pnm_pore** pores,
                      int64_t* n_pores) {
  if (!ctx) return PNM_ERR_ARG;
  Ctx& c = ctx->c;
  auto run = [&]() -> Status {
    if (!sdf || !origin_xyz || !pores || !n_pores) return Status{PNM_ERR_ARG, "null argument"};
    const Dims d{nx, ny, nz};
    PNM_TRY(pnm::check_dims(d, spacing_xyz, true));
    if (d.n() == 0) {
      *pores = static_cast<pnm_pore*>(std::malloc(sizeof(pnm_pore)));
      *n_pores = 0;
      return Status::ok();
    }
    PNM_TRY(enter(c));
    const float* d_sdf;
    PNM_TRY(upload_sdf(c, sdf, d, &d_sdf));
    pnm_pore* d_out = nullptr;
    PNM_TRY(c.buf(pnm::S_PORES, kMaxPores, &d_out));
    int64_t np = 0;
    PNM_TRY(do_pores(c, d_sdf, d, origin_xyz, spacing_xyz, d_out, kMaxPores, &np));
    np = std::min(np, kMaxPores);
    pnm_pore* h = static_cast<pnm_pore*>(std::malloc(sizeof(pnm_pore) * (np ? np : 1)));
    if (!h) return Status{PNM_ERR_INTERNAL, "out of host memory"};
    if (np) PNM_CUDA(cudaMemcpyAsync(h, d_out, np * sizeof(pnm_pore), cudaMemcpyDeviceToHost,
                                     c.stream));
    PNM_CUDA(cudaStreamSynchronize(c.stream));
    *pores = h;
    *n_pores = np;
    return Status::ok();
  };
  return finish(ctx, run());
}

int pnm_segment_volume(pnm_ctx* ctx, const float* sdf, int32_t nx, int32_t ny, int32_t nz,
                       const float spacing_xyz[3], int32_t* seg) {
  if (!ctx) return PNM_ERR_ARG;
  Ctx& c = ctx->c;
  auto run = [&]() -> Status {
    const Dims d{nx, ny, nz};
    PNM_TRY(pnm::check_dims(d, spacing_xyz, true));
    if (d.n() == 0) return Status::ok();
    if (!sdf || !seg) return Status{PNM_ERR_ARG, "null argument"};
    PNM_TRY(enter(c));
    float* d_sdf = nullptr;
    PNM_TRY(c.buf(pnm::S_SDF, d.n(), &d_sdf));
    int32_t* d_seg = nullptr;
    PNM_TRY(c.buf(pnm::S_SEG, d.n(), &d_seg));
    int64_t dummy = 0;
    int32_t* dp = nullptr;
    pnm::HostXfer xfer;
    CopyDrain drain{c};
    xfer.h_sdf = sdf;
    xfer.h_seg = seg;
    PNM_TRY(do_network(c, d_sdf, d, spacing_xyz, spacing_xyz, nullptr, 0, &dummy, d_seg, false,
                       &dp, &dummy, &xfer));
    if (!xfer.seg_sent)
      PNM_CUDA(cudaMemcpyAsync(seg, d_seg, d.n() * sizeof(int32_t), cudaMemcpyDeviceToHost,
                               c.stream));
    PNM_CUDA(cudaStreamSynchronize(c.stream));
    if (c.copy_stream) PNM_CUDA(cudaStreamSynchronize(c.copy_stream));
    return Status::ok();
  };
  return finish(ctx, run());
}

int pnm_pore_peaks_dev(pnm_ctx* ctx, const float* d_sdf, int32_t nx, int32_t ny, int32_t nz,
                       int32_t* d_voxels, int64_t cap, int64_t* n_peaks) {
  if (!ctx) return PNM_ERR_ARG;
  Ctx& c = ctx->c;
  auto run = [&]() -> Status {
    if (!n_peaks) return Status{PNM_ERR_ARG, "null argument"};
    *n_peaks = 0;
    const Dims d{nx, ny, nz};
    const float unit[3] = {1.0f, 1.0f, 1.0f};  // peaks do not depend on the spacing
    PNM_TRY(pnm::check_dims(d, unit, true));
    if (d.n() == 0) return Status::ok();
    if (!d_sdf || (!d_voxels && cap > 0)) return Status{PNM_ERR_ARG, "null argument"};
    PNM_TRY(enter(c));
    pnm::SegState st;
    PNM_TRY(pnm::run_sdf_pass(c, d_sdf, d, unit, &st));
    int64_t np = 0;
    PNM_TRY(pnm::run_peak_ids(c, st, d_voxels, std::min<int64_t>(cap, kMaxPores), &np));
    np = std::min(np, kMaxPores);
    *n_peaks = np;
    if (np > cap) return Status{PNM_ERR_CAPACITY, "device output capacity too small"};
    return Status::ok();
  };
  return finish(ctx, run());
}

int pnm_segment_volume_dev(pnm_ctx* ctx, const float* d_sdf, int32_t nx, int32_t ny, int32_t nz,
                           const float spacing_xyz[3], int32_t* d_seg) {
  if (!ctx) return PNM_ERR_ARG;
  Ctx& c = ctx->c;
  auto run = [&]() -> Status {
    const Dims d{nx, ny, nz};
    PNM_TRY(pnm::check_dims(d, spacing_xyz, true));
    if (d.n() == 0) return Status::ok();
    if (!d_sdf || !d_seg) return Status{PNM_ERR_ARG, "null argument"};
    PNM_TRY(enter(c));
    int64_t dummy = 0;
    int32_t* dp = nullptr;
    PNM_TRY(do_network(c, d_sdf, d, spacing_xyz, spacing_xyz, nullptr, 0, &dummy, d_seg, false,
                       &dp, &dummy));
    PNM_CUDA(cudaStreamSynchronize(c.stream));
    return Status::ok();
  };
  return finish(ctx, run());
}

int pnm_extract_topology(pnm_ctx* ctx, const int32_t* seg, int32_t nx, int32_t ny, int32_t nz,
                         int32_t** pairs, int64_t* n_pairs) {
  if (!ctx) return PNM_ERR_ARG;
  Ctx& c = ctx->c;
  auto run = [&]() -> Status {
    if (!seg || !pairs || !n_pairs) return Status{PNM_ERR_ARG, "null argument"};
    const Dims d{nx, ny, nz};
    PNM_TRY(pnm::check_dims(d, nullptr, false));
    if (d.n() == 0) {
      *pairs = static_cast<int32_t*>(std::malloc(sizeof(int32_t) * 2));
      *n_pairs = 0;
      return Status::ok();
    }
    PNM_TRY(enter(c));
    int32_t* d_seg = nullptr;
    PNM_TRY(c.buf(pnm::S_SEGIN, d.n(), &d_seg));
    PNM_CUDA(cudaMemcpyAsync(d_seg, seg, d.n() * sizeof(int32_t), cudaMemcpyHostToDevice,
                             c.stream));
    PNM_CUDA(cudaMemsetAsync(c.d_cnt, 0, pnm::CNT_COUNT * sizeof(unsigned), c.stream));
    int32_t* d_pairs = nullptr;
    int64_t m = 0;
    PNM_TRY(pnm::run_topology_of_seg(c, d_seg, d, &d_pairs, &m));
    int32_t* h = static_cast<int32_t*>(std::malloc(sizeof(int32_t) * (2 * m + 2)));
    if (!h) return Status{PNM_ERR_INTERNAL, "out of host memory"};
    if (m) PNM_CUDA(cudaMemcpyAsync(h, d_pairs, 2 * m * sizeof(int32_t), cudaMemcpyDeviceToHost,
                                    c.stream));
    PNM_CUDA(cudaStreamSynchronize(c.stream));
    *pairs = h;
    *n_pairs = m;
    return Status::ok();
  };
  return finish(ctx, run());
}

int pnm_extract_pore_network(pnm_ctx* ctx, const float* sdf, int32_t nx, int32_t ny, int32_t nz,
                             const float origin_xyz[3], const float spacing_xyz[3],
                             pnm_pore** pores, int64_t* n_pores, int32_t* seg, int32_t** pairs,
                             int64_t* n_pairs) {
  if (!ctx) return PNM_ERR_ARG;
  Ctx& c = ctx->c;
  auto run = [&]() -> Status {
    if (!sdf || !origin_xyz || !pores || !n_pores || !seg || !pairs || !n_pairs)
      return Status{PNM_ERR_ARG, "null argument"};
    const Dims d{nx, ny, nz};
    PNM_TRY(pnm::check_dims(d, spacing_xyz, true));
    if (d.n() == 0) {
      *pores = static_cast<pnm_pore*>(std::malloc(sizeof(pnm_pore)));
      *pairs = static_cast<int32_t*>(std::malloc(sizeof(int32_t) * 2));
      *n_pores = 0;
      *n_pairs = 0;
      return Status::ok();
    }
    PNM_TRY(enter(c));
    float* d_sdf = nullptr;
    PNM_TRY(c.buf(pnm::S_SDF, d.n(), &d_sdf));
    pnm_pore* d_pores = nullptr;
    int32_t* d_seg = nullptr;
    PNM_TRY(c.buf(pnm::S_PORES, kMaxPores, &d_pores));
    PNM_TRY(c.buf(pnm::S_SEG, d.n(), &d_seg));
    int64_t np = 0, m = 0;
    int32_t* d_pairs = nullptr;
    // the SDF goes up and the labels come back in z-slabs, overlapped with the pipeline
    pnm::HostXfer xfer;
    CopyDrain drain{c};
    xfer.h_sdf = sdf;
    xfer.h_seg = seg;
    PNM_TRY(do_network(c, d_sdf, d, origin_xyz, spacing_xyz, d_pores, kMaxPores, &np, d_seg, true,
                       &d_pairs, &m, &xfer));
    np = std::min(np, kMaxPores);
    pnm_pore* hp = static_cast<pnm_pore*>(std::malloc(sizeof(pnm_pore) * (np ? np : 1)));
    int32_t* hq = static_cast<int32_t*>(std::malloc(sizeof(int32_t) * (2 * m + 2)));
    if (!hp || !hq) {
      std::free(hp);
      std::free(hq);
      return Status{PNM_ERR_INTERNAL, "out of host memory"};
    }
    if (!xfer.seg_sent)
      PNM_CUDA(cudaMemcpyAsync(seg, d_seg, d.n() * sizeof(int32_t), cudaMemcpyDeviceToHost,
                               c.stream));
    if (np) PNM_CUDA(cudaMemcpyAsync(hp, d_pores, np * sizeof(pnm_pore), cudaMemcpyDeviceToHost,
                                     c.stream));
    if (m) PNM_CUDA(cudaMemcpyAsync(hq, d_pairs, 2 * m * sizeof(int32_t), cudaMemcpyDeviceToHost,
                                    c.stream));
    PNM_CUDA(cudaStreamSynchronize(c.stream));
    if (c.copy_stream) PNM_CUDA(cudaStreamSynchronize(c.copy_stream));
    *pores = hp;
    *n_pores = np;
    *pairs = hq;
    *n_pairs = m;
    return Status::ok();
  };
  return finish(ctx, run());
}

int pnm_extract_pore_network_dev(pnm_ctx* ctx, const float* d_sdf, int32_t nx, int32_t ny,
                                 int32_t nz, const float origin_xyz[3], const float spacing_xyz[3],
                                 pnm_pore* d_pores, int64_t pore_cap, int64_t* n_pores,
                                 int32_t* d_seg, int32_t* d_pairs, int64_t pair_cap,
                                 int64_t* n_pairs) {
  if (!ctx) return PNM_ERR_ARG;
  Ctx& c = ctx->c;
  auto run = [&]() -> Status {
    if (!d_sdf || !origin_xyz || !d_pores || !n_pores || !d_pairs || !n_pairs)
      return Status{PNM_ERR_ARG, "null argument"};
    const Dims d{nx, ny, nz};
    PNM_TRY(pnm::check_dims(d, spacing_xyz, true));
    *n_pores = 0;
    *n_pairs = 0;
    if (d.n() == 0) return Status::ok();
    PNM_TRY(enter(c));
    int64_t np = 0, m = 0;
    int32_t* w_pairs = nullptr;
    const int64_t cap = std::min<int64_t>(pore_cap, kMaxPores);
    PNM_TRY(do_network(c, d_sdf, d, origin_xyz, spacing_xyz, d_pores, cap, &np, d_seg, true,
                       &w_pairs, &m));
    const int64_t np_out = std::min(np, kMaxPores);
    if (m) PNM_CUDA(cudaMemcpyAsync(d_pairs, w_pairs, std::min(m, pair_cap) * 2 * sizeof(int32_t),
                                    cudaMemcpyDeviceToDevice, c.stream));
    PNM_CUDA(cudaStreamSynchronize(c.stream));
    *n_pores = np_out;
    *n_pairs = m;
    if (np_out > pore_cap || m > pair_cap)
      return Status{PNM_ERR_CAPACITY, "device output capacity too small"};
    return Status::ok();
  };
  return finish(ctx, run());
}

int pnm_extract_network_flow(pnm_ctx* ctx, const float* sdf, int32_t nx, int32_t ny, int32_t nz,
                             const float origin_xyz[3], const float spacing_xyz[3],
                             const double* u, const double* v, const double* w, const double* p,
                             const double* ox, const double* oy, const double* oz,
                             const double grad_p_xyz[3], pnm_flow_result** out) {
  if (!ctx) return PNM_ERR_ARG;
  Ctx& c = ctx->c;
  auto run = [&]() -> Status {
    if (!sdf || !origin_xyz || !u || !v || !w || !p || !grad_p_xyz || !out)
      return Status{PNM_ERR_ARG, "null argument"};
    if ((ox == nullptr) != (oy == nullptr) || (ox == nullptr) != (oz == nullptr))
      return Status{PNM_ERR_ARG, "pass all three openness arrays (ox,oy,oz) or none"};
    const Dims d{nx, ny, nz};
    PNM_TRY(pnm::check_dims(d, spacing_xyz, true));
    if (d.n() == 0) {
      *out = static_cast<pnm_flow_result*>(std::calloc(1, sizeof(pnm_flow_result)));
      return Status::ok();
    }
    if (3 * d.n() > (long long)INT_MAX - 8)
      return Status{PNM_ERR_SHAPE, "volume too large for network flow: 3*nx*ny*nz must be < 2^31"};
    PNM_TRY(enter(c));
    float* d_sdf = nullptr;
    PNM_TRY(c.buf(pnm::S_SDF, d.n(), &d_sdf));
    const size_t nb = d.n() * sizeof(double);
    const double* hf[7] = {u, v, w, p, ox, oy, oz};
    const int slots[7] = {pnm::S_U, pnm::S_V, pnm::S_W, pnm::S_P, pnm::S_OX, pnm::S_OY, pnm::S_OZ};
    double* df[7] = {};
    // the SDF goes up in slabs ahead of the SDF pass; the fields follow on the copy stream and
    // arrive while the segmentation runs: openness and velocities first (the face stages wait
    // for them), the pressure last (only the pore pressures and throat dp read it)
    pnm::HostXfer xfer;
    CopyDrain drain{c};
    xfer.h_sdf = sdf;
    for (int i : {4, 5, 6, 0, 1, 2, 3}) {
      if (!hf[i]) continue;
      PNM_TRY(c.buf(slots[i], d.n(), &df[i]));
      xfer.extra.push_back({df[i], hf[i], nb});
    }
    pnm::SegState st;
    PNM_TRY(pnm::run_segmentation(c, d_sdf, d, spacing_xyz, &st, /*all_ascent=*/true, &xfer));
    pnm::FlowInputs in{df[0], df[1], df[2], df[3], df[4], df[5], df[6],
                       {grad_p_xyz[0], grad_p_xyz[1], grad_p_xyz[2]}};
    in.fields_ready = xfer.extra_early;
    in.p_ready = xfer.extra_done;
    pnm::FlowOutputsDev od;
    PNM_TRY(pnm::run_network_flow(c, st, origin_xyz, spacing_xyz, in, &od));
    pnm::FlowOutputsHost o;
    PNM_TRY(pnm::flow_outputs_to_host(c, od, &o));
    record(c, st, 0, 0);
    auto* r = static_cast<pnm_flow_result*>(std::calloc(1, sizeof(pnm_flow_result)));
    if (!r) return Status{PNM_ERR_INTERNAL, "out of host memory"};
    r->n_pores = (int64_t)o.pores.size();
    r->n_throats = (int64_t)o.throat_flow.size();
    r->pores = host_dup(o.pores.data(), o.pores.size());
    r->pore_pressure = host_dup(o.pore_pressure.data(), o.pore_pressure.size());
    r->pore_residual = host_dup(o.pore_residual.data(), o.pore_residual.size());
    r->throats = host_dup(o.throats.data(), o.throats.size());
    r->throat_flow = host_dup(o.throat_flow.data(), o.throat_flow.size());
    r->throat_area = host_dup(o.throat_area.data(), o.throat_area.size());
    r->throat_dp = host_dup(o.throat_dp.data(), o.throat_dp.size());
    *out = r;
    return Status::ok();
  };
  return finish(ctx, run());
}

int pnm_extract_network_flow_dev(pnm_ctx* ctx, const float* d_sdf, int32_t nx, int32_t ny,
                                 int32_t nz, const float origin_xyz[3], const float spacing_xyz[3],
                                 const double* d_u, const double* d_v, const double* d_w,
                                 const double* d_p, const double* d_ox, const double* d_oy,
                                 const double* d_oz, const double grad_p_xyz[3],
                                 pnm_flow_result_dev* out) {
  if (!ctx) return PNM_ERR_ARG;
  Ctx& c = ctx->c;
  auto run = [&]() -> Status {
    if (!d_sdf || !origin_xyz || !d_u || !d_v || !d_w || !d_p || !grad_p_xyz || !out)
      return Status{PNM_ERR_ARG, "null argument"};
    *out = pnm_flow_result_dev{};
    if ((d_ox == nullptr) != (d_oy == nullptr) || (d_ox == nullptr) != (d_oz == nullptr))
      return Status{PNM_ERR_ARG, "pass all three openness arrays (ox,oy,oz) or none"};
    const Dims d{nx, ny, nz};
    PNM_TRY(pnm::check_dims(d, spacing_xyz, true));
    if (d.n() == 0) return Status::ok();
    if (3 * d.n() > (long long)INT_MAX - 8)
      return Status{PNM_ERR_SHAPE, "volume too large for network flow: 3*nx*ny*nz must be < 2^31"};
    PNM_TRY(enter(c));
    pnm::SegState st;
    PNM_TRY(pnm::run_segmentation(c, d_sdf, d, spacing_xyz, &st, /*all_ascent=*/true));
    pnm::FlowInputs in{d_u, d_v, d_w, d_p, d_ox, d_oy, d_oz,
                       {grad_p_xyz[0], grad_p_xyz[1], grad_p_xyz[2]}};
    pnm::FlowOutputsDev od;
    PNM_TRY(pnm::run_network_flow(c, st, origin_xyz, spacing_xyz, in, &od));
    record(c, st, 0, 0);
    out->n_pores = od.np;
    out->n_throats = od.nt;
    out->pores = od.pores;
    out->pore_pressure = od.pore_pressure;
    out->pore_residual = od.pore_residual;
    out->throats = od.throats;
    out->throat_flow = od.throat_flow;
    out->throat_area = od.throat_area;
    out->throat_dp = od.throat_dp;
    return Status::ok();
  };
  return finish(ctx, run());
}

void pnm_flow_result_free(pnm_flow_result* r) {
  if (!r) return;
  std::free(r->pores);
  std::free(r->pore_pressure);
  std::free(r->pore_residual);
  std::free(r->throats);
  std::free(r->throat_flow);
  std::free(r->throat_area);
  std::free(r->throat_dp);
  std::free(r);
}

}  // extern "C"
