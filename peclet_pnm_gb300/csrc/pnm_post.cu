// Pore-network post-processing on device-resident flow results (pnm_flow_stats_dev): throat
// conductance g = Q / dp and the network statistics the reference's packing demo prints from the
// extract_network_flow dict (scripts/demo_network_flow_packing.py:44-67): mean / max |Q|,
// mean |dp|, max |pore residual|, the share of throats with g > 0, whether every g is finite,
// and the mass-balance verdict max|res| < 1e-6 max|Q| && all g finite. Pore coordination numbers
// (throats per pore, repeated pairs counted) come with it.
//
// One pass over throats and pores writes g, counts coordination with integer atomics and leaves
// per-block partials; a one-block pass folds the partials in block order. Sums are therefore
// deterministic for a given device (fixed grid), and maxima and counts are exact.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>

#include "pnm_ctx.h"
#include "pnm_device.cuh"

namespace pnm {
namespace {

constexpr int kPostThreads = 256;

struct Partial {
  double sum_q, sum_dp, max_q, max_res;
  unsigned long long n_pos, n_fin;
};

// maximum that propagates NaN, as numpy's max
__device__ __forceinline__ double max_nan(double a, double b) {
  return (a != a || b != b) ? a + b : fmax(a, b);
}

__device__ __forceinline__ void fold(Partial& a, const Partial& b) {
  a.sum_q += b.sum_q;
  a.sum_dp += b.sum_dp;
  a.max_q = max_nan(a.max_q, b.max_q);
  a.max_res = max_nan(a.max_res, b.max_res);
  a.n_pos += b.n_pos;
  a.n_fin += b.n_fin;
}

// fixed-order tree over the block's threads
__device__ void block_fold(Partial& v, Partial* sh) {
  sh[threadIdx.x] = v;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) fold(sh[threadIdx.x], sh[threadIdx.x + w]);
    __syncthreads();
  }
  v = sh[0];
}

__global__ void __launch_bounds__(kPostThreads)
k_flow_stats(long long nt, long long np, const int32_t* __restrict__ throats,
             const double* __restrict__ q, const double* __restrict__ dp,
             const double* __restrict__ res, double* __restrict__ g, int* __restrict__ coord,
             Partial* __restrict__ part) {
  __shared__ Partial sh[kPostThreads];
  Partial v{0.0, 0.0, 0.0, 0.0, 0ull, 0ull};
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < nt; t += stride) {
    const double qt = q[t], dt = dp[t];
    const double gt = qt / dt;  // IEEE division, as numpy's: 0/0 -> NaN, x/0 -> +-inf
    if (g) g[t] = gt;
    v.sum_q += fabs(qt);
    v.sum_dp += fabs(dt);
    v.max_q = max_nan(v.max_q, fabs(qt));
    v.n_pos += gt > 0.0;
    v.n_fin += isfinite(gt) ? 1ull : 0ull;
    const int2 ij = reinterpret_cast<const int2*>(throats)[t];
    if (ij.x >= 1 && ij.x <= np) atomicAdd(&coord[ij.x - 1], 1);
    if (ij.y >= 1 && ij.y <= np) atomicAdd(&coord[ij.y - 1], 1);
  }
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < np; i += stride)
    v.max_res = max_nan(v.max_res, fabs(res[i]));
  block_fold(v, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = v;
}

__global__ void __launch_bounds__(kPostThreads)
k_flow_stats_final(int nblocks, const Partial* __restrict__ part, long long np,
                   const int* __restrict__ coord, Partial* __restrict__ total,
                   int* __restrict__ max_coord) {
  __shared__ Partial sh[kPostThreads];
  __shared__ int mc[kPostThreads];
  Partial v{0.0, 0.0, 0.0, 0.0, 0ull, 0ull};
  for (int b = threadIdx.x; b < nblocks; b += blockDim.x) fold(v, part[b]);
  int m = 0;
  for (long long i = threadIdx.x; i < np; i += blockDim.x) m = max(m, coord[i]);
  mc[threadIdx.x] = m;
  block_fold(v, sh);
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) mc[threadIdx.x] = max(mc[threadIdx.x], mc[threadIdx.x + w]);
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    *total = v;
    *max_coord = mc[0];
  }
}

}  // namespace
}  // namespace pnm

extern "C" int pnm_flow_stats_dev(pnm_ctx* ctx, const pnm_flow_result_dev* r,
                                  double* d_conductance, int32_t* d_coordination,
                                  pnm_flow_stats* out) {
  using namespace pnm;
  if (!ctx) return PNM_ERR_ARG;
  Ctx& c = ctx->c;
  auto run = [&]() -> Status {
    if (!r || !out) return Status{PNM_ERR_ARG, "null argument"};
    const long long np = r->n_pores, nt = r->n_throats;
    if (np < 0 || nt < 0) return Status{PNM_ERR_ARG, "negative count"};
    if ((nt > 0 && (!r->throats || !r->throat_flow || !r->throat_dp)) ||
        (np > 0 && !r->pore_residual))
      return Status{PNM_ERR_ARG, "null result array"};
    if (reinterpret_cast<uintptr_t>(r->throats) % 8 != 0)
      return Status{PNM_ERR_ARG, "throats must be 8-byte aligned (read as int32 pairs)"};
    *out = pnm_flow_stats{};
    out->n_pores = np;
    out->n_throats = nt;
    if (np == 0 && nt == 0) {
      out->mass_balance_ok = 1;
      return Status::ok();
    }
    PNM_CUDA(cudaSetDevice(c.device));
    cudaStream_t s = c.stream;
    int* coord = d_coordination;
    if (!coord) PNM_TRY(c.buf(S_POSTCOORD, np + 1, &coord));
    if (np) PNM_CUDA(cudaMemsetAsync(coord, 0, np * sizeof(int), s));
    const int blocks = (int)std::max<long long>(
        1, std::min<long long>((std::max(nt, np) + kPostThreads - 1) / kPostThreads,
                               (long long)c.sm_count * 8));
    // partials, the folded total and the largest coordination, then pinned-free readback
    Partial* part = nullptr;
    PNM_TRY(c.buf(S_POST, (size_t)blocks + 2, &part));
    Partial* total = part + blocks;
    int* maxc = reinterpret_cast<int*>(total + 1);
    k_flow_stats<<<blocks, kPostThreads, 0, s>>>(nt, np, r->throats, r->throat_flow,
                                                 r->throat_dp, r->pore_residual, d_conductance,
                                                 coord, part);
    ++c.launches;
    k_flow_stats_final<<<1, kPostThreads, 0, s>>>(blocks, part, np, coord, total, maxc);
    ++c.launches;
    PNM_CUDA(cudaGetLastError());
    Partial h{};
    int hmax = 0;
    PNM_CUDA(cudaMemcpyAsync(&h, total, sizeof(Partial), cudaMemcpyDeviceToHost, s));
    PNM_CUDA(cudaMemcpyAsync(&hmax, maxc, sizeof(int), cudaMemcpyDeviceToHost, s));
    PNM_CUDA(cudaStreamSynchronize(s));
    out->mean_abs_flow = nt ? h.sum_q / (double)nt : NAN;
    out->max_abs_flow = nt ? h.max_q : NAN;
    out->mean_abs_dp = nt ? h.sum_dp / (double)nt : NAN;
    out->max_abs_residual = np ? h.max_res : NAN;
    out->n_positive_conductance = (int64_t)h.n_pos;
    out->n_finite_conductance = (int64_t)h.n_fin;
    out->mean_coordination = np ? 2.0 * (double)nt / (double)np : 0.0;
    out->max_coordination = hmax;
    out->mass_balance_ok =
        (np == 0 || h.max_res < 1e-6 * (nt ? h.max_q : 0.0)) && h.n_fin == (unsigned long long)nt;
    return Status::ok();
  };
  const Status st = run();
  ++c.calls;
  if (!st.good()) c.last_error = st.msg;
  return st.code;
}
