// Device primitives shared by the pnm kernels: voxel codes, periodic neighbour arithmetic,
// bounded union-find, warp aggregation, bitmap rank, a three-phase exclusive scan and a stable
// LSD radix sort. Everything is integer work; no floating-point contraction matters here.
#pragma once

#include <cuda_runtime.h>

#include <climits>
#include <cstdint>

#include "pnm_ctx.h"

namespace pnm {

// ---- per-voxel code byte ------------------------------------------------------------------------
// bits 0..4 : ascent direction k = (dz+1)*9 + (dy+1)*3 + (dx+1) of the lexicographic (value,
//             wrapped index) maximum over the voxel and its 26 periodic neighbours; 13 = itself.
// bits 5..6 : class of the voxel under the reference's predicates (pore_extraction.hpp:163-164,
//             :245, :276, :333): PORE sdf>0; MARKER sdf<thr; FLOOD !(sdf>=0) (and not marker);
//             ZERO otherwise (sdf == 0, never labelled).
// bit 7     : flood seed — a FLOOD voxel with at least one MARKER neighbour (first Jacobi sweep).
constexpr int kSelf = 13;
enum : int { CLS_PORE = 0, CLS_MARKER = 1, CLS_FLOOD = 2, CLS_ZERO = 3 };
__host__ __device__ __forceinline__ uint8_t make_code(int dir, int cls, bool seed) {
  return (uint8_t)(dir | (cls << 5) | (seed ? 0x80 : 0));
}
__device__ __forceinline__ int code_dir(uint8_t c) { return c & 31; }
__device__ __forceinline__ int code_cls(uint8_t c) { return (c >> 5) & 3; }
__device__ __forceinline__ bool code_seed(uint8_t c) { return (c & 0x80) != 0; }

// key encoding (int32 per voxel): pore -> basin root voxel id (>= 0); labelled solid -> ~label
// (<= -1); unlabelled -> KEY_NONE; flood voxel awaiting its label -> KEY_PENDING.
constexpr int KEY_NONE = INT_MIN;
constexpr int KEY_PENDING = INT_MIN + 1;
__device__ __forceinline__ bool key_is_solid(int k) { return k < 0 && k > KEY_PENDING; }

// periodic wrap of a coordinate displaced by at most one period
__device__ __forceinline__ int wrap1(int v, int n) { return v < 0 ? v + n : (v >= n ? v - n : v); }

// ---- relaxed memory helpers (union-find reads race with atomicMin writes by design) -------------
__device__ __forceinline__ int ld_relaxed(const int* p) {
  int v;
  asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_relaxed(int* p, int v) {
  asm volatile("st.relaxed.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// A read through L1 that may return an older value of the word (another SM's later store is not
// seen until the line leaves this SM's L1). Used for union-find parents, which only ever move to
// smaller ids of the same set: an older parent is still an ancestor, so a find over such reads
// still ends in the set, and every link re-checks with an atomic that sees the current value.
// Hot words (the roots of big components) are then served by L1 instead of one L2 slice.
__device__ __forceinline__ int ld_cached(const int* p) {
  int v;
  asm volatile("ld.global.ca.s32 %0, [%1];" : "=r"(v) : "l"(p));
  return v;
}

// Bounded find with path halving (ECL-CC style). Parents always point to smaller ids in the same
// set, so a concurrent atomicMin link can only shorten a path; halving stores never break a set.
// It may end on a node that was linked meanwhile (see ld_cached): callers that link re-check
// with the atomic, and after the linking kernel every node's chain ends at the root.
constexpr int kUfLimit = 1 << 22;
__device__ __forceinline__ int uf_find(int* L, int x, unsigned* err) {
  for (int it = 0; it < kUfLimit; ++it) {
    const int p = ld_cached(&L[x]);
    if (p == x) return x;
    const int gp = ld_cached(&L[p]);
    if (gp != p) st_relaxed(&L[x], gp);
    x = gp;
  }
  atomicOr(err, ERRF_UF_LIMIT);
  return x;
}
// Links the sets of a and b; the surviving root is the smaller id, so a fully merged component's
// root is its minimum voxel id (the reference's canonical CCL label, pore_extraction.hpp:217-219).
__device__ __forceinline__ void uf_unite(int* L, int a, int b, unsigned* err) {
  for (int it = 0; it < kUfLimit; ++it) {
    a = uf_find(L, a, err);
    b = uf_find(L, b, err);
    if (a == b) return;
    if (a < b) {
      const int t = a;
      a = b;
      b = t;
    }
    const int old = atomicMin(&L[a], b);
    if (old == a) return;
    a = old;
  }
  atomicOr(err, ERRF_UF_LIMIT);
}

// Links the set of `a` with the set of b and returns the root of the merged set as far as this
// thread knows it. Passing the returned root back as `a` for the next link of the same node
// keeps its find short (a root, or one hop from one).
__device__ __forceinline__ int uf_link(int* L, int a, int b, unsigned* err) {
  for (int it = 0; it < kUfLimit; ++it) {
    a = uf_find(L, a, err);
    b = uf_find(L, b, err);
    if (a == b) return a;
    const int hi = a > b ? a : b, lo = a > b ? b : a;
    const int old = atomicMin(&L[hi], lo);
    if (old == hi) return lo;
    // hi was linked meanwhile: retry from its new parent
    a = old;
    b = lo;
  }
  atomicOr(err, ERRF_UF_LIMIT);
  return a;
}

// Gradient root: follow the ascent pointers (nxt, a voxel id; a local max points at itself) for
// at most 512 moves (pore_extraction.hpp:277-309 and :626-648; MAX_STEPS = 512).
__device__ __forceinline__ int chase_root(const int* __restrict__ nxt, int v) {
  int cur = v;
  for (int s = 0; s < 512; ++s) {
    const int n2 = __ldg(&nxt[cur]);
    if (n2 == cur) break;
    cur = n2;
  }
  return cur;
}

// ---- grid barrier for persistent (cooperatively launched) kernels ---------------------------------
// bar[0] counts arrivals, bar[1] is the generation. Every wait is bounded: after `limit_ns` of
// global time (kBarrierNs unless the context sets another limit) the waiting block sets
// ERRF_BARRIER and returns false, so a kernel whose blocks were not all resident ends with an
// error status instead of spinning. `extra` > 0 makes the barrier wait for that many arrivals
// beyond the grid, which never come: every block's wait runs out (the host's test of this path).
constexpr unsigned long long kBarrierNs = 1000000000ull;  // 1 s
__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ unsigned ld_relaxed_u32(const unsigned* p) {
  unsigned v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ bool grid_barrier(unsigned* bar, unsigned* err,
                                             unsigned long long limit_ns = kBarrierNs,
                                             unsigned extra = 0) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    ok = 1;
    const unsigned gen = ld_acquire_u32(&bar[1]);  // cannot advance before this block arrives
    __threadfence();
    if (atomicAdd(&bar[0], 1u) == gridDim.x - 1 + extra) {
      atomicExch(&bar[0], 0u);
      __threadfence();
      atomicAdd(&bar[1], 1u);
    } else {
      const unsigned long long t0 = global_ns();
      while (ld_acquire_u32(&bar[1]) == gen) {
        if (global_ns() - t0 > limit_ns) {
          atomicOr(err, ERRF_BARRIER);
          ok = 0;
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
  }
  __syncthreads();
  return ok != 0;
}

// ---- warp helpers -------------------------------------------------------------------------------
__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31; }
__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}
// Warp-aggregated append: every active lane with `take` gets a slot in [*cnt, ...).
__device__ __forceinline__ int warp_append(unsigned* cnt, bool take) {
  const unsigned act = __activemask();
  const unsigned m = __ballot_sync(act, take);
  if (!m) return -1;
  const int leader = __ffs(m) - 1;
  unsigned base = 0;
  if ((int)lane_id() == leader) base = atomicAdd(cnt, (unsigned)__popc(m));
  base = __shfl_sync(act, base, leader);
  return take ? (int)(base + __popc(m & lanemask_lt())) : -1;
}

// rank of bit `i` in a bitmap with exclusive word prefix counts
__device__ __forceinline__ unsigned bitmap_rank(const uint32_t* bits, const uint32_t* pref,
                                                long long i) {
  const long long w = i >> 5;
  return pref[w] + __popc(bits[w] & ((1u << (i & 31)) - 1u));
}
__device__ __forceinline__ bool bitmap_test(const uint32_t* bits, long long i) {
  return (bits[i >> 5] >> (i & 31)) & 1u;
}

// ---- three-phase exclusive scan of uint32 values v(i), i < m ------------------------------------
constexpr int SCAN_THREADS = 256;
constexpr int SCAN_ITEMS = 8;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

__device__ __forceinline__ unsigned block_exclusive_sum(unsigned v, unsigned* total) {
  __shared__ unsigned warp_tot[SCAN_THREADS / 32];
  const unsigned lane = lane_id(), wid = threadIdx.x >> 5;
  unsigned x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned y = __shfl_up_sync(0xffffffffu, x, o);
    if ((int)lane >= o) x += y;
  }
  if (lane == 31) warp_tot[wid] = x;
  __syncthreads();
  if (wid == 0) {
    unsigned t = lane < SCAN_THREADS / 32 ? warp_tot[lane] : 0u;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned y = __shfl_up_sync(0xffffffffu, t, o);
      if ((int)lane >= o) t += y;
    }
    if (lane < SCAN_THREADS / 32) warp_tot[lane] = t;
  }
  __syncthreads();
  const unsigned warp_base = wid ? warp_tot[wid - 1] : 0u;
  *total = warp_tot[SCAN_THREADS / 32 - 1];
  __syncthreads();
  return warp_base + x - v;
}

template <class F>
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_reduce(F f, long long m, unsigned* sums) {
  const long long base = (long long)blockIdx.x * SCAN_TILE;
  unsigned s = 0;
#pragma unroll
  for (int j = 0; j < SCAN_ITEMS; ++j) {
    const long long i = base + (long long)j * SCAN_THREADS + threadIdx.x;
    if (i < m) s += f(i);
  }
  unsigned tot;
  block_exclusive_sum(s, &tot);
  if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

// exclusive scan of a[0..k) in place by one block; total -> a[k]
static __global__ void __launch_bounds__(SCAN_THREADS) k_scan_single(unsigned* a, long long k) {
  __shared__ unsigned carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (long long base = 0; base < k; base += SCAN_TILE) {
    unsigned vals[SCAN_ITEMS];
    unsigned s = 0;
#pragma unroll
    for (int j = 0; j < SCAN_ITEMS; ++j) {
      const long long i = base + (long long)threadIdx.x * SCAN_ITEMS + j;
      vals[j] = i < k ? a[i] : 0u;
      s += vals[j];
    }
    unsigned tot;
    unsigned off = block_exclusive_sum(s, &tot) + carry;
#pragma unroll
    for (int j = 0; j < SCAN_ITEMS; ++j) {
      const long long i = base + (long long)threadIdx.x * SCAN_ITEMS + j;
      if (i < k) a[i] = off;
      off += vals[j];
    }
    __syncthreads();
    if (threadIdx.x == 0) carry += tot;
    __syncthreads();
  }
  if (threadIdx.x == 0) a[k] = carry;
}

template <class F>
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_down(F f, long long m, const unsigned* offs,
                                                             unsigned* out) {
  const long long base = (long long)blockIdx.x * SCAN_TILE;
  unsigned vals[SCAN_ITEMS];
  unsigned s = 0;
#pragma unroll
  for (int j = 0; j < SCAN_ITEMS; ++j) {
    const long long i = base + (long long)threadIdx.x * SCAN_ITEMS + j;
    vals[j] = i < m ? f(i) : 0u;
    s += vals[j];
  }
  unsigned tot;
  unsigned off = block_exclusive_sum(s, &tot) + offs[blockIdx.x];
#pragma unroll
  for (int j = 0; j < SCAN_ITEMS; ++j) {
    const long long i = base + (long long)threadIdx.x * SCAN_ITEMS + j;
    if (i < m) out[i] = off;
    off += vals[j];
  }
  if (blockIdx.x == gridDim.x - 1 && threadIdx.x == SCAN_THREADS - 1) out[m] = off;
}

// Exclusive scan: out[i] = sum_{j<i} f(j), out[m] = total. `tmp` needs ceil(m/TILE)+1 entries.
template <class F>
inline void exclusive_scan(F f, long long m, unsigned* out, unsigned* tmp, cudaStream_t s,
                           long long* launches) {
  if (m <= 0) {
    cudaMemsetAsync(out, 0, sizeof(unsigned), s);
    return;
  }
  const long long nb = (m + SCAN_TILE - 1) / SCAN_TILE;
  k_scan_reduce<<<(unsigned)nb, SCAN_THREADS, 0, s>>>(f, m, tmp);
  k_scan_single<<<1, SCAN_THREADS, 0, s>>>(tmp, nb);
  k_scan_down<<<(unsigned)nb, SCAN_THREADS, 0, s>>>(f, m, tmp, out);
  *launches += 3;
}

struct PopcountOf {
  const uint32_t* w;
  __device__ unsigned operator()(long long i) const { return __popc(w[i]); }
};
struct ValueOf {
  const unsigned* v;
  __device__ unsigned operator()(long long i) const { return v[i]; }
};

// ---- stable LSD radix sort of (uint64 key, uint32 value), 8 bits per pass ------------------------
constexpr int RS_THREADS = 256;
constexpr int RS_ROUNDS = 4;
constexpr int RS_TILE = RS_THREADS * RS_ROUNDS;

// m_dev (optional): the live key count on the device, at most m; tiles past it stay empty, so a
// sort sized for a capacity can be enqueued before the count is known (graph capture).
static __global__ void __launch_bounds__(RS_THREADS) k_rs_hist(const uint64_t* keys, long long m,
                                                        int shift, unsigned* hist,
                                                        const unsigned* m_dev) {
  __shared__ unsigned h[256];
  if (m_dev) m = min(m, (long long)*m_dev);
  h[threadIdx.x] = 0;
  __syncthreads();
  const long long base = (long long)blockIdx.x * RS_TILE;
  for (int r = 0; r < RS_ROUNDS; ++r) {
    const long long i = base + (long long)r * RS_THREADS + threadIdx.x;
    if (i < m) atomicAdd(&h[(keys[i] >> shift) & 255u], 1u);
  }
  __syncthreads();
  hist[(long long)threadIdx.x * gridDim.x + blockIdx.x] = h[threadIdx.x];
}

static __global__ void __launch_bounds__(RS_THREADS) k_rs_scatter(const uint64_t* kin, const unsigned* vin,
                                                           uint64_t* kout, unsigned* vout,
                                                           long long m, int shift,
                                                           const unsigned* offs,
                                                           const unsigned* m_dev) {
  __shared__ unsigned base[256];
  if (m_dev) m = min(m, (long long)*m_dev);
  __shared__ unsigned wc[RS_THREADS / 32][257];
  const int wid = threadIdx.x >> 5;
  base[threadIdx.x] = offs[(long long)threadIdx.x * gridDim.x + blockIdx.x];
  const long long tile = (long long)blockIdx.x * RS_TILE;
  for (int r = 0; r < RS_ROUNDS; ++r) {
    for (int j = threadIdx.x; j < (RS_THREADS / 32) * 257; j += RS_THREADS) (&wc[0][0])[j] = 0;
    __syncthreads();
    const long long i = tile + (long long)r * RS_THREADS + threadIdx.x;
    const bool valid = i < m;
    uint64_t k = 0;
    unsigned v = 0;
    int d = 256;
    if (valid) {
      k = kin[i];
      v = vin ? vin[i] : 0u;
      d = (int)((k >> shift) & 255u);
    }
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    const unsigned rank = __popc(peers & lanemask_lt());
    if (valid && rank == 0) wc[wid][d] = __popc(peers);
    __syncthreads();
    {
      unsigned run = base[threadIdx.x];
      for (int w = 0; w < RS_THREADS / 32; ++w) {
        const unsigned cnt = wc[w][threadIdx.x];
        wc[w][threadIdx.x] = run;
        run += cnt;
      }
      base[threadIdx.x] = run;
    }
    __syncthreads();
    if (valid) {
      const unsigned pos = wc[wid][d] + rank;
      kout[pos] = k;
      if (vout) vout[pos] = v;
    }
    __syncthreads();
  }
}

// Sorts keys[0..m) (with optional values) over bits [lo_bit, hi_bit). Ping-pongs between (ka,va)
// and (kb,vb); returns true if the result ended in (kb, vb). hist needs 256*ceil(m/TILE) entries,
// scan_tmp ceil(256*nb/SCAN_TILE)+1.
inline bool radix_sort(uint64_t* ka, unsigned* va, uint64_t* kb, unsigned* vb, long long m,
                       int lo_bit, int hi_bit, unsigned* hist, unsigned* scan_tmp,
                       cudaStream_t s, long long* launches, const unsigned* m_dev = nullptr) {
  if (m <= 1 && !m_dev) return false;
  if (m <= 0) return false;
  const long long nb = (m + RS_TILE - 1) / RS_TILE;
  bool in_b = false;
  for (int sh = lo_bit; sh < hi_bit; sh += 8) {
    uint64_t* ki = in_b ? kb : ka;
    unsigned* vi = in_b ? vb : va;
    uint64_t* ko = in_b ? ka : kb;
    unsigned* vo = in_b ? va : vb;
    k_rs_hist<<<(unsigned)nb, RS_THREADS, 0, s>>>(ki, m, sh, hist, m_dev);
    exclusive_scan(ValueOf{hist}, 256 * nb, hist, scan_tmp, s, launches);
    k_rs_scatter<<<(unsigned)nb, RS_THREADS, 0, s>>>(ki, vi, ko, vo, m, sh, hist, m_dev);
    *launches += 2;
    in_b = !in_b;
  }
  return in_b;
}

}  // namespace pnm
