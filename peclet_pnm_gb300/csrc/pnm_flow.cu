// Network flow on the segmentation: basin peaks and pore centres, trilinear pore pressures,
// flow basins (gradient ascent from every cell), per-patch throats by a two-tier CCL over the
// compacted interface faces, openness-weighted MAC face fluxes, and throat pressure drops.
//
// Reference: src/pore_extraction.hpp:493-997 (extract_network_flow_k), cited per kernel.
//
// FP64 sums (pore_residual, throat_flow, throat_area, throat centroid moments) are accumulated
// EXACTLY: every term is converted to a 128-bit two's-complement fixed-point integer at a common
// power-of-two scale chosen from a bound on the terms, and integer atomics add them. Integer
// addition is associative, so the sums are independent of thread order (deterministic), and the
// only rounding is the final conversion back to double (correctly rounded). The reference's
// atomic double sums carry order-dependent rounding; they agree with these to their own rounding
// error.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstring>

#include "pnm_ctx.h"
#include "pnm_device.cuh"

namespace pnm {

namespace {

__device__ __forceinline__ int3 coords_of(long long v, int nx, int ny) {
  return make_int3((int)(v % nx), (int)((v / nx) % ny), (int)(v / ((long long)nx * ny)));
}
__device__ __forceinline__ int pmod(int v, int n) {
  const int r = v % n;
  return r < 0 ? r + n : r;
}

// ---- exact 128-bit fixed-point accumulation --------------------------------------------------
struct I128 {
  unsigned long long lo;
  long long hi;
};
// trunc(x * 2^scale) as a 128-bit two's-complement integer, from the bits of x (integer
// instructions only: GB300's FP64 rate is low); 0 for zero, inf and NaN. Exact: the shift of the
// 53-bit significand is clamped at 73, which the chosen scales never reach.
__device__ __forceinline__ I128 to_fixed(double x, int scale) {
  I128 r{0ull, 0ll};
  const unsigned long long bits = (unsigned long long)__double_as_longlong(x);
  const int e = (int)((bits >> 52) & 0x7ffull);
  unsigned long long m = bits & ((1ull << 52) - 1ull);
  if (e == 0x7ff || (e == 0 && m == 0)) return r;
  int sh;
  if (e == 0) {
    sh = 1 - 1075 + scale;  // subnormal: no implicit bit
  } else {
    m |= 1ull << 52;
    sh = e - 1075 + scale;
  }
  unsigned long long mlo, mhi;
  if (sh >= 0) {
    sh = min(sh, 73);
    if (sh >= 64) {
      mlo = 0;
      mhi = m << (sh - 64);
    } else if (sh == 0) {
      mlo = m;
      mhi = 0;
    } else {
      mlo = m << sh;
      mhi = m >> (64 - sh);
    }
  } else {
    mlo = -sh >= 64 ? 0ull : (m >> -sh);  // truncation toward zero of the magnitude
    mhi = 0;
  }
  if (bits >> 63) {  // two's complement negate
    mlo = ~mlo + 1ull;
    mhi = ~mhi + (mlo == 0 ? 1ull : 0ull);
  }
  r.lo = mlo;
  r.hi = (long long)mhi;
  return r;
}
__device__ __forceinline__ I128 add128(I128 a, I128 b) {
  I128 r;
  r.lo = a.lo + b.lo;
  r.hi = a.hi + b.hi + (r.lo < a.lo ? 1 : 0);
  return r;
}
__device__ __forceinline__ void atomic_add128(unsigned long long* acc, I128 v) {
  if (v.lo == 0 && v.hi == 0) return;
  const unsigned long long old = atomicAdd(&acc[0], v.lo);
  const unsigned long long carry = (old + v.lo < old) ? 1ull : 0ull;
  const unsigned long long hi = (unsigned long long)v.hi + carry;
  if (hi) atomicAdd(&acc[1], hi);
}
// Adds each lane's I128 values to acc[k][2*target] for target >= 0. Lanes are summed over runs of
// consecutive lanes with the same target (a segmented scan: 5 shuffle steps), and the last lane of
// each run issues the atomics, so a warp needs one atomic per run instead of one per lane. The
// sums are exact integers, so how lanes are grouped never changes a result.
template <int N>
__device__ __forceinline__ void warp_accumulate(unsigned long long* const (&acc)[N], int target,
                                                I128 (&v)[N]) {
  if (!__any_sync(0xffffffffu, target >= 0)) return;  // no face of this kind in the warp
  const int lane = (int)lane_id();
  const int prev = __shfl_up_sync(0xffffffffu, target, 1);
  const unsigned heads = __ballot_sync(0xffffffffu, lane == 0 || prev != target);
  const int start = 31 - __clz(heads & (0xffffffffu >> (31 - lane)));  // this lane's run start
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
#pragma unroll
    for (int k = 0; k < N; ++k) {
      I128 u;
      u.lo = __shfl_up_sync(0xffffffffu, v[k].lo, o);
      u.hi = __shfl_up_sync(0xffffffffu, v[k].hi, o);
      if (lane - o >= start) v[k] = add128(v[k], u);
    }
  }
  const int next = __shfl_down_sync(0xffffffffu, target, 1);
  if (target >= 0 && (lane == 31 || next != target)) {
#pragma unroll
    for (int k = 0; k < N; ++k) atomic_add128(&acc[k][2 * (long long)target], v[k]);
  }
}
__device__ __forceinline__ double from_fixed(unsigned long long lo, long long hi, int scale) {
  const bool neg = hi < 0;
  unsigned long long mlo = lo, mhi = (unsigned long long)hi;
  if (neg) {
    mlo = ~mlo + 1ull;
    mhi = ~mhi + (mlo == 0 ? 1ull : 0ull);
  }
  double d;
  if (mhi == 0) {
    d = (double)mlo;  // correctly rounded u64 -> double
  } else {
    const int sh = 64 - __clzll((long long)mhi);  // bits of mhi
    unsigned long long top = (mhi << (64 - sh)) | (mlo >> sh);
    if (mlo & ((1ull << sh) - 1ull)) top |= 1ull;  // sticky bit for correct rounding
    d = scalbn((double)top, sh);
  }
  d = scalbn(d, -scale);
  return neg ? -d : d;
}

__device__ __forceinline__ void atomic_max_abs(unsigned long long* slot, double v) {
  const double a = fabs(v);
  if (!(a > 0.0) || !isfinite(a)) return;
  atomicMax(slot, (unsigned long long)__double_as_longlong(a));
}
__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int o = 16; o; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// =============================================================================================
// kernels
// =============================================================================================

// basin peaks (pore_extraction.hpp:527-533): a pore voxel that is its own ascent target is the
// root of its basin; peak[label-1] = voxel. Labels whose root is a walk capped at 512 steps have
// no peak and keep 0 (the zero-initialised view).
__global__ void k_peaks(const uint32_t* __restrict__ peakbits, long long words,
                        const uint8_t* __restrict__ code, const int* __restrict__ seg,
                        int* __restrict__ peak) {
  for (long long w = (long long)blockIdx.x * blockDim.x + threadIdx.x; w < words;
       w += (long long)gridDim.x * blockDim.x) {
    uint32_t b = peakbits[w];
    while (b) {
      const int j = __ffs(b) - 1;
      b &= b - 1;
      const long long v = w * 32 + j;
      if (code_cls(code[v]) == CLS_PORE) peak[seg[v] - 1] = (int)v;
    }
  }
}

// pore centres (:534-566): the extract_pores centroid at the basin peak, radius = sdf(peak)
__device__ __forceinline__ pnm_pore centroid_pore(const float* __restrict__ sdf, Dims d, int ix,
                                                  int iy, int iz, const float* o, const float* s,
                                                  float radius) {
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  float sw = 0.0f, px = 0.0f, py = 0.0f, pz = 0.0f;
  for (int dz = -1; dz <= 1; ++dz)
    for (int dy = -1; dy <= 1; ++dy)
      for (int dx = -1; dx <= 1; ++dx) {
        const long long u = ((long long)wrap1(iz + dz, nz) * ny + wrap1(iy + dy, ny)) * nx +
                            wrap1(ix + dx, nx);
        const float v = sdf[u];
        float w = v > 0.0f ? v : 0.0f;
        w = __fmul_rn(w, w);
        sw = __fadd_rn(sw, w);
        px = __fadd_rn(px, __fmul_rn((float)dx, w));
        py = __fadd_rn(py, __fmul_rn((float)dy, w));
        pz = __fadd_rn(pz, __fmul_rn((float)dz, w));
      }
  float fx = 0.0f, fy = 0.0f, fz = 0.0f;
  if (sw > 1e-6f) {
    fx = __fdiv_rn(px, sw);
    fy = __fdiv_rn(py, sw);
    fz = __fdiv_rn(pz, sw);
  }
  pnm_pore p;
  p.x = __fadd_rn(o[0], __fmul_rn(__fadd_rn((float)ix, fx), s[0]));
  p.y = __fadd_rn(o[1], __fmul_rn(__fadd_rn((float)iy, fy), s[1]));
  p.z = __fadd_rn(o[2], __fmul_rn(__fadd_rn((float)iz, fz), s[2]));
  p.radius = radius;
  return p;
}

struct Geo {
  float o[3], s[3];
};

// centres and trilinear periodic pore pressures (:534-613). g = (x - o)/s is evaluated in float
// and widened, exactly as the reference's float Pore members and float origin/spacing.
__global__ void k_centers_pressure(const float* __restrict__ sdf, Dims d, Geo g,
                                   const int* __restrict__ peak, int np,
                                   const double* __restrict__ p, pnm_pore* __restrict__ pores,
                                   double* __restrict__ ppres) {
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < np; k += gridDim.x * blockDim.x) {
    const int ci = peak[k];
    const int3 c = coords_of(ci, nx, ny);
    const pnm_pore po = centroid_pore(sdf, d, c.x, c.y, c.z, g.o, g.s, sdf[ci]);
    pores[k] = po;
    const double gg[3] = {(double)__fdiv_rn(__fsub_rn(po.x, g.o[0]), g.s[0]),
                          (double)__fdiv_rn(__fsub_rn(po.y, g.o[1]), g.s[1]),
                          (double)__fdiv_rn(__fsub_rn(po.z, g.o[2]), g.s[2])};
    int b[3];
    double f[3];
    for (int a = 0; a < 3; ++a) {
      const double fl = floor(gg[a]);
      b[a] = (int)fl;
      f[a] = __dsub_rn(gg[a], fl);
    }
    double acc = 0.0;
    for (int dz = 0; dz < 2; ++dz)
      for (int dy = 0; dy < 2; ++dy)
        for (int dx = 0; dx < 2; ++dx) {
          const double wx = dx ? f[0] : __dsub_rn(1.0, f[0]);
          const double wy = dy ? f[1] : __dsub_rn(1.0, f[1]);
          const double wz = dz ? f[2] : __dsub_rn(1.0, f[2]);
          const double wt = __dmul_rn(__dmul_rn(wx, wy), wz);
          const long long u = ((long long)pmod(b[2] + dz, nz) * ny + pmod(b[1] + dy, ny)) * nx +
                              pmod(b[0] + dx, nx);
          acc = __dadd_rn(acc, __dmul_rn(wt, p[u]));
        }
    ppres[k] = acc;
  }
}

// flow basins (:621-652): flowLab = seg at the <=512-step ascent root of EVERY cell. Pore voxels
// already carry their root in key[]; other cells chase the ascent pointers.
__global__ void __launch_bounds__(256)
    k_flow_basins(Dims d, const uint8_t* __restrict__ code, const int* __restrict__ nxt,
                  const int* __restrict__ key,
                  const int* __restrict__ seg, int* __restrict__ flowLab) {
  const long long n = d.n();
  for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < n;
       v += (long long)gridDim.x * blockDim.x) {
    const uint8_t c0 = code[v];
    const int root = code_cls(c0) == CLS_PORE ? key[v] : chase_root(nxt, (int)v);
    flowLab[v] = __ldg(&seg[root]);
  }
}

struct FieldPtrs {
  const double *u, *v, *w, *ox, *oy, *oz;
};
__device__ __forceinline__ double openness(const FieldPtrs& f, int dd, long long nb) {
  if (!f.ox) return 1.0;
  return dd == 0 ? f.ox[nb] : (dd == 1 ? f.oy[nb] : f.oz[nb]);
}
__device__ __forceinline__ double velocity(const FieldPtrs& f, int dd, long long nb) {
  return dd == 0 ? f.u[nb] : (dd == 1 ? f.v[nb] : f.w[nb]);
}

// face classification (:681-696): face fid = 3*cell + d is the +d face of the cell; interface if
// the flow labels differ, both are pores (> 0) and the openness (of the +d neighbour's -d face)
// is > 0; core if both cell centres are fluid (sdf > 0). Writes the interface and core bitmaps
// over fids (a warp's 32 cells own exactly three 32-bit words) and the bounds of |q| and |o*A|
// over the differing faces, which fix the fixed-point scales.
__global__ void __launch_bounds__(256)
    k_face_class(Dims d, const uint8_t* __restrict__ code, const int* __restrict__ flowLab,
                 FieldPtrs f, double A0, double A1, double A2, uint32_t* __restrict__ ifbits,
                 uint32_t* __restrict__ corebits, unsigned long long* bounds) {
  const long long n = d.n();
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  const double area[3] = {A0, A1, A2};
  double mq = 0.0, mw = 0.0;
  for (long long base = (long long)blockIdx.x * blockDim.x; base < n;
       base += (long long)gridDim.x * blockDim.x) {
    const long long c = base + threadIdx.x;
    unsigned ib = 0, cb = 0;
    if (c < n) {
      const int3 q = coords_of(c, nx, ny);
      const int a = flowLab[c];
      const bool cpore = code_cls(code[c]) == CLS_PORE;
#pragma unroll
      for (int dd = 0; dd < 3; ++dd) {
        const long long nb = ((long long)(dd == 2 ? wrap1(q.z + 1, nz) : q.z) * ny +
                              (dd == 1 ? wrap1(q.y + 1, ny) : q.y)) * nx +
                             (dd == 0 ? wrap1(q.x + 1, nx) : q.x);
        const int b = flowLab[nb];
        if (a == b) continue;
        const double opn = openness(f, dd, nb);
        const double qv = __dmul_rn(__dmul_rn(opn, velocity(f, dd, nb)), area[dd]);
        mq = fmax(mq, fabs(qv));
        if (a > 0 && b > 0 && opn > 0.0) {
          ib |= 1u << dd;
          mw = fmax(mw, fabs(__dmul_rn(opn, area[dd])));
          if (cpore && code_cls(code[nb]) == CLS_PORE) cb |= 1u << dd;
        }
      }
    }
    const unsigned l = lane_id();
    const long long wbase = (base + (threadIdx.x & ~31u)) * 3 / 32;  // first word of this warp
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const int bit = 32 * j + (int)l;  // face index within the warp's 96 faces
      const int src = bit / 3, dd = bit % 3;
      const unsigned ibs = __shfl_sync(0xffffffffu, ib, src);
      const unsigned cbs = __shfl_sync(0xffffffffu, cb, src);
      const unsigned wi = __ballot_sync(0xffffffffu, (ibs >> dd) & 1u);
      const unsigned wc = __ballot_sync(0xffffffffu, (cbs >> dd) & 1u);
      if (l == 0 && (wbase + j) * 32 < 3 * n) {
        ifbits[wbase + j] = wi;
        corebits[wbase + j] = wc;
      }
    }
  }
  mq = warp_max(mq);
  mw = warp_max(mw);
  if (lane_id() == 0) {
    atomic_max_abs(&bounds[0], mq);
    atomic_max_abs(&bounds[1], mw);
  }
}

// compaction of the interface faces (fid order) with their pair keys (lo << 32 | hi)
__global__ void k_face_compact(Dims d, const uint32_t* __restrict__ ifbits,
                               const unsigned* __restrict__ ifpref, long long words,
                               const int* __restrict__ flowLab, int* __restrict__ fid,
                               unsigned long long* __restrict__ fpair, int* __restrict__ par) {
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  for (long long w = (long long)blockIdx.x * blockDim.x + threadIdx.x; w < words;
       w += (long long)gridDim.x * blockDim.x) {
    uint32_t b = ifbits[w];
    unsigned k = ifpref[w];
    while (b) {
      const int j = __ffs(b) - 1;
      b &= b - 1;
      const long long fl = w * 32 + j;
      const long long c = fl / 3;
      const int dd = (int)(fl % 3);
      const int3 q = coords_of(c, nx, ny);
      const long long nb = ((long long)(dd == 2 ? wrap1(q.z + 1, nz) : q.z) * ny +
                            (dd == 1 ? wrap1(q.y + 1, ny) : q.y)) * nx +
                           (dd == 0 ? wrap1(q.x + 1, nx) : q.x);
      const int a = flowLab[c], bb = flowLab[nb];
      const int lo = a < bb ? a : bb, hi = a < bb ? bb : a;
      fid[k] = (int)fl;
      fpair[k] = ((unsigned long long)(unsigned)lo << 32) | (unsigned)hi;
      par[k] = (int)k;
      ++k;
    }
  }
}

struct FaceIndex {
  const uint32_t* ifbits;
  const unsigned* ifpref;
  const uint32_t* corebits;
  const unsigned long long* fpair;
};

// The reference's adjacency of faces (:711-723, :776-791): face (c, dd) and face (c + dc, d2)
// are adjacent when |2*dc + e_d2 - e_dd|^2 <= 8. For each dd, the 42 admitted (dc, d2) as bytes
// (dz+1) << 6 | (dy+1) << 4 | (dx+1) << 2 | d2, built at compile time.
struct FaceAdjacency {
  uint8_t e[3][42];
};
constexpr FaceAdjacency make_face_adjacency() {
  FaceAdjacency t{};
  for (int dd = 0; dd < 3; ++dd) {
    int k = 0;
    for (int dz = -1; dz <= 1; ++dz)
      for (int dy = -1; dy <= 1; ++dy)
        for (int dx = -1; dx <= 1; ++dx)
          for (int d2 = 0; d2 < 3; ++d2) {
            const int Dx = 2 * dx + (d2 == 0) - (dd == 0);
            const int Dy = 2 * dy + (d2 == 1) - (dd == 1);
            const int Dz = 2 * dz + (d2 == 2) - (dd == 2);
            if (Dx * Dx + Dy * Dy + Dz * Dz > 8) continue;
            if (dx == 0 && dy == 0 && dz == 0 && d2 == dd) continue;
            t.e[dd][k++] = (uint8_t)(((dz + 1) << 6) | ((dy + 1) << 4) | ((dx + 1) << 2) | d2);
          }
  }
  return t;
}
__constant__ FaceAdjacency kFaceAdj = make_face_adjacency();

// Visits every interface face of the same pair adjacent to face (c, dd) over the 27 wrapped
// neighbour cells, calling fn(k2, is_core): a walk over the table, not a test of all 81
// (cell, direction) candidates.
template <class Fn>
__device__ __forceinline__ void for_adjacent_faces(Dims d, const FaceIndex& fx, long long f,
                                                   unsigned long long pk, Fn fn) {
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  const long long c = f / 3;
  const int dd = (int)(f % 3);
  const int3 q = coords_of(c, nx, ny);
  const int xm = wrap1(q.x - 1, nx), xp = wrap1(q.x + 1, nx);
  const long long ym = (long long)wrap1(q.y - 1, ny) * nx, y0 = (long long)q.y * nx,
                  yp = (long long)wrap1(q.y + 1, ny) * nx;
  const long long plane = (long long)nx * ny;
  const long long zm = wrap1(q.z - 1, nz) * plane, z0 = q.z * plane,
                  zp = wrap1(q.z + 1, nz) * plane;
#pragma unroll 1
  for (int i = 0; i < 42; ++i) {
    const unsigned e = kFaceAdj.e[dd][i];
    const unsigned ez = e >> 6, ey = (e >> 4) & 3u, ex = (e >> 2) & 3u, d2 = e & 3u;
    const long long c2 = (ez == 0 ? zm : (ez == 1 ? z0 : zp)) +
                         (ey == 0 ? ym : (ey == 1 ? y0 : yp)) +
                         (ex == 0 ? xm : (ex == 1 ? q.x : xp));
    const long long f2 = 3 * c2 + d2;
    if (f2 == f) continue;  // a wrapped copy of the face itself (an axis of 1 or 2 cells)
    if (!bitmap_test(fx.ifbits, f2)) continue;
    const unsigned k2 = bitmap_rank(fx.ifbits, fx.ifpref, f2);
    if (fx.fpair[k2] != pk) continue;
    fn(k2, bitmap_test(fx.corebits, f2));
  }
}

// Tier unions: core faces with adjacent core faces (core CCL, :699-756) and film faces with
// adjacent film faces (the film components; :763-818). Roots are the minimum compact index,
// which is the minimum fid since compaction preserves fid order.
__global__ void __launch_bounds__(256)
    k_face_unite(Dims d, FaceIndex fx, const int* __restrict__ fid, long long M, int* par,
                 unsigned* err) {
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < M;
       k += (long long)gridDim.x * blockDim.x) {
    const long long f = fid[k];
    const bool core = bitmap_test(fx.corebits, f);
    const unsigned long long pk = fx.fpair[k];
    for_adjacent_faces(d, fx, f, pk, [&](unsigned k2, bool core2) {
      if (core2 == core && (long long)k2 > k) uf_unite(par, (int)k, (int)k2, err);
    });
  }
}

// Roots of the face forest into a separate array: a read-only walk, so no store can overwrite a
// flattened root with a stale ancestor (path-halving stores racing the final writes would).
__global__ void k_face_flatten(long long M, const int* __restrict__ par, int* __restrict__ root,
                               unsigned* err) {
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < M;
       k += (long long)gridDim.x * blockDim.x) {
    int x = (int)k;
    int it = 0;
    for (; it < kUfLimit; ++it) {
      const int p = par[x];
      if (p == x) break;
      x = p;
    }
    if (it == kUfLimit) atomicOr(err, ERRF_UF_LIMIT);
    root[k] = x;
  }
}

// Film attachment: a film component takes the smallest core-patch root adjacent to any of its
// faces — the fixpoint of the reference's min propagation through films (:763-805). Components
// adjacent to no core keep their own minimum (the leftover tier, :807-818).
__global__ void __launch_bounds__(256, 8)
    k_film_attach(Dims d, FaceIndex fx, const int* __restrict__ fid, long long M,
                  const int* __restrict__ par, int* __restrict__ minCore) {
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < M;
       k += (long long)gridDim.x * blockDim.x) {
    const long long f = fid[k];
    if (bitmap_test(fx.corebits, f)) continue;
    const unsigned long long pk = fx.fpair[k];
    const int myroot = par[k];
    for_adjacent_faces(d, fx, f, pk, [&](unsigned k2, bool core2) {
      if (core2) atomicMin(&minCore[myroot], par[k2]);
    });
  }
}

__global__ void k_face_label(long long M, const FaceIndex fx, const int* __restrict__ fid,
                             const int* __restrict__ par, const int* __restrict__ minCore,
                             int* __restrict__ label, unsigned* __restrict__ isroot) {
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < M;
       k += (long long)gridDim.x * blockDim.x) {
    const int r = par[k];
    int l = r;
    if (!bitmap_test(fx.corebits, fid[k]) && minCore[r] != INT_MAX) l = minCore[r];
    label[k] = l;
    isroot[k] = (l == (int)k) ? 1u : 0u;
  }
}

struct IsRoot {
  const unsigned* f;
  __device__ unsigned operator()(long long i) const { return f[i]; }
};

__global__ void k_root_keys(long long M, const unsigned* __restrict__ isroot,
                            const unsigned* __restrict__ rpos,
                            const unsigned long long* __restrict__ fpair, int b,
                            uint64_t* __restrict__ keys, unsigned* __restrict__ vals) {
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < M;
       k += (long long)gridDim.x * blockDim.x) {
    if (!isroot[k]) continue;
    const unsigned long long pk = fpair[k];
    const unsigned lo = (unsigned)(pk >> 32), hi = (unsigned)(pk & 0xffffffffu);
    const unsigned t = rpos[k];
    keys[t] = ((uint64_t)(lo - 1u) << b) | (uint64_t)(hi - 1u);
    vals[t] = (unsigned)k;
  }
}

// throat slots in (pair, root fid) order (:820-862)
__global__ void k_slots(long long nt, const uint64_t* __restrict__ keys,
                        const unsigned* __restrict__ vals, int b, int* __restrict__ slotOf,
                        int* __restrict__ throats) {
  const uint64_t lowmask = (1ull << b) - 1ull;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < nt;
       t += (long long)gridDim.x * blockDim.x) {
    slotOf[vals[t]] = (int)t;
    throats[2 * t] = (int)(keys[t] >> b) + 1;
    throats[2 * t + 1] = (int)(keys[t] & lowmask) + 1;
  }
}

// Face / cell-centre coordinates along one axis: F[2c + h] = o + (c + h/2) * s with the
// reference's roundings (double of the float origin and spacing, :876-900).
__global__ void k_coord_table(double* __restrict__ F, int n, float o, float s) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 2 * n; i += gridDim.x * blockDim.x)
    F[i] = __dadd_rn((double)o, __dmul_rn(__dadd_rn((double)(i >> 1), (i & 1) ? 0.5 : 0.0),
                                          (double)s));
}

struct FluxParams {
  double area[3];
  double L[3];
  float o[3], s[3];
  const double* F[3];  // per axis: F[2c + h] = o + (c + h/2) s, rounded as the reference does
  int N[3];
  int fast[3];     // per axis: |origin| + L small enough for the integer minimum-image test
  int sq, sa, sc;  // fixed-point scales: fluxes/residuals, areas, centroid moments
};

// pore_residual (:883-942) per cell: resid[a-1] += q over every +d face whose flow labels differ
// and resid[b-1] -= q on the other side. A cell takes both roles itself: +q over its own +d faces
// (fields of the +d neighbour, as the reference's face loop reads them) and -q over its -d faces
// (its own fields), so each cell has one target (its own label) and each warp one segmented
// sum. q is rounded the same on both sides and to_fixed(-q) == -to_fixed(q), so the integer
// sums are exactly those of a face-by-face loop.
__global__ void __launch_bounds__(256)
    k_flux_resid(Dims d, const int* __restrict__ flowLab, FieldPtrs f, FluxParams P,
                 unsigned long long* accR) {
  const long long n = d.n();
  const int nx = d.nx, ny = d.ny, nz = d.nz, nxy = nx * ny;
  for (long long base = (long long)blockIdx.x * blockDim.x; base < n;
       base += (long long)gridDim.x * blockDim.x) {
    const long long c = base + threadIdx.x;
    int target = -1;
    I128 sum{0ull, 0ll};
    if (c < n) {
      const int ci = (int)c;
      const int z = ci / nxy, r = ci - z * nxy, y = r / nx, x = r - y * nx;
      const int a = flowLab[ci];
      if (a > 0) {
        target = a - 1;
        int up[3], dn[3];
        up[0] = ci - x + (x + 1 == nx ? 0 : x + 1);
        dn[0] = ci - x + (x == 0 ? nx - 1 : x - 1);
        up[1] = ci + ((y + 1 == ny ? 0 : y + 1) - y) * nx;
        dn[1] = ci + ((y == 0 ? ny - 1 : y - 1) - y) * nx;
        up[2] = ci + ((z + 1 == nz ? 0 : z + 1) - z) * nxy;
        dn[2] = ci + ((z == 0 ? nz - 1 : z - 1) - z) * nxy;
        int bu[3], bd[3];
#pragma unroll
        for (int dd = 0; dd < 3; ++dd) {
          bu[dd] = flowLab[up[dd]];
          bd[dd] = flowLab[dn[dd]];
        }
#pragma unroll
        for (int dd = 0; dd < 3; ++dd) {
          if (bu[dd] != a) {
            const double qv =
                __dmul_rn(__dmul_rn(openness(f, dd, up[dd]), velocity(f, dd, up[dd])), P.area[dd]);
            sum = add128(sum, to_fixed(qv, P.sq));
          }
          if (bd[dd] != a) {
            const double qv =
                __dmul_rn(__dmul_rn(openness(f, dd, ci), velocity(f, dd, ci)), P.area[dd]);
            sum = add128(sum, to_fixed(-qv, P.sq));
          }
        }
      }
    }
    unsigned long long* const r1[1] = {accR};
    I128 v1[1] = {sum};
    warp_accumulate<1>(r1, target, v1);
  }
}

// Throat sums (:883-942) per compacted interface face k (face order): +-q by the pair's order,
// o*A, and the area-weighted centroid moment min-imaged against the lower pore's peak voxel, into
// the face's throat slot. Consecutive faces mostly share a throat: one segmented sum per run.
__global__ void __launch_bounds__(256)
    k_flux_throats(Dims d, long long M, const int* __restrict__ fid,
                   const int* __restrict__ flowLab, FieldPtrs f, const int* __restrict__ label,
                   const int* __restrict__ slotOf, const int* __restrict__ peak, FluxParams P,
                   unsigned long long* accQ, unsigned long long* accA, unsigned long long* accCx,
                   unsigned long long* accCy, unsigned long long* accCz) {
  const int nx = d.nx, ny = d.ny, nz = d.nz, nxy = nx * ny;
  for (long long base = (long long)blockIdx.x * blockDim.x; base < M;
       base += (long long)gridDim.x * blockDim.x) {
    const long long k = base + threadIdx.x;
    int ts = -1;
    I128 vQ{0ull, 0ll}, vA{0ull, 0ll}, vC[3];
    vC[0] = vC[1] = vC[2] = I128{0ull, 0ll};
    if (k < M) {
      const int fl = fid[k];
      const int ci = fl / 3, dd = fl - 3 * ci;
      const int z = ci / nxy, r = ci - z * nxy, y = r / nx, x = r - y * nx;
      const int nb = dd == 0 ? ci - x + (x + 1 == nx ? 0 : x + 1)
                     : dd == 1 ? ci + ((y + 1 == ny ? 0 : y + 1) - y) * nx
                               : ci + ((z + 1 == nz ? 0 : z + 1) - z) * nxy;
      const int a = flowLab[ci], b = flowLab[nb];
      ts = slotOf[label[k]];
      const double opn = openness(f, dd, nb);
      const double area = P.area[dd];
      const double qv = __dmul_rn(__dmul_rn(opn, velocity(f, dd, nb)), area);
      const int lo = a < b ? a : b;
      const double w0 = __dmul_rn(opn, area);
      vQ = to_fixed(a < b ? qv : -qv, P.sq);
      vA = to_fixed(w0, P.sa);
      const int pk = peak[lo - 1];
      const int pz = pk / nxy, pr = pk - pz * nxy, py = pr / nx, px = pr - py * nx;
      const int cc[3] = {x, y, z};
      const int pi[3] = {px, py, pz};
#pragma unroll
      for (int a2 = 0; a2 < 3; ++a2) {
        const double fpv = __ldg(&P.F[a2][2 * cc[a2] + (dd == a2 ? 1 : 0)]);
        const double pcv = __ldg(&P.F[a2][2 * pi[a2]]);
        double dv = __dsub_rn(fpv, pcv);
        // minimum image: k = round(dv / L). In half-voxel units the exact difference is
        // t2 = 2 (c - p) + h; away from |t2| ~ N the rounding errors (< 2^-13 voxel when
        // P.fast[a2]) cannot move dv/L across +-0.5, so k follows from integers
        const int t2 = 2 * (cc[a2] - pi[a2]) + (dd == a2 ? 1 : 0);
        const int at = t2 < 0 ? -t2 : t2;
        if (!P.fast[a2] || (at > P.N[a2] - 2 && at < P.N[a2] + 2)) {
          dv = __dsub_rn(dv, __dmul_rn(P.L[a2], round(__ddiv_rn(dv, P.L[a2]))));
        } else if (at >= P.N[a2] + 2) {
          dv = __dsub_rn(dv, __dmul_rn(P.L[a2], t2 < 0 ? -1.0 : 1.0));
        }
        vC[a2] = to_fixed(__dmul_rn(w0, dv), P.sc);
      }
    }
    unsigned long long* const r5[5] = {accQ, accA, accCx, accCy, accCz};
    I128 v5[5] = {vQ, vA, vC[0], vC[1], vC[2]};
    warp_accumulate<5>(r5, ts, v5);
  }
}

__global__ void k_fixed_to_double(const unsigned long long* __restrict__ acc, long long count,
                                  int scale, double* __restrict__ out) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < count;
       i += (long long)gridDim.x * blockDim.x)
    out[i] = from_fixed(acc[2 * i], (long long)acc[2 * i + 1], scale);
}

struct DpParams {
  float o[3], s[3];
  int N[3];
  double L[3];
  double g[3];
};
// throat_dp (:962-995): two-leg min-image image count from snapped integers, then
// dp = (p_i - p_j) - sum_a g_a ((x_j - x_i) - L_a k_a); no contraction.
__global__ void k_throat_dp(long long nt, const int* __restrict__ throats,
                            const pnm_pore* __restrict__ pores, const double* __restrict__ ppres,
                            const int* __restrict__ peak, const double* __restrict__ A,
                            const double* __restrict__ Cx, const double* __restrict__ Cy,
                            const double* __restrict__ Cz, DpParams P, double* __restrict__ dp) {
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < nt;
       t += (long long)gridDim.x * blockDim.x) {
    const int li = throats[2 * t], lj = throats[2 * t + 1];
    const pnm_pore pi = pores[li - 1], pj = pores[lj - 1];
    const double aw = A[t];
    const int pk = peak[li - 1], pkj = peak[lj - 1];
    const int ci[3] = {pk % P.N[0], (pk / P.N[0]) % P.N[1], pk / (P.N[0] * P.N[1])};
    const int cj[3] = {pkj % P.N[0], (pkj / P.N[0]) % P.N[1], pkj / (P.N[0] * P.N[1])};
    const double pip[3] = {(double)pi.x, (double)pi.y, (double)pi.z};
    const double pjp[3] = {(double)pj.x, (double)pj.y, (double)pj.z};
    const double C[3] = {Cx[t], Cy[t], Cz[t]};
    double macro = 0.0;
    for (int a = 0; a < 3; ++a) {
      const double sp = (double)P.s[a];
      const double anc = __dadd_rn((double)P.o[a], __dmul_rn((double)ci[a], sp));
      const double ancj = __dadd_rn((double)P.o[a], __dmul_rn((double)cj[a], sp));
      const double ct = __ddiv_rn(C[a], aw);
      const long long Dc =
          llround(__ddiv_rn(__dsub_rn(ancj, anc), sp)) - llround(__dadd_rn(__ddiv_rn(ct, sp), 1e-6));
      const long long k = llround(__ddiv_rn((double)Dc, (double)P.N[a]));
      const double leg = __dsub_rn(__dsub_rn(pjp[a], pip[a]), __dmul_rn(P.L[a], (double)k));
      macro = __dadd_rn(macro, __dmul_rn(P.g[a], leg));
    }
    dp[t] = __dsub_rn(__dsub_rn(ppres[li - 1], ppres[lj - 1]), macro);
  }
}

__global__ void k_fill_int(int* p, long long m, int v) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < m;
       i += (long long)gridDim.x * blockDim.x)
    p[i] = v;
}

// Blocks of 256 threads of `kernel` resident on one SM (its registers decide): grid-stride
// kernels sized to one wave of them run without a partial second wave.
template <class K>
int resident_per_sm(K kernel) {
  int b = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, kernel, 256, 0) != cudaSuccess) {
    cudaGetLastError();
    return 8;
  }
  return b < 1 ? 1 : b;
}
inline unsigned gridn(long long work, int sm_count, int per_sm = 8) {
  long long b = (work + 255) / 256;
  const long long cap = (long long)sm_count * per_sm;
  if (b > cap) b = cap;
  if (b < 1) b = 1;
  return (unsigned)b;
}

// scale so that 2^31 terms of magnitude <= bound sum below 2^125 (headroom in a signed 128-bit)
inline int fixed_scale(double bound) {
  if (!(bound > 0.0) || !std::isfinite(bound)) return 0;
  int e;
  std::frexp(bound, &e);  // bound < 2^e
  return 125 - 31 - e;
}

}  // namespace

Status run_network_flow(Ctx& c, const SegState& st, const float origin[3], const float spacing[3],
                        const FlowInputs& in, FlowOutputsDev* out) {
  StageScope stage(c, PNM_STAGE_NETWORK_FLOW, "nf::network_flow");
  cudaStream_t s = c.stream;
  const Dims d = st.d;
  const long long n = d.n();
  const int np = st.n_pore_labels;
  *out = FlowOutputsDev{};
  if (np <= 0) return Status::ok();  // no pore label: empty network (:523-524)

  // seg (labels) for the flow-basin lookup
  int32_t* seg = nullptr;
  PNM_TRY(c.buf(S_SEG, n, &seg));
  {
    int32_t* dummy = nullptr;
    int64_t m = 0;
    PNM_TRY(run_seg_and_topology(c, st, seg, false, &dummy, &m));
  }

  int *peak, *flowLab;
  pnm_pore* pores;
  double* ppres;
  PNM_TRY(c.buf(S_PEAK, np, &peak));
  PNM_TRY(c.buf(S_FLOWLAB, n, &flowLab));
  PNM_TRY(c.buf(S_NPORES_OUT, np, &pores));
  PNM_TRY(c.buf(S_PPRES, np, &ppres));
  PNM_CUDA(cudaMemsetAsync(peak, 0, np * sizeof(int), s));
  const long long words = (n + 31) / 32;
  k_peaks<<<gridn(words, c.sm_count), 256, 0, s>>>(st.peakbits, words, st.code, seg, peak); ++c.launches;
  Geo geo;
  for (int a = 0; a < 3; ++a) {
    geo.o[a] = origin[a];
    geo.s[a] = spacing[a];
  }
  k_flow_basins<<<gridn(n, c.sm_count), 256, 0, s>>>(d, st.code, st.nxt, st.key, seg, flowLab); ++c.launches;
  PNM_CUDA(cudaGetLastError());

  // face classification + bounds
  const long long nf = 3 * n;
  const long long fwords = (nf + 31) / 32;
  uint32_t *ifbits, *corebits;
  unsigned *ifpref, *scan0;
  unsigned long long* bounds;
  PNM_TRY(c.buf(S_FBITS, fwords + 1, &ifbits));
  PNM_TRY(c.buf(S_FCORE, fwords + 1, &corebits));
  PNM_TRY(c.buf(S_FPREF, fwords + 1, &ifpref));
  PNM_TRY(c.buf(S_SCAN0, nf / SCAN_TILE + 2, &scan0));  // bounds every scan below (m <= 3n)
  PNM_TRY(c.buf(S_ACC, 4, &bounds));
  PNM_CUDA(cudaMemsetAsync(bounds, 0, 4 * sizeof(unsigned long long), s));
  const double Ax = (double)spacing[1] * spacing[2], Ay = (double)spacing[0] * spacing[2],
               Az = (double)spacing[0] * spacing[1];  // :869-870
  const FieldPtrs fp{in.u, in.v, in.w, in.ox, in.oy, in.oz};
  if (in.fields_ready) PNM_CUDA(cudaStreamWaitEvent(s, in.fields_ready, 0));
  k_face_class<<<gridn(n, c.sm_count, resident_per_sm(k_face_class)), 256, 0, s>>>(
      d, st.code, flowLab, fp, Ax, Ay, Az, ifbits, corebits, bounds);
  ++c.launches;
  exclusive_scan(PopcountOf{ifbits}, fwords, ifpref, scan0, s, &c.launches);
  PNM_CUDA(cudaGetLastError());
  unsigned M32 = 0;
  unsigned long long hb[2];
  PNM_CUDA(cudaMemcpyAsync(&M32, ifpref + fwords, 4, cudaMemcpyDeviceToHost, s));
  PNM_CUDA(cudaMemcpyAsync(hb, bounds, sizeof(hb), cudaMemcpyDeviceToHost, s));
  PNM_CUDA(cudaStreamSynchronize(s));
  const long long M = M32;
  double bq, bw;
  std::memcpy(&bq, &hb[0], 8);
  std::memcpy(&bw, &hb[1], 8);

  // compaction + two-tier face CCL
  int *fid, *par, *minCore, *label, *slotOf, *throats_d;
  unsigned long long* fpair;
  unsigned *isroot, *rpos;
  const long long Mx = std::max<long long>(M, 1);
  PNM_TRY(c.buf(S_FID, Mx, &fid));
  PNM_TRY(c.buf(S_FPAIR, Mx, &fpair));
  PNM_TRY(c.buf(S_FPAR, Mx, &par));
  int* froot;
  PNM_TRY(c.buf(S_FFILM, Mx, &froot));
  PNM_TRY(c.buf(S_FMINCORE, Mx, &minCore));
  PNM_TRY(c.buf(S_FLABEL, Mx, &label));
  PNM_TRY(c.buf(S_ROOTFLAG, Mx, &isroot));
  PNM_TRY(c.buf(S_TDP, Mx + 1, &rpos));
  PNM_TRY(c.buf(S_SLOTOF, Mx, &slotOf));
  PNM_CUDA(cudaMemsetAsync(&c.d_cnt[CNT_ERR], 0, sizeof(unsigned), s));
  long long nt = 0;
  const FaceIndex fx{ifbits, ifpref, corebits, fpair};
  int b = 1;
  while ((1ll << b) < (long long)np) ++b;  // pore labels 1..np -> (label-1) in b bits
  if (M > 0) {
    k_face_compact<<<gridn(fwords, c.sm_count), 256, 0, s>>>(d, ifbits, ifpref, fwords, flowLab,
                                                             fid, fpair, par); ++c.launches;
    k_face_unite<<<gridn(M, c.sm_count), 256, 0, s>>>(d, fx, fid, M, par, &c.d_cnt[CNT_ERR]); ++c.launches;
    k_face_flatten<<<gridn(M, c.sm_count), 256, 0, s>>>(M, par, froot, &c.d_cnt[CNT_ERR]); ++c.launches;
    par = froot;  // every later reader wants the flattened roots
    k_fill_int<<<gridn(M, c.sm_count), 256, 0, s>>>(minCore, M, INT_MAX); ++c.launches;
    k_film_attach<<<gridn(M, c.sm_count), 256, 0, s>>>(d, fx, fid, M, par, minCore); ++c.launches;
    k_face_label<<<gridn(M, c.sm_count), 256, 0, s>>>(M, fx, fid, par, minCore, label, isroot); ++c.launches;
    exclusive_scan(IsRoot{isroot}, M, rpos, scan0, s, &c.launches);
    PNM_CUDA(cudaGetLastError());
    unsigned nt32 = 0;
    PNM_CUDA(cudaMemcpyAsync(&nt32, rpos + M, 4, cudaMemcpyDeviceToHost, s));
    PNM_TRY(c.read_counters());
    if (c.h_cnt[CNT_ERR] & ERRF_UF_LIMIT)
      return Status{PNM_ERR_NOT_CONVERGED, "face union-find exceeded its iteration limit"};
    nt = nt32;
  }

  // throat order (pair, root fid): roots are listed in fid order; a stable sort by pair keeps it
  PNM_TRY(c.buf(S_THROATS, 2 * std::max<long long>(nt, 1), &throats_d));
  if (nt > 0) {
    uint64_t *ka, *kb;
    unsigned *va, *vb, *hist, *stmp;
    PNM_TRY(c.buf(S_KEYS_A, nt, &ka));
    PNM_TRY(c.buf(S_KEYS_B, nt, &kb));
    PNM_TRY(c.buf(S_VALS_A, nt, &va));
    PNM_TRY(c.buf(S_VALS_B, nt, &vb));
    PNM_TRY(c.buf(S_RSHIST, 256 * (nt / RS_TILE + 1) + 1, &hist));
    PNM_TRY(c.buf(S_SCAN1, (256 * (nt / RS_TILE + 1)) / SCAN_TILE + 2, &stmp));
    k_root_keys<<<gridn(M, c.sm_count), 256, 0, s>>>(M, isroot, rpos, fpair, b, ka, va); ++c.launches;
    const bool in_b = radix_sort(ka, va, kb, vb, nt, 0, 2 * b, hist, stmp, s, &c.launches);
    k_slots<<<gridn(nt, c.sm_count), 256, 0, s>>>(nt, in_b ? kb : ka, in_b ? vb : va, b, slotOf,
                                                  throats_d); ++c.launches;
    PNM_CUDA(cudaGetLastError());
  }

  // fluxes: exact fixed-point sums
  FluxParams P;
  P.area[0] = Ax;
  P.area[1] = Ay;
  P.area[2] = Az;
  const int N[3] = {d.nx, d.ny, d.nz};
  double Lmax = 0.0;
  for (int a = 0; a < 3; ++a) {
    P.L[a] = (double)N[a] * spacing[a];  // :876
    P.o[a] = origin[a];
    P.s[a] = spacing[a];
    P.N[a] = N[a];
    // face and peak coordinates carry rounding errors below 4 ulp of |o| + L; the integer test
    // keeps a one-voxel margin, so it applies while that is far below a voxel
    P.fast[a] = (std::fabs((double)origin[a]) + P.L[a]) < std::ldexp((double)spacing[a], 40) &&
                N[a] >= 4;
    Lmax = std::max(Lmax, P.L[a]);
  }
  P.sq = fixed_scale(bq);
  P.sa = fixed_scale(bw);
  P.sc = fixed_scale(bw * (Lmax + 1.0));
  {
    double* F = nullptr;
    PNM_TRY(c.buf(S_COORD, 2 * ((long long)N[0] + N[1] + N[2]), &F));
    long long at = 0;
    for (int a = 0; a < 3; ++a) {
      P.F[a] = F + at;
      k_coord_table<<<(unsigned)std::min<long long>((2 * N[a] + 255) / 256, 1024), 256, 0, s>>>(
          F + at, N[a], P.o[a], P.s[a]);
      ++c.launches;
      at += 2 * (long long)N[a];
    }
  }
  const long long nacc = (long long)np + 5 * std::max<long long>(nt, 1);
  unsigned long long* acc;
  PNM_TRY(c.buf(S_REC, 2 * nacc, &acc));
  PNM_CUDA(cudaMemsetAsync(acc, 0, 2 * nacc * sizeof(unsigned long long), s));
  unsigned long long* accR = acc;
  unsigned long long* accQ = accR + 2 * (long long)np;
  const long long ntx = std::max<long long>(nt, 1);
  unsigned long long* accA = accQ + 2 * ntx;
  unsigned long long* accCx = accA + 2 * ntx;
  unsigned long long* accCy = accCx + 2 * ntx;
  unsigned long long* accCz = accCy + 2 * ntx;
  // pore centres and pressures: the pressure field is the last host upload
  if (in.p_ready) PNM_CUDA(cudaStreamWaitEvent(s, in.p_ready, 0));
  k_centers_pressure<<<gridn(np, c.sm_count), 256, 0, s>>>(st.sdf, d, geo, peak, np, in.p, pores,
                                                           ppres);
  ++c.launches;
  k_flux_resid<<<gridn(n, c.sm_count, resident_per_sm(k_flux_resid)), 256, 0, s>>>(d, flowLab, fp,
                                                                                  P, accR);
  ++c.launches;
  if (M > 0 && nt > 0) {
    k_flux_throats<<<gridn(M, c.sm_count, resident_per_sm(k_flux_throats)), 256, 0, s>>>(
        d, M, fid, flowLab, fp, label, slotOf, peak, P, accQ, accA, accCx, accCy, accCz);
    ++c.launches;
  }
  double* dres;
  PNM_TRY(c.buf(S_FLOWOUT, nacc + ntx, &dres));
  double* resid = dres;
  double* Q = resid + np;
  double* A = Q + ntx;
  double* Cx = A + ntx;
  double* Cy = Cx + ntx;
  double* Cz = Cy + ntx;
  double* dp = Cz + ntx;
  k_fixed_to_double<<<gridn(np, c.sm_count), 256, 0, s>>>(accR, np, P.sq, resid); ++c.launches;
  if (nt > 0) {
    k_fixed_to_double<<<gridn(nt, c.sm_count), 256, 0, s>>>(accQ, nt, P.sq, Q); ++c.launches;
    k_fixed_to_double<<<gridn(nt, c.sm_count), 256, 0, s>>>(accA, nt, P.sa, A); ++c.launches;
    k_fixed_to_double<<<gridn(nt, c.sm_count), 256, 0, s>>>(accCx, nt, P.sc, Cx); ++c.launches;
    k_fixed_to_double<<<gridn(nt, c.sm_count), 256, 0, s>>>(accCy, nt, P.sc, Cy); ++c.launches;
    k_fixed_to_double<<<gridn(nt, c.sm_count), 256, 0, s>>>(accCz, nt, P.sc, Cz); ++c.launches;
    DpParams D;
    for (int a = 0; a < 3; ++a) {
      D.o[a] = origin[a];
      D.s[a] = spacing[a];
      D.N[a] = N[a];
      D.L[a] = P.L[a];
      D.g[a] = in.grad_p[a];
    }
    k_throat_dp<<<gridn(nt, c.sm_count), 256, 0, s>>>(nt, throats_d, pores, ppres, peak, A, Cx,
                                                      Cy, Cz, D, dp); ++c.launches;
  }
  PNM_CUDA(cudaGetLastError());

  out->np = np;
  out->nt = nt;
  out->pores = pores;
  out->pore_pressure = ppres;
  out->pore_residual = resid;
  out->throats = throats_d;
  out->throat_flow = Q;
  out->throat_area = A;
  out->throat_dp = dp;
  return Status::ok();
}

Status flow_outputs_to_host(Ctx& c, const FlowOutputsDev& o, FlowOutputsHost* out) {
  cudaStream_t s = c.stream;
  const long long np = o.np, nt = o.nt;
  *out = FlowOutputsHost{};
  out->pores.resize(np);
  out->pore_pressure.resize(np);
  out->pore_residual.resize(np);
  out->throats.resize(2 * nt);
  out->throat_flow.resize(nt);
  out->throat_area.resize(nt);
  out->throat_dp.resize(nt);
  if (np > 0) {
    PNM_CUDA(cudaMemcpyAsync(out->pores.data(), o.pores, np * sizeof(pnm_pore),
                             cudaMemcpyDeviceToHost, s));
    PNM_CUDA(cudaMemcpyAsync(out->pore_pressure.data(), o.pore_pressure, np * 8,
                             cudaMemcpyDeviceToHost, s));
    PNM_CUDA(cudaMemcpyAsync(out->pore_residual.data(), o.pore_residual, np * 8,
                             cudaMemcpyDeviceToHost, s));
  }
  if (nt > 0) {
    PNM_CUDA(cudaMemcpyAsync(out->throats.data(), o.throats, 2 * nt * 4, cudaMemcpyDeviceToHost, s));
    PNM_CUDA(cudaMemcpyAsync(out->throat_flow.data(), o.throat_flow, nt * 8, cudaMemcpyDeviceToHost,
                             s));
    PNM_CUDA(cudaMemcpyAsync(out->throat_area.data(), o.throat_area, nt * 8, cudaMemcpyDeviceToHost,
                             s));
    PNM_CUDA(cudaMemcpyAsync(out->throat_dp.data(), o.throat_dp, nt * 8, cudaMemcpyDeviceToHost, s));
  }
  PNM_CUDA(cudaStreamSynchronize(s));
  return Status::ok();
}

}  // namespace pnm
