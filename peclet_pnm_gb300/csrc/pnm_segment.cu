// Extraction kernels: SDF pass (pores, ascent pointers, classes, tile-local marker CCL),
// cross-tile CCL merge, resolve (CCL roots, gradient roots, first flood sweep), BFS-layer flood,
// first-appearance renumbering, fused seg write + topology pair emission, and pore compaction.
//
// Reference: src/pore_extraction.hpp (cited per kernel). The integer results are bit-exact with
// it; float pore records are bit-exact because every float operation is an explicit
// round-to-nearest intrinsic in the reference's order (and the library is built with
// -fmad=false).
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <climits>
#include <cstdint>
#include <cstring>

#include "pnm_ctx.h"
#include "pnm_device.cuh"
#include "pnm_geo.cuh"

namespace pnm {

constexpr int TX = 32, TY = 8;  // SDF-pass tile: 32 x 8 x TZ voxels (TZ = 8 unless tuned), 256 threads
// launch shape of the single-volume entry points (the batch path tunes its own)
constexpr int TZ_PLAIN = 16;           // SDF-pass / flood-seed tile depth
constexpr int PLAIN_GRID_PER_SM = 8;  // marker CCL: one wave of resident blocks per SM
constexpr int PLAIN_FLOOD_PER_SM = 4;  // persistent flood loop: resident blocks per SM
constexpr int kBig = INT_MAX;           // unset min-index / non-marker parent

// ---- 1. SDF pass ---------------------------------------------------------------------------
// A 32x8xTZ tile in shared memory with a one-voxel periodic halo; one warp = one 32-voxel x-row
// chunk, each thread walks the z-planes of its column. Per voxel:
//  * ascent direction = lexicographic max of (sdf, wrapped index) over the voxel and its 26
//    neighbours (pore_extraction.hpp:284-304, :632-644); it points at the voxel itself exactly
//    when the voxel is a strict local max (:93-104). Stored as direction bits of `code` and as
//    the neighbour's id in nxt;
//  * class (marker :177, flood :245-248, pore :276), flood seed (has a marker neighbour), peak
//    bit for extract_pores (:89-106): !(sdf <= 0) and the voxel is its own ascent target.
// The lexicographic maximum is taken separably: over x within each halo row, then over y, then
// over z from a three-plane window in registers. The order is total on (value key, wrapped
// index), so the separable maximum is the 27-point one, ties included. Value keys order the
// floats as the reference's comparisons do: -0 == +0, and NaN below every number (a NaN
// neighbour never wins; a NaN voxel stays on itself, as nothing compares above it).
// Marker CCL (:181-230), first half: a marker's union-find parent is the first marker of its run
// inside the 32-voxel chunk (runs are connected), and the chunk's marker bits go to the marker
// bitmap (one word per chunk, bits past the volume's x extent clear) for k_ccl_words.

__device__ __forceinline__ uint32_t ord_key(float v) {
  const uint32_t b = __float_as_uint(v == 0.0f ? 0.0f : v);
  return v != v ? 0u : (b ^ ((b >> 31) ? 0xffffffffu : 0x80000000u));
}
constexpr uint32_t kOrdZero = 0x80000000u;  // ord_key(+-0); 0 is NaN, nothing else maps there
// (o1, p1) above (o0, p0) in (value key, position) order
__device__ __forceinline__ bool key_above(uint32_t o1, uint32_t p1, uint32_t o0, uint32_t p0) {
  return (((uint64_t)o1 << 32) | p1) > (((uint64_t)o0 << 32) | p0);
}

// Candidate (0, 1, 2) = (c-1, c, c+1) of an axis holding the maximum (bits of `m`, at least
// one set) with the largest wrapped coordinate. r: 0 no wrap (c+1 > c > c-1), 1 c == 0 (c-1
// wraps to n-1: c-1 > c+1 > c), 2 c == n-1 (c+1 wraps to 0: c > c-1 > c+1). A table of 2-bit
// answers indexed by (r, m).
__device__ __forceinline__ int pick_ranked(unsigned m, int r) {
  constexpr unsigned long long kLut =
      // r = 0: 2 if bit 2, else 1 if bit 1, else 0
      (0ull << 0) | (0ull << 2) | (1ull << 4) | (1ull << 6) | (2ull << 8) | (2ull << 10) |
      (2ull << 12) | (2ull << 14) |
      // r = 1: order 0, 2, 1
      (0ull << 16) | (0ull << 18) | (1ull << 20) | (0ull << 22) | (2ull << 24) | (0ull << 26) |
      (2ull << 28) | (0ull << 30) |
      // r = 2: order 1, 0, 2
      (0ull << 32) | (0ull << 34) | (1ull << 36) | (1ull << 38) | (2ull << 40) | (0ull << 42) |
      (1ull << 44) | (1ull << 46);
  return (int)((kLut >> (2 * (8 * r + m))) & 3ull);
}

template <bool ALL_ASCENT, class G, int TZ = 8>
__global__ void __launch_bounds__(TX* TY, 8)  // 8 resident tiles per SM (32 registers)
    k_sdf_pass(const float* __restrict__ sdf, G geo, uint8_t* __restrict__ code,
               int* __restrict__ nxt, int* __restrict__ L, uint32_t* __restrict__ peakbits,
               uint32_t* __restrict__ mbits) {
  constexpr int HX = TX + 2, HY = TY + 2, HZ = TZ + 2, NT = TX * TY;
  __shared__ uint32_t so[HZ][HY][HX];     // value keys of the halo tile
  __shared__ int wx[HX], wy[HY], wz[HZ];
  __shared__ unsigned rowm[HZ][HY];  // markers of each halo row at x = X0 .. X0+31
  __shared__ unsigned rowd[HZ][HY];  // the same row's markers at x-1, x or x+1 (x = X0 .. X0+31)
  const Box bx = geo.tile(blockIdx.x, TX, TY, TZ, false);
  const int off = bx.off;  // the volume's first global voxel id: added to every stored id
  const float thr = bx.thr;
  const uint32_t othr = ord_key(thr);
  sdf += off;
  code += off;
  nxt += off;
  L += off;
  peakbits += off >> 5;
  const int nx = bx.nx, ny = bx.ny, nz = bx.nz;
  const int nxy = nx * ny;
  const int X0 = bx.X0, Y0 = bx.Y0, Z0 = bx.Z0;
  const int t = threadIdx.x;
  const int lane = t & 31;  // == tx (TX == 32)
  if (G::kBatch && bx.first) {  // the gap up to the next volume: never-labelled ZERO codes
    const int n = nx * ny * nz;
    for (int i = n + t; i < ((n + 31) & ~31); i += NT) code[i] = make_code(kSelf, CLS_ZERO, false);
  }
  if (t < HX) wx[t] = ((X0 - 1 + t) % nx + nx) % nx;
  if (t < HY) wy[t] = ((Y0 - 1 + t) % ny + ny) % ny;
  if (t < HZ) wz[t] = ((Z0 - 1 + t) % nz + nz) % nz;
  __syncthreads();
  static_assert(NT / 32 < HY, "a warp steps at most one halo plane per row iteration");
  // halo rows and their marker masks: warp w takes rows w, w + 8, ... (plane-major)
  for (int hy = t >> 5, hz = 0; hz < HZ; hy += NT / 32) {
    if (hy >= HY) {
      hy -= HY;
      ++hz;
      if (hz >= HZ) break;
    }
    const float* src = sdf + (wz[hz] * nxy + wy[hy] * nx);
    const float v0 = __ldg(&src[wx[lane + 1]]);
    so[hz][hy][lane + 1] = ord_key(v0);
    float vh = 0.0f;
    if (lane < 2) {
      vh = __ldg(&src[wx[lane == 0 ? 0 : HX - 1]]);
      so[hz][hy][lane == 0 ? 0 : HX - 1] = ord_key(vh);
    }
    const unsigned m = __ballot_sync(0xffffffffu, v0 < thr);
    const unsigned h = __ballot_sync(0xffffffffu, lane < 2 && vh < thr);  // x = X0-1, X0+32
    if (lane == 0) {
      rowm[hz][hy] = m;
      rowd[hz][hy] = m | (m << 1) | (m >> 1) | (h & 1u) | ((h & 2u) << 30);
    }
  }
  __syncthreads();
  const int tx = lane, ty = t >> 5;
  const int gx = X0 + tx, gy = Y0 + ty;
  const bool inxy = gx < nx && gy < ny;
  const unsigned upto = lane == 31 ? 0xffffffffu : ((2u << lane) - 1u);
  // Everything of an output voxel but its ascent direction: class, flood seed, code byte,
  // marker run head and the chunk's marker word.
  auto finish_voxel = [&](int tz, bool valid, int ci, int cls, int bk, unsigned nb) {
    const int gz = Z0 + tz;
    if (valid) {
      const bool seed = cls == CLS_FLOOD && ((nb >> lane) & 1u);
      code[ci] = make_code(bk, cls, seed);
    }
    // marker runs of this chunk row
    const unsigned m = rowm[tz + 1][ty + 1];
    const bool marker = valid && ((m >> lane) & 1u);
    const int hl = marker ? 31 - __clz((m & ~(m << 1)) & upto) : 0;
    const int head = off + gz * nxy + gy * nx + X0 + hl;
    if (valid) L[ci] = marker ? head : kBig;
    if (lane == 0 && gy < ny && gz < nz) {
      const int xe = nx - X0;  // valid x positions of this chunk
      mbits[bx.word0 + (gz * ny + gy) * ((nx + 31) >> 5) + (X0 >> 5)] =
          m & (xe >= 32 ? 0xffffffffu : ((1u << xe) - 1u));
    }
  };
  auto voxel_class = [&](uint32_t oc) {
    return oc > kOrdZero ? CLS_PORE
           : (oc != 0u && oc < othr) ? CLS_MARKER
           : (oc == 0u || oc < kOrdZero) ? CLS_FLOOD
                                         : CLS_ZERO;
  };
  if (nx >= 3 && ny >= 3 && nz >= 3) {  // block-uniform
    // Every axis has three distinct wrapped positions around each voxel, so the lexicographic
    // maximum of (value key, wrapped index) is: the largest value key (a plain 32-bit maximum,
    // separable), then among the candidates holding it the one of largest wrapped index, i.e.
    // the highest-ranked plane, then row, then column. The rank order of (c-1, c, c+1) is
    // natural unless c-1 wraps to n-1 (c == 0: c-1 ranks first) or c+1 wraps to 0
    // (c == n-1: c+1 ranks last). Plane maxima of the last three planes sit in a register
    // window; the winner's row and column are found again from shared memory.
    const int rx = gx == 0 ? 1 : (gx == nx - 1 ? 2 : 0);
    const int ry = gy == 0 ? 1 : (gy == ny - 1 ? 2 : 0);
    auto rowmax = [&](int hz, int hy) {
      const uint32_t* row = &so[hz][hy][lane];
      return max(max(row[0], row[1]), row[2]);
    };
    uint32_t w0 = 0, w1 = 0, w2 = 0;
    unsigned d0 = 0, d1 = 0, d2 = 0;  // marker rows at y-1..y+1 of the last three planes
#pragma unroll 1
    for (int hz = 0; hz < HZ; ++hz) {
      const uint32_t pm = max(max(rowmax(hz, ty), rowmax(hz, ty + 1)), rowmax(hz, ty + 2));
      w0 = w1;
      w1 = w2;
      w2 = pm;
      d0 = d1;
      d1 = d2;
      d2 = rowd[hz][ty] | rowd[hz][ty + 1] | rowd[hz][ty + 2];
      if (hz < 2) continue;
      const int tz = hz - 2;  // output plane: its z-neighbours are the window's planes
      const int gz = Z0 + tz;
      const bool valid = inxy && gz < nz;
      const int ci = gz * nxy + gy * nx + gx;
      const uint32_t oc = so[tz + 1][ty + 1][tx + 1];
      const int cls = voxel_class(oc);
      int bk = kSelf;
      if (valid) {
        const bool up = oc > kOrdZero || oc == 0u;  // !(sdf <= 0): where walks start, peaks sit
        if (ALL_ASCENT || up) {
          int nb = ci;
          if (oc != 0u) {  // a NaN voxel stays on itself
            const uint32_t v = max(max(w0, w1), w2);
            const int rz = gz == 0 ? 1 : (gz == nz - 1 ? 2 : 0);
            const int dz = pick_ranked((w0 == v) | ((w1 == v) << 1) | ((w2 == v) << 2), rz);
            const int pz = tz + dz;
            const int dy = pick_ranked((rowmax(pz, ty) == v) | ((rowmax(pz, ty + 1) == v) << 1) |
                                           ((rowmax(pz, ty + 2) == v) << 2),
                                       ry);
            const uint32_t* row = &so[pz][ty + dy][lane];
            const int dx =
                pick_ranked((row[0] == v) | ((row[1] == v) << 1) | ((row[2] == v) << 2), rx);
            bk = 9 * dz + 3 * dy + dx;
            if (bk != kSelf) nb = wz[pz] * nxy + wy[ty + dy] * nx + wx[lane + dx];
          }
          nxt[ci] = off + nb;
          if (up && bk == kSelf) atomicOr(&peakbits[ci >> 5], 1u << (ci & 31));
        }
      }
      finish_voxel(tz, valid, ci, cls, bk, d0 | d1 | d2);
    }
    return;
  }
  // Volumes with an axis of fewer than three voxels: wrapped neighbours can coincide with each
  // other or with the voxel itself, so candidates are compared as (value key, wrapped index)
  // pairs throughout.
  // x positions of the three candidates of this lane and the y offsets of this warp's rows
  const uint32_t px0 = wx[lane], px1 = wx[lane + 1], px2 = wx[lane + 2];
  const uint32_t py[3] = {(uint32_t)(wy[ty] * nx), (uint32_t)(wy[ty + 1] * nx),
                          (uint32_t)(wy[ty + 2] * nx)};
  uint32_t wo[3] = {0, 0, 0}, wp[3] = {0, 0, 0};  // window: x-y maxima of the last three planes
  int wd[3] = {0, 0, 0};
#pragma unroll 1
  for (int hz = 0; hz < HZ; ++hz) {
    // maximum over the 3x3 (y, x) block of plane hz around this lane
    uint32_t yo = 0, yp = 0;
    int yd = 0;
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const uint32_t* row = &so[hz][ty + j][lane];
      uint32_t o = row[0], q = px0;
      int d = 0;
      const uint32_t o1 = row[1], o2 = row[2];
      if (key_above(o1, px1, o, q)) {
        o = o1;
        q = px1;
        d = 1;
      }
      if (key_above(o2, px2, o, q)) {
        o = o2;
        q = px2;
        d = 2;
      }
      q += py[j];
      if (j == 0 || key_above(o, q, yo, yp)) {
        yo = o;
        yp = q;
        yd = 3 * j + d;
      }
    }
    wo[0] = wo[1];
    wp[0] = wp[1];
    wd[0] = wd[1];
    wo[1] = wo[2];
    wp[1] = wp[2];
    wd[1] = wd[2];
    wo[2] = yo;
    wp[2] = yp + (uint32_t)(wz[hz] * nxy);
    wd[2] = yd;
    if (hz < 2) continue;
    const int tz = hz - 2;  // output plane: its z-neighbours are the window's planes
    const int gz = Z0 + tz;
    const bool valid = inxy && gz < nz;
    const int ci = gz * nxy + gy * nx + gx;
    const uint32_t oc = so[tz + 1][ty + 1][tx + 1];
    const int cls = voxel_class(oc);
    int bk = kSelf;
    if (valid) {
      const bool up = oc > kOrdZero || oc == 0u;  // !(sdf <= 0): where walks start, peaks sit
      if (ALL_ASCENT || up) {
        uint32_t bo = wo[0], bp = wp[0];
        int bd = wd[0];
        if (key_above(wo[1], wp[1], bo, bp)) {
          bo = wo[1];
          bp = wp[1];
          bd = 9 + wd[1];
        }
        if (key_above(wo[2], wp[2], bo, bp)) {
          bo = wo[2];
          bp = wp[2];
          bd = 18 + wd[2];
        }
        // the voxel itself (or a wrapped copy of it) wins, and a NaN voxel stays
        bk = ((int)bp == ci || oc == 0u) ? kSelf : bd;
        nxt[ci] = off + (bk == kSelf ? ci : (int)bp);
        if (up && bk == kSelf) atomicOr(&peakbits[ci >> 5], 1u << (ci & 31));
      }
    }
    unsigned nbm = 0;
    if (__any_sync(0xffffffffu, valid && cls == CLS_FLOOD)) {
#pragma unroll
      for (int k = 0; k < 9; ++k) nbm |= rowd[tz + k / 3][ty + k % 3];
    }
    finish_voxel(tz, valid, ci, cls, bk, nbm);
  }
}

// ---- 2. marker CCL, second half ------------------------------------------------------------
// One thread per marker-bitmap word (a 32-voxel row chunk). For every run of the word (a
// union-find node, identified by its first voxel) it unites the nodes its 13 forward neighbours
// (pore_extraction.hpp:204-206) touch: the next node along +x (across the chunk end, or the
// periodic wrap at the volume end), and in each forward row (dy,dz) = (1,0), (-1,1), (0,1), (1,1)
// the node covering x_start-1 and every node starting in [x_start, x_end+1] (positions wrap).
// Links go straight into the union-find (link to the smaller root), so the surviving root of a
// component is its minimum voxel id, the reference's canonical label (:217-219).
// node (first voxel of the chunk-local run) covering x of row `row` (z * ny + y) of a volume
// starting at voxel `off` with bitmap words vb, or -1
__device__ __forceinline__ int ccl_node_at(const uint32_t* __restrict__ vb, int off, int nx,
                                           int ncx, int row, int x) {
  const int c2 = x >> 5, b = x & 31;
  const uint32_t w = __ldg(&vb[row * ncx + c2]);
  if (!((w >> b) & 1u)) return -1;
  const uint32_t st = w & ~(w << 1);
  return off + row * nx + (c2 << 5) + 31 - __clz(st & ((2u << b) - 1u));
}

template <class G>
__global__ void __launch_bounds__(256)
    k_ccl_words(G geo, const uint32_t* __restrict__ mbits, long long n_words, int* L,
                unsigned* cnt, long long w_begin = 0) {
  // words [w_begin, n_words): a z-slab's words when the links are made slab by slab
  unsigned* err = &cnt[CNT_ERR];
  unsigned links = 0;
  for (long long wi = w_begin + (long long)blockIdx.x * blockDim.x + threadIdx.x; wi < n_words;
       wi += (long long)gridDim.x * blockDim.x) {
    const uint32_t m = __ldg(&mbits[wi]);
    if (!m) continue;
    int off, nx, ny, nz, word0;
    geo.locate_word((int)wi, off, nx, ny, nz, word0);
    const int ncx = (nx + 31) >> 5;
    const int lw = (int)wi - word0;
    const int c = lw % ncx, row = lw / ncx;
    const int y = row % ny, z = row / ny;
    const uint32_t* vb = mbits + word0;
    uint32_t rem = m;
    while (rem) {
      const int p = __ffs(rem) - 1;
      const int len = __ffsll(~(unsigned long long)(rem >> p)) - 1;
      rem &= len == 32 ? 0u : ~(((1u << len) - 1u) << p);
      const int e = p + len - 1;
      const int xs = (c << 5) + p, xe = (c << 5) + e;
      int root = off + row * nx + xs;  // this run's set: carried from link to link
      // +x: the node after the run in this row
      if (xe == nx - 1) {
        const int t = ccl_node_at(vb, off, nx, ncx, row, 0);
        if (t >= 0) {
          root = uf_link(L, root, t, err);
          ++links;
        }
      } else if (e == 31 && (__ldg(&vb[row * ncx + c + 1]) & 1u)) {
        root = uf_link(L, root, off + row * nx + ((c + 1) << 5), err);
        ++links;
      }
#pragma unroll 1
      for (int f = 0; f < 4; ++f) {
        const int dy = (f == 0 || f == 3) ? 1 : (f == 1 ? -1 : 0), dz = f == 0 ? 0 : 1;
        const int row2 = wrap1(z + dz, nz) * ny + wrap1(y + dy, ny);
        const int rowb = off + row2 * nx;
        const int t0 = ccl_node_at(vb, off, nx, ncx, row2, xs == 0 ? nx - 1 : xs - 1);
        if (t0 >= 0) {
          root = uf_link(L, root, t0, err);
          ++links;
        }
        const uint32_t w2 = __ldg(&vb[row2 * ncx + c]);
        const int hi = e + 1 > 31 ? 31 : e + 1;
        uint32_t sm = (w2 & ~(w2 << 1)) & ((2u << hi) - 1u) & ~((1u << p) - 1u);
        while (sm) {
          const int b = __ffs(sm) - 1;
          sm &= sm - 1;
          root = uf_link(L, root, rowb + (c << 5) + b, err);
          ++links;
        }
        if (xe + 1 == nx) {
          const int t = ccl_node_at(vb, off, nx, ncx, row2, 0);
          if (t >= 0) {
            root = uf_link(L, root, t, err);
            ++links;
          }
        } else if (e == 31 && (__ldg(&vb[row2 * ncx + c + 1]) & 1u)) {
          root = uf_link(L, root, rowb + ((c + 1) << 5), err);
          ++links;
        }
      }
    }
  }
#pragma unroll
  for (int o = 16; o; o >>= 1) links += __shfl_xor_sync(0xffffffffu, links, o);
  if ((threadIdx.x & 31) == 0 && links) atomicAdd(&cnt[CNT_EDGES], links);
}

// ---- 3. resolve ----------------------------------------------------------------------------------
// Gradient root of a voxel: follow the ascent pointers for at most 512 moves
// (pore_extraction.hpp:277-309 and :626-648; MAX_STEPS = 512). One thread per voxel, no shared
// memory: a walk's loads mostly hit L1/L2 (neighbouring walks share their upper parts), and the
// block stays small enough for full occupancy, which hides the chains' load latency.
constexpr int RTX = 32, RTY = 8, RTZ = 16;

// For every voxel: marker -> key ~root(CCL), the root joins the key list; pore -> key = gradient
// root, atomicMin of the voxel id into L[root] (its first-appearance index; pore voxels' L started
// at kBig) and, on first touch, the root joins the key list; flood and zero voxels -> KEY_NONE
// (flood labels follow in k_flood_seed). Lanes of a warp hold consecutive voxels of a row; lanes
// whose markers share a union-find parent run one find for the group.
template <class G>
__global__ void __launch_bounds__(RTX* RTY)
    k_resolve(G geo, const uint8_t* __restrict__ code, const int* __restrict__ nxt, int* L,
              int* __restrict__ key, int* __restrict__ keylist, unsigned* cnt) {
  unsigned* err = &cnt[CNT_ERR];
  const Box bx = geo.tile(blockIdx.x, RTX, RTY, RTZ, true);
  const int off = bx.off, nx = bx.nx, ny = bx.ny, nz = bx.nz;
  const int nxy = nx * ny;
  const int lane = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const int gx = bx.X0 + lane, gy = bx.Y0 + ty;
  const bool inxy = gx < nx && gy < ny;
  // the next plane's code byte is loaded while this plane's is used
  uint8_t cnext = (inxy && bx.Z0 < nz) ? __ldg(&code[off + bx.Z0 * nxy + gy * nx + gx]) : 0;
  for (int tz = 0; tz < RTZ; ++tz) {
    const int gz = bx.Z0 + tz;
    const bool valid = inxy && gz < nz;
    const int v = off + gz * nxy + gy * nx + gx;
    const uint8_t c = cnext;
    if (tz + 1 < RTZ) cnext = (inxy && gz + 1 < nz) ? __ldg(&code[v + nxy]) : 0;
    int k = KEY_NONE, agg = -1, par = -1;
    bool new_key = false;
    if (valid) {
      const int cls = code_cls(c);
      if (cls == CLS_MARKER) {
        par = ld_cached(&L[v]);  // the run head, or an ancestor of it
      } else if (cls == CLS_PORE) {
        k = chase_root(nxt, v);
        agg = k;
      }
    }
    {  // one find per run of lanes sharing a parent (lanes hold consecutive voxels)
      const int pp = __shfl_up_sync(0xffffffffu, par, 1);
      const bool lead = par >= 0 && (lane == 0 || pp != par);
      const unsigned leaders = __ballot_sync(0xffffffffu, lead);
      int r = 0;
      if (lead) r = uf_find(L, par, err);
      const int src = 31 - __clz(leaders & (lane == 31 ? 0xffffffffu : ((2u << lane) - 1u)));
      r = __shfl_sync(0xffffffffu, r, src < 0 ? 0 : src);
      if (par >= 0) {
        k = ~r;
        new_key = (r == v);
      }
    }
    if (valid) key[v] = k;
    // first-appearance minimum for pore basins: the first lane of each run of lanes with the same
    // root carries that run's minimum voxel id. L[root] of a pore root only decreases, so a read
    // (possibly older, see ld_cached) at or below v shows the atomic would change nothing.
    const int pa = __shfl_up_sync(0xffffffffu, agg, 1);
    if (agg >= 0 && (lane == 0 || pa != agg) && ld_cached(&L[agg]) > v) {
      const int old = atomicMin(&L[agg], v);
      if (old == kBig) new_key = true;
    }
    const int kpos = warp_append(&cnt[CNT_KEYS], new_key);
    if (new_key) keylist[kpos] = (agg >= 0 ? agg : v);
  }
}

// ---- 4. flood of the shallow solid (the reference's Jacobi sweeps, pore_extraction.hpp:237-269) --
// Sweep 1 labels every flood voxel next to a marker (a "seed") with the smallest neighbouring
// marker label; sweep t labels the still-unlabelled flood voxels adjacent to sweep t-1's with the
// smallest label among neighbours labelled before sweep t. Seeds are labelled from the markers'
// final keys; the remaining flood voxels go to a list U, and deeper layers are discovered from U
// (layer 2) and from each previous layer (t >= 3). Discovery marks a layer PENDING, assignment
// computes its labels into `tmp`, and the next discovery publishes them, so no voxel ever sees a
// same-sweep label — exactly the double-buffered Jacobi sweep.
template <class G, int TZ = 8>
__global__ void __launch_bounds__(TX* TY, 8)
    k_flood_seed(G geo, const uint8_t* __restrict__ code, int* __restrict__ key, int* L,
                 int* __restrict__ ulist, unsigned* cnt) {
  constexpr int HX = TX + 2, HY = TY + 2, HZ = TZ + 2, NT = TX * TY;
  // per halo row: the largest marker key (~root; INT_MIN for non-markers) over x-1..x+1
  __shared__ int xm[HZ][HY][TX];
  __shared__ int wx[HX], wy[HY], wz[HZ];
  const Box bx = geo.tile(blockIdx.x, TX, TY, TZ, false);
  const int off = bx.off;
  code += off;
  key += off;
  const int nx = bx.nx, ny = bx.ny, nz = bx.nz;
  const int nxy = nx * ny;
  const int X0 = bx.X0, Y0 = bx.Y0, Z0 = bx.Z0;
  const int t = threadIdx.x;
  const int lane = t & 31;
  if (t < HX) wx[t] = ((X0 - 1 + t) % nx + nx) % nx;
  if (t < HY) wy[t] = ((Y0 - 1 + t) % ny + ny) % ny;
  if (t < HZ) wz[t] = ((Z0 - 1 + t) % nz + nz) % nz;
  __syncthreads();
  const int hx = lane == 0 ? 0 : HX - 1;
  // lane l holds x = X0-1+l+1; lanes 0 and 1 also hold the halo ends x = X0-1 and X0+32
  auto row_xmax = [&](int r, int km, int kh) {
    int up = __shfl_up_sync(0xffffffffu, km, 1);
    int dn = __shfl_down_sync(0xffffffffu, km, 1);
    const int h1 = __shfl_sync(0xffffffffu, kh, 1);
    if (lane == 0) up = kh;
    if (lane == 31) dn = h1;
    xm[r / HY][r % HY][lane] = max(max(up, km), dn);
  };
  // halo rows, two per warp iteration with all their loads issued before any is used
  for (int r = t >> 5; r < HY * HZ; r += 2 * (NT / 32)) {
    const int r2 = r + NT / 32;  // warp-uniform
    const int rb = wz[r / HY] * nxy + wy[r % HY] * nx;
    const int rb2 = r2 < HY * HZ ? wz[r2 / HY] * nxy + wy[r2 % HY] * nx : rb;
    const uint8_t c0 = __ldg(&code[rb + wx[lane + 1]]);
    const int k0 = __ldg(&key[rb + wx[lane + 1]]);
    const uint8_t c2 = __ldg(&code[rb2 + wx[lane + 1]]);
    const int k2 = __ldg(&key[rb2 + wx[lane + 1]]);
    uint8_t c1 = 0, c3 = 0;
    int k1 = 0, k3 = 0;
    if (lane < 2) {
      c1 = __ldg(&code[rb + wx[hx]]);
      k1 = __ldg(&key[rb + wx[hx]]);
      c3 = __ldg(&code[rb2 + wx[hx]]);
      k3 = __ldg(&key[rb2 + wx[hx]]);
    }
    row_xmax(r, code_cls(c0) == CLS_MARKER ? k0 : INT_MIN,
             code_cls(c1) == CLS_MARKER ? k1 : INT_MIN);
    if (r2 < HY * HZ)
      row_xmax(r2, code_cls(c2) == CLS_MARKER ? k2 : INT_MIN,
               code_cls(c3) == CLS_MARKER ? k3 : INT_MIN);
  }
  __syncthreads();
  const int tx = lane, ty = t >> 5;
  const int gx = X0 + tx, gy = Y0 + ty;
  const bool inxy = gx < nx && gy < ny;
  auto plane_max = [&](int hz) {
    return max(max(xm[hz][ty][tx], xm[hz][ty + 1][tx]), xm[hz][ty + 2][tx]);
  };
  // the 27-voxel maximum is the 26-neighbour one: the voxel itself (flood) holds no marker key
  int w0, w1 = plane_max(0), w2 = plane_max(1);
  // the next plane's code byte is loaded while this plane's is used
  uint8_t cnext = (inxy && Z0 < nz) ? __ldg(&code[Z0 * nxy + gy * nx + gx]) : 0;
  for (int tz = 0; tz < TZ; ++tz) {
    w0 = w1;
    w1 = w2;
    w2 = plane_max(tz + 2);
    const int gz = Z0 + tz;
    const bool valid = inxy && gz < nz;
    const int ci = gz * nxy + gy * nx + gx;
    const uint8_t c = cnext;
    if (tz + 1 < TZ) cnext = (inxy && gz + 1 < nz) ? __ldg(&code[ci + nxy]) : 0;
    bool rest = false;
    if (valid) {
      if (code_cls(c) == CLS_FLOOD) {
        if (code_seed(c)) {
          const int bestk = max(max(w0, w1), w2);  // largest marker key == smallest label
          key[ci] = bestk;
          const int lab = ~bestk;
          // first appearance: the label's minimum starts at its root id L[lab] == lab
          if (off + ci < lab) atomicMin(&L[lab], off + ci);
        } else {
          rest = true;
        }
      }
    }
    const int pos = warp_append(&cnt[CNT_ULIST], rest);
    if (rest) ulist[pos] = off + ci;
  }
}

// Layer 2 with its labels: a listed flood voxel (no marker neighbour) with a seed neighbour joins
// the layer, and its sweep-2 label is already known here: the neighbours labelled before sweep 2
// are the seeds alone (solid keys; the other flood voxels hold KEY_NONE or PENDING, pores their
// basin roots), so the flood loop starts by publishing these labels.
template <class G>
__global__ void __launch_bounds__(256)
    k_flood_layer2(G geo, int* key, const int* __restrict__ ulist, const unsigned* nu_p,
                   int* __restrict__ fout, int* __restrict__ tmp, unsigned* nout_p) {
  const unsigned nu = *nu_p;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < nu;
       i += (long long)gridDim.x * blockDim.x) {
    const int v = ulist[i];
    int off, nx, ny, nz;
    geo.locate(v, off, nx, ny, nz);
    const int lv = v - off;
    const int x = lv % nx, y = (lv / nx) % ny, z = lv / (nx * ny);
    int bestk = INT_MIN;
    for (int dz = -1; dz <= 1; ++dz)
      for (int dy = -1; dy <= 1; ++dy)
        for (int dx = -1; dx <= 1; ++dx) {
          if (!dx && !dy && !dz) continue;
          const int u =
              off + (wrap1(z + dz, nz) * ny + wrap1(y + dy, ny)) * nx + wrap1(x + dx, nx);
          const int k = key[u];
          if (key_is_solid(k)) bestk = max(bestk, k);
        }
    if (bestk != INT_MIN) {
      key[v] = KEY_PENDING;
      const unsigned pos = atomicAdd(nout_p, 1u);
      fout[pos] = v;
      tmp[pos] = ~bestk;
    }
  }
}

// Flood label of a layer voxel v: the smallest label (largest solid key) among its neighbours
// labelled before this sweep. COH: loads bypass L1 (the persistent loop reads what other blocks
// wrote earlier in the same launch).
template <bool COH, class G>
__device__ __forceinline__ int flood_assign_one(const G& geo, const int* key, int v) {
  int off, nx, ny, nz;
  geo.locate(v, off, nx, ny, nz);
  const int lv = v - off;
  const int x = lv % nx, y = (lv / nx) % ny, z = lv / (nx * ny);
  int bestk = INT_MIN;
  for (int dz = -1; dz <= 1; ++dz)
    for (int dy = -1; dy <= 1; ++dy)
      for (int dx = -1; dx <= 1; ++dx) {
        if (!dx && !dy && !dz) continue;
        const int u = off + (wrap1(z + dz, nz) * ny + wrap1(y + dy, ny)) * nx + wrap1(x + dx, nx);
        const int k = COH ? ld_relaxed(&key[u]) : key[u];
        if (key_is_solid(k)) bestk = max(bestk, k);
      }
  return ~bestk;
}

// Publishes v's label and discovers the next layer among its unlabelled flood neighbours.
template <class G>
__device__ __forceinline__ void flood_discover_one(const G& geo, const uint8_t* __restrict__ code,
                                                   int* key, int* L, int v, int lab,
                                                   int* __restrict__ fout, unsigned* nout_p) {
  key[v] = ~lab;
  if (v < lab) atomicMin(&L[lab], v);  // a label's minimum starts at its root id
  int off, nx, ny, nz;
  geo.locate(v, off, nx, ny, nz);
  const int lv = v - off;
  const int x = lv % nx, y = (lv / nx) % ny, z = lv / (nx * ny);
  for (int dz = -1; dz <= 1; ++dz)
    for (int dy = -1; dy <= 1; ++dy)
      for (int dx = -1; dx <= 1; ++dx) {
        if (!dx && !dy && !dz) continue;
        const int u = off + (wrap1(z + dz, nz) * ny + wrap1(y + dy, ny)) * nx + wrap1(x + dx, nx);
        if (code_cls(__ldg(&code[u])) != CLS_FLOOD) continue;
        if (ld_relaxed(&key[u]) != KEY_NONE) continue;
        if (atomicCAS(&key[u], KEY_NONE, KEY_PENDING) == KEY_NONE) {
          const unsigned pos = atomicAdd(nout_p, 1u);
          fout[pos] = u;
        }
      }
}

// publishes the labels of layer t (from tmp) and discovers layer t+1 among its neighbours
template <class G>
__global__ void __launch_bounds__(256)
    k_flood_discover(G geo, const uint8_t* __restrict__ code, int* key, int* L,
                     const int* __restrict__ fin, const unsigned* nin_p, const int* tmp,
                     int* __restrict__ fout, unsigned* nout_p) {
  const unsigned nin = *nin_p;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < nin;
       i += (long long)gridDim.x * blockDim.x)
    flood_discover_one(geo, code, key, L, fin[i], tmp[i], fout, nout_p);
}

template <class G>
__global__ void __launch_bounds__(256)
    k_flood_assign(G geo, const int* __restrict__ key, const int* __restrict__ f,
                   const unsigned* n_p, int* __restrict__ tmp) {
  const unsigned nf = *n_p;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < nf;
       i += (long long)gridDim.x * blockDim.x)
    tmp[i] = flood_assign_one<false>(geo, key, f[i]);
}

// All remaining sweeps in one cooperatively launched kernel: per sweep, assign (layer -> tmp),
// grid barrier, publish + discover (next layer), grid barrier; it ends when a layer is empty, so
// no host round trip sits between sweeps. The frontier starts in (fa, cnt[CNT_FRONT0]);
// cnt[CNT_SWEEPS] receives 1 + the number of layer sweeps.
template <class G>
__global__ void __launch_bounds__(256)
    k_flood_loop(G geo, const uint8_t* __restrict__ code, int* key, int* L, int* fa, int* fb,
                 int* tmp, unsigned* cnt, int max_sweeps, unsigned long long wait_ns,
                 unsigned wait_extra) {
  // the first layer (k_flood_layer2's) arrives with its labels in tmp and an empty (zeroed)
  // next-layer counter, so the first sweep starts at publishing
  unsigned* err = &cnt[CNT_ERR];
  unsigned* bar = &cnt[CNT_BAR0];
  int* fin = fa;
  int* fout = fb;
  int cin = CNT_FRONT0, cout = CNT_FRONT1;
  const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long stride = (long long)gridDim.x * blockDim.x;
  __shared__ unsigned s_nin;
  __shared__ int s_stop;
  int sweeps = 1;
  while (true) {
    if (threadIdx.x == 0) {  // one reading per block keeps every decision block-uniform
      s_nin = ld_relaxed_u32(&cnt[cin]);
      s_stop = s_nin == 0 || (ld_relaxed_u32(err) & ERRF_BARRIER) != 0;
      if (!s_stop && sweeps >= max_sweeps) {
        atomicOr(err, ERRF_FLOOD_LIMIT);
        s_stop = 1;
      }
    }
    __syncthreads();
    const unsigned nin = s_nin;
    if (s_stop) break;
    if (sweeps > 1) {
      for (long long i = tid; i < nin; i += stride)
        tmp[i] = flood_assign_one<true>(geo, key, __ldcg(&fin[i]));
      if (tid == 0) atomicExch(&cnt[cout], 0u);  // read by nobody since the last barrier
      if (!grid_barrier(bar, err, wait_ns, wait_extra)) break;
    }
    for (long long i = tid; i < nin; i += stride)
      flood_discover_one(geo, code, key, L, __ldcg(&fin[i]), __ldcg(&tmp[i]), fout, &cnt[cout]);
    if (!grid_barrier(bar, err, wait_ns, wait_extra)) break;
    int* t = fin;
    fin = fout;
    fout = t;
    const int c = cin;
    cin = cout;
    cout = c;
    ++sweeps;
  }
  if (tid == 0) cnt[CNT_SWEEPS] = (unsigned)sweeps;
}

// ---- 5. first-appearance renumbering (pore_extraction.hpp:319-382) --------------------------------
// Label ids are ranks of each label's minimum voxel id: flag those minima in two bitmaps (pore /
// solid), prefix-count the bitmaps, and write the signed id back into L[key].
// A key voxel k and its label minimum m = L[k] are voxel ids below n_vox whenever the stages
// before ran to completion; an id outside [0, n_vox) (an upstream stage that stopped early) sets
// ERRF_LABEL_RANGE and is skipped instead of indexing the bitmaps with it.
__device__ __forceinline__ bool key_in_range(int k, int m, long long n_vox, unsigned* err) {
  if (k >= 0 && k < n_vox && m >= 0 && m < n_vox) return true;
  atomicOr(err, ERRF_LABEL_RANGE);
  return false;
}

__global__ void k_key_first(const int* __restrict__ keylist, const unsigned* nkeys_p,
                            const int* __restrict__ L, const uint8_t* __restrict__ code,
                            uint32_t* firstP, uint32_t* firstS, long long n_vox, unsigned* err) {
  const unsigned nk = *nkeys_p;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < nk;
       i += (long long)gridDim.x * blockDim.x) {
    const int k = keylist[i];
    if (k < 0 || k >= n_vox) {
      atomicOr(err, ERRF_LABEL_RANGE);
      continue;
    }
    const int m = L[k];
    if (!key_in_range(k, m, n_vox, err)) continue;
    uint32_t* bits = code_cls(code[k]) == CLS_PORE ? firstP : firstS;
    atomicOr(&bits[m >> 5], 1u << (m & 31));
  }
}

template <class G>
__global__ void k_key_id(G geo, const int* __restrict__ keylist, const unsigned* nkeys_p, int* L,
                         const uint8_t* __restrict__ code, const uint32_t* firstP,
                         const unsigned* prefP, const uint32_t* firstS, const unsigned* prefS,
                         long long n_vox, unsigned* err) {
  const unsigned nk = *nkeys_p;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < nk;
       i += (long long)gridDim.x * blockDim.x) {
    const int k = keylist[i];
    if (k < 0 || k >= n_vox) {
      atomicOr(err, ERRF_LABEL_RANGE);
      continue;
    }
    const int m = L[k];
    if (!key_in_range(k, m, n_vox, err)) continue;
    int off, nx, ny, nz;  // ranks count from the volume's first voxel (a word boundary)
    geo.locate(k, off, nx, ny, nz);
    L[k] = code_cls(code[k]) == CLS_PORE
               ? (int)(bitmap_rank(firstP, prefP, m) - prefP[off >> 5]) + 1
               : -(int)(bitmap_rank(firstS, prefS, m) - prefS[off >> 5]) - 1;
  }
}

// ---- 6. seg write + topology pair emission (pore_extraction.hpp:378-381 and :414-431) -----------
__device__ __forceinline__ int label_of_key(const int* __restrict__ L, int k) {
  if (k >= 0) return __ldg(&L[k]);
  if (key_is_solid(k)) return __ldg(&L[~k]);
  return 0;
}
__device__ __forceinline__ uint64_t pair_key(int a, int b) {
  const int lo = a < b ? a : b, hi = a < b ? b : a;
  return ((uint64_t)((uint32_t)lo ^ 0x80000000u) << 32) | (uint64_t)((uint32_t)hi ^ 0x80000000u);
}
constexpr uint64_t kEmpty = ~0ull;  // no valid pair key is all ones (lo < hi)
// Slot hash of a pair key: a 32-bit multiplicative mix of its two halves (the set is kept
// sparse, so a cheap mix is enough; probing is linear).
__device__ __forceinline__ uint32_t pair_hash(uint64_t k) {
  uint32_t h = (uint32_t)(k >> 32) * 0x9e3779b1u ^ (uint32_t)k * 0x85ebca77u;
  return h ^ (h >> 15);
}
constexpr int kMaxProbe = 4096;
// A slot changes once, from kEmpty to its final key, so a read through L1 that returns an older
// value returns kEmpty (and the CAS decides) or that final key; repeated proposals of a popular
// pair are then answered by L1.
__device__ __forceinline__ unsigned long long ld_slot(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.global.ca.u64 %0, [%1];" : "=l"(v) : "l"(p));
  return v;
}
// Inserts k; a new key is counted and, with `dense`, appended there at its count.
__device__ __forceinline__ void hash_insert(unsigned long long* table, uint64_t mask, uint64_t k,
                                            unsigned* err, unsigned* count,
                                            unsigned long long* dense) {
  uint64_t h = pair_hash(k) & mask;
  for (int p = 0; p < kMaxProbe; ++p) {
    const unsigned long long cur = ld_slot(&table[h]);
    if (cur == k) return;
    if (cur == kEmpty) {
      const unsigned long long old = atomicCAS(&table[h], kEmpty, (unsigned long long)k);
      if (old == kEmpty) {
        const unsigned at = atomicAdd(count, 1u);
        if (dense) dense[at] = k;
        return;
      }
      if (old == k) return;
    }
    h = (h + 1) & mask;
  }
  atomicOr(err, ERRF_HASH_FULL);
}

// Label of voxel v for a warp whose lanes hold consecutive voxels of one row: from key[] and
// the id table in L[] — lanes repeating the previous lane's key take the label from the first
// lane of their run instead of gathering it again — or straight from a seg array.
// Labels come as ids (key[] entries, or seg[] labels themselves) and the labels they map to:
// distinct keys have distinct labels (pore roots, marker roots, none), so faces compare ids and
// only differing faces look their labels up. The seg output needs every label: a warp's row of
// ids is mapped with one lookup per run of lanes holding the same id.
struct KeyLabels {
  // faces compare keys, and the set holds key pairs (mapped to label pairs once per unique pair)
  static constexpr bool kKeyPairs = true;
  const int* key;
  const int* L;
  __device__ int id(int v, bool active) const { return active ? __ldg(&key[v]) : KEY_NONE; }
  __device__ int label(int k) const { return label_of_key(L, k); }
  __device__ int labels_warp(int k, bool active) const {
    const unsigned lane = threadIdx.x & 31;
    const int pk = __shfl_up_sync(0xffffffffu, k, 1);
    const bool lead = lane == 0 || pk != k;
    const unsigned leaders = __ballot_sync(0xffffffffu, lead);
    int lab = 0;
    if (lead && active) lab = label_of_key(L, k);
    const int src = 31 - __clz(leaders & (lane == 31 ? 0xffffffffu : ((2u << lane) - 1u)));
    return __shfl_sync(0xffffffffu, lab, src);
  }
  // the same labels for a volume starting at global voxel `off` (keys are global ids)
  __device__ KeyLabels at(int off) const { return KeyLabels{key + off, L}; }
};
struct SegLabels {
  static constexpr bool kKeyPairs = false;
  const int* seg;
  __device__ int id(int v, bool active) const { return active ? __ldg(&seg[v]) : 0; }
  __device__ int label(int k) const { return k; }
  __device__ int labels_warp(int k, bool) const { return k; }
  __device__ SegLabels at(int off) const { return SegLabels{seg + off}; }
};

// One pass over 32 x 8 x 16 bricks (a warp owns a 32-voxel x-row and walks 16 z-planes): seg[v]
// (optional) and every differing (+x,+y,+z) periodic face pair into the hash set. The +x id
// comes from the neighbouring lane, the +z id is carried to the next plane. Lanes proposing the
// pair of the previous lane skip their insert; lab_min/lab_max track the label range. In a
// batch, pair labels are ordered as gbase(volume) + label, so one set holds every volume's pairs
// and sorting it groups them by volume.
constexpr int STX = 32, STY = 8, STZ = 16;
template <class G, class Lab>
__global__ void __launch_bounds__(STX* STY)
    k_seg_topo(G geo, Lab lab_all, int* __restrict__ seg, int want_pairs,
               unsigned long long* table, uint64_t mask, unsigned* cnt, int* range,
               unsigned long long* dense) {
  const Box bx = geo.tile(blockIdx.x, STX, STY, STZ, true);
  const Lab lab = lab_all.at(bx.off);
  if (seg) seg += bx.off;
  const int gb = geo.gbase(bx.vol);
  const int nx = bx.nx, ny = bx.ny, nz = bx.nz;
  const int lane = threadIdx.x & 31;
  const int x = bx.X0 + lane;
  const int y = bx.Y0 + (threadIdx.x >> 5);
  const int z0 = bx.Z0, z1 = min(z0 + STZ, nz);
  const bool in = x < nx && y < ny;
  const int xp = x + 1 >= nx ? 0 : x + 1;
  const int yp = y + 1 >= ny ? 0 : y + 1;
  const int nxy = nx * ny;
  int lmin = INT_MAX, lmax = INT_MIN;
  if (y >= ny) return;  // warp-uniform: a warp is one row
  int kc = lab.id(z0 * nxy + y * nx + x, in);
  int cur = lab.labels_warp(kc, in);
  for (int z = z0; z < z1; ++z) {
    const int row = z * nxy + y * nx;
    const int s0 = cur, k0 = kc;
    if (seg && in) seg[row + x] = s0;
    const int zn = z + 1 >= nz ? 0 : z + 1;
    int kz = 0;
    if (want_pairs || z + 1 < z1) kz = lab.id(zn * nxy + y * nx + x, in);
    if (want_pairs) {
      int kx = __shfl_down_sync(0xffffffffu, k0, 1);
      const int ky = lab.id(z * nxy + yp * nx + x, in);
      if (in && (lane == 31 || x + 1 >= nx)) kx = lab.id(row + xp, true);
#pragma unroll
      for (int dd = 0; dd < 3; ++dd) {
        const int k1 = dd == 0 ? kx : (dd == 1 ? ky : kz);
        uint64_t pk = kEmpty;
        if (in && k1 != k0) {
          if (Lab::kKeyPairs) {
            pk = pair_key(k0, k1);
          } else {
            const int g0 = gb + s0, g1 = gb + lab.label(k1);
            pk = pair_key(g0, g1);
            lmin = min(lmin, min(g0, g1));
            lmax = max(lmax, max(g0, g1));
          }
        }
        const uint64_t pp = __shfl_up_sync(0xffffffffu, pk, 1);
        if (pk != kEmpty && (lane == 0 || pp != pk))
          hash_insert(table, mask, pk, &cnt[CNT_ERR], &cnt[CNT_PAIRS], dense);
      }
    }
    if (z + 1 < z1) {  // warp-uniform
      // a row whose ids all repeat the plane below keeps its labels
      if (!__all_sync(0xffffffffu, kz == kc)) cur = lab.labels_warp(kz, in);
      kc = kz;
    }
  }
  if (want_pairs && !Lab::kKeyPairs) {
#pragma unroll
    for (int o = 16; o; o >>= 1) {
      lmin = min(lmin, __shfl_xor_sync(0xffffffffu, lmin, o));
      lmax = max(lmax, __shfl_xor_sync(0xffffffffu, lmax, o));
    }
    if (lane == 0 && lmin <= lmax) {
      atomicMin(&range[0], lmin);
      atomicMax(&range[1], lmax);
    }
  }
}

struct Occupied {
  const unsigned long long* t;
  __device__ unsigned operator()(long long i) const { return t[i] != kEmpty ? 1u : 0u; }
};

// Gathers the occupied hash slots into dense keys re-encoded as (lo - base) << b | (hi - base):
// at their rank among the occupied slots (pos), or in place (pos == nullptr: a dense key list).
__device__ __forceinline__ long long gather_slot(long long i, const unsigned* pos) {
  return pos ? (long long)pos[i] : i;
}
__global__ void k_hash_gather(const unsigned long long* __restrict__ table, long long cap,
                              const unsigned* __restrict__ pos, const int* range, int b,
                              uint64_t* __restrict__ keys) {
  const int base = range[0];
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < cap;
       i += (long long)gridDim.x * blockDim.x) {
    const unsigned long long k = table[i];
    if (k == kEmpty) continue;
    const int lo = (int)((uint32_t)(k >> 32) ^ 0x80000000u);
    const int hi = (int)((uint32_t)k ^ 0x80000000u);
    const uint32_t dlo = (uint32_t)lo - (uint32_t)base, dhi = (uint32_t)hi - (uint32_t)base;
    keys[gather_slot(i, pos)] = ((uint64_t)dlo << b) | (uint64_t)dhi;
  }
}

// Key pairs -> label pairs: a key's label is its id in L (pore key = basin root; solid key =
// ~label root; KEY_NONE = debris, label 0); in a batch the label is offset by its volume's pair
// base, the volume being that of the pair's voxel key (a KEY_NONE face always pairs with a key of
// its own volume). Then re-encoded as (lo - base) << b | (hi - base) like k_hash_gather.
template <class G>
__global__ void k_hash_gather_keys(const unsigned long long* __restrict__ table, long long cap,
                                   const unsigned* __restrict__ pos, G geo,
                                   const int* __restrict__ L, const int* range, int b,
                                   uint64_t* __restrict__ keys) {
  const int base = range[0];
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < cap;
       i += (long long)gridDim.x * blockDim.x) {
    const unsigned long long k = table[i];
    if (k == kEmpty) continue;
    const int ka = (int)((uint32_t)(k >> 32) ^ 0x80000000u);
    const int kb = (int)((uint32_t)k ^ 0x80000000u);
    const int va = ka >= 0 ? ka : (key_is_solid(ka) ? ~ka : -1);
    const int vb = kb >= 0 ? kb : (key_is_solid(kb) ? ~kb : -1);
    const int vol = geo.vol_of(va >= 0 ? va : vb);
    const int gb = geo.gbase(vol);
    const int la = gb + label_of_key(L, ka), lb = gb + label_of_key(L, kb);
    const int lo = min(la, lb), hi = max(la, lb);
    const uint32_t dlo = (uint32_t)lo - (uint32_t)base, dhi = (uint32_t)hi - (uint32_t)base;
    keys[gather_slot(i, pos)] = ((uint64_t)dlo << b) | (uint64_t)dhi;
  }
}

__global__ void k_pairs_decode(const uint64_t* __restrict__ keys, long long m, const int* range,
                               int b, int* __restrict__ out) {
  const int base = range[0];
  const uint64_t lowmask = (b >= 64) ? ~0ull : ((1ull << b) - 1ull);
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < m;
       i += (long long)gridDim.x * blockDim.x) {
    const uint64_t k = keys[i];
    out[2 * i] = (int)((uint32_t)(k >> b) + (uint32_t)base);
    out[2 * i + 1] = (int)((uint32_t)(k & lowmask) + (uint32_t)base);
  }
}

// ---- 7. pores (pore_extraction.hpp:107-127) -----------------------------------------------------
// The SDF^2-weighted centroid with every float operation rounded exactly as the reference's
// sequence: w = max(v,0)^2; sw += w; p* += d* w in dz->dy->dx order; f = p/sw if sw > 1e-6.
__device__ __forceinline__ pnm_pore make_pore(const float* __restrict__ sdf, Dims d, int ix,
                                              int iy, int iz, float ox, float oy, float oz,
                                              float sx, float sy, float sz, float radius) {
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  float sw = 0.0f, px = 0.0f, py = 0.0f, pz = 0.0f;
  for (int dz = -1; dz <= 1; ++dz)
    for (int dy = -1; dy <= 1; ++dy)
      for (int dx = -1; dx <= 1; ++dx) {
        const long long u = ((long long)wrap1(iz + dz, nz) * ny + wrap1(iy + dy, ny)) * nx +
                            wrap1(ix + dx, nx);
        const float v = __ldg(&sdf[u]);
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
  p.x = __fadd_rn(ox, __fmul_rn(__fadd_rn((float)ix, fx), sx));
  p.y = __fadd_rn(oy, __fmul_rn(__fadd_rn((float)iy, fy), sy));
  p.z = __fadd_rn(oz, __fmul_rn(__fadd_rn((float)iz, fz), sz));
  p.radius = radius;
  return p;
}

// One thread per bitmap word: set bits are peaks in voxel order; pore r = prefix rank.
__global__ void k_pores_emit(const float* __restrict__ sdf, Dims d, const uint32_t* __restrict__ bits,
                             const unsigned* __restrict__ pref, long long words, float ox, float oy,
                             float oz, float sx, float sy, float sz, pnm_pore* __restrict__ out,
                             long long cap) {
  const int nx = d.nx, ny = d.ny;
  for (long long w = (long long)blockIdx.x * blockDim.x + threadIdx.x; w < words;
       w += (long long)gridDim.x * blockDim.x) {
    uint32_t b = bits[w];
    unsigned r = pref[w];
    while (b) {
      const int j = __ffs(b) - 1;
      b &= b - 1;
      if ((long long)r < cap) {
        const long long v = w * 32 + j;
        const int ix = (int)(v % nx), iy = (int)((v / nx) % ny), iz = (int)(v / ((long long)nx * ny));
        out[r] = make_pore(sdf, d, ix, iy, iz, ox, oy, oz, sx, sy, sz, __ldg(&sdf[v]));
      }
      ++r;
    }
  }
}

void launch_pores_emit(const float* sdf, Dims d, const uint32_t* bits, const unsigned* pref,
                       long long words, const float origin[3], const float spacing[3],
                       pnm_pore* out, long long cap, unsigned grid, cudaStream_t s) {
  k_pores_emit<<<grid, 256, 0, s>>>(sdf, d, bits, pref, words, origin[0], origin[1], origin[2],
                                    spacing[0], spacing[1], spacing[2], out, cap);
}

// The voxel id of every set bit of the peak bitmap, at its prefix rank (voxel order): the voxel
// each pore record of k_pores_emit is centred on.
__global__ void k_peak_ids(const uint32_t* __restrict__ bits, const unsigned* __restrict__ pref,
                           long long words, int* __restrict__ out, long long cap) {
  for (long long w = (long long)blockIdx.x * blockDim.x + threadIdx.x; w < words;
       w += (long long)gridDim.x * blockDim.x) {
    uint32_t b = bits[w];
    unsigned r = pref[w];
    while (b) {
      const int j = __ffs(b) - 1;
      b &= b - 1;
      if ((long long)r < cap) out[r] = (int)(w * 32 + j);
      ++r;
    }
  }
}


// ---- 8. batch bookkeeping -----------------------------------------------------------------------
// One pore per set bit of the peak bitmap of a whole batch; a word's volume is found from its
// first voxel (volumes start on word boundaries). Records land at the batch-wide rank, so each
// volume's pores are contiguous and in voxel order.
__global__ void k_pores_emit_batch(const float* __restrict__ sdf, VolTab geo,
                                   const uint32_t* __restrict__ bits,
                                   const unsigned* __restrict__ pref, long long words,
                                   pnm_pore* __restrict__ out, long long cap) {
  for (long long w = (long long)blockIdx.x * blockDim.x + threadIdx.x; w < words;
       w += (long long)gridDim.x * blockDim.x) {
    uint32_t b = bits[w];
    if (!b) continue;
    unsigned r = pref[w];
    const int vol = geo.vol_of((int)(w * 32));
    const VolDesc& vd = geo.v[vol];
    const int off = vd.off;
    const Dims d{vd.nx, vd.ny, vd.nz};
    while (b) {
      const int j = __ffs(b) - 1;
      b &= b - 1;
      if ((long long)r < cap) {
        const int v = (int)(w * 32 + j) - off;
        const int ix = v % d.nx, iy = (v / d.nx) % d.ny, iz = v / (d.nx * d.ny);
        out[r] = make_pore(sdf + off, d, ix, iy, iz, vd.ox, vd.oy, vd.oz, vd.sx, vd.sy, vd.sz,
                           __ldg(&sdf[off + v]));
      }
      ++r;
    }
  }
}

// Pair labels of a batch are gbase + label >= 0: the sort keys count from 0.
__global__ void k_batch_init(int* range) {
  range[0] = 0;
  range[1] = 0;
}

// Per-volume label counts (rank differences over the volume's words) and pair-label bases: an
// exclusive scan of nS + nP + 1 over the volumes, one block.
__global__ void __launch_bounds__(SCAN_THREADS)
    k_batch_labels(const VolDesc* __restrict__ v, VolResult* r, int nvol,
                   const unsigned* __restrict__ prefP, const unsigned* __restrict__ prefS) {
  __shared__ unsigned carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < nvol; base += SCAN_THREADS) {
    const int i = base + threadIdx.x;
    unsigned np = 0, ns = 0;
    if (i < nvol) {
      const long long off = v[i].off, n = (long long)v[i].nx * v[i].ny * v[i].nz;
      const long long w0 = off >> 5, w1 = (off + n + 31) >> 5;
      np = prefP[w1] - prefP[w0];
      ns = prefS[w1] - prefS[w0];
    }
    unsigned tot;
    const unsigned ex = block_exclusive_sum(i < nvol ? np + ns + 1u : 0u, &tot);
    if (i < nvol) {
      r[i].n_pore_labels = np;
      r[i].n_solid_labels = ns;
      r[i].gstart = (int)(carry + ex);
      r[i].gbase = (int)(carry + ex + ns);
    }
    __syncthreads();
    if (threadIdx.x == 0) carry += tot;
    __syncthreads();
  }
}

// Sorted re-encoded pair keys -> (label_a, label_b) of their own volume.
__global__ void k_pairs_decode_batch(const uint64_t* __restrict__ keys, const unsigned* m_p,
                                     const int* range, int b, VolTab geo, int* __restrict__ out) {
  const unsigned m = *m_p;
  const int base = range[0];
  const uint64_t lowmask = (1ull << b) - 1ull;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < m;
       i += (long long)gridDim.x * blockDim.x) {
    const uint64_t k = keys[i];
    const int glo = (int)((uint32_t)(k >> b) + (uint32_t)base);
    const int ghi = (int)((uint32_t)(k & lowmask) + (uint32_t)base);
    const int gb = geo.r[geo.vol_of_label(glo)].gbase;
    out[2 * i] = glo - gb;
    out[2 * i + 1] = ghi - gb;
  }
}

// Per-volume pore and pair ranges; thread 0 also records the batch's peak total.
__global__ void k_batch_tail(const VolDesc* __restrict__ v, VolResult* r, int nvol,
                             const unsigned* __restrict__ peakpref, long long words,
                             const uint64_t* __restrict__ keys, const unsigned* m_p,
                             const int* range, int b, unsigned* cnt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0) cnt[CNT_PEAKS] = peakpref[words];
  if (i >= nvol) return;
  const long long off = v[i].off, n = (long long)v[i].nx * v[i].ny * v[i].nz;
  const long long w0 = off >> 5, w1 = (off + n + 31) >> 5;
  r[i].peak0 = peakpref[w0];
  r[i].n_peaks = peakpref[w1] - peakpref[w0];
  const long long m = *m_p;
  const long long base = range[0];
  // first sorted pair whose smaller label is >= the label range start of volume j
  auto lower = [&](int j) -> long long {
    if (j >= nvol) return m;
    const long long target = (long long)r[j].gstart - base;
    long long lo = 0, hi = m;
    while (lo < hi) {
      const long long mid = (lo + hi) >> 1;
      if ((long long)(keys[mid] >> b) < target) lo = mid + 1;
      else hi = mid;
    }
    return lo;
  };
  const long long p0 = lower(i), p1 = lower(i + 1);
  r[i].pair0 = (unsigned)p0;
  r[i].n_pairs = (unsigned)(p1 - p0);
}

// =================================================================================================
// host stages
// =================================================================================================
namespace {
inline unsigned grid_for(long long work, int threads, int sm_count, int per_sm = 8) {
  long long b = (work + threads - 1) / threads;
  const long long cap = (long long)sm_count * per_sm;
  if (b > cap) b = cap;
  if (b < 1) b = 1;
  return (unsigned)b;
}
inline long long boxes_of(Dims d, int bx, int by, int bz) {
  return (long long)((d.nx + bx - 1) / bx) * ((d.ny + by - 1) / by) * ((d.nz + bz - 1) / bz);
}
inline float marker_threshold(const float spacing[3]) {
  const float min_sp = std::min(spacing[0], std::min(spacing[1], spacing[2]));
  return -1.5f * min_sp;  // pore_extraction.hpp:163-164
}

// Cooperative launch of the persistent flood loop: as many blocks as can be resident at once.
// blocks_per_sm stays well under the kernel's occupancy (8 blocks of 256 threads per SM), so that
// loops of batches running on concurrent streams fit on the device together.
template <class G>
cudaError_t launch_flood_loop(G geo, const uint8_t* code, int* key, int* L, int* fa, int* fb,
                              int* tmp, unsigned* cnt, int max_sweeps, int sm_count,
                              long long work, cudaStream_t s, int blocks_per_sm = 2,
                              unsigned long long wait_ns = kBarrierNs, unsigned wait_extra = 0) {
  int per_sm = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_flood_loop<G>, 256, 0);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) return cudaErrorCooperativeLaunchTooLarge;
  const unsigned grid = grid_for(work, 256, sm_count, std::min(per_sm, blocks_per_sm));
  void* args[] = {&geo, &code, &key, &L, &fa, &fb, &tmp, &cnt, &max_sweeps, &wait_ns, &wait_extra};
  return cudaLaunchCooperativeKernel((const void*)k_flood_loop<G>, dim3(grid), dim3(256), args, 0,
                                     s);
}
}  // namespace

int xfer_slab_planes(int nz) {
  const int k = std::max(1, std::min(16, (nz + 15) / 16));  // up to 16 slabs
  return ((nz + k - 1) / k + 15) / 16 * 16;
}

Status run_sdf_pass(Ctx& c, const float* d_sdf, Dims d, const float spacing[3], SegState* st,
                    bool all_ascent, HostXfer* xfer, bool ccl_in_slabs) {
  const long long n = d.n();
  const long long words = (n + 31) / 32;
  StageScope stage(c, PNM_STAGE_SDF_PASS, "pnm::extract_pores+init_markers");
  st->d = d;
  st->sdf = d_sdf;
  PNM_TRY(c.buf(S_CODE, n, &st->code));
  int* L = nullptr;
  PNM_TRY(c.buf(S_L, n, &L));
  PNM_TRY(c.buf(S_PEAKBITS, words, &st->peakbits));
  PNM_CUDA(cudaMemsetAsync(st->peakbits, 0, words * sizeof(uint32_t), c.stream));
  st->n_words = (long long)d.nz * d.ny * ((d.nx + 31) / 32);
  PNM_TRY(c.buf(S_EDGES, st->n_words, &st->mbits));
  PNM_TRY(c.buf(S_NXT, n, &st->nxt));
  OneVol geo{d, marker_threshold(spacing)};
  auto launch = [&](unsigned tiles) {
    if (all_ascent)
      k_sdf_pass<true, OneVol, TZ_PLAIN><<<tiles, TX * TY, 0, c.stream>>>(
          d_sdf, geo, st->code, st->nxt, L, st->peakbits, st->mbits);
    else
      k_sdf_pass<false, OneVol, TZ_PLAIN><<<tiles, TX * TY, 0, c.stream>>>(
          d_sdf, geo, st->code, st->nxt, L, st->peakbits, st->mbits);
    ++c.launches;
  };
  if (!xfer || !xfer->h_sdf) {
    launch((unsigned)boxes_of(d, TX, TY, TZ_PLAIN));
  } else {
    // upload in z-slabs (the last plane first: the first slab's periodic halo), and run the
    // SDF pass of each slab once its own planes and the next slab's first plane have arrived
    const int zs = xfer_slab_planes(d.nz), k = (d.nz + zs - 1) / zs;
    const long long plane = (long long)d.nx * d.ny;
    float* dst = const_cast<float*>(d_sdf);
    PNM_TRY(c.ensure_copy_events(2 * k + 3));
    PNM_CUDA(cudaEventRecord(c.events[2 * k], c.stream));  // the device buffer is free
    PNM_CUDA(cudaStreamWaitEvent(c.copy_stream, c.events[2 * k], 0));
    PNM_CUDA(cudaMemcpyAsync(dst + (d.nz - 1) * plane, xfer->h_sdf + (d.nz - 1) * plane,
                             plane * sizeof(float), cudaMemcpyHostToDevice, c.copy_stream));
    // copy i ends one plane into slab i+1 (and, for i > 0, starts one plane into slab i), so
    // event i marks the arrival of every plane the SDF pass of slab i reads
    for (int i = 0; i < k; ++i) {
      const int a = i == 0 ? 0 : i * zs + 1, b = std::min(d.nz, (i + 1) * zs + 1);
      if (b > a)
        PNM_CUDA(cudaMemcpyAsync(dst + a * plane, xfer->h_sdf + a * plane,
                                 (b - a) * plane * sizeof(float), cudaMemcpyHostToDevice,
                                 c.copy_stream));
      PNM_CUDA(cudaEventRecord(c.events[i], c.copy_stream));
    }
    if (!xfer->extra.empty()) {
      for (size_t j = 0; j < xfer->extra.size(); ++j) {
        const auto& cp = xfer->extra[j];
        if (j + 1 == xfer->extra.size() && j > 0) {
          PNM_CUDA(cudaEventRecord(c.events[2 * k + 2], c.copy_stream));
          xfer->extra_early = c.events[2 * k + 2];
        }
        PNM_CUDA(cudaMemcpyAsync(cp.dst, cp.src, cp.bytes, cudaMemcpyHostToDevice,
                                 c.copy_stream));
      }
      PNM_CUDA(cudaEventRecord(c.events[2 * k + 1], c.copy_stream));
      xfer->extra_done = c.events[2 * k + 1];
    }
    const long long tpp = (long long)((d.nx + TX - 1) / TX) * ((d.ny + TY - 1) / TY);
    // With ccl_in_slabs, the marker links of slab i are made once slab i+1 has had its SDF pass
    // (a word's forward rows reach one plane up), while later slabs are still uploading; the
    // last slab's links (wrapping to plane 0) follow the loop.
    const long long wpp = (long long)d.ny * ((d.nx + 31) / 32);  // bitmap words per plane
    const OneVol cgeo{d, geo.thr};
    auto ccl_slab = [&](int j) {
      StageScope stage(c, PNM_STAGE_MERGE_MARKERS, "pnm::merge_markers");
      const int a = j * zs, b = std::min(d.nz, a + zs);
      k_ccl_words<<<grid_for((b - a) * wpp, 256, c.sm_count, PLAIN_GRID_PER_SM), 256, 0,
                    c.stream>>>(cgeo, st->mbits, b * wpp, L, c.d_cnt, a * wpp);
      ++c.launches;
    };
    for (int i = 0; i < k; ++i) {
      const int z0 = i * zs, z1 = std::min(d.nz, z0 + zs);
      PNM_CUDA(cudaStreamWaitEvent(c.stream, c.events[i], 0));
      geo.base = (int)(z0 / TZ_PLAIN * tpp);
      launch((unsigned)(((z1 - z0 + TZ_PLAIN - 1) / TZ_PLAIN) * tpp));
      if (ccl_in_slabs && i > 0) ccl_slab(i - 1);
    }
    if (ccl_in_slabs) {
      ccl_slab(k - 1);
      st->ccl_done = true;
    }
  }
  PNM_CUDA(cudaGetLastError());
  st->idtab = L;
  return Status::ok();
}

Status run_segmentation(Ctx& c, const float* d_sdf, Dims d, const float spacing[3], SegState* st,
                        bool all_ascent, HostXfer* xfer, const std::function<Status()>* after_sdf) {
  const long long n = d.n();
  const long long words = (n + 31) / 32;
  cudaStream_t s = c.stream;
  PNM_CUDA(cudaMemsetAsync(c.d_cnt, 0, CNT_COUNT * sizeof(unsigned), s));
  PNM_TRY(run_sdf_pass(c, d_sdf, d, spacing, st, all_ascent, xfer, /*ccl_in_slabs=*/true));
  if (after_sdf) PNM_TRY((*after_sdf)());
  const OneVol geo{d, marker_threshold(spacing)};
  int* L = st->idtab;
  int *key, *keylist, *f0, *f1, *tmp, *ulist;
  PNM_TRY(c.buf(S_ULIST, n, &ulist));
  PNM_TRY(c.buf(S_KEY, n, &key));
  PNM_TRY(c.buf(S_KEYLIST, n, &keylist));
  PNM_TRY(c.buf(S_FRONT0, n, &f0));
  PNM_TRY(c.buf(S_FRONT1, n, &f1));
  PNM_TRY(c.buf(S_TMP, n, &tmp));
  st->key = key;
  const unsigned tiles = (unsigned)boxes_of(d, TX, TY, TZ_PLAIN);

  if (!st->ccl_done) {  // (a host upload made the links slab by slab behind it)
    StageScope stage(c, PNM_STAGE_MERGE_MARKERS, "pnm::merge_markers");
    k_ccl_words<<<grid_for(st->n_words, 256, c.sm_count, PLAIN_GRID_PER_SM), 256, 0, s>>>(
        geo, st->mbits, st->n_words, L, c.d_cnt);
    ++c.launches;
  }
  {
    StageScope stage(c, PNM_STAGE_GRADIENT_PATH, "pnm::gradient_path");
    k_resolve<<<(unsigned)boxes_of(d, RTX, RTY, RTZ), RTX * RTY, 0, s>>>(geo, st->code, st->nxt,
                                                                        L, key, keylist, c.d_cnt);
    ++c.launches;
  }
  PNM_TRY(c.join_side());  // the cooperative flood loop below wants every SM to itself
  StageScope flood_stage(c, PNM_STAGE_FLOOD, "pnm::flood");
  k_flood_seed<OneVol, TZ_PLAIN><<<tiles, TX * TY, 0, s>>>(geo, st->code, key, L, ulist, c.d_cnt);
  const unsigned fgrid = grid_for(n, 256, c.sm_count, 4);
  k_flood_layer2<<<fgrid, 256, 0, s>>>(geo, key, ulist, &c.d_cnt[CNT_ULIST], f0, tmp,
                                       &c.d_cnt[CNT_FRONT0]);
  c.launches += 2;
  PNM_CUDA(cudaGetLastError());

  // deeper layers: the persistent loop; if a cooperative launch is refused, the same sweeps as
  // separate launches in batches between host checks (empty sweeps are no-ops)
  const int kMaxSweeps = 1 << 20;
  cudaError_t le = launch_flood_loop(geo, st->code, key, L, f0, f1, tmp, c.d_cnt, kMaxSweeps,
                                     c.sm_count, n, s, PLAIN_FLOOD_PER_SM, c.wait_ns,
                                     c.wait_extra);
  ++c.launches;
  if (le != cudaSuccess) {
    cudaGetLastError();
    int* fin = f0;
    int* fout = f1;
    int cin = CNT_FRONT0, cout = CNT_FRONT1;
    const int kBatch = 4;
    int sweeps = 1;
    while (true) {
      for (int b = 0; b < kBatch; ++b) {
        PNM_CUDA(cudaMemsetAsync(&c.d_cnt[cout], 0, sizeof(unsigned), s));
        if (sweeps > 1) {  // the first layer's labels came with it (k_flood_layer2)
          k_flood_assign<<<fgrid, 256, 0, s>>>(geo, key, fin, &c.d_cnt[cin], tmp);
          ++c.launches;
        }
        k_flood_discover<<<fgrid, 256, 0, s>>>(geo, st->code, key, L, fin, &c.d_cnt[cin], tmp,
                                               fout, &c.d_cnt[cout]);
        ++c.launches;
        std::swap(fin, fout);
        std::swap(cin, cout);
        ++sweeps;
      }
      PNM_CUDA(cudaGetLastError());
      PNM_TRY(c.read_counters());
      if (c.h_cnt[cin] == 0) break;
      if (sweeps > kMaxSweeps) return Status{PNM_ERR_NOT_CONVERGED, "flood did not converge"};
    }
    st->flood_sweeps = sweeps;
  }
  flood_stage.next(PNM_STAGE_RELABEL, "pnm::relabel");
  uint32_t *firstP, *firstS;
  unsigned *prefP, *prefS, *scan0;
  PNM_TRY(c.buf(S_FIRSTP, words, &firstP));
  PNM_TRY(c.buf(S_FIRSTS, words, &firstS));
  PNM_TRY(c.buf(S_PREFP, words + 1, &prefP));
  PNM_TRY(c.buf(S_PREFS, words + 1, &prefS));
  PNM_TRY(c.buf(S_SCAN0, words / SCAN_TILE + 2, &scan0));
  PNM_CUDA(cudaMemsetAsync(firstP, 0, words * 4, s));
  PNM_CUDA(cudaMemsetAsync(firstS, 0, words * 4, s));
  const unsigned kgrid = grid_for(n / 16 + 1, 256, c.sm_count);  // grid-stride over the keys
  k_key_first<<<kgrid, 256, 0, s>>>(keylist, &c.d_cnt[CNT_KEYS], L, st->code, firstP, firstS, n,
                                    &c.d_cnt[CNT_ERR]);
  exclusive_scan(PopcountOf{firstP}, words, prefP, scan0, s, &c.launches);
  exclusive_scan(PopcountOf{firstS}, words, prefS, scan0, s, &c.launches);
  k_key_id<<<kgrid, 256, 0, s>>>(geo, keylist, &c.d_cnt[CNT_KEYS], L, st->code, firstP, prefP,
                                 firstS, prefS, n, &c.d_cnt[CNT_ERR]);
  c.launches += 2;
  PNM_CUDA(cudaGetLastError());
  unsigned tot[2];
  PNM_CUDA(cudaMemcpyAsync(&tot[0], prefP + words, 4, cudaMemcpyDeviceToHost, s));
  PNM_CUDA(cudaMemcpyAsync(&tot[1], prefS + words, 4, cudaMemcpyDeviceToHost, s));
  PNM_TRY(c.read_counters());
  st->n_pore_labels = (int)tot[0];
  st->n_solid_labels = (int)tot[1];
  st->n_edges = c.h_cnt[CNT_EDGES];
  if (le == cudaSuccess) st->flood_sweeps = (int)c.h_cnt[CNT_SWEEPS];
  if (c.h_cnt[CNT_ERR] & ERRF_UF_LIMIT)
    return Status{PNM_ERR_NOT_CONVERGED, "union-find exceeded its iteration limit"};
  if (c.h_cnt[CNT_ERR] & ERRF_FLOOD_LIMIT)
    return Status{PNM_ERR_NOT_CONVERGED, "flood did not converge"};
  if (c.h_cnt[CNT_ERR] & ERRF_BARRIER)
    return Status{PNM_ERR_NOT_CONVERGED,
                  "flood loop: a grid barrier wait ran out (blocks not all resident?)"};
  if (c.h_cnt[CNT_ERR] & ERRF_LABEL_RANGE)
    return Status{PNM_ERR_INTERNAL, "renumbering: a label minimum is outside the volume"};
  return Status::ok();
}

namespace {
Status emit_pairs(Ctx& c, Dims d, bool from_keys, const SegState* st, const int32_t* d_seg_in,
                  int32_t* d_seg_out, bool want_pairs, long long cap_hint, int32_t** d_pairs_out,
                  int64_t* n_pairs, HostXfer* xfer = nullptr) {
  cudaStream_t s = c.stream;
  const long long n = d.n();
  long long cap = 4096;
  while (cap < cap_hint) cap <<= 1;
  for (int attempt = 0; attempt < 8; ++attempt) {
    StageScope stage(c, PNM_STAGE_SEG_PAIRS, "pnm::relabel_seg+boundary_pairs");
    unsigned long long* table = nullptr;
    unsigned long long* dense = nullptr;  // the set's keys in insertion order
    int* range = nullptr;
    PNM_TRY(c.buf(S_HASH, want_pairs ? cap : 1, &table));
    if (want_pairs) PNM_TRY(c.buf(S_HASHKEYS, cap, &dense));
    PNM_TRY(c.buf(S_MAXBITS, 2, &range));
    if (want_pairs) PNM_CUDA(cudaMemsetAsync(table, 0xff, cap * sizeof(unsigned long long), s));
    // key pairs: the label range is known ([-nS, nP]); label pairs of a given seg: tracked
    const int init[2] = {from_keys ? -st->n_solid_labels : INT_MAX,
                         from_keys ? st->n_pore_labels : INT_MIN};
    PNM_CUDA(cudaMemcpyAsync(range, init, sizeof(init), cudaMemcpyHostToDevice, s));
    PNM_CUDA(cudaMemsetAsync(&c.d_cnt[CNT_ERR], 0, sizeof(unsigned), s));
    PNM_CUDA(cudaMemsetAsync(&c.d_cnt[CNT_PAIRS], 0, sizeof(unsigned), s));
    const unsigned g = (unsigned)boxes_of(d, STX, STY, STZ);
    OneVol geo{d, 0.0f};
    // labels already on their way to the host (an earlier attempt) are not written again
    int32_t* seg_out = (xfer && xfer->seg_sent) ? nullptr : d_seg_out;
    if (from_keys && xfer && xfer->h_seg && seg_out) {
      // z-slabs of bricks; each slab's labels go to the host while the next slabs and the
      // pair stages run
      const int zs = xfer_slab_planes(d.nz), k = (d.nz + zs - 1) / zs;
      const long long plane = (long long)d.nx * d.ny;
      const long long bpp = (long long)((d.nx + STX - 1) / STX) * ((d.ny + STY - 1) / STY);
      PNM_TRY(c.ensure_copy_events(2 * k + 2));
      for (int i = 0; i < k; ++i) {
        const int z0 = i * zs, z1 = std::min(d.nz, z0 + zs);
        geo.base = (int)(z0 / STZ * bpp);
        k_seg_topo<<<(unsigned)(((z1 - z0 + STZ - 1) / STZ) * bpp), STX * STY, 0, s>>>(
            geo, KeyLabels{st->key, st->idtab}, seg_out, want_pairs ? 1 : 0, table,
            (uint64_t)(cap - 1), c.d_cnt, range, dense);
        ++c.launches;
        PNM_CUDA(cudaEventRecord(c.events[k + i], s));
        PNM_CUDA(cudaStreamWaitEvent(c.copy_stream, c.events[k + i], 0));
        PNM_CUDA(cudaMemcpyAsync(xfer->h_seg + z0 * plane, seg_out + z0 * plane,
                                 (z1 - z0) * plane * sizeof(int32_t), cudaMemcpyDeviceToHost,
                                 c.copy_stream));
      }
      xfer->seg_sent = true;
    } else if (from_keys) {
      k_seg_topo<<<g, STX * STY, 0, s>>>(geo, KeyLabels{st->key, st->idtab}, seg_out,
                                         want_pairs ? 1 : 0, table, (uint64_t)(cap - 1), c.d_cnt,
                                         range, dense);
      ++c.launches;
    } else {
      k_seg_topo<<<g, STX * STY, 0, s>>>(geo, SegLabels{d_seg_in}, seg_out, want_pairs ? 1 : 0,
                                         table, (uint64_t)(cap - 1), c.d_cnt, range, dense);
      ++c.launches;
    }
    PNM_CUDA(cudaGetLastError());
    if (!want_pairs) return Status::ok();
    PNM_TRY(c.read_counters());
    if (c.h_cnt[CNT_ERR] & ERRF_HASH_FULL) {
      cap <<= 2;
      continue;
    }
    stage.next(PNM_STAGE_PAIR_SORT, "pnm::unique_pairs");
    const long long m = c.h_cnt[CNT_PAIRS];
    *n_pairs = m;
    int32_t* out = nullptr;
    PNM_TRY(c.buf(S_PAIRS, 2 * m + 2, &out));
    *d_pairs_out = out;
    if (m == 0) return Status::ok();
    int hr[2] = {init[0], init[1]};
    if (!from_keys) {
      PNM_CUDA(cudaMemcpyAsync(hr, range, sizeof(hr), cudaMemcpyDeviceToHost, s));
      PNM_CUDA(cudaStreamSynchronize(s));
    }
    const unsigned long long span = (unsigned long long)((long long)hr[1] - (long long)hr[0]);
    int b = 1;
    while (b < 32 && (1ull << b) <= span) ++b;
    unsigned *scan0, *hist;
    uint64_t *ka, *kb;
    PNM_TRY(c.buf(S_SCAN0, (256 * (m / RS_TILE + 1)) / SCAN_TILE + 2, &scan0));
    PNM_TRY(c.buf(S_KEYS_A, m, &ka));
    PNM_TRY(c.buf(S_KEYS_B, m, &kb));
    PNM_TRY(c.buf(S_RSHIST, 256 * (m / RS_TILE + 1) + 1, &hist));
    // the m keys the inserts appended (no sweep of the set)
    if (from_keys)
      k_hash_gather_keys<<<grid_for(m, 256, c.sm_count), 256, 0, s>>>(dense, m, nullptr, geo,
                                                                      st->idtab, range, b, ka);
    else
      k_hash_gather<<<grid_for(m, 256, c.sm_count), 256, 0, s>>>(dense, m, nullptr, range, b, ka);
    ++c.launches;
    const bool in_b = radix_sort(ka, nullptr, kb, nullptr, m, 0, 2 * b, hist, scan0, s, &c.launches);
    k_pairs_decode<<<grid_for(m, 256, c.sm_count), 256, 0, s>>>(in_b ? kb : ka, m, range, b, out); ++c.launches;
    PNM_CUDA(cudaGetLastError());
    return Status::ok();
  }
  return Status{PNM_ERR_INTERNAL, "pair hash set kept overflowing"};
}
}  // namespace

Status run_seg_and_topology(Ctx& c, const SegState& st, int32_t* d_seg, bool want_pairs,
                            int32_t** d_pairs_out, int64_t* n_pairs, HostXfer* xfer) {
  const long long labels = (long long)st.n_pore_labels + st.n_solid_labels + 2;
  const long long hint =
      std::min<long long>(std::max<long long>(64 * labels, 4096), 3 * st.d.n() + 64);
  return emit_pairs(c, st.d, true, &st, nullptr, d_seg, want_pairs, hint, d_pairs_out, n_pairs,
                    xfer);
}

Status run_topology_of_seg(Ctx& c, const int32_t* d_seg, Dims d, int32_t** d_pairs_out,
                           int64_t* n_pairs) {
  const long long hint = std::min<long long>(std::max<long long>(d.n() / 8, 4096), 3 * d.n() + 64);
  return emit_pairs(c, d, false, nullptr, d_seg, nullptr, true, hint, d_pairs_out, n_pairs);
}

Status run_pores(Ctx& c, const SegState& st, const float origin[3], const float spacing[3],
                 pnm_pore* d_out, int64_t cap, int64_t* n_pores) {
  StageScope stage(c, PNM_STAGE_PORES, "pnm::extract_pores(records)");
  cudaStream_t s = c.stream;
  const long long words = (st.d.n() + 31) / 32;
  unsigned *pref, *scan0;
  PNM_TRY(c.buf(S_PEAKPREF, words + 1, &pref));
  PNM_TRY(c.buf(S_SCAN1, words / SCAN_TILE + 2, &scan0));
  exclusive_scan(PopcountOf{st.peakbits}, words, pref, scan0, s, &c.launches);
  k_pores_emit<<<grid_for(words, 256, c.sm_count), 256, 0, s>>>(
      st.sdf, st.d, st.peakbits, pref, words, origin[0], origin[1], origin[2], spacing[0],
      spacing[1], spacing[2], d_out, cap); ++c.launches;
  PNM_CUDA(cudaGetLastError());
  unsigned tot = 0;
  PNM_CUDA(cudaMemcpyAsync(&tot, pref + words, 4, cudaMemcpyDeviceToHost, s));
  PNM_CUDA(cudaStreamSynchronize(s));
  *n_pores = tot;
  return Status::ok();
}

Status run_pores_side(Ctx& c, const SegState& st, const float origin[3], const float spacing[3],
                      pnm_pore* d_out, int64_t cap) {
  PNM_TRY(c.ensure_side());
  cudaStream_t s = c.side_stream;
  struct Range {  // the stage's NVTX range on the host thread
    Range() { nvtxRangePushA("pnm::extract_pores(records)"); }
    ~Range() { nvtxRangePop(); }
  } range;
  const long long words = (st.d.n() + 31) / 32;
  unsigned *pref, *scan0;
  PNM_TRY(c.buf(S_PEAKPREF, words + 1, &pref));
  PNM_TRY(c.buf(S_SCAN2, words / SCAN_TILE + 2, &scan0));
  PNM_CUDA(cudaEventRecord(c.side_fork, c.stream));
  PNM_CUDA(cudaStreamWaitEvent(s, c.side_fork, 0));
  if (c.timing) PNM_CUDA(cudaEventRecord(c.side_t0, s));
  exclusive_scan(PopcountOf{st.peakbits}, words, pref, scan0, s, &c.launches);
  k_pores_emit<<<grid_for(words, 256, c.sm_count), 256, 0, s>>>(
      st.sdf, st.d, st.peakbits, pref, words, origin[0], origin[1], origin[2], spacing[0],
      spacing[1], spacing[2], d_out, cap);
  ++c.launches;
  PNM_CUDA(cudaGetLastError());
  PNM_CUDA(cudaMemcpyAsync(c.h_side, pref + words, 4, cudaMemcpyDeviceToHost, s));
  if (c.timing) {
    PNM_CUDA(cudaEventRecord(c.side_t1, s));
    c.side_timed = true;
    c.side_stage = PNM_STAGE_PORES;
  }
  PNM_CUDA(cudaEventRecord(c.side_join, s));
  c.side_pending = true;
  return Status::ok();
}

Status side_pores_count(Ctx& c, int64_t* n_pores) {
  PNM_TRY(c.join_side());
  PNM_CUDA(cudaEventSynchronize(c.side_join));
  *n_pores = *c.h_side;
  return Status::ok();
}

Status run_peak_ids(Ctx& c, const SegState& st, int32_t* d_out, int64_t cap, int64_t* n_peaks) {
  StageScope stage(c, PNM_STAGE_PORES, "pnm::extract_pores(peak voxels)");
  cudaStream_t s = c.stream;
  const long long words = (st.d.n() + 31) / 32;
  unsigned *pref, *scan0;
  PNM_TRY(c.buf(S_PEAKPREF, words + 1, &pref));
  PNM_TRY(c.buf(S_SCAN1, words / SCAN_TILE + 2, &scan0));
  exclusive_scan(PopcountOf{st.peakbits}, words, pref, scan0, s, &c.launches);
  k_peak_ids<<<grid_for(words, 256, c.sm_count), 256, 0, s>>>(st.peakbits, pref, words, d_out,
                                                              cap);
  ++c.launches;
  PNM_CUDA(cudaGetLastError());
  unsigned tot = 0;
  PNM_CUDA(cudaMemcpyAsync(&tot, pref + words, 4, cudaMemcpyDeviceToHost, s));
  PNM_CUDA(cudaStreamSynchronize(s));
  *n_peaks = tot;
  return Status::ok();
}

Status enqueue_batch(BatchPlan& p, cudaStream_t s, long long* launches) {
  const long long n = p.n_total, words = p.words;
  const int sm = p.sm_count;
  const VolTab geo{p.vols, p.res, p.nvol};
  PNM_CUDA(cudaMemsetAsync(p.cnt, 0, CNT_COUNT * sizeof(unsigned), s));
  PNM_CUDA(cudaMemsetAsync(p.peakbits, 0, words * sizeof(uint32_t), s));
  PNM_CUDA(cudaMemsetAsync(p.firstP, 0, words * sizeof(uint32_t), s));
  PNM_CUDA(cudaMemsetAsync(p.firstS, 0, words * sizeof(uint32_t), s));
  PNM_CUDA(cudaMemsetAsync(p.table, 0xff, p.hash_cap * sizeof(unsigned long long), s));
  k_batch_init<<<1, 1, 0, s>>>(p.range);
  const unsigned tiles = (unsigned)p.tiles;
  switch (p.tile_z) {  // the volume table's tile numbering was planned for this depth
    case 4:
      k_sdf_pass<false, VolTab, 4><<<tiles, TX * TY, 0, s>>>(p.sdf, geo, p.code, p.nxt, p.L,
                                                             p.peakbits, p.mbits);
      break;
    case 16:
      k_sdf_pass<false, VolTab, 16><<<tiles, TX * TY, 0, s>>>(p.sdf, geo, p.code, p.nxt, p.L,
                                                             p.peakbits, p.mbits);
      break;
    default:
      k_sdf_pass<false, VolTab, 8><<<tiles, TX * TY, 0, s>>>(p.sdf, geo, p.code, p.nxt, p.L,
                                                             p.peakbits, p.mbits);
  }
  k_ccl_words<<<grid_for(p.n_words, 256, sm, p.ccl_per_sm), 256, 0, s>>>(geo, p.mbits, p.n_words,
                                                                          p.L, p.cnt);
  k_resolve<<<(unsigned)p.bricks, RTX * RTY, 0, s>>>(geo, p.code, p.nxt, p.L, p.key, p.keylist,
                                                     p.cnt);
  switch (p.tile_z) {
    case 4:
      k_flood_seed<VolTab, 4><<<tiles, TX * TY, 0, s>>>(geo, p.code, p.key, p.L, p.ulist, p.cnt);
      break;
    case 16:
      k_flood_seed<VolTab, 16><<<tiles, TX * TY, 0, s>>>(geo, p.code, p.key, p.L, p.ulist, p.cnt);
      break;
    default:
      k_flood_seed<VolTab, 8><<<tiles, TX * TY, 0, s>>>(geo, p.code, p.key, p.L, p.ulist, p.cnt);
  }
  k_flood_layer2<<<grid_for(n, 256, sm, 4), 256, 0, s>>>(
      geo, p.key, p.ulist, &p.cnt[CNT_ULIST], p.f0, p.tmp, &p.cnt[CNT_FRONT0]);
  *launches += 6;
  PNM_CUDA(cudaGetLastError());
  PNM_CUDA(launch_flood_loop(geo, p.code, p.key, p.L, p.f0, p.f1, p.tmp, p.cnt, p.max_sweeps, sm,
                             n, s, p.flood_blocks_per_sm));
  const unsigned kgrid = grid_for(n / 16 + 1, 256, sm, p.grid_per_sm);
  k_key_first<<<kgrid, 256, 0, s>>>(p.keylist, &p.cnt[CNT_KEYS], p.L, p.code, p.firstP, p.firstS,
                                    n, &p.cnt[CNT_ERR]);
  exclusive_scan(PopcountOf{p.firstP}, words, p.prefP, p.scan_tmp, s, launches);
  exclusive_scan(PopcountOf{p.firstS}, words, p.prefS, p.scan_tmp, s, launches);
  k_key_id<<<kgrid, 256, 0, s>>>(geo, p.keylist, &p.cnt[CNT_KEYS], p.L, p.code, p.firstP,
                                 p.prefP, p.firstS, p.prefS, n, &p.cnt[CNT_ERR]);
  k_batch_labels<<<1, SCAN_THREADS, 0, s>>>(p.vols, p.res, p.nvol, p.prefP, p.prefS);
  k_seg_topo<<<(unsigned)p.bricks, STX * STY, 0, s>>>(geo, KeyLabels{p.key, p.L}, p.seg, 1,
                                                       p.table, (uint64_t)(p.hash_cap - 1), p.cnt,
                                                       p.range, nullptr);
  *launches += 5;
  PNM_CUDA(cudaGetLastError());
  // unique pairs: compact the set, sort, decode per volume (counts stay on the device)
  exclusive_scan(Occupied{p.table}, p.hash_cap, p.hpos, p.scan_tmp, s, launches);
  const unsigned* m_p = p.hpos + p.hash_cap;
  const unsigned hgrid = grid_for(p.hash_cap, 256, sm);
  k_hash_gather_keys<<<hgrid, 256, 0, s>>>(p.table, p.hash_cap, p.hpos, geo, p.L, p.range,
                                           p.label_bits, p.ka);
  p.pairs_in_b = radix_sort(p.ka, nullptr, p.kb, nullptr, p.hash_cap, 0, 2 * p.label_bits, p.hist,
                            p.scan_tmp, s, launches, m_p);
  const uint64_t* sorted = p.pairs_in_b ? p.kb : p.ka;
  k_pairs_decode_batch<<<hgrid, 256, 0, s>>>(sorted, m_p, p.range, p.label_bits, geo, p.pairs);
  // pores
  exclusive_scan(PopcountOf{p.peakbits}, words, p.peakpref, p.scan_tmp, s, launches);
  k_pores_emit_batch<<<grid_for(words, 256, sm), 256, 0, s>>>(p.sdf, geo, p.peakbits, p.peakpref,
                                                              words, p.pores, p.pore_cap);
  k_batch_tail<<<(unsigned)((p.nvol + 255) / 256), 256, 0, s>>>(
      p.vols, p.res, p.nvol, p.peakpref, words, sorted, m_p, p.range, p.label_bits, p.cnt);
  *launches += 4;
  PNM_CUDA(cudaGetLastError());
  PNM_CUDA(cudaMemcpyAsync(p.h_cnt, p.cnt, CNT_COUNT * sizeof(unsigned), cudaMemcpyDeviceToHost,
                           s));
  PNM_CUDA(cudaMemcpyAsync(p.h_res, p.res, p.nvol * sizeof(VolResult), cudaMemcpyDeviceToHost,
                           s));
  return Status::ok();
}

}  // namespace pnm
