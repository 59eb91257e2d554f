// Volume geometry for the extraction kernels: one periodic volume, or a ragged batch of them laid
// end to end in one voxel id space.
//
// Batch layout: volume i occupies global voxel ids [off_i, off_i + n_i), x fastest, with off_i a
// multiple of 32 (so every 32-bit bitmap word belongs to one volume) and the gap up to the next
// volume holding ZERO-class codes. Every stored id (ascent pointers, union-find parents, keys,
// edges, list entries) is global, so union-find roots, first-appearance minima and bitmap ranks
// need no per-volume treatment; only neighbour arithmetic wraps per volume (each volume is its own
// periodic box, the reference's get_idx, pore_extraction.hpp:59-64), and label ids are rank
// differences against the rank at the volume's first voxel.
#pragma once

#include <cuda_runtime.h>

#include <climits>
#include <cstdint>

#include "pnm_ctx.h"

namespace pnm {

// Host-built description of one volume of a batch (device copy is read-only while running).
struct VolDesc {
  int off;            // first global voxel id (multiple of 32)
  int nx, ny, nz;
  int tile0;          // first SDF-pass tile (32 x 8 x tile depth) of this volume, batch-wide
  int brick0;         // first resolve / seg-topology brick (32 x 8 x 16)
  int word0;          // first marker-bitmap word (one per 32-voxel row chunk)
  float thr;          // marker threshold: -1.5 * min spacing (pore_extraction.hpp:163-164)
  float ox, oy, oz;   // origin, xyz
  float sx, sy, sz;   // spacing, xyz
};

// Per-volume figures written by the device during a batch run. Pair labels of volume i are
// ordered batch-wide as gbase + label, with the volume's labels -nS..nP filling
// [gstart, gstart + nS + nP] (gbase = gstart + nS): every volume's pairs share one hash set and
// one sort and come out grouped by volume.
struct VolResult {
  unsigned n_pore_labels, n_solid_labels;
  int gstart, gbase;
  unsigned peak0, n_peaks;
  unsigned pair0, n_pairs;
};

// One tile (or brick) of one volume: what a block of a tiled kernel works on.
struct Box {
  int off, nx, ny, nz;
  int word0;
  int X0, Y0, Z0;
  int vol;
  float thr;
  bool first;  // the volume's first tile
};

__device__ __forceinline__ void box_decode(Box& b, int local, int TXv, int TYv, int TZv) {
  const int tnx = (b.nx + TXv - 1) / TXv, tny = (b.ny + TYv - 1) / TYv;
  const int bx = local % tnx, r = local / tnx;
  b.X0 = bx * TXv;
  b.Y0 = (r % tny) * TYv;
  b.Z0 = (r / tny) * TZv;
  b.first = local == 0;
}

// A single volume at voxel id 0 (the plain entry points).
struct OneVol {
  static constexpr bool kBatch = false;
  Dims d;
  float thr;
  int base = 0;  // first tile / brick of a launch that covers a z-slab only
  __device__ Box tile(int b, int TXv, int TYv, int TZv, bool /*brick*/) const {
    b += base;
    Box x;
    x.off = 0;
    x.word0 = 0;
    x.nx = d.nx;
    x.ny = d.ny;
    x.nz = d.nz;
    x.vol = 0;
    x.thr = thr;
    box_decode(x, b, TXv, TYv, TZv);
    return x;
  }
  // volume of global voxel v: offset and dims
  __device__ void locate(int /*v*/, int& off, int& nx, int& ny, int& nz) const {
    off = 0;
    nx = d.nx;
    ny = d.ny;
    nz = d.nz;
  }
  __device__ int vol_of(int /*v*/) const { return 0; }
  __device__ int gbase(int /*vol*/) const { return 0; }
  __device__ void locate_word(int /*w*/, int& off, int& nx, int& ny, int& nz, int& word0) const {
    off = 0;
    word0 = 0;
    nx = d.nx;
    ny = d.ny;
    nz = d.nz;
  }
};

// A ragged batch: binary searches over the volume table (a few dozen to a few thousand entries,
// L1-resident).
struct VolTab {
  static constexpr bool kBatch = true;
  const VolDesc* v;
  const VolResult* r;  // gbase, read by the topology pass (written by the summary kernel)
  int nvol;
  __device__ int find_tile(int b, bool brick) const {
    int lo = 0, hi = nvol - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      const int t0 = brick ? __ldg(&v[mid].brick0) : __ldg(&v[mid].tile0);
      if (t0 <= b) lo = mid;
      else hi = mid - 1;
    }
    return lo;
  }
  __device__ int vol_of(int gv) const {
    int lo = 0, hi = nvol - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (__ldg(&v[mid].off) <= gv) lo = mid;
      else hi = mid - 1;
    }
    return lo;
  }
  __device__ Box tile(int b, int TXv, int TYv, int TZv, bool brick) const {
    const int i = find_tile(b, brick);
    Box x;
    x.off = __ldg(&v[i].off);
    x.word0 = __ldg(&v[i].word0);
    x.nx = __ldg(&v[i].nx);
    x.ny = __ldg(&v[i].ny);
    x.nz = __ldg(&v[i].nz);
    x.vol = i;
    x.thr = __ldg(&v[i].thr);
    box_decode(x, b - (brick ? __ldg(&v[i].brick0) : __ldg(&v[i].tile0)), TXv, TYv, TZv);
    return x;
  }
  __device__ void locate(int gv, int& off, int& nx, int& ny, int& nz) const {
    const int i = vol_of(gv);
    off = __ldg(&v[i].off);
    nx = __ldg(&v[i].nx);
    ny = __ldg(&v[i].ny);
    nz = __ldg(&v[i].nz);
  }
  __device__ int gbase(int vol) const { return r[vol].gbase; }
  __device__ void locate_word(int w, int& off, int& nx, int& ny, int& nz, int& word0) const {
    int lo = 0, hi = nvol - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (__ldg(&v[mid].word0) <= w) lo = mid;
      else hi = mid - 1;
    }
    off = __ldg(&v[lo].off);
    word0 = __ldg(&v[lo].word0);
    nx = __ldg(&v[lo].nx);
    ny = __ldg(&v[lo].ny);
    nz = __ldg(&v[lo].nz);
  }
  // volume owning batch-wide pair label g
  __device__ int vol_of_label(int g) const {
    int lo = 0, hi = nvol - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (r[mid].gstart <= g) lo = mid;
      else hi = mid - 1;
    }
    return lo;
  }
};

// Device buffers and sizes of one planned batch (owned by the batch object; fixed for its life,
// so the enqueued work can be captured once and replayed).
struct BatchPlan {
  int nvol = 0;
  long long n_total = 0;  // global voxel ids in use: last volume's offset + its voxel count
  long long words = 0;    // 32-voxel bitmap words
  long long tiles = 0, bricks = 0;
  int sm_count = 0;
  const VolDesc* vols = nullptr;
  VolResult* res = nullptr;
  const float* sdf = nullptr;
  uint8_t* code = nullptr;
  int *nxt = nullptr, *L = nullptr, *key = nullptr, *seg = nullptr;
  int *ulist = nullptr, *keylist = nullptr, *f0 = nullptr, *f1 = nullptr, *tmp = nullptr;
  uint32_t* mbits = nullptr;  // marker bitmap: one word per 32-voxel row chunk of every volume
  long long n_words = 0;
  uint32_t *peakbits = nullptr, *firstP = nullptr, *firstS = nullptr;
  unsigned *prefP = nullptr, *prefS = nullptr, *peakpref = nullptr, *scan_tmp = nullptr;
  unsigned long long* table = nullptr;
  long long hash_cap = 0;  // power of two
  unsigned* hpos = nullptr;  // hash_cap + 1 (exclusive scan of occupied slots; [cap] = pairs)
  uint64_t *ka = nullptr, *kb = nullptr;
  unsigned* hist = nullptr;
  int* range = nullptr;
  int label_bits = 0;      // bits of one re-encoded pair label
  int* pairs = nullptr;    // 2 * hash_cap
  pnm_pore* pores = nullptr;
  long long pore_cap = 0;
  unsigned* cnt = nullptr;  // CNT_COUNT device counters of this batch
  unsigned* h_cnt = nullptr;      // pinned mirrors, filled by the enqueued copies
  VolResult* h_res = nullptr;
  int max_sweeps = 1 << 20;
  // launch shape (autotuned per volume-size class; results do not depend on it)
  int tile_z = 16;              // SDF-pass / flood-seed tile depth: 4, 8 or 16
  int grid_per_sm = 16;         // grid-stride kernels: blocks of 256 threads per SM
  int ccl_per_sm = 8;           // CCL edge-union pass: blocks per SM
  int flood_blocks_per_sm = 4;  // persistent flood loop: resident blocks per SM
  bool pairs_in_b = false;  // set by enqueue: which radix buffer holds the sorted keys
};

// Enqueues the whole extraction of a planned batch on stream s: no host synchronisation, no
// allocation, every count read on the device (capturable into a CUDA graph). Returns the first
// launch error.
Status enqueue_batch(BatchPlan& p, cudaStream_t s, long long* launches);

}  // namespace pnm
