// pnm oracle — CPU restatement of the reference's single-rank extraction path.
//
// TEST AND BASELINE INFRASTRUCTURE ONLY. Only tests/, __graft_entry__.smoke() and bench.py's
// CPU-baseline / reference legs load this library, and only as the checker or as the timed CPU
// baseline. The product path (peclet_pnm_gb300/) never calls it.
//
// Every function restates one stage of src/pore_extraction.hpp (cited file:line), with the same
// loops, the same tie-breaks, the same fixpoint schedule (union-find rounds, Jacobi flood with a
// full label copy per sweep, 512-step gradient walks from every voxel, first-appearance
// renumbering, host sort + unique of every emitted pair, face-CCL fixpoints over all 3n faces).
// Parallel loops use OpenMP where the reference uses Kokkos::parallel_for; `threads` = 1 gives a
// deterministic serial run. Differences from the reference, all deliberate:
//   * pores are returned in voxel-index order (the reference's order is an atomic-slot race);
//     the max_pores cap keeps the first 1e6 in voxel order;
//   * extract_network_flow returns empty results when the largest label is < 1 (the reference
//     sizes views with a negative count there, which is undefined).
// Build: g++ -std=c++20 -O3 -fopenmp -ffp-contract=off (no FMA contraction, so float centroids
// and the float64 pressure / dp arithmetic round exactly like the reference's host build).
#include "pnm_oracle.h"

#include <omp.h>

#include <algorithm>
#include <atomic>
#include <climits>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <utility>
#include <vector>

namespace {

struct Dims {
  int x, y, z;
};

// pore_extraction.hpp:59-64 — periodic wrap on every axis, x-fastest flat index.
inline int get_idx(int x, int y, int z, Dims r) {
  x = (x % r.x + r.x) % r.x;
  y = (y % r.y + r.y) % r.y;
  z = (z % r.z + r.z) % r.z;
  return z * r.y * r.x + y * r.x + x;
}

template <class T>
inline T ld(const T* p) {
  return std::atomic_ref<T>(*const_cast<T*>(p)).load(std::memory_order_relaxed);
}
template <class T>
inline void st(T* p, T v) {
  std::atomic_ref<T>(*p).store(v, std::memory_order_relaxed);
}
template <class T>
inline void amin(T* p, T v) {
  std::atomic_ref<T> a(*p);
  T cur = a.load(std::memory_order_relaxed);
  while (v < cur && !a.compare_exchange_weak(cur, v, std::memory_order_relaxed)) {
  }
}
inline void aadd(double* p, double v) {
  std::atomic_ref<double>(*p).fetch_add(v, std::memory_order_relaxed);
}

template <class T>
T* dup(const std::vector<T>& v) {
  T* p = static_cast<T*>(std::malloc(sizeof(T) * (v.empty() ? 1 : v.size())));
  if (!v.empty()) std::memcpy(p, v.data(), sizeof(T) * v.size());
  return p;
}

// pore_extraction.hpp:107-124 — SDF^2-weighted 27-point centroid offset, float, fixed
// dz->dy->dx order, no contraction.
inline void centroid(const float* sdf, int ix, int iy, int iz, Dims r, float& fx, float& fy,
                     float& fz) {
  float sw = 0.0f, px = 0.0f, py = 0.0f, pz = 0.0f;
  for (int dz = -1; dz <= 1; ++dz)
    for (int dy = -1; dy <= 1; ++dy)
      for (int dx = -1; dx <= 1; ++dx) {
        const float v = sdf[get_idx(ix + dx, iy + dy, iz + dz, r)];
        float w = v > 0.0f ? v : 0.0f;
        w = w * w;
        sw += w;
        px += dx * w;
        py += dy * w;
        pz += dz * w;
      }
  fx = 0;
  fy = 0;
  fz = 0;
  if (sw > 1e-6f) {
    fx = px / sw;
    fy = py / sw;
    fz = pz / sw;
  }
}

// pore_extraction.hpp:69-140 extractPoresView.
std::vector<pnmo_pore> extract_pores(const float* sdf, Dims r, const float* org, const float* spc,
                                     int threads) {
  const float ox = org[0], oy = org[1], oz = org[2];
  const float sx = spc[0], sy = spc[1], sz = spc[2];
  const int max_pores = 1000000;  // pore_extraction.hpp:77
  std::vector<std::vector<pnmo_pore>> per_z(r.z);
#pragma omp parallel for schedule(dynamic, 1) num_threads(threads)
  for (int iz = 0; iz < r.z; ++iz)
    for (int iy = 0; iy < r.y; ++iy)
      for (int ix = 0; ix < r.x; ++ix) {
        const int ci = get_idx(ix, iy, iz, r);
        const float cv = sdf[ci];
        if (cv <= 0.0f) continue;
        bool peak = true;
        for (int dz = -1; dz <= 1 && peak; ++dz)
          for (int dy = -1; dy <= 1 && peak; ++dy)
            for (int dx = -1; dx <= 1; ++dx) {
              if (dx == 0 && dy == 0 && dz == 0) continue;
              const int ni = get_idx(ix + dx, iy + dy, iz + dz, r);
              const float nv = sdf[ni];
              if (nv > cv || (nv == cv && ni > ci)) {  // pore_extraction.hpp:100
                peak = false;
                break;
              }
            }
        if (!peak) continue;
        float fx, fy, fz;
        centroid(sdf, ix, iy, iz, r, fx, fy, fz);
        per_z[iz].push_back({ox + (ix + fx) * sx, oy + (iy + fy) * sy, oz + (iz + fz) * sz, cv});
      }
  std::vector<pnmo_pore> out;
  for (auto& v : per_z) out.insert(out.end(), v.begin(), v.end());
  if (out.size() > std::size_t(max_pores)) out.resize(max_pores);
  return out;
}

// pore_extraction.hpp:157-386 segmentVolumeView. Returns seg; `roots` receives the gradient-path
// roots (pore_extraction.hpp:273-311, ascent for sdf>0, descent otherwise).
void segment(const float* sdf, Dims r, const float* spc, int* seg, std::vector<int>& roots,
             int threads) {
  const long long n = (long long)r.x * r.y * r.z;
  const float min_sp = std::min(spc[0], std::min(spc[1], spc[2]));
  const float thr = -1.5f * min_sp;  // pore_extraction.hpp:163-164
  std::vector<int> labels(n), labelsN(n);
  roots.assign(n, 0);
  int* L = labels.data();

  // 1. markers (pore_extraction.hpp:174-178)
#pragma omp parallel for schedule(static) num_threads(threads)
  for (long long i = 0; i < n; ++i) L[i] = (sdf[i] < thr) ? int(i) : -1;

  // 2. union-find CCL rounds over 13 forward neighbours + flatten, to fixpoint
  //    (pore_extraction.hpp:183-230)
  static const int dz_l[13] = {1, 1, 1, 1, 1, 1, 1, 1, 1, 0, 0, 0, 0};
  static const int dy_l[13] = {-1, -1, -1, 0, 0, 0, 1, 1, 1, 1, 1, 1, 0};
  static const int dx_l[13] = {-1, 0, 1, -1, 0, 1, -1, 0, 1, -1, 0, 1, 1};
  int changed = 1;
  while (changed) {
    changed = 0;
#pragma omp parallel for schedule(dynamic, 1) num_threads(threads) reduction(| : changed)
    for (int iz = 0; iz < r.z; ++iz)
      for (int iy = 0; iy < r.y; ++iy)
        for (int ix = 0; ix < r.x; ++ix) {
          const int idx = get_idx(ix, iy, iz, r);
          const int my = ld(&L[idx]);
          if (my == -1) continue;
          for (int k = 0; k < 13; ++k) {
            const int ni = get_idx(ix + dx_l[k], iy + dy_l[k], iz + dz_l[k], r);
            const int nl = ld(&L[ni]);
            if (nl != -1 && my != nl) {
              int rm = my;
              while (rm != ld(&L[rm])) rm = ld(&L[rm]);
              int rn = nl;
              while (rn != ld(&L[rn])) rn = ld(&L[rn]);
              if (rm != rn) {
                const int small = rm < rn ? rm : rn, large = rm < rn ? rn : rm;
                amin(&L[large], small);
                changed = 1;
              }
            }
          }
        }
#pragma omp parallel for schedule(static) num_threads(threads)
    for (long long idx = 0; idx < n; ++idx) {
      int l = ld(&L[idx]);
      if (l != -1) {
        while (l != ld(&L[l])) l = ld(&L[l]);
        st(&L[idx], l);
      }
    }
  }

  // 3. Jacobi flood of the shallow solid: each sweep reads the previous sweep's labels
  //    (full copy per sweep), smallest labelled 26-neighbour wins (pore_extraction.hpp:237-269)
  changed = 1;
  while (changed) {
    changed = 0;
    std::memcpy(labelsN.data(), labels.data(), sizeof(int) * n);
    const int* Lc = labels.data();
    int* LN = labelsN.data();
#pragma omp parallel for schedule(dynamic, 1) num_threads(threads) reduction(| : changed)
    for (int iz = 0; iz < r.z; ++iz)
      for (int iy = 0; iy < r.y; ++iy)
        for (int ix = 0; ix < r.x; ++ix) {
          const int idx = get_idx(ix, iy, iz, r);
          if (sdf[idx] >= 0.0f) continue;
          if (Lc[idx] != -1) continue;
          int best = -1;
          for (int dz = -1; dz <= 1; ++dz)
            for (int dy = -1; dy <= 1; ++dy)
              for (int dx = -1; dx <= 1; ++dx) {
                if (dx == 0 && dy == 0 && dz == 0) continue;
                const int nl = Lc[get_idx(ix + dx, iy + dy, iz + dz, r)];
                if (nl != -1 && (best == -1 || nl < best)) best = nl;
              }
          if (best != -1) {
            LN[idx] = best;
            changed = 1;
          }
        }
    std::swap(labels, labelsN);
  }
  L = labels.data();

  // 4. gradient-path roots, at most 512 steps (pore_extraction.hpp:273-311)
  int* R = roots.data();
#pragma omp parallel for schedule(dynamic, 1) num_threads(threads)
  for (int iz = 0; iz < r.z; ++iz)
    for (int iy = 0; iy < r.y; ++iy)
      for (int ix = 0; ix < r.x; ++ix) {
        const int ci = get_idx(ix, iy, iz, r);
        const bool ascent = (sdf[ci] > 0.0f);
        int walker = ci;
        const int MAX_STEPS = 512;
        for (int s = 0; s < MAX_STEPS; ++s) {
          int best = walker;
          float bv = sdf[walker];
          const int wx = walker % r.x, wy = (walker / r.x) % r.y, wz = walker / (r.x * r.y);
          for (int dz = -1; dz <= 1; ++dz)
            for (int dy = -1; dy <= 1; ++dy)
              for (int dx = -1; dx <= 1; ++dx) {
                if (dx == 0 && dy == 0 && dz == 0) continue;
                const int ni = get_idx(wx + dx, wy + dy, wz + dz, r);
                const float nv = sdf[ni];
                if (ascent) {
                  if (nv > bv) {
                    bv = nv;
                    best = ni;
                  } else if (nv == bv && ni > best)
                    best = ni;
                } else {
                  if (nv < bv) {
                    bv = nv;
                    best = ni;
                  } else if (nv == bv && ni > best)
                    best = ni;
                }
              }
          if (best == walker) break;
          walker = best;
        }
        R[ci] = walker;
      }

  // 5. first-appearance renumbering (pore_extraction.hpp:319-382)
  constexpr int kBig = 0x7fffffff;
  std::vector<int> minPoreIdx(n, kBig), minSolidIdx(n, kBig);
  std::vector<int> poreFirst(n), solidFirst(n), poreRank(n), solidRank(n), poreId(n), solidId(n);
#pragma omp parallel for schedule(static) num_threads(threads)
  for (long long i = 0; i < n; ++i) {  // :331-337
    if (sdf[i] > 0.0f)
      amin(&minPoreIdx[R[i]], int(i));
    else if (L[i] != -1)
      amin(&minSolidIdx[L[i]], int(i));
  }
#pragma omp parallel for schedule(static) num_threads(threads)
  for (long long i = 0; i < n; ++i) {  // :340-347
    poreFirst[i] = (sdf[i] > 0.0f && minPoreIdx[R[i]] == int(i)) ? 1 : 0;
    solidFirst[i] = (sdf[i] <= 0.0f && L[i] != -1 && minSolidIdx[L[i]] == int(i)) ? 1 : 0;
  }
  // :350-365 exclusive prefix sums (two-pass parallel scan)
  auto exscan = [&](const std::vector<int>& f, std::vector<int>& out) {
    const int nt = std::max(1, threads);
    std::vector<long long> part(nt + 1, 0);
#pragma omp parallel num_threads(nt)
    {
      const int t = omp_get_thread_num(), T = omp_get_num_threads();
      const long long lo = n * t / T, hi = n * (t + 1) / T;
      long long s = 0;
      for (long long i = lo; i < hi; ++i) s += f[i];
      part[t + 1] = s;
#pragma omp barrier
#pragma omp single
      for (int k = 1; k <= T; ++k) part[k] += part[k - 1];
      long long u = part[t];
      for (long long i = lo; i < hi; ++i) {
        out[i] = int(u);
        u += f[i];
      }
    }
  };
  exscan(poreFirst, poreRank);
  exscan(solidFirst, solidRank);
#pragma omp parallel for schedule(static) num_threads(threads)
  for (long long i = 0; i < n; ++i) {  // :368-374
    if (poreFirst[i]) poreId[R[i]] = poreRank[i] + 1;
    if (solidFirst[i]) solidId[L[i]] = -(solidRank[i] + 1);
  }
#pragma omp parallel for schedule(static) num_threads(threads)
  for (long long i = 0; i < n; ++i)  // :378-381
    seg[i] = (sdf[i] > 0.0f) ? poreId[R[i]] : (L[i] == -1 ? 0 : solidId[L[i]]);
}

// pore_extraction.hpp:401-451 extractTopologyView: emit (min,max) across +x/+y/+z faces,
// host sort + unique.
std::vector<std::pair<int, int>> topology(const int* seg, Dims r, int threads) {
  std::vector<std::vector<std::pair<int, int>>> per_z(r.z);
#pragma omp parallel for schedule(dynamic, 1) num_threads(threads)
  for (int iz = 0; iz < r.z; ++iz)
    for (int iy = 0; iy < r.y; ++iy)
      for (int ix = 0; ix < r.x; ++ix) {
        const int idx = get_idx(ix, iy, iz, r);
        const int my = seg[idx];
        const int dx_l[3] = {1, 0, 0}, dy_l[3] = {0, 1, 0}, dz_l[3] = {0, 0, 1};
        for (int k = 0; k < 3; ++k) {
          const int nl = seg[get_idx(ix + dx_l[k], iy + dy_l[k], iz + dz_l[k], r)];
          if (my != nl) per_z[iz].push_back({my < nl ? my : nl, my < nl ? nl : my});
        }
      }
  std::vector<std::pair<int, int>> out;
  std::size_t tot = 0;
  for (auto& v : per_z) tot += v.size();
  out.reserve(tot);
  for (auto& v : per_z) out.insert(out.end(), v.begin(), v.end());
  std::sort(out.begin(), out.end());
  out.erase(std::unique(out.begin(), out.end()), out.end());
  return out;
}

}  // namespace

extern "C" {

void pnmo_free(void* p) { std::free(p); }

int64_t pnmo_extract_pores(const float* sdf, int nx, int ny, int nz, const float* origin,
                           const float* spacing, pnmo_pore** pores, int threads) {
  const long long n = (long long)nx * ny * nz;
  std::vector<pnmo_pore> v;
  if (n > 0) v = extract_pores(sdf, {nx, ny, nz}, origin, spacing, threads);
  *pores = dup(v);
  return (int64_t)v.size();
}

void pnmo_segment_volume(const float* sdf, int nx, int ny, int nz, const float* spacing,
                         int32_t* seg, int32_t* roots, int threads) {
  const long long n = (long long)nx * ny * nz;
  if (n <= 0) return;
  std::vector<int> r;
  segment(sdf, {nx, ny, nz}, spacing, seg, r, threads);
  if (roots) std::memcpy(roots, r.data(), sizeof(int) * n);
}

int64_t pnmo_extract_topology(const int32_t* seg, int nx, int ny, int nz, int32_t** pairs,
                              int threads) {
  const long long n = (long long)nx * ny * nz;
  std::vector<std::pair<int, int>> c;
  if (n > 0) c = topology(seg, {nx, ny, nz}, threads);
  std::vector<int> flat;
  flat.reserve(2 * c.size());
  for (auto& p : c) {
    flat.push_back(p.first);
    flat.push_back(p.second);
  }
  *pairs = dup(flat);
  return (int64_t)c.size();
}

// pore_extraction.hpp:1011-1025 extract_pore_network_k: the three stages on one SDF.
void pnmo_extract_pore_network(const float* sdf, int nx, int ny, int nz, const float* origin,
                               const float* spacing, pnmo_pore** pores, int64_t* n_pores,
                               int32_t* seg, int32_t** pairs, int64_t* n_pairs, int threads) {
  *n_pores = pnmo_extract_pores(sdf, nx, ny, nz, origin, spacing, pores, threads);
  pnmo_segment_volume(sdf, nx, ny, nz, spacing, seg, nullptr, threads);
  *n_pairs = pnmo_extract_topology(seg, nx, ny, nz, pairs, threads);
}

}  // extern "C"

// ---- network flow (pore_extraction.hpp:493-997) ---------------------------------------------
namespace {

pnmo_flow_result* empty_flow() {
  return static_cast<pnmo_flow_result*>(std::calloc(1, sizeof(pnmo_flow_result)));
}

pnmo_flow_result* network_flow(const float* sdf, Dims r, const float* org, const float* spc,
                               const double* u, const double* v, const double* w, const double* p,
                               const double* oxf, const double* oyf, const double* ozf,
                               const double* grad_p, int threads) {
  const long long n = (long long)r.x * r.y * r.z;
  if (n <= 0) return empty_flow();
  std::vector<int> seg(n), roots;
  segment(sdf, r, spc, seg.data(), roots, threads);
  const int* R = roots.data();

  // np = max seg (pore_extraction.hpp:514-524)
  int np = INT_MIN;
  for (long long i = 0; i < n; ++i) np = std::max(np, seg[i]);
  if (np <= 0) return empty_flow();  // reference: np==0 -> empty; np<0 undefined there

  // basin peaks (:527-533) — zero-initialised like the Kokkos view
  std::vector<int> peak(np, 0);
  for (long long i = 0; i < n; ++i)
    if (sdf[i] > 0.0f && R[i] == int(i)) peak[seg[i] - 1] = int(i);

  // pore centres (:534-566)
  std::vector<pnmo_pore> pores(np);
  {
    const float oxo = org[0], oyo = org[1], ozo = org[2];
    const float sx = spc[0], sy = spc[1], sz = spc[2];
#pragma omp parallel for schedule(static) num_threads(threads)
    for (int k = 0; k < np; ++k) {
      const int ci = peak[k];
      const int ix = ci % r.x, iy = (ci / r.x) % r.y, iz = ci / (r.x * r.y);
      float fx, fy, fz;
      centroid(sdf, ix, iy, iz, r, fx, fy, fz);
      pores[k] = {oxo + (ix + fx) * sx, oyo + (iy + fy) * sy, ozo + (iz + fz) * sz, sdf[ci]};
    }
  }

  const bool hasOpen = oxf != nullptr;

  // pore-centre pressures: trilinear periodic p (:581-613)
  std::vector<double> ppres(np);
  {
    const float oxo = org[0], oyo = org[1], ozo = org[2];
    const float sx = spc[0], sy = spc[1], sz = spc[2];
#pragma omp parallel for schedule(static) num_threads(threads)
    for (int k = 0; k < np; ++k) {
      const pnmo_pore po = pores[k];
      const double g[3] = {(po.x - oxo) / sx, (po.y - oyo) / sy, (po.z - ozo) / sz};
      int b[3];
      double f[3];
      for (int a = 0; a < 3; ++a) {
        const double fl = std::floor(g[a]);
        b[a] = static_cast<int>(fl);
        f[a] = g[a] - fl;
      }
      double acc = 0.0;
      for (int dz = 0; dz < 2; ++dz)
        for (int dy = 0; dy < 2; ++dy)
          for (int dx = 0; dx < 2; ++dx) {
            const double wt =
                (dx ? f[0] : 1.0 - f[0]) * (dy ? f[1] : 1.0 - f[1]) * (dz ? f[2] : 1.0 - f[2]);
            acc += wt * p[get_idx(b[0] + dx, b[1] + dy, b[2] + dz, r)];
          }
      ppres[k] = acc;
    }
  }

  // flow basins: ascent from EVERY cell, <= 512 steps, label = seg at the walker (:621-652)
  std::vector<int> flowLab(n);
#pragma omp parallel for schedule(dynamic, 4096) num_threads(threads)
  for (long long i0 = 0; i0 < n; ++i0) {
    int walker = int(i0);
    for (int s0 = 0; s0 < 512; ++s0) {
      int best = walker;
      float bv = sdf[walker];
      const int wx = walker % r.x, wy = (walker / r.x) % r.y, wz = walker / (r.x * r.y);
      for (int dz = -1; dz <= 1; ++dz)
        for (int dy = -1; dy <= 1; ++dy)
          for (int dx = -1; dx <= 1; ++dx) {
            if (dx == 0 && dy == 0 && dz == 0) continue;
            const int ni = get_idx(wx + dx, wy + dy, wz + dz, r);
            const float nv = sdf[ni];
            if (nv > bv) {
              bv = nv;
              best = ni;
            } else if (nv == bv && ni > best)
              best = ni;
          }
      if (best == walker) break;
      walker = best;
    }
    flowLab[i0] = seg[walker];
  }

  // per-patch face CCL (:670-819)
  const long long nf = 3 * n;
  constexpr long long kSent = 0x7ffffffffffffffeLL;
  std::vector<long long> fpar(nf), fpair(nf), par(nf);
  std::vector<char> core(nf);
  auto openness = [&](int d, int nb) -> double {
    return hasOpen ? (d == 0 ? oxf[nb] : (d == 1 ? oyf[nb] : ozf[nb])) : 1.0;
  };
#pragma omp parallel for schedule(static) num_threads(threads)
  for (int izz = 0; izz < r.z; ++izz)
    for (int iyy = 0; iyy < r.y; ++iyy)
      for (int ixx = 0; ixx < r.x; ++ixx) {  // face_init :681-696
        const int c = get_idx(ixx, iyy, izz, r);
        for (int d = 0; d < 3; ++d) {
          const long long f = 3 * (long long)c + d;
          const int nb = get_idx(ixx + (d == 0), iyy + (d == 1), izz + (d == 2), r);
          const int a = flowLab[c], b = flowLab[nb];
          const double opn = openness(d, nb);
          const bool itf = (a != b && a > 0 && b > 0 && opn > 0.0);
          core[f] = (itf && sdf[c] > 0.0f && sdf[nb] > 0.0f) ? 1 : 0;
          par[f] = core[f] ? f : -1;
          fpar[f] = itf ? (core[f] ? f : kSent) : -1;
          fpair[f] = itf ? (((long long)(a < b ? a : b) << 32) | (a < b ? b : a)) : -1;
        }
      }
  long long* PAR = par.data();
  auto cclPass = [&]() {  // :699-755
    int ch = 1;
    while (ch) {
      ch = 0;
#pragma omp parallel for schedule(dynamic, 1) num_threads(threads) reduction(| : ch)
      for (int izz = 0; izz < r.z; ++izz)
        for (int iyy = 0; iyy < r.y; ++iyy)
          for (int ixx = 0; ixx < r.x; ++ixx) {
            const int c = get_idx(ixx, iyy, izz, r);
            for (int d = 0; d < 3; ++d) {
              const long long f = 3 * (long long)c + d;
              if (ld(&PAR[f]) < 0) continue;
              const long long pk = fpair[f];
              for (int dz = -1; dz <= 1; ++dz)
                for (int dy = -1; dy <= 1; ++dy)
                  for (int dx = -1; dx <= 1; ++dx) {
                    const int c2 = get_idx(ixx + dx, iyy + dy, izz + dz, r);
                    for (int d2 = 0; d2 < 3; ++d2) {
                      const long long f2 = 3 * (long long)c2 + d2;
                      if (f2 == f || ld(&PAR[f2]) < 0 || fpair[f2] != pk) continue;
                      const int Dx = 2 * dx + (d2 == 0) - (d == 0);
                      const int Dy = 2 * dy + (d2 == 1) - (d == 1);
                      const int Dz = 2 * dz + (d2 == 2) - (d == 2);
                      if (Dx * Dx + Dy * Dy + Dz * Dz > 8) continue;
                      long long rm = f;
                      while (rm != ld(&PAR[rm])) rm = ld(&PAR[rm]);
                      long long rn = f2;
                      while (rn != ld(&PAR[rn])) rn = ld(&PAR[rn]);
                      if (rm != rn) {
                        const long long sml = rm < rn ? rm : rn, lrg = rm < rn ? rn : rm;
                        amin(&PAR[lrg], sml);
                        ch = 1;
                      }
                    }
                  }
            }
          }
#pragma omp parallel for schedule(static) num_threads(threads)
      for (long long f = 0; f < nf; ++f) {
        long long l = ld(&PAR[f]);
        if (l >= 0) {
          while (l != ld(&PAR[l])) l = ld(&PAR[l]);
          st(&PAR[f], l);
        }
      }
    }
  };
  cclPass();  // core tier
#pragma omp parallel for schedule(static) num_threads(threads)
  for (long long f = 0; f < nf; ++f)  // core_label :757-761
    if (core[f]) fpar[f] = par[f];
  {  // film attachment, in-place min propagation to fixpoint (:763-805)
    long long* FP = fpar.data();
    int ch = 1;
    while (ch) {
      ch = 0;
#pragma omp parallel for schedule(dynamic, 1) num_threads(threads) reduction(| : ch)
      for (int izz = 0; izz < r.z; ++izz)
        for (int iyy = 0; iyy < r.y; ++iyy)
          for (int ixx = 0; ixx < r.x; ++ixx) {
            const int c = get_idx(ixx, iyy, izz, r);
            for (int d = 0; d < 3; ++d) {
              const long long f = 3 * (long long)c + d;
              if (ld(&FP[f]) < 0 || core[f]) continue;
              long long best = ld(&FP[f]);
              const long long pk = fpair[f];
              for (int dz = -1; dz <= 1; ++dz)
                for (int dy = -1; dy <= 1; ++dy)
                  for (int dx = -1; dx <= 1; ++dx) {
                    const int c2 = get_idx(ixx + dx, iyy + dy, izz + dz, r);
                    for (int d2 = 0; d2 < 3; ++d2) {
                      const long long f2 = 3 * (long long)c2 + d2;
                      if (f2 == f || fpair[f2] != pk) continue;
                      const long long l2 = ld(&FP[f2]);
                      if (l2 < 0 || l2 >= kSent || l2 >= best) continue;
                      const int Dx = 2 * dx + (d2 == 0) - (d == 0);
                      const int Dy = 2 * dy + (d2 == 1) - (d == 1);
                      const int Dz = 2 * dz + (d2 == 2) - (d == 2);
                      if (Dx * Dx + Dy * Dy + Dz * Dz > 8) continue;
                      best = l2;
                    }
                  }
              if (best < ld(&FP[f])) {
                st(&FP[f], best);
                ch = 1;
              }
            }
          }
    }
  }
#pragma omp parallel for schedule(static) num_threads(threads)
  for (long long f = 0; f < nf; ++f) par[f] = (fpar[f] == kSent) ? f : -1;  // :807-809
  cclPass();                                                                 // leftover tier
#pragma omp parallel for schedule(static) num_threads(threads)
  for (long long f = 0; f < nf; ++f)
    if (fpar[f] == kSent) fpar[f] = par[f];  // :812-817

  // patch roots -> throat slots ordered by (pair key, root fid) (:821-862)
  std::vector<std::pair<int, int>> throats;
  std::vector<long long> rootF, rootSlotKey;
  {
    std::vector<long long> hr, hp;
    for (long long f = 0; f < nf; ++f)
      if (fpar[f] == f) {
        hr.push_back(f);
        hp.push_back(fpair[f]);
      }
    std::vector<std::size_t> ord(hr.size());
    std::iota(ord.begin(), ord.end(), 0);
    std::sort(ord.begin(), ord.end(), [&](std::size_t a, std::size_t b) {
      return hp[a] != hp[b] ? hp[a] < hp[b] : hr[a] < hr[b];
    });
    for (auto i : ord) {
      throats.push_back({int(hp[i] >> 32), int(hp[i] & 0x7fffffff)});
      rootF.push_back(hr[i]);
    }
    rootSlotKey = rootF;
    std::sort(rootSlotKey.begin(), rootSlotKey.end());
  }
  const std::size_t nt = throats.size();
  std::vector<int> slotOf(nt);
  for (std::size_t t = 0; t < nt; ++t) {
    const auto it = std::lower_bound(rootSlotKey.begin(), rootSlotKey.end(), rootF[t]);
    slotOf[std::size_t(it - rootSlotKey.begin())] = int(t);
  }

  // throat fluxes, areas, centroid moments; per-pore residual (:866-944)
  std::vector<double> Q(nt, 0.0), A(nt, 0.0), Cx(nt, 0.0), Cy(nt, 0.0), Cz(nt, 0.0), resid(np, 0.0);
  // sums of |q| over the same terms: the per-element scale of a cancelling sum's rounding error
  std::vector<double> absQ(nt, 0.0), absR(np, 0.0);
  {
    const double Ax = double(spc[1]) * spc[2], Ay = double(spc[0]) * spc[2],
                 Az = double(spc[0]) * spc[1];
    const long long ntl = (long long)nt;
    const float oxo = org[0], oyo = org[1], ozo = org[2];
    const float sx = spc[0], sy = spc[1], sz = spc[2];
    const double Lx = double(r.x) * sx, Ly = double(r.y) * sy, Lz = double(r.z) * sz;
#pragma omp parallel for schedule(dynamic, 1) num_threads(threads)
    for (int izz = 0; izz < r.z; ++izz)
      for (int iyy = 0; iyy < r.y; ++iyy)
        for (int ixx = 0; ixx < r.x; ++ixx) {
          const int c = get_idx(ixx, iyy, izz, r);
          const int a = flowLab[c];
          for (int d = 0; d < 3; ++d) {
            const int nb = get_idx(ixx + (d == 0), iyy + (d == 1), izz + (d == 2), r);
            const int b = flowLab[nb];
            if (a == b) continue;
            const double vel = d == 0 ? u[nb] : (d == 1 ? v[nb] : w[nb]);
            const double opn = openness(d, nb);
            const double area = d == 0 ? Ax : (d == 1 ? Ay : Az);
            const double q = opn * vel * area;
            if (a > 0) aadd(&resid[a - 1], q);
            if (b > 0) aadd(&resid[b - 1], -q);
            if (a > 0) aadd(&absR[a - 1], std::fabs(q));
            if (b > 0) aadd(&absR[b - 1], std::fabs(q));
            const long long rt = fpar[3 * (long long)c + d];
            if (rt >= 0) {
              long long l = 0, hgh = ntl - 1, slot = -1;
              while (l <= hgh) {
                const long long mid = l + (hgh - l) / 2;
                if (rootSlotKey[mid] == rt) {
                  slot = slotOf[mid];
                  break;
                }
                if (rootSlotKey[mid] < rt)
                  l = mid + 1;
                else
                  hgh = mid - 1;
              }
              const int lo = a < b ? a : b;
              if (slot >= 0) {
                const double w0 = opn * area;
                aadd(&Q[slot], a < b ? q : -q);
                aadd(&absQ[slot], std::fabs(q));
                aadd(&A[slot], w0);
                const int pk = peak[lo - 1];
                const int pkx = pk % r.x, pky = (pk / r.x) % r.y, pkz = pk / (r.x * r.y);
                double fp[3] = {oxo + (ixx + (d == 0 ? 0.5 : 0.0)) * double(sx),
                                oyo + (iyy + (d == 1 ? 0.5 : 0.0)) * double(sy),
                                ozo + (izz + (d == 2 ? 0.5 : 0.0)) * double(sz)};
                const double pc[3] = {oxo + pkx * double(sx), oyo + pky * double(sy),
                                      ozo + pkz * double(sz)};
                const double Lw[3] = {Lx, Ly, Lz};
                for (int a2 = 0; a2 < 3; ++a2) {
                  double dv = fp[a2] - pc[a2];
                  dv -= Lw[a2] * std::round(dv / Lw[a2]);
                  fp[a2] = dv;
                }
                aadd(&Cx[slot], w0 * fp[0]);
                aadd(&Cy[slot], w0 * fp[1]);
                aadd(&Cz[slot], w0 * fp[2]);
              }
            }
          }
        }
  }

  // total-pressure drop per throat (host, :962-995)
  std::vector<double> dp(nt);
  const double L[3] = {double(r.x) * spc[0], double(r.y) * spc[1], double(r.z) * spc[2]};
  const int N[3] = {r.x, r.y, r.z};
  for (std::size_t t = 0; t < nt; ++t) {
    const int li = throats[t].first, lj = throats[t].second;
    const pnmo_pore& pi = pores[li - 1];
    const pnmo_pore& pj = pores[lj - 1];
    const double aw = A[t];
    const int pk = peak[li - 1];
    const double anc[3] = {org[0] + (pk % r.x) * double(spc[0]),
                           org[1] + ((pk / r.x) % r.y) * double(spc[1]),
                           org[2] + (pk / (r.x * r.y)) * double(spc[2])};
    const int pkj = peak[lj - 1];
    const double ancj[3] = {org[0] + (pkj % r.x) * double(spc[0]),
                            org[1] + ((pkj / r.x) % r.y) * double(spc[1]),
                            org[2] + (pkj / (r.x * r.y)) * double(spc[2])};
    double macro = 0.0;
    const double pip[3] = {double(pi.x), double(pi.y), double(pi.z)};
    const double pjp[3] = {double(pj.x), double(pj.y), double(pj.z)};
    for (int a = 0; a < 3; ++a) {
      const double ct = (Cx[t] * (a == 0) + Cy[t] * (a == 1) + Cz[t] * (a == 2)) / aw;
      const long long Dc = llround((ancj[a] - anc[a]) / double(spc[a])) -
                           llround(ct / double(spc[a]) + 1e-6);
      const long long k = llround(double(Dc) / N[a]);
      macro += grad_p[a] * ((pjp[a] - pip[a]) - L[a] * double(k));
    }
    dp[t] = (ppres[li - 1] - ppres[lj - 1]) - macro;
  }

  auto* res = empty_flow();
  res->n_pores = np;
  res->n_throats = (int64_t)nt;
  res->pores = dup(pores);
  res->pore_pressure = dup(ppres);
  res->pore_residual = dup(resid);
  std::vector<int> tf;
  tf.reserve(2 * nt);
  for (auto& q : throats) {
    tf.push_back(q.first);
    tf.push_back(q.second);
  }
  res->throats = dup(tf);
  res->throat_flow = dup(Q);
  res->throat_area = dup(A);
  res->throat_dp = dup(dp);
  // per-throat patch root fid and peak voxels, exposed for stage-level parity checks
  res->throat_root = dup(rootF);
  res->pore_peak = dup(peak);
  res->throat_absflow = dup(absQ);
  res->pore_absflux = dup(absR);
  return res;
}

}  // namespace

extern "C" {

pnmo_flow_result* pnmo_extract_network_flow(const float* sdf, int nx, int ny, int nz,
                                            const float* origin, const float* spacing,
                                            const double* u, const double* v, const double* w,
                                            const double* p, const double* ox, const double* oy,
                                            const double* oz, const double* grad_p, int threads) {
  return network_flow(sdf, {nx, ny, nz}, origin, spacing, u, v, w, p, ox, oy, oz, grad_p,
                      threads);
}

void pnmo_flow_result_free(pnmo_flow_result* r) {
  if (!r) return;
  std::free(r->pores);
  std::free(r->pore_pressure);
  std::free(r->pore_residual);
  std::free(r->throats);
  std::free(r->throat_flow);
  std::free(r->throat_area);
  std::free(r->throat_dp);
  std::free(r->throat_root);
  std::free(r->pore_peak);
  std::free(r->throat_absflow);
  std::free(r->pore_absflux);
  std::free(r);
}

}  // extern "C"
