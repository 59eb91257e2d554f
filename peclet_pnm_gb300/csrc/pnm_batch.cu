// Batched extraction (pnm_batch_*): plans a ragged batch of periodic volumes once, allocates every
// device buffer up front, and runs the whole pipeline for all volumes with one launch per stage
// (enqueue_batch in pnm_segment.cu). The first run is captured into a CUDA graph and later runs
// replay it; nothing inside a run waits on the host. Capacities that depend on the data (the pair
// hash set, the pore records) are checked after the run and grown for a re-run when exceeded.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <new>
#include <sstream>
#include <string>
#include <vector>

#include "pnm_ctx.h"
#include "pnm_device.cuh"
#include "pnm_geo.cuh"

namespace pnm {
namespace {

constexpr long long kMaxBatchVoxels = (long long)INT_MAX - 64;
constexpr long long kMaxPoresPerVolume = 1000000;  // max_pores, pore_extraction.hpp:77
constexpr size_t kAlign = 256;

inline size_t align_up(size_t x) { return (x + kAlign - 1) & ~(kAlign - 1); }
inline long long pow2_at_least(long long x) {
  long long p = 1;
  while (p < x) p <<= 1;
  return p;
}

// Sizes of one plan (derived from the volume shapes and the two growable capacities).
struct Layout {
  std::vector<VolDesc> vols;
  long long n_total = 0, words = 0, tiles = 0, bricks = 0;
  long long n_words = 0;  // marker-bitmap words of all volumes
  long long hash_cap = 0, pore_cap = 0;
  int label_bits = 0;
  size_t arena = 0, pairbuf = 0, porebuf = 0;
};

inline long long boxes(int nx, int ny, int nz, int bx, int by, int bz) {
  return (long long)((nx + bx - 1) / bx) * ((ny + by - 1) / by) * ((nz + bz - 1) / bz);
}

long long scan_len(long long m) { return m / SCAN_TILE + 2; }
long long rs_blocks(long long cap) { return (cap + RS_TILE - 1) / RS_TILE; }

Status make_layout(int nvol, const int32_t* dims, const float* org, const float* spc,
                   long long hash_cap, long long pore_cap, Layout* L, int tile_z = 16) {
  if (nvol <= 0) return Status{PNM_ERR_ARG, "a batch needs at least one volume"};
  if (!dims) return Status{PNM_ERR_ARG, "dims is null"};
  L->vols.assign(nvol, VolDesc{});
  long long off = 0, tiles = 0, bricks = 0, words = 0;
  for (int i = 0; i < nvol; ++i) {
    const int nx = dims[3 * i], ny = dims[3 * i + 1], nz = dims[3 * i + 2];
    if (nx < 0 || ny < 0 || nz < 0) return Status{PNM_ERR_ARG, "dims must be non-negative"};
    const long long n = (long long)nx * ny * nz;
    if (n > kMaxBatchVoxels || off + n > kMaxBatchVoxels)
      return Status{PNM_ERR_SHAPE, "batch too large: voxel ids are int32 (< 2^31 - 64 in all)"};
    VolDesc& v = L->vols[i];
    v.off = (int)off;
    v.nx = nx;
    v.ny = ny;
    v.nz = nz;
    v.tile0 = (int)tiles;
    v.brick0 = (int)bricks;
    v.word0 = (int)words;
    words += (long long)nz * ny * ((nx + 31) / 32);
    float mn = 1.0f;
    if (spc) {
      for (int a = 0; a < 3; ++a)
        if (!(spc[3 * i + a] > 0.0f) || !std::isfinite(spc[3 * i + a]))
          return Status{PNM_ERR_ARG, "spacing must be finite and positive"};
      mn = std::min(spc[3 * i], std::min(spc[3 * i + 1], spc[3 * i + 2]));
      v.sx = spc[3 * i];
      v.sy = spc[3 * i + 1];
      v.sz = spc[3 * i + 2];
    } else {
      v.sx = v.sy = v.sz = 1.0f;
    }
    v.thr = -1.5f * mn;  // pore_extraction.hpp:163-164
    v.ox = org ? org[3 * i] : 0.0f;
    v.oy = org ? org[3 * i + 1] : 0.0f;
    v.oz = org ? org[3 * i + 2] : 0.0f;
    if (n > 0) {
      tiles += boxes(nx, ny, nz, 32, 8, tile_z);
      bricks += boxes(nx, ny, nz, 32, 8, 16);
    }
    L->n_total = off + n;
    off = (off + n + 31) & ~31LL;  // next volume starts on a bitmap word
  }
  const long long n = std::max<long long>(L->n_total, 1);
  L->words = (n + 31) / 32;
  L->tiles = tiles;
  L->bricks = bricks;
  L->n_words = std::max<long long>(words, 1);
  L->hash_cap = hash_cap > 0 ? hash_cap : pow2_at_least(std::max<long long>(1 << 14, n / 16));
  L->pore_cap = pore_cap > 0 ? pore_cap : n / 32 + 1024;
  int b = 1;
  while ((1ll << b) <= n + nvol + 1) ++b;  // pair labels span at most one per voxel + one per volume
  L->label_bits = b;
  const long long W = L->words;
  const long long sl = std::max(scan_len(W), std::max(scan_len(L->hash_cap),
                                                      scan_len(256 * rs_blocks(L->hash_cap))));
  size_t a = 0;
  a += align_up(n * 4);                     // sdf
  a += align_up(n + 64);                    // code
  a += 9 * align_up(n * 4);                 // nxt L key seg ulist keylist f0 f1 tmp
  a += align_up((size_t)L->n_words * 4);    // marker bitmap
  a += 3 * align_up(W * 4);                 // peakbits firstP firstS
  a += 3 * align_up((W + 1) * 4);           // prefP prefS peakpref
  a += align_up(sl * 4);                    // scan partials
  a += align_up(CNT_COUNT * 4) + align_up(8);
  a += align_up(nvol * sizeof(VolDesc)) + align_up(nvol * sizeof(VolResult));
  L->arena = a;
  const long long hc = L->hash_cap;
  L->pairbuf = align_up(hc * 8) + align_up((hc + 1) * 4) + 2 * align_up(hc * 8) +
               align_up((256 * rs_blocks(hc) + 1) * 4) + align_up(2 * hc * 4 + 8);
  L->porebuf = align_up(L->pore_cap * sizeof(pnm_pore));
  return Status::ok();
}

}  // namespace
}  // namespace pnm

using pnm::Status;

struct pnm_batch {
  int device = 0;
  int sm_count = 0;
  cudaStream_t stream = nullptr;
  pnm::Layout lay;
  pnm::BatchPlan plan;
  void* arena = nullptr;
  void* pairbuf = nullptr;
  void* porebuf = nullptr;
  void* pinned = nullptr;
  bool own_stream = true;
  bool own_pinned = true;
  bool use_graph = true;
  pnm_tuning tuning{16, 16, 8, 4};
  cudaGraphExec_t exec = nullptr;
  long long launches_per_run = 0;
  long long runs = 0;
  bool pending = false;    // a launched run not yet waited for
  bool have_result = false;
  std::string last_error;
  std::string graph_note;
};

namespace {

using pnm::BatchPlan;
using pnm::Layout;

Status carve(pnm_batch& b) {
  const Layout& L = b.lay;
  BatchPlan& p = b.plan;
  const long long n = std::max<long long>(L.n_total, 1), W = L.words;
  char* a = static_cast<char*>(b.arena);
  auto take = [&](size_t bytes) {
    char* r = a;
    a += pnm::align_up(bytes);
    return r;
  };
  p.nvol = (int)L.vols.size();
  p.n_total = L.n_total;
  p.words = W;
  p.tiles = L.tiles;
  p.bricks = L.bricks;
  p.sm_count = b.sm_count;
  p.sdf = reinterpret_cast<float*>(take(n * 4));
  p.code = reinterpret_cast<uint8_t*>(take(n + 64));
  int** ints[] = {&p.nxt, &p.L, &p.key, &p.seg, &p.ulist, &p.keylist, &p.f0, &p.f1, &p.tmp};
  for (int** q : ints) *q = reinterpret_cast<int*>(take(n * 4));
  p.n_words = L.n_words;
  p.mbits = reinterpret_cast<uint32_t*>(take((size_t)L.n_words * 4));
  p.peakbits = reinterpret_cast<uint32_t*>(take(W * 4));
  p.firstP = reinterpret_cast<uint32_t*>(take(W * 4));
  p.firstS = reinterpret_cast<uint32_t*>(take(W * 4));
  p.prefP = reinterpret_cast<unsigned*>(take((W + 1) * 4));
  p.prefS = reinterpret_cast<unsigned*>(take((W + 1) * 4));
  p.peakpref = reinterpret_cast<unsigned*>(take((W + 1) * 4));
  const long long hc = L.hash_cap;
  const long long sl = std::max(pnm::scan_len(W), std::max(pnm::scan_len(hc),
                                                           pnm::scan_len(256 * pnm::rs_blocks(hc))));
  p.scan_tmp = reinterpret_cast<unsigned*>(take(sl * 4));
  p.cnt = reinterpret_cast<unsigned*>(take(pnm::CNT_COUNT * 4));
  p.range = reinterpret_cast<int*>(take(8));
  p.vols = reinterpret_cast<pnm::VolDesc*>(take(p.nvol * sizeof(pnm::VolDesc)));
  p.res = reinterpret_cast<pnm::VolResult*>(take(p.nvol * sizeof(pnm::VolResult)));
  char* h = static_cast<char*>(b.pairbuf);
  auto takeh = [&](size_t bytes) {
    char* r = h;
    h += pnm::align_up(bytes);
    return r;
  };
  p.hash_cap = hc;
  p.table = reinterpret_cast<unsigned long long*>(takeh(hc * 8));
  p.hpos = reinterpret_cast<unsigned*>(takeh((hc + 1) * 4));
  p.ka = reinterpret_cast<uint64_t*>(takeh(hc * 8));
  p.kb = reinterpret_cast<uint64_t*>(takeh(hc * 8));
  p.hist = reinterpret_cast<unsigned*>(takeh((256 * pnm::rs_blocks(hc) + 1) * 4));
  p.pairs = reinterpret_cast<int*>(takeh(2 * hc * 4 + 8));
  p.label_bits = L.label_bits;
  p.pores = static_cast<pnm_pore*>(b.porebuf);
  p.pore_cap = L.pore_cap;
  p.h_cnt = static_cast<unsigned*>(b.pinned);
  p.h_res = reinterpret_cast<pnm::VolResult*>(static_cast<char*>(b.pinned) + 256);
  p.max_sweeps = 1 << 20;
  p.tile_z = b.tuning.tile_z;
  p.grid_per_sm = b.tuning.blocks_per_sm;
  p.ccl_per_sm = b.tuning.ccl_blocks_per_sm;
  p.flood_blocks_per_sm = b.tuning.flood_blocks_per_sm;
  return Status::ok();
}

void drop_graph(pnm_batch& b) {
  if (b.exec) cudaGraphExecDestroy(b.exec);
  b.exec = nullptr;
}

// (Re)allocates the growable buffers after a capacity change; the graph is re-captured.
Status regrow(pnm_batch& b, long long hash_cap, long long pore_cap) {
  Layout L;
  std::vector<int32_t> dims;
  for (const auto& v : b.lay.vols) {
    dims.push_back(v.nx);
    dims.push_back(v.ny);
    dims.push_back(v.nz);
  }
  // origin / spacing stay as planned: only capacities change
  std::vector<pnm::VolDesc> keep = b.lay.vols;
  PNM_TRY(pnm::make_layout((int)keep.size(), dims.data(), nullptr, nullptr, hash_cap, pore_cap, &L,
                           b.tuning.tile_z));
  L.vols = keep;
  PNM_CUDA(cudaStreamSynchronize(b.stream));
  drop_graph(b);
  if (L.pairbuf != b.lay.pairbuf) {
    cudaFreeAsync(b.pairbuf, b.stream);
    b.pairbuf = nullptr;
    PNM_CUDA(cudaMallocAsync(&b.pairbuf, L.pairbuf, b.stream));
  }
  if (L.porebuf != b.lay.porebuf) {
    cudaFreeAsync(b.porebuf, b.stream);
    b.porebuf = nullptr;
    PNM_CUDA(cudaMallocAsync(&b.porebuf, L.porebuf, b.stream));
  }
  L.arena = b.lay.arena;  // unchanged sizes (the scan partials were sized for the first hash cap)
  const long long W = L.words, hc = L.hash_cap;
  const long long need = std::max(pnm::scan_len(W), std::max(pnm::scan_len(hc),
                                                             pnm::scan_len(256 * pnm::rs_blocks(hc))));
  const long long had = std::max(pnm::scan_len(W),
                                 std::max(pnm::scan_len(b.lay.hash_cap),
                                          pnm::scan_len(256 * pnm::rs_blocks(b.lay.hash_cap))));
  if (need > had) {  // a larger hash set needs larger scan partials: re-plan the arena too
    Layout full;
    PNM_TRY(pnm::make_layout((int)keep.size(), dims.data(), nullptr, nullptr, hash_cap, pore_cap,
                             &full, b.tuning.tile_z));
    const size_t sdf_bytes = (size_t)b.lay.n_total * 4;
    void* na = nullptr;
    PNM_CUDA(cudaMallocAsync(&na, full.arena, b.stream));
    // the SDF lives at the start of the arena: keep it across the move
    PNM_CUDA(cudaMemcpyAsync(na, b.plan.sdf, sdf_bytes, cudaMemcpyDeviceToDevice, b.stream));
    cudaFreeAsync(b.arena, b.stream);
    b.arena = na;
    L.arena = full.arena;
  }
  b.lay = L;
  PNM_TRY(carve(b));
  PNM_CUDA(cudaMemcpyAsync(const_cast<pnm::VolDesc*>(b.plan.vols), b.lay.vols.data(),
                           b.lay.vols.size() * sizeof(pnm::VolDesc), cudaMemcpyHostToDevice,
                           b.stream));
  PNM_CUDA(cudaStreamSynchronize(b.stream));
  return Status::ok();
}

Status launch(pnm_batch& b) {
  PNM_CUDA(cudaSetDevice(b.device));
  if (b.lay.n_total == 0) {  // nothing to extract: results are all empty
    b.pending = true;
    return Status::ok();
  }
  if (b.use_graph && !b.exec) {
    cudaGraph_t g = nullptr;
    long long n_launch = 0;
    cudaError_t e = cudaStreamBeginCapture(b.stream, cudaStreamCaptureModeThreadLocal);
    Status st = Status::ok();
    if (e == cudaSuccess) {
      st = pnm::enqueue_batch(b.plan, b.stream, &n_launch);
      e = cudaStreamEndCapture(b.stream, &g);
    }
    if (e == cudaSuccess && st.good() && g) {
      e = cudaGraphInstantiate(&b.exec, g, 0);
    }
    if (g) cudaGraphDestroy(g);
    if (e != cudaSuccess || !st.good() || !b.exec) {
      // capture unavailable (for example a cooperative launch inside capture): run eagerly
      b.graph_note = std::string("graph capture failed: ") +
                     (st.good() ? cudaGetErrorString(e) : st.msg.c_str());
      cudaGetLastError();
      b.exec = nullptr;
      b.use_graph = false;
    } else {
      b.launches_per_run = n_launch;
    }
  }
  if (b.exec) {
    PNM_CUDA(cudaGraphLaunch(b.exec, b.stream));
  } else {
    long long n_launch = 0;
    PNM_TRY(pnm::enqueue_batch(b.plan, b.stream, &n_launch));
    b.launches_per_run = n_launch;
  }
  b.pending = true;
  return Status::ok();
}

Status wait_checked(pnm_batch& b) {
  if (!b.pending) return Status{PNM_ERR_ARG, "no run was launched"};
  PNM_CUDA(cudaSetDevice(b.device));
  for (int attempt = 0; attempt < 6; ++attempt) {
    PNM_CUDA(cudaStreamSynchronize(b.stream));
    b.pending = false;
    if (b.lay.n_total == 0) {
      b.have_result = true;
      ++b.runs;
      return Status::ok();
    }
    const unsigned err = b.plan.h_cnt[pnm::CNT_ERR];
    if (err & pnm::ERRF_UF_LIMIT)
      return Status{PNM_ERR_NOT_CONVERGED, "union-find exceeded its iteration limit"};
    if (err & pnm::ERRF_FLOOD_LIMIT) return Status{PNM_ERR_NOT_CONVERGED, "flood did not converge"};
    if (err & pnm::ERRF_BARRIER)
      return Status{PNM_ERR_NOT_CONVERGED,
                    "flood loop: a grid barrier wait ran out (blocks not all resident?)"};
    if (err & pnm::ERRF_LABEL_RANGE)
      return Status{PNM_ERR_INTERNAL, "renumbering: a label minimum is outside the volume"};
    long long hc = b.lay.hash_cap, pc = b.lay.pore_cap;
    bool grow = false;
    if (err & pnm::ERRF_HASH_FULL) {
      hc *= 4;
      grow = true;
    }
    const long long peaks = b.plan.h_cnt[pnm::CNT_PEAKS];
    if (peaks > pc) {
      pc = peaks + peaks / 8 + 1024;
      grow = true;
    }
    if (!grow) {
      b.have_result = true;
      ++b.runs;
      return Status::ok();
    }
    PNM_TRY(regrow(b, hc, pc));
    PNM_TRY(launch(b));
  }
  return Status{PNM_ERR_INTERNAL, "batch capacities kept growing"};
}

// ---- launch-shape tuning -------------------------------------------------------------------------
bool tuning_valid(const pnm_tuning& t) {
  return (t.tile_z == 4 || t.tile_z == 8 || t.tile_z == 16) && t.blocks_per_sm >= 1 &&
         t.blocks_per_sm <= 32 && t.ccl_blocks_per_sm >= 1 && t.ccl_blocks_per_sm <= 64 &&
         t.flood_blocks_per_sm >= 1 && t.flood_blocks_per_sm <= 4;
}

// Re-plans the tile numbering when the tile depth changes; the graph is captured again.
Status apply_tuning(pnm_batch& b, const pnm_tuning& t) {
  if (!tuning_valid(t)) return Status{PNM_ERR_ARG, "invalid tuning"};
  PNM_CUDA(cudaSetDevice(b.device));
  PNM_CUDA(cudaStreamSynchronize(b.stream));
  if (t.tile_z != b.tuning.tile_z) {
    long long tiles = 0;
    for (auto& v : b.lay.vols) {
      v.tile0 = (int)tiles;
      if ((long long)v.nx * v.ny * v.nz > 0) tiles += pnm::boxes(v.nx, v.ny, v.nz, 32, 8, t.tile_z);
    }
    b.lay.tiles = tiles;
    PNM_CUDA(cudaMemcpyAsync(const_cast<pnm::VolDesc*>(b.plan.vols), b.lay.vols.data(),
                             b.lay.vols.size() * sizeof(pnm::VolDesc), cudaMemcpyHostToDevice,
                             b.stream));
    PNM_CUDA(cudaStreamSynchronize(b.stream));
  }
  b.tuning = t;
  b.plan.tiles = b.lay.tiles;
  b.plan.tile_z = t.tile_z;
  b.plan.grid_per_sm = t.blocks_per_sm;
  b.plan.ccl_per_sm = t.ccl_blocks_per_sm;
  b.plan.flood_blocks_per_sm = t.flood_blocks_per_sm;
  drop_graph(b);
  return Status::ok();
}

// Median device time of `reps` runs enqueued without a graph (after one untimed run).
Status time_runs(pnm_batch& b, int reps, double* ms) {
  cudaEvent_t e0, e1;
  PNM_CUDA(cudaEventCreate(&e0));
  PNM_CUDA(cudaEventCreate(&e1));
  std::vector<double> t;
  long long nl = 0;
  Status st = Status::ok();
  for (int r = 0; r <= reps && st.good(); ++r) {
    cudaEventRecord(e0, b.stream);
    st = pnm::enqueue_batch(b.plan, b.stream, &nl);
    cudaEventRecord(e1, b.stream);
    if (cudaStreamSynchronize(b.stream) != cudaSuccess) st = Status{PNM_ERR_CUDA, "tuning run"};
    float f = 0.0f;
    cudaEventElapsedTime(&f, e0, e1);
    if (r > 0) t.push_back(f);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  PNM_TRY(st);
  if (b.plan.h_cnt[pnm::CNT_ERR] != 0)
    return Status{PNM_ERR_INTERNAL, "tuning run reported a device error"};
  std::sort(t.begin(), t.end());
  *ms = t.empty() ? 0.0 : t[t.size() / 2];
  return Status::ok();
}

// Size class of a batch: device, typical edge (cube root of the mean volume, in the bins the
// batched workloads use) and the volume count's power of two.
std::string size_class(const pnm_batch& b) {
  cudaDeviceProp prop;
  std::string dev = "device";
  if (cudaGetDeviceProperties(&prop, b.device) == cudaSuccess) dev = prop.name;
  for (char& c : dev)
    if (c == ' ' || c == '|') c = '_';
  const double nv = (double)b.lay.vols.size();
  long long vox = 0;
  for (const auto& v : b.lay.vols) vox += (long long)v.nx * v.ny * v.nz;
  const double edge = std::cbrt((double)vox / std::max(nv, 1.0));
  static const int bins[] = {32, 48, 64, 96, 128, 160, 192, 256, 384, 512, 768, 1024};
  int best = bins[0];
  for (int e : bins)
    if (std::fabs(std::log(edge + 1.0) - std::log((double)e)) <
        std::fabs(std::log(edge + 1.0) - std::log((double)best)))
      best = e;
  int nb = 0;
  while ((1 << (nb + 1)) <= (int)nv) ++nb;
  return dev + "|e" + std::to_string(best) + "|n" + std::to_string(1 << nb);
}

bool cache_lookup(const char* path, const std::string& key, pnm_tuning* t) {
  if (!path) return false;
  std::ifstream f(path);
  std::string line;
  bool found = false;
  while (std::getline(f, line)) {
    std::istringstream is(line);
    std::string k;
    pnm_tuning c{};
    double ms = 0;
    if (is >> k >> c.tile_z >> c.blocks_per_sm >> c.ccl_blocks_per_sm >> c.flood_blocks_per_sm >>
        ms) {
      if (k == key && tuning_valid(c)) {
        *t = c;
        found = true;  // the last entry wins
      }
    }
  }
  return found;
}

void cache_store(const char* path, const std::string& key, const pnm_tuning& t, double ms) {
  if (!path) return;
  std::vector<std::string> keep;
  {
    std::ifstream f(path);
    std::string line;
    while (std::getline(f, line)) {
      std::istringstream is(line);
      std::string k;
      if ((is >> k) && k != key) keep.push_back(line);
    }
  }
  const std::string tmp = std::string(path) + ".tmp";
  {
    std::ofstream o(tmp);
    for (const auto& l : keep) o << l << "\n";
    o << key << " " << t.tile_z << " " << t.blocks_per_sm << " " << t.ccl_blocks_per_sm << " "
      << t.flood_blocks_per_sm << " " << ms << "\n";
  }
  std::rename(tmp.c_str(), path);
}

// Coordinate descent over the launch-shape knobs, starting from the current shape.
Status autotune(pnm_batch& b, const char* cache, int reps, int flags, double* ms_out) {
  if (b.lay.n_total == 0) return Status::ok();
  const std::string key = size_class(b);
  pnm_tuning best = b.tuning;
  if (!(flags & PNM_TUNE_FORCE) && cache_lookup(cache, key, &best)) {
    PNM_TRY(apply_tuning(b, best));
    if (ms_out) *ms_out = 0.0;
    return Status::ok();
  }
  // one complete run first: it grows data-dependent capacities if this data needs it
  const bool g = b.use_graph;
  b.use_graph = false;
  Status st = launch(b);
  if (st.good()) st = wait_checked(b);
  b.use_graph = g;
  PNM_TRY(st);
  double best_ms = 0.0;
  PNM_TRY(time_runs(b, reps, &best_ms));
  const std::vector<int> tz = {4, 8, 16}, grid = {4, 8, 16}, ccl = {4, 8, 16, 32},
                         flood = {1, 2, 4};
  for (int knob = 0; knob < 4; ++knob) {
    const std::vector<int>& vals = knob == 0 ? tz : knob == 1 ? ccl : knob == 2 ? grid : flood;
    for (int v : vals) {
      pnm_tuning c = best;
      int* field = knob == 0 ? &c.tile_z
                   : knob == 1 ? &c.ccl_blocks_per_sm
                   : knob == 2 ? &c.blocks_per_sm
                               : &c.flood_blocks_per_sm;
      if (*field == v) continue;
      *field = v;
      PNM_TRY(apply_tuning(b, c));
      double ms = 0.0;
      PNM_TRY(time_runs(b, reps, &ms));
      if (ms < best_ms) {
        best_ms = ms;
        best = c;
      }
    }
  }
  PNM_TRY(apply_tuning(b, best));
  cache_store(cache, key, best, best_ms);
  if (ms_out) *ms_out = best_ms;
  return Status::ok();
}

int fail(pnm_batch* b, Status s) {
  if (!s.good() && b) b->last_error = s.msg;
  return s.code;
}

}  // namespace

namespace pnm {

// Keeps freed batch memory in the device's default pool (stream-ordered allocations are then
// served from it), once per process and device.
void keep_pool(int device) {
  static bool done[64] = {};
  if (device < 0 || device >= 64 || done[device]) return;
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
    unsigned long long thr = ~0ull;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
  }
  cudaGetLastError();
  done[device] = true;
}

Status batch_new(int device, int sm_count, cudaStream_t stream, void* pinned, int flags, int nvol,
                 const int32_t* dims_xyz, const float* origin_xyz, const float* spacing_xyz,
                 pnm_batch** out) {
  *out = nullptr;
  auto* b = new (std::nothrow) pnm_batch();
  if (!b) return Status{PNM_ERR_INTERNAL, "out of host memory"};
  auto body = [&]() -> Status {
    b->device = device;
    b->sm_count = sm_count;
    b->use_graph = !(flags & PNM_BATCH_NO_GRAPH);
    PNM_TRY(make_layout(nvol, dims_xyz, origin_xyz, spacing_xyz, 0, 0, &b->lay));
    PNM_CUDA(cudaSetDevice(device));
    keep_pool(device);
    if (stream) {
      b->stream = stream;
      b->own_stream = false;
    } else {
      PNM_CUDA(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
    }
    PNM_CUDA(cudaMallocAsync(&b->arena, b->lay.arena, b->stream));
    PNM_CUDA(cudaMallocAsync(&b->pairbuf, b->lay.pairbuf, b->stream));
    PNM_CUDA(cudaMallocAsync(&b->porebuf, b->lay.porebuf, b->stream));
    const size_t pin_bytes = 256 + nvol * sizeof(VolResult);
    if (pinned) {
      b->pinned = pinned;
      b->own_pinned = false;
    } else {
      PNM_CUDA(cudaMallocHost(&b->pinned, pin_bytes));
    }
    std::memset(b->pinned, 0, pin_bytes);
    PNM_TRY(carve(*b));
    PNM_CUDA(cudaMemcpyAsync(const_cast<VolDesc*>(b->plan.vols), b->lay.vols.data(),
                             nvol * sizeof(VolDesc), cudaMemcpyHostToDevice, b->stream));
    PNM_CUDA(cudaMemsetAsync(b->plan.res, 0, nvol * sizeof(VolResult), b->stream));
    return Status::ok();
  };
  Status s = body();
  if (!s.good()) {
    cudaGetLastError();
    pnm_batch_destroy(b);
    return s;
  }
  *out = b;
  return Status::ok();
}

size_t batch_pinned_bytes(int nvol) { return 256 + (size_t)nvol * sizeof(VolResult); }

Status batch_rebind(pnm_batch* b, cudaStream_t stream, const float* origin_xyz,
                    const float* spacing_xyz, bool use_graph) {
  if (b->pending) return Status{PNM_ERR_ARG, "a run is in flight"};
  if (stream && !b->own_stream) b->stream = stream;
  for (size_t i = 0; i < b->lay.vols.size(); ++i) {
    VolDesc& v = b->lay.vols[i];
    const float* o = origin_xyz + 3 * i;
    const float* sp = spacing_xyz + 3 * i;
    for (int a = 0; a < 3; ++a)
      if (!(sp[a] > 0.0f) || !std::isfinite(sp[a]))
        return Status{PNM_ERR_ARG, "spacing must be finite and positive"};
    v.ox = o[0];
    v.oy = o[1];
    v.oz = o[2];
    v.sx = sp[0];
    v.sy = sp[1];
    v.sz = sp[2];
    v.thr = -1.5f * std::min(sp[0], std::min(sp[1], sp[2]));  // pore_extraction.hpp:163-164
  }
  PNM_CUDA(cudaSetDevice(b->device));
  PNM_CUDA(cudaMemcpyAsync(const_cast<VolDesc*>(b->plan.vols), b->lay.vols.data(),
                           b->lay.vols.size() * sizeof(VolDesc), cudaMemcpyHostToDevice,
                           b->stream));
  if (use_graph && !b->use_graph && b->graph_note.empty())
    b->use_graph = true;  // captured on the next launch (unless a capture already failed)
  return Status::ok();
}

}  // namespace pnm

extern "C" {

int pnm_batch_plan_bytes(int32_t n_volumes, const int32_t* dims_xyz, int64_t* bytes) {
  if (!bytes) return PNM_ERR_ARG;
  Layout L;
  Status s = pnm::make_layout(n_volumes, dims_xyz, nullptr, nullptr, 0, 0, &L);
  if (!s.good()) return s.code;
  *bytes = (int64_t)(L.arena + L.pairbuf + L.porebuf);
  return PNM_OK;
}

int pnm_batch_create(pnm_ctx* ctx, int32_t n_volumes, const int32_t* dims_xyz,
                     const float* origin_xyz, const float* spacing_xyz, int32_t flags,
                     pnm_batch** out) {
  if (!ctx || !out || !origin_xyz || !spacing_xyz) return PNM_ERR_ARG;
  *out = nullptr;
  Status s = pnm::batch_new(ctx->c.device, ctx->c.sm_count, nullptr, nullptr, flags, n_volumes,
                            dims_xyz, origin_xyz, spacing_xyz, out);
  if (!s.good()) ctx->c.last_error = s.msg;
  return s.code;
}

void pnm_batch_destroy(pnm_batch* b) {
  if (!b) return;
  cudaSetDevice(b->device);
  // pending copies into host mirrors this batch owns; a borrowed stream may already carry other
  // work, and the stream-ordered frees below need no wait
  if (b->stream && (b->own_pinned || b->own_stream)) cudaStreamSynchronize(b->stream);
  drop_graph(*b);
  // stream-ordered frees: no device-wide synchronisation, memory goes back to the pool
  if (b->arena) cudaFreeAsync(b->arena, b->stream);
  if (b->pairbuf) cudaFreeAsync(b->pairbuf, b->stream);
  if (b->porebuf) cudaFreeAsync(b->porebuf, b->stream);
  if (b->pinned && b->own_pinned) cudaFreeHost(b->pinned);
  if (b->stream && b->own_stream) cudaStreamDestroy(b->stream);
  delete b;
}

const char* pnm_batch_last_error(const pnm_batch* b) { return b ? b->last_error.c_str() : ""; }

void* pnm_batch_stream(const pnm_batch* b) { return b ? (void*)b->stream : nullptr; }

int pnm_batch_set_sdf(pnm_batch* b, int32_t i, const float* sdf) {
  if (!b || !sdf || i < 0 || i >= (int32_t)b->lay.vols.size()) return PNM_ERR_ARG;
  const pnm::VolDesc& v = b->lay.vols[i];
  const long long n = (long long)v.nx * v.ny * v.nz;
  if (n == 0) return PNM_OK;
  auto body = [&]() -> Status {
    PNM_CUDA(cudaSetDevice(b->device));
    PNM_CUDA(cudaMemcpyAsync(const_cast<float*>(b->plan.sdf) + v.off, sdf, n * sizeof(float),
                             cudaMemcpyDefault, b->stream));  // host or device source
    return Status::ok();
  };
  return fail(b, body());
}

int pnm_batch_sdf_dev(pnm_batch* b, float** d_sdf, int64_t* n) {
  if (!b || !d_sdf || !n) return PNM_ERR_ARG;
  *d_sdf = const_cast<float*>(b->plan.sdf);
  *n = b->lay.n_total;
  return PNM_OK;
}

int pnm_batch_launch(pnm_batch* b) {
  if (!b) return PNM_ERR_ARG;
  if (b->pending) return fail(b, Status{PNM_ERR_ARG, "a run is already in flight"});
  return fail(b, launch(*b));
}

int pnm_batch_wait(pnm_batch* b) {
  if (!b) return PNM_ERR_ARG;
  return fail(b, wait_checked(*b));
}

int pnm_batch_run(pnm_batch* b) {
  if (!b) return PNM_ERR_ARG;
  int rc = pnm_batch_launch(b);
  if (rc != PNM_OK) return rc;
  return pnm_batch_wait(b);
}

int pnm_batch_volume_info(const pnm_batch* b, int32_t i, pnm_batch_volume* out) {
  if (!b || !out || i < 0 || i >= (int32_t)b->lay.vols.size()) return PNM_ERR_ARG;
  if (!b->have_result && b->lay.n_total > 0) return PNM_ERR_ARG;
  const pnm::VolDesc& v = b->lay.vols[i];
  std::memset(out, 0, sizeof(*out));
  out->voxel_offset = v.off;
  out->nx = v.nx;
  out->ny = v.ny;
  out->nz = v.nz;
  if (b->lay.n_total == 0) return PNM_OK;
  const pnm::VolResult& r = b->plan.h_res[i];
  out->n_pore_labels = (int32_t)r.n_pore_labels;
  out->n_solid_labels = (int32_t)r.n_solid_labels;
  out->pore_offset = r.peak0;
  out->n_pores = std::min<int64_t>(r.n_peaks, pnm::kMaxPoresPerVolume);
  out->pair_offset = r.pair0;
  out->n_pairs = r.n_pairs;
  return PNM_OK;
}

int pnm_batch_results_dev(const pnm_batch* b, pnm_pore** d_pores, int32_t** d_seg,
                          int32_t** d_pairs) {
  if (!b) return PNM_ERR_ARG;
  if (d_pores) *d_pores = b->plan.pores;
  if (d_seg) *d_seg = b->plan.seg;
  if (d_pairs) *d_pairs = b->plan.pairs;
  return PNM_OK;
}

int pnm_batch_copy_out(pnm_batch* b, int32_t i, pnm_pore* pores, int32_t* seg, int32_t* pairs) {
  if (!b) return PNM_ERR_ARG;
  pnm_batch_volume info;
  int rc = pnm_batch_volume_info(b, i, &info);
  if (rc != PNM_OK) return rc;
  auto body = [&]() -> Status {
    PNM_CUDA(cudaSetDevice(b->device));
    const long long n = (long long)info.nx * info.ny * info.nz;
    if (pores && info.n_pores)
      PNM_CUDA(cudaMemcpyAsync(pores, b->plan.pores + info.pore_offset,
                               info.n_pores * sizeof(pnm_pore), cudaMemcpyDeviceToHost,
                               b->stream));
    if (seg && n)
      PNM_CUDA(cudaMemcpyAsync(seg, b->plan.seg + info.voxel_offset, n * sizeof(int32_t),
                               cudaMemcpyDeviceToHost, b->stream));
    if (pairs && info.n_pairs)
      PNM_CUDA(cudaMemcpyAsync(pairs, b->plan.pairs + 2 * info.pair_offset,
                               2 * info.n_pairs * sizeof(int32_t), cudaMemcpyDeviceToHost,
                               b->stream));
    PNM_CUDA(cudaStreamSynchronize(b->stream));
    return Status::ok();
  };
  return fail(b, body());
}

int pnm_batch_get_stats(const pnm_batch* b, pnm_stats* out) {
  if (!b || !out) return PNM_ERR_ARG;
  std::memset(out, 0, sizeof(*out));
  out->launches = b->launches_per_run;
  out->calls = b->runs;
  out->voxels = 0;
  for (const auto& v : b->lay.vols) out->voxels += (int64_t)v.nx * v.ny * v.nz;
  out->workspace_bytes = (int64_t)(b->lay.arena + b->lay.pairbuf + b->lay.porebuf);
  if (b->have_result && b->lay.n_total > 0) {
    const unsigned* h = b->plan.h_cnt;
    out->ccl_edges = h[pnm::CNT_EDGES];
    out->flood_sweeps = (int32_t)h[pnm::CNT_SWEEPS];
    out->n_pores = h[pnm::CNT_PEAKS];
    out->n_pairs = h[pnm::CNT_PAIRS];
    int64_t np = 0, ns = 0;
    for (size_t i = 0; i < b->lay.vols.size(); ++i) {
      np += b->plan.h_res[i].n_pore_labels;
      ns += b->plan.h_res[i].n_solid_labels;
    }
    out->n_pore_labels = (int32_t)std::min<int64_t>(np, INT_MAX);
    out->n_solid_labels = (int32_t)std::min<int64_t>(ns, INT_MAX);
  }
  return PNM_OK;
}

int pnm_batch_uses_graph(const pnm_batch* b) { return b && b->exec ? 1 : 0; }

int pnm_batch_set_tuning(pnm_batch* b, const pnm_tuning* t) {
  if (!b || !t) return PNM_ERR_ARG;
  if (b->pending) return fail(b, Status{PNM_ERR_ARG, "a run is in flight"});
  return fail(b, apply_tuning(*b, *t));
}

int pnm_batch_get_tuning(const pnm_batch* b, pnm_tuning* t) {
  if (!b || !t) return PNM_ERR_ARG;
  *t = b->tuning;
  return PNM_OK;
}

int pnm_batch_autotune(pnm_batch* b, const char* cache_path, int32_t reps, int32_t flags,
                       double* ms_out) {
  if (!b) return PNM_ERR_ARG;
  if (b->pending) return fail(b, Status{PNM_ERR_ARG, "a run is in flight"});
  return fail(b, autotune(*b, cache_path, std::max(1, (int)reps), flags, ms_out));
}

}  // extern "C"
