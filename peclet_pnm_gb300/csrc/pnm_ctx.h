// Host-side internals shared by the translation units of libpnm_gb300.so: the context, its
// grow-only device workspace, the device counter block, and the stage entry points that the C
// ABI (pnm_capi.cu) sequences.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <functional>
#include <string>
#include <vector>

#include "pnm_gb300.h"

namespace pnm {

// ---- status plumbing ---------------------------------------------------------------------------
struct Status {
  int code = PNM_OK;
  std::string msg;
  static Status ok() { return {}; }
  bool good() const { return code == PNM_OK; }
};
#define PNM_TRY(expr)            \
  do {                           \
    ::pnm::Status _s = (expr);   \
    if (!_s.good()) return _s;   \
  } while (0)
Status cuda_status(cudaError_t e, const char* what);
#define PNM_CUDA(call)                                              \
  do {                                                              \
    cudaError_t _e = (call);                                        \
    if (_e != cudaSuccess) return ::pnm::cuda_status(_e, #call);    \
  } while (0)

// ---- device error flags (set by kernels instead of trapping; read back by the host) -------------
enum ErrFlag : unsigned {
  ERRF_UF_LIMIT = 1u,       // a union-find find/unite exceeded its iteration limit
  ERRF_HASH_FULL = 2u,      // the pair hash set ran out of probes
  ERRF_FLOOD_LIMIT = 4u,    // the flood wavefront exceeded its sweep limit
  ERRF_FACE_LIMIT = 8u,     // a face-CCL find/unite exceeded its iteration limit
  ERRF_BARRIER = 16u,       // a grid barrier of a persistent kernel timed out
  ERRF_LABEL_RANGE = 32u,   // renumbering met a key or label minimum outside the volume
};

// ---- counter block (device ints; one copy per context) ------------------------------------------
enum Counter : int {
  CNT_ERR = 0,
  CNT_KEYS,          // distinct basin / solid keys seen (keylist length)
  CNT_FRONT0,        // flood frontier length, ping
  CNT_FRONT1,        // flood frontier length, pong
  CNT_ULIST,         // flood voxels without a marker neighbour (list U)
  CNT_EDGES,         // marker-CCL links united (run pairs that touch)
  CNT_PEAKS,         // batch: extract_pores peaks over all volumes
  CNT_PAIRS,         // distinct label pairs in the hash set
  CNT_SWEEPS,        // flood sweeps run by the persistent flood loop
  CNT_BAR0,          // grid barrier of the persistent flood loop: arrivals
  CNT_BAR1,          //   and generation
  CNT_COUNT = 32
};

// ---- grow-only device workspace ---------------------------------------------------------------
enum Slot : int {
  S_SDF = 0, S_CODE, S_L, S_KEY, S_IDTAB, S_SEG, S_FRONT0, S_FRONT1, S_TMP, S_KEYLIST,
  S_PEAKBITS, S_PEAKPREF, S_FIRSTP, S_FIRSTS, S_PREFP, S_PREFS, S_SCAN0, S_SCAN1,
  S_HASH, S_KEYS_A, S_KEYS_B, S_VALS_A, S_VALS_B, S_RSHIST, S_PORES, S_PAIRS, S_SEGIN,
  // network flow
  S_U, S_V, S_W, S_P, S_OX, S_OY, S_OZ, S_FLOWLAB, S_FBITS, S_FCORE, S_FPREF, S_FID, S_FPAIR,
  S_FPAR, S_FFILM, S_FMINCORE, S_FLABEL, S_ROOTFLAG, S_SLOTOF, S_PEAK, S_NPORES_OUT,
  S_PPRES, S_REC, S_ACC, S_TDP, S_THROATS, S_MAXBITS, S_FLOWOUT, S_ULIST, S_EDGES, S_NXT, S_STEPS,
  S_COORD, S_SCAN2, S_HASHKEYS,
  // post-processing
  S_POST, S_POSTCOORD,
  S_COUNT
};

struct Workspace {
  std::vector<void*> ptr = std::vector<void*>(S_COUNT, nullptr);
  std::vector<size_t> cap = std::vector<size_t>(S_COUNT, 0);
  // Returns a device buffer of at least `bytes` for `slot` (grow-only; contents undefined).
  Status get(int slot, size_t bytes, void** out);
  void release();
  size_t total_bytes() const;
};

struct Ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t own_stream = nullptr;
  cudaStream_t copy_stream = nullptr;  // host transfers overlapped with the pipeline
  std::vector<cudaEvent_t> events;     // slab events of those transfers
  Workspace ws;
  unsigned* d_cnt = nullptr;  // CNT_COUNT device counters
  unsigned* h_cnt = nullptr;      // pinned, mapped host mirror
  unsigned* h_cnt_dev = nullptr;  // its device address
  int sm_count = 0;
  long long launches = 0;   // kernels launched by this context (cumulative)
  long long calls = 0;      // entry-point calls (cumulative)
  pnm_stats last{};         // per-call statistics of the last call
  // bounded device waits (pnm_ctx_set_wait_limit): grid-barrier limit in ns of GPU global time,
  // and arrivals beyond the grid that a barrier waits for (0; > 0 only to test the error path)
  unsigned long long wait_ns = 1000000000ull;
  unsigned wait_extra = 0;
  // stages (PNM_STAGE_*): an NVTX range each, and with timing on a pair of CUDA events on the
  // stream around each, summed per stage into last.stage_ms when the call ends
  // Stages nest (network flow runs a seg-only pass inside its own stage): an inner stage pauses
  // the outer one, so the recorded intervals partition the call's device time.
  bool timing = false;
  std::vector<cudaEvent_t> tev;  // event pool, two per recorded stage interval
  std::vector<int> tstage;       // stage id of each recorded interval
  std::vector<int> open_stages;  // stack of open stage ids
  int nvtx_depth = 0;
  void interval_begin(int id);
  void interval_end();
  void call_begin();                           // clears the last call's stage times
  void stage_begin(int id, const char* name);  // NVTX push (+ start event)
  void stage_end();                            // (end event +) NVTX pop
  void stage_collect();                        // waits for the events, fills last.stage_ms
  // Side stream: work that depends on the SDF pass alone (the pore records) runs there while the
  // main stream runs the marker CCL and the resolve; the main stream joins it before the flood
  // (whose cooperative launch wants the whole GPU). Its stage interval is timed on its own.
  cudaStream_t side_stream = nullptr;
  cudaEvent_t side_fork = nullptr, side_join = nullptr, side_t0 = nullptr, side_t1 = nullptr;
  bool side_pending = false;  // work enqueued there that the main stream has not joined yet
  bool side_timed = false;    // side_t0/side_t1 hold this call's side interval
  int side_stage = 0;
  unsigned* h_side = nullptr;  // pinned: a count the side stream copied back
  Status ensure_side();
  Status join_side();
  std::string last_error;
  Status fail(Status s) {
    last_error = s.msg;
    return s;
  }
  template <class T>
  Status buf(int slot, size_t count, T** out) {
    void* p = nullptr;
    Status s = ws.get(slot, count * sizeof(T) + 16, &p);
    *out = static_cast<T*>(p);
    return s;
  }
  Status read_counters();  // copies d_cnt -> h_cnt on the stream and synchronises it
  Status ensure_copy_events(int n);  // creates the copy stream and at least n events
};

// One stage of a call for the lifetime of the scope (early returns included); next() ends it
// and opens the following stage in the same scope.
struct StageScope {
  Ctx& c;
  StageScope(Ctx& ctx, int id, const char* name) : c(ctx) { c.stage_begin(id, name); }
  void next(int id, const char* name) {
    c.stage_end();
    c.stage_begin(id, name);
  }
  ~StageScope() { c.stage_end(); }
  StageScope(const StageScope&) = delete;
  StageScope& operator=(const StageScope&) = delete;
};

// Host buffers of a host-pointer call. With them the stages overlap the transfers with the
// pipeline: the SDF is uploaded in z-slabs on ctx.copy_stream while the SDF pass runs slab by
// slab behind it, and the labels go back slab by slab as the seg / topology pass writes them.
struct HostXfer {
  const float* h_sdf = nullptr;  // host SDF, uploaded into the stage's device SDF
  int32_t* h_seg = nullptr;      // host labels (filled from the device labels)
  bool seg_sent = false;         // set once the label copies are enqueued
  // further host -> device copies, queued behind the SDF slabs (they run during the pipeline);
  // extra_done is recorded on the copy stream after them
  struct Copy {
    void* dst;
    const void* src;
    size_t bytes;
  };
  std::vector<Copy> extra;
  cudaEvent_t extra_done = nullptr;
  cudaEvent_t extra_early = nullptr;  // after every extra copy but the last (two or more)
};
// z-planes per transfer slab (a multiple of 16, the tile and brick depth) for nz planes
int xfer_slab_planes(int nz);

#ifdef __CUDACC__
#define PNM_HD __host__ __device__
#else
#define PNM_HD
#endif
struct Dims {
  int nx, ny, nz;
  PNM_HD long long n() const { return (long long)nx * ny * nz; }
};

// Validates dims (positive, n < 2^31 - 3) and spacing (finite, > 0).
Status check_dims(Dims d, const float* spacing, bool need_spacing);

// ---- stages (pnm_segment.cu) -------------------------------------------------------------------
// Everything below runs on ctx.stream over a device SDF; results stay in the workspace.

struct SegState {
  Dims d;
  const float* sdf = nullptr;
  uint8_t* code = nullptr;      // per voxel: ascent direction (5 bits), class (2), flood-seed (1)
  int32_t* nxt = nullptr;       // per voxel: ascent pointer (voxel id; itself at a local max)
  int32_t* key = nullptr;       // per voxel: basin root (>=0), ~solid label (<0), INT_MIN none
  int32_t* idtab = nullptr;     // per key voxel: final signed label id
  uint32_t* peakbits = nullptr; // bitmap of extract_pores peaks
  uint32_t* mbits = nullptr;    // marker bitmap, one word per 32-voxel row chunk
  long long n_words = 0;
  bool ccl_done = false;        // the marker links were made during the SDF pass (host upload)
  unsigned n_edges = 0;         // marker-CCL links united
  int n_pore_labels = 0;        // np
  int n_solid_labels = 0;
  int flood_sweeps = 0;
};

// Fused SDF pass + CCL + flood + gradient roots + first-appearance renumbering. all_ascent:
// also compute the ascent pointer of non-pore voxels (network flow's basins need every cell).
// after_sdf (optional) runs once the SDF pass is enqueued: it may fork work onto the side
// stream, which is joined before the flood.
Status run_segmentation(Ctx& c, const float* d_sdf, Dims d, const float spacing[3], SegState* st,
                        bool all_ascent = false, HostXfer* xfer = nullptr,
                        const std::function<Status()>* after_sdf = nullptr);
// Writes seg (if d_seg != null) and the unique sorted label pairs (if want_pairs) from the state.
Status run_seg_and_topology(Ctx& c, const SegState& st, int32_t* d_seg, bool want_pairs,
                            int32_t** d_pairs_out, int64_t* n_pairs, HostXfer* xfer = nullptr);
// Topology of a caller-provided device seg.
Status run_topology_of_seg(Ctx& c, const int32_t* d_seg, Dims d, int32_t** d_pairs_out,
                           int64_t* n_pairs);
// Compacts the peak bitmap into pores (voxel order, centroid-refined) in d_out (cap entries).
Status run_pores(Ctx& c, const SegState& st, const float origin[3], const float spacing[3],
                 pnm_pore* d_out, int64_t cap, int64_t* n_pores);
// run_pores on the side stream, forked from the main stream after the SDF pass; the count
// is read with side_pores_count once the side stream is joined.
Status run_pores_side(Ctx& c, const SegState& st, const float origin[3], const float spacing[3],
                      pnm_pore* d_out, int64_t cap);
Status side_pores_count(Ctx& c, int64_t* n_pores);
// Pore records from a peak bitmap and its exclusive word prefix counts (voxel order, <= cap).
void launch_pores_emit(const float* sdf, Dims d, const uint32_t* bits, const unsigned* pref,
                       long long words, const float origin[3], const float spacing[3],
                       pnm_pore* out, long long cap, unsigned grid, cudaStream_t s);
// Peak voxel ids of the pore records (voxel order, <= cap written; the count in *n_peaks).
Status run_peak_ids(Ctx& c, const SegState& st, int32_t* d_out, int64_t cap, int64_t* n_peaks);
// SDF pass only (for extract_pores alone).
// ccl_in_slabs: with a host upload, make the marker links slab by slab behind the SDF pass.
Status run_sdf_pass(Ctx& c, const float* d_sdf, Dims d, const float spacing[3], SegState* st,
                    bool all_ascent = false, HostXfer* xfer = nullptr, bool ccl_in_slabs = false);

// ---- network flow (pnm_flow.cu) ------------------------------------------------------------
struct FlowInputs {
  const double *u, *v, *w, *p, *ox, *oy, *oz;  // device pointers; o* may be null
  double grad_p[3];
  // host uploads still in flight (null: resident): the velocities and openness, and p
  cudaEvent_t fields_ready = nullptr, p_ready = nullptr;
};
struct FlowOutputsHost {
  std::vector<pnm_pore> pores;
  std::vector<double> pore_pressure, pore_residual, throat_flow, throat_area, throat_dp;
  std::vector<int32_t> throats;
};
// Device-resident results of run_network_flow: context slots, valid until the context's next
// call; complete once the context's stream reaches the point where run_network_flow returned.
struct FlowOutputsDev {
  long long np = 0, nt = 0;
  pnm_pore* pores = nullptr;
  double *pore_pressure = nullptr, *pore_residual = nullptr;
  int32_t* throats = nullptr;
  double *throat_flow = nullptr, *throat_area = nullptr, *throat_dp = nullptr;
};
Status run_network_flow(Ctx& c, const SegState& st, const float origin[3], const float spacing[3],
                        const FlowInputs& in, FlowOutputsDev* out);
// Copies the results to host vectors (synchronises the context's stream).
Status flow_outputs_to_host(Ctx& c, const FlowOutputsDev& o, FlowOutputsHost* out);

}  // namespace pnm

// ---- batches (pnm_batch.cu) ---------------------------------------------------------------------
namespace pnm {
// Plans and allocates a batch (stream-ordered allocations on `stream`; null: the batch creates
// and owns a stream). `pinned` (optional, batch_pinned_bytes(nvol)) receives the per-run
// figures; null: the batch allocates its own.
Status batch_new(int device, int sm_count, cudaStream_t stream, void* pinned, int flags, int nvol,
                 const int32_t* dims_xyz, const float* origin_xyz, const float* spacing_xyz,
                 pnm_batch** out);
size_t batch_pinned_bytes(int nvol);
// Re-targets an idle batch: the stream its runs go to (batches on a borrowed stream only), the
// origin and spacing of its volumes (same shapes), and graph replay from the next run on.
Status batch_rebind(pnm_batch* b, cudaStream_t stream, const float* origin_xyz,
                    const float* spacing_xyz, bool use_graph);
}  // namespace pnm

// The opaque handle of the C ABI.
struct pnm_ctx {
  pnm::Ctx c;
};
