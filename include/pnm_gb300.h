/* pnm_gb300 — GB300-native (sm_103a) pore-network extraction: the C ABI.
 *
 * Drop-in replacement for the single-rank path of peclet.pnm (reference: src/pore_extraction.hpp
 * and its nanobind binding src/pnm_bindings.cpp). All array arguments are plain pointers:
 *   - volumes are flat x-fastest arrays of nx*ny*nz elements (== zyx C-order (Nz,Ny,Nx));
 *   - origin / spacing are xyz float32 triples (the binding's zyx doubles, reversed and cast);
 *   - grad_p is an xyz float64 triple;
 *   - the SDF is float32 and negative inside the solid.
 * Every function returns a status (PNM_OK = 0); pnm_last_error(ctx) holds the message of the last
 * failure on that context. Functions are thread-safe across distinct contexts; one context must
 * not be used by two threads at once. Host-pointer entry points copy inputs to the device and
 * results back; *_dev entry points take device pointers and leave results on the device.
 *
 * Limits: nx*ny*nz < 2^31 - 3 (voxel ids and labels are int32, as in the reference's get_idx);
 * extract_network_flow additionally needs 3*nx*ny*nz < 2^31 (face ids are compacted to int32).
 */
#ifndef PNM_GB300_H
#define PNM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PNM_OK 0
#define PNM_ERR_ARG 1           /* null pointer, non-positive dims or spacing, partial openness */
#define PNM_ERR_SHAPE 2         /* volume too large for int32 voxel ids / int32 face ids */
#define PNM_ERR_CAPACITY 3      /* a caller-provided device output is too small; the count
                                   argument receives the required size */
#define PNM_ERR_NOT_CONVERGED 4 /* a bounded device fixpoint / wait hit its iteration limit */
#define PNM_ERR_CUDA 5          /* a CUDA runtime call failed */
#define PNM_ERR_NO_DEVICE 6     /* no CUDA device, or the device is not sm_103 */
#define PNM_ERR_INTERNAL 7

/* struct Pore (pore_extraction.hpp:24-26): world position of the refined SDF peak and its value. */
typedef struct {
  float x, y, z, radius;
} pnm_pore;

typedef struct pnm_ctx pnm_ctx;

/* Context: owns the device, a CUDA stream, a grow-only device workspace and the error message.
 * Replaces the reference's global Kokkos::initialize / per-call View allocation
 * (pnm_bindings.cpp:73-84). device < 0 picks the current device. */
int pnm_ctx_create(int device, pnm_ctx** out);
void pnm_ctx_destroy(pnm_ctx* ctx);
const char* pnm_last_error(const pnm_ctx* ctx);
/* Use a caller-owned cudaStream_t (passed as void*) for all work of this context; NULL restores
 * the context's own stream. */
int pnm_ctx_set_stream(pnm_ctx* ctx, void* stream);
/* Releases the workspace (it regrows on the next call). */
int pnm_ctx_trim(pnm_ctx* ctx);
/* Name of the execution space (the reference exposes Kokkos' backend name as
 * `execution_space`, pnm_bindings.cpp:83). */
const char* pnm_execution_space(void);
/* Frees buffers returned by the host entry points. */
void pnm_free(void* p);

/* Stages of a call, named after the reference's kernel labels (src/pore_extraction.hpp:86-884).
 * Every stage is enclosed in an NVTX range of that name (visible to Nsight tools; a no-op
 * otherwise); with timing on, pnm_stats.stage_ms holds each stage's device time in the last call. */
#define PNM_STAGE_SDF_PASS 0      /* "pnm::extract_pores" + "pnm::init_markers": one pass over the
                                     SDF (peaks, classes, ascent directions, marker runs) */
#define PNM_STAGE_MERGE_MARKERS 1 /* "pnm::merge_markers": marker CCL */
#define PNM_STAGE_GRADIENT_PATH 2 /* "pnm::gradient_path": basin roots (and marker roots) */
#define PNM_STAGE_FLOOD 3         /* "pnm::flood": Jacobi sweeps over the shallow solid */
#define PNM_STAGE_RELABEL 4       /* "pnm::relabel_min" .. "pnm::relabel_assign": label ids */
#define PNM_STAGE_SEG_PAIRS 5     /* "pnm::relabel_seg" + "pnm::boundary_pairs" */
#define PNM_STAGE_PAIR_SORT 6     /* unique sorted pairs (the reference sorts on the host) */
#define PNM_STAGE_PORES 7         /* pore records with their centroids; in extract_pore_network
                                     calls they run on a second stream, overlapping
                                     merge_markers and gradient_path (their time is their own
                                     span, not a share of the call's) */
#define PNM_STAGE_NETWORK_FLOW 8  /* "nf::*": network flow after the segmentation */
#define PNM_STAGE_COUNT 9

/* Per-context statistics: cumulative counters and figures of the last call. */
typedef struct {
  int64_t launches;        /* CUDA kernels launched by this context since creation */
  int64_t calls;           /* entry-point calls since creation */
  int64_t voxels;          /* last call: nx*ny*nz */
  int64_t ccl_edges;       /* last call: marker-CCL links united (run pairs that touch) */
  int32_t flood_sweeps;    /* last call: Jacobi flood sweeps run (incl. the empty final one) */
  int32_t n_pore_labels;   /* last call: pore labels (np) */
  int32_t n_solid_labels;  /* last call: solid labels */
  int32_t reserved;
  int64_t n_pores;         /* last call: extract_pores peaks */
  int64_t n_pairs;         /* last call: unique connections */
  int64_t workspace_bytes; /* device workspace currently held */
  double stage_ms[PNM_STAGE_COUNT]; /* last call, timing on: device ms per PNM_STAGE_* (0 off) */
} pnm_stats;
int pnm_ctx_get_stats(const pnm_ctx* ctx, pnm_stats* out);
/* Per-stage device timing (CUDA events on the context's stream around each stage), off by
 * default: on, every call also waits for its last stage before it returns. */
int pnm_ctx_set_timing(pnm_ctx* ctx, int32_t on);

/* Bounded device waits. The persistent flood loop's grid barrier (the fixpoint of
 * pore_extraction.hpp:237-269 in one launch) waits at most limit_ns of GPU time per barrier
 * (default 1e9, 1 s; 1 .. 6e10 accepted); when a wait runs out the kernel returns and the call
 * fails with PNM_ERR_NOT_CONVERGED, and the context stays usable. extra_arrivals > 0 makes every
 * barrier wait for that many arrivals that never come, so its wait runs out: a test of that error
 * path without a device fault. 0 in normal use. */
int pnm_ctx_set_wait_limit(pnm_ctx* ctx, int64_t limit_ns, int32_t extra_arrivals);

/* ---- host-pointer entry points ------------------------------------------------------------ */

/* extract_pores (pore_extraction.hpp:143 extract_pores_k; binding pnm_bindings.cpp:110-121).
 * Pores are the SDF voxels whose (value, wrapped index) is a strict maximum over their 26
 * periodic neighbours, refined by the SDF^2-weighted 27-point centroid. Returned in voxel-index
 * order (the reference's order is an atomic race); at most 1e6, the first in voxel order.
 * *pores is allocated by the library (pnm_free); *n_pores receives the count. */
int pnm_extract_pores(pnm_ctx* ctx, const float* sdf, int32_t nx, int32_t ny, int32_t nz,
                      const float origin_xyz[3], const float spacing_xyz[3], pnm_pore** pores,
                      int64_t* n_pores);

/* segment_volume (pore_extraction.hpp:389 segment_volume_k; pnm_bindings.cpp:123-132).
 * Writes the flat per-voxel labels: pores 1,2,... (gradient-ascent basins), solid -1,-2,...
 * (marker CCL + Jacobi flood), debris 0. seg has nx*ny*nz int32 elements. */
int pnm_segment_volume(pnm_ctx* ctx, const float* sdf, int32_t nx, int32_t ny, int32_t nz,
                       const float spacing_xyz[3], int32_t* seg);

/* extract_topology_gpu (pore_extraction.hpp:454 extract_topology_k; pnm_bindings.cpp:134-140).
 * Unique (min, max) label pairs across the +x/+y/+z periodic faces, sorted lexicographically.
 * *pairs (2 * n_pairs int32, interleaved) is allocated by the library (pnm_free). */
int pnm_extract_topology(pnm_ctx* ctx, const int32_t* seg, int32_t nx, int32_t ny, int32_t nz,
                         int32_t** pairs, int64_t* n_pairs);

/* extract_pore_network (pore_extraction.hpp:1011 extract_pore_network_k;
 * pnm_bindings.cpp:143-157): pores, seg (caller buffer, nx*ny*nz) and pairs in one pass over a
 * device-resident SDF. */
int pnm_extract_pore_network(pnm_ctx* ctx, const float* sdf, int32_t nx, int32_t ny, int32_t nz,
                             const float origin_xyz[3], const float spacing_xyz[3],
                             pnm_pore** pores, int64_t* n_pores, int32_t* seg, int32_t** pairs,
                             int64_t* n_pairs);

/* Result of extract_network_flow (struct NetworkFlow, pore_extraction.hpp:482-491). */
typedef struct {
  int64_t n_pores, n_throats;
  pnm_pore* pores;       /* by label: pores[k] <-> label k+1 */
  double* pore_pressure; /* n_pores */
  double* pore_residual; /* n_pores */
  int32_t* throats;      /* 2 * n_throats, (li < lj) interleaved; a pair may repeat */
  double* throat_flow;   /* n_throats, positive li -> lj */
  double* throat_area;   /* n_throats */
  double* throat_dp;     /* n_throats */
} pnm_flow_result;

/* extract_network_flow (pore_extraction.hpp:493 extract_network_flow_k;
 * pnm_bindings.cpp:162-209). u, v, w, p: float64 MAC fields on the SDF grid (u(i,j,k) on the -x
 * face of cell (i,j,k)); ox, oy, oz: openness, all three or none (NULL = fully open).
 * FP64 sums are accumulated exactly (128-bit fixed point), so results are deterministic.
 * *out is allocated by the library (pnm_flow_result_free). */
int pnm_extract_network_flow(pnm_ctx* ctx, const float* sdf, int32_t nx, int32_t ny, int32_t nz,
                             const float origin_xyz[3], const float spacing_xyz[3],
                             const double* u, const double* v, const double* w, const double* p,
                             const double* ox, const double* oy, const double* oz,
                             const double grad_p_xyz[3], pnm_flow_result** out);
void pnm_flow_result_free(pnm_flow_result* r);

/* ---- device-pointer entry points (resident / serving path) -------------------------------- */

/* extract_pore_network on a device SDF. Outputs are device buffers: d_pores (pore_cap entries),
 * d_seg (nx*ny*nz), d_pairs (2 * pair_cap int32). Counts are returned to the host. If a count
 * exceeds its cap, returns PNM_ERR_CAPACITY with the count set to the required size and the
 * first `cap` entries written. d_seg may be NULL (labels not needed). */
int pnm_extract_pore_network_dev(pnm_ctx* ctx, const float* d_sdf, int32_t nx, int32_t ny,
                                 int32_t nz, const float origin_xyz[3], const float spacing_xyz[3],
                                 pnm_pore* d_pores, int64_t pore_cap, int64_t* n_pores,
                                 int32_t* d_seg, int32_t* d_pairs, int64_t pair_cap,
                                 int64_t* n_pairs);

/* The peak voxel of every pore, in the order of the pore records (voxel order): the voxel the
 * record's SDF^2-weighted centroid is refined around, whose SDF value is the record's radius
 * (pore_extraction.hpp:89-127). The distributed surface assigns each pore to the rank whose
 * block holds this voxel, as the reference's extract_pore_network_mpi keeps the pores whose peak
 * its block owns (pore_extraction_mpi.hpp:208-212, :308-368). At most min(cap, 1e6) ids are
 * written; *n_peaks receives the count (PNM_ERR_CAPACITY when it exceeds cap). */
int pnm_pore_peaks_dev(pnm_ctx* ctx, const float* d_sdf, int32_t nx, int32_t ny, int32_t nz,
                       int32_t* d_voxels, int64_t cap, int64_t* n_peaks);

/* segment_volume on a device SDF into a device seg buffer. */
int pnm_segment_volume_dev(pnm_ctx* ctx, const float* d_sdf, int32_t nx, int32_t ny, int32_t nz,
                           const float spacing_xyz[3], int32_t* d_seg);

/* Result of pnm_extract_network_flow_dev: the fields of pnm_flow_result as device arrays owned
 * by the context. They are valid until the context's next call (or pnm_ctx_trim / destroy) and
 * complete in stream order on the context's stream: work queued on that stream after the call
 * may read them without a synchronisation; copy them out before the next call. */
typedef struct {
  int64_t n_pores, n_throats;
  const pnm_pore* pores;
  const double* pore_pressure;
  const double* pore_residual;
  const int32_t* throats; /* 2 * n_throats */
  const double* throat_flow;
  const double* throat_area;
  const double* throat_dp;
} pnm_flow_result_dev;

/* extract_network_flow on device-resident inputs (SDF and float64 MAC fields, same layout as
 * pnm_extract_network_flow): nothing crosses the host boundary but the counts. */
int pnm_extract_network_flow_dev(pnm_ctx* ctx, const float* d_sdf, int32_t nx, int32_t ny,
                                 int32_t nz, const float origin_xyz[3], const float spacing_xyz[3],
                                 const double* d_u, const double* d_v, const double* d_w,
                                 const double* d_p, const double* d_ox, const double* d_oy,
                                 const double* d_oz, const double grad_p_xyz[3],
                                 pnm_flow_result_dev* out);

/* ---- pore-network post-processing (scripts/demo_network_flow_packing.py:44-67) --------------
 * Throat conductance g = Q / dp (IEEE division: dp = 0 gives +-inf or NaN) and the statistics
 * the reference's demo derives from an extract_network_flow result. Means are over throats,
 * maxima of absolute values propagate NaN (as numpy's max); sums are folded in a fixed order
 * (deterministic on a given device). mass_balance_ok = max|pore_residual| < 1e-6 * max|throat_flow| and every g
 * finite (the demo's PASS test; 1 for an empty network). */
typedef struct {
  int64_t n_pores, n_throats;
  double mean_abs_flow, max_abs_flow, mean_abs_dp, max_abs_residual;
  int64_t n_positive_conductance; /* throats with g > 0 */
  int64_t n_finite_conductance;
  double mean_coordination;       /* 2 * n_throats / n_pores (repeated pairs count) */
  int32_t max_coordination;
  int32_t mass_balance_ok;
} pnm_flow_stats;

/* Statistics of device-resident flow results (any device arrays in the pnm_flow_result_dev
 * layout, e.g. straight from pnm_extract_network_flow_dev; throats 8-byte aligned). Optional
 * outputs: d_conductance (n_throats doubles) and d_coordination (n_pores int32, throats per pore
 * label). Runs on the context's stream and returns when the statistics are on the host. */
int pnm_flow_stats_dev(pnm_ctx* ctx, const pnm_flow_result_dev* r, double* d_conductance,
                       int32_t* d_coordination, pnm_flow_stats* out);

/* ---- allocation-free entry point -------------------------------------------------------------
 * No counterpart in the reference. extract_pores on a device SDF for callers that cannot let a
 * library allocate device memory: frameworks that hand out every byte of device memory from
 * their own pool under a fixed budget, and serving loops that must not enter the driver's
 * allocator (cudaMalloc / cudaFree can synchronise the device) while other work is in flight.
 * The caller passes the device SDF, a device output array of pore_cap pores and a stream
 * (cudaStream_t as void*, NULL = default stream); results match pnm_extract_pores. The only
 * scratch is a static device array of the library (about 16 MiB, held on every device that
 * loads the library until the process exits), so volumes above 2^26 voxels (67,108,864, e.g.
 * 406^3) are rejected with PNM_ERR_SHAPE. All calls on a device share that array: calls whose
 * work overlaps on the GPU race and must be serialised. The first call on each device looks up
 * the array's address; under CUDA's lazy module loading (the default since CUDA 12.2) that first
 * call is also when the driver loads the library's kernels on the device and reserves the array,
 * which allocates and may synchronise. So make the first call at start-up, before the caller's
 * pool claims the device's memory and before any stream capture (or run with
 * CUDA_MODULE_LOADING=EAGER). Returns PNM_ERR_CAPACITY (with *n_pores = the count found, and
 * only the first pore_cap records written) when pore_cap is too small. No context is used. */
int pnm_extract_pores_noalloc(const float* d_sdf, int32_t nx, int32_t ny, int32_t nz,
                              const float origin_xyz[3], const float spacing_xyz[3],
                              pnm_pore* d_pores, int64_t pore_cap, int64_t* n_pores,
                              void* stream);

/* ---- batched extraction ------------------------------------------------------------------
 * No counterpart in the reference: its bindings (src/pnm_bindings.cpp:143-160) take one volume
 * per call, so a caller with many volumes loops over extract_pore_network_k
 * (src/pore_extraction.hpp:1011-1025). A batch is planned once for a fixed list of periodic
 * volumes of any shapes; every device buffer is allocated at creation. Each run extracts all
 * volumes with one launch per stage over a ragged volume table (per-volume wrap, per-volume
 * label numbering), with the flood fixpoint in one persistent kernel and no host round trip
 * inside the run; after the first run the whole run is replayed from a CUDA graph. The labels,
 * pores and pairs of every volume are bit-identical to pnm_extract_pore_network on that volume
 * alone. A batch owns its stream; calls on one batch must not overlap. */
typedef struct pnm_batch pnm_batch;

typedef struct {
  int64_t voxel_offset;   /* first voxel of the volume in the batch SDF / label buffers */
  int32_t nx, ny, nz;
  int32_t n_pore_labels, n_solid_labels;
  int32_t reserved;
  int64_t pore_offset;    /* first pore record of the volume in the batch pore buffer */
  int64_t n_pores;        /* pores of the volume (at most 1e6, the reference's max_pores) */
  int64_t pair_offset;    /* first (label_a, label_b) pair of the volume in the pair buffer */
  int64_t n_pairs;
} pnm_batch_volume;

#define PNM_BATCH_NO_GRAPH 1 /* enqueue the stages on every run instead of replaying a graph */

/* Device bytes a batch of these shapes allocates at creation (before any capacity growth). */
int pnm_batch_plan_bytes(int32_t n_volumes, const int32_t* dims_xyz, int64_t* bytes);
/* dims_xyz: 3 per volume (nx, ny, nz); origin_xyz / spacing_xyz: 3 per volume. */
int pnm_batch_create(pnm_ctx* ctx, int32_t n_volumes, const int32_t* dims_xyz,
                     const float* origin_xyz, const float* spacing_xyz, int32_t flags,
                     pnm_batch** out);
void pnm_batch_destroy(pnm_batch* b);
const char* pnm_batch_last_error(const pnm_batch* b);
/* The batch's CUDA stream (cudaStream_t); every batch call is ordered on it. */
void* pnm_batch_stream(const pnm_batch* b);
/* Copies volume i's SDF (float32, x fastest) into the batch, from host or device memory (async
   on the batch stream; a device source must stay valid until the copy has run). */
int pnm_batch_set_sdf(pnm_batch* b, int32_t i, const float* sdf);
/* The batch SDF buffer on the device (volume i at voxel_offset) and its length in floats. */
int pnm_batch_sdf_dev(pnm_batch* b, float** d_sdf, int64_t* n);
/* Enqueues one run (async); pnm_batch_wait completes it (and re-runs once if a capacity grew). */
int pnm_batch_launch(pnm_batch* b);
int pnm_batch_wait(pnm_batch* b);
int pnm_batch_run(pnm_batch* b); /* launch + wait */
/* Results of the last completed run. */
int pnm_batch_volume_info(const pnm_batch* b, int32_t i, pnm_batch_volume* out);
/* Device buffers of the last run: pore records, labels (voxel_offset-based), pairs (2 ints each). */
int pnm_batch_results_dev(const pnm_batch* b, pnm_pore** d_pores, int32_t** d_seg,
                          int32_t** d_pairs);
/* Copies volume i's results to host buffers sized from pnm_batch_volume_info (any may be null). */
int pnm_batch_copy_out(pnm_batch* b, int32_t i, pnm_pore* pores, int32_t* seg, int32_t* pairs);
/* launches: kernels of one run; calls: runs so far; voxels: batch voxels; workspace_bytes. */
int pnm_batch_get_stats(const pnm_batch* b, pnm_stats* out);
/* 1 if runs replay a CUDA graph, 0 if they enqueue the stages (flag, or capture unavailable). */
int pnm_batch_uses_graph(const pnm_batch* b);

/* Launch shape of a batch's stages. Results never depend on it; the fastest shape depends on
   the volume sizes, so pnm_batch_autotune picks it per size class. */
typedef struct {
  int32_t tile_z;              /* SDF-pass and flood-seed tile depth: 4, 8 or 16 (default 16) */
  int32_t blocks_per_sm;       /* grid-stride stages: blocks of 256 threads per SM, 1..32 (16) */
  int32_t ccl_blocks_per_sm;   /* CCL edge-union stage: blocks per SM, 1..64 (8) */
  int32_t flood_blocks_per_sm; /* persistent flood loop: resident blocks per SM, 1..4 (4) */
} pnm_tuning;
#define PNM_TUNE_FORCE 1 /* time the candidates even when the cache holds the size class */
int pnm_batch_set_tuning(pnm_batch* b, const pnm_tuning* t);
int pnm_batch_get_tuning(const pnm_batch* b, pnm_tuning* t);
/* Times candidate shapes on the batch's current SDFs (coordinate descent over the four knobs;
   each candidate: one untimed and `reps` timed runs, median kept), applies the fastest and
   records it for the (device, typical edge, volume count) class in cache_path (a text file;
   null: no cache). A cached class is applied without timing. ms_out (optional): best run time. */
int pnm_batch_autotune(pnm_batch* b, const char* cache_path, int32_t reps, int32_t flags,
                       double* ms_out);

/* ---- serving ----------------------------------------------------------------------------
 * No counterpart in the reference (its calls are serial and blocking, src/pnm_bindings.cpp:143).
 * A request loop over batches: every request (one periodic volume) is queued on submit and
 * admitted while the device-memory budget allows; requests queued when a stream slot frees are
 * coalesced into one batch (continuous batching: arrivals during a run join the next batch), up
 * to max_inflight batches run concurrently on their own streams, and each request's labels,
 * pores and pairs stay resident on the device until it is released. The SDF passed to submit
 * (host or device memory) must stay valid until the request is done or cancelled. */
typedef struct pnm_server pnm_server;

typedef struct {
  int64_t budget_bytes;      /* device bytes for running batches and held results; 0: 120 GB */
  int32_t max_inflight;      /* batches running at once, one stream each; 0: 3 */
  int32_t max_batch_volumes; /* requests per batch; 0: 64 */
  int64_t max_batch_voxels;  /* voxels per batch (a larger request runs alone); 0: 2^28 */
  int32_t reserved[4];
} pnm_server_config;

typedef struct {
  int64_t submitted, completed, failed, cancelled;
  int64_t queued, running;   /* now */
  int64_t batches;           /* batches launched */
  int64_t bytes_in_use;      /* now: running batches + held results */
  int64_t peak_bytes;
  int64_t voxels_completed;
  double p50_ms, p99_ms, mean_ms, max_ms; /* submit -> results resident, completed requests */
  double busy_s;             /* first submit -> last completion */
  double gvoxel_per_s;       /* voxels_completed / busy_s / 1e9 */
  int64_t cache_hits;        /* batches that reused an idle batch of the same shapes */
  int64_t cached;            /* idle batches held now */
} pnm_server_stats;

#define PNM_REQ_QUEUED 0
#define PNM_REQ_RUNNING 1
#define PNM_REQ_DONE 2
#define PNM_REQ_FAILED 3
#define PNM_REQ_CANCELLED 4

int pnm_server_create(pnm_ctx* ctx, const pnm_server_config* cfg, pnm_server** out);
/* Fails queued requests as cancelled, waits for running batches, frees everything. */
void pnm_server_destroy(pnm_server* s);
const char* pnm_server_last_error(const pnm_server* s);
int pnm_server_submit(pnm_server* s, const float* sdf, int32_t nx, int32_t ny, int32_t nz,
                      const float origin_xyz[3], const float spacing_xyz[3], int64_t* ticket);
/* state: PNM_REQ_*; status: the request's PNM_* result once done or failed. */
int pnm_server_state(pnm_server* s, int64_t ticket, int32_t* state, int32_t* status);
/* Blocks until the request is done, failed or cancelled; returns its status
   (PNM_ERR_NOT_CONVERGED if timeout_s > 0 passes first). */
int pnm_server_wait(pnm_server* s, int64_t ticket, double timeout_s);
/* Removes a queued request (PNM_ERR_ARG once it is running or finished). */
int pnm_server_cancel(pnm_server* s, int64_t ticket);
/* Counts (info) and device pointers of a done request's resident results (any may be null). */
int pnm_server_result(pnm_server* s, int64_t ticket, pnm_batch_volume* info, pnm_pore** d_pores,
                      int32_t** d_seg, int32_t** d_pairs);
int pnm_server_copy_out(pnm_server* s, int64_t ticket, pnm_pore* pores, int32_t* seg,
                        int32_t* pairs);
/* Drops a finished request (its batch's memory returns when all its requests are released). */
int pnm_server_release(pnm_server* s, int64_t ticket);
int pnm_server_get_stats(pnm_server* s, pnm_server_stats* out);
int pnm_server_reset_stats(pnm_server* s);

/* ---- VTI ingest: SDFReader::read_vti (reference src/sdf_reader.cpp:28-152, bound as
 * peclet.pnm.SDFReader.read_vti in src/pnm_bindings.cpp:87-102). ImageData with one appended raw
 * float32 array behind a UInt64 byte count (the layout scripts/vti.py writes). The header is the
 * first 8 KiB of text: resolution from WholeExtent (max - min + 1 per axis), the first Origin and
 * Spacing attributes (0 when absent), the array after the first '_' past
 * <AppendedData encoding="raw">. A byte count other than nx*ny*nz*4 reads what both allow and
 * leaves the rest zero. These calls report failures through pnm_vti_last_error() (per thread);
 * pnm_read_vti_dev also through pnm_last_error(ctx). */
const char* pnm_vti_last_error(void);
/* Parses the header: dims / origin / spacing as xyz, *data_bytes the file's byte count. */
int pnm_read_vti_header(const char* path, int32_t dims_xyz[3], float origin_xyz[3],
                        float spacing_xyz[3], int64_t* data_bytes);
/* Reads the n = nx*ny*nz values (x fastest) into host memory. */
int pnm_read_vti(const char* path, float* values, int64_t n);
/* Streams the n values into device memory through pinned double-buffered staging on the
 * context's stream (file reads overlap the copies); returns once they are on the device. */
int pnm_read_vti_dev(pnm_ctx* ctx, const char* path, float* d_values, int64_t n);

#ifdef __cplusplus
}
#endif

#endif /* PNM_GB300_H */
