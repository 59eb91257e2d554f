"""ctypes binding of libpnm_gb300.so (the C ABI declared in include/pnm_gb300.h).

The shared library must have been built (``peclet_pnm_gb300.build.build()``); there is no
fallback implementation, so importing this module without it raises ImportError.
"""
from __future__ import annotations

import ctypes
import os
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libpnm_gb300.so")

PNM_OK = 0
PNM_ERR_ARG = 1
PNM_ERR_SHAPE = 2
PNM_ERR_CAPACITY = 3
PNM_ERR_NOT_CONVERGED = 4
PNM_ERR_CUDA = 5
PNM_ERR_NO_DEVICE = 6
PNM_ERR_INTERNAL = 7

if not os.path.exists(LIB_PATH):
    raise ImportError(f"{LIB_PATH} is not built; run `python peclet_pnm_gb300/build.py` "
                      "(no CPU fallback exists)")

lib = ctypes.CDLL(LIB_PATH)

_P = ctypes.POINTER
_vp = ctypes.c_void_p
_i32 = ctypes.c_int32
_i64 = ctypes.c_int64


class PnmPore(ctypes.Structure):
    _fields_ = [("x", ctypes.c_float), ("y", ctypes.c_float), ("z", ctypes.c_float),
                ("radius", ctypes.c_float)]


class PnmFlowResultDev(ctypes.Structure):
    _fields_ = [("n_pores", _i64), ("n_throats", _i64), ("pores", _vp), ("pore_pressure", _vp),
                ("pore_residual", _vp), ("throats", _vp), ("throat_flow", _vp),
                ("throat_area", _vp), ("throat_dp", _vp)]


class PnmFlowStats(ctypes.Structure):
    _fields_ = [("n_pores", _i64), ("n_throats", _i64), ("mean_abs_flow", ctypes.c_double),
                ("max_abs_flow", ctypes.c_double), ("mean_abs_dp", ctypes.c_double),
                ("max_abs_residual", ctypes.c_double), ("n_positive_conductance", _i64),
                ("n_finite_conductance", _i64), ("mean_coordination", ctypes.c_double),
                ("max_coordination", _i32), ("mass_balance_ok", _i32)]


class PnmFlowResult(ctypes.Structure):
    _fields_ = [("n_pores", _i64), ("n_throats", _i64), ("pores", _P(PnmPore)),
                ("pore_pressure", _P(ctypes.c_double)), ("pore_residual", _P(ctypes.c_double)),
                ("throats", _P(ctypes.c_int32)), ("throat_flow", _P(ctypes.c_double)),
                ("throat_area", _P(ctypes.c_double)), ("throat_dp", _P(ctypes.c_double))]


#: PNM_STAGE_* in order: the reference kernel labels each stage covers
STAGES = ["sdf_pass", "merge_markers", "gradient_path", "flood", "relabel", "seg_pairs",
          "pair_sort", "pores", "network_flow"]


class PnmStats(ctypes.Structure):
    _fields_ = [("launches", _i64), ("calls", _i64), ("voxels", _i64), ("ccl_edges", _i64),
                ("flood_sweeps", _i32), ("n_pore_labels", _i32), ("n_solid_labels", _i32),
                ("reserved", _i32), ("n_pores", _i64), ("n_pairs", _i64),
                ("workspace_bytes", _i64), ("stage_ms", ctypes.c_double * len(STAGES))]


def _sig(name, res, *args):
    f = getattr(lib, name)
    f.restype = res
    f.argtypes = list(args)
    return f


pnm_ctx_create = _sig("pnm_ctx_create", ctypes.c_int, ctypes.c_int, _P(_vp))
pnm_ctx_destroy = _sig("pnm_ctx_destroy", None, _vp)
pnm_last_error = _sig("pnm_last_error", ctypes.c_char_p, _vp)
pnm_ctx_set_stream = _sig("pnm_ctx_set_stream", ctypes.c_int, _vp, _vp)
pnm_ctx_trim = _sig("pnm_ctx_trim", ctypes.c_int, _vp)
pnm_execution_space = _sig("pnm_execution_space", ctypes.c_char_p)
pnm_ctx_get_stats = _sig("pnm_ctx_get_stats", ctypes.c_int, _vp, _P(PnmStats))
pnm_ctx_set_timing = _sig("pnm_ctx_set_timing", ctypes.c_int, _vp, _i32)
pnm_ctx_set_wait_limit = _sig("pnm_ctx_set_wait_limit", ctypes.c_int, _vp, _i64, _i32)
pnm_free = _sig("pnm_free", None, _vp)
pnm_extract_pores = _sig("pnm_extract_pores", ctypes.c_int, _vp, _vp, _i32, _i32, _i32, _vp, _vp,
                         _P(_P(PnmPore)), _P(_i64))
pnm_segment_volume = _sig("pnm_segment_volume", ctypes.c_int, _vp, _vp, _i32, _i32, _i32, _vp,
                          _vp)
pnm_pore_peaks_dev = _sig("pnm_pore_peaks_dev", ctypes.c_int, _vp, _vp, _i32, _i32, _i32, _vp,
                          _i64, _P(_i64))
pnm_segment_volume_dev = _sig("pnm_segment_volume_dev", ctypes.c_int, _vp, _vp, _i32, _i32, _i32,
                              _vp, _vp)
pnm_extract_topology = _sig("pnm_extract_topology", ctypes.c_int, _vp, _vp, _i32, _i32, _i32,
                            _P(_P(ctypes.c_int32)), _P(_i64))
pnm_extract_pore_network = _sig("pnm_extract_pore_network", ctypes.c_int, _vp, _vp, _i32, _i32,
                                _i32, _vp, _vp, _P(_P(PnmPore)), _P(_i64), _vp,
                                _P(_P(ctypes.c_int32)), _P(_i64))
pnm_extract_pore_network_dev = _sig("pnm_extract_pore_network_dev", ctypes.c_int, _vp, _vp, _i32,
                                    _i32, _i32, _vp, _vp, _vp, _i64, _P(_i64), _vp, _vp, _i64,
                                    _P(_i64))
pnm_extract_network_flow = _sig("pnm_extract_network_flow", ctypes.c_int, _vp, _vp, _i32, _i32,
                                _i32, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp,
                                _P(_P(PnmFlowResult)))
pnm_flow_result_free = _sig("pnm_flow_result_free", None, _P(PnmFlowResult))
pnm_extract_network_flow_dev = _sig("pnm_extract_network_flow_dev", ctypes.c_int, _vp, _vp, _i32,
                                    _i32, _i32, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp,
                                    _P(PnmFlowResultDev))
pnm_flow_stats_dev = _sig("pnm_flow_stats_dev", ctypes.c_int, _vp, _P(PnmFlowResultDev), _vp, _vp,
                          _P(PnmFlowStats))
pnm_extract_pores_noalloc = _sig("pnm_extract_pores_noalloc", ctypes.c_int, _vp, _i32, _i32, _i32,
                                 _vp, _vp, _vp, _i64, _P(_i64), _vp)



class PnmBatchVolume(ctypes.Structure):
    _fields_ = [("voxel_offset", _i64), ("nx", _i32), ("ny", _i32), ("nz", _i32),
                ("n_pore_labels", _i32), ("n_solid_labels", _i32), ("reserved", _i32),
                ("pore_offset", _i64), ("n_pores", _i64), ("pair_offset", _i64),
                ("n_pairs", _i64)]


PNM_BATCH_NO_GRAPH = 1
pnm_batch_plan_bytes = _sig("pnm_batch_plan_bytes", ctypes.c_int, _i32, _vp, _P(_i64))
pnm_batch_create = _sig("pnm_batch_create", ctypes.c_int, _vp, _i32, _vp, _vp, _vp, _i32,
                        _P(_vp))
pnm_batch_destroy = _sig("pnm_batch_destroy", None, _vp)
pnm_batch_last_error = _sig("pnm_batch_last_error", ctypes.c_char_p, _vp)
pnm_batch_stream = _sig("pnm_batch_stream", _vp, _vp)
pnm_batch_set_sdf = _sig("pnm_batch_set_sdf", ctypes.c_int, _vp, _i32, _vp)
pnm_batch_sdf_dev = _sig("pnm_batch_sdf_dev", ctypes.c_int, _vp, _P(_vp), _P(_i64))
pnm_batch_launch = _sig("pnm_batch_launch", ctypes.c_int, _vp)
pnm_batch_wait = _sig("pnm_batch_wait", ctypes.c_int, _vp)
pnm_batch_run = _sig("pnm_batch_run", ctypes.c_int, _vp)
pnm_batch_volume_info = _sig("pnm_batch_volume_info", ctypes.c_int, _vp, _i32,
                             _P(PnmBatchVolume))
pnm_batch_results_dev = _sig("pnm_batch_results_dev", ctypes.c_int, _vp, _P(_vp), _P(_vp),
                             _P(_vp))
pnm_batch_copy_out = _sig("pnm_batch_copy_out", ctypes.c_int, _vp, _i32, _vp, _vp, _vp)
pnm_batch_get_stats = _sig("pnm_batch_get_stats", ctypes.c_int, _vp, _P(PnmStats))
pnm_batch_uses_graph = _sig("pnm_batch_uses_graph", ctypes.c_int, _vp)


class PnmTuning(ctypes.Structure):
    _fields_ = [("tile_z", _i32), ("blocks_per_sm", _i32), ("ccl_blocks_per_sm", _i32),
                ("flood_blocks_per_sm", _i32)]


PNM_TUNE_FORCE = 1
pnm_batch_set_tuning = _sig("pnm_batch_set_tuning", ctypes.c_int, _vp, _P(PnmTuning))
pnm_batch_get_tuning = _sig("pnm_batch_get_tuning", ctypes.c_int, _vp, _P(PnmTuning))
pnm_batch_autotune = _sig("pnm_batch_autotune", ctypes.c_int, _vp, ctypes.c_char_p, _i32, _i32,
                          _P(ctypes.c_double))



class PnmServerConfig(ctypes.Structure):
    _fields_ = [("budget_bytes", _i64), ("max_inflight", _i32), ("max_batch_volumes", _i32),
                ("max_batch_voxels", _i64), ("reserved", _i32 * 4)]


class PnmServerStats(ctypes.Structure):
    _fields_ = [("submitted", _i64), ("completed", _i64), ("failed", _i64), ("cancelled", _i64),
                ("queued", _i64), ("running", _i64), ("batches", _i64), ("bytes_in_use", _i64),
                ("peak_bytes", _i64), ("voxels_completed", _i64), ("p50_ms", ctypes.c_double),
                ("p99_ms", ctypes.c_double), ("mean_ms", ctypes.c_double),
                ("max_ms", ctypes.c_double), ("busy_s", ctypes.c_double),
                ("gvoxel_per_s", ctypes.c_double), ("cache_hits", _i64), ("cached", _i64)]


PNM_REQ_QUEUED, PNM_REQ_RUNNING, PNM_REQ_DONE, PNM_REQ_FAILED, PNM_REQ_CANCELLED = range(5)
pnm_server_create = _sig("pnm_server_create", ctypes.c_int, _vp, _P(PnmServerConfig), _P(_vp))
pnm_server_destroy = _sig("pnm_server_destroy", None, _vp)
pnm_server_last_error = _sig("pnm_server_last_error", ctypes.c_char_p, _vp)
pnm_server_submit = _sig("pnm_server_submit", ctypes.c_int, _vp, _vp, _i32, _i32, _i32, _vp, _vp,
                         _P(_i64))
pnm_server_state = _sig("pnm_server_state", ctypes.c_int, _vp, _i64, _P(_i32), _P(_i32))
pnm_server_wait = _sig("pnm_server_wait", ctypes.c_int, _vp, _i64, ctypes.c_double)
pnm_server_cancel = _sig("pnm_server_cancel", ctypes.c_int, _vp, _i64)
pnm_server_result = _sig("pnm_server_result", ctypes.c_int, _vp, _i64, _P(PnmBatchVolume),
                         _P(_vp), _P(_vp), _P(_vp))
pnm_server_copy_out = _sig("pnm_server_copy_out", ctypes.c_int, _vp, _i64, _vp, _vp, _vp)
pnm_server_release = _sig("pnm_server_release", ctypes.c_int, _vp, _i64)
pnm_server_get_stats = _sig("pnm_server_get_stats", ctypes.c_int, _vp, _P(PnmServerStats))
pnm_server_reset_stats = _sig("pnm_server_reset_stats", ctypes.c_int, _vp)

pnm_vti_last_error = _sig("pnm_vti_last_error", ctypes.c_char_p)
pnm_read_vti_header = _sig("pnm_read_vti_header", ctypes.c_int, ctypes.c_char_p, _vp, _vp, _vp,
                           _P(_i64))
pnm_read_vti = _sig("pnm_read_vti", ctypes.c_int, ctypes.c_char_p, _vp, _i64)
pnm_read_vti_dev = _sig("pnm_read_vti_dev", ctypes.c_int, _vp, ctypes.c_char_p, _vp, _i64)

#: every symbol include/pnm_gb300.h declares
EXPORTED = ["pnm_ctx_create", "pnm_ctx_destroy", "pnm_last_error", "pnm_ctx_set_stream",
            "pnm_ctx_trim", "pnm_execution_space", "pnm_free", "pnm_extract_pores",
            "pnm_segment_volume", "pnm_extract_topology", "pnm_extract_pore_network",
            "pnm_extract_network_flow", "pnm_flow_result_free", "pnm_extract_pore_network_dev",
            "pnm_segment_volume_dev", "pnm_pore_peaks_dev", "pnm_ctx_get_stats", "pnm_ctx_set_timing",
            "pnm_ctx_set_wait_limit", "pnm_extract_pores_noalloc",
            "pnm_batch_plan_bytes", "pnm_batch_create", "pnm_batch_destroy",
            "pnm_batch_last_error", "pnm_batch_stream", "pnm_batch_set_sdf", "pnm_batch_sdf_dev",
            "pnm_batch_launch", "pnm_batch_wait", "pnm_batch_run", "pnm_batch_volume_info",
            "pnm_batch_results_dev", "pnm_batch_copy_out", "pnm_batch_get_stats",
            "pnm_batch_uses_graph", "pnm_batch_set_tuning", "pnm_batch_get_tuning",
            "pnm_batch_autotune", "pnm_server_create", "pnm_server_destroy",
            "pnm_server_last_error", "pnm_server_submit", "pnm_server_state", "pnm_server_wait",
            "pnm_server_cancel", "pnm_server_result", "pnm_server_copy_out", "pnm_server_release",
            "pnm_server_get_stats", "pnm_server_reset_stats", "pnm_vti_last_error",
            "pnm_read_vti_header", "pnm_read_vti", "pnm_read_vti_dev",
            "pnm_extract_network_flow_dev", "pnm_flow_stats_dev"]


class PnmError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(msg)
        self.code = code


class Context:
    """One pnm_ctx (device, stream, workspace). Not shared between threads."""

    def __init__(self, device: int = -1):
        h = _vp()
        rc = pnm_ctx_create(int(device), ctypes.byref(h))
        if rc != PNM_OK:
            raise PnmError(rc, {PNM_ERR_NO_DEVICE: "no sm_103 CUDA device available",
                                PNM_ERR_CUDA: "CUDA initialisation failed"}.get(
                rc, f"pnm_ctx_create failed ({rc})"))
        self.h = h
        self.device = int(device) if device >= 0 else None  # None: the device current at creation
        self.stream_ptr = None  # the caller-owned stream set with set_stream, if any

    def check(self, rc: int):
        if rc != PNM_OK:
            msg = pnm_last_error(self.h).decode(errors="replace")
            raise PnmError(rc, msg or f"pnm error {rc}")

    def set_stream(self, stream_ptr: int | None):
        """Runs this context's work on a caller-owned cudaStream_t (None: its own stream)."""
        self.check(pnm_ctx_set_stream(self.h, stream_ptr or None))
        self.stream_ptr = stream_ptr or None

    def trim(self):
        self.check(pnm_ctx_trim(self.h))

    def stats(self) -> dict:
        """Cumulative counters and the last call's figures; ``stage_ms`` maps each stage to its
        device time in the last call (zeros unless timing is on)."""
        st = PnmStats()
        self.check(pnm_ctx_get_stats(self.h, ctypes.byref(st)))
        out = {k: getattr(st, k) for k, _ in PnmStats._fields_
               if k not in ("reserved", "stage_ms")}
        out["stage_ms"] = {name: float(st.stage_ms[i]) for i, name in enumerate(STAGES)}
        return out

    def set_timing(self, on: bool = True):
        """Per-stage device timing (CUDA events) of every following call."""
        self.check(pnm_ctx_set_timing(self.h, 1 if on else 0))

    def set_wait_limit(self, limit_ns: int = 1_000_000_000, extra_arrivals: int = 0):
        """Limit of each bounded device wait (the flood loop's grid barrier). extra_arrivals > 0
        makes those waits run out on purpose (tests of the error path); 0 in normal use."""
        self.check(pnm_ctx_set_wait_limit(self.h, int(limit_ns), int(extra_arrivals)))

    def close(self):
        if getattr(self, "h", None):
            pnm_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_tls = threading.local()


def default_context() -> Context:
    """The calling thread's context on the current device (created on first use)."""
    ctx = getattr(_tls, "ctx", None)
    if ctx is None:
        ctx = Context(-1)
        _tls.ctx = ctx
    return ctx


def as_ptr(a: np.ndarray):
    return a.ctypes.data_as(_vp)


def take_array(ptr, count: int, dtype, free: bool = True) -> np.ndarray:
    """Copies a library-allocated host buffer into numpy and frees it."""
    if count > 0:
        out = np.ctypeslib.as_array(ctypes.cast(ptr, _P(np.ctypeslib.as_ctypes_type(dtype))),
                                    (int(count),)).copy()
    else:
        out = np.zeros((0,), dtype)
    if free and ptr:
        pnm_free(ctypes.cast(ptr, _vp))
    return out
