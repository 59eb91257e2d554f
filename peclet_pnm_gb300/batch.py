"""Batched extraction: many periodic SDF volumes of uneven shapes in one run (``pnm_batch_*``).

No counterpart in the reference, whose bindings take one volume per call
(``src/pnm_bindings.cpp:143-160``). A :class:`Batch` is planned once for a list of shapes; each
:meth:`Batch.run` extracts every volume with one launch per pipeline stage over a ragged volume
table (replayed from a CUDA graph after the first run). Per volume the results equal
``extract_pore_network`` on that volume alone, bit for bit.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _capi
from ._capi import Context, PnmError, default_context

__all__ = ["Batch", "extract_pore_network_batch", "batch_plan_bytes"]


def _xyz_rows(vals_zyx, n, default):
    if vals_zyx is None:
        return np.tile(np.asarray(default, np.float32), (n, 1))
    a = np.asarray(vals_zyx, dtype=np.float32).reshape(-1, 3)
    if a.shape[0] == 1 and n > 1:
        a = np.tile(a, (n, 1))
    if a.shape[0] != n:
        raise RuntimeError("one origin / spacing (zyx) per volume expected")
    return np.ascontiguousarray(a[:, ::-1])


def _dims(shapes_zyx) -> np.ndarray:
    rows = []
    for s in shapes_zyx:
        s = tuple(int(v) for v in s)
        if len(s) != 3:
            raise RuntimeError("SDF array must be 3D (Nz,Ny,Nx)")
        rows.append((s[2], s[1], s[0]))
    if not rows:
        raise RuntimeError("a batch needs at least one volume")
    return np.ascontiguousarray(np.array(rows, dtype=np.int32))


def batch_plan_bytes(shapes_zyx) -> int:
    """Device bytes a batch of these shapes allocates when created."""
    d = _dims(shapes_zyx)
    out = _capi._i64()
    rc = _capi.pnm_batch_plan_bytes(len(d), _capi.as_ptr(d), ctypes.byref(out))
    if rc != _capi.PNM_OK:
        raise PnmError(rc, "invalid batch shapes")
    return int(out.value)


class Batch:
    """A planned ragged batch (device buffers allocated once, reused by every run)."""

    def __init__(self, shapes_zyx, origins_zyx=None, spacings_zyx=None, *,
                 ctx: Context | None = None, graph: bool = True):
        self.shapes = [tuple(int(v) for v in s) for s in shapes_zyx]
        d = _dims(self.shapes)
        n = len(d)
        o = _xyz_rows(origins_zyx, n, (0.0, 0.0, 0.0))
        sp = _xyz_rows(spacings_zyx, n, (1.0, 1.0, 1.0))
        self.ctx = ctx or default_context()
        h = _capi._vp()
        flags = 0 if graph else _capi.PNM_BATCH_NO_GRAPH
        rc = _capi.pnm_batch_create(self.ctx.h, n, _capi.as_ptr(d), _capi.as_ptr(o),
                                    _capi.as_ptr(sp), flags, ctypes.byref(h))
        if rc != _capi.PNM_OK:
            msg = _capi.pnm_last_error(self.ctx.h).decode(errors="replace")
            raise PnmError(rc, msg or f"pnm_batch_create failed ({rc})")
        self.h = h

    def __len__(self):
        return len(self.shapes)

    def check(self, rc: int):
        if rc != _capi.PNM_OK:
            msg = _capi.pnm_batch_last_error(self.h).decode(errors="replace")
            raise PnmError(rc, msg or f"pnm batch error {rc}")

    @property
    def stream(self) -> int:
        """The batch's cudaStream_t as an integer."""
        return int(_capi.pnm_batch_stream(self.h) or 0)

    def set_sdf(self, i: int, sdf):
        a = np.ascontiguousarray(np.asarray(sdf), dtype=np.float32)
        if a.shape != self.shapes[i]:
            raise RuntimeError(f"volume {i}: SDF shape {a.shape} != planned {self.shapes[i]}")
        # from pageable memory the copy has left `a` when the call returns
        self.check(_capi.pnm_batch_set_sdf(self.h, int(i), _capi.as_ptr(a)))

    def sdf_device(self):
        """(device pointer, length in floats) of the batch SDF buffer (volume i at offset(i))."""
        p = _capi._vp()
        n = _capi._i64()
        self.check(_capi.pnm_batch_sdf_dev(self.h, ctypes.byref(p), ctypes.byref(n)))
        return int(p.value or 0), int(n.value)

    def offset(self, i: int) -> int:
        """First voxel of volume i in the batch buffers (available before any run)."""
        off = 0
        for s in self.shapes[:i]:
            off = (off + s[0] * s[1] * s[2] + 31) & ~31
        return off

    def launch(self):
        self.check(_capi.pnm_batch_launch(self.h))

    def wait(self):
        self.check(_capi.pnm_batch_wait(self.h))

    def run(self):
        self.check(_capi.pnm_batch_run(self.h))

    def volume(self, i: int) -> dict:
        info = _capi.PnmBatchVolume()
        self.check(_capi.pnm_batch_volume_info(self.h, int(i), ctypes.byref(info)))
        return {k: getattr(info, k) for k, _ in _capi.PnmBatchVolume._fields_ if k != "reserved"}

    def result(self, i: int, seg: bool = True):
        """(pores (n,4) float32, labels (n_voxels,) int32 or None, pairs (m,2) int32)."""
        v = self.volume(i)
        pores = np.empty((v["n_pores"], 4), np.float32)
        pairs = np.empty((v["n_pairs"], 2), np.int32)
        labels = np.empty(v["nx"] * v["ny"] * v["nz"], np.int32) if seg else None
        self.check(_capi.pnm_batch_copy_out(self.h, int(i), _capi.as_ptr(pores),
                                            _capi.as_ptr(labels) if seg else None,
                                            _capi.as_ptr(pairs)))
        return pores, labels, pairs

    def results(self, seg: bool = True):
        return [self.result(i, seg) for i in range(len(self))]

    def results_device(self):
        """Device pointers (pores, labels, pairs) of the last run; slice with volume(i)."""
        p, s, q = _capi._vp(), _capi._vp(), _capi._vp()
        self.check(_capi.pnm_batch_results_dev(self.h, ctypes.byref(p), ctypes.byref(s),
                                               ctypes.byref(q)))
        return int(p.value or 0), int(s.value or 0), int(q.value or 0)

    @property
    def uses_graph(self) -> bool:
        return bool(_capi.pnm_batch_uses_graph(self.h))

    @property
    def tuning(self) -> dict:
        """Launch shape of the stages (tile_z, blocks_per_sm, ccl_blocks_per_sm,
        flood_blocks_per_sm); results never depend on it."""
        t = _capi.PnmTuning()
        self.check(_capi.pnm_batch_get_tuning(self.h, ctypes.byref(t)))
        return {k: getattr(t, k) for k, _ in _capi.PnmTuning._fields_}

    def set_tuning(self, **kw):
        t = _capi.PnmTuning(**{**self.tuning, **kw})
        self.check(_capi.pnm_batch_set_tuning(self.h, ctypes.byref(t)))

    def autotune(self, cache: str | None = None, reps: int = 3, force: bool = False) -> dict:
        """Times candidate launch shapes on the current SDFs and keeps the fastest; `cache` (a
        text file) remembers the choice per (device, typical edge, volume count) class."""
        ms = ctypes.c_double()
        self.check(_capi.pnm_batch_autotune(self.h, cache.encode() if cache else None, int(reps),
                                            _capi.PNM_TUNE_FORCE if force else 0,
                                            ctypes.byref(ms)))
        return {**self.tuning, "ms": ms.value}

    def stats(self) -> dict:
        st = _capi.PnmStats()
        self.check(_capi.pnm_batch_get_stats(self.h, ctypes.byref(st)))
        return {k: getattr(st, k) for k, _ in _capi.PnmStats._fields_
                if k not in ("reserved", "stage_ms")}

    def close(self):
        if getattr(self, "h", None):
            _capi.pnm_batch_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def extract_pore_network_batch(sdfs, origins_zyx=None, spacings_zyx=None, *,
                               ctx: Context | None = None, graph: bool = True):
    """extract_pore_network over a list of volumes in one batched run.

    Returns one (pores (n,4) float32, labels (Nz*Ny*Nx,) int32, pairs (m,2) int32) per volume.
    """
    arrs = [np.ascontiguousarray(np.asarray(a), dtype=np.float32) for a in sdfs]
    for a in arrs:
        if a.ndim != 3:
            raise RuntimeError("SDF array must be 3D (Nz,Ny,Nx)")
    with Batch([a.shape for a in arrs], origins_zyx, spacings_zyx, ctx=ctx, graph=graph) as b:
        for i, a in enumerate(arrs):
            b.set_sdf(i, a)
        b.run()
        return b.results()
