"""Serving: a request loop with continuous batching over the batched pipeline (``pnm_server_*``).

No counterpart in the reference (its calls are serial and blocking). A :class:`Server` owns a
native scheduler thread: :meth:`Server.submit` queues one periodic volume and returns a ticket;
requests are admitted under a device-memory budget (120 GB by default), whatever is queued when a
stream slot frees runs as one batch, several batches run concurrently, and results stay resident
on the device until :meth:`Server.release`.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _capi
from ._capi import Context, PnmError, default_context

__all__ = ["Server"]

_STATES = {_capi.PNM_REQ_QUEUED: "queued", _capi.PNM_REQ_RUNNING: "running",
           _capi.PNM_REQ_DONE: "done", _capi.PNM_REQ_FAILED: "failed",
           _capi.PNM_REQ_CANCELLED: "cancelled"}


class Server:
    def __init__(self, budget_bytes: int = 0, max_inflight: int = 0, max_batch_volumes: int = 0,
                 max_batch_voxels: int = 0, *, ctx: Context | None = None):
        self.ctx = ctx or default_context()
        cfg = _capi.PnmServerConfig(int(budget_bytes), int(max_inflight), int(max_batch_volumes),
                                    int(max_batch_voxels))
        h = _capi._vp()
        rc = _capi.pnm_server_create(self.ctx.h, ctypes.byref(cfg), ctypes.byref(h))
        if rc != _capi.PNM_OK:
            raise PnmError(rc, _capi.pnm_last_error(self.ctx.h).decode(errors="replace"))
        self.h = h
        self._inputs = {}  # ticket -> the array the request reads (kept alive until it is done)

    def _check(self, rc: int):
        if rc != _capi.PNM_OK:
            msg = _capi.pnm_server_last_error(self.h).decode(errors="replace")
            raise PnmError(rc, msg or f"pnm server error {rc}")

    def submit(self, sdf, origin_zyx=(0.0, 0.0, 0.0), spacing_zyx=(1.0, 1.0, 1.0)) -> int:
        """Queues one volume; `sdf` is a (Nz,Ny,Nx) array (numpy, or an object exposing
        ``data_ptr()`` and ``shape`` such as a CUDA tensor, read in place)."""
        o = np.array(list(origin_zyx)[::-1], np.float32)
        s = np.array(list(spacing_zyx)[::-1], np.float32)
        if hasattr(sdf, "data_ptr"):
            nz, ny, nx = (int(v) for v in sdf.shape)
            ptr, keep = ctypes.c_void_p(sdf.data_ptr()), sdf
        else:
            a = np.ascontiguousarray(np.asarray(sdf), dtype=np.float32)
            if a.ndim != 3:
                raise RuntimeError("SDF array must be 3D (Nz,Ny,Nx)")
            nz, ny, nx = a.shape
            ptr, keep = _capi.as_ptr(a), a
        t = _capi._i64()
        self._check(_capi.pnm_server_submit(self.h, ptr, nx, ny, nz, _capi.as_ptr(o),
                                            _capi.as_ptr(s), ctypes.byref(t)))
        self._inputs[t.value] = keep
        return int(t.value)

    def state(self, ticket: int):
        st, code = _capi._i32(), _capi._i32()
        self._check(_capi.pnm_server_state(self.h, int(ticket), ctypes.byref(st),
                                           ctypes.byref(code)))
        return _STATES[st.value], int(code.value)

    def wait(self, ticket: int, timeout_s: float = 0.0) -> int:
        """Blocks until the request finishes; returns its status code (0 = ok)."""
        return int(_capi.pnm_server_wait(self.h, int(ticket), float(timeout_s)))

    def cancel(self, ticket: int):
        self._check(_capi.pnm_server_cancel(self.h, int(ticket)))

    def info(self, ticket: int) -> dict:
        v = _capi.PnmBatchVolume()
        self._check(_capi.pnm_server_result(self.h, int(ticket), ctypes.byref(v), None, None,
                                            None))
        return {k: getattr(v, k) for k, _ in _capi.PnmBatchVolume._fields_ if k != "reserved"}

    def result(self, ticket: int, seg: bool = True):
        """(pores (n,4) float32, labels (Nz*Ny*Nx,) int32 or None, pairs (m,2) int32)."""
        v = self.info(ticket)
        pores = np.empty((v["n_pores"], 4), np.float32)
        pairs = np.empty((v["n_pairs"], 2), np.int32)
        labels = np.empty(v["nx"] * v["ny"] * v["nz"], np.int32) if seg else None
        self._check(_capi.pnm_server_copy_out(self.h, int(ticket), _capi.as_ptr(pores),
                                              _capi.as_ptr(labels) if seg else None,
                                              _capi.as_ptr(pairs)))
        return pores, labels, pairs

    def release(self, ticket: int):
        self._check(_capi.pnm_server_release(self.h, int(ticket)))
        self._inputs.pop(int(ticket), None)

    def stats(self) -> dict:
        st = _capi.PnmServerStats()
        self._check(_capi.pnm_server_get_stats(self.h, ctypes.byref(st)))
        return {k: getattr(st, k) for k, _ in _capi.PnmServerStats._fields_}

    def reset_stats(self):
        self._check(_capi.pnm_server_reset_stats(self.h))

    def close(self):
        if getattr(self, "h", None):
            _capi.pnm_server_destroy(self.h)
            self.h = None
            self._inputs.clear()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
