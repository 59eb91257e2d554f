"""Device-resident surface: the extraction calls on CUDA arrays, zero-copy.

Inputs are any CUDA array exporting DLPack (``__dlpack__``) or a ``torch`` CUDA tensor: a
simulation that holds its SDF and MAC fields on the GPU hands them over in place, with no host
round trip (the host surface of ``peclet_pnm_gb300`` mirrors the reference binding, which takes
numpy arrays and copies them to the device on every call, ``src/pnm_bindings.cpp:55-75``). Shapes
and dtypes are the reference's: (Nz,Ny,Nx) C-order, a float32 SDF and float64 fields; other
dtypes are converted on the device. Work runs on the caller's current ``torch`` CUDA stream, so
results are ordered with the caller's own kernels; outputs are ``torch`` tensors on the same
device.

* ``segment_volume_device(sdf, spacing_zyx) -> seg`` (int32, (Nz,Ny,Nx))
* ``extract_pore_network_device(sdf, origin_zyx, spacing_zyx) -> (pores (n,4) f32, seg, pairs
  (m,2) i32)``
* ``extract_network_flow_device(sdf, origin_zyx, spacing_zyx, u, v, w, p, ox=None, oy=None,
  oz=None, grad_p_zyx=(0,0,0)) -> dict`` of the reference's keys (``src/pnm_bindings.cpp:
  162-209``), every value a tensor.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _capi
from ._capi import Context, default_context

__all__ = ["segment_volume_device", "extract_pore_network_device", "extract_network_flow_device"]


def _torch():
    import torch
    return torch


def _dev_arg(x, dtype, name: str, shape=None):
    torch = _torch()
    t = x if isinstance(x, torch.Tensor) else torch.from_dlpack(x)
    if not t.is_cuda:
        raise RuntimeError(f"{name} must be a CUDA array")
    if t.ndim != 3:
        raise RuntimeError(f"{name} must be 3D (Nz,Ny,Nx)")
    if shape is not None and tuple(t.shape) != shape:
        raise RuntimeError(f"{name} must be (Nz,Ny,Nx) matching the SDF")
    return t.to(dtype).contiguous()


def _xyz32(v_zyx) -> np.ndarray:
    v = list(v_zyx)
    return np.array([v[2], v[1], v[0]], np.float32)


class _Stream:
    """Runs the context on the current torch stream for the duration of a call. A call on
    another stream than the context's previous one first waits for the previous call's work (the
    context's buffers are reused from call to call)."""

    def __init__(self, ctx: Context, device):
        self.ctx, self.device = ctx, device

    def __enter__(self):
        torch = _torch()
        self.guard = torch.cuda.device(self.device)
        self.guard.__enter__()
        self.stream = torch.cuda.current_stream(self.device)
        last = getattr(self.ctx, "_device_last", None)
        if last is not None and last[0] != self.stream.cuda_stream:
            self.stream.wait_event(last[1])
        self.saved = self.ctx.stream_ptr
        self.ctx.set_stream(self.stream.cuda_stream)
        return self

    def __exit__(self, *exc):
        ev = _torch().cuda.Event()
        ev.record(self.stream)
        self.ctx._device_last = (self.stream.cuda_stream, ev)
        self.ctx.set_stream(self.saved)  # the stream the caller had set on the context, if any
        self.guard.__exit__(*exc)


class _View:
    """A borrowed device array (``__cuda_array_interface__``) over library-owned memory."""

    def __init__(self, ptr: int, shape, typestr: str):
        self.__cuda_array_interface__ = {"shape": tuple(shape), "typestr": typestr,
                                         "data": (int(ptr or 0), False), "version": 2,
                                         "strides": None}


def _owned(ptr, shape, typestr, torch_dtype, device):
    """Copies a context-owned result into a new tensor (on the current stream)."""
    torch = _torch()
    if int(np.prod(shape)) == 0 or not ptr:
        return torch.zeros(shape, dtype=torch_dtype, device=device)
    return torch.as_tensor(_View(ptr, shape, typestr), device=device).clone()


def segment_volume_device(sdf, spacing_zyx, *, ctx: Context | None = None):
    torch = _torch()
    a = _dev_arg(sdf, torch.float32, "SDF")
    nz, ny, nx = a.shape
    seg = torch.empty((nz, ny, nx), dtype=torch.int32, device=a.device)
    if a.numel() == 0:
        return seg
    ctx = ctx or default_context()
    s = _xyz32(spacing_zyx)
    with _Stream(ctx, a.device):
        ctx.check(_capi.pnm_segment_volume_dev(ctx.h, a.data_ptr(), nx, ny, nz, _capi.as_ptr(s),
                                               seg.data_ptr()))
    return seg


def extract_pore_network_device(sdf, origin_zyx, spacing_zyx, *, ctx: Context | None = None,
                                want_seg: bool = True, pore_cap: int | None = None,
                                pair_cap: int | None = None):
    """Returns (pores, seg or None, pairs) as device tensors. `pore_cap` / `pair_cap` size the
    first attempt's outputs (default: one pore per 64 voxels, eight pairs per pore); a volume that
    needs more is run again with the counts the first attempt reports."""
    torch = _torch()
    a = _dev_arg(sdf, torch.float32, "SDF")
    nz, ny, nx = a.shape
    dev = a.device
    n = a.numel()
    seg = torch.empty((nz, ny, nx), dtype=torch.int32, device=dev) if want_seg else None
    if n == 0:
        return (torch.zeros((0, 4), dtype=torch.float32, device=dev), seg,
                torch.zeros((0, 2), dtype=torch.int32, device=dev))
    ctx = ctx or default_context()
    o, s = _xyz32(origin_zyx), _xyz32(spacing_zyx)
    pore_cap = max(1, int(pore_cap)) if pore_cap is not None else max(64, n // 64)
    pair_cap = max(1, int(pair_cap)) if pair_cap is not None else 8 * pore_cap
    for _ in range(2):
        pores = torch.empty((pore_cap, 4), dtype=torch.float32, device=dev)
        pairs = torch.empty((pair_cap, 2), dtype=torch.int32, device=dev)
        npo, npa = _capi._i64(), _capi._i64()
        with _Stream(ctx, dev):
            rc = _capi.pnm_extract_pore_network_dev(
                ctx.h, a.data_ptr(), nx, ny, nz, _capi.as_ptr(o), _capi.as_ptr(s),
                pores.data_ptr(), pore_cap, ctypes.byref(npo),
                seg.data_ptr() if want_seg else None, pairs.data_ptr(), pair_cap,
                ctypes.byref(npa))
        if rc == _capi.PNM_ERR_CAPACITY:
            pore_cap, pair_cap = max(pore_cap, npo.value), max(pair_cap, npa.value)
            continue
        ctx.check(rc)
        return pores[:npo.value], seg, pairs[:npa.value]
    ctx.check(rc)


def extract_network_flow_device(sdf, origin_zyx, spacing_zyx, u, v, w, p, ox=None, oy=None,
                                oz=None, grad_p_zyx=(0.0, 0.0, 0.0), *,
                                ctx: Context | None = None) -> dict:
    torch = _torch()
    if (ox is None) != (oy is None) or (ox is None) != (oz is None):
        raise RuntimeError("pass all three openness arrays (ox,oy,oz) or none")
    a = _dev_arg(sdf, torch.float32, "SDF")
    shape = tuple(a.shape)
    dev = a.device
    f = [_dev_arg(x, torch.float64, nm, shape) for x, nm in ((u, "u"), (v, "v"), (w, "w"),
                                                             (p, "p"))]
    opn = [None if x is None else _dev_arg(x, torch.float64, nm, shape)
           for x, nm in ((ox, "ox"), (oy, "oy"), (oz, "oz"))]
    nz, ny, nx = shape
    gp = list(grad_p_zyx)
    g = np.array([gp[2], gp[1], gp[0]], np.float64)
    o, s = _xyz32(origin_zyx), _xyz32(spacing_zyx)
    r = _capi.PnmFlowResultDev()
    if a.numel() > 0:
        ctx = ctx or default_context()
        with _Stream(ctx, dev):
            ctx.check(_capi.pnm_extract_network_flow_dev(
                ctx.h, a.data_ptr(), nx, ny, nz, _capi.as_ptr(o), _capi.as_ptr(s),
                *[x.data_ptr() for x in f], *[None if x is None else x.data_ptr() for x in opn],
                _capi.as_ptr(g), ctypes.byref(r)))
            # copies out of the context's buffers, queued behind the extraction
            npo, nt = int(r.n_pores), int(r.n_throats)
            f64 = torch.float64
            return {
                "pores": _owned(r.pores, (npo, 4), "<f4", torch.float32, dev),
                "pore_pressure": _owned(r.pore_pressure, (npo,), "<f8", f64, dev),
                "pore_residual": _owned(r.pore_residual, (npo,), "<f8", f64, dev),
                "throats": _owned(r.throats, (nt, 2), "<i4", torch.int32, dev),
                "throat_flow": _owned(r.throat_flow, (nt,), "<f8", f64, dev),
                "throat_area": _owned(r.throat_area, (nt,), "<f8", f64, dev),
                "throat_dp": _owned(r.throat_dp, (nt,), "<f8", f64, dev),
            }
    z = lambda *sh, dt=torch.float64: torch.zeros(sh, dtype=dt, device=dev)  # noqa: E731
    return {"pores": z(0, 4, dt=torch.float32), "pore_pressure": z(0), "pore_residual": z(0),
            "throats": z(0, 2, dt=torch.int32), "throat_flow": z(0), "throat_area": z(0),
            "throat_dp": z(0)}
