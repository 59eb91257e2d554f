"""peclet_pnm_gb300 — GB300-native drop-in for the ``peclet.pnm`` extraction path.

Same Python surface as the reference module (``src/pnm_bindings.cpp:86-209``, re-exported by
``packaging/pnm_init.py``):

* ``Pore`` with read/write ``x, y, z, radius`` (stored as float32)
* ``extract_pores(sdf, origin_zyx, spacing_zyx) -> list[Pore]``
* ``segment_volume(sdf, spacing_zyx) -> list[int]``
* ``extract_topology_gpu(segmentation, shape) -> list[tuple[int, int]]``
* ``extract_pore_network(sdf, origin_zyx, spacing_zyx) -> (pores, segmentation, connections)``
* ``extract_network_flow(sdf, origin_zyx, spacing_zyx, u, v, w, p, ox=None, oy=None, oz=None,
  grad_p_zyx=[0, 0, 0]) -> dict``
* ``execution_space``
* ``SDFReader.read_vti(filename) -> (sdf_3d, origin_zyx, spacing_zyx)`` (``vti.py``)

Beyond the reference: ``*_device`` calls on CUDA tensors / DLPack arrays (``device.py``), batches
(``batch.py``), a serving loop (``server.py``), ``read_vti_device`` and ``network_stats``
(conductance and network statistics of a flow result, ``post.py``).

Arrays are ``(Nz, Ny, Nx)`` C-order (x fastest); the SDF is cast to float32 and the MAC fields
to float64 like nanobind's implicit conversion; origin / spacing are zyx and cast to float32.
Each call runs hand-written sm_103a CUDA kernels through ``libpnm_gb300.so``; there is no CPU
fallback. Every function also takes a keyword-only ``numpy=True`` that returns arrays instead of
Python lists (the list conversion of a large segmentation dominates Python-level time).
"""
from __future__ import annotations

import numpy as np

from . import _capi
from ._capi import Context, PnmError, default_context

__all__ = ["Pore", "extract_pores", "segment_volume", "extract_topology_gpu",
           "extract_pore_network", "extract_network_flow", "execution_space", "Context",
           "PnmError", "Batch", "extract_pore_network_batch", "batch_plan_bytes", "Server",
           "SDFReader", "read_vti_device", "save_vti", "write_sdf_vti", "write_edge_list",
           "segment_volume_device", "extract_pore_network_device", "extract_network_flow_device",
           "network_stats", "throat_conductance", "mpi_rank", "mpi_size", "mpi_block",
           "extract_pore_network_mpi", "extract_network_flow_mpi"]

execution_space = _capi.pnm_execution_space().decode()

from .batch import Batch, batch_plan_bytes, extract_pore_network_batch  # noqa: E402
from .server import Server  # noqa: E402
from .vti import SDFReader, read_vti_device, save_vti, write_edge_list, write_sdf_vti  # noqa: E402
from .device import (extract_network_flow_device, extract_pore_network_device,  # noqa: E402
                     segment_volume_device)
from .post import network_stats, throat_conductance  # noqa: E402
from .distributed import (extract_network_flow_mpi, extract_pore_network_mpi,  # noqa: E402
                          mpi_block, mpi_rank, mpi_size)


class Pore:
    """Pore record (``struct Pore``, ``pore_extraction.hpp:24-26``); fields are float32."""

    __slots__ = ("_v",)

    def __init__(self, x=0.0, y=0.0, z=0.0, radius=0.0):
        self._v = np.array([x, y, z, radius], dtype=np.float32)

    @classmethod
    def _from_row(cls, row):
        p = cls.__new__(cls)
        p._v = np.array(row, dtype=np.float32)
        return p

    def _get(i):
        return property(lambda self: float(self._v[i]),
                        lambda self, val: self._v.__setitem__(i, np.float32(val)))

    x = _get(0)
    y = _get(1)
    z = _get(2)
    radius = _get(3)
    del _get

    def __repr__(self):
        return f"Pore(x={self.x!r}, y={self.y!r}, z={self.z!r}, radius={self.radius!r})"


def _sdf_arg(sdf) -> np.ndarray:
    a = np.asarray(sdf)
    if a.ndim != 3:
        raise RuntimeError("SDF array must be 3D (Nz,Ny,Nx)")  # pnm_bindings.cpp:58-59
    return np.ascontiguousarray(a, dtype=np.float32)


def _field_arg(a, shape, name) -> np.ndarray:
    f = np.asarray(a)
    if f.ndim != 3 or f.shape != shape:
        raise RuntimeError(f"{name} must be (Nz,Ny,Nx) matching the SDF")  # :67-69
    return np.ascontiguousarray(f, dtype=np.float64)


def _xyz32(v_zyx) -> np.ndarray:
    v = list(v_zyx)
    return np.array([v[2], v[1], v[0]], dtype=np.float32)


def _pores_out(rows: np.ndarray, numpy: bool):
    rows = rows.reshape(-1, 4)
    if numpy:
        return rows
    return [Pore._from_row(r) for r in rows]


def _pairs_out(pairs: np.ndarray, numpy: bool):
    pairs = pairs.reshape(-1, 2)
    if numpy:
        return pairs
    return [(int(a), int(b)) for a, b in pairs.tolist()]


# ---- array-level calls (xyz float32 origin/spacing), used by the list-returning surface --------
def pores_array(sdf: np.ndarray, origin_xyz, spacing_xyz, ctx: Context | None = None):
    a = _sdf_arg(sdf)
    nz, ny, nx = a.shape
    o = np.asarray(origin_xyz, np.float32)
    s = np.asarray(spacing_xyz, np.float32)
    if a.size == 0:
        return np.zeros((0, 4), np.float32)
    ctx = ctx or default_context()
    pp = _capi._P(_capi.PnmPore)()
    cnt = _capi._i64()
    ctx.check(_capi.pnm_extract_pores(ctx.h, _capi.as_ptr(a), nx, ny, nz, _capi.as_ptr(o),
                                      _capi.as_ptr(s), _capi.ctypes.byref(pp),
                                      _capi.ctypes.byref(cnt)))
    return _capi.take_array(pp, 4 * cnt.value, np.float32).reshape(-1, 4)


def segment_array(sdf: np.ndarray, spacing_xyz, ctx: Context | None = None) -> np.ndarray:
    a = _sdf_arg(sdf)
    nz, ny, nx = a.shape
    s = np.asarray(spacing_xyz, np.float32)
    seg = np.empty(a.size, np.int32)
    if a.size == 0:
        return seg
    ctx = ctx or default_context()
    ctx.check(_capi.pnm_segment_volume(ctx.h, _capi.as_ptr(a), nx, ny, nz, _capi.as_ptr(s),
                                       _capi.as_ptr(seg)))
    return seg


def topology_array(seg, nx: int, ny: int, nz: int, ctx: Context | None = None) -> np.ndarray:
    sg = np.ascontiguousarray(np.asarray(seg).reshape(-1), dtype=np.int32)
    if sg.size == 0:
        return np.zeros((0, 2), np.int32)
    if sg.size != nx * ny * nz:
        raise RuntimeError("segmentation length does not match shape")
    ctx = ctx or default_context()
    pr = _capi._P(_capi.ctypes.c_int32)()
    cnt = _capi._i64()
    ctx.check(_capi.pnm_extract_topology(ctx.h, _capi.as_ptr(sg), nx, ny, nz,
                                         _capi.ctypes.byref(pr), _capi.ctypes.byref(cnt)))
    return _capi.take_array(pr, 2 * cnt.value, np.int32).reshape(-1, 2)


def pore_network_arrays(sdf: np.ndarray, origin_xyz, spacing_xyz, ctx: Context | None = None):
    a = _sdf_arg(sdf)
    nz, ny, nx = a.shape
    o = np.asarray(origin_xyz, np.float32)
    s = np.asarray(spacing_xyz, np.float32)
    seg = np.empty(a.size, np.int32)
    if a.size == 0:
        return np.zeros((0, 4), np.float32), seg, np.zeros((0, 2), np.int32)
    ctx = ctx or default_context()
    pp = _capi._P(_capi.PnmPore)()
    npp = _capi._i64()
    pr = _capi._P(_capi.ctypes.c_int32)()
    npr = _capi._i64()
    ctx.check(_capi.pnm_extract_pore_network(ctx.h, _capi.as_ptr(a), nx, ny, nz, _capi.as_ptr(o),
                                             _capi.as_ptr(s), _capi.ctypes.byref(pp),
                                             _capi.ctypes.byref(npp), _capi.as_ptr(seg),
                                             _capi.ctypes.byref(pr), _capi.ctypes.byref(npr)))
    pores = _capi.take_array(pp, 4 * npp.value, np.float32).reshape(-1, 4)
    pairs = _capi.take_array(pr, 2 * npr.value, np.int32).reshape(-1, 2)
    return pores, seg, pairs


def network_flow_arrays(sdf, origin_xyz, spacing_xyz, u, v, w, p, ox=None, oy=None, oz=None,
                        grad_p_xyz=(0.0, 0.0, 0.0), ctx: Context | None = None) -> dict:
    a = _sdf_arg(sdf)
    if (ox is None) != (oy is None) or (ox is None) != (oz is None):
        raise RuntimeError("pass all three openness arrays (ox,oy,oz) or none")  # :173-174
    fields = [_field_arg(x, a.shape, nm) for x, nm in ((u, "u"), (v, "v"), (w, "w"), (p, "p"))]
    opn = [None if x is None else _field_arg(x, a.shape, nm)
           for x, nm in ((ox, "ox"), (oy, "oy"), (oz, "oz"))]
    empty = {"pores": np.zeros((0, 4), np.float32), "pore_pressure": np.zeros(0),
             "pore_residual": np.zeros(0), "throats": np.zeros((0, 2), np.int32),
             "throat_flow": np.zeros(0), "throat_area": np.zeros(0), "throat_dp": np.zeros(0)}
    if a.size == 0:
        return empty
    ctx = ctx or default_context()
    nz, ny, nx = a.shape
    o = np.asarray(origin_xyz, np.float32)
    s = np.asarray(spacing_xyz, np.float32)
    g = np.asarray(grad_p_xyz, np.float64)
    res = _capi._P(_capi.PnmFlowResult)()
    ptrs = [_capi.as_ptr(x) for x in fields] + [None if x is None else _capi.as_ptr(x) for x in opn]
    ctx.check(_capi.pnm_extract_network_flow(ctx.h, _capi.as_ptr(a), nx, ny, nz, _capi.as_ptr(o),
                                             _capi.as_ptr(s), *ptrs, _capi.as_ptr(g),
                                             _capi.ctypes.byref(res)))
    r = res.contents
    npo, nt = r.n_pores, r.n_throats

    def grab(ptr, count, dtype):
        if count <= 0:
            return np.zeros((0,), dtype)
        return np.ctypeslib.as_array(_capi.ctypes.cast(ptr, _capi._P(
            np.ctypeslib.as_ctypes_type(dtype))), (int(count),)).copy()

    out = {
        "pores": grab(r.pores, 4 * npo, np.float32).reshape(-1, 4),
        "pore_pressure": grab(r.pore_pressure, npo, np.float64),
        "pore_residual": grab(r.pore_residual, npo, np.float64),
        "throats": grab(r.throats, 2 * nt, np.int32).reshape(-1, 2),
        "throat_flow": grab(r.throat_flow, nt, np.float64),
        "throat_area": grab(r.throat_area, nt, np.float64),
        "throat_dp": grab(r.throat_dp, nt, np.float64),
    }
    _capi.pnm_flow_result_free(res)
    return out


# ---- the reference's Python surface ------------------------------------------------------------
def extract_pores(sdf, origin_zyx, spacing_zyx, *, numpy: bool = False):
    """Pores = strict local SDF maxima (26-neighbour, periodic), centroid-refined."""
    return _pores_out(pores_array(sdf, _xyz32(origin_zyx), _xyz32(spacing_zyx)), numpy)


def segment_volume(sdf, spacing_zyx, *, numpy: bool = False):
    """Flat x-fastest labels: pores 1,2,..., solid -1,-2,..., debris 0."""
    seg = segment_array(sdf, _xyz32(spacing_zyx))
    return seg if numpy else seg.tolist()


def extract_topology_gpu(segmentation, shape, *, numpy: bool = False):
    """Sorted unique (min, max) label pairs across +x/+y/+z periodic faces; shape is zyx."""
    sh = list(shape)
    pairs = topology_array(segmentation, int(sh[2]), int(sh[1]), int(sh[0]))
    return _pairs_out(pairs, numpy)


def extract_pore_network(sdf, origin_zyx, spacing_zyx, *, numpy: bool = False):
    """Fused extraction (SDF uploaded once): (pores, segmentation_flat, connections)."""
    pores, seg, pairs = pore_network_arrays(sdf, _xyz32(origin_zyx), _xyz32(spacing_zyx))
    if numpy:
        return pores, seg, pairs
    return _pores_out(pores, False), seg.tolist(), _pairs_out(pairs, False)


def extract_network_flow(sdf, origin_zyx, spacing_zyx, u, v, w, p, ox=None, oy=None, oz=None,
                         grad_p_zyx=(0.0, 0.0, 0.0), *, numpy: bool = False):
    """Pore-network flow data from a MAC field on the SDF grid (see the reference docstring,
    ``pnm_bindings.cpp:194-208``). Returns the dict of pores, pore_pressure, pore_residual,
    throats, throat_flow, throat_area, throat_dp."""
    gp = list(grad_p_zyx)
    g = [gp[2], gp[1], gp[0]]
    r = network_flow_arrays(sdf, _xyz32(origin_zyx), _xyz32(spacing_zyx), u, v, w, p, ox, oy, oz,
                            g)
    if numpy:
        return r
    return {"pores": _pores_out(r["pores"], False),
            "pore_pressure": r["pore_pressure"].tolist(),
            "pore_residual": r["pore_residual"].tolist(),
            "throats": _pairs_out(r["throats"], False),
            "throat_flow": r["throat_flow"].tolist(),
            "throat_area": r["throat_area"].tolist(),
            "throat_dp": r["throat_dp"].tolist()}
