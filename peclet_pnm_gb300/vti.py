"""VTI (VTK ImageData) ingest and output for the extraction path.

* :class:`SDFReader` — ``SDFReader.read_vti(filename) -> (sdf (Nz,Ny,Nx) float32, origin_zyx,
  spacing_zyx)``, the reference binding (``src/pnm_bindings.cpp:87-102``) over the native reader
  ``pnm_read_vti`` (semantics of ``src/sdf_reader.cpp:28-152``). ``read_vti_device`` streams the
  values straight into a device buffer through ``pnm_read_vti_dev``.
* :func:`save_vti` — the reference's general field writer (``scripts/vti.py:10-80``): CellData
  arrays, ``WholeExtent="0 nx 0 ny 0 nz"``, Int32 / Float64 / Float32, appended raw with a UInt64
  byte count before each array.
* :func:`write_sdf_vti` — the input layout ``read_vti`` expects (PointData, one Float32 array,
  ``WholeExtent="0 nx-1 0 ny-1 0 nz-1"``), so volumes can be written and read back unchanged.
* :func:`write_edge_list` — one ``"u v"`` line per connection (``scripts/verify_segmentation.py:
  49-51``).
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import _capi
from ._capi import Context, PnmError, default_context

__all__ = ["SDFReader", "read_vti_header", "read_vti_device", "save_vti", "write_sdf_vti",
           "write_edge_list"]


def _path(filename) -> bytes:
    return os.fsencode(os.fspath(filename))


def _vti_check(rc: int):
    if rc != _capi.PNM_OK:
        raise RuntimeError(_capi.pnm_vti_last_error().decode(errors="replace")
                           or f"pnm vti error {rc}")


def read_vti_header(filename) -> dict:
    """Header fields: ``dims_xyz``, ``origin_xyz``, ``spacing_xyz`` (float32 as parsed) and
    ``data_bytes`` (the byte count stored before the first appended array)."""
    d = np.zeros(3, np.int32)
    o = np.zeros(3, np.float32)
    s = np.zeros(3, np.float32)
    nb = _capi._i64()
    _vti_check(_capi.pnm_read_vti_header(_path(filename), _capi.as_ptr(d), _capi.as_ptr(o),
                                         _capi.as_ptr(s), ctypes.byref(nb)))
    return {"dims_xyz": tuple(int(v) for v in d), "origin_xyz": o, "spacing_xyz": s,
            "data_bytes": int(nb.value)}


def _zyx(v_xyz) -> list:
    return [float(v_xyz[2]), float(v_xyz[1]), float(v_xyz[0])]


class SDFReader:
    """``peclet.pnm.SDFReader`` (``src/sdf_reader.h``)."""

    @staticmethod
    def read_vti(filename):
        """Returns ``(sdf_3d (Nz,Ny,Nx) float32, origin_zyx, spacing_zyx)``; origin and spacing
        are the float32 header values as Python floats, like the binding's double lists."""
        h = read_vti_header(filename)
        nx, ny, nz = h["dims_xyz"]
        if nx < 0 or ny < 0 or nz < 0:
            raise RuntimeError("negative extent in VTI header")
        sdf = np.empty((nz, ny, nx), np.float32)
        _vti_check(_capi.pnm_read_vti(_path(filename), _capi.as_ptr(sdf), sdf.size))
        return sdf, _zyx(h["origin_xyz"]), _zyx(h["spacing_xyz"])


def read_vti_device(filename, out=None, *, ctx: Context | None = None):
    """Reads the values into device memory without a host-side copy of the volume.

    `out` is a contiguous float32 CUDA tensor with at least Nz*Ny*Nx elements; when omitted a
    ``torch`` tensor of shape (Nz,Ny,Nx) is allocated on the context's device. Returns
    ``(out, origin_zyx, spacing_zyx)``.
    The copy runs on the context's stream and is complete when this returns."""
    import torch

    h = read_vti_header(filename)
    nx, ny, nz = h["dims_xyz"]
    if nx < 0 or ny < 0 or nz < 0:
        raise RuntimeError("negative extent in VTI header")
    n = nx * ny * nz
    if out is not None:
        if not (isinstance(out, torch.Tensor) and out.is_cuda and out.dtype == torch.float32
                and out.is_contiguous()):
            raise RuntimeError("out must be a contiguous float32 CUDA tensor")
        if int(out.numel()) < n:
            raise RuntimeError(f"device buffer holds {int(out.numel())} values, the file {n}")
    ctx = ctx or default_context()
    if out is None:
        dev = ctx.device if ctx.device is not None else torch.cuda.current_device()
        out = torch.empty((nz, ny, nx), dtype=torch.float32, device=f"cuda:{dev}")
    rc = _capi.pnm_read_vti_dev(ctx.h, _path(filename), ctypes.c_void_p(out.data_ptr()), n)
    if rc != _capi.PNM_OK:
        raise PnmError(rc, _capi.pnm_last_error(ctx.h).decode(errors="replace"))
    return out, _zyx(h["origin_xyz"]), _zyx(h["spacing_xyz"])


def save_vti(filename, fields, spacing=(1.0, 1.0, 1.0), origin=(0.0, 0.0, 0.0)):
    """Writes `fields` ({name: (Nz,Ny,Nx) or (Nz,Ny,Nx,3) array}) as CellData of one ImageData
    piece; `spacing` and `origin` are zyx. Byte-for-byte the layout of the reference writer."""
    first = next(iter(fields.values()))
    shape = tuple(first.shape[:3])
    nz, ny, nx = shape
    dz, dy, dx = spacing
    oz, oy, ox = origin
    arrays = []
    head = [b'<?xml version="1.0"?>\n',
            b'<VTKFile type="ImageData" version="1.0" byte_order="LittleEndian" '
            b'header_type="UInt64">\n',
            f'  <ImageData WholeExtent="0 {nx} 0 {ny} 0 {nz}" Origin="{ox} {oy} {oz}" '
            f'Spacing="{dx} {dy} {dz}">\n'.encode("ascii"),
            f'    <Piece Extent="0 {nx} 0 {ny} 0 {nz}">\n'.encode("ascii"),
            b'      <CellData>\n']
    offset = 0
    for name, arr in fields.items():
        arr = np.asarray(arr)
        if tuple(arr.shape[:3]) != shape:
            raise ValueError(f"Field '{name}' shape {arr.shape} inconsistent with {shape}")
        if np.issubdtype(arr.dtype, np.integer):
            kind, fixed = "Int32", arr.astype("<i4")
        elif arr.dtype == np.float64:
            kind, fixed = "Float64", arr.astype("<f8")
        else:
            kind, fixed = "Float32", arr.astype("<f4")
        comps = 3 if arr.ndim == 4 else 1
        head.append(f'        <DataArray type="{kind}" Name="{name}" NumberOfComponents="{comps}"'
                    f' format="appended" offset="{offset}"/>\n'.encode("ascii"))
        arrays.append(fixed)
        offset += fixed.nbytes + 8
    head.append(b'      </CellData>\n    </Piece>\n  </ImageData>\n')
    head.append(b'  <AppendedData encoding="raw">\n_')
    with open(filename, "wb") as f:
        f.writelines(head)
        for a in arrays:
            raw = np.ascontiguousarray(a)
            f.write(np.array([raw.nbytes], "<u8").tobytes())
            raw.tofile(f)
        f.write(b'\n  </AppendedData>\n</VTKFile>\n')


def write_sdf_vti(filename, sdf, origin_zyx=(0.0, 0.0, 0.0), spacing_zyx=(1.0, 1.0, 1.0),
                  name: str = "sdf"):
    """Writes a (Nz,Ny,Nx) SDF as one Float32 PointData array in the layout
    :meth:`SDFReader.read_vti` reads back unchanged (extent 0..n-1 per axis)."""
    a = np.ascontiguousarray(np.asarray(sdf), dtype="<f4")
    if a.ndim != 3:
        raise RuntimeError("SDF array must be 3D (Nz,Ny,Nx)")
    nz, ny, nx = a.shape
    ext = f"0 {nx - 1} 0 {ny - 1} 0 {nz - 1}"
    oz, oy, ox = (float(v) for v in origin_zyx)
    dz, dy, dx = (float(v) for v in spacing_zyx)
    with open(filename, "wb") as f:
        f.write(b'<?xml version="1.0"?>\n'
                b'<VTKFile type="ImageData" version="1.0" byte_order="LittleEndian" '
                b'header_type="UInt64">\n')
        f.write(f'  <ImageData WholeExtent="{ext}" Origin="{ox!r} {oy!r} {oz!r}" '
                f'Spacing="{dx!r} {dy!r} {dz!r}">\n    <Piece Extent="{ext}">\n'
                f'      <PointData Scalars="{name}">\n        <DataArray type="Float32" '
                f'Name="{name}" NumberOfComponents="1" format="appended" offset="0"/>\n'
                f'      </PointData>\n    </Piece>\n  </ImageData>\n'.encode("ascii"))
        f.write(b'  <AppendedData encoding="raw">\n_')
        f.write(np.array([a.nbytes], "<u8").tobytes())
        a.tofile(f)
        f.write(b'\n  </AppendedData>\n</VTKFile>\n')


def write_edge_list(filename, connections):
    """One ``"u v"`` line per (u, v) connection."""
    pairs = np.asarray(connections, dtype=np.int64).reshape(-1, 2)
    with open(filename, "w") as f:
        f.writelines(f"{u} {v}\n" for u, v in pairs.tolist())
