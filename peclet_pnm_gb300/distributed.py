"""The reference's distributed extraction surface as volume-split replicas over torch.distributed.

The reference builds ``mpi_rank``, ``mpi_size``, ``mpi_block``, ``extract_pore_network_mpi`` and
``extract_network_flow_mpi`` when compiled with MPI (``src/pnm_bindings.cpp:211-317``): the grid is
decomposed over the ranks, each rank passes its block, and a halo-exchanging pipeline
(``src/pore_extraction_mpi.hpp``) returns results bit-exact to the single-rank path on the
gathered grid.

Here a single volume does not shard (the marker CCL, the flood fixpoint and the first-appearance
renumbering are global over the grid), so the same functions run as replicas: every rank gathers
all blocks (one all-gather of the SDF, and of the MAC fields for network flow), runs the
single-GPU pipeline on the whole grid on its own GPU, and returns what the reference returns to
that rank:

* ``extract_pore_network_mpi``: the pores whose peak voxel lies in this rank's block (voxel
  order), the flat labels of this rank's block, and the global connection list;
* ``extract_network_flow_mpi``: the global result dict, identical on every rank.

Results are therefore bit-identical to ``extract_pore_network`` / ``extract_network_flow`` on the
gathered grid, the reference's own guarantee. The decomposition differs from the reference's:
its blocks come from peclet-core's ORB ``BlockDecomposer``, which is not part of the reference
checkout; here rank r owns a z-slab of whole planes (slab sizes differ by at most one plane), so
callers take their block from :func:`mpi_block` of this module. Outside an initialised
torch.distributed process group the functions act as one rank owning the whole grid.
"""
from __future__ import annotations

import numpy as np

__all__ = ["mpi_rank", "mpi_size", "mpi_block", "extract_pore_network_mpi",
           "extract_network_flow_mpi"]


def _dist():
    try:
        import torch.distributed as dist
    except ImportError:  # pragma: no cover - torch is a dependency of the package
        return None
    return dist if dist.is_available() and dist.is_initialized() else None


def mpi_rank() -> int:
    """This rank's index in the process group (0 without one)."""
    d = _dist()
    return d.get_rank() if d else 0


def mpi_size() -> int:
    """Number of ranks in the process group (1 without one)."""
    d = _dist()
    return d.get_world_size() if d else 1


def _slab(nz: int, rank: int, size: int):
    base, extra = divmod(nz, size)
    z0 = rank * base + min(rank, extra)
    return z0, base + (1 if rank < extra else 0)


def mpi_block(global_shape_zyx, rank: int | None = None, size: int | None = None):
    """This rank's block of the global grid: (origin_zyx, shape_zyx), a z-slab of whole planes.
    Slice the global SDF with these and pass the block to the *_mpi functions."""
    nz, ny, nx = (int(v) for v in global_shape_zyx)
    r = mpi_rank() if rank is None else int(rank)
    s = mpi_size() if size is None else int(size)
    z0, dz = _slab(nz, r, s)
    return [z0, 0, 0], [dz, ny, nx]


def _check_block(a, global_shape_zyx, name):
    o, shp = mpi_block(global_shape_zyx)
    if tuple(a.shape) != tuple(shp):
        raise RuntimeError(f"{name} shape does not match this rank's mpi_block")


def _gather(local, global_shape_zyx, dtype):
    """The global array from every rank's z-slab (all-gather, padded to the largest slab)."""
    import torch

    a = np.ascontiguousarray(np.asarray(local), dtype=dtype)
    d = _dist()
    if d is None:
        return a
    nz, ny, nx = (int(v) for v in global_shape_zyx)
    size = d.get_world_size()
    plane = ny * nx
    most = max(_slab(nz, r, size)[1] for r in range(size)) * plane
    dev = torch.device("cuda", torch.cuda.current_device()) \
        if d.get_backend() == "nccl" else torch.device("cpu")
    buf = torch.zeros(max(most, 1), dtype=torch.from_numpy(a[:0].reshape(-1)).dtype, device=dev)
    buf[:a.size] = torch.from_numpy(a.reshape(-1)).to(dev)
    parts = [torch.empty_like(buf) for _ in range(size)]
    d.all_gather(parts, buf)
    out = [parts[r][:_slab(nz, r, size)[1] * plane].cpu().numpy() for r in range(size)]
    return np.concatenate(out).reshape(nz, ny, nx)


def _network_gpu(sdf, origin_zyx, spacing_zyx):
    """(pores (n,4) float32, peak voxel ids (n,), flat labels, pairs (m,2)) of the whole grid on
    this rank's GPU."""
    import ctypes

    import torch

    from . import _capi
    from . import extract_pore_network

    pores, seg, pairs = extract_pore_network(sdf, origin_zyx, spacing_zyx, numpy=True)
    ctx = _capi.default_context()
    d_sdf = torch.from_numpy(np.ascontiguousarray(sdf, np.float32)).cuda()
    d_ids = torch.empty(max(len(pores), 1), dtype=torch.int32, device="cuda")
    n = _capi._i64()
    nz, ny, nx = sdf.shape
    torch.cuda.synchronize()
    ctx.check(_capi.pnm_pore_peaks_dev(ctx.h, d_sdf.data_ptr(), nx, ny, nz, d_ids.data_ptr(),
                                       len(pores), ctypes.byref(n)))
    return pores, d_ids[:n.value].cpu().numpy(), seg, pairs


def extract_pore_network_mpi(sdf_local, global_shape_zyx, origin_zyx, spacing_zyx, *,
                             numpy: bool = False, _compute=None):
    """Replica of the reference's distributed fused extraction (collective over the group).
    sdf_local is this rank's block (from mpi_block). Returns (pores whose peak voxel this rank's
    block holds, flat labels of this rank's block, global connections); every part equals the
    single-rank extract_pore_network on the gathered grid."""
    from . import _pairs_out, _pores_out

    a = np.asarray(sdf_local)
    if a.ndim != 3:
        raise RuntimeError("SDF array must be 3D (Nz,Ny,Nx)")
    _check_block(a, global_shape_zyx, "sdf_local")
    sdf = _gather(a, global_shape_zyx, np.float32)
    pores, peaks, seg, pairs = (_compute or _network_gpu)(sdf, origin_zyx, spacing_zyx)
    (z0, _, _), (dz, ny, nx) = mpi_block(global_shape_zyx)
    plane = ny * nx
    own = (peaks // plane >= z0) & (peaks // plane < z0 + dz)
    mine = np.asarray(pores, np.float32).reshape(-1, 4)[own]
    seg_local = np.asarray(seg).reshape(-1)[z0 * plane:(z0 + dz) * plane]
    if numpy:
        return mine, seg_local, np.asarray(pairs).reshape(-1, 2)
    return _pores_out(mine, False), seg_local.tolist(), _pairs_out(np.asarray(pairs), False)


def extract_network_flow_mpi(sdf_local, global_shape_zyx, origin_zyx, spacing_zyx, u, v, w, p,
                             ox=None, oy=None, oz=None, grad_p_zyx=(0.0, 0.0, 0.0), *,
                             numpy: bool = False, _compute=None):
    """Replica of the reference's distributed network-flow extraction (collective): every array
    is this rank's block; the returned dict is the global result, identical on every rank."""
    from . import extract_network_flow

    a = np.asarray(sdf_local)
    if a.ndim != 3:
        raise RuntimeError("SDF array must be 3D (Nz,Ny,Nx)")
    _check_block(a, global_shape_zyx, "sdf_local")
    if (ox is None) != (oy is None) or (ox is None) != (oz is None):
        raise RuntimeError("pass all three openness arrays (ox,oy,oz) or none")
    fields = {}
    for name, f in (("u", u), ("v", v), ("w", w), ("p", p), ("ox", ox), ("oy", oy), ("oz", oz)):
        if f is None:
            continue
        f = np.asarray(f)
        if f.shape != a.shape:
            raise RuntimeError(f"{name} must be (Nz,Ny,Nx) matching the SDF")
        fields[name] = _gather(f, global_shape_zyx, np.float64)
    sdf = _gather(a, global_shape_zyx, np.float32)
    run = _compute or (lambda *args, **kw: extract_network_flow(*args, numpy=numpy, **kw))
    return run(sdf, origin_zyx, spacing_zyx, fields["u"], fields["v"], fields["w"], fields["p"],
               ox=fields.get("ox"), oy=fields.get("oy"), oz=fields.get("oz"),
               grad_p_zyx=grad_p_zyx)
