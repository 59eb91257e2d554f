"""Seeded synthetic SDF volumes and MAC fields for the extraction path.

Every generator returns arrays in the reference's binding layout: ``(Nz, Ny, Nx)`` C-order,
SDF negative inside the solid. Shapes, sizes and value distributions follow the workloads the
reference is exercised on:

* ``ci_lattice``        — the reference CI smoke geometry (``.github/workflows/ci.yml:61-73``):
                          32^3, 2x2x2 solid spheres R=10 at 8/24, non-periodic distance, float32.
* ``sphere_lattice``    — ``sphereLatticeSdf`` of ``tests/kokkos_mpi/test_pnm_mpi.cpp:29-44``
                          (periodic min-image 2x2x2 lattice, R = 0.22 * min(dims)).
* ``trig_field``        — ``trigSdf`` of ``tests/kokkos_mpi/test_pnm_mpi.cpp:46-51``.
* ``mac_fields``        — the ``fld`` fields + openness of ``tests/kokkos_mpi/test_pnm_flow_mpi.cpp:43-56``.
* ``chamber_tube``      — the chamber-tube chain of ``scripts/verify_network_flow.py:23-36``.
* ``capsules``          — case 4 of ``scripts/verify_network_flow.py:196-209``.
* ``random_spheres``    — 64^3 float64, 40 spheres r~U[4,9], plain Euclidean distance (seed 1).
* ``packing``           — polydisperse overlapping spheres, log-normal radii (mean 10,
                          sigma 0.25), periodic min-image SDF, target porosity (boolean model).
* ``fourier_fields``    — u, v, w, p as sums of 32 random Fourier modes (|k| <= 8, amplitude
                          1e-3) zeroed in solid, openness = clamp(0.5 + face SDF, 0, 1).
"""
from __future__ import annotations

import math

import numpy as np


def ci_lattice(n: int = 32, R: float = 10.0) -> np.ndarray:
    z, y, x = np.meshgrid(*(np.arange(n, dtype=np.float32),) * 3, indexing="ij")
    sdf = np.full((n, n, n), np.inf, dtype=np.float32)
    for cz in (8, 24):
        for cy in (8, 24):
            for cx in (8, 24):
                d = np.sqrt((x - cx) ** 2 + (y - cy) ** 2 + (z - cz) ** 2) - R
                sdf = np.minimum(sdf, d.astype(np.float32))
    return np.ascontiguousarray(sdf)


def sphere_lattice(gx: int, gy: int, gz: int) -> np.ndarray:
    """Periodic 2x2x2 lattice of solid spheres; pores at the interstices (float32 math)."""
    R = np.float32(0.22) * np.float32(min(gx, gy, gz))
    z, y, x = np.meshgrid(np.arange(gz, dtype=np.float32), np.arange(gy, dtype=np.float32),
                          np.arange(gx, dtype=np.float32), indexing="ij")
    best = np.full((gz, gy, gx), np.float32(1e30), dtype=np.float32)
    for cz in range(2):
        for cy in range(2):
            for cx in range(2):
                ccx = np.float32(gx * (2 * cx + 1)) / np.float32(4.0)
                ccy = np.float32(gy * (2 * cy + 1)) / np.float32(4.0)
                ccz = np.float32(gz * (2 * cz + 1)) / np.float32(4.0)
                dx = np.abs(x - ccx)
                dy = np.abs(y - ccy)
                dz = np.abs(z - ccz)
                dx = np.minimum(dx, np.float32(gx) - dx)
                dy = np.minimum(dy, np.float32(gy) - dy)
                dz = np.minimum(dz, np.float32(gz) - dz)
                d = np.sqrt(dx * dx + dy * dy + dz * dz) - R
                best = np.minimum(best, d.astype(np.float32))
    return np.ascontiguousarray(best)


def trig_field(gx: int, gy: int, gz: int) -> np.ndarray:
    z, y, x = np.meshgrid(np.arange(gz, dtype=np.float32), np.arange(gy, dtype=np.float32),
                          np.arange(gx, dtype=np.float32), indexing="ij")
    tp = np.float32(2.0 * math.pi)
    X = tp * x / np.float32(gx)
    Y = tp * y / np.float32(gy)
    Z = tp * z / np.float32(gz)
    s = np.sin(X) * np.cos(Y) + np.float32(0.7) * np.sin(np.float32(2.0) * Z) - np.float32(0.1)
    return np.ascontiguousarray(s.astype(np.float32))


def _fld(c: int, x, y, z, gd):
    X = 2.0 * np.pi * x / gd[0]
    Y = 2.0 * np.pi * y / gd[1]
    Z = 2.0 * np.pi * z / gd[2]
    if c == 0:
        return np.sin(X) * np.cos(Y) + 0.3 * np.cos(2 * Z)
    if c == 1:
        return np.cos(X) * np.sin(Z) - 0.2 * np.sin(Y)
    if c == 2:
        return np.sin(Y) * np.sin(Z) + 0.1 * np.cos(X)
    if c == 3:
        return np.cos(X + Y) + 0.5 * np.sin(Z - X)
    s = 0.5 + 0.5 * np.sin(X + 2 * Y - Z)
    return np.where(s < 0.02, 0.0, s)


def mac_fields(gx: int, gy: int, gz: int):
    """(u, v, w, p, ox, oy, oz) float64 (Nz,Ny,Nx); openness fields shifted in x by 4, 5, 6."""
    z, y, x = np.meshgrid(np.arange(gz, dtype=np.float64), np.arange(gy, dtype=np.float64),
                          np.arange(gx, dtype=np.float64), indexing="ij")
    gd = (gx, gy, gz)
    f = [np.ascontiguousarray(_fld(c, x, y, z, gd)) for c in range(4)]
    f += [np.ascontiguousarray(_fld(4, x + c, y, z, gd)) for c in range(4, 7)]
    return tuple(f)


def chamber_tube(NX: int = 48, NY: int = 32, NZ: int = 32, RC: float = 9.0, RT: float = 4.0):
    x, y, z = np.meshgrid(np.arange(NX), np.arange(NY), np.arange(NZ), indexing="ij")
    x = x.astype(np.float64)
    y = y.astype(np.float64)
    z = z.astype(np.float64)
    CY, CZ = NY / 2.0, NZ / 2.0
    sdf = np.full((NX, NY, NZ), -1e30)
    for cx in (12.0, 36.0):
        dx = np.abs(x - cx)
        dx = np.minimum(dx, NX - dx)
        d = np.sqrt(dx ** 2 + (y - CY) ** 2 + (z - CZ) ** 2)
        sdf = np.maximum(sdf, RC - d)
    sdf = np.maximum(sdf, RT - np.sqrt((y - CY) ** 2 + (z - CZ) ** 2))
    return np.ascontiguousarray(sdf.T, dtype=np.float32)


def capsules(NX: int = 48, NY: int = 32, NZ: int = 32):
    x, y, z = np.meshgrid(*(np.arange(d, dtype=np.float64) for d in (NX, NY, NZ)), indexing="ij")
    sdf = np.full((NX, NY, NZ), -1e30)
    for cx in (12.0, 36.0):
        dx = np.abs(x - cx)
        dx = np.minimum(dx, NX - dx)
        sdf = np.maximum(sdf, 8.0 - np.sqrt(dx ** 2 + (y - 16.0) ** 2 + (z - 16.0) ** 2))
    for (cy, rt) in ((12.0, 3.0), (20.0, 4.2)):
        xs = np.clip(x, 12.0, 36.0)
        sdf = np.maximum(sdf, rt - np.sqrt((x - xs) ** 2 + (y - cy) ** 2 + (z - 16.0) ** 2))
    xw = np.where(x < 12.0, x + NX, x)
    xs = np.clip(xw, 36.0, 12.0 + NX)
    sdf = np.maximum(sdf, 4.0 - np.sqrt((xw - xs) ** 2 + (y - 16.0) ** 2 + (z - 16.0) ** 2))
    return np.ascontiguousarray(sdf.T, dtype=np.float32)


def random_spheres(n: int = 64, count: int = 40, rmin: float = 4.0, rmax: float = 9.0,
                   seed: int = 1) -> np.ndarray:
    """float64 SDF = min_i(|x - c_i| - r_i), plain (non-periodic) Euclidean distance."""
    rng = np.random.default_rng(seed)
    c = rng.uniform(0.0, n, size=(count, 3))
    r = rng.uniform(rmin, rmax, size=count)
    z, y, x = np.meshgrid(*(np.arange(n, dtype=np.float64),) * 3, indexing="ij")
    sdf = np.full((n, n, n), np.inf)
    for (cx, cy, cz), ri in zip(c, r):
        sdf = np.minimum(sdf, np.sqrt((x - cx) ** 2 + (y - cy) ** 2 + (z - cz) ** 2) - ri)
    return np.ascontiguousarray(sdf)


def packing_spheres(shape_zyx, porosity: float = 0.4, mean_r: float = 10.0, sigma: float = 0.25,
                    seed: int = 2):
    """Sphere centres (x, y, z) and radii of a boolean-model packing of the given porosity."""
    nz, ny, nx = shape_zyx
    rng = np.random.default_rng(seed)
    mu = math.log(mean_r) - sigma * sigma / 2.0
    er3 = math.exp(3 * mu + 4.5 * sigma * sigma)
    ev = 4.0 / 3.0 * math.pi * er3
    count = max(1, int(round(-math.log(porosity) / ev * nx * ny * nz)))
    c = rng.uniform(0.0, 1.0, size=(count, 3)) * np.array([nx, ny, nz], np.float64)
    r = rng.lognormal(mu, sigma, size=count)
    return c, r


def packing(shape_zyx, porosity: float = 0.4, mean_r: float = 10.0, sigma: float = 0.25,
            seed: int = 2, dtype=np.float32, device: str | None = None, reach: float = 32.0):
    """Periodic polydisperse overlapping-sphere packing SDF (negative inside the spheres).

    The SDF is min_i(|x - c_i|_minimage - r_i), evaluated exactly for every voxel within
    ``reach`` of a sphere surface (every sphere splats into its own box of half-width r + reach);
    the generator checks that no voxel lies farther than that from all surfaces. With
    ``device`` set (e.g. "cuda") the splat runs in torch on that device and a torch tensor is
    returned; otherwise numpy on the host.
    """
    nz, ny, nx = (int(v) for v in shape_zyx)
    c, r = packing_spheres((nz, ny, nx), porosity, mean_r, sigma, seed)
    M = int(math.ceil(float(r.max()) + reach)) + 2
    if device is not None:
        import torch
        tdt = torch.float64 if dtype == np.float64 else torch.float32
        vol = torch.full((nz + 2 * M, ny + 2 * M, nx + 2 * M), float("inf"), dtype=tdt,
                         device=device)
        for (cx, cy, cz), ri in zip(c, r):
            h = int(math.ceil(ri + reach))
            ix0, iy0, iz0 = int(math.floor(cx)) - h, int(math.floor(cy)) - h, int(math.floor(cz)) - h
            ax = torch.arange(ix0, ix0 + 2 * h + 2, dtype=tdt, device=device) - cx
            ay = torch.arange(iy0, iy0 + 2 * h + 2, dtype=tdt, device=device) - cy
            az = torch.arange(iz0, iz0 + 2 * h + 2, dtype=tdt, device=device) - cz
            d = torch.sqrt(az[:, None, None] ** 2 + ay[None, :, None] ** 2 + ax[None, None, :] ** 2) - ri
            box = vol[iz0 + M:iz0 + M + 2 * h + 2, iy0 + M:iy0 + M + 2 * h + 2,
                      ix0 + M:ix0 + M + 2 * h + 2]
            torch.minimum(box, d, out=box)
        out = _fold_periodic_torch(vol, M, (nz, ny, nx))
        if torch.isinf(out).any() or float(out.max()) >= reach - 1.0:
            raise RuntimeError("packing: a voxel lies beyond the splat reach; raise `reach`")
        return out.contiguous()
    vol = np.full((nz + 2 * M, ny + 2 * M, nx + 2 * M), np.inf, dtype=dtype)
    for (cx, cy, cz), ri in zip(c, r):
        h = int(math.ceil(ri + reach))
        ix0, iy0, iz0 = int(math.floor(cx)) - h, int(math.floor(cy)) - h, int(math.floor(cz)) - h
        ax = np.arange(ix0, ix0 + 2 * h + 2, dtype=np.float64) - cx
        ay = np.arange(iy0, iy0 + 2 * h + 2, dtype=np.float64) - cy
        az = np.arange(iz0, iz0 + 2 * h + 2, dtype=np.float64) - cz
        d = (np.sqrt(az[:, None, None] ** 2 + ay[None, :, None] ** 2 + ax[None, None, :] ** 2)
             - ri).astype(dtype)
        box = vol[iz0 + M:iz0 + M + 2 * h + 2, iy0 + M:iy0 + M + 2 * h + 2,
                  ix0 + M:ix0 + M + 2 * h + 2]
        np.minimum(box, d, out=box)
    out = _fold_periodic_np(vol, M, (nz, ny, nx))
    if not np.isfinite(out).all() or float(out.max()) >= reach - 1.0:
        raise RuntimeError("packing: a voxel lies beyond the splat reach; raise `reach`")
    return np.ascontiguousarray(out)


def _fold_periodic_np(vol, M, shape):
    nz, ny, nx = shape
    for ax, n in ((0, nz), (1, ny), (2, nx)):
        v = np.moveaxis(vol, ax, 0)
        core = v[M:M + n].copy()
        # every padded plane p folds onto core plane (p - M) mod n
        idx = (np.arange(v.shape[0]) - M) % n
        for p in range(v.shape[0]):
            if M <= p < M + n:
                continue
            np.minimum(core[idx[p]], v[p], out=core[idx[p]])
        vol = np.moveaxis(core, 0, ax)
    return vol


def _fold_periodic_torch(vol, M, shape):
    import torch
    nz, ny, nx = shape
    for ax, n in ((0, nz), (1, ny), (2, nx)):
        v = vol.movedim(ax, 0)
        core = v[M:M + n].clone()
        P = v.shape[0]
        for p in range(P):
            if M <= p < M + n:
                continue
            q = (p - M) % n
            torch.minimum(core[q], v[p], out=core[q])
        vol = core.movedim(0, ax)
    return vol


def fourier_fields(sdf_zyx: np.ndarray, modes: int = 32, kmax: int = 8, amplitude: float = 1e-3,
                   seed: int = 4):
    """(u, v, w, p, ox, oy, oz) float64 (Nz,Ny,Nx) on the SDF's grid.

    u, v, w, p: each a sum of ``modes`` modes amp * dir * sin(2 pi k.x / N + phase) with integer
    wavevectors 0 < |k| <= kmax, random phases, random unit directions (velocities) and
    amplitude ``amplitude``; zeroed where the cell's sdf <= 0. Openness o_d at the -d face of cell
    i is clamp(0.5 + (sdf[i - e_d] + sdf[i]) / 2, 0, 1) with periodic wrap.
    """
    sdf = np.asarray(sdf_zyx, np.float64)
    nz, ny, nx = sdf.shape
    rng = np.random.default_rng(seed)
    z = np.arange(nz, dtype=np.float64)[:, None, None] / nz
    y = np.arange(ny, dtype=np.float64)[None, :, None] / ny
    x = np.arange(nx, dtype=np.float64)[None, None, :] / nx

    def one(is_vec_comp: bool):
        acc = np.zeros((nz, ny, nx))
        m = 0
        while m < modes:
            k = rng.integers(-kmax, kmax + 1, size=3)
            if not (0 < np.sqrt((k * k).sum()) <= kmax):
                continue
            ph = rng.uniform(0.0, 2 * np.pi)
            a = amplitude * (rng.normal() if is_vec_comp else 1.0)
            acc += a * np.sin(2 * np.pi * (k[0] * x + k[1] * y + k[2] * z) + ph)
            m += 1
        return acc

    solid = sdf <= 0.0
    out = []
    for comp in range(4):
        f = one(comp < 3)
        f[solid] = 0.0
        out.append(np.ascontiguousarray(f))
    for ax in (2, 1, 0):  # x, y, z faces
        face = 0.5 * (np.roll(sdf, 1, axis=ax) + sdf)
        out.append(np.ascontiguousarray(np.clip(0.5 + face, 0.0, 1.0)))
    return tuple(out)


def fourier_fields_device(sdf, modes: int = 32, kmax: int = 8, amplitude: float = 1e-3,
                          seed: int = 4):
    """fourier_fields evaluated in torch on the SDF tensor's device (float64): the same modes,
    phases and directions (same random stream), for volumes where the host version is slow."""
    import torch

    dev = sdf.device
    sdf = sdf.to(torch.float64)
    nz, ny, nx = sdf.shape
    rng = np.random.default_rng(seed)
    z = torch.arange(nz, dtype=torch.float64, device=dev)[:, None, None] / nz
    y = torch.arange(ny, dtype=torch.float64, device=dev)[None, :, None] / ny
    x = torch.arange(nx, dtype=torch.float64, device=dev)[None, None, :] / nx

    def one(is_vec_comp: bool):
        acc = torch.zeros((nz, ny, nx), dtype=torch.float64, device=dev)
        m = 0
        while m < modes:
            k = rng.integers(-kmax, kmax + 1, size=3)
            if not (0 < np.sqrt((k * k).sum()) <= kmax):
                continue
            ph = rng.uniform(0.0, 2 * np.pi)
            a = amplitude * (rng.normal() if is_vec_comp else 1.0)
            acc += a * torch.sin(2 * np.pi * (float(k[0]) * x + float(k[1]) * y + float(k[2]) * z)
                                 + ph)
            m += 1
        return acc

    solid = sdf <= 0.0
    out = []
    for comp in range(4):
        f = one(comp < 3)
        f[solid] = 0.0
        out.append(f.contiguous())
    for ax in (2, 1, 0):
        face = 0.5 * (torch.roll(sdf, 1, dims=ax) + sdf)
        out.append(torch.clamp(0.5 + face, 0.0, 1.0).contiguous())
    return tuple(out)


def batch_shapes(count: int = 96, edges=(48, 64, 96, 128, 160, 192), seed: int = 5):
    """Per-volume (nz, ny, nx) and porosity of the ragged batch: edges drawn per axis, seed+i."""
    out = []
    for i in range(count):
        rng = np.random.default_rng(seed + i)
        e = rng.choice(np.asarray(edges), size=3)
        phi = float(rng.uniform(0.3, 0.6))
        out.append(((int(e[2]), int(e[1]), int(e[0])), phi, seed + i))
    return out
