"""Seeded parity cases shared by the oracle tests (CPU) and the GPU parity tests.

Each case is (name, sdf (Nz,Ny,Nx) float32, origin_zyx, spacing_zyx). They cover the edge cases
the reference's semantics hinge on: periodic wrap aliasing on dims 1-3, plateaus and ties broken
by the wrapped index, sdf == 0 debris, NaN / inf values, all-pore / all-solid volumes, gradient
walks longer than the 512-step cap, and flood wavefronts many layers deep.
"""
from __future__ import annotations

import numpy as np

from peclet_pnm_gb300 import synthetic as syn

UNIT = ([0.0, 0.0, 0.0], [1.0, 1.0, 1.0])


def _tent(n):
    x = np.arange(n, dtype=np.float32)
    return (np.float32(1.0) + np.minimum(x, np.float32(n) - x)).astype(np.float32)


def edge_cases():
    rng = np.random.default_rng(11)
    out = []
    for shp in [(1, 1, 1), (1, 1, 2), (2, 2, 2), (1, 3, 5), (3, 1, 4), (2, 5, 3), (4, 4, 1),
                (3, 3, 3), (1, 7, 9), (5, 2, 6)]:
        a = rng.normal(0.0, 2.0, size=shp).astype(np.float32)
        out.append((f"tiny_{'x'.join(map(str, shp))}", a, *UNIT))
    # plateaus: integer-valued SDF, ties everywhere
    pk = syn.packing((24, 20, 28), 0.45, mean_r=5.0, seed=21)
    out.append(("plateau_floor", np.floor(pk).astype(np.float32), *UNIT))
    out.append(("plateau_round_half", (np.round(pk * 2) / 2).astype(np.float32), *UNIT))
    # constant volumes
    out.append(("all_pore_const", np.ones((6, 5, 7), np.float32), *UNIT))
    out.append(("all_marker_const", np.full((5, 6, 4), -5.0, np.float32), *UNIT))
    out.append(("all_flood_const", np.full((4, 5, 6), -0.5, np.float32), *UNIT))
    out.append(("all_zero", np.zeros((5, 4, 6), np.float32), *UNIT))
    # sdf == 0 band: debris
    z = pk.copy()
    z[np.abs(z) < 0.8] = 0.0
    out.append(("zero_band", z.astype(np.float32), *UNIT))
    # NaN / inf sprinkled
    q = syn.packing((16, 18, 20), 0.4, mean_r=4.0, seed=22).astype(np.float32)
    idx = rng.choice(q.size, size=40, replace=False)
    q.reshape(-1)[idx[:15]] = np.nan
    q.reshape(-1)[idx[15:28]] = np.inf
    q.reshape(-1)[idx[28:]] = -np.inf
    out.append(("nan_inf", q, *UNIT))
    # gradient walks longer than 512 steps (a 1-D tent: the ascent from x=1 needs ~600 moves)
    out.append(("walk_cap_line", _tent(1200).reshape(1, 1, 1200), *UNIT))
    out.append(("walk_cap_plateau", np.ones((1, 1, 700), np.float32), *UNIT))
    out.append(("walk_cap_2d", np.tile(_tent(1100), (2, 1)).reshape(1, 2, 1100), *UNIT))
    # deep flood: a floodable serpentine sheet fed by one marker blob (many BFS layers)
    s = np.full((6, 40, 40), 2.0, np.float32)
    s[2:4, :, :] = -0.5
    s[2:4, ::4, 5:] = 2.0
    s[2:4, 2::4, :35] = 2.0
    s[1:5, 0:3, 0:3] = -4.0
    out.append(("deep_flood_serpentine", s, *UNIT))
    # adversarial marker patterns for the CCL edge lists: runs of length one everywhere
    zz, yy, xx = np.meshgrid(np.arange(20), np.arange(18), np.arange(40), indexing="ij")
    chk = np.where((xx + yy + zz) % 2 == 0, -3.0, 0.75).astype(np.float32)
    out.append(("checker_markers", chk, *UNIT))
    rm = np.where(rng.random((24, 20, 70)) < 0.5, -3.0, 1.0).astype(np.float32)
    rm += rng.uniform(0, 0.01, size=rm.shape).astype(np.float32)
    out.append(("random_markers", rm, *UNIT))
    # random noise (many tiny components) with anisotropic spacing and an origin
    out.append(("noise_16_aniso", rng.normal(0.0, 1.5, size=(16, 17, 18)).astype(np.float32),
                [0.25, -3.0, 7.5], [0.7, 1.3, 2.1]))
    # thin spacing: marker threshold scales with min spacing
    out.append(("packing_fine_spacing", pk.astype(np.float32) * 0.1, [0.0, 0.0, 0.0],
                [0.1, 0.1, 0.25]))
    # walks longer than the cap in volumes of three or more voxels per axis (ties across the
    # short axes), along x and along z
    out.append(("walk_cap_3d_x", np.tile(_tent(1300), (3, 3, 1)), *UNIT))
    out.append(("walk_cap_3d_z", np.tile(_tent(1300)[:, None, None], (1, 3, 3)), *UNIT))
    out.append(("serpentine_walk", _serpentine(), *UNIT))
    return out


def _serpentine():
    """A pore path snaking through rows y = 1, 3, 5 of a 32-voxel-wide block between walls: the
    ascent from its start makes ~90 moves without leaving a 32 x 8 x 16 block."""
    s = np.full((3, 8, 40), -2.0, np.float32)
    cells = [(1, x) for x in range(1, 31)] + [(2, 30)] + [(3, x) for x in range(30, 0, -1)]
    cells += [(4, 1)] + [(5, x) for x in range(1, 31)]
    for p, (y, x) in enumerate(cells):
        s[:, y, x] = np.float32(1.0 + 0.01 * p)
    return s


def standard_cases():
    return [
        ("ci_lattice", syn.ci_lattice(), *UNIT),
        ("sphere_lattice_36x30x24", syn.sphere_lattice(36, 30, 24), *UNIT),
        ("trig_32_aniso", syn.trig_field(32, 32, 32), [0.5, 2.0, -1.0], [2.0, 1.0, 0.5]),
        ("random_spheres_64", syn.random_spheres().astype(np.float32), *UNIT),
        ("chamber_tube", syn.chamber_tube(), *UNIT),
        ("capsules", syn.capsules(), *UNIT),
        ("packing_40x48x56", syn.packing((40, 48, 56), 0.4, seed=7), *UNIT),
    ]


def flow_fields(sdf, seed=5):
    """Random-normal MAC fields (u, v, w, p) and openness in [0, 1] with exact zeros."""
    rng = np.random.default_rng(seed)
    sh = sdf.shape
    f = [np.ascontiguousarray(rng.normal(0.0, 1e-3, size=sh)) for _ in range(4)]
    o = []
    for _ in range(3):
        x = rng.uniform(-0.3, 1.0, size=sh)
        o.append(np.ascontiguousarray(np.clip(x, 0.0, 1.0)))
    return f + o


def random_volume(seed):
    """A seeded volume of random shape (1..20 per axis) from one of four value families: smooth
    noise, values quantised to a few levels (plateaus and ties), a marker-heavy field and a
    packing with noise; spacing anisotropic and origin offset at random."""
    rng = np.random.default_rng(1000 + seed)
    shp = tuple(int(v) for v in rng.integers(1, 21, size=3))
    kind = seed % 4
    if kind == 0:
        a = rng.normal(0.0, 2.0, size=shp)
    elif kind == 1:
        a = np.round(rng.normal(0.0, 1.5, size=shp) * 2.0) / 2.0
    elif kind == 2:
        a = np.where(rng.random(shp) < 0.6, -3.0, rng.uniform(-1.0, 2.0, size=shp))
    else:
        a = syn.packing(tuple(max(4, s) for s in shp), 0.4, mean_r=2.5, seed=seed)
        a = a + rng.normal(0.0, 0.1, size=a.shape)
    spc = [float(v) for v in rng.uniform(0.5, 2.0, size=3)]
    org = [float(v) for v in rng.uniform(-5.0, 5.0, size=3)]
    return np.ascontiguousarray(a, dtype=np.float32), org, spc
