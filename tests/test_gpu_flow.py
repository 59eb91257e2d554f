"""GPU parity of extract_network_flow against the CPU oracle and the reference goldens.

Bar: throat list (order included) exact; pores and pore_pressure bitwise (per-pore fixed-order
arithmetic without contraction); throat_dp within 1e-12 relative; the FP64 sums per element:
throat_area (a sum of non-negative terms) within 1e-12 relative, throat_flow and pore_residual
(cancelling sums) within 1e-12 of max(|oracle value|, sum of |terms|), the sum of |q| over that
element's own faces, which the oracle reports. The GPU sums exactly (128-bit fixed point); the
oracle's double sums carry order-dependent rounding of at most (terms - 1) * 2^-53 of that scale.
"""
import os

import numpy as np
import pytest

from cases import edge_cases, flow_fields, standard_cases
from peclet_pnm_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
TOL = 1e-12


def check_sums(r, o, scales):
    """Per-element tolerance of the FP64 sums. scales: the oracle's sums of |q| per throat and
    per pore (throat_absflow, pore_absflux)."""
    worst = {}
    for k, sk in (("throat_flow", "throat_absflow"), ("pore_residual", "pore_absflux"),
                  ("throat_area", None)):
        ref = np.asarray(o[k], np.float64)
        got = np.asarray(r[k], np.float64)
        assert got.shape == ref.shape, k
        if not len(ref):
            continue
        scale = np.abs(ref) if sk is None else np.maximum(np.abs(ref), scales[sk])
        err = np.abs(got - ref)
        ok = err <= TOL * scale
        assert ok.all(), (k, int((~ok).sum()), float((err / np.maximum(scale, 1e-300)).max()))
        worst[k] = float((err / np.maximum(scale, 1e-300)).max())
    return worst


def _check(r, o):
    assert np.array_equal(r["throats"], o["throats"]), f"{len(r['throats'])} vs {len(o['throats'])}"
    assert np.array_equal(r["pores"].view(np.int32), o["pores"].view(np.int32))
    check_sums(r, o, o)
    assert np.array_equal(r["pore_pressure"], o["pore_pressure"])
    assert np.allclose(r["throat_dp"], o["throat_dp"], rtol=TOL, atol=0)


@pytest.mark.parametrize("case", standard_cases() + [c for c in edge_cases()
                                                     if np.all(np.isfinite(c[1]))],
                         ids=lambda c: c[0])
@pytest.mark.parametrize("with_openness", [True, False])
def test_network_flow_matches_oracle(gpu, port, case, with_openness):
    pnm, _ = gpu
    name, sdf, org, spc = case
    f = flow_fields(sdf)
    kw = dict(ox=f[4], oy=f[5], oz=f[6]) if with_openness else {}
    gp = [1e-3, -2e-3, 5e-4]
    r = pnm.extract_network_flow(sdf, org, spc, *f[:4], grad_p_zyx=gp, numpy=True, **kw)
    o = port.extract_network_flow(sdf, org, spc, *f[:4], grad_p_zyx=gp, **kw)
    _check(r, o)


@pytest.mark.parametrize("nz", [33, 257])
def test_flow_host_slab_boundaries(gpu, port, nz):
    """The seven fields follow the SDF's z-slabs on the copy stream; at these depths the last
    slab is one plane, already carried by the copy before it."""
    pnm, _ = gpu
    sdf = syn.packing((nz, 9, 11), 0.4, mean_r=3.0, seed=nz)
    f = flow_fields(sdf)
    gp = [1e-3, -2e-3, 5e-4]
    kw = dict(ox=f[4], oy=f[5], oz=f[6])
    r = pnm.extract_network_flow(sdf, [0] * 3, [1] * 3, *f[:4], grad_p_zyx=gp, numpy=True, **kw)
    _check(r, port.extract_network_flow(sdf, [0] * 3, [1] * 3, *f[:4], grad_p_zyx=gp, **kw))


def test_flow_goldens(gpu, port):
    pnm, _ = gpu
    from golden.make_golden import FLOW_CASES

    for name, (mk, mkf, org, spc, gp, opn) in FLOW_CASES.items():
        g = dict(np.load(os.path.join(GOLDEN, name + ".npz")))
        sdf = np.ascontiguousarray(mk(), dtype=np.float32)
        f = mkf(sdf)
        kw = dict(ox=f[4], oy=f[5], oz=f[6]) if opn else {}
        r = pnm.extract_network_flow(sdf, org, spc, *f[:4], grad_p_zyx=gp, numpy=True, **kw)
        assert np.array_equal(r["throats"], g["throats"]), name
        assert np.array_equal(r["pores"].view(np.int32), g["pores"].view(np.int32)), name
        # the reference's own output; the per-element |q| sums come from the oracle port (pinned
        # to the reference bitwise on these cases)
        o = port.extract_network_flow(sdf, org, spc, *f[:4], grad_p_zyx=gp, **kw)
        check_sums(r, g, o)
        assert np.allclose(r["pore_pressure"], g["pore_pressure"], rtol=1e-12, atol=1e-15), name
        assert np.allclose(r["throat_dp"], g["throat_dp"], rtol=1e-12, atol=1e-15), name


def test_flow_known_answers(gpu):
    pnm, _ = gpu
    sdf = syn.chamber_tube()
    f = syn.fourier_fields(sdf, seed=4)
    r = pnm.extract_network_flow(sdf, [0] * 3, [1] * 3, *f[:4], ox=f[4], oy=f[5], oz=f[6],
                                 numpy=True)
    assert len(r["pores"]) == 3 and len(r["throats"]) == 3
    sdf = syn.capsules()
    f = syn.fourier_fields(sdf, seed=4)
    r = pnm.extract_network_flow(sdf, [0] * 3, [1] * 3, *f[:4], ox=f[4], oy=f[5], oz=f[6],
                                 numpy=True)
    assert len(r["pores"]) == 3
    assert sum(1 for t in r["throats"].tolist() if t == [1, 2]) == 2


def test_flow_is_deterministic(gpu):
    pnm, _ = gpu
    sdf = syn.packing((48, 52, 56), 0.4, seed=3)
    f = syn.fourier_fields(sdf, seed=4)
    a = pnm.extract_network_flow(sdf, [0] * 3, [1] * 3, *f[:4], ox=f[4], oy=f[5], oz=f[6],
                                 grad_p_zyx=[0, 0, -1e-4], numpy=True)
    b = pnm.extract_network_flow(sdf, [0] * 3, [1] * 3, *f[:4], ox=f[4], oy=f[5], oz=f[6],
                                 grad_p_zyx=[0, 0, -1e-4], numpy=True)
    for k in a:
        assert np.array_equal(np.asarray(a[k]).view(np.uint8), np.asarray(b[k]).view(np.uint8)), k


def test_flow_list_surface(gpu):
    pnm, _ = gpu
    sdf = syn.sphere_lattice(36, 30, 24)
    u, v, w, p, ox, oy, oz = syn.mac_fields(36, 30, 24)
    d = pnm.extract_network_flow(sdf, [2.0, -1.0, 0.5], [1.5, 1.0, 0.5], u, v, w, p, ox, oy, oz,
                                 grad_p_zyx=[0.5e-3, -2e-3, 1e-3])
    assert set(d) == {"pores", "pore_pressure", "pore_residual", "throats", "throat_flow",
                      "throat_area", "throat_dp"}
    assert isinstance(d["pores"][0], pnm.Pore) and isinstance(d["throats"][0], tuple)


@pytest.mark.slow
def test_flow_packing_96_matches_oracle(gpu, port):
    pnm, _ = gpu
    sdf = syn.packing((96, 96, 96), 0.4, seed=3)
    f = syn.fourier_fields(sdf, seed=4)
    kw = dict(ox=f[4], oy=f[5], oz=f[6])
    r = pnm.extract_network_flow(sdf, [0] * 3, [1] * 3, *f[:4], grad_p_zyx=[0, 0, -1e-4],
                                 numpy=True, **kw)
    o = port.extract_network_flow(sdf, [0] * 3, [1] * 3, *f[:4], grad_p_zyx=[0, 0, -1e-4], **kw)
    _check(r, o)
