"""Pins the CPU oracle (oracle/pnm_oracle.cpp) — CPU only.

1. Against golden fixtures produced by the reference's own implementation
   (tests/golden/make_golden.py): bit-exact labels, pore sets and connections; throat lists
   exact and FP64 flow outputs to 1e-12 of the largest throat flux.
2. Against the reference compiled here (oracle/_ref, when the reference checkout exists) on
   the edge cases of tests/cases.py.
3. The reference's own known answers (CI smoke test, scripts/verify_network_flow.py topology).
"""
import glob
import os

import numpy as np
import pytest

from cases import edge_cases, flow_fields, random_volume, standard_cases
from oracle import Oracle, reference_available, sorted_pores
from peclet_pnm_gb300 import synthetic as syn

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _bits(p):
    return sorted_pores(p).view(np.int32)


def _load(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


def _golden_input(name, g):
    from golden.make_golden import NETWORK_CASES, digest

    if "sdf" in g:
        return g["sdf"]
    sdf = np.ascontiguousarray(NETWORK_CASES[name][0](), dtype=np.float32)
    assert digest(sdf) == str(g["input_sha256"]), "regenerated input differs from the fixture's"
    return sdf


NETWORK_GOLDENS = sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz"))
                         if not os.path.basename(p).startswith("flow_"))
FLOW_GOLDENS = sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "flow_*.npz")))


@pytest.mark.parametrize("name", NETWORK_GOLDENS)
def test_port_matches_reference_golden(port, name):
    g = _load(name)
    sdf = _golden_input(name, g)
    pores, seg, pairs = port.extract_pore_network(sdf, g["origin"].tolist(), g["spacing"].tolist())
    assert np.array_equal(seg, g["seg"])
    assert np.array_equal(pairs, g["pairs"])
    assert np.array_equal(_bits(pores), g["pores"].view(np.int32))
    staged = port.extract_pores(sdf, g["origin"].tolist(), g["spacing"].tolist())
    assert np.array_equal(_bits(staged), g["staged_pores"].view(np.int32))


@pytest.mark.parametrize("name", FLOW_GOLDENS)
def test_port_flow_matches_reference_golden(port, name):
    from golden.make_golden import FLOW_CASES

    g = _load(name)
    mk, mkf, org, spc, gp, opn = FLOW_CASES[name]
    sdf = np.ascontiguousarray(mk(), dtype=np.float32)
    f = mkf(sdf)
    kw = dict(ox=f[4], oy=f[5], oz=f[6]) if opn else {}
    r = port.extract_network_flow(sdf, org, spc, *f[:4], grad_p_zyx=gp, **kw)
    assert np.array_equal(r["throats"], g["throats"])
    assert np.array_equal(r["pores"].view(np.int32), g["pores"].view(np.int32))
    qs = max(1e-300, float(np.abs(g["throat_flow"]).max()) if len(g["throat_flow"]) else 1.0)
    for k in ("throat_flow", "throat_area", "pore_residual"):
        assert np.allclose(r[k], g[k], rtol=0, atol=1e-12 * qs), k
    for k in ("pore_pressure", "throat_dp"):
        assert np.allclose(r[k], g[k], rtol=1e-12, atol=1e-15), k


needs_ref = pytest.mark.skipif(not reference_available(),
                               reason="reference checkout not built here (oracle/_ref)")


@needs_ref
@pytest.mark.parametrize("case", edge_cases() + standard_cases(), ids=lambda c: c[0])
def test_port_matches_reference_edge_cases(port, case):
    name, sdf, org, spc = case
    ref = Oracle("reference")
    a = ref.extract_pore_network(sdf, org, spc)
    b = port.extract_pore_network(sdf, org, spc)
    assert np.array_equal(a[1], b[1]), "seg"
    assert np.array_equal(a[2], b[2]), "pairs"
    assert np.array_equal(_bits(a[0]), _bits(b[0])), "pores"
    # stage-level: gradient roots of every pore voxel
    _, ra = ref.segment_xyz(sdf, [spc[2], spc[1], spc[0]], roots=True)
    _, rb = port.segment_xyz(sdf, [spc[2], spc[1], spc[0]], roots=True)
    pore = np.asarray(sdf, np.float32).reshape(-1) > 0
    assert np.array_equal(ra[pore], rb[pore]), "gradient roots"


@needs_ref
@pytest.mark.parametrize("case", [c for c in edge_cases() if np.all(np.isfinite(c[1]))
                                  and c[1].size >= 8] + standard_cases()[:3],
                         ids=lambda c: c[0])
def test_port_flow_matches_reference_edge_cases(port, case):
    name, sdf, org, spc = case
    f = flow_fields(sdf)
    ref = Oracle("reference")
    for opn in (True, False):
        kw = dict(ox=f[4], oy=f[5], oz=f[6]) if opn else {}
        try:
            a = ref.extract_network_flow(sdf, org, spc, *f[:4], grad_p_zyx=[1e-3, 2e-3, -1e-3], **kw)
        except Exception:  # the reference is undefined when every voxel is labelled solid
            continue
        b = port.extract_network_flow(sdf, org, spc, *f[:4], grad_p_zyx=[1e-3, 2e-3, -1e-3], **kw)
        assert np.array_equal(a["throats"], b["throats"])
        assert np.array_equal(a["pores"].view(np.int32), b["pores"].view(np.int32))
        for k in ("throat_flow", "throat_area", "pore_residual", "pore_pressure", "throat_dp"):
            assert np.array_equal(a[k], b[k]), k  # same serial order -> bitwise


@needs_ref
@pytest.mark.parametrize("seed", range(40))
def test_port_matches_reference_random_volumes(port, seed):
    sdf, org, spc = random_volume(seed)
    ref = Oracle("reference")
    a = ref.extract_pore_network(sdf, org, spc)
    b = port.extract_pore_network(sdf, org, spc)
    assert np.array_equal(a[1], b[1]), "seg"
    assert np.array_equal(a[2], b[2]), "pairs"
    assert np.array_equal(_bits(a[0]), _bits(b[0])), "pores"
    if seed % 5 == 0 and sdf.size >= 8:
        f = flow_fields(sdf)
        try:
            fa = ref.extract_network_flow(sdf, org, spc, *f[:4], grad_p_zyx=[2e-3, -1e-3, 5e-4],
                                          ox=f[4], oy=f[5], oz=f[6])
        except Exception:  # the reference is undefined when every voxel is labelled solid
            return
        fb = port.extract_network_flow(sdf, org, spc, *f[:4], grad_p_zyx=[2e-3, -1e-3, 5e-4],
                                       ox=f[4], oy=f[5], oz=f[6])
        assert np.array_equal(fa["throats"], fb["throats"])
        assert np.array_equal(fa["pores"].view(np.int32), fb["pores"].view(np.int32))
        for k in ("throat_flow", "throat_area", "pore_residual", "pore_pressure", "throat_dp"):
            assert np.array_equal(fa[k], fb[k]), k


_SPECIALS = np.array([np.nan, np.inf, -np.inf, 0.0, -0.0, 1.0, -1.0, -1.5, -1.4999999, -1.5000001,
                      2.0, 1e-30, -1e-30], np.float32)


def _fuzz_volume(rng, it):
    """Shapes 1..6 per axis: special values only (NaN, +-inf, -0, values at the marker threshold
    -1.5 x spacing and one ulp either side), noise with 20% special values, coarse integers
    (plateaus), quarter-step quantised noise."""
    shp = tuple(int(v) for v in rng.integers(1, 7, size=3))
    mode = it % 4
    if mode == 0:
        a = rng.choice(_SPECIALS, size=shp)
    elif mode == 1:
        a = rng.normal(0, 2, size=shp).astype(np.float32)
        m = rng.random(shp) < 0.2
        a[m] = rng.choice(_SPECIALS, size=int(m.sum()))
    elif mode == 2:
        a = rng.integers(-3, 3, size=shp).astype(np.float32) * 0.5
    else:
        a = np.round(rng.normal(0, 1.5, size=shp) * 4) / 4
    spc = [float(x) for x in rng.choice([0.5, 1.0, 1.0, 2.0, 0.75], size=3)]
    org = [float(x) for x in rng.uniform(-2, 2, size=3)]
    return np.ascontiguousarray(a, np.float32), org, spc


@needs_ref
@pytest.mark.parametrize("seed", range(4))
def test_port_matches_reference_fuzz(port, seed):
    """500 tiny volumes per seed, bitwise against the reference's own code."""
    rng = np.random.default_rng(7000 + seed)
    ref = Oracle("reference")
    for it in range(500):
        sdf, org, spc = _fuzz_volume(rng, it)
        a = ref.extract_pore_network(sdf, org, spc)
        b = port.extract_pore_network(sdf, org, spc)
        assert np.array_equal(a[1], b[1]), (it, "seg")
        assert np.array_equal(a[2], b[2]), (it, "pairs")
        assert np.array_equal(_bits(a[0]), _bits(b[0])), (it, "pores")


@needs_ref
def test_port_staged_calls_match_reference_fuzz(port):
    """The staged calls on 500 fuzzed tiny volumes, and the topology of random labels."""
    rng = np.random.default_rng(7500)
    ref = Oracle("reference")
    for it in range(500):
        sdf, org, spc = _fuzz_volume(rng, it)
        assert np.array_equal(_bits(ref.extract_pores(sdf, org, spc)),
                              _bits(port.extract_pores(sdf, org, spc))), it
        seg = ref.segment_volume(sdf, spc)
        assert np.array_equal(seg, port.segment_volume(sdf, spc)), it
        shape = list(sdf.shape)
        assert np.array_equal(ref.extract_topology_gpu(seg, shape),
                              port.extract_topology_gpu(seg, shape)), it
        lab = rng.integers(-4, 5, size=sdf.size).astype(np.int32)
        assert np.array_equal(ref.extract_topology_gpu(lab, shape),
                              port.extract_topology_gpu(lab, shape)), it


@needs_ref
@pytest.mark.parametrize("seed", range(2))
def test_port_flow_matches_reference_fuzz(port, seed):
    """500 small volumes (2..8 per axis) per seed with random MAC fields, openness on every other,
    random spacing, origin and pressure gradient: every output bitwise (same serial order)."""
    rng = np.random.default_rng(8000 + seed)
    ref = Oracle("reference")
    for it in range(500):
        shp = tuple(int(v) for v in rng.integers(2, 9, size=3))
        sdf = rng.normal(0, 2, size=shp).astype(np.float32)
        if it % 3 == 0:
            sdf = (np.round(sdf * 2) / 2).astype(np.float32)
        f = [np.ascontiguousarray(rng.normal(0, 1e-3, size=shp)) for _ in range(4)]
        o = [np.ascontiguousarray(np.clip(rng.uniform(-0.3, 1.0, size=shp), 0, 1))
             for _ in range(3)]
        spc = [float(x) for x in rng.choice([0.5, 1.0, 2.0], size=3)]
        org = [float(x) for x in rng.uniform(-2, 2, size=3)]
        gp = [float(x) for x in rng.normal(0, 1e-3, size=3)]
        kw = dict(ox=o[0], oy=o[1], oz=o[2]) if it % 2 else {}
        try:
            a = ref.extract_network_flow(sdf, org, spc, *f, grad_p_zyx=gp, **kw)
        except Exception:  # the reference is undefined when every voxel is labelled solid
            continue
        b = port.extract_network_flow(sdf, org, spc, *f, grad_p_zyx=gp, **kw)
        assert np.array_equal(a["throats"], b["throats"]), it
        assert np.array_equal(a["pores"].view(np.int32), b["pores"].view(np.int32)), it
        for k in ("throat_flow", "throat_area", "pore_residual", "pore_pressure", "throat_dp"):
            assert np.array_equal(a[k], b[k]), (it, k)


def test_port_thread_count_invariance():
    sdf = syn.packing((40, 44, 48), 0.35, seed=9)
    a = Oracle("port", threads=1).extract_pore_network(sdf, [0, 0, 0], [1, 1, 1])
    b = Oracle("port", threads=4).extract_pore_network(sdf, [0, 0, 0], [1, 1, 1])
    assert np.array_equal(a[1], b[1]) and np.array_equal(a[2], b[2])
    assert np.array_equal(_bits(a[0]), _bits(b[0]))


def test_known_answer_ci_smoke(port):
    """.github/workflows/ci.yml:61-73: pores > 0, connections > 0, staged count == fused count."""
    sdf = syn.ci_lattice()
    pores, seg, conns = port.extract_pore_network(sdf, [0.0] * 3, [1.0] * 3)
    assert len(pores) > 0 and len(conns) > 0
    assert len(port.extract_pores(sdf, [0.0] * 3, [1.0] * 3)) == len(pores)


def test_known_answer_chamber_tube(port):
    """scripts/verify_network_flow.py:88-90: 3 pores, a single loop (#throats == #pores)."""
    sdf = syn.chamber_tube()
    f = syn.fourier_fields(sdf, seed=4)
    r = port.extract_network_flow(sdf, [0, 0, 0], [1, 1, 1], *f[:4], ox=f[4], oy=f[5], oz=f[6])
    assert len(r["pores"]) == 3
    assert len(r["throats"]) == len(r["pores"])


def test_known_answer_parallel_capsules(port):
    """scripts/verify_network_flow.py:233-235: 3 pores and pair (1,2) twice (per-patch)."""
    sdf = syn.capsules()
    f = syn.fourier_fields(sdf, seed=4)
    r = port.extract_network_flow(sdf, [0, 0, 0], [1, 1, 1], *f[:4], ox=f[4], oy=f[5], oz=f[6])
    assert len(r["pores"]) == 3
    assert sum(1 for t in r["throats"].tolist() if t == [1, 2]) == 2


def test_empty_volume(port):
    pores, seg, pairs = port.extract_pore_network(np.zeros((0, 3, 3), np.float32), [0] * 3, [1] * 3)
    assert len(pores) == 0 and len(seg) == 0 and len(pairs) == 0
