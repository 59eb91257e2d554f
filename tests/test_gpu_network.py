"""GPU parity: the CUDA path through the C ABI against the CPU oracle and the reference goldens.

Bar: bit-exact for every integer output (labels, connections), bit-exact float32 pore records
(compared as sorted sets; the reference's pore order is an atomic race).
"""
import os

import numpy as np
import pytest

from cases import edge_cases, flow_fields, random_volume, standard_cases
from oracle import sorted_pores
from peclet_pnm_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _bits(p):
    return sorted_pores(p).view(np.int32)


def _check(gpu_out, ora_out):
    gp, gs, gq = gpu_out
    op, os_, oq = ora_out
    assert np.array_equal(gs, os_), f"seg: {int((gs != os_).sum())} voxels differ"
    assert np.array_equal(gq, oq), f"pairs: {len(gq)} vs {len(oq)}"
    assert np.array_equal(_bits(gp), _bits(op)), f"pores: {len(gp)} vs {len(op)}"


@pytest.mark.parametrize("case", standard_cases() + edge_cases(), ids=lambda c: c[0])
def test_pore_network_matches_oracle(gpu, port, case):
    pnm, ctx = gpu
    name, sdf, org, spc = case
    out = pnm.extract_pore_network(sdf, org, spc, numpy=True)
    _check(out, port.extract_pore_network(sdf, org, spc))
    # pores come back in voxel order
    pores = out[0]
    assert len(pores) == len(port.extract_pores(sdf, org, spc))


@pytest.mark.parametrize("case", standard_cases()[:4] + edge_cases()[:6], ids=lambda c: c[0])
def test_staged_calls_match_oracle(gpu, port, case):
    pnm, _ = gpu
    name, sdf, org, spc = case
    p = pnm.extract_pores(sdf, org, spc, numpy=True)
    assert np.array_equal(_bits(p), _bits(port.extract_pores(sdf, org, spc)))
    seg = pnm.segment_volume(sdf, spc, numpy=True)
    assert np.array_equal(seg, port.segment_volume(sdf, spc))
    pairs = pnm.extract_topology_gpu(seg, list(sdf.shape), numpy=True)
    assert np.array_equal(pairs, port.extract_topology_gpu(seg, list(sdf.shape)))


def test_goldens(gpu):
    import glob

    pnm, _ = gpu
    from golden.make_golden import NETWORK_CASES, digest

    names = [os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz"))
             if not os.path.basename(p).startswith("flow_")]
    assert names
    for name in names:
        g = dict(np.load(os.path.join(GOLDEN, name + ".npz")))
        sdf = g["sdf"] if "sdf" in g else np.ascontiguousarray(NETWORK_CASES[name][0](), np.float32)
        assert digest(sdf) == str(g["input_sha256"])
        pores, seg, pairs = pnm.extract_pore_network(sdf, g["origin"].tolist(),
                                                     g["spacing"].tolist(), numpy=True)
        assert np.array_equal(seg, g["seg"]), name
        assert np.array_equal(pairs, g["pairs"]), name
        assert np.array_equal(_bits(pores), g["pores"].view(np.int32)), name


def test_topology_of_arbitrary_labels(gpu, port):
    pnm, _ = gpu
    rng = np.random.default_rng(3)
    for shape in [(1, 1, 1), (2, 3, 4), (9, 8, 7), (30, 31, 33)]:
        seg = rng.integers(-2**31, 2**31 - 1, size=shape, dtype=np.int64).astype(np.int32)
        seg.reshape(-1)[::3] = rng.integers(-5, 5, size=seg.reshape(-1)[::3].shape)
        a = pnm.extract_topology_gpu(seg.reshape(-1), list(shape), numpy=True)
        b = port.extract_topology_gpu(seg.reshape(-1), list(shape))
        assert np.array_equal(a, b), shape


def test_list_surface_matches_reference_types(gpu):
    pnm, _ = gpu
    sdf = syn.ci_lattice()
    pores, seg, conns = pnm.extract_pore_network(sdf, [0.0] * 3, [1.0] * 3)
    assert isinstance(pores, list) and isinstance(pores[0], pnm.Pore)
    assert isinstance(seg, list) and isinstance(seg[0], int) and len(seg) == sdf.size
    assert isinstance(conns, list) and isinstance(conns[0], tuple)
    assert len(pores) > 0 and len(conns) > 0
    assert len(pnm.extract_pores(sdf, [0.0] * 3, [1.0] * 3)) == len(pores)
    # float64 SDF is cast to float32 like nanobind's implicit conversion
    seg64 = pnm.segment_volume(sdf.astype(np.float64), [1.0] * 3, numpy=True)
    assert np.array_equal(seg64, np.asarray(seg, np.int32))


def test_repeated_calls_are_identical_and_reuse_workspace(gpu):
    pnm, _ = gpu
    a = syn.packing((48, 40, 56), 0.4, seed=31)
    b = syn.packing((20, 64, 24), 0.5, seed=32)
    r1 = pnm.extract_pore_network(a, [0] * 3, [1] * 3, numpy=True)
    pnm.extract_pore_network(b, [0] * 3, [1] * 3, numpy=True)
    r2 = pnm.extract_pore_network(a, [0] * 3, [1] * 3, numpy=True)
    for x, y in zip(r1, r2):
        assert np.array_equal(x, y)


@pytest.mark.parametrize("seed", range(40))
def test_random_volumes_match_oracle(gpu, port, seed):
    """Seeded volumes of random shape, value family, anisotropic spacing and origin (the oracle
    equals the reference bitwise on the same volumes): the network and the staged calls
    bit-exact, and on every fifth volume the network flow within the flow bar."""
    pnm, _ = gpu
    sdf, org, spc = random_volume(seed)
    _check(pnm.extract_pore_network(sdf, org, spc, numpy=True),
           port.extract_pore_network(sdf, org, spc))
    # the staged entry points on the same volume
    assert np.array_equal(_bits(pnm.extract_pores(sdf, org, spc, numpy=True)),
                          _bits(port.extract_pores(sdf, org, spc)))
    seg = pnm.segment_volume(sdf, spc, numpy=True)
    assert np.array_equal(seg, port.segment_volume(sdf, spc))
    assert np.array_equal(pnm.extract_topology_gpu(seg, list(sdf.shape), numpy=True),
                          port.extract_topology_gpu(seg, list(sdf.shape)))
    if seed % 5 == 0 and sdf.size >= 8:
        from test_gpu_flow import _check as check_flow

        f = flow_fields(sdf)
        kw = dict(ox=f[4], oy=f[5], oz=f[6])
        gp = [2e-3, -1e-3, 5e-4]
        check_flow(pnm.extract_network_flow(sdf, org, spc, *f[:4], grad_p_zyx=gp, numpy=True, **kw),
                   port.extract_network_flow(sdf, org, spc, *f[:4], grad_p_zyx=gp, **kw))


@pytest.mark.parametrize("nz", [17, 33, 48, 257, 271])
def test_host_slab_boundaries(gpu, port, nz):
    """Host-buffer calls upload the SDF in z-slabs of 16-plane multiples, each copy ending one
    plane into the next slab; these depths leave a last slab of one plane (nothing left to copy
    for it), a ragged one, or an even split."""
    pnm, _ = gpu
    rng = np.random.default_rng(nz)
    sdf = syn.packing((nz, 9, 11), 0.4, mean_r=3.0, seed=nz)
    sdf += rng.normal(0.0, 0.05, size=sdf.shape).astype(np.float32)
    out = pnm.extract_pore_network(sdf, [0] * 3, [1] * 3, numpy=True)
    _check(out, port.extract_pore_network(sdf, [0] * 3, [1] * 3))


@pytest.mark.slow
def test_packing_128_matches_oracle(gpu, port):
    pnm, _ = gpu
    sdf = syn.packing((128, 128, 128), 0.4, seed=2)
    _check(pnm.extract_pore_network(sdf, [0] * 3, [1] * 3, numpy=True),
           port.extract_pore_network(sdf, [0] * 3, [1] * 3))


def test_device_entry_points_with_torch(gpu, port):
    torch = pytest.importorskip("torch")
    pnm, ctx = gpu
    from peclet_pnm_gb300 import _capi

    sdf = syn.packing((40, 36, 44), 0.4, seed=41)
    d_sdf = torch.from_numpy(sdf).cuda()
    d_seg = torch.empty(sdf.size, dtype=torch.int32, device="cuda")
    d_pores = torch.empty((1000, 4), dtype=torch.float32, device="cuda")
    d_pairs = torch.empty((100000, 2), dtype=torch.int32, device="cuda")
    o = np.zeros(3, np.float32)
    s = np.ones(3, np.float32)
    npo, npa = _capi._i64(), _capi._i64()
    torch.cuda.synchronize()
    ctx.check(_capi.pnm_extract_pore_network_dev(
        ctx.h, d_sdf.data_ptr(), 44, 36, 40, _capi.as_ptr(o), _capi.as_ptr(s), d_pores.data_ptr(),
        1000, _capi.ctypes.byref(npo), d_seg.data_ptr(), d_pairs.data_ptr(), 100000,
        _capi.ctypes.byref(npa)))
    op, oseg, opairs = port.extract_pore_network(sdf, [0] * 3, [1] * 3)
    assert np.array_equal(d_seg.cpu().numpy(), oseg)
    assert np.array_equal(d_pairs[:npa.value].cpu().numpy(), opairs)
    assert np.array_equal(_bits(d_pores[:npo.value].cpu().numpy()), _bits(op))
    # capacity error reports the required size
    rc = _capi.pnm_extract_pore_network_dev(
        ctx.h, d_sdf.data_ptr(), 44, 36, 40, _capi.as_ptr(o), _capi.as_ptr(s), d_pores.data_ptr(),
        1000, _capi.ctypes.byref(npo), d_seg.data_ptr(), d_pairs.data_ptr(), 3,
        _capi.ctypes.byref(npa))
    assert rc == _capi.PNM_ERR_CAPACITY and npa.value == len(opairs)
