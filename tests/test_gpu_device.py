"""GPU parity of the device-resident surface (peclet_pnm_gb300.device, *_dev entry points of the
C ABI) and of the streaming VTI reader (pnm_read_vti_dev).

Device calls take torch CUDA tensors (or DLPack producers) and must give exactly what the
host-pointer calls give on the same volume; those are pinned to the oracle elsewhere, and here
segment_volume / extract_pore_network are checked against the oracle directly as well."""
import math
import os

import numpy as np
import pytest

from cases import edge_cases, flow_fields, standard_cases
from oracle import sorted_pores

pytestmark = pytest.mark.gpu
VTI_GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "vti", "cases.npz")


@pytest.fixture(scope="module")
def torch():
    import torch

    assert torch.cuda.is_available()
    return torch


class _DLPackOnly:
    """A producer that exposes nothing but the DLPack protocol."""

    def __init__(self, t):
        self._t = t

    def __dlpack__(self, **kw):
        return self._t.__dlpack__(**kw)

    def __dlpack_device__(self):
        return self._t.__dlpack_device__()


CASES = standard_cases() + [c for c in edge_cases() if np.all(np.isfinite(c[1]))][:6]


@pytest.mark.parametrize("case", CASES, ids=lambda c: c[0])
def test_pore_network_device_matches_oracle(gpu, port, torch, case):
    pnm, _ = gpu
    from peclet_pnm_gb300 import device

    name, sdf, org, spc = case
    d = torch.from_numpy(np.ascontiguousarray(sdf, np.float32)).cuda()
    pores, seg, pairs = device.extract_pore_network_device(_DLPackOnly(d), org, spc)
    assert pores.is_cuda and seg.is_cuda and pairs.is_cuda
    op, oseg, opairs = port.extract_pore_network(sdf, org, spc)
    assert np.array_equal(sorted_pores(pores.cpu().numpy()).view(np.int32),
                          sorted_pores(op).view(np.int32))
    assert np.array_equal(seg.cpu().numpy().reshape(-1), np.asarray(oseg).reshape(-1))
    assert np.array_equal(pairs.cpu().numpy(), np.asarray(opairs).reshape(-1, 2))
    seg2 = device.segment_volume_device(d, spc)
    assert torch.equal(seg2, seg)


def test_pore_network_device_on_a_side_stream(gpu, torch):
    """The pore records run on the context's second stream: on a caller stream that is not the
    default one, synchronising that stream alone must leave every output complete, and a
    launch queued on it right after the call (a copy of the records) must see them."""
    pnm, _ = gpu
    from peclet_pnm_gb300 import device
    from peclet_pnm_gb300 import synthetic as syn

    sdf = syn.packing((64, 72, 80), 0.4, seed=9)
    hp, hs, hq = pnm.extract_pore_network(sdf, [0, 0, 0], [1, 1, 1], numpy=True)
    d = torch.from_numpy(sdf).cuda()
    caller = torch.cuda.Stream()
    for _ in range(3):
        with torch.cuda.stream(caller):
            pores, seg, pairs = device.extract_pore_network_device(d, [0, 0, 0], [1, 1, 1])
            copied = pores.clone()  # queued on the caller's stream behind the call
        caller.synchronize()
        assert np.array_equal(copied.cpu().numpy(), hp)
        assert np.array_equal(seg.cpu().numpy().reshape(-1), hs)
        assert np.array_equal(pairs.cpu().numpy(), hq)


@pytest.mark.parametrize("caps", [(1, 1), (1, 10 ** 6), (10 ** 6, 1)])
def test_pore_network_device_capacity_retry(gpu, torch, caps):
    """Outputs smaller than the result: the call reports the counts and is re-run."""
    pnm, _ = gpu
    from peclet_pnm_gb300 import device
    from peclet_pnm_gb300 import synthetic as syn

    sdf = syn.packing((40, 48, 56), 0.4, seed=7)
    d = torch.from_numpy(sdf).cuda()
    pores, seg, pairs = device.extract_pore_network_device(d, [0, 0, 0], [1, 1, 1],
                                                           pore_cap=caps[0], pair_cap=caps[1])
    hp, hs, hq = pnm.extract_pore_network(sdf, [0, 0, 0], [1, 1, 1], numpy=True)
    assert len(hp) > 1 and len(hq) > 1
    assert np.array_equal(pores.cpu().numpy(), hp)
    assert np.array_equal(seg.cpu().numpy().reshape(-1), hs)
    assert np.array_equal(pairs.cpu().numpy(), hq)


@pytest.mark.parametrize("case", standard_cases(), ids=lambda c: c[0])
@pytest.mark.parametrize("with_openness", [True, False])
def test_network_flow_device_matches_host(gpu, torch, case, with_openness):
    pnm, _ = gpu
    from peclet_pnm_gb300 import device

    name, sdf, org, spc = case
    f = flow_fields(sdf)
    kw = dict(ox=f[4], oy=f[5], oz=f[6]) if with_openness else {}
    gp = [1e-3, -2e-3, 5e-4]
    h = pnm.extract_network_flow(sdf, org, spc, *f[:4], grad_p_zyx=gp, numpy=True, **kw)
    dv = {k: torch.from_numpy(v).cuda() for k, v in kw.items()}
    side = torch.cuda.Stream()
    with torch.cuda.stream(side):  # the caller's stream, not the default one
        r = device.extract_network_flow_device(torch.from_numpy(sdf).cuda(), org, spc,
                                               *[torch.from_numpy(x).cuda() for x in f[:4]],
                                               grad_p_zyx=gp, **dv)
    side.synchronize()
    assert set(r) == set(h)
    for k in h:
        got = r[k].cpu().numpy()
        assert got.dtype == h[k].dtype and got.shape == h[k].shape, k
        assert np.array_equal(got.view(np.uint8), h[k].view(np.uint8)), k


def test_network_flow_device_back_to_back(gpu, torch):
    """Two calls in a row on one context: the first call's results are copies, not views of the
    context's buffers that the second call overwrites."""
    pnm, _ = gpu
    from peclet_pnm_gb300 import device
    from peclet_pnm_gb300 import synthetic as syn

    a = syn.packing((40, 48, 56), 0.4, seed=7)
    b = syn.packing((40, 48, 56), 0.4, seed=8)
    fa, fb = flow_fields(a, seed=1), flow_fields(b, seed=2)
    ra = device.extract_network_flow_device(torch.from_numpy(a).cuda(), [0] * 3, [1] * 3,
                                            *[torch.from_numpy(x).cuda() for x in fa[:4]])
    rb = device.extract_network_flow_device(torch.from_numpy(b).cuda(), [0] * 3, [1] * 3,
                                            *[torch.from_numpy(x).cuda() for x in fb[:4]])
    ha = pnm.extract_network_flow(a, [0] * 3, [1] * 3, *fa[:4], numpy=True)
    hb = pnm.extract_network_flow(b, [0] * 3, [1] * 3, *fb[:4], numpy=True)
    for k in ha:
        assert np.array_equal(ra[k].cpu().numpy(), ha[k]), k
        assert np.array_equal(rb[k].cpu().numpy(), hb[k]), k


def test_device_empty_and_errors(gpu, torch):
    from peclet_pnm_gb300 import device

    e = torch.zeros((0, 4, 4), dtype=torch.float32, device="cuda")
    p, s, q = device.extract_pore_network_device(e, [0] * 3, [1] * 3)
    assert p.shape == (0, 4) and q.shape == (0, 2) and s.numel() == 0
    with pytest.raises(RuntimeError):
        device.extract_pore_network_device(torch.zeros((4, 4), device="cuda"), [0] * 3, [1] * 3)
    with pytest.raises(RuntimeError):
        device.extract_pore_network_device(torch.zeros((4, 4, 4)), [0] * 3, [1] * 3)
    x = torch.zeros((4, 4, 4), dtype=torch.float64, device="cuda")
    with pytest.raises(RuntimeError, match="openness"):
        device.extract_network_flow_device(x.float(), [0] * 3, [1] * 3, x, x, x, x, ox=x)


# ---- VTI straight to the device ---------------------------------------------------------------
def test_read_vti_device_multi_chunk(gpu, torch, tmp_path):
    """A volume larger than two staging chunks (64 MiB each) arrives unchanged."""
    pnm, _ = gpu
    rng = np.random.default_rng(3)
    a = rng.standard_normal((136, 260, 300), dtype=np.float32)  # 42.4 M values, 170 MB
    p = tmp_path / "big.vti"
    pnm.write_sdf_vti(str(p), a, [0.5, 1.0, -2.0], [0.1, 0.2, 0.3])
    t, org, spc = pnm.read_vti_device(str(p))
    assert t.is_cuda and tuple(t.shape) == a.shape
    assert torch.equal(t.cpu(), torch.from_numpy(a))
    h, horg, hspc = pnm.SDFReader.read_vti(str(p))
    assert org == horg and spc == hspc


@pytest.mark.parametrize("name", ["point_7x5x3", "short_count", "odd_count", "celldata_labels"])
def test_read_vti_device_matches_host(gpu, torch, tmp_path, name):
    pnm, _ = gpu
    g = np.load(VTI_GOLDEN)
    p = tmp_path / f"{name}.vti"
    p.write_bytes(g[f"{name}__file"].tobytes())
    out = torch.full((int(np.prod(g[f"{name}__dims"])) + 5,), 7.0, device="cuda")
    t, _, _ = pnm.read_vti_device(str(p), out)
    h, _, _ = pnm.SDFReader.read_vti(str(p))
    n = h.size
    got = t.cpu().numpy()
    assert np.array_equal(got[:n].view(np.uint32), h.reshape(-1).view(np.uint32))
    assert np.all(got[n:] == 7.0)  # nothing past the volume is touched


def test_read_vti_device_then_extract(gpu, port, torch, tmp_path):
    """File -> device -> network without the volume passing through host arrays."""
    pnm, _ = gpu
    from peclet_pnm_gb300 import device
    from peclet_pnm_gb300 import synthetic as syn

    sdf = syn.packing((40, 48, 56), 0.4, seed=7)
    p = tmp_path / "pk.vti"
    pnm.write_sdf_vti(str(p), sdf, [0.0, 0.0, 0.0], [1.0, 1.0, 1.0])
    t, org, spc = pnm.read_vti_device(str(p))
    pores, seg, pairs = device.extract_pore_network_device(t, org, spc)
    op, oseg, opairs = port.extract_pore_network(sdf, org, spc)
    assert np.array_equal(sorted_pores(pores.cpu().numpy()).view(np.int32),
                          sorted_pores(op).view(np.int32))
    assert np.array_equal(pairs.cpu().numpy(), np.asarray(opairs).reshape(-1, 2))


# ---- post-processing on the device ------------------------------------------------------------
@pytest.mark.parametrize("case", standard_cases()[:5], ids=lambda c: c[0])
def test_network_stats_device_matches_host(gpu, torch, case):
    """pnm_flow_stats_dev against the numpy arithmetic of the reference demo: conductance
    bitwise (IEEE division on both sides), counts and maxima exact, means within 1e-12."""
    pnm, _ = gpu
    from peclet_pnm_gb300 import device

    name, sdf, org, spc = case
    f = flow_fields(sdf)
    r = device.extract_network_flow_device(torch.from_numpy(sdf).cuda(), org, spc,
                                           *[torch.from_numpy(x).cuda() for x in f[:4]])
    hs = pnm.network_stats({k: v.cpu().numpy() for k, v in r.items()})
    ds = pnm.network_stats(r)
    assert ds["conductance"].is_cuda
    assert np.array_equal(ds["conductance"].cpu().numpy().view(np.uint64),
                          hs["conductance"].view(np.uint64))
    assert np.array_equal(ds["coordination"].cpu().numpy(), hs["coordination"])
    for k in ("n_pores", "n_throats", "max_abs_flow", "max_abs_residual", "max_coordination",
              "frac_positive_conductance", "all_conductance_finite", "mass_balance_ok",
              "mean_coordination"):
        assert ds[k] == hs[k], (k, ds[k], hs[k])
    for k in ("mean_abs_flow", "mean_abs_dp"):
        assert abs(ds[k] - hs[k]) <= 1e-12 * abs(hs[k]), k


def test_network_stats_device_special_values(gpu, torch):
    pnm, _ = gpu
    net = {"pore_residual": np.array([1e-12, -3e-12, np.nan, 2e-12]),
           "throats": np.array([[1, 2], [1, 3], [2, 3], [2, 3], [3, 4]], np.int32),
           "throat_flow": np.array([2.0, -1.0, 0.5, 0.0, 4.0]),
           "throat_dp": np.array([1.0, 2.0, -0.5, 0.0, 0.0])}
    hs = pnm.network_stats(net)
    ds = pnm.network_stats({k: torch.from_numpy(v).cuda() for k, v in net.items()})
    g = ds["conductance"].cpu().numpy()
    assert np.array_equal(np.isnan(g), np.isnan(hs["conductance"]))
    assert np.array_equal(g[~np.isnan(g)], hs["conductance"][~np.isnan(hs["conductance"])])
    assert math.isnan(ds["max_abs_residual"]) and math.isnan(hs["max_abs_residual"])
    for k in ("frac_positive_conductance", "all_conductance_finite", "mass_balance_ok",
              "max_coordination", "max_abs_flow"):
        assert ds[k] == hs[k], k
    assert ds["coordination"].cpu().tolist() == [2, 3, 4, 1]
    big = 300_000  # several blocks of partials
    rng = np.random.default_rng(9)
    net2 = {"pore_residual": rng.normal(0, 1e-9, 50_000),
            "throats": rng.integers(1, 50_001, (big, 2)).astype(np.int32),
            "throat_flow": rng.normal(0, 1, big), "throat_dp": rng.normal(0, 1, big)}
    hs2 = pnm.network_stats(net2)
    ds2 = pnm.network_stats({k: torch.from_numpy(v).cuda() for k, v in net2.items()})
    assert np.array_equal(ds2["coordination"].cpu().numpy(), hs2["coordination"])
    assert ds2["max_abs_flow"] == hs2["max_abs_flow"]
    assert abs(ds2["mean_abs_flow"] - hs2["mean_abs_flow"]) <= 1e-12 * hs2["mean_abs_flow"]


def test_device_call_keeps_the_callers_context_stream(gpu, torch):
    """A device call runs on the current torch stream and then restores the stream the caller had
    set on the context."""
    pnm, _ = gpu
    from peclet_pnm_gb300 import device
    from peclet_pnm_gb300 import synthetic as syn

    ctx = pnm.Context(0)
    own = torch.cuda.Stream()
    ctx.set_stream(own.cuda_stream)
    sdf = syn.sphere_lattice(36, 30, 24)
    seg = device.segment_volume_device(torch.from_numpy(sdf).cuda(), [1, 1, 1], ctx=ctx)
    torch.cuda.synchronize()
    assert ctx.stream_ptr == own.cuda_stream
    assert np.array_equal(seg.cpu().numpy().reshape(-1), pnm.segment_volume(sdf, [1, 1, 1], numpy=True))
    ctx.close()


def test_read_vti_device_rejects_host_destinations(gpu, torch, tmp_path):
    pnm, ctx = gpu
    from peclet_pnm_gb300 import _capi

    p = tmp_path / "h.vti"
    pnm.write_sdf_vti(str(p), np.ones((2, 3, 4), np.float32))
    with pytest.raises(RuntimeError, match="CUDA tensor"):
        pnm.read_vti_device(str(p), torch.zeros(24))
    host = torch.zeros(24, pin_memory=True)
    rc = _capi.pnm_read_vti_dev(ctx.h, str(p).encode(), host.data_ptr(), 24)
    assert rc == _capi.PNM_ERR_ARG
    assert host.sum().item() == 0.0
