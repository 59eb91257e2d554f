"""The serving loop on the GPU: results identical alone and in the mix (continuous batching
across concurrent streams), device-resident inputs, admission by memory budget, refusals,
cancellation, and that the server keeps serving after each of them."""
import numpy as np
import pytest

from cases import edge_cases, random_volume
from oracle import sorted_pores
from peclet_pnm_gb300 import PnmError, synthetic as syn
from peclet_pnm_gb300._capi import PNM_ERR_ARG, PNM_ERR_CAPACITY, PNM_OK

pytestmark = pytest.mark.gpu


def _same(got, want, what):
    gp, gs, gq = got
    wp, ws, wq = want
    assert np.array_equal(gs, ws), f"{what}: labels differ in {int((gs != ws).sum())} voxels"
    assert np.array_equal(gq, wq), f"{what}: pairs {len(gq)} vs {len(wq)}"
    assert np.array_equal(sorted_pores(gp).view(np.int32), sorted_pores(wp).view(np.int32)), what


def _mix(n, seed=31):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        e = int(np.exp(rng.uniform(np.log(24), np.log(72))))
        shape = (e, int(rng.integers(20, 70)), int(rng.integers(20, 70)))
        sdf = syn.packing(shape, float(rng.uniform(0.3, 0.6)), mean_r=5.0, seed=200 + i)
        out.append((sdf.astype(np.float32), [0.0, 1.0, 2.0], [1.0, 1.0, 0.5]))
    return out


def test_results_identical_alone_and_in_the_mix(gpu):
    pnm, _ = gpu
    big = syn.packing((160, 160, 160), 0.45, mean_r=8.0, seed=9).astype(np.float32)
    reqs = [(big, [0, 0, 0], [1, 1, 1])] + _mix(20) + \
        [(c[1], c[2], c[3]) for c in edge_cases()[10:16]]
    with pnm.Server(max_inflight=2) as srv:
        tickets = [srv.submit(*r) for r in reqs]
        for t in tickets:
            assert srv.wait(t, 120.0) == PNM_OK, srv.state(t)
        st = srv.stats()
        assert st["completed"] == len(reqs) and st["failed"] == 0
        assert st["batches"] < len(reqs), "arrivals during a run were not coalesced"
        assert st["p99_ms"] >= st["p50_ms"] > 0 and st["gvoxel_per_s"] > 0
        for t, r in zip(tickets, reqs):
            _same(srv.result(t), pnm.extract_pore_network(*r, numpy=True), f"ticket {t}")
            srv.release(t)
        st = srv.stats()  # only idle batches kept for reuse still hold memory
        assert st["running"] == 0 and st["queued"] == 0
        assert (st["bytes_in_use"] == 0) == (st["cached"] == 0)


def test_random_volumes_served_match_oracle(gpu, port):
    """The 40 seeded random volumes (random shapes from 1 to 20 per axis, anisotropic spacing,
    offset origins) submitted at once, so they are coalesced into shared batches."""
    pnm, _ = gpu
    reqs = [random_volume(s) for s in range(40)]
    with pnm.Server(max_inflight=2) as srv:
        tickets = [srv.submit(*r) for r in reqs]
        for t in tickets:
            assert srv.wait(t, 60.0) == PNM_OK, srv.state(t)
        for t, r in zip(tickets, reqs):
            _same(srv.result(t), port.extract_pore_network(*r), f"ticket {t}")
            srv.release(t)


def test_device_resident_inputs(gpu):
    import torch

    pnm, _ = gpu
    reqs = _mix(6, seed=5)
    dev = [torch.from_numpy(r[0]).cuda() for r in reqs]
    torch.cuda.synchronize()
    with pnm.Server() as srv:
        tickets = [srv.submit(d, r[1], r[2]) for d, r in zip(dev, reqs)]
        for t, r in zip(tickets, reqs):
            assert srv.wait(t, 60.0) == PNM_OK
            _same(srv.result(t), pnm.extract_pore_network(*r, numpy=True), f"ticket {t}")


def test_budget_refusal_cancel_and_recovery(gpu):
    pnm, _ = gpu
    small = _mix(4, seed=8)
    huge = np.ones((256, 256, 256), np.float32)
    big = syn.packing((192, 192, 192), 0.4, mean_r=8.0, seed=4).astype(np.float32)
    budget = int(pnm.batch_plan_bytes([big.shape]) * 1.3)
    assert pnm.batch_plan_bytes([huge.shape]) > budget
    # one slot, one request per batch: a request submitted while another runs stays queued
    with pnm.Server(budget_bytes=budget, max_inflight=1, max_batch_volumes=1) as srv:
        t_huge = srv.submit(huge)  # can never fit the budget: refused, the loop goes on
        assert srv.wait(t_huge, 60.0) == PNM_ERR_CAPACITY
        assert srv.state(t_huge)[0] == "failed"
        with pytest.raises(PnmError) as e:
            srv.submit(small[0][0], [0, 0, 0], [0.0, 1.0, 1.0])
        assert e.value.code == PNM_ERR_ARG
        # one slot: the second request waits in the queue while the first runs
        t1 = srv.submit(big)
        t2 = srv.submit(*small[1])
        srv.cancel(t2)
        assert srv.state(t2)[0] == "cancelled"
        with pytest.raises(PnmError):
            srv.cancel(t1)  # running or done: not cancellable
        assert srv.wait(t1, 60.0) == PNM_OK
        _same(srv.result(t1), pnm.extract_pore_network(big, [0, 0, 0], [1, 1, 1], numpy=True),
              "big")
        # held results count against the budget until released
        ts = [srv.submit(*r) for r in small]
        srv.release(t1)
        for t, r in zip(ts, small):
            assert srv.wait(t, 60.0) == PNM_OK
            _same(srv.result(t), pnm.extract_pore_network(*r, numpy=True), f"ticket {t}")
        st = srv.stats()
        assert st["peak_bytes"] <= budget
        assert st["cancelled"] == 1 and st["failed"] == 1


def test_batch_reuse_keeps_results(gpu):
    """Released batches are reused for later requests of the same shapes (new origin and spacing,
    graph replay); every reused run still equals the request alone."""
    pnm, _ = gpu
    vols = _mix(3, seed=21)
    with pnm.Server(max_inflight=1, max_batch_volumes=1) as srv:
        for rep in range(3):
            for i, (sdf, org, spc) in enumerate(vols):
                spc2 = [spc[0] * (1.0 + 0.25 * rep), spc[1], spc[2] * (1.0 + 0.5 * rep)]
                org2 = [org[0] + rep, org[1] - rep, org[2]]
                t = srv.submit(sdf, org2, spc2)
                assert srv.wait(t, 60.0) == PNM_OK
                _same(srv.result(t), pnm.extract_pore_network(sdf, org2, spc2, numpy=True),
                      f"rep {rep} volume {i}")
                srv.release(t)
        st = srv.stats()
        assert st["cache_hits"] >= 6 and st["cached"] >= 1
