"""Bounded device waits and per-stage timing, through the C ABI.

The persistent flood loop runs every Jacobi sweep of the reference's flood
(src/pore_extraction.hpp:237-269) in one cooperative launch with a grid barrier between phases.
Each barrier wait is bounded. Here a context makes the barrier wait for one arrival beyond the
grid, which never comes, so every block's wait runs out after a short limit: the call must fail
with PNM_ERR_NOT_CONVERGED (the reference's counterpart is the non-convergence abort of its
distributed flood, src/pore_extraction_mpi.hpp:679), and the same context must then produce the
oracle's result. No device fault is involved: the kernel returns on its own.
"""
import numpy as np
import pytest

from cases import edge_cases
from oracle import sorted_pores
from peclet_pnm_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu


def _case(name):
    for c in edge_cases():
        if c[0] == name:
            return c
    raise KeyError(name)


def _xyz(v):
    return [v[2], v[1], v[0]]


def test_flood_barrier_wait_runs_out_then_context_recovers(port):
    import peclet_pnm_gb300 as pnm
    from peclet_pnm_gb300 import _capi

    _, sdf, org, spc = _case("deep_flood_serpentine")  # many flood layers: the loop runs
    ctx = pnm.Context(0)
    try:
        ctx.set_wait_limit(2_000_000, extra_arrivals=1)  # 2 ms per wait, a barrier never met
        with pytest.raises(pnm.PnmError) as ei:
            pnm.pore_network_arrays(sdf, _xyz(org), _xyz(spc), ctx=ctx)
        assert ei.value.code == _capi.PNM_ERR_NOT_CONVERGED
        assert "barrier" in str(ei.value)
        ctx.set_wait_limit()  # back to the default limit, no extra arrivals
        pores, seg, pairs = pnm.pore_network_arrays(sdf, _xyz(org), _xyz(spc), ctx=ctx)
        op, oseg, opairs = port.extract_pore_network(sdf, org, spc)
        assert np.array_equal(seg, oseg)
        assert np.array_equal(pairs, opairs)
        assert np.array_equal(sorted_pores(pores).view(np.int32),
                              sorted_pores(op).view(np.int32))
        assert ctx.stats()["flood_sweeps"] > 3
    finally:
        ctx.close()


def test_stage_times_cover_the_call():
    import peclet_pnm_gb300 as pnm

    sdf = syn.packing((64, 72, 80), 0.4, seed=12)
    ctx = pnm.Context(0)
    try:
        pnm.pore_network_arrays(sdf, [0.0] * 3, [1.0] * 3, ctx=ctx)
        assert all(v == 0.0 for v in ctx.stats()["stage_ms"].values())  # timing is off
        ctx.set_timing(True)
        pnm.pore_network_arrays(sdf, [0.0] * 3, [1.0] * 3, ctx=ctx)
        st = ctx.stats()["stage_ms"]
        for k in ("sdf_pass", "merge_markers", "gradient_path", "flood", "relabel", "seg_pairs",
                  "pair_sort", "pores"):
            assert st[k] > 0.0, k
        assert st["network_flow"] == 0.0
        assert sum(st.values()) < 1000.0
        ctx.set_timing(False)
        pnm.pore_network_arrays(sdf, [0.0] * 3, [1.0] * 3, ctx=ctx)
        assert all(v == 0.0 for v in ctx.stats()["stage_ms"].values())
    finally:
        ctx.close()
