"""The allocation-free extract_pores entry point, through the C ABI.

It serves callers that cannot let a library allocate device memory (frameworks that hand out
all device memory from their own budgeted pool, serving loops that must not enter the driver's
allocator mid-stream): they pass device input/output buffers and a stream, and the entry point
works in a static scratch array of the library. Checked here against the regular entry point
(pnm_extract_pores) on two calls in a row — the scratch keeps the previous call's contents, so
the second call shows that the entry point clears what it must — and for its size limit.
This file is collected last so that a failure here leaves every other test already run.
"""
import ctypes

import numpy as np
import pytest

from peclet_pnm_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu


def _regular(pnm, sdf):
    return pnm.pores_array(sdf, [0.0, 0.0, 0.0], [1.0, 1.0, 1.0])


def _noalloc(capi, torch, sdf, cap=200000, rows=None, stream=None):
    """Runs the entry point on `stream` (default: torch's current stream) into an output of
    `rows` records (default: cap) filled with a canary value; returns (rc, output, count)."""
    rows = cap if rows is None else rows
    st = stream if stream is not None else torch.cuda.current_stream()
    with torch.cuda.stream(st):
        d_sdf = torch.from_numpy(np.ascontiguousarray(sdf, np.float32)).cuda()
        d_out = torch.full((rows, 4), -7.5, dtype=torch.float32, device="cuda")
    nz, ny, nx = sdf.shape
    o = np.zeros(3, np.float32)
    s = np.ones(3, np.float32)
    n = capi._i64()
    rc = capi.pnm_extract_pores_noalloc(d_sdf.data_ptr(), nx, ny, nz, capi.as_ptr(o),
                                        capi.as_ptr(s), d_out.data_ptr(), cap, ctypes.byref(n),
                                        st.cuda_stream)
    st.synchronize()
    return rc, d_out.cpu().numpy(), n.value


def test_noalloc_matches_regular_entry_point_twice():
    torch = pytest.importorskip("torch")
    import peclet_pnm_gb300 as pnm
    from peclet_pnm_gb300 import _capi

    a = syn.packing((72, 80, 96), 0.4, seed=51)  # many pores: fills much of the scratch
    b = syn.sphere_lattice(36, 30, 24)          # few pores: stale bits would show up
    for sdf in (a, b):
        rc, got, n = _noalloc(_capi, torch, sdf)
        assert rc == _capi.PNM_OK
        want = _regular(pnm, sdf)
        assert n == len(want)
        # same voxel order, bitwise
        assert np.array_equal(got[:n].view(np.int32), want.view(np.int32))


def test_noalloc_capacity_and_side_stream():
    """pore_cap below the count: PNM_ERR_CAPACITY, the full count reported, only the first
    pore_cap records written; then a call on a fresh (non-default) stream."""
    torch = pytest.importorskip("torch")
    import peclet_pnm_gb300 as pnm
    from peclet_pnm_gb300 import _capi

    sdf = syn.packing((72, 80, 96), 0.4, seed=51)
    want = _regular(pnm, sdf)
    assert len(want) > 3
    rc, got, n = _noalloc(_capi, torch, sdf, cap=3, rows=8)
    assert rc == _capi.PNM_ERR_CAPACITY and n == len(want)
    assert np.array_equal(got[:3].view(np.int32), want[:3].view(np.int32))
    assert np.all(got[3:] == np.float32(-7.5)), "records past pore_cap were written"
    side = torch.cuda.Stream()
    rc, got, n = _noalloc(_capi, torch, sdf, stream=side)
    assert rc == _capi.PNM_OK and n == len(want)
    assert np.array_equal(got[:n].view(np.int32), want.view(np.int32))


def test_noalloc_rejects_volumes_beyond_its_scratch():
    pytest.importorskip("torch")
    from peclet_pnm_gb300 import _capi

    o = np.zeros(3, np.float32)
    s = np.ones(3, np.float32)
    n = _capi._i64()
    # 1024*1024*128 = 2^27 voxels > 2^26: rejected before any device access
    rc = _capi.pnm_extract_pores_noalloc(None, 1024, 1024, 128, _capi.as_ptr(o), _capi.as_ptr(s),
                                         None, 0, ctypes.byref(n), None)
    assert rc == _capi.PNM_ERR_SHAPE and n.value == 0
