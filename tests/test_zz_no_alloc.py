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


def _noalloc(capi, torch, sdf, cap=200000):
    d_sdf = torch.from_numpy(np.ascontiguousarray(sdf, np.float32)).cuda()
    d_out = torch.empty((cap, 4), dtype=torch.float32, device="cuda")
    nz, ny, nx = sdf.shape
    o = np.zeros(3, np.float32)
    s = np.ones(3, np.float32)
    n = capi._i64()
    stream = torch.cuda.current_stream().cuda_stream
    rc = capi.pnm_extract_pores_noalloc(d_sdf.data_ptr(), nx, ny, nz, capi.as_ptr(o),
                                        capi.as_ptr(s), d_out.data_ptr(), cap, ctypes.byref(n),
                                        stream)
    return rc, d_out[: n.value].cpu().numpy(), n.value


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
        assert np.array_equal(got.view(np.int32), want.view(np.int32))  # same voxel order, bitwise


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
