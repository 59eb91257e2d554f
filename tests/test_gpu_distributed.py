"""The distributed surface's GPU compute path in one process (one rank owning the whole grid), and
the pore peak voxels it assigns ownership by, through the C ABI."""
import ctypes

import numpy as np
import pytest

from oracle import sorted_pores
from peclet_pnm_gb300 import synthetic as syn
from test_distributed import _peak_voxels

pytestmark = pytest.mark.gpu


def test_pore_peaks_are_the_record_voxels(gpu):
    torch = pytest.importorskip("torch")
    pnm, ctx = gpu
    from peclet_pnm_gb300 import _capi

    sdf = syn.packing((40, 36, 44), 0.4, seed=41)
    want = _peak_voxels(sdf)
    d = torch.from_numpy(sdf).cuda()
    ids = torch.empty(len(want) + 8, dtype=torch.int32, device="cuda")
    n = _capi._i64()
    torch.cuda.synchronize()
    ctx.check(_capi.pnm_pore_peaks_dev(ctx.h, d.data_ptr(), 44, 36, 40, ids.data_ptr(),
                                       len(want) + 8, ctypes.byref(n)))
    got = ids[:n.value].cpu().numpy()
    assert np.array_equal(got, want)
    pores = pnm.extract_pores(sdf, [0.0] * 3, [1.0] * 3, numpy=True)
    assert np.array_equal(pores[:, 3], sdf.reshape(-1)[got])  # radius = the peak's SDF value
    rc = _capi.pnm_pore_peaks_dev(ctx.h, d.data_ptr(), 44, 36, 40, ids.data_ptr(), 2,
                                  ctypes.byref(n))
    assert rc == _capi.PNM_ERR_CAPACITY and n.value == len(want)


def test_single_rank_mpi_equals_plain(gpu):
    pnm, _ = gpu
    sdf = syn.packing((24, 32, 40), 0.45, seed=42)
    pores, seg, pairs = pnm.extract_pore_network_mpi(sdf, sdf.shape, [0.0] * 3, [1.0] * 3,
                                                     numpy=True)
    wp, ws, wq = pnm.extract_pore_network(sdf, [0.0] * 3, [1.0] * 3, numpy=True)
    assert np.array_equal(seg, ws) and np.array_equal(pairs, wq)
    assert np.array_equal(sorted_pores(pores).view(np.int32), sorted_pores(wp).view(np.int32))
