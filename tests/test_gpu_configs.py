"""GPU parity at the full sizes the benchmark figures are quoted on.

* 512^3 float32 packing (porosity 0.4, log-normal radii mean 10, seed 2): extract_pore_network
  through the C ABI against the oracle (labels, connections, pore set bitwise).
* 256^3 float64 packing (seed 3) with 32-mode Fourier u, v, w, p (seed 4), openness from the face
  SDF, grad_p_zyx [0, 0, -1e-4]: extract_network_flow against the oracle (throat list exact, pores
  and pore_pressure bitwise, FP64 sums per element within 1e-12 of max(|value|, sum of |terms|),
  throat_area within 1e-12 relative, throat_dp within 1e-12 relative).
* The ragged 96-volume batch (edges per axis from {48, ..., 192}, porosity U[0.3, 0.6], seeds
  5 + i): every volume's batched result against the plain per-volume path, bitwise, and a
  sample of the volumes against the oracle.

The algorithm being matched is src/pore_extraction.hpp:157-461 (segmentation, topology) and
:493-997 (network flow); the oracle runs on every host core. The volumes are generated on the
device (the same generators the benchmark uses).
"""
import os

import numpy as np
import pytest

from oracle import Oracle, sorted_pores
from peclet_pnm_gb300 import synthetic as syn
from test_gpu_flow import _check as check_flow

pytestmark = [pytest.mark.gpu, pytest.mark.slow]


@pytest.fixture(scope="module")
def port_all():
    return Oracle("port", threads=os.cpu_count() or 1)


def _bits(p):
    return sorted_pores(p).view(np.int32)


def test_packing_512_matches_oracle(gpu, port_all):
    pnm, ctx = gpu
    sdf = syn.packing((512, 512, 512), 0.4, seed=2, device="cuda").cpu().numpy()
    pores, seg, pairs = pnm.pore_network_arrays(sdf, [0.0] * 3, [1.0] * 3, ctx=ctx)
    st = ctx.stats()
    op, oseg, opairs = port_all.extract_pore_network(sdf, [0.0] * 3, [1.0] * 3)
    assert np.array_equal(seg, oseg), f"seg: {int((seg != oseg).sum())} voxels differ"
    assert np.array_equal(pairs, opairs), f"pairs: {len(pairs)} vs {len(opairs)}"
    assert np.array_equal(_bits(pores), _bits(op)), f"pores: {len(pores)} vs {len(op)}"
    assert st["n_pore_labels"] == int(oseg.max()) and st["n_solid_labels"] == -int(oseg.min())
    assert len(pores) > 50000 and len(pairs) > 200000  # the workload is what it claims to be


def test_network_flow_256_matches_oracle(gpu, port_all):
    import torch

    pnm, ctx = gpu
    n = 256
    dsdf = syn.packing((n, n, n), 0.4, seed=3, dtype=np.float64, device="cuda")
    fields = [f.cpu().numpy() for f in syn.fourier_fields_device(dsdf)]
    sdf = dsdf.cpu().numpy()
    del dsdf
    torch.cuda.empty_cache()
    gp = [0.0, 0.0, -1e-4]
    kw = dict(ox=fields[4], oy=fields[5], oz=fields[6])
    r = pnm.network_flow_arrays(sdf, [0.0] * 3, [1.0] * 3, *fields[:4], grad_p_xyz=gp[::-1],
                                ctx=ctx, **kw)
    o = port_all.extract_network_flow(sdf, [0.0] * 3, [1.0] * 3, *fields[:4], grad_p_zyx=gp, **kw)
    check_flow(r, o)
    assert len(r["throats"]) > 10000


def test_ragged_batch_96_equals_plain(gpu, port_all):
    import torch

    pnm, ctx = gpu
    shapes = syn.batch_shapes(96)
    vols = [syn.packing(sh, phi, seed=sd, device="cuda").cpu().numpy() for sh, phi, sd in shapes]
    torch.cuda.empty_cache()
    b = pnm.Batch([v.shape for v in vols])
    try:
        for i, v in enumerate(vols):
            b.set_sdf(i, v)
        b.run()
        got = b.results()
    finally:
        b.close()
    for i, v in enumerate(vols):
        gp, gs, gq = got[i]
        pp, ps, pq = pnm.pore_network_arrays(v, [0.0] * 3, [1.0] * 3, ctx=ctx)
        assert np.array_equal(gs, ps), f"volume {i}: seg, {int((gs != ps).sum())} voxels differ"
        assert np.array_equal(gq, pq), f"volume {i}: pairs {len(gq)} vs {len(pq)}"
        assert np.array_equal(gp.view(np.int32), pp.view(np.int32)), f"volume {i}: pores"
    for i in (0, 17, 58, 95):  # and a sample against the oracle
        op, oseg, opairs = port_all.extract_pore_network(vols[i], [0.0] * 3, [1.0] * 3)
        gp, gs, gq = got[i]
        assert np.array_equal(gs, oseg) and np.array_equal(gq, opairs), f"volume {i}"
        assert np.array_equal(_bits(gp), _bits(op)), f"volume {i}: pores"
