"""The distributed surface (the reference's *_mpi functions) on CPU: two and four gloo ranks, each
passing its z-slab block. The compute step is the oracle here (no GPU); what is tested is the host logic
the GPU path shares: the decomposition, the all-gather of the blocks, the pore ownership by peak
voxel, the slicing of the labels, and that every rank's flow result is the global one."""
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
TESTS = os.path.dirname(os.path.abspath(__file__))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _volume():
    sys.path.insert(0, ROOT)
    from peclet_pnm_gb300 import synthetic as syn

    return syn.packing((21, 18, 24), 0.45, mean_r=4.0, seed=77)


def _peak_voxels(sdf):
    """Strict lexicographic (value, wrapped index) maxima with sdf > 0, in voxel order: the pore
    peaks of pore_extraction.hpp:89-106, for a volume without NaN."""
    nz, ny, nx = sdf.shape
    idx = np.arange(sdf.size).reshape(sdf.shape)
    peak = sdf > 0
    for dz in (-1, 0, 1):
        for dy in (-1, 0, 1):
            for dx in (-1, 0, 1):
                if dx == dy == dz == 0:
                    continue
                nv = np.roll(sdf, (-dz, -dy, -dx), axis=(0, 1, 2))
                ni = np.roll(idx, (-dz, -dy, -dx), axis=(0, 1, 2))
                peak &= (sdf > nv) | ((sdf == nv) & (idx > ni))
    return np.nonzero(peak.reshape(-1))[0].astype(np.int64)


def _oracle_network(sdf, origin_zyx, spacing_zyx):
    from oracle import Oracle

    pores, seg, pairs = Oracle("port", threads=1).extract_pore_network(sdf, origin_zyx,
                                                                       spacing_zyx)
    return pores, _peak_voxels(np.asarray(sdf, np.float32)), seg, pairs


def _oracle_flow(sdf, origin_zyx, spacing_zyx, u, v, w, p, ox=None, oy=None, oz=None,
                 grad_p_zyx=(0.0, 0.0, 0.0)):
    from oracle import Oracle

    return Oracle("port", threads=1).extract_network_flow(sdf, origin_zyx, spacing_zyx, u, v, w,
                                                          p, ox=ox, oy=oy, oz=oz,
                                                          grad_p_zyx=grad_p_zyx)


def _rank_main(rank, world, port, q):
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    sys.path.insert(0, TESTS)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from cases import flow_fields
        from peclet_pnm_gb300 import distributed as D

        sdf = _volume()
        (z0, _, _), (dz, ny, nx) = D.mpi_block(sdf.shape)
        local = sdf[z0:z0 + dz]
        org, spc = [0.5, -1.0, 2.0], [1.0, 1.0, 1.0]
        pores, seg_local, pairs = D.extract_pore_network_mpi(
            local, sdf.shape, org, spc, numpy=True, _compute=_oracle_network)
        f = flow_fields(sdf)
        blk = [x[z0:z0 + dz] for x in f]
        flow = D.extract_network_flow_mpi(local, sdf.shape, org, spc, *blk[:4], ox=blk[4],
                                          oy=blk[5], oz=blk[6], grad_p_zyx=[1e-3, 0.0, -2e-3],
                                          _compute=_oracle_flow)
        try:
            D.extract_pore_network_mpi(sdf, sdf.shape, org, spc, _compute=_oracle_network)
            mismatch = None
        except RuntimeError as e:
            mismatch = str(e)
        dist.barrier()
        q.put((rank, D.mpi_rank(), D.mpi_size(), z0, dz, pores, seg_local, pairs,
               {k: np.asarray(v) for k, v in flow.items()}, mismatch))
    finally:
        dist.destroy_process_group()


def test_blocks_partition_the_grid():
    from peclet_pnm_gb300 import distributed as D

    for nz, size in [(21, 2), (5, 3), (64, 8), (3, 4)]:
        covered = []
        for r in range(size):
            (z0, y0, x0), (dz, ny, nx) = D.mpi_block((nz, 7, 9), rank=r, size=size)
            assert (y0, x0, ny, nx) == (0, 0, 7, 9)
            covered += list(range(z0, z0 + dz))
        assert covered == list(range(nz))
    # without a process group: one rank owning the whole grid
    assert D.mpi_rank() == 0 and D.mpi_size() == 1
    assert D.mpi_block((4, 5, 6)) == ([0, 0, 0], [4, 5, 6])


@pytest.mark.parametrize("world", [2, 4])
def test_gloo_ranks_match_the_whole_grid(world):
    """2 ranks split the 21 planes 11 + 10; 4 ranks split them 6 + 5 + 5 + 5, and the third
    block holds no pore peak, so that rank owns no pores."""
    pytest.importorskip("torch")
    import torch.multiprocessing as mp

    sys.path.insert(0, TESTS)
    from cases import flow_fields
    from oracle import sorted_pores

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    got = sorted((q.get(timeout=300) for _ in range(world)), key=lambda g: g[0])
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    sdf = _volume()
    org, spc = [0.5, -1.0, 2.0], [1.0, 1.0, 1.0]
    wp, peaks, ws, wq = _oracle_network(sdf, org, spc)
    assert [g[1] for g in got] == list(range(world)) and all(g[2] == world for g in got)
    # labels: the blocks in rank order are the whole grid's labels
    assert got[0][3] == 0 and all(got[r][3] == got[r - 1][3] + got[r - 1][4] for r in range(1, world))
    assert np.array_equal(np.concatenate([g[6] for g in got]), ws)
    # pores: each rank owns those whose peak voxel lies in its block (records in voxel order)
    pz = peaks // (sdf.shape[1] * sdf.shape[2])
    for g in got:
        own = wp[(pz >= g[3]) & (pz < g[3] + g[4])]
        assert np.array_equal(sorted_pores(g[5]).view(np.int32), sorted_pores(own).view(np.int32))
    both = np.concatenate([g[5] for g in got])
    assert np.array_equal(sorted_pores(both).view(np.int32), sorted_pores(wp).view(np.int32))
    # connections and the flow result: global, the same on every rank
    for g in got:
        assert np.array_equal(g[7], wq)
    f = flow_fields(sdf)
    want = _oracle_flow(sdf, org, spc, *f[:4], ox=f[4], oy=f[5], oz=f[6],
                        grad_p_zyx=[1e-3, 0.0, -2e-3])
    for g in got:
        for k in ("pores", "throats", "throat_flow", "pore_pressure", "throat_dp"):
            assert np.array_equal(g[8][k], want[k]), k
        assert g[9] == "sdf_local shape does not match this rank's mpi_block"
