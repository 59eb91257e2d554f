"""GPU parity of the batched path: every volume of a ragged batch equals the CPU oracle (and so
the plain per-volume path) bit for bit — labels, connections, pore records — whatever its
neighbours in the batch, with and without graph replay, across re-runs and capacity growth."""
import numpy as np
import pytest

from cases import edge_cases, random_volume, standard_cases
from oracle import sorted_pores
from peclet_pnm_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu


def _bits(p):
    return sorted_pores(p).view(np.int32)


def _check(i, got, want):
    gp, gs, gq = got
    op, os_, oq = want
    assert np.array_equal(gs, os_), f"volume {i}: seg, {int((gs != os_).sum())} voxels differ"
    assert np.array_equal(gq, oq), f"volume {i}: pairs {len(gq)} vs {len(oq)}"
    # batch pores are in voxel order, like the plain path; compare as exact bit patterns
    assert np.array_equal(_bits(gp), _bits(op)), f"volume {i}: pores {len(gp)} vs {len(op)}"


def _run(pnm, cases, graph=True):
    b = pnm.Batch([c[1].shape for c in cases], [c[2] for c in cases], [c[3] for c in cases],
                  graph=graph)
    for i, c in enumerate(cases):
        b.set_sdf(i, c[1])
    b.run()
    return b


def test_ragged_batch_matches_oracle(gpu, port):
    pnm, _ = gpu
    cases = standard_cases() + edge_cases()
    b = _run(pnm, cases)
    for i, (name, sdf, org, spc) in enumerate(cases):
        _check(f"{i} {name}", b.result(i), port.extract_pore_network(sdf, org, spc))
    st = b.stats()
    assert st["launches"] > 0 and st["voxels"] == sum(c[1].size for c in cases)
    b.close()


def test_random_volumes_in_one_batch_match_oracle(gpu, port):
    """The 40 seeded random volumes (random shapes from 1 to 20 per axis, anisotropic spacing,
    offset origins) as one ragged batch, with and without graph replay."""
    pnm, _ = gpu
    cases = [(f"r{s}", *random_volume(s)) for s in range(40)]
    want = [port.extract_pore_network(sdf, org, spc) for _, sdf, org, spc in cases]
    for graph in (True, False):
        b = _run(pnm, cases, graph=graph)
        for i, (name, *_rest) in enumerate(cases):
            _check(f"{name} graph={graph}", b.result(i), want[i])
        b.close()


def test_batch_equals_plain_and_graph_replay(gpu):
    pnm, _ = gpu
    rng = np.random.default_rng(12)
    cases = []
    for i in range(9):
        shape = tuple(int(v) for v in rng.choice([17, 32, 33, 48, 64], size=3))
        sdf = syn.packing(shape, float(rng.uniform(0.3, 0.6)), mean_r=4.0, seed=100 + i)
        cases.append((f"p{i}", sdf.astype(np.float32), [0.5, 0.0, -1.0], [1.0, 0.5, 2.0]))
    plain = [pnm.extract_pore_network(c[1], c[2], c[3], numpy=True) for c in cases]
    b = _run(pnm, cases, graph=True)
    first = b.results()
    for i in range(len(cases)):
        _check(i, first[i], plain[i])
    # replays of the captured run give the same answer
    for _ in range(3):
        b.run()
    again = b.results()
    for i in range(len(cases)):
        _check(i, again[i], plain[i])
    # new data in the same shapes
    for i, c in enumerate(cases):
        b.set_sdf(i, -c[1])
    b.run()
    for i, c in enumerate(cases):
        _check(i, b.result(i), pnm.extract_pore_network(-c[1], c[2], c[3], numpy=True))
    b.close()
    e = _run(pnm, cases, graph=False)
    assert not e.uses_graph
    for i in range(len(cases)):
        _check(i, e.result(i), plain[i])
    e.close()


def test_batch_capacity_growth(gpu, port):
    """Dense pair sets and dense peaks overflow the first hash set / pore buffer; the batch grows
    them and re-runs."""
    pnm, _ = gpu
    rng = np.random.default_rng(5)
    z, y, x = np.meshgrid(np.arange(40), np.arange(36), np.arange(42), indexing="ij")
    lattice = np.where((x % 2 == 0) & (y % 2 == 0) & (z % 2 == 0), 2.0, 1.0).astype(np.float32)
    cases = [("noise", rng.normal(0, 1.5, size=(40, 40, 40)).astype(np.float32), [0, 0, 0],
              [1, 1, 1]),
             ("peaks", lattice, [0, 0, 0], [1, 1, 1]),
             ("noise2", rng.normal(0, 1.0, size=(33, 47, 29)).astype(np.float32), [0, 0, 0],
              [1, 1, 1])]
    b = _run(pnm, cases)
    for i, (name, sdf, org, spc) in enumerate(cases):
        _check(f"{i} {name}", b.result(i), port.extract_pore_network(sdf, org, spc))
    b.close()


def test_batch_with_empty_volumes(gpu, port):
    pnm, _ = gpu
    s = syn.sphere_lattice(20, 18, 22)
    cases = [("empty", np.zeros((0, 4, 4), np.float32), [0, 0, 0], [1, 1, 1]),
             ("lattice", s, [0, 0, 0], [1, 1, 1]),
             ("empty2", np.zeros((3, 0, 2), np.float32), [0, 0, 0], [1, 1, 1]),
             ("one", np.ones((1, 1, 1), np.float32), [0, 0, 0], [1, 1, 1])]
    b = _run(pnm, cases)
    for i, (name, sdf, org, spc) in enumerate(cases):
        if sdf.size == 0:
            v = b.volume(i)
            assert v["n_pores"] == 0 and v["n_pairs"] == 0
            continue
        _check(f"{i} {name}", b.result(i), port.extract_pore_network(sdf, org, spc))
    b.close()
    only_empty = pnm.Batch([(0, 0, 0)])
    only_empty.run()
    assert only_empty.volume(0)["n_pores"] == 0
    only_empty.close()


def test_launch_shapes_and_autotune_keep_results(gpu, tmp_path):
    """Every launch shape (tile depth, grids, flood residency) gives the same bits; the autotuner
    picks one, caches it per size class, and re-applies it from the cache."""
    pnm, _ = gpu
    rng = np.random.default_rng(3)
    cases = []
    for i in range(6):
        shape = tuple(int(v) for v in rng.choice([20, 33, 48, 65], size=3))
        cases.append((f"t{i}", syn.packing(shape, 0.45, mean_r=4.0, seed=300 + i)
                      .astype(np.float32), [0, 0, 0], [1, 1, 1]))
    cases.append(edge_cases()[0])
    cases.append(edge_cases()[17])
    want = [pnm.extract_pore_network(c[1], c[2], c[3], numpy=True) for c in cases]
    b = _run(pnm, cases)
    for shape in [dict(tile_z=4), dict(tile_z=16, blocks_per_sm=4), dict(ccl_blocks_per_sm=32),
                  dict(tile_z=8, flood_blocks_per_sm=1, blocks_per_sm=16),
                  dict(flood_blocks_per_sm=4, tile_z=16)]:
        b.set_tuning(**shape)
        b.run()
        assert {k: b.tuning[k] for k in shape} == shape
        for i in range(len(cases)):
            _check(f"{shape} {i}", b.result(i), want[i])
    cache = str(tmp_path / "tune.txt")
    got = b.autotune(cache=cache, reps=1)
    assert got["tile_z"] in (4, 8, 16) and got["ms"] > 0
    assert open(cache).read().count("|e") == 1
    b.run()
    assert b.uses_graph
    for i in range(len(cases)):
        _check(f"tuned {i}", b.result(i), want[i])
    b.close()
    b2 = _run(pnm, cases)
    again = b2.autotune(cache=cache)  # cached: applied without timing
    assert again["ms"] == 0.0 and {k: again[k] for k in b2.tuning} == \
        {k: got[k] for k in b2.tuning}
    b2.close()
