"""C-ABI library checks that need no GPU: the library loads, exports every symbol the public
header declares, rejects bad arguments with the reference binding's errors before touching a
device, and never routes through the oracle."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "pnm_gb300.h")


def declared_symbols():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(pnm_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    from peclet_pnm_gb300 import _capi

    syms = declared_symbols()
    assert len(syms) >= 14
    for s in syms:
        assert hasattr(_capi.lib, s), f"{s} not exported"
    assert sorted(_capi.EXPORTED) == syms


def test_null_context_is_rejected():
    from peclet_pnm_gb300 import _capi

    a = np.zeros((2, 2, 2), np.float32)
    o = np.zeros(3, np.float32)
    s = np.ones(3, np.float32)
    seg = np.zeros(8, np.int32)
    assert _capi.pnm_segment_volume(None, _capi.as_ptr(a), 2, 2, 2, _capi.as_ptr(s),
                                    _capi.as_ptr(seg)) == _capi.PNM_ERR_ARG
    pp = ctypes.POINTER(_capi.PnmPore)()
    n = _capi._i64()
    assert _capi.pnm_extract_pores(None, _capi.as_ptr(a), 2, 2, 2, _capi.as_ptr(o),
                                   _capi.as_ptr(s), ctypes.byref(pp), ctypes.byref(n)) == \
        _capi.PNM_ERR_ARG
    assert _capi.pnm_ctx_set_stream(None, None) == _capi.PNM_ERR_ARG
    assert _capi.pnm_ctx_set_timing(None, 1) == _capi.PNM_ERR_ARG
    assert _capi.pnm_ctx_set_wait_limit(None, 1000, 0) == _capi.PNM_ERR_ARG


def test_stats_struct_matches_header():
    """pnm_stats in the header ends with stage_ms[PNM_STAGE_COUNT]; the ctypes mirror has the
    same stage count and names every PNM_STAGE_* in order."""
    from peclet_pnm_gb300 import _capi

    text = open(HEADER).read()
    count = int(re.search(r"#define PNM_STAGE_COUNT (\d+)", text).group(1))
    stages = re.findall(r"#define PNM_STAGE_([A-Z_]+) (\d+)", text)
    ids = {name: int(v) for name, v in stages if name != "COUNT"}
    assert sorted(ids.values()) == list(range(count)) == list(range(len(_capi.STAGES)))
    for name, i in ids.items():
        assert _capi.STAGES[i] == name.lower()
    assert _capi.PnmStats.stage_ms.size == count * 8


def test_no_cpu_fallback_without_device():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from peclet_pnm_gb300 import _capi

    h = ctypes.c_void_p()
    assert _capi.pnm_ctx_create(0, ctypes.byref(h)) == _capi.PNM_ERR_NO_DEVICE
    import peclet_pnm_gb300 as pnm

    with pytest.raises(pnm.PnmError):
        pnm.extract_pore_network(np.ones((4, 4, 4), np.float32), [0] * 3, [1] * 3)


def test_argument_errors_match_reference_binding():
    import peclet_pnm_gb300 as pnm

    with pytest.raises(RuntimeError, match=r"SDF array must be 3D \(Nz,Ny,Nx\)"):
        pnm.extract_pores(np.zeros((4, 4), np.float32), [0] * 3, [1] * 3)
    sdf = np.zeros((3, 4, 5), np.float32)
    good = np.zeros((3, 4, 5))
    with pytest.raises(RuntimeError, match=r"u must be \(Nz,Ny,Nx\) matching the SDF"):
        pnm.extract_network_flow(sdf, [0] * 3, [1] * 3, np.zeros((3, 4, 4)), good, good, good)
    with pytest.raises(RuntimeError, match=r"pass all three openness arrays"):
        pnm.extract_network_flow(sdf, [0] * 3, [1] * 3, good, good, good, good, ox=good)


def test_empty_volume_returns_empty_without_device():
    import peclet_pnm_gb300 as pnm

    e = np.zeros((0, 5, 5), np.float32)
    assert pnm.extract_pores(e, [0] * 3, [1] * 3) == []
    assert pnm.segment_volume(e, [1] * 3) == []
    pores, seg, conns = pnm.extract_pore_network(e, [0] * 3, [1] * 3)
    assert pores == [] and seg == [] and conns == []
    assert pnm.extract_topology_gpu([], [0, 0, 0]) == []


def test_pore_fields_are_float32():
    import peclet_pnm_gb300 as pnm

    p = pnm.Pore()
    p.x = 0.1
    assert p.x == float(np.float32(0.1))
    p.radius = 3
    assert p.radius == 3.0


def test_product_never_imports_the_oracle():
    pkg = os.path.join(ROOT, "peclet_pnm_gb300")
    for dirpath, _, files in os.walk(pkg):
        for f in files:
            if f.endswith((".py", ".cu", ".cuh", ".h", ".cpp")):
                text = open(os.path.join(dirpath, f)).read()
                assert not re.search(r"^\s*(from|import)\s+oracle\b", text, re.M), f
                assert "libpnm_oracle" not in text and "libpnm_ref" not in text, f


def test_batch_planning_without_device():
    """Batch layout and admission sizes are host arithmetic: 32-voxel-aligned volume offsets,
    monotone plan bytes, and the reference binding's argument errors."""
    import peclet_pnm_gb300 as pnm
    from peclet_pnm_gb300 import _capi

    small = pnm.batch_plan_bytes([(8, 8, 8)])
    two = pnm.batch_plan_bytes([(8, 8, 8), (9, 7, 5)])
    big = pnm.batch_plan_bytes([(64, 64, 64)])
    assert 0 < small < two < big
    # about 50 device bytes per voxel once the fixed parts are amortised
    per_voxel = (pnm.batch_plan_bytes([(256, 256, 256)]) - big) / (256 ** 3 - 64 ** 3)
    assert 30 < per_voxel < 80
    d = np.array([[4, 4, -1]], np.int32)
    out = _capi._i64()
    assert _capi.pnm_batch_plan_bytes(1, _capi.as_ptr(d), ctypes.byref(out)) == _capi.PNM_ERR_ARG
    d = np.array([[2048, 2048, 1024]], np.int32)
    assert _capi.pnm_batch_plan_bytes(1, _capi.as_ptr(d), ctypes.byref(out)) == \
        _capi.PNM_ERR_SHAPE
    assert _capi.pnm_batch_plan_bytes(0, None, ctypes.byref(out)) == _capi.PNM_ERR_ARG
    h = ctypes.c_void_p()
    dims = np.array([[4, 4, 4]], np.int32)
    f = np.zeros(3, np.float32)
    assert _capi.pnm_batch_create(None, 1, _capi.as_ptr(dims), _capi.as_ptr(f), _capi.as_ptr(f),
                                  0, ctypes.byref(h)) == _capi.PNM_ERR_ARG
    assert _capi.pnm_server_create(None, None, ctypes.byref(h)) == _capi.PNM_ERR_ARG
    t = _capi._i64()
    assert _capi.pnm_server_submit(None, None, 1, 1, 1, _capi.as_ptr(f), _capi.as_ptr(f),
                                   ctypes.byref(t)) == _capi.PNM_ERR_ARG
    assert _capi.pnm_batch_run(None) == _capi.PNM_ERR_ARG
    assert _capi.pnm_server_wait(None, 1, 0.0) == _capi.PNM_ERR_ARG
