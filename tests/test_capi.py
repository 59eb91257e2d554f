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
