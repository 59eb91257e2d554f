"""VTI ingest and output (CPU): the native reader against the reference reader's recorded outputs
(tests/golden/vti/cases.npz, made by tests/golden/make_vti_golden.py from src/sdf_reader.cpp),
the writer against the reference writer's bytes (scripts/vti.py), round trips and error paths."""
from __future__ import annotations

import os

import numpy as np
import pytest

import peclet_pnm_gb300 as pnm
from peclet_pnm_gb300 import vti

GOLDEN = np.load(os.path.join(os.path.dirname(__file__), "golden", "vti", "cases.npz"))
READER_CASES = sorted({k.split("__")[0] for k in GOLDEN.files if not k.startswith("writer__")})


@pytest.mark.parametrize("name", READER_CASES)
def test_reader_matches_reference(tmp_path, name):
    p = tmp_path / f"{name}.vti"
    p.write_bytes(GOLDEN[f"{name}__file"].tobytes())
    sdf, org, spc = pnm.SDFReader.read_vti(str(p))
    nx, ny, nz = (int(v) for v in GOLDEN[f"{name}__dims"])
    assert sdf.shape == (nz, ny, nx) and sdf.dtype == np.float32
    assert sdf.flags.c_contiguous
    ref = GOLDEN[f"{name}__values"]
    assert np.array_equal(sdf.reshape(-1).view(np.uint32), ref.view(np.uint32))
    assert org == [float(v) for v in GOLDEN[f"{name}__origin"][::-1]]
    assert spc == [float(v) for v in GOLDEN[f"{name}__spacing"][::-1]]


def test_header(tmp_path):
    p = tmp_path / "h.vti"
    p.write_bytes(GOLDEN["offset_extent__file"].tobytes())
    h = vti.read_vti_header(str(p))
    assert h["dims_xyz"] == (7, 5, 3)
    assert h["data_bytes"] == 7 * 5 * 3 * 4
    assert np.array_equal(h["origin_xyz"], np.float32([1e-3, -2.5e2, 7]))


def test_save_vti_matches_reference_writer(tmp_path):
    fields = {k.split("__")[2]: GOLDEN[k] for k in GOLDEN.files if k.startswith("writer__field")}
    assert list(fields) == ["Labels", "SDF", "vel"]
    p = tmp_path / "w.vti"
    pnm.save_vti(str(p), fields, spacing=(0.5, 0.25, 1.0), origin=(0.10000000149011612, -2.0, 3.5))
    assert p.read_bytes() == GOLDEN["writer__bytes"].tobytes()


WRITER = np.load(os.path.join(os.path.dirname(__file__), "golden", "vti", "writer_cases.npz"))


@pytest.mark.parametrize("i", range(8))
def test_save_vti_matches_reference_writer_more(tmp_path, i):
    """Every integer width (written as Int32), float16 / 32 / 64, bool, vector fields, integer
    spacing and float origins, against the reference writer's bytes."""
    names = [str(n) for n in WRITER[f"w{i}__names"]]
    fields = {n: WRITER[f"w{i}__f{j}"] for j, n in enumerate(names)}
    sp = WRITER[f"w{i}__spacing"]
    spacing = tuple(int(v) for v in sp) if bool(WRITER[f"w{i}__int_spacing"]) else \
        tuple(float(v) for v in sp)
    origin = tuple(float(v) for v in WRITER[f"w{i}__origin"])
    p = tmp_path / "w.vti"
    pnm.save_vti(str(p), fields, spacing=spacing, origin=origin)
    assert p.read_bytes() == WRITER[f"w{i}__bytes"].tobytes()


@pytest.mark.parametrize("shape", [(1, 1, 1), (3, 5, 7), (16, 9, 33), (40, 2, 1)])
def test_round_trip(tmp_path, shape):
    rng = np.random.default_rng(sum(shape))
    a = rng.standard_normal(shape).astype(np.float32)
    a.reshape(-1)[:: max(1, a.size // 5)] = np.float32(-0.0)
    org, spc = [0.1, -2.5, 3e-7], [0.25, 1.0 / 3.0, 2.0]
    p = tmp_path / "rt.vti"
    pnm.write_sdf_vti(str(p), a, org, spc)
    sdf, o, s = pnm.SDFReader.read_vti(str(p))
    assert np.array_equal(sdf.view(np.uint32), a.view(np.uint32))
    assert o == [float(np.float32(v)) for v in org]
    assert s == [float(np.float32(v)) for v in spc]


def test_byte_count_beyond_volume_is_clamped(tmp_path):
    # the reference would read past its buffer here; this reader stops at the volume's end
    a = np.arange(24, dtype=np.float32)
    p = tmp_path / "big.vti"
    pnm.write_sdf_vti(str(p), a.reshape(2, 3, 4))
    raw = bytearray(p.read_bytes())
    at = raw.index(b"_", raw.index(b'<AppendedData encoding="raw">')) + 1
    raw[at:at + 8] = np.array([10 ** 6], "<u8").tobytes()
    p.write_bytes(bytes(raw))
    sdf, _, _ = pnm.SDFReader.read_vti(str(p))
    assert np.array_equal(sdf.reshape(-1), a)


def test_missing_origin_spacing_read_as_zero(tmp_path):
    p = tmp_path / "no_org.vti"
    p.write_bytes(b'<VTKFile><ImageData WholeExtent="0 1 0 0 0 0">\n'
                  b'<AppendedData encoding="raw">_' + np.array([8], "<u8").tobytes() +
                  np.float32([1.5, -2]).tobytes())
    sdf, o, s = pnm.SDFReader.read_vti(str(p))
    assert sdf.shape == (1, 1, 2) and sdf.tolist() == [[[1.5, -2.0]]]
    assert o == [0.0, 0.0, 0.0] and s == [0.0, 0.0, 0.0]


@pytest.mark.parametrize("blob,msg", [
    (b"<VTKFile><ImageData Origin=\"0 0 0\"></VTKFile>", "Could not find WholeExtent"),
    (b'<ImageData WholeExtent="0 1 0 1 0 1"><AppendedData encoding="base64">_',
     "Could not find AppendedData tag"),
    (b'<ImageData WholeExtent="0 1 0 1 0 1"><AppendedData encoding="raw">' + b" " * 9000 + b"_",
     "Could not find binary data marker"),
    (b'<ImageData WholeExtent="0 1 0 1 0 1"><AppendedData encoding="raw">_\x01\x02',
     "Failed to read data_bytes"),
])
def test_reader_errors(tmp_path, blob, msg):
    p = tmp_path / "bad.vti"
    p.write_bytes(blob)
    with pytest.raises(RuntimeError, match=msg):
        pnm.SDFReader.read_vti(str(p))


def test_missing_file(tmp_path):
    with pytest.raises(RuntimeError, match="Could not open file"):
        pnm.SDFReader.read_vti(str(tmp_path / "absent.vti"))


def test_edge_list(tmp_path):
    p = tmp_path / "edges.txt"
    pnm.write_edge_list(str(p), [(1, 4), (2, 3)])
    assert p.read_text() == "1 4\n2 3\n"
    pnm.write_edge_list(str(p), np.zeros((0, 2), np.int32))
    assert p.read_text() == ""


REF_VTI = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle",
                       "_ref", "libpnm_ref_vti.so")


@pytest.mark.skipif(not os.path.exists(REF_VTI),
                    reason="reference reader not built here (oracle/_ref)")
def test_reader_matches_reference_reader_fuzz(tmp_path):
    """600 generated files read by this reader and by the reference's own (src/sdf_reader.cpp):
    offset extents, number formats in Origin / Spacing, names with '_', padding before the
    marker, byte counts short, odd or exact, files cut inside the payload. Both fail, or both
    return the same dims, origin, spacing and value bits. Byte counts beyond the volume are left
    out: there the reference writes past its buffer (this reader clamps, tested above)."""
    import ctypes

    from golden.make_vti_golden import point_file

    lib = ctypes.CDLL(REF_VTI)
    lib.ref_read_vti.argtypes = [ctypes.c_char_p, ctypes.c_void_p, ctypes.c_void_p,
                                 ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p),
                                 ctypes.POINTER(ctypes.c_longlong)]
    lib.ref_vti_free.argtypes = [ctypes.c_void_p]
    rng = np.random.default_rng(424242)

    def num(x):
        return str(rng.choice([f"{x}", f"{x:.3e}", f"{x:E}", f"{x:.9g}", f"  {x}", f"{x:+g}"]))

    p = tmp_path / "f.vti"
    for it in range(600):
        nx, ny, nz = (int(v) for v in rng.integers(1, 6, size=3))
        o = [int(v) for v in rng.integers(-3, 4, size=3)]
        ext = f"{o[0]} {o[0] + nx - 1} {o[1]} {o[1] + ny - 1} {o[2]} {o[2] + nz - 1}"
        org = " ".join(num(float(v)) for v in rng.normal(0, 100, size=3))
        spc = " ".join(num(float(v)) for v in rng.uniform(1e-3, 5, size=3))
        vals = rng.standard_normal((nz, ny, nx)).astype(np.float32)
        nbytes = vals.size * 4
        mode = it % 4
        count = None
        if mode == 1:
            count = int(rng.integers(0, nbytes + 1))
        elif mode == 2:
            count = int(rng.integers(0, nbytes)) | 1
        name = str(rng.choice(["sdf", "signed_distance", "a_b_c", "x"]))
        pad = [b"\n", b"\n  ", b" ", b"\n\n    "][int(rng.integers(0, 4))]
        blob = point_file(vals, ext, org, spc, name=name, count=count, pad=pad)
        if mode == 3:  # cut inside the payload
            blob = blob[:int(rng.integers(len(blob) - nbytes - 40, len(blob)))]
        p.write_bytes(blob)
        dims = np.zeros(3, np.int32)
        ro = np.zeros(3, np.float32)
        rs = np.zeros(3, np.float32)
        vp, n = ctypes.c_void_p(), ctypes.c_longlong()
        rc = lib.ref_read_vti(str(p).encode(), dims.ctypes.data, ro.ctypes.data, rs.ctypes.data,
                              ctypes.byref(vp), ctypes.byref(n))
        rv = np.zeros(0, np.float32)
        if rc == 0:
            if n.value:
                rv = np.ctypeslib.as_array(ctypes.cast(vp, ctypes.POINTER(ctypes.c_float)),
                                           (n.value,)).copy()
            lib.ref_vti_free(vp)
        try:
            sdf, go, gs = pnm.SDFReader.read_vti(str(p))
        except RuntimeError:
            assert rc != 0, it
            continue
        assert rc == 0, it
        assert sdf.shape == (int(dims[2]), int(dims[1]), int(dims[0])), it
        assert np.array_equal(np.float32(go), ro[::-1]) and np.array_equal(np.float32(gs), rs[::-1])
        assert np.array_equal(sdf.reshape(-1).view(np.uint32), rv.view(np.uint32)), it
