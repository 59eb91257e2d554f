"""Generates tests/golden/vti/cases.npz from the REFERENCE's own VTI reader and writer.

Reader: src/sdf_reader.cpp compiled unmodified (oracle/build_ref.sh -> oracle/_ref/
libpnm_ref_vti.so) is run on a set of hand-built files: the PointData layout it is written for,
offset extents, exponents in Origin / Spacing, short and odd byte counts, a '_' inside an
attribute before the AppendedData tag, and a CellData file from the reference writer (whose
WholeExtent is one larger than the arrays). Each case stores the file bytes and what the reader
returned. Writer: scripts/vti.py save_vti is imported from the reference checkout and its output
for a small labelled volume is stored byte for byte.

    PNM_REFERENCE=<reference checkout> python tests/golden/make_vti_golden.py [--writer-extra]

(--writer-extra: only the eight extra writer cases, tests/golden/vti/writer_cases.npz)
"""
from __future__ import annotations

import ctypes
import importlib.util
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF = os.environ.get("PNM_REFERENCE", "")  # the reference checkout (read-only)

HEAD = (b'<?xml version="1.0"?>\n<VTKFile type="ImageData" version="1.0" '
        b'byte_order="LittleEndian" header_type="UInt64">\n')


def point_file(values: np.ndarray, extent: str, origin: str, spacing: str, name: str = "sdf",
               count: int | None = None, pad: bytes = b"\n", payload: bytes | None = None) -> bytes:
    """A PointData ImageData file; `count` overrides the stored byte count and `payload` the
    bytes after it."""
    body = values.astype("<f4").tobytes() if payload is None else payload
    n = len(body) if count is None else count
    xml = (f'  <ImageData WholeExtent="{extent}" Origin="{origin}" Spacing="{spacing}">\n'
           f'    <Piece Extent="{extent}">\n      <PointData Scalars="{name}">\n'
           f'        <DataArray type="Float32" Name="{name}" NumberOfComponents="1" '
           f'format="appended" offset="0"/>\n      </PointData>\n    </Piece>\n'
           f'  </ImageData>\n').encode()
    return (HEAD + xml + b'  <AppendedData encoding="raw">' + pad + b"_" +
            np.array([n], "<u8").tobytes() + body + b"\n  </AppendedData>\n</VTKFile>\n")


def reader_cases(rng) -> dict:
    v = lambda *s: rng.standard_normal(s).astype(np.float32)  # noqa: E731
    cases = {
        "point_7x5x3": point_file(v(3, 5, 7), "0 6 0 4 0 2", "0.5 -1.25 3", "0.1 0.2 0.30000001"),
        "offset_extent": point_file(v(3, 5, 7), "3 9 -2 2 5 7", "1e-3 -2.5e+2 7",
                                    "5E-1 0.25 2"),
        "one_voxel": point_file(v(1, 1, 1), "0 0 0 0 0 0", "0 0 0", "1 1 1"),
        "short_count": point_file(v(2, 3, 4)[:1], "0 3 0 2 0 1", "0 0 0", "1 1 1"),
        "odd_count": point_file(v(2, 3, 4), "0 3 0 2 0 1", "0 0 0", "1 1 1", count=4 * 9 + 2),
        "name_underscore": point_file(v(4, 4, 4), "0 3 0 3 0 3", "0 0 0", "1 1 1",
                                      name="signed_distance_field", pad=b"\n  "),
    }
    # the reference writer's CellData layout: WholeExtent "0 nx 0 ny 0 nz", Int32 labels first
    spec = importlib.util.spec_from_file_location("ref_vti", os.path.join(REF, "scripts", "vti.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    with tempfile.TemporaryDirectory() as d:
        p = os.path.join(d, "cells.vti")
        lab = rng.integers(-5, 9, (3, 4, 5)).astype(np.int32)
        mod.save_vti(p, {"Labels": lab, "SDF": v(3, 4, 5)}, spacing=(0.5, 0.25, 1.0),
                     origin=(0.10000000149011612, -2.0, 3.5))
        cases["celldata_labels"] = open(p, "rb").read()
    return cases, mod


def writer_case(rng, mod) -> bytes:
    fields = {"Labels": rng.integers(-3, 12, (3, 4, 5)).astype(np.int64),
              "SDF": rng.standard_normal((3, 4, 5)).astype(np.float32),
              "vel": rng.standard_normal((3, 4, 5, 3))}
    with tempfile.TemporaryDirectory() as d:
        p = os.path.join(d, "w.vti")
        mod.save_vti(p, fields, spacing=(0.5, 0.25, 1.0), origin=(0.10000000149011612, -2.0, 3.5))
        return fields, open(p, "rb").read()


def extra_writer_cases(rng, mod) -> dict:
    """Eight more field sets through the reference writer: every integer width (written as
    Int32), float16 / float32 / float64, bool, vector fields, integer spacing (formatted without
    a decimal point) and float origins."""
    dts = [np.int8, np.uint8, np.int16, np.int64, np.uint32, np.float16, np.float32, np.float64,
           np.bool_]
    out = {}
    with tempfile.TemporaryDirectory() as d:
        for i in range(8):
            shp = tuple(int(v) for v in rng.integers(1, 5, size=3))
            names = []
            for j in range(1 + i % 3):
                dt = dts[(3 * i + j) % len(dts)]
                s = shp + ((3,) if (i + j) % 3 == 0 else ())
                if np.issubdtype(dt, np.floating):
                    arr = rng.normal(0, 10, size=s).astype(dt)
                else:
                    arr = rng.integers(-50, 50, size=s).astype(dt)
                name = ["Labels", "SDF", "vel"][j] + str(i)
                names.append(name)
                out[f"w{i}__f{j}"] = arr
            int_spacing = i % 4 == 0
            spacing = (tuple(int(v) for v in rng.integers(1, 4, size=3)) if int_spacing else
                       tuple(float(v) for v in rng.choice([0.5, 0.1, 1e-3, 2.0, 0.30000001],
                                                          size=3)))
            origin = tuple(float(v) for v in rng.normal(0, 5, size=3))
            p = os.path.join(d, "w.vti")
            mod.save_vti(p, {n: out[f"w{i}__f{j}"] for j, n in enumerate(names)},
                         spacing=spacing, origin=origin)
            out[f"w{i}__names"] = np.array(names)
            out[f"w{i}__spacing"] = np.array(spacing, np.float64)
            out[f"w{i}__int_spacing"] = np.array(int_spacing)
            out[f"w{i}__origin"] = np.array(origin, np.float64)
            out[f"w{i}__bytes"] = np.frombuffer(open(p, "rb").read(), np.uint8)
    return out


def main():
    if not os.path.exists(os.path.join(REF, "scripts", "vti.py")):
        sys.stderr.write("set PNM_REFERENCE to the reference checkout\n")
        return 2
    lib = ctypes.CDLL(os.path.join(ROOT, "oracle", "_ref", "libpnm_ref_vti.so"))
    lib.ref_read_vti.argtypes = [ctypes.c_char_p, ctypes.c_void_p, ctypes.c_void_p,
                                 ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p),
                                 ctypes.POINTER(ctypes.c_longlong)]
    lib.ref_vti_free.argtypes = [ctypes.c_void_p]
    rng = np.random.default_rng(20261203)
    cases, mod = reader_cases(rng)
    out = {}
    with tempfile.TemporaryDirectory() as d:
        for name, blob in cases.items():
            p = os.path.join(d, name + ".vti")
            open(p, "wb").write(blob)
            dims = np.zeros(3, np.int32)
            org = np.zeros(3, np.float32)
            spc = np.zeros(3, np.float32)
            vp, n = ctypes.c_void_p(), ctypes.c_longlong()
            rc = lib.ref_read_vti(p.encode(), dims.ctypes.data, org.ctypes.data, spc.ctypes.data,
                                  ctypes.byref(vp), ctypes.byref(n))
            assert rc == 0, name
            vals = np.ctypeslib.as_array(ctypes.cast(vp, ctypes.POINTER(ctypes.c_float)),
                                         (n.value,)).copy()
            lib.ref_vti_free(vp)
            out[f"{name}__file"] = np.frombuffer(blob, np.uint8)
            out[f"{name}__dims"] = dims
            out[f"{name}__origin"] = org
            out[f"{name}__spacing"] = spc
            out[f"{name}__values"] = vals
    fields, wbytes = writer_case(rng, mod)
    for k, a in fields.items():
        out[f"writer__field__{k}"] = a
    out["writer__bytes"] = np.frombuffer(wbytes, np.uint8)
    if "--writer-extra" not in sys.argv:
        np.savez_compressed(os.path.join(HERE, "vti", "cases.npz"), **out)
        print(f"wrote {len(cases)} reader cases and one writer case")
    extra = extra_writer_cases(np.random.default_rng(20261204), mod)
    np.savez_compressed(os.path.join(HERE, "vti", "writer_cases.npz"), **extra)
    print("wrote 8 more writer cases")


if __name__ == "__main__":
    sys.exit(main())
