"""CPU oracle for the peclet.pnm extraction path — TEST AND BASELINE INFRASTRUCTURE ONLY.

Two back ends with one Python surface (``Oracle``):

* ``port``      — ``oracle/libpnm_oracle.so``, the project's C++ restatement of the reference's
                  single-rank algorithm (``oracle/pnm_oracle.cpp``). Builds anywhere (x86, Arm).
* ``reference`` — ``oracle/_ref/libpnm_ref.so``, the reference's own ``src/pore_extraction.hpp``
                  compiled unmodified against the project's Kokkos shim
                  (``oracle/build_ref.sh``). Exists only where the reference checkout exists.

Inputs follow the reference's Python binding (``src/pnm_bindings.cpp``): SDF and fields are
``(Nz, Ny, Nx)`` C-order arrays; origin / spacing / grad_p are given in zyx order and converted
to the xyz order (origin/spacing cast to float32) the C++ core takes.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU legs import this package.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_LIB = os.path.join(HERE, "libpnm_oracle.so")
REF_LIBS = {False: os.path.join(HERE, "_ref", "libpnm_ref.so"),
            True: os.path.join(HERE, "_ref", "libpnm_ref_omp.so")}

_P = ctypes.POINTER
_vp = ctypes.c_void_p
_i = ctypes.c_int
_i64 = ctypes.c_int64


class _FlowResult(ctypes.Structure):
    _fields_ = [("n_pores", _i64), ("n_throats", _i64),
                ("pores", _P(ctypes.c_float)), ("pore_pressure", _P(ctypes.c_double)),
                ("pore_residual", _P(ctypes.c_double)), ("throats", _P(ctypes.c_int32)),
                ("throat_flow", _P(ctypes.c_double)), ("throat_area", _P(ctypes.c_double)),
                ("throat_dp", _P(ctypes.c_double))]


class _PortFlowResult(ctypes.Structure):
    _fields_ = _FlowResult._fields_ + [("throat_root", _P(ctypes.c_longlong)),
                                       ("pore_peak", _P(ctypes.c_int32)),
                                       ("throat_absflow", _P(ctypes.c_double)),
                                       ("pore_absflux", _P(ctypes.c_double))]


def _arr(ptr, count, dtype):
    if count <= 0:
        return np.zeros((0,), dtype)
    return np.ctypeslib.as_array(ptr, (int(count),)).astype(dtype, copy=True)


def _sdf(sdf):
    a = np.ascontiguousarray(sdf, dtype=np.float32)
    if a.ndim != 3:
        raise RuntimeError("SDF array must be 3D (Nz,Ny,Nx)")
    return a


def _xyz32(v_zyx):
    return np.array([v_zyx[2], v_zyx[1], v_zyx[0]], dtype=np.float32)


def _field(a, shape, name):
    if a is None:
        return None
    f = np.ascontiguousarray(a, dtype=np.float64)
    if f.shape != shape:
        raise RuntimeError(f"{name} must be (Nz,Ny,Nx) matching the SDF")
    return f


class Oracle:
    """One CPU back end (``kind`` = "port" or "reference")."""

    def __init__(self, kind: str = "port", threads: int = 1, openmp_ref: bool = False):
        self.kind = kind
        self.threads = int(threads)
        if kind == "port":
            if not os.path.exists(PORT_LIB):
                raise FileNotFoundError(f"{PORT_LIB} missing: run oracle/build.sh")
            lib = ctypes.CDLL(PORT_LIB)
            self._pre = "pnmo_"
            self._flow_t = _PortFlowResult
        elif kind == "reference":
            path = REF_LIBS[bool(openmp_ref)]
            if not os.path.exists(path):
                raise FileNotFoundError(f"{path} missing: run oracle/build_ref.sh")
            lib = ctypes.CDLL(path)
            self._pre = "ref_"
            self._flow_t = _FlowResult
        else:
            raise ValueError(kind)
        self.lib = lib
        pre = self._pre
        self._f_pores = getattr(lib, pre + "extract_pores")
        self._f_seg = getattr(lib, pre + "segment_volume")
        self._f_topo = getattr(lib, pre + "extract_topology")
        self._f_net = getattr(lib, pre + "extract_pore_network")
        self._f_flow = getattr(lib, pre + "extract_network_flow")
        self._f_flow.restype = _P(self._flow_t)
        self._f_flowfree = getattr(lib, pre + "flow_result_free")
        self._f_free = getattr(lib, pre + "free")
        self._f_pores.restype = ctypes.c_longlong
        self._f_topo.restype = ctypes.c_longlong

    def _targs(self):
        return (_i(self.threads),) if self.kind == "port" else ()

    # -- stages, array-level (xyz float32 origin/spacing) ---------------------------------------
    def pores_xyz(self, sdf, origin_xyz, spacing_xyz):
        a = _sdf(sdf)
        nz, ny, nx = a.shape
        o = np.asarray(origin_xyz, np.float32)
        s = np.asarray(spacing_xyz, np.float32)
        out = _P(ctypes.c_float)()
        k = self._f_pores(a.ctypes.data_as(_vp), _i(nx), _i(ny), _i(nz), o.ctypes.data_as(_vp),
                          s.ctypes.data_as(_vp), ctypes.byref(out), *self._targs())
        res = _arr(out, 4 * k, np.float32).reshape(-1, 4)
        self._f_free(out)
        return res

    def segment_xyz(self, sdf, spacing_xyz, roots=False):
        a = _sdf(sdf)
        nz, ny, nx = a.shape
        s = np.asarray(spacing_xyz, np.float32)
        seg = np.zeros(a.size, np.int32)
        if roots:
            rts = np.zeros(a.size, np.int32)
            if self.kind == "port":
                self._f_seg(a.ctypes.data_as(_vp), _i(nx), _i(ny), _i(nz), s.ctypes.data_as(_vp),
                            seg.ctypes.data_as(_vp), rts.ctypes.data_as(_vp), *self._targs())
            else:
                self.lib.ref_segment_with_roots(a.ctypes.data_as(_vp), _i(nx), _i(ny), _i(nz),
                                                s.ctypes.data_as(_vp), seg.ctypes.data_as(_vp),
                                                rts.ctypes.data_as(_vp))
            return seg, rts
        if self.kind == "port":
            self._f_seg(a.ctypes.data_as(_vp), _i(nx), _i(ny), _i(nz), s.ctypes.data_as(_vp),
                        seg.ctypes.data_as(_vp), None, *self._targs())
        else:
            self._f_seg(a.ctypes.data_as(_vp), _i(nx), _i(ny), _i(nz), s.ctypes.data_as(_vp),
                        seg.ctypes.data_as(_vp))
        return seg

    def topology_xyz(self, seg, nx, ny, nz):
        sg = np.ascontiguousarray(seg, dtype=np.int32).reshape(-1)
        out = _P(ctypes.c_int32)()
        m = self._f_topo(sg.ctypes.data_as(_vp), _i(nx), _i(ny), _i(nz), ctypes.byref(out),
                         *self._targs())
        res = _arr(out, 2 * m, np.int32).reshape(-1, 2)
        self._f_free(out)
        return res

    def pore_network_xyz(self, sdf, origin_xyz, spacing_xyz):
        a = _sdf(sdf)
        nz, ny, nx = a.shape
        o = np.asarray(origin_xyz, np.float32)
        s = np.asarray(spacing_xyz, np.float32)
        pp = _P(ctypes.c_float)()
        npp = ctypes.c_longlong()
        seg = np.zeros(a.size, np.int32)
        pr = _P(ctypes.c_int32)()
        npr = ctypes.c_longlong()
        self._f_net(a.ctypes.data_as(_vp), _i(nx), _i(ny), _i(nz), o.ctypes.data_as(_vp),
                    s.ctypes.data_as(_vp), ctypes.byref(pp), ctypes.byref(npp),
                    seg.ctypes.data_as(_vp), ctypes.byref(pr), ctypes.byref(npr), *self._targs())
        pores = _arr(pp, 4 * npp.value, np.float32).reshape(-1, 4)
        pairs = _arr(pr, 2 * npr.value, np.int32).reshape(-1, 2)
        self._f_free(pp)
        self._f_free(pr)
        return pores, seg, pairs

    def network_flow_xyz(self, sdf, origin_xyz, spacing_xyz, u, v, w, p, ox=None, oy=None,
                         oz=None, grad_p_xyz=(0.0, 0.0, 0.0)):
        a = _sdf(sdf)
        nz, ny, nx = a.shape
        o = np.asarray(origin_xyz, np.float32)
        s = np.asarray(spacing_xyz, np.float32)
        g = np.asarray(grad_p_xyz, np.float64)
        f = [_field(x, a.shape, nm) for x, nm in
             ((u, "u"), (v, "v"), (w, "w"), (p, "p"), (ox, "ox"), (oy, "oy"), (oz, "oz"))]
        ptr = [x.ctypes.data_as(_vp) if x is not None else None for x in f]
        r = self._f_flow(a.ctypes.data_as(_vp), _i(nx), _i(ny), _i(nz), o.ctypes.data_as(_vp),
                         s.ctypes.data_as(_vp), *ptr, g.ctypes.data_as(_vp), *self._targs())
        if not r:
            raise RuntimeError("extract_network_flow failed in the reference implementation")
        c = r.contents
        npo, nt = c.n_pores, c.n_throats
        out = {
            "pores": _arr(c.pores, 4 * npo, np.float32).reshape(-1, 4),
            "pore_pressure": _arr(c.pore_pressure, npo, np.float64),
            "pore_residual": _arr(c.pore_residual, npo, np.float64),
            "throats": _arr(c.throats, 2 * nt, np.int32).reshape(-1, 2),
            "throat_flow": _arr(c.throat_flow, nt, np.float64),
            "throat_area": _arr(c.throat_area, nt, np.float64),
            "throat_dp": _arr(c.throat_dp, nt, np.float64),
        }
        if self.kind == "port":
            out["throat_root"] = _arr(c.throat_root, nt, np.int64)
            out["pore_peak"] = _arr(c.pore_peak, npo, np.int32)
            # sums of |q| over each throat's and each pore's terms: the per-element scale of the
            # rounding error of those cancelling sums
            out["throat_absflow"] = _arr(c.throat_absflow, nt, np.float64)
            out["pore_absflux"] = _arr(c.pore_absflux, npo, np.float64)
        self._f_flowfree(r)
        return out

    # -- the reference's Python surface (zyx origin/spacing, pnm_bindings.cpp:110-209) -----------
    def extract_pores(self, sdf, origin_zyx, spacing_zyx):
        return self.pores_xyz(sdf, _xyz32(origin_zyx), _xyz32(spacing_zyx))

    def segment_volume(self, sdf, spacing_zyx):
        return self.segment_xyz(sdf, _xyz32(spacing_zyx))

    def extract_topology_gpu(self, segmentation, shape):
        return self.topology_xyz(segmentation, int(shape[2]), int(shape[1]), int(shape[0]))

    def extract_pore_network(self, sdf, origin_zyx, spacing_zyx):
        return self.pore_network_xyz(sdf, _xyz32(origin_zyx), _xyz32(spacing_zyx))

    def extract_network_flow(self, sdf, origin_zyx, spacing_zyx, u, v, w, p, ox=None, oy=None,
                             oz=None, grad_p_zyx=(0.0, 0.0, 0.0)):
        if (ox is None) != (oy is None) or (ox is None) != (oz is None):
            raise RuntimeError("pass all three openness arrays (ox,oy,oz) or none")
        g = np.array([grad_p_zyx[2], grad_p_zyx[1], grad_p_zyx[0]], np.float64)
        return self.network_flow_xyz(sdf, _xyz32(origin_zyx), _xyz32(spacing_zyx), u, v, w, p,
                                     ox, oy, oz, g)


def port_available() -> bool:
    return os.path.exists(PORT_LIB)


def reference_available() -> bool:
    return os.path.exists(REF_LIBS[False])


def sorted_pores(p: np.ndarray) -> np.ndarray:
    """Pores as a set: rows sorted lexicographically by (x, y, z, radius). NaNs are replaced by
    one canonical quiet NaN (the payload and sign of a NaN differ between x86, Arm and the GPU and
    carry no meaning), so bitwise comparison of the result treats NaN as equal to NaN."""
    p = np.array(p, np.float32).reshape(-1, 4)
    if len(p) == 0:
        return p
    p[np.isnan(p)] = np.float32(np.nan)
    bits = p.view(np.int32)
    bits[np.isnan(p)] = 0x7FC00000
    order = np.lexsort((p[:, 3], p[:, 2], p[:, 1], p[:, 0]))
    return p[order]
