"""Pore-network post-processing of an ``extract_network_flow`` result.

The reference leaves this to its scripts: ``scripts/demo_network_flow_packing.py:44-67`` takes
the result dict, forms the throat conductance ``g = Q / dp`` and prints the mass-balance and
network statistics below; its PASS test is ``max|res| < 1e-6 max|Q|`` with every g finite.

:func:`network_stats` returns those figures for either form of the result: a dict of device
tensors (``extract_network_flow_device``) is reduced on the GPU by ``pnm_flow_stats_dev`` with
nothing but the figures coming back, a dict of host arrays or lists (``extract_network_flow``)
is reduced with numpy exactly as the demo does.

Keys: ``n_pores, n_throats, mean_abs_flow, max_abs_flow, mean_abs_dp, max_abs_residual,
frac_positive_conductance, all_conductance_finite, mean_coordination, max_coordination,
mass_balance_ok`` and the arrays ``conductance`` (per throat) and ``coordination`` (throats per
pore label, repeated pairs counted).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _capi
from ._capi import Context, default_context

__all__ = ["network_stats", "throat_conductance"]


def _on_device(x) -> bool:
    return hasattr(x, "is_cuda") and bool(x.is_cuda)


def throat_conductance(net):
    """g = throat_flow / throat_dp (IEEE division), on the device for device results."""
    q, dp = net["throat_flow"], net["throat_dp"]
    if _on_device(q):
        return q / dp
    with np.errstate(divide="ignore", invalid="ignore"):
        return np.asarray(q, np.float64) / np.asarray(dp, np.float64)


def _finish(d: dict) -> dict:
    nt = d["n_throats"]
    d["frac_positive_conductance"] = d.pop("n_positive_conductance") / nt if nt else float("nan")
    d["all_conductance_finite"] = d.pop("n_finite_conductance") == nt
    d["mass_balance_ok"] = bool(d["mass_balance_ok"])
    return d


def _device_stats(net, ctx: Context | None) -> dict:
    import torch

    from .device import _Stream

    q = net["throat_flow"]
    dev = q.device
    f64 = lambda k: net[k].to(torch.float64).contiguous()  # noqa: E731
    qv, dp, res = f64("throat_flow"), f64("throat_dp"), f64("pore_residual")
    th = net["throats"].to(torch.int32).contiguous()
    nt, np_ = qv.numel(), res.numel()
    if th.numel() != 2 * nt or dp.numel() != nt:
        raise RuntimeError("throats, throat_flow and throat_dp disagree in length")
    g = torch.empty(nt, dtype=torch.float64, device=dev)
    coord = torch.empty(np_, dtype=torch.int32, device=dev)
    r = _capi.PnmFlowResultDev()
    r.n_pores, r.n_throats = np_, nt
    r.pore_residual = res.data_ptr() if np_ else None
    r.throats = th.data_ptr() if nt else None
    r.throat_flow = qv.data_ptr() if nt else None
    r.throat_dp = dp.data_ptr() if nt else None
    st = _capi.PnmFlowStats()
    ctx = ctx or default_context()
    with _Stream(ctx, dev):
        ctx.check(_capi.pnm_flow_stats_dev(ctx.h, ctypes.byref(r), g.data_ptr() if nt else None,
                                           coord.data_ptr() if np_ else None, ctypes.byref(st)))
    d = {k: getattr(st, k) for k, _ in _capi.PnmFlowStats._fields_}
    d["conductance"], d["coordination"] = g, coord
    return _finish(d)


def _host_stats(net) -> dict:
    q = np.asarray(net["throat_flow"], np.float64).reshape(-1)
    dp = np.asarray(net["throat_dp"], np.float64).reshape(-1)
    res = np.asarray(net["pore_residual"], np.float64).reshape(-1)
    th = np.asarray(net["throats"], np.int64).reshape(-1, 2)
    nt, np_ = len(q), len(res)
    g = throat_conductance(net)
    lab = th.reshape(-1)
    lab = lab[(lab >= 1) & (lab <= np_)]
    coord = np.bincount(lab - 1, minlength=np_).astype(np.int32)
    nan = float("nan")
    max_q = float(np.abs(q).max()) if nt else nan
    max_res = float(np.abs(res).max()) if np_ else nan
    n_fin = int(np.isfinite(g).sum())
    d = {"n_pores": np_, "n_throats": nt,
         "mean_abs_flow": float(np.abs(q).mean()) if nt else nan,
         "max_abs_flow": max_q,
         "mean_abs_dp": float(np.abs(dp).mean()) if nt else nan,
         "max_abs_residual": max_res,
         "n_positive_conductance": int((g > 0).sum()),
         "n_finite_conductance": n_fin,
         "mean_coordination": 2.0 * nt / np_ if np_ else 0.0,
         "max_coordination": int(coord.max()) if np_ else 0,
         "mass_balance_ok": (np_ == 0 or max_res < 1e-6 * (max_q if nt else 0.0)) and n_fin == nt,
         "conductance": g, "coordination": coord}
    return _finish(d)


def network_stats(net: dict, *, ctx: Context | None = None) -> dict:
    """Conductance and network statistics of an extract_network_flow result (module doc)."""
    if _on_device(net["throat_flow"]) or _on_device(net["pore_residual"]):
        return _device_stats(net, ctx)
    return _host_stats(net)
