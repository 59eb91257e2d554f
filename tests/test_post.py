"""Post-processing of flow results on the host (numpy, the reference demo's arithmetic,
scripts/demo_network_flow_packing.py:44-67)."""
import math

import numpy as np

import peclet_pnm_gb300 as pnm


def _net():
    return {"pores": np.zeros((4, 4), np.float32),
            "pore_pressure": np.zeros(4),
            "pore_residual": np.array([1e-12, -3e-12, 0.0, 2e-12]),
            "throats": np.array([[1, 2], [1, 3], [2, 3], [2, 3], [3, 4]], np.int32),
            "throat_flow": np.array([2.0, -1.0, 0.5, 0.0, 4.0]),
            "throat_area": np.ones(5),
            "throat_dp": np.array([1.0, 2.0, -0.5, 0.0, 0.0])}


def test_host_stats_known_answer():
    s = pnm.network_stats(_net())
    g = s["conductance"]
    assert g[0] == 2.0 and g[1] == -0.5 and g[2] == -1.0
    assert math.isnan(g[3]) and g[4] == math.inf
    assert s["n_pores"] == 4 and s["n_throats"] == 5
    assert s["mean_abs_flow"] == 7.5 / 5 and s["max_abs_flow"] == 4.0
    assert s["mean_abs_dp"] == 3.5 / 5
    assert s["max_abs_residual"] == 3e-12
    assert s["frac_positive_conductance"] == 2 / 5  # 2.0 and +inf
    assert s["all_conductance_finite"] is False
    assert s["mass_balance_ok"] is False  # g has a NaN and an inf
    assert s["coordination"].tolist() == [2, 3, 4, 1]
    assert s["max_coordination"] == 4 and s["mean_coordination"] == 2.5


def test_host_stats_list_form_and_pass():
    n = _net()
    n["throat_dp"] = np.array([1.0, 2.0, -0.5, 1.0, 3.0])
    lists = {k: (v.tolist() if k != "throats" else [tuple(t) for t in v.tolist()])
             for k, v in n.items()}
    a, b = pnm.network_stats(n), pnm.network_stats(lists)
    for k in a:
        assert np.array_equal(np.asarray(a[k]), np.asarray(b[k])), k
    assert a["mass_balance_ok"] is True and a["all_conductance_finite"] is True


def test_host_stats_empty():
    e = {"pores": [], "pore_pressure": [], "pore_residual": [], "throats": [],
         "throat_flow": [], "throat_area": [], "throat_dp": []}
    s = pnm.network_stats(e)
    assert s["n_pores"] == 0 and s["n_throats"] == 0 and s["mass_balance_ok"] is True
    assert len(s["conductance"]) == 0 and len(s["coordination"]) == 0
