"""Argument checks of the device-resident surface that run before any CUDA call (CPU)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from peclet_pnm_gb300 import device  # noqa: E402
from peclet_pnm_gb300 import vti  # noqa: E402


def test_host_tensors_are_refused():
    x = torch.zeros((4, 4, 4))
    with pytest.raises(RuntimeError, match="CUDA array"):
        device.extract_pore_network_device(x, [0] * 3, [1] * 3)
    with pytest.raises(RuntimeError, match="CUDA array"):
        device.segment_volume_device(x, [1] * 3)


def test_partial_openness_is_refused_first():
    x = torch.zeros((4, 4, 4), dtype=torch.float64)
    with pytest.raises(RuntimeError, match="openness"):
        device.extract_network_flow_device(x, [0] * 3, [1] * 3, x, x, x, x, ox=x)


def test_vti_device_destination_checked_before_reading(tmp_path):
    p = tmp_path / "a.vti"
    vti.write_sdf_vti(str(p), np.ones((2, 3, 4), np.float32))
    with pytest.raises(RuntimeError, match="CUDA tensor"):
        vti.read_vti_device(str(p), torch.zeros(24))
