"""The argument checks every apply runs before a pointer reaches the C ABI
(TMR._check_vectors): wrong sizes, mixed host/device arguments and host
tensors passed where CUDA tensors are required raise ValueError instead of
letting a kernel read or write past a buffer.  Host-side logic only."""
import numpy as np
import pytest
import torch

from tmr_gb300 import TMR

CHECK = TMR._check_vectors


def test_host_arrays_give_the_vector_count():
    assert CHECK("P", np.zeros(10 * 3), np.zeros(40 * 3), 10, 40, ("float64",)) == 3
    assert CHECK("P", np.zeros(7), np.zeros(5), 7, 5, ("float64",)) == 1


@pytest.mark.parametrize("nx,ny", [(0, 0), (11, 40), (10 * 3, 40 * 2), (10, 41)])
def test_host_size_mismatch_raises(nx, ny):
    with pytest.raises(ValueError):
        CHECK("P", np.zeros(nx), np.zeros(ny), 10, 40, ("float64",))


def test_empty_operator_raises():
    with pytest.raises(ValueError):
        CHECK("P", np.zeros(3), np.zeros(3), 0, 3, ("float64",))


def test_mixed_or_host_tensors_raise():
    x = torch.zeros(10, dtype=torch.float64)
    y = np.zeros(40)
    with pytest.raises(ValueError, match="CUDA"):
        CHECK("P", x, y, 10, 40, ("float64",))
    with pytest.raises(ValueError, match="CUDA"):
        CHECK("P", y[:10], torch.zeros(40, dtype=torch.float64), 10, 40, ("float64",))
    # torch tensors on the host are not device pointers
    with pytest.raises(ValueError, match="CUDA"):
        CHECK("P", x, torch.zeros(40, dtype=torch.float64), 10, 40, ("float64",))
