"""Host-side logic that needs no GPU."""
import numpy as np
import pytest
import torch

import pot_gb300 as pg
from pot_gb300._arrays import Boundary, is_empty


def test_no_cpu_fallback():
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(RuntimeError, match="CUDA"):
        pg.sinkhorn([0.5, 0.5], [0.5, 0.5], [[0.0, 1.0], [1.0, 0.0]], 1.0)


def test_unknown_method_raises_before_any_device_work():
    with pytest.raises(ValueError):
        pg.sinkhorn([0.5, 0.5], [0.5, 0.5], [[0.0, 1.0], [1.0, 0.0]], 1.0, method="new_method")
    with pytest.raises(ValueError):
        pg.sinkhorn2([0.5, 0.5], [0.5, 0.5], [[0.0, 1.0], [1.0, 0.0]], 1.0, method="new_method")


def test_is_empty():
    assert is_empty([]) and is_empty(np.array([])) and is_empty(torch.tensor([]))
    assert not is_empty([1.0])
