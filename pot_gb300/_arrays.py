"""Input coercion at the drop-in boundary.

The reference accepts lists, numpy arrays and backend tensors
(``ot/utils.py:59`` ``list_to_array``, ``ot/backend.py:245`` ``get_backend``)
and returns results of the input's type, dtype and device.  Here every input
is moved to the CUDA device (host arrays are copied; CUDA tensors are used in
place) and results are converted back to the caller's array type.
"""
import numpy as np
import torch


class Boundary:
    """Remembers how the caller's arrays looked so results can go back."""

    def __init__(self, *arrays):
        self.kind = "numpy"
        self.device = None
        for x in arrays:
            if isinstance(x, torch.Tensor):
                self.kind = "torch"
                if x.is_cuda:
                    self.device = x.device
                break
        if self.device is None:
            if not torch.cuda.is_available():
                raise RuntimeError("pot_gb300 runs on a CUDA GPU only; no CUDA device is visible")
            self.device = torch.device("cuda", torch.cuda.current_device())
        self.host_torch = self.kind == "torch" and not any(
            isinstance(x, torch.Tensor) and x.is_cuda for x in arrays)

    def to_dev(self, x, dtype=None):
        if x is None:
            return None
        if isinstance(x, torch.Tensor):
            t = x.detach()
        else:
            arr = np.asarray(x)
            if arr.dtype.kind not in "fc":
                arr = arr.astype(np.float64)
            t = torch.from_numpy(np.ascontiguousarray(arr))
        if dtype is not None and t.dtype != dtype:
            t = t.to(dtype)
        elif t.dtype not in (torch.float32, torch.float64):
            t = t.to(torch.float64)
        return t.to(self.device, non_blocking=True)

    def out(self, t):
        """Device tensor -> caller's array type."""
        if t is None:
            return None
        if self.kind == "numpy":
            return t.detach().cpu().numpy()
        if self.host_torch:
            return t.cpu()
        return t

    def scalar(self, t):
        """0-d result: numpy float for numpy callers, 0-d tensor otherwise."""
        if self.kind == "numpy":
            return t.detach().cpu().numpy()[()]
        if self.host_torch:
            return t.cpu()
        return t


def shape_of(x):
    """Shape of a caller's array (list, numpy array or tensor) without copying it."""
    return tuple(x.shape) if hasattr(x, "shape") else np.shape(x)


def check_shape(name, x, shapes):
    """Raise ValueError unless `x` (when given and non-empty) has one of
    `shapes`.  Called on the caller's arrays before any device work: the
    kernels read as many entries as the problem's sizes say, so a wrong
    shape must stop here rather than become an out-of-bounds read."""
    if x is None or is_empty(x):
        return
    s = shape_of(x)
    if s not in [tuple(t) for t in shapes]:
        raise ValueError("%s has shape %s, expected %s" % (name, s, " or ".join(str(tuple(t)) for t in shapes)))


def is_empty(x):
    if x is None:
        return True
    if isinstance(x, torch.Tensor):
        return x.numel() == 0
    return len(x) == 0
