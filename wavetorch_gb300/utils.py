"""Host-side helpers mirroring wavetorch/utils.py (dtype switch, loss glue)."""
from __future__ import annotations

import weakref

import numpy as np
import torch


def to_tensor(x, dtype=None):
    """Tensor of `x` in `dtype` (default: torch's default dtype), wavetorch/utils.py:6-11."""
    dtype = dtype if dtype is not None else torch.get_default_dtype()
    if isinstance(x, np.ndarray):
        return torch.from_numpy(x).type(dtype=dtype)
    if isinstance(x, torch.Tensor):
        return x.detach().clone().type(dtype)
    return torch.tensor(x, dtype=dtype)


# Host copies of small device tensors (coordinates, physics scalars), keyed by
# the tensor object and checked against its version counter, which every
# in-place change bumps.  Reading a CUDA tensor on the host synchronises the
# device, so without this each forward would stall the GPU once per value.
_HOST_VALUES = {}


def host_list(t: torch.Tensor) -> list:
    """Python list of the values of a small tensor, read from the device only
    when the tensor object is new or was modified in place."""
    if t.device.type == "cpu":
        return t.reshape(-1).tolist()
    key, ver = id(t), t._version
    hit = _HOST_VALUES.get(key)
    if hit is not None and hit[0]() is t and hit[1] == ver:
        return hit[2]
    vals = t.reshape(-1).tolist()
    _HOST_VALUES[key] = (weakref.ref(t, lambda _r, k=key: _HOST_VALUES.pop(k, None)), ver, vals)
    return vals


def host_scalar(t) -> float:
    """Python value of a one-element tensor (or a number), cached like host_list."""
    if isinstance(t, torch.Tensor):
        v = host_list(t)
        if len(v) != 1:
            raise ValueError("expected a one-element tensor")
        return v[0]
    return t


def set_dtype(dtype=None):
    """Select float32 (default) or float64 as torch's default dtype, wavetorch/utils.py:14-20.

    The GPU kernels compute in float32; float64 exists for building oracle
    models on the CPU side."""
    if dtype == 'float32' or dtype is None:
        torch.set_default_dtype(torch.float32)
    elif dtype == 'float64':
        torch.set_default_dtype(torch.float64)
    else:
        raise ValueError('Unsupported data type: %s; should be either float32 or float64' % dtype)


def window_data(X, window_length):
    """Centered window of length `window_length`, wavetorch/utils.py:23-26."""
    start = int(len(X) / 2 - window_length / 2)
    return X[start:int(len(X) / 2 + window_length / 2)]


def accuracy_onehot(y_pred, y_label):
    """Fraction of rows whose argmax matches the label, wavetorch/utils.py:29-32."""
    return (y_pred.argmax(dim=1) == y_label).float().mean().item()


def normalize_power(X):
    """Row-normalise time-integrated intensities, wavetorch/utils.py:35-36."""
    return X / torch.sum(X, dim=1, keepdim=True)
