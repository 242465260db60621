"""Host-side helpers mirroring wavetorch/utils.py (dtype switch, loss glue)."""
from __future__ import annotations

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
