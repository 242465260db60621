"""Probes: field read-out points (wavetorch/probe.py:6-27).

Inside :class:`~wavetorch_gb300.rnn.WaveRNN` the probes are not called per
step: their coordinates become probe-table entries of the sequence kernels,
which gather (and square) the field in the kernel epilogue.  ``forward`` is
kept for direct use on a field tensor.
"""
from __future__ import annotations

import torch

from .utils import host_list, to_tensor


class WaveProbe(torch.nn.Module):
    """Amplitude probe at (x, y): ``out = field[:, x, y]``."""
    kind = 0

    def __init__(self, x, y):
        super().__init__()
        self.register_buffer('x', to_tensor(x, dtype=torch.int64))
        self.register_buffer('y', to_tensor(y, dtype=torch.int64))

    def forward(self, x):
        return x[:, self.x, self.y]

    def cells(self):
        """Flat list of (x, y) cells this probe reads, in output order."""
        xs = host_list(self.x)
        ys = host_list(self.y)
        if len(xs) != len(ys):
            raise ValueError("probe x and y must have the same length")
        return list(zip(xs, ys))

    def plot(self, ax, color='k'):
        marker, = ax.plot(self.x.cpu().numpy(), self.y.cpu().numpy(), 'o', markeredgecolor=color,
                          markerfacecolor='none', markeredgewidth=1.0, markersize=4)
        return marker


class WaveIntensityProbe(WaveProbe):
    """Intensity probe at (x, y): ``out = field[:, x, y] ** 2``."""
    kind = 1

    def forward(self, x):
        return super().forward(x).pow(2)
