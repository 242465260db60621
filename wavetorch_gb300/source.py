"""Sources: additive injection of the input series (wavetorch/source.py:7-41).

Inside :class:`~wavetorch_gb300.rnn.WaveRNN` sources become source-table
entries of the sequence kernels (the injection is fused into the update).
``forward`` is kept for direct use on a field tensor.
"""
from __future__ import annotations

import torch

from .utils import host_list, to_tensor


def bresenham(r0, c0, r1, c1):
    """Cells of the digital line from (r0, c0) to (r1, c1), both ends included
    (Bresenham's algorithm, the algorithm of skimage.draw.line that the
    reference calls at wavetorch/source.py:31)."""
    r0, c0, r1, c1 = int(r0), int(c0), int(r1), int(c1)
    dr, dc = abs(r1 - r0), abs(c1 - c0)
    sr = 1 if r1 >= r0 else -1
    sc = 1 if c1 >= c0 else -1
    rr, cc = [], []
    if dr > dc:
        err, c = dr // 2, c0
        for r in range(r0, r1 + sr, sr):
            rr.append(r)
            cc.append(c)
            err -= dc
            if err < 0:
                c += sc
                err += dr
    else:
        err, r = dc // 2, r0
        for c in range(c0, c1 + sc, sc):
            rr.append(r)
            cc.append(c)
            err -= dr
            if err < 0:
                r += sr
                err += dc
    return rr, cc


class WaveSource(torch.nn.Module):
    """Point (or multi-cell) source: ``Y + dt**2 * scatter(X at (x, y))``."""

    def __init__(self, x, y):
        super().__init__()
        # int64 coordinates, as advanced indexing wants them
        self.register_buffer('x', to_tensor(x, dtype=torch.int64))
        self.register_buffer('y', to_tensor(y, dtype=torch.int64))

    def forward(self, Y, X, dt=1.0):
        X_expanded = torch.zeros(Y.size(), dtype=Y.dtype, device=Y.device)
        X_expanded[:, self.x, self.y] = X
        return Y + dt ** 2 * X_expanded

    def cells(self):
        """Flat list of (x, y) cells this source drives."""
        xs = host_list(self.x)
        ys = host_list(self.y)
        return list(zip(xs, ys))

    def plot(self, ax, color='r'):
        marker, = ax.plot(self.x.cpu().numpy(), self.y.cpu().numpy(), 'o', markeredgecolor=color,
                          markerfacecolor='none', markeredgewidth=1.0, markersize=4)
        return marker


class WaveLineSource(WaveSource):
    """Source on the digital line from (r0, c0) to (r1, c1)."""

    def __init__(self, r0, c0, r1, c1):
        x, y = bresenham(r0, c0, r1, c1)
        self.r0, self.c0, self.r1, self.c1 = r0, c0, r1, c1
        super().__init__(x, y)

    def plot(self, ax, color='r'):
        line, = ax.plot([self.r0, self.r1], [self.c0, self.c1], '-', color=color, lw=2)
        return line
