"""The RNN cell: one leapfrog step of the damped scalar wave equation
(wavetorch/cell.py:8-107), with the step and its adjoint on the GPU.
"""
from __future__ import annotations

import numpy as np
import torch

from .functional import WaveStepFn, _f32
from .utils import host_scalar, to_tensor


def saturable_damping(u, uth, b0):
    """b0 / (1 + |u/uth|^2) (wavetorch/cell.py:8-9)."""
    return b0 / (1 + torch.abs(u / uth).pow(2))


class TimeStep:
    """``TimeStep.apply(b, c, y1, y2, dt, h)`` -- the reference's autograd
    Function name, served by the CUDA step kernels."""
    apply = staticmethod(WaveStepFn.apply)


class WaveCell(torch.nn.Module):
    """The recurrent cell implementing the scalar wave equation."""

    def __init__(self, dt: float, geometry, satdamp_b0: float = 0.0, satdamp_uth: float = 0.0,
                 c_nl: float = 0.0):
        super().__init__()
        self.register_buffer("dt", to_tensor(dt))
        self.geom = geometry
        self.register_buffer("satdamp_b0", to_tensor(satdamp_b0))
        self.register_buffer("satdamp_uth", to_tensor(satdamp_uth))
        self.register_buffer("c_nl", to_tensor(c_nl))
        cmax = self.geom.cmax
        h = float(self.geom.h)
        if dt > 1 / cmax * h / np.sqrt(2):
            raise ValueError(
                'The spatial discretization defined by the geometry `h = %f` and the temporal '
                'discretization defined by the model `dt = %f` do not satisfy the CFL stability criteria'
                % (h, dt))

    def parameters(self, recursive=True):
        for param in self.geom.parameters():
            yield param

    def scalars(self):
        """Python values of (dt, h, satdamp_b0, satdamp_uth, c_nl) -- one host
        read per sequence instead of one per step."""
        return (_f32(self.dt), _f32(self.geom.h), float(host_scalar(self.satdamp_b0)),
                float(host_scalar(self.satdamp_uth)), float(host_scalar(self.c_nl)))

    def is_linear(self) -> bool:
        return not (float(host_scalar(self.satdamp_b0)) > 0 or float(host_scalar(self.c_nl)) != 0)

    def forward(self, h1, h2, c_linear, rho, _scalars=None):
        """Take a step through time: returns (y_{t+1}, y_t).

        h1, h2: fields one and two steps ago [batch, nx, ny]; c_linear: the
        linear wave speed [nx, ny]; rho: the density that weights the
        nonlinear terms."""
        dt, h, b0, uth, cnl = _scalars if _scalars is not None else self.scalars()
        if b0 > 0:
            b = self.geom.b + rho * saturable_damping(h1, uth=self.satdamp_uth, b0=self.satdamp_b0)
        else:
            b = self.geom.b
        if cnl != 0:
            c = c_linear + rho * self.c_nl * h1.pow(2)
        else:
            c = c_linear
        y = TimeStep.apply(b, c, h1, h2, dt, h)
        return y, h1
