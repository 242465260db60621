"""Geometry: PML damping profile and the density -> wave-speed map
(wavetorch/geom.py:11-233).

Buffer and parameter names are the reference's, so ``state_dict`` files and
``state_reconstruction_args`` round-trip between the two implementations.
The free-form map rho -> c and the hole geometry run on the GPU
(:class:`~wavetorch_gb300.functional.RhoToCFn`, :class:`~wavetorch_gb300.functional.HoleyFn`).
"""
from __future__ import annotations

from copy import deepcopy
from typing import Tuple

import numpy as np
import torch

from . import _lib
from .functional import HoleyFn, RhoToCFn, _f32
from .utils import host_scalar, to_tensor


def disk_kernel(radius: int) -> torch.Tensor:
    """Normalised (2r+1)^2 blur kernel: ones on the open disk of radius r+1
    centred on the middle cell (the rule of skimage.draw.circle(r, r, r+1)
    used at wavetorch/geom.py:149-152), divided by its sum."""
    n = 2 * radius + 1
    ii, jj = np.meshgrid(np.arange(n), np.arange(n), indexing='ij')
    mask = (ii - radius) ** 2 + (jj - radius) ** 2 < (radius + 1) ** 2
    k = torch.zeros((n, n), dtype=torch.get_default_dtype())
    k[torch.from_numpy(mask)] = 1
    return k / k.sum()


def pml_profile(shape, abs_N: int, abs_sig: float, abs_p) -> torch.Tensor:
    """Damping b = sqrt(b_x^2 + b_y^2) of the absorbing layer
    (wavetorch/geom.py:63-85): a polynomial ramp abs_sig * s^abs_p,
    s = 0 .. 1 over abs_N + 1 cells, rising towards each edge."""
    Nx, Ny = shape
    ramp = abs_sig * torch.linspace(0.0, 1.0, abs_N + 1) ** abs_p
    prof_x = torch.zeros(Nx)
    prof_y = torch.zeros(Ny)
    if abs_N > 0:
        prof_x[:abs_N + 1] = ramp.flip(0)
        prof_x[Nx - abs_N - 1:] = ramp
        prof_y[:abs_N + 1] = ramp.flip(0)
        prof_y[Ny - abs_N - 1:] = ramp
    b_x = prof_x[:, None].expand(Nx, Ny)
    b_y = prof_y[None, :].expand(Nx, Ny)
    return torch.sqrt(b_x ** 2 + b_y ** 2)


class WaveGeometry(torch.nn.Module):
    def __init__(self, domain_shape: Tuple, h: float, c0: float, c1: float, abs_N: int = 20,
                 abs_sig: float = 11, abs_p: float = 4.0):
        super().__init__()
        assert len(domain_shape) == 2, \
            "len(domain_shape) must be equal to 2: only two-dimensional (2D) domains are supported"
        self.domain_shape = tuple(int(v) for v in domain_shape)
        self.register_buffer("h", to_tensor(h))
        self.register_buffer("c0", to_tensor(c0))
        self.register_buffer("c1", to_tensor(c1))
        self.register_buffer("abs_N", to_tensor(abs_N, dtype=torch.uint8))
        self.register_buffer("abs_sig", to_tensor(abs_sig))
        self.register_buffer("abs_p", to_tensor(abs_p, dtype=torch.uint8))
        self._init_b(abs_N, abs_sig, abs_p)

    def state_reconstruction_args(self):
        return {"domain_shape": self.domain_shape,
                "h": self.h.item(),
                "c0": self.c0.item(),
                "c1": self.c1.item(),
                "abs_N": self.abs_N.item(),
                "abs_sig": self.abs_sig.item(),
                "abs_p": self.abs_p.item()}

    def __repr__(self):
        return "WaveGeometry shape={}, h={}".format(self.domain_shape, self.h)

    def forward(self):
        raise NotImplementedError(
            "WaveGeometry forward() is not implemented; the geometry only parameterises a WaveCell.")

    @property
    def c(self):
        raise NotImplementedError

    @property
    def b(self):
        return self._b

    @property
    def cmax(self):
        """Largest wave speed, used by the CFL check."""
        return max(self.c0.item(), self.c1.item())

    def constrain_to_design_region(self):
        pass

    def _init_b(self, abs_N: int, abs_sig: float, abs_p: float):
        Nx, Ny = self.domain_shape
        assert Nx > 2 * abs_N + 1, \
            "The domain isn't large enough in the x-direction to fit absorbing layer. Nx = {} and N = {}".format(Nx, abs_N)
        assert Ny > 2 * abs_N + 1, \
            "The domain isn't large enough in the y-direction to fit absorbing layer. Ny = {} and N = {}".format(Ny, abs_N)
        self.register_buffer("_b", pml_profile((Nx, Ny), abs_N, abs_sig, abs_p).contiguous())


class WaveGeometryHoley(WaveGeometry):
    """Density from a sum of exponential holes, projected (wavetorch/geom.py:88-132).

    rho and c come from one kernel (:class:`~wavetorch_gb300.functional.HoleyFn`,
    ``wt_holey_fwd``) and their gradients with respect to the holes' centres
    and radii from its adjoint (``wt_holey_bwd``).  The holes must be on a
    CUDA device: like every other operation here, reading ``rho`` or ``c`` of
    CPU-held holes raises (there is no CPU path)."""

    def __init__(self, domain_shape: Tuple, h: float, c0: float, c1: float, abs_N: int = 20,
                 abs_sig: float = 11, abs_p: float = 4.0, eta: float = 0.5, beta: float = 100.0,
                 x=None, y=None, r=None):
        super().__init__(domain_shape, h, c0, c1, abs_N, abs_sig, abs_p)
        self.x = torch.nn.Parameter(to_tensor(x))
        self.y = torch.nn.Parameter(to_tensor(y))
        self.r = torch.nn.Parameter(to_tensor(r))
        self.register_buffer("eta", to_tensor(eta))
        self.register_buffer("beta", to_tensor(beta))

    def state_reconstruction_args(self):
        my_args = {"eta": self.eta.item(), "beta": self.beta.item(),
                   "x": deepcopy(self.x.detach()), "y": deepcopy(self.y.detach()),
                   "r": deepcopy(self.r.detach())}
        return {**super().state_reconstruction_args(), **my_args}

    def holey_desc(self) -> _lib.HoleyDesc:
        for name in ("x", "y", "r"):
            if getattr(self, name).dim() != 1:
                raise TypeError(f"the holes' {name} must be a 1-D tensor (one entry per hole)")
        n = min(self.x.numel(), self.y.numel(), self.r.numel())   # zip() stops at the shortest
        return _lib.HoleyDesc(self.domain_shape[0], self.domain_shape[1], n, _f32(self.eta),
                              _f32(self.beta), _f32(self.c0), _f32(self.c1))

    def _rho_c(self):
        """(rho, c) on the GPU: one kernel evaluates both."""
        return HoleyFn.apply(self.x, self.y, self.r, self.holey_desc())

    @property
    def rho(self):
        """Projected density of the holes (a CUDA tensor; CPU holes raise)."""
        return self._rho_c()[0]

    @property
    def c(self):
        """Wave speed c = c0 + (c1 - c0) * rho, from the same kernel as rho."""
        return self._rho_c()[1]


class WaveGeometryFreeForm(WaveGeometry):
    """Free-form density rho, blurred and projected to c (wavetorch/geom.py:136-233)."""

    def __init__(self, domain_shape: Tuple, h: float, c0: float, c1: float, abs_N: int = 20,
                 abs_sig: float = 11, abs_p: float = 4.0, eta: float = 0.5, beta: float = 100.0,
                 design_region=None, rho='half', blur_radius: int = 1, blur_N: int = 1):
        super().__init__(domain_shape, h, c0, c1, abs_N, abs_sig, abs_p)
        self.register_buffer("eta", to_tensor(eta))
        self.register_buffer("beta", to_tensor(beta))
        self._init_design_region(design_region, self.domain_shape)
        self._init_rho(rho, self.domain_shape)
        self.register_buffer("blur_kernel", disk_kernel(int(blur_radius)).unsqueeze(0).unsqueeze(0))
        self.register_buffer("blur_N", to_tensor(blur_N, dtype=torch.int))
        # the reference stores blur_N under this name too (wavetorch/geom.py:156)
        self.register_buffer("blur_radius", to_tensor(blur_N, dtype=torch.int))
        self.constrain_to_design_region()

    def state_reconstruction_args(self):
        my_args = {"eta": self.eta.item(), "beta": self.beta.item(),
                   "design_region": deepcopy(self.design_region),
                   "rho": deepcopy(self.rho.detach()),
                   "blur_radius": self.blur_radius.item(),
                   "blur_N": self.blur_N.item()}
        return {**super().state_reconstruction_args(), **my_args}

    def __repr__(self):
        return super().__repr__() + ", " + str(self.design_region.sum().item()) + " DOFs"

    def _init_design_region(self, design_region, domain_shape):
        if design_region is not None:
            assert tuple(design_region.shape) == tuple(domain_shape), \
                "The design region shape must match domain shape; design_region.shape = {} domain_shape = {}".format(
                    design_region.shape, domain_shape)
            if isinstance(design_region, np.ndarray):
                design_region = torch.from_numpy(design_region.astype(np.uint8))
        else:
            design_region = torch.ones(domain_shape, dtype=torch.uint8)
        self.register_buffer("design_region", design_region)

    def _init_rho(self, rho, domain_shape):
        if isinstance(rho, (torch.Tensor, np.ndarray)):
            assert tuple(rho.shape) == tuple(domain_shape)
            self.rho = torch.nn.Parameter(to_tensor(rho))
        elif isinstance(rho, str):
            if rho == 'rand':
                self.rho = torch.nn.Parameter(torch.round(torch.rand(domain_shape)))
            elif rho == 'half':
                self.rho = torch.nn.Parameter(torch.ones(domain_shape) * 0.5)
            elif rho == 'blank':
                self.rho = torch.nn.Parameter(torch.zeros(domain_shape))
            else:
                raise ValueError('The domain initialization defined by `rho = %s` is invalid' % rho)
        else:
            raise ValueError('The domain initialization is invalid')

    def constrain_to_design_region(self):
        """Zero the density outside the design region and inside the PML
        (wavetorch/geom.py:201-205).  A masked fill on the device: unlike
        boolean-index assignment it needs no device-to-host round trip, so an
        optimiser step followed by this call stays asynchronous."""
        with torch.no_grad():
            self.rho.masked_fill_((self.design_region == 0) | (self.b > 0), 0.0)

    def geom_desc(self) -> _lib.GeomDesc:
        k = self.blur_kernel.shape[-1]
        return _lib.GeomDesc(self.domain_shape[0], self.domain_shape[1], (k - 1) // 2,
                             int(host_scalar(self.blur_N)), _f32(self.eta), _f32(self.beta),
                             _f32(self.c0), _f32(self.c1))

    @property
    def c(self):
        """Wave speed c = c0 + (c1 - c0) * P(blur(rho)), computed on the GPU."""
        return RhoToCFn.apply(self.rho, self.blur_kernel[0, 0], self.geom_desc())
