"""autograd Functions over the CUDA C ABI.

* :class:`WaveStepFn`  -- drop-in for ``TimeStep`` (wavetorch/cell.py:20-44).
* :class:`WaveSeqFn`   -- the whole time loop of ``WaveRNN.forward``
  (wavetorch/rnn.py:50-70) with a hand-written adjoint in place of the T-node
  autograd tape; plain (per-step kernels, every field kept) or fused
  (persistent cluster kernels, checkpointed) form.
* :class:`RhoToCFn`    -- the free-form rho -> c map (wavetorch/geom.py:207-233).

Every tensor handed to the kernels must be a float32 CUDA tensor; anything
else raises (there is no CPU path).
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import struct
from dataclasses import dataclass
from typing import Optional, Sequence

import torch

from . import _lib
from .utils import host_scalar

ONEDNN_MIN_CELLS = 20480   # torch CPU conv2d uses oneDNN above this (batch 1)


def lap_order(batch: int, nx: int, ny: int, h: float) -> int:
    """Association order of the reference's Laplacian for this shape.

    torch's CPU conv2d runs oneDNN when the batch is above one or the grid
    has more than 20480 cells, and an im2col+GEMM path otherwise; the two sum
    the taps in different orders (wavetorch/operators.py:5-11)."""
    if batch > 1 or nx * ny > ONEDNN_MIN_CELLS or h != 1.0:
        return _lib.WT_LAP_SEQ
    return _lib.WT_LAP_PAIRED


def _ptr(t: Optional[torch.Tensor]):
    return None if t is None else C.c_void_p(t.data_ptr())


def _stream(dev: torch.device):
    return C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)


def _require_cuda_f32(name: str, t: torch.Tensor) -> torch.Tensor:
    if not isinstance(t, torch.Tensor):
        raise TypeError(f"{name} must be a tensor")
    if t.device.type != "cuda":
        raise RuntimeError(
            f"wavetorch_gb300 runs on CUDA devices only: {name} is on {t.device}; "
            "move the model and inputs with .to('cuda')")
    if t.dtype != torch.float32:
        raise TypeError(f"wavetorch_gb300 kernels compute in float32: {name} is {t.dtype}")
    return t.contiguous()


def _f32(v) -> float:
    """float32 value of a python number or one-element tensor (device tensors
    are read once and cached, see utils.host_scalar)."""
    return struct.unpack("f", struct.pack("f", float(host_scalar(v))))[0]


def scalars(dt, h, order: int) -> _lib.Scalars:
    return _lib.Scalars(_f32(dt), _f32(h), order)


# ---------------------------------------------------------------------------
class WaveStepFn(torch.autograd.Function):
    """One leapfrog step, the drop-in for ``TimeStep.apply(b, c, y1, y2, dt, h)``."""

    @staticmethod
    def forward(ctx, b, c, y1, y2, dt, h):
        y1 = _require_cuda_f32("y1", y1)
        y2 = _require_cuda_f32("y2", y2)
        if y1.dim() != 3 or y2.shape != y1.shape:
            raise ValueError(f"y1/y2 must be [batch, nx, ny] of equal shape, got {tuple(y1.shape)}, {tuple(y2.shape)}")
        B, nx, ny = y1.shape
        b = _require_cuda_f32("b", b)
        c = _require_cuda_f32("c", c)
        batched = b.dim() == 3 or c.dim() == 3
        if batched:
            b = b.expand(B, nx, ny).contiguous()
            c = c.expand(B, nx, ny).contiguous()
        elif b.shape != (nx, ny) or c.shape != (nx, ny):
            raise ValueError("b and c must be [nx, ny] or [batch, nx, ny]")
        sc = scalars(dt, h, lap_order(B, nx, ny, _f32(h)))
        y = torch.empty_like(y1)
        lib = _lib.load()
        _lib.check(lib.wt_step_fwd(C.byref(sc), B, nx, ny, int(batched), _ptr(b), _ptr(c),
                                   _ptr(y1), _ptr(y2), _ptr(y), _stream(y1.device)), "wt_step_fwd")
        ctx.save_for_backward(b, c, y1, y2)
        ctx.sc = (sc.dt, sc.h, sc.lap_order)
        ctx.batched = batched
        return y

    @staticmethod
    def backward(ctx, grad_y):
        b, c, y1, y2 = ctx.saved_tensors
        g = _require_cuda_f32("grad", grad_y)
        B, nx, ny = y1.shape
        need = ctx.needs_input_grad
        cshape = (B, nx, ny) if ctx.batched else (nx, ny)
        gb = torch.empty(cshape, device=g.device) if need[0] else None
        gc = torch.empty(cshape, device=g.device) if need[1] else None
        gy1 = torch.empty_like(y1) if need[2] else None
        gy2 = torch.empty_like(y1) if need[3] else None
        sc = _lib.Scalars(*ctx.sc)
        lib = _lib.load()
        _lib.check(lib.wt_step_bwd(C.byref(sc), B, nx, ny, int(ctx.batched), _ptr(b), _ptr(c),
                                   _ptr(y1), _ptr(y2), _ptr(g), _ptr(gb), _ptr(gc), _ptr(gy1),
                                   _ptr(gy2), _stream(g.device)), "wt_step_bwd")
        return gb, gc, gy1, gy2, None, None


# ---------------------------------------------------------------------------
@dataclass
class SeqSpec:
    """Static description of one WaveRNN time loop (built by WaveRNN)."""
    batch: int
    nx: int
    ny: int
    steps: int
    sources: Sequence[tuple]        # (cell, in_row) in application order
    probes: Sequence[tuple]         # (cell, kind, order) per output column
    form: int = _lib.WT_FORM_FUSED
    segment: int = 0
    cluster: int = 0
    output_fields: bool = False
    coef_batched: bool = False      # one geometry (b, c) per instance
    sm_count: int = 0               # SMs the band layout may use (0: the device's)

    def desc(self):
        ns, np_ = len(self.sources), len(self.probes)
        src = (_lib.SourceEntry * max(ns, 1))(*[_lib.SourceEntry(int(c), int(r)) for c, r in self.sources])
        prb = (_lib.ProbeEntry * max(np_, 1))(*[_lib.ProbeEntry(int(c), int(k), int(o)) for c, k, o in self.probes])
        d = _lib.SeqDesc(self.batch, self.nx, self.ny, self.steps, ns,
                         C.cast(src, C.POINTER(_lib.SourceEntry)), np_,
                         C.cast(prb, C.POINTER(_lib.ProbeEntry)), self.form, self.segment,
                         self.cluster, int(self.output_fields), int(self.coef_batched),
                         int(self.sm_count))
        return d, (src, prb)   # keep the arrays alive with the descriptor


def seq_workspace_bytes(spec: SeqSpec) -> int:
    d, keep = spec.desc()
    n = C.c_size_t(0)
    _lib.check(_lib.load().wt_seq_workspace_bytes(C.byref(d), C.byref(n)), "wt_seq_workspace_bytes")
    return int(n.value)


def fused_supported(spec: SeqSpec) -> bool:
    """Whether the fused form can plan this sequence: on one thread-block
    cluster per instance (grids up to 256x256 cells), or in bands of rows, one
    CTA per band and SM (up to 1024 columns; a batch whose bands outnumber the
    SMs runs its instances in rounds).  Any other error is left for the real
    call to report."""
    d, keep = dataclasses.replace(spec, form=_lib.WT_FORM_FUSED).desc()
    n = C.c_size_t(0)
    return _lib.load().wt_seq_workspace_bytes(C.byref(d), C.byref(n)) != _lib.WT_ERR_UNSUPPORTED


def fused_uses_tape(spec: SeqSpec) -> bool:
    """Whether the fused adjoint of this sequence runs in tape mode (the
    forward stores every step's Laplacian) rather than from checkpoints."""
    if spec.form != _lib.WT_FORM_FUSED or spec.segment > 0:
        return False
    if spec.segment == -1:
        return True
    return seq_workspace_bytes(spec) == seq_workspace_bytes(dataclasses.replace(spec, segment=-1))


def seq_forward(spec: SeqSpec, sc: _lib.Scalars, b, c, x, want_sum: bool = False):
    """Run the forward sequence; returns (out, fields, probe_sum, workspace)."""
    dev = c.device
    d, keep = spec.desc()
    n = C.c_size_t(0)
    lib = _lib.load()
    _lib.check(lib.wt_seq_workspace_bytes(C.byref(d), C.byref(n)), "wt_seq_workspace_bytes")
    ws = torch.empty(int(n.value), dtype=torch.uint8, device=dev)
    out = torch.empty((spec.batch, spec.steps, len(spec.probes)), device=dev)
    fields = (torch.empty((spec.batch, spec.steps, spec.nx, spec.ny), device=dev)
              if spec.output_fields else None)
    psum = torch.empty((spec.batch, len(spec.probes)), device=dev) if want_sum else None
    _lib.check(lib.wt_seq_fwd(C.byref(sc), C.byref(d), _ptr(b), _ptr(c), _ptr(x), _ptr(out),
                              _ptr(fields), _ptr(psum), _ptr(ws), ws.numel(), _stream(dev)),
               "wt_seq_fwd")
    return out, fields, psum, ws


def seq_backward(spec: SeqSpec, sc: _lib.Scalars, b, c, x, grad_out, ws, want_x: bool):
    dev = c.device
    d, keep = spec.desc()
    gc = torch.empty(((spec.batch,) if spec.coef_batched else ()) + (spec.nx, spec.ny), device=dev)
    gx = torch.empty((spec.batch, spec.steps), device=dev) if want_x else None
    _lib.check(_lib.load().wt_seq_bwd(C.byref(sc), C.byref(d), _ptr(b), _ptr(c), _ptr(x),
                                      _ptr(grad_out), _ptr(gc), _ptr(gx), _ptr(ws), ws.numel(),
                                      _stream(dev)), "wt_seq_bwd")
    return gc, gx


def seq_device_status(spec: SeqSpec, ws: torch.Tensor) -> int:
    d, keep = spec.desc()
    return int(_lib.load().wt_seq_device_status(C.byref(d), _ptr(ws), ws.numel(), _stream(ws.device)))


class WaveSeqFn(torch.autograd.Function):
    """The whole time loop: returns the probe series [batch, steps, n_probe_columns]."""

    @staticmethod
    def forward(ctx, c, b, x, spec: SeqSpec, sc: _lib.Scalars):
        c = _require_cuda_f32("c", c)
        b = _require_cuda_f32("b", b)
        x = _require_cuda_f32("x", x)
        out, fields, _, ws = seq_forward(spec, sc, b, c, x)
        ctx.spec, ctx.sc = spec, sc
        ctx.save_for_backward(c, b, x, ws)
        if spec.output_fields:
            ctx.mark_non_differentiable(fields)
            return fields
        return out

    @staticmethod
    def backward(ctx, grad_out):
        c, b, x, ws = ctx.saved_tensors
        if ctx.spec.output_fields:
            raise RuntimeError("the fused sequence does not differentiate field outputs; "
                               "use WaveRNN(..., form='step') for gradients of fields")
        g = _require_cuda_f32("grad_out", grad_out)
        gc, gx = seq_backward(ctx.spec, ctx.sc, b, c, x, g, ws, ctx.needs_input_grad[2])
        return (gc if ctx.needs_input_grad[0] else None), None, gx, None, None


# ---------------------------------------------------------------------------
def nl_supported(spec: SeqSpec) -> bool:
    """Whether the fused nonlinear sequence can plan this shape (its adjoint
    needs a two-part tape ring in shared memory)."""
    d, keep = dataclasses.replace(spec, form=_lib.WT_FORM_FUSED).desc()
    n = C.c_size_t(0)
    return _lib.load().wt_seq_workspace_bytes_nl(C.byref(d), C.byref(n)) == _lib.WT_OK


class WaveSeqNLFn(torch.autograd.Function):
    """The whole time loop of a nonlinear cell (saturable damping and/or Kerr
    term, wavetorch/cell.py:8-9, :93-101) in the fused form: b and c are
    formed every step from the field inside the kernels.  Inputs: the linear
    speed c_lin, the density rho that weights the nonlinear terms, b_pml, x.
    Gradients: dL/dc_lin and the direct dL/drho (rho also reaches c_lin
    through the projection; autograd adds both)."""

    @staticmethod
    def forward(ctx, c_lin, rho, b, x, spec: SeqSpec, sc: _lib.Scalars, nl: _lib.NonLinear):
        c_lin = _require_cuda_f32("c", c_lin)
        rho = _require_cuda_f32("rho", rho)
        b = _require_cuda_f32("b", b)
        x = _require_cuda_f32("x", x)
        dev = c_lin.device
        d, keep = spec.desc()
        n = C.c_size_t(0)
        lib = _lib.load()
        _lib.check(lib.wt_seq_workspace_bytes_nl(C.byref(d), C.byref(n)), "wt_seq_workspace_bytes_nl")
        ws = torch.empty(int(n.value), dtype=torch.uint8, device=dev)
        out = torch.empty((spec.batch, spec.steps, len(spec.probes)), device=dev)
        _lib.check(lib.wt_seq_fwd_nl(C.byref(sc), C.byref(d), C.byref(nl), _ptr(b), _ptr(c_lin),
                                     _ptr(rho), _ptr(x), _ptr(out), None, _ptr(ws), ws.numel(),
                                     _stream(dev)), "wt_seq_fwd_nl")
        ctx.spec, ctx.sc, ctx.nl = spec, sc, nl
        ctx.save_for_backward(c_lin, rho, b, x, ws)
        return out

    @staticmethod
    def backward(ctx, grad_out):
        c_lin, rho, b, x, ws = ctx.saved_tensors
        spec = ctx.spec
        g = _require_cuda_f32("grad_out", grad_out)
        dev = g.device
        shape = ((spec.batch,) if spec.coef_batched else ()) + (spec.nx, spec.ny)
        gc = torch.empty(shape, device=dev)
        gr = torch.empty(shape, device=dev)
        gx = torch.empty((spec.batch, spec.steps), device=dev) if ctx.needs_input_grad[3] else None
        d, keep = spec.desc()
        _lib.check(_lib.load().wt_seq_bwd_nl(C.byref(ctx.sc), C.byref(d), C.byref(ctx.nl), _ptr(b),
                                             _ptr(c_lin), _ptr(rho), _ptr(x), _ptr(g), _ptr(gc),
                                             _ptr(gr), _ptr(gx), _ptr(ws), ws.numel(), _stream(dev)),
                   "wt_seq_bwd_nl")
        return (gc if ctx.needs_input_grad[0] else None), (gr if ctx.needs_input_grad[1] else None), \
            None, gx, None, None, None


# ---------------------------------------------------------------------------
class HoleyFn(torch.autograd.Function):
    """(rho, c) of the hole geometry (wavetorch/geom.py:109-132) from the
    holes' centres x, y and radii r; one kernel forward, two backward."""

    @staticmethod
    def forward(ctx, x, y, r, hdesc: _lib.HoleyDesc):
        ctx.set_materialize_grads(False)
        x, y, r = (_require_cuda_f32(n, t).reshape(-1) for n, t in (("x", x), ("y", y), ("r", r)))
        lib = _lib.load()
        n = C.c_size_t(0)
        _lib.check(lib.wt_holey_work_bytes(C.byref(hdesc), C.byref(n)), "wt_holey_work_bytes")
        work = torch.empty((int(n.value) + 7) // 8, dtype=torch.float64, device=x.device)
        shape = (hdesc.nx, hdesc.ny)
        rho = torch.empty(shape, device=x.device)
        c = torch.empty(shape, device=x.device)
        _lib.check(lib.wt_holey_fwd(C.byref(hdesc), _ptr(x), _ptr(y), _ptr(r), _ptr(rho),
                                    _ptr(c), _ptr(work), _stream(x.device)), "wt_holey_fwd")
        ctx.save_for_backward(x, y, r, work)
        ctx.hdesc = hdesc
        return rho, c

    @staticmethod
    def backward(ctx, grad_rho, grad_c):
        x, y, r, work = ctx.saved_tensors
        if grad_rho is None and grad_c is None:
            return None, None, None, None
        grho = None if grad_rho is None else _require_cuda_f32("grad_rho", grad_rho)
        gc = None if grad_c is None else _require_cuda_f32("grad_c", grad_c)
        gx, gy, gr = torch.zeros_like(x), torch.zeros_like(y), torch.zeros_like(r)
        work = work.clone()   # the adjoint writes its partial sums into it
        _lib.check(_lib.load().wt_holey_bwd(C.byref(ctx.hdesc), _ptr(x), _ptr(y), _ptr(r),
                                            _ptr(grho), _ptr(gc), _ptr(gx), _ptr(gy), _ptr(gr),
                                            _ptr(work), _stream(x.device)), "wt_holey_bwd")
        return gx, gy, gr, None


class RhoToCFn(torch.autograd.Function):
    """c = c0 + (c1 - c0) * P(blur^n(rho)) (wavetorch/geom.py:207-233)."""

    @staticmethod
    def forward(ctx, rho, blur_kernel, gdesc: _lib.GeomDesc):
        rho = _require_cuda_f32("rho", rho)
        k = _require_cuda_f32("blur_kernel", blur_kernel)
        lib = _lib.load()
        n = C.c_size_t(0)
        _lib.check(lib.wt_rho_to_c_work_bytes(C.byref(gdesc), C.byref(n)), "wt_rho_to_c_work_bytes")
        work = torch.empty(int(n.value) // 4, device=rho.device)
        c = torch.empty_like(rho)
        _lib.check(lib.wt_rho_to_c_fwd(C.byref(gdesc), _ptr(rho), _ptr(k), _ptr(c), _ptr(work),
                                       _stream(rho.device)), "wt_rho_to_c_fwd")
        ctx.save_for_backward(rho, k, work)
        ctx.gdesc = gdesc
        return c

    @staticmethod
    def backward(ctx, grad_c):
        rho, k, work = ctx.saved_tensors
        g = _require_cuda_f32("grad_c", grad_c)
        gr = torch.empty_like(rho)
        work = work.clone()   # the adjoint reuses half of it as scratch
        _lib.check(_lib.load().wt_rho_to_c_bwd(C.byref(ctx.gdesc), _ptr(rho), _ptr(k), _ptr(g),
                                               _ptr(gr), _ptr(work), _stream(g.device)),
                   "wt_rho_to_c_bwd")
        return gr, None, None
