"""The reference's training loss fused with the wave sequence.

wavetorch trains on ``CrossEntropyLoss(normalize_power(y.sum(dim=1)), labels)``
(wavetorch/train.py:61-62, utils.py:35-36): the loss sees the probe series
only through its time sums.  :func:`cross_entropy_normalize_power` computes
those sums in the forward kernel's epilogue (Kahan-compensated), the loss
and dLoss/dsum in one small kernel, and hands the adjoint per-probe weights
instead of a [batch, T, probes] gradient, so nothing of size T is formed
for the loss.  Models the fused form cannot take fall back to the same loss
built from torch operations.
"""
from __future__ import annotations

import ctypes as C

import torch

from . import _lib
from .functional import (SeqSpec, _ptr, _require_cuda_f32, _stream, fused_supported, lap_order,
                         scalars, seq_forward)
from .utils import normalize_power


class SeqCELossFn(torch.autograd.Function):
    """(loss, probe series) of one fused sequence; differentiable in c."""

    @staticmethod
    def forward(ctx, c, b, x, labels, spec: SeqSpec, sc: _lib.Scalars):
        c = _require_cuda_f32("c", c)
        b = _require_cuda_f32("b", b)
        x = _require_cuda_f32("x", x)
        labels = labels.to(device=c.device, dtype=torch.int64).contiguous()
        out, _, psum, ws = seq_forward(spec, sc, b, c, x, want_sum=True)
        loss = torch.empty((), device=c.device)
        gsum = torch.empty((spec.batch, len(spec.probes)), device=c.device)
        _lib.check(_lib.load().wt_loss_ce_normalize_power(
            spec.batch, len(spec.probes), _ptr(psum), _ptr(labels), _ptr(loss), _ptr(gsum),
            _stream(c.device)), "wt_loss_ce_normalize_power")
        ctx.spec, ctx.sc = spec, sc
        ctx.save_for_backward(c, b, x, gsum, ws)
        ctx.mark_non_differentiable(out)
        return loss, out

    @staticmethod
    def backward(ctx, grad_loss, grad_out_unused):
        c, b, x, gsum, ws = ctx.saved_tensors
        spec = ctx.spec
        gw = (gsum * grad_loss).contiguous()
        gc = torch.empty(((spec.batch,) if spec.coef_batched else ()) + (spec.nx, spec.ny),
                         device=c.device)
        d, keep = spec.desc()
        _lib.check(_lib.load().wt_seq_bwd_sum(C.byref(ctx.sc), C.byref(d), _ptr(b), _ptr(c), _ptr(x),
                                              _ptr(gw), _ptr(gc), _ptr(ws), ws.numel(),
                                              _stream(c.device)), "wt_seq_bwd_sum")
        return gc, None, None, None, None, None


def cross_entropy_normalize_power(model, x, labels):
    """``(loss, y)`` with ``loss = CrossEntropyLoss(normalize_power(y.sum(1)),
    labels)`` and ``y = model(x)`` the probe series [batch, T, P]; ``loss``
    backpropagates to the geometry's rho like the unfused expression."""
    geom = model.cell.geom
    nx, ny = geom.domain_shape
    batch, steps = x.shape[0], x.shape[1]
    ptab, L = model.probe_table() if model._seq_ok() and len(model.probes) else (None, 0)
    if L == 1 and model.form == "fused":
        dt, h = model.cell.scalars()[:2]
        spec = SeqSpec(batch, nx, ny, steps, model.source_table(batch), ptab,
                       form=_lib.WT_FORM_FUSED, segment=model.segment, cluster=model.cluster)
        if fused_supported(spec):
            sc = scalars(dt, h, lap_order(batch, nx, ny, h))
            return SeqCELossFn.apply(geom.c, geom.b, x.contiguous(), labels, spec, sc)
    y = model(x)
    loss = torch.nn.CrossEntropyLoss()(normalize_power(y.sum(dim=1)), labels)
    return loss, y
