"""WaveRNN: the time loop (wavetorch/rnn.py:4-72) on the GPU.

For the reference's own source and probe types and a linear cell, the whole
loop is one :class:`~wavetorch_gb300.functional.WaveSeqFn` call:

* ``form='fused'`` (default): persistent kernels -- one thread-block cluster
  per instance (grids up to 256x256), the adjoint from a Laplacian tape or
  from checkpoints with segment recompute; larger grids (up to 1024 columns)
  in bands of rows, one CTA per band and SM; shapes neither layout plans run
  in the plain form instead.  ``cluster`` fixes the cluster size (-1: bands);
* ``form='plain'``: one forward kernel per step with every field kept, and one
  adjoint kernel per step -- the reference's dataflow, bit-exact with it;
* ``form='step'``: the reference's Python loop structure, each step a
  :class:`~wavetorch_gb300.functional.WaveStepFn` (used for nonlinear cells
  and for gradients of field outputs).
"""
from __future__ import annotations

import torch

from . import _lib
from .functional import (SeqSpec, WaveSeqFn, WaveSeqNLFn, fused_supported, lap_order,
                         nl_supported, scalars)
from .probe import WaveProbe
from .source import WaveSource

_FORMS = {"fused": _lib.WT_FORM_FUSED, "plain": _lib.WT_FORM_PLAIN}


class WaveRNN(torch.nn.Module):
    def __init__(self, cell, sources, probes=[], form: str = "fused", segment: int = 0,
                 cluster: int = 0):
        super().__init__()
        self.cell = cell
        self.sources = torch.nn.ModuleList(sources if isinstance(sources, list) else [sources])
        self.probes = torch.nn.ModuleList(probes if isinstance(probes, list) else [probes])
        if form not in ("fused", "plain", "step"):
            raise ValueError("form must be 'fused', 'plain' or 'step'")
        self.form = form
        self.segment = int(segment)
        self.cluster = int(cluster)

    # -- tables for the sequence kernels ----------------------------------
    def source_table(self, batch: int):
        """(cell, in_row) entries in application order.  A source over L cells
        assigns the [batch] input to its cells the way the reference's
        ``X_expanded[:, xs, ys] = X`` broadcasts (wavetorch/source.py:19-20):
        every cell gets the instance's own value when L == 1 or batch == 1,
        cell l gets instance l's value when L == batch."""
        nx, ny = self.cell.geom.domain_shape
        table = []
        for s in self.sources:
            cells = s.cells()
            L = len(cells)
            if L != 1 and batch != 1 and L != batch:
                raise RuntimeError(
                    f"shape mismatch: a source over {L} cells cannot take a batch of {batch} inputs")
            seen = {}
            for l, (x, y) in enumerate(cells):
                if not (0 <= x < nx and 0 <= y < ny):
                    raise IndexError(f"source cell ({x}, {y}) outside the {nx}x{ny} domain")
                row = l if (L == batch and L != 1 and batch != 1) else -1
                seen[x * ny + y] = row      # index_put: the last write wins
            table.extend(seen.items())
        return table

    def probe_table(self):
        """(cell, kind, order) per output column; columns ordered (l, p) so
        that [batch, T, L*P] views as the reference's stacked [batch, T, L, P]."""
        nx, ny = self.cell.geom.domain_shape
        per = [p.cells() for p in self.probes]
        Ls = {len(c) for c in per}
        if len(Ls) > 1:
            raise RuntimeError("probes with different numbers of cells cannot be stacked")
        L = Ls.pop() if Ls else 0
        table = []
        for l in range(L):
            for p, (probe, cells) in enumerate(zip(self.probes, per)):
                x, y = cells[l]
                if not (0 <= x < nx and 0 <= y < ny):
                    raise IndexError(f"probe cell ({x}, {y}) outside the {nx}x{ny} domain")
                table.append((x * ny + y, probe.kind, p))
        return table, L

    def _taps_ok(self) -> bool:
        return (all(isinstance(s, WaveSource) for s in self.sources)
                and all(isinstance(p, WaveProbe) for p in self.probes))

    def _seq_ok(self) -> bool:
        return self.cell.is_linear() and self._taps_ok()

    def _forward_nonlinear(self, x, c):
        """The nonlinear cell's time loop as one fused sequence (b and c formed
        every step inside the kernels), or None when the shape does not fit
        the fused form (the caller then steps it)."""
        geom = self.cell.geom
        nx, ny = geom.domain_shape
        batch, steps = x.shape[0], x.shape[1]
        dt, h, b0, uth, cnl = self.cell.scalars()
        ptab, L = self.probe_table()
        spec = SeqSpec(batch, nx, ny, steps, self.source_table(batch), ptab,
                       form=_lib.WT_FORM_FUSED, segment=self.segment, cluster=self.cluster)
        if not nl_supported(spec):
            return None
        sc = scalars(dt, h, lap_order(batch, nx, ny, h))
        nl = _lib.NonLinear(b0, uth, cnl)
        out = WaveSeqNLFn.apply(c, geom.rho, geom.b, x.contiguous(), spec, sc, nl)
        if L != 1:
            out = out.view(batch, steps, L, len(self.probes))
        return out

    # -- forward ----------------------------------------------------------
    def forward(self, x, output_fields=False, form: str | None = None):
        """Propagate the input series x [batch, T] through T steps.

        Returns the probe series [batch, T, P] (or [batch, T, L, P] for probes
        over L cells), or the fields [batch, T, nx, ny] when ``output_fields``
        is set or there are no probes."""
        form = form or self.form
        geom = self.cell.geom
        nx, ny = geom.domain_shape
        batch, steps = x.shape[0], x.shape[1]
        c = geom.c
        fields_out = output_fields or len(self.probes) == 0
        use_seq = form != "step" and self._seq_ok()
        if use_seq and fields_out and torch.is_grad_enabled() and (
                c.requires_grad or x.requires_grad):
            use_seq = False   # field outputs are differentiated step by step
        if (form == "fused" and not fields_out and not self.cell.is_linear()
                and self._taps_ok()):
            out = self._forward_nonlinear(x, c)
            if out is not None:
                return out
        if not use_seq:
            return self._forward_steps(x, c, fields_out)
        dt, h = self.cell.scalars()[:2]
        sc = scalars(dt, h, lap_order(batch, nx, ny, h))
        ptab, L = self.probe_table()
        spec = SeqSpec(batch, nx, ny, steps, self.source_table(batch),
                       [] if fields_out else ptab,
                       form=_FORMS[form if form in _FORMS else "fused"], segment=self.segment,
                       cluster=self.cluster, output_fields=fields_out)
        if spec.form == _lib.WT_FORM_FUSED and not fused_supported(spec):
            spec.form = _lib.WT_FORM_PLAIN   # neither fused layout plans this shape
        b = geom.b
        out = WaveSeqFn.apply(c, b, x.contiguous(), spec, sc)
        if fields_out:
            return out
        P = len(self.probes)
        if L != 1:
            out = out.view(batch, steps, L, P)
        return out

    def _forward_steps(self, x, c, fields_out):
        """The reference's loop (wavetorch/rnn.py:36-72), one CUDA step kernel
        per iteration; sources and probes as tensor ops."""
        geom = self.cell.geom
        shape = (x.shape[0],) + tuple(geom.domain_shape)
        h1 = torch.zeros(shape, device=x.device, dtype=x.dtype)
        h2 = torch.zeros(shape, device=x.device, dtype=x.dtype)
        rho = geom.rho
        sc = self.cell.scalars()
        y_all = []
        for xi in x.chunk(x.size(1), dim=1):
            h1, h2 = self.cell(h1, h2, c, rho, _scalars=sc)
            for source in self.sources:
                h1 = source(h1, xi.squeeze(-1))
            if not fields_out:
                y_all.append(torch.stack([probe(h1) for probe in self.probes], dim=-1))
            else:
                y_all.append(h1)
        return torch.stack(y_all, dim=1)
