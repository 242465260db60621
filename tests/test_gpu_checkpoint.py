"""The fused adjoint from checkpoints: the forward keeps the pair
(h_{t-1}, h_{t-2}) every `segment` steps, and the adjoint recomputes each
segment's Laplacians in one group of threads while a second group runs the
adjoint steps of the segment recomputed before.  It does the tape adjoint's
arithmetic on the same values (wavetorch/cell.py:26-44 per step, in
autograd's order), so its outputs, dL/dc and dL/dx must equal the tape
mode's bit for bit, for every checkpoint interval, including intervals that
do not divide T, one-step segments and a single segment."""
import numpy as np
import pytest
import torch

from conftest import FUSED_DC_TOL
from wavetorch_gb300 import _lib
from wavetorch_gb300.data import vowel_like
from wavetorch_gb300.functional import (SeqSpec, lap_order, scalars, seq_backward,
                                        seq_device_status, seq_forward)
import wavetorch_gb300 as wt

pytestmark = pytest.mark.gpu


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def problem(dev, B, nx, ny, steps, seed, src_cell, prb_cells):
    geom = wt.WaveGeometryFreeForm((nx, ny), 1.0, c0=1.0, c1=0.5, abs_N=10 if nx < 100 else 20,
                                   abs_sig=3.0, abs_p=2,
                                   rho=torch.rand(nx, ny, generator=torch.Generator().manual_seed(seed)))
    geom = geom.to(dev)
    with torch.no_grad():
        c = geom.c.detach().contiguous()
    b = geom.b.contiguous()
    x = torch.from_numpy(vowel_like(B, steps, seed=seed)[0]).to(dev)
    src = [(src_cell, -1)]
    prb = [(cell, 1, i) for i, cell in enumerate(prb_cells)]
    g = torch.randn(B, steps, len(prb), generator=torch.Generator().manual_seed(seed + 1)).to(dev)
    return b, c, x, src, prb, g


def run(spec, sc, b, c, x, g):
    out, _, _, ws = seq_forward(spec, sc, b, c, x)
    gc, gx = seq_backward(spec, sc, b, c, x, g, ws, True)
    torch.cuda.synchronize()
    assert seq_device_status(spec, ws) == _lib.WT_OK
    return out, gc, gx


def test_checkpoints_equal_the_tape_at_the_benchmark_size(cuda):
    """B=32, 120x120, T=3500 with sqrt(T) = 60-step segments: the
    checkpoint adjoint's dL/dc and dL/dx equal the tape adjoint's."""
    N, B, T = 120, 32, 3500
    b, c, x, src, prb, g = problem(cuda, B, N, N, T, 21, 20 * N + 60,
                                   [80 * N + y for y in (35, 50, 65)])
    sc = scalars(0.707, 1.0, lap_order(B, N, N, 1.0))
    tape = run(SeqSpec(B, N, N, T, src, prb, segment=-1), sc, b, c, x, g)
    ckpt = run(SeqSpec(B, N, N, T, src, prb, segment=60), sc, b, c, x, g)
    for a, t_ in zip(ckpt, tape):
        assert torch.equal(a, t_)


@pytest.mark.parametrize("segment", [1, 2, 7, 64, 300, 301, 5000])
def test_checkpoint_intervals_equal_the_tape(cuda, segment):
    """B=3, 120x120, T=301: one-step segments, intervals that do not divide
    T, one segment short of T, and intervals of T or more (one segment)."""
    N, B, T = 120, 3, 301
    b, c, x, src, prb, g = problem(cuda, B, N, N, T, 22, 20 * N + 60,
                                   [80 * N + y for y in (35, 50, 65)])
    sc = scalars(0.707, 1.0, lap_order(B, N, N, 1.0))
    tape = run(SeqSpec(B, N, N, T, src, prb, segment=-1), sc, b, c, x, g)
    ckpt = run(SeqSpec(B, N, N, T, src, prb, segment=segment), sc, b, c, x, g)
    for a, t_ in zip(ckpt, tape):
        assert torch.equal(a, t_)


def test_checkpoints_on_a_narrow_grid_with_taps_on_cta_edges(cuda):
    """40 x 72 on four CTAs of 10 rows (72 columns: a partly filled warp per
    strip), the source on a CTA's first row and probes on CTA boundary rows:
    checkpoints equal the tape, and both agree with the plain form (which is
    bit-exact with the reference) within the fused tolerance."""
    nx, ny, B, T = 40, 72, 5, 150
    b, c, x, src, prb, g = problem(cuda, B, nx, ny, T, 23, 10 * ny + 30,
                                   [9 * ny + 40, 20 * ny + 40, 29 * ny + 11])
    sc = scalars(0.707, 1.0, lap_order(B, nx, ny, 1.0))
    tape = run(SeqSpec(B, nx, ny, T, src, prb, segment=-1), sc, b, c, x, g)
    ckpt = run(SeqSpec(B, nx, ny, T, src, prb, segment=13), sc, b, c, x, g)
    for a, t_ in zip(ckpt, tape):
        assert torch.equal(a, t_)
    pout, pgc, pgx = run(SeqSpec(B, nx, ny, T, src, prb, form=_lib.WT_FORM_PLAIN), sc, b, c, x, g)
    assert torch.equal(ckpt[0], pout)
    assert rel(ckpt[1].cpu().numpy(), pgc.cpu().numpy()) <= FUSED_DC_TOL
    assert rel(ckpt[2].cpu().numpy(), pgx.cpu().numpy()) <= FUSED_DC_TOL

