"""Edge cases of the sequence kernels against the oracle (which is pinned
bit for bit to the reference): rectangular grids, one- and two-step
sequences, sources and probes on the rows where the fused form's CTAs meet
and on the grid's edges, several taps on one cell, no sources, and batch
rows shared by a line source.  Forward outputs and fields bit-exact in both
forms; dL/dc bit-exact in the plain form, within FUSED_DC_TOL in the fused form."""
import numpy as np
import pytest

from conftest import FUSED_DC_TOL
import torch

import oracle.oracle as o
from wavetorch_gb300 import _lib
from wavetorch_gb300.functional import (SeqSpec, lap_order, scalars, seq_backward,
                                        seq_device_status, seq_forward)
from wavetorch_gb300.geom import pml_profile

pytestmark = pytest.mark.gpu


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def problem(nx, ny, B, T, seed):
    rng = np.random.default_rng(seed)
    b = pml_profile((nx, ny), min(8, min(nx, ny) // 5), 3.0, 2).numpy()
    c = (0.5 + 0.5 * rng.random((nx, ny))).astype(np.float32)
    x = rng.standard_normal((B, T)).astype(np.float32)
    return b, c, x


def check(cuda, nx, ny, B, T, src, prb, seed=0):
    b, c, x = problem(nx, ny, B, T, seed)
    g = np.random.default_rng(seed + 1).standard_normal((B, T, max(len(prb), 1))).astype(np.float32)
    g = g[:, :, :len(prb)]
    S = o.Seq(B, nx, ny, T, 0.707, 1.0, src, prb)
    oout, hist = S.forward(b, c, x)
    ogc = S.backward(b, c, hist, g)[0] if prb else None
    sc = scalars(0.707, 1.0, lap_order(B, nx, ny, 1.0))
    tb, tc, tx = (torch.from_numpy(v).to(cuda) for v in (b, c, x))
    for form in (_lib.WT_FORM_PLAIN, _lib.WT_FORM_FUSED):
        spec = SeqSpec(B, nx, ny, T, src, prb, form=form)
        out, _, _, ws = seq_forward(spec, sc, tb, tc, tx)
        if prb:
            gc, _ = seq_backward(spec, sc, tb, tc, tx, torch.from_numpy(g).to(cuda), ws, False)
        torch.cuda.synchronize()
        assert seq_device_status(spec, ws) == _lib.WT_OK
        assert np.array_equal(out.cpu().numpy(), oout), form
        if prb:
            if form == _lib.WT_FORM_PLAIN:
                assert np.array_equal(gc.cpu().numpy(), ogc)
            else:
                assert rel(gc.cpu().numpy(), ogc) <= FUSED_DC_TOL
        # fields output too
        spec_f = SeqSpec(B, nx, ny, T, src, [], form=form, output_fields=True)
        _, fields, _, _ = seq_forward(spec_f, sc, tb, tc, tx)
        assert np.array_equal(fields.cpu().numpy(), hist), form


@pytest.mark.parametrize("nx,ny", [(72, 100), (100, 72), (37, 53), (64, 33), (45, 260), (130, 136)])
def test_rectangular_grids(cuda, nx, ny):
    src = [((nx // 4) * ny + ny // 2, -1)]
    prb = [((3 * nx // 4) * ny + ny // 3, 1, 0), ((3 * nx // 4) * ny + 2 * ny // 3, 0, 1)]
    check(cuda, nx, ny, 3, 90, src, prb)


@pytest.mark.parametrize("T", [1, 2, 3])
def test_very_short_sequences(cuda, T):
    N = 48
    src = [(10 * N + 24, -1)]
    prb = [(12 * N + 24, 1, 0), (10 * N + 24, 0, 1)]      # a probe on the source cell
    check(cuda, N, N, 2, T, src, prb)


def test_taps_where_ctas_meet_and_on_edges(cuda):
    """120x120 runs on 4 CTAs of 30 rows: sources and probes on rows 29, 30,
    59, 60 (the rows exchanged between CTAs) and on the grid's border."""
    N = 120
    src = [(29 * N + 40, -1), (30 * N + 41, -1), (0 * N + 0, -1), (119 * N + 119, -1)]
    prb = [(59 * N + 50, 1, 0), (60 * N + 51, 1, 1), (89 * N + 0, 0, 2), (90 * N + 119, 1, 3),
           (0 * N + 60, 1, 4), (119 * N + 60, 0, 5)]
    check(cuda, N, N, 2, 120, src, prb)


def test_taps_sharing_a_cell(cuda):
    """Two sources on one cell (applied in table order), three probes on one
    cell of both kinds (seeds added in descending probe order)."""
    N = 64
    src = [(20 * N + 32, -1), (20 * N + 32, -1)]
    prb = [(40 * N + 32, 1, 0), (40 * N + 32, 0, 1), (40 * N + 32, 1, 2), (44 * N + 30, 1, 3)]
    check(cuda, N, N, 3, 100, src, prb)


def test_no_sources(cuda):
    """No injection at all: the fields stay zero, the outputs are zero and so
    is dL/dc."""
    N = 40
    check(cuda, N, N, 2, 30, [], [(20 * N + 20, 1, 0)])


def test_fixed_input_rows(cuda):
    """A line source over as many cells as the batch: cell l takes instance
    l's input (in_row = l), the reference's broadcast of a [batch] input."""
    N, B = 48, 4
    src = [((10 + l) * N + 20, l) for l in range(B)]
    prb = [(30 * N + 20, 1, 0)]
    check(cuda, N, N, B, 60, src, prb)


def test_taps_on_column_chunk_edges(cuda):
    """45 x 260: the plain form's vector kernels cut rows into 128-column
    chunks (lanes of 4 cells) and groups of 4 rows, so sources and probes sit
    on chunk edges (columns 127, 128, 255, 256, 259) and on the ragged last
    row group (rows 44)."""
    nx, ny = 45, 260
    src = [(10 * ny + 127, -1), (11 * ny + 128, -1), (44 * ny + 259, -1)]
    prb = [(30 * ny + 255, 1, 0), (30 * ny + 256, 0, 1), (44 * ny + 128, 1, 2), (3 * ny + 127, 1, 3)]
    check(cuda, nx, ny, 2, 80, src, prb)


@pytest.mark.parametrize("B,nx,ny", [(400, 45, 260), (700, 61, 100)])
def test_row_streaming_kernels_on_ragged_rows_and_chunk_edges(cuda, B, nx, ny):
    """Batches past the row-streaming kernels' threshold (4 M cells per step)
    on grids whose rows do not fill the last group of 4 (forward) and whose
    columns span several 128-column chunks, taps on chunk edges and on the
    last rows, and a batch that ends in a short block of 16 (the adjoint's
    block sums): outputs, fields and dL/dc bit-exact with the oracle."""
    assert B * nx * ny >= 4 << 20
    src = [(10 * ny + min(127, ny - 1), -1), ((nx - 1) * ny + ny - 1, -1)]
    prb = [(30 * ny + min(128, ny - 2), 1, 0), ((nx - 1) * ny + ny // 2, 0, 1), (3 * ny + 127 % ny, 1, 2)]
    T = 10
    b, c, x = problem(nx, ny, B, T, 5)
    g = np.random.default_rng(6).standard_normal((B, T, len(prb))).astype(np.float32)
    S = o.Seq(B, nx, ny, T, 0.707, 1.0, src, prb)
    oout, hist = S.forward(b, c, x)
    ogc = S.backward(b, c, hist, g)[0]
    sc = scalars(0.707, 1.0, lap_order(B, nx, ny, 1.0))
    tb, tc, tx = (torch.from_numpy(v).to(cuda) for v in (b, c, x))
    spec = SeqSpec(B, nx, ny, T, src, prb, form=_lib.WT_FORM_PLAIN)
    out, _, _, ws = seq_forward(spec, sc, tb, tc, tx)
    gc, _ = seq_backward(spec, sc, tb, tc, tx, torch.from_numpy(g).to(cuda), ws, False)
    torch.cuda.synchronize()
    assert seq_device_status(spec, ws) == _lib.WT_OK
    assert np.array_equal(out.cpu().numpy(), oout)
    assert np.array_equal(gc.cpu().numpy(), ogc)
    spec_f = SeqSpec(B, nx, ny, T, src, [], form=_lib.WT_FORM_PLAIN, output_fields=True)
    _, fields, _, _ = seq_forward(spec_f, sc, tb, tc, tx)
    assert np.array_equal(fields.cpu().numpy(), hist)


def test_row_streaming_kernels_on_one_large_instance(cuda):
    """One instance of 2052 x 2052 (past the row-streaming threshold on its
    own): the adjoint accumulates dL/dc into the result itself (a block of
    one instance), 17 column chunks with taps on chunk edges; outputs and
    dL/dc bit-exact with the oracle."""
    B, nx, ny, T = 1, 2052, 2052, 6
    assert B * nx * ny >= 4 << 20
    src = [(1000 * ny + 1023, -1)]
    prb = [(1001 * ny + 1024, 1, 0), (1003 * ny + 2047, 0, 1), (999 * ny + 1151, 1, 2)]
    b, c, x = problem(nx, ny, B, T, 8)
    g = np.random.default_rng(9).standard_normal((B, T, len(prb))).astype(np.float32)
    S = o.Seq(B, nx, ny, T, 0.707, 1.0, src, prb)
    oout, hist = S.forward(b, c, x)
    ogc = S.backward(b, c, hist, g)[0]
    sc = scalars(0.707, 1.0, lap_order(B, nx, ny, 1.0))
    tb, tc, tx = (torch.from_numpy(v).to(cuda) for v in (b, c, x))
    spec = SeqSpec(B, nx, ny, T, src, prb, form=_lib.WT_FORM_PLAIN)
    out, _, _, ws = seq_forward(spec, sc, tb, tc, tx)
    gc, _ = seq_backward(spec, sc, tb, tc, tx, torch.from_numpy(g).to(cuda), ws, False)
    torch.cuda.synchronize()
    assert seq_device_status(spec, ws) == _lib.WT_OK
    assert np.array_equal(out.cpu().numpy(), oout)
    assert np.array_equal(gc.cpu().numpy(), ogc)
