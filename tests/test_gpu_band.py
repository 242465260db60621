"""The fused form's band layout (grids too large for one thread-block cluster:
bands of rows, one CTA per band, boundaries exchanged through global memory)
against the oracle, which is pinned bit for bit to the reference.  Probe
outputs bit-exact; dL/dc within FUSED_DC_TOL (the cluster layout's arithmetic)."""
import numpy as np
import pytest

from conftest import FUSED_DC_TOL
import torch

import oracle.oracle as o
from wavetorch_gb300 import _lib
from wavetorch_gb300.functional import (SeqSpec, fused_supported, lap_order, scalars,
                                        seq_backward, seq_device_status, seq_forward)
from wavetorch_gb300.geom import pml_profile

pytestmark = pytest.mark.gpu


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def problem(nx, ny, B, T, seed, abs_N=8, batched=False):
    rng = np.random.default_rng(seed)
    b = pml_profile((nx, ny), abs_N, 3.0, 2).numpy()
    shape = (B, nx, ny) if batched else (nx, ny)
    if batched:   # one geometry per instance: b and c are both [B, nx, ny]
        b = np.stack([b * np.float32(1 + 0.5 * k) for k in range(B)]).astype(np.float32)
    c = (0.5 + 0.5 * rng.random(shape)).astype(np.float32)
    t = np.arange(T, dtype=np.float32)
    x = np.stack([np.sin(0.21 * (k + 1) * t) for k in range(B)]).astype(np.float32)
    return b, c, x


def check(cuda, nx, ny, B, T, src, prb, seed=0, sm_count=0, grad_x=False, batched=False,
          cluster=0):
    b, c, x = problem(nx, ny, B, T, seed, batched=batched)
    g = np.random.default_rng(seed + 1).standard_normal((B, T, len(prb))).astype(np.float32)
    order = lap_order(B, nx, ny, 1.0)
    spec = SeqSpec(B, nx, ny, T, src, prb, form=_lib.WT_FORM_FUSED, sm_count=sm_count,
                   coef_batched=batched, cluster=cluster)
    assert fused_supported(spec)
    sc = scalars(0.707, 1.0, order)
    tb, tc, tx = (torch.from_numpy(v).to(cuda) for v in (b, c, x))
    out, _, psum, ws = seq_forward(spec, sc, tb, tc, tx, want_sum=True)
    gc, gx = seq_backward(spec, sc, tb, tc, tx, torch.from_numpy(g).to(cuda), ws, grad_x)
    torch.cuda.synchronize()
    assert seq_device_status(spec, ws) == _lib.WT_OK
    insts = range(B) if batched else [None]
    for k in insts:
        S = o.Seq(1 if batched else B, nx, ny, T, 0.707, 1.0, src, prb, order=order)
        ck = c[k] if batched else c
        bk = b[k] if batched else b
        xk = x[k:k + 1] if batched else x
        gk = g[k:k + 1] if batched else g
        oout, hist = S.forward(bk, ck, xk)
        ogc, ogx = S.backward(bk, ck, hist, gk, want_x=grad_x)
        got_out = out.cpu().numpy()[k:k + 1] if batched else out.cpu().numpy()
        assert np.array_equal(got_out, oout)
        got_gc = gc.cpu().numpy()[k] if batched else gc.cpu().numpy()
        assert rel(got_gc, ogc) <= FUSED_DC_TOL, rel(got_gc, ogc)
        if grad_x:
            assert rel(gx.cpu().numpy(), ogx) <= 1e-6
    # Kahan time sums of the outputs, as the cluster layout forms them
    s = np.zeros(psum.shape, np.float32)
    comp = np.zeros_like(s)
    for t in range(T):
        y = out.cpu().numpy()[:, t, :] - comp
        tk = s + y
        comp = (tk - s) - y
        s = tk
    assert np.array_equal(psum.cpu().numpy(), s)
    return out, gc


def test_lens_grid_line_source(cuda):
    """1024 x 1024 (the lens configuration's grid, 147 bands of 7 rows on
    152 SMs): a 625-cell line source on row 60, probes on the rows where
    bands meet (55/56, 62/63) and inside a band."""
    N, T = 1024, 48
    src = [(60 * N + y, -1) for y in range(200, 825)]
    prb = [(62 * N + 512, 1, 0), (63 * N + 500, 1, 1), (55 * N + 530, 0, 2), (70 * N + 512, 1, 3)]
    check(cuda, N, N, 1, T, src, prb)


def test_sources_and_probes_on_strip_and_band_edges(cuda):
    """1024 x 512, two instances on 152 SMs: 74 bands of 14 rows, each two
    strips of 7 rows (1024 threads).  Sources on row 63 (a band's second
    strip, first row), 69 (the band's last row) and 70 (the next band's first
    row): those strips pass their edge values on after the injection.  Probes
    on the rows where strips and bands meet."""
    N, W, T = 1024, 512, 40
    src = [(63 * W + 200, -1), (69 * W + 201, -1), (70 * W + 300, 1)]
    prb = [(56 * W + 200, 1, 0), (62 * W + 201, 1, 1), (70 * W + 301, 0, 2), (84 * W + 300, 1, 3)]
    check(cuda, N, W, 2, T, src, prb, sm_count=152)


@pytest.mark.parametrize("nx,ny,B", [(301, 530, 1), (301, 530, 2), (24, 600, 1), (160, 1000, 1)])
def test_ragged_edges(cuda, nx, ny, B):
    """Rows not a multiple of the band height (padding rows in the last band),
    columns not a multiple of 32 (padding threads), batches of two; 24 x 600
    takes the Laplacian order of torch's small-grid path."""
    src = [((nx // 3) * ny + ny // 2, -1)]
    prb = [((nx // 3 + 3) * ny + ny // 2 + 1, 1, 0), ((nx // 3 - 2) * ny + ny // 2, 0, 1),
           ((nx - 1) * ny + ny - 1, 1, 2)]
    check(cuda, nx, ny, B, 70, src, prb, seed=nx)


def test_several_strips_per_band(cuda):
    """Fewer SMs than bands of one strip: with 20 SMs a 300 x 300 grid runs
    19 bands of two 8-row strips (640 threads), exchanging inside a band
    through the tile and between bands through global memory."""
    N = 300
    src = [(40 * N + 150, -1), (40 * N + 151, -1)]
    prb = [(15 * N + 150, 1, 0), (16 * N + 149, 1, 1), (31 * N + 152, 0, 2), (100 * N + 150, 1, 3)]
    check(cuda, N, N, 1, 90, src, prb, sm_count=20)


def test_bands_requested_for_a_cluster_sized_grid(cuda):
    """cluster = -1 runs a grid one cluster would hold in bands (here 120 x 120,
    two instances on 16 SMs: bands of several strips), with the same results."""
    N = 120
    src = [(20 * N + 60, -1)]
    prb = [(80 * N + y, 1, k) for k, y in enumerate((35, 50, 65))]
    check(cuda, N, N, 2, 150, src, prb, sm_count=16, cluster=-1)


def test_input_gradient_and_per_instance_geometry(cuda):
    """dL/dx at a point source, and one geometry per instance
    (coef_batched) with per-instance dL/dc."""
    nx, ny = 280, 400
    src = [(100 * ny + 200, -1)]
    prb = [(110 * ny + 200, 1, 0), (95 * ny + 210, 1, 1)]
    check(cuda, nx, ny, 1, 60, src, prb, grad_x=True)
    check(cuda, nx, ny, 2, 60, src, prb, batched=True, seed=3)


def test_missing_arrival_times_out_and_the_context_survives(cuda):
    """A host-forced missing arrival: one band never sends its boundary rows
    (the test hook wt_test_band_missing_arrival).  Its neighbours' bounded
    waits give up after about 2 s, the launch's abort word stops every band,
    the status word reads WT_ERR_TIMEOUT, and the next sequence on the same
    context is correct."""
    import ctypes as C
    import time
    from wavetorch_gb300.functional import _ptr, _stream, seq_workspace_bytes
    nx, ny, B, T = 300, 400, 1, 40
    src = [(100 * ny + 200, -1)]
    prb = [(110 * ny + 200, 1, 0)]
    b, c, x = problem(nx, ny, B, T, 7)
    spec = SeqSpec(B, nx, ny, T, src, prb, form=_lib.WT_FORM_FUSED)
    sc = scalars(0.707, 1.0, lap_order(B, nx, ny, 1.0))
    d, keep = spec.desc()
    n = seq_workspace_bytes(spec)
    ws = torch.empty(n, dtype=torch.uint8, device=cuda)
    out = torch.empty(B, T, 1, device=cuda)
    tb, tc, tx = (torch.from_numpy(v).to(cuda) for v in (b, c, x))
    lib = _lib.load()
    fn = lib.wt_test_band_missing_arrival
    fn.argtypes = [C.POINTER(_lib.Scalars), C.POINTER(_lib.SeqDesc)] + [C.c_void_p] * 5 + \
                  [C.c_size_t, C.c_int32, C.c_void_p]
    fn.restype = C.c_int
    torch.cuda.synchronize()
    t0 = time.time()
    assert fn(C.byref(sc), C.byref(d), _ptr(tb), _ptr(tc), _ptr(tx), _ptr(out), _ptr(ws), n, 2,
              _stream(cuda)) == _lib.WT_OK
    torch.cuda.synchronize()
    elapsed = time.time() - t0
    assert seq_device_status(spec, ws) == _lib.WT_ERR_TIMEOUT
    assert 1.5 < elapsed < 60, elapsed
    check(cuda, nx, ny, B, T, src, prb, seed=7)



@pytest.mark.parametrize("B", [2, 3])
def test_band_rounds_against_oracle(cuda, B):
    """A batch whose bands outnumber the SMs it may use (300 x 300 grid: 13
    bands per instance on 16 SMs): the band layout runs in rounds, a work
    list of (instance, band) items per CTA; probe outputs bit-exact with the
    oracle, dL/dc within FUSED_DC_TOL, the status word clean."""
    nx, ny, T = 300, 300, 60
    src = [(100 * ny + 200, -1)]
    prb = [(110 * ny + 200, 1, 0), (150 * ny + 101, 0, 1)]
    b, c, x = problem(nx, ny, B, T, 9)
    g = np.random.default_rng(10).standard_normal((B, T, 2)).astype(np.float32)
    spec = SeqSpec(B, nx, ny, T, src, prb, form=_lib.WT_FORM_FUSED, sm_count=16)
    assert fused_supported(spec)
    sc = scalars(0.707, 1.0, lap_order(B, nx, ny, 1.0))
    tb, tc, tx = (torch.from_numpy(v).to(cuda) for v in (b, c, x))
    out, _, _, ws = seq_forward(spec, sc, tb, tc, tx)
    gc, _ = seq_backward(spec, sc, tb, tc, tx, torch.from_numpy(g).to(cuda), ws, False)
    torch.cuda.synchronize()
    assert seq_device_status(spec, ws) == _lib.WT_OK
    S = o.Seq(B, nx, ny, T, 0.707, 1.0, src, prb)
    oout, hist = S.forward(b, c, x)
    ogc, _ = S.backward(b, c, hist, g)
    assert np.array_equal(out.cpu().numpy(), oout)
    assert rel(gc.cpu().numpy(), ogc) <= FUSED_DC_TOL


def test_lens_grid_batch_of_two_runs_fused(cuda):
    """The lens grid (1024x1024, PML 40) with a batch of two: 2 x 147 bands
    outnumber the 152 SMs, so the fused form runs the bands in rounds
    instead of falling back to the plain form.  A point source per instance
    (the reference's line source broadcasts a batch only when it equals the
    line's length, wavetorch/source.py:19-20); T=200; outputs bit-exact with
    the oracle, dL/dc within FUSED_DC_TOL."""
    import wavetorch_gb300 as wt
    N, B, T = 1024, 2, 200
    geom = wt.WaveGeometryFreeForm((N, N), 1.0, c0=1.0, c1=0.5, abs_N=40, abs_sig=3.0, abs_p=2,
                                   rho=torch.rand(N, N, generator=torch.Generator().manual_seed(3)))
    geom = geom.to(cuda)
    with torch.no_grad():
        c = geom.c.detach().contiguous()
    b = geom.b.contiguous()
    src = [(60 * N + 512, -1)]
    prb = [(160 * N + 512, 1, 0)]
    t = np.arange(T, dtype=np.float32)
    x = np.stack([np.sin(2 * np.pi * 0.02 * t), np.sin(2 * np.pi * 0.03 * t)]).astype(np.float32)
    g = np.random.default_rng(4).standard_normal((B, T, 1)).astype(np.float32)
    spec = SeqSpec(B, N, N, T, src, prb, form=_lib.WT_FORM_FUSED)
    assert fused_supported(spec)
    sc = scalars(0.707, 1.0, lap_order(B, N, N, 1.0))
    tx = torch.from_numpy(x).to(cuda)
    out, _, _, ws = seq_forward(spec, sc, b, c, tx)
    gc, _ = seq_backward(spec, sc, b, c, tx, torch.from_numpy(g).to(cuda), ws, False)
    torch.cuda.synchronize()
    assert seq_device_status(spec, ws) == _lib.WT_OK
    S = o.Seq(B, N, N, T, 0.707, 1.0, src, prb)
    oout, hist = S.forward(b.cpu().numpy(), c.cpu().numpy(), x)
    ogc, _ = S.backward(b.cpu().numpy(), c.cpu().numpy(), hist, g)
    assert np.abs(oout).max() > 0
    assert np.array_equal(out.cpu().numpy(), oout)
    assert rel(gc.cpu().numpy(), ogc) <= FUSED_DC_TOL


def _band_modes(cuda, nx, ny, B, T, src, prb, segments, sm_count, seed):
    """Outputs, probe sums, dL/dc and dL/dx of the band layout from the tape
    and from checkpoints every `segment` steps (each segment recomputed by
    one launch, its adjoint steps run by the next)."""
    b, c, x = problem(nx, ny, B, T, seed)
    g = np.random.default_rng(seed + 1).standard_normal((B, T, len(prb))).astype(np.float32)
    sc = scalars(0.707, 1.0, lap_order(B, nx, ny, 1.0))
    tb, tc, tx = (torch.from_numpy(v).to(cuda) for v in (b, c, x))
    tg = torch.from_numpy(g).to(cuda)
    res = {}
    for seg in (-1,) + tuple(segments):
        spec = SeqSpec(B, nx, ny, T, src, prb, form=_lib.WT_FORM_FUSED, sm_count=sm_count,
                       segment=seg, cluster=-1)
        out, _, psum, ws = seq_forward(spec, sc, tb, tc, tx, want_sum=True)
        gc, gx = seq_backward(spec, sc, tb, tc, tx, tg, ws, len(src) == 1)
        torch.cuda.synchronize()
        assert seq_device_status(spec, ws) == _lib.WT_OK
        res[seg] = (out, psum, gc) + ((gx,) if gx is not None else ())
    return res


@pytest.mark.parametrize("segments", [(1, 7, 50), (120, 500)])
def test_band_checkpoints_equal_the_tape(cuda, segments):
    """300 x 300 in bands on 16 SMs, T=120: from checkpoints (one-step
    segments, intervals that do not divide T, a single segment) the outputs,
    probe sums, dL/dc and dL/dx equal the tape mode's bit for bit."""
    N = 300
    src = [(40 * N + 150, -1)]
    prb = [(260 * N + 150, 1, 0), (131 * N + 20, 0, 1)]
    res = _band_modes(cuda, N, N, 1, 120, src, prb, segments, 16, 41)
    for seg in segments:
        for a, t_ in zip(res[seg], res[-1]):
            assert torch.equal(a, t_), seg


def test_band_checkpoints_in_rounds_equal_the_tape(cuda):
    """Three instances whose bands outnumber 16 SMs run in rounds; from
    checkpoints every 13 steps they agree with the tape bit for bit."""
    N = 300
    src = [(40 * N + 150, -1)]
    prb = [(260 * N + 150, 1, 0)]
    res = _band_modes(cuda, N, N, 3, 90, src, prb, (13,), 16, 42)
    for a, t_ in zip(res[13], res[-1]):
        assert torch.equal(a, t_)


def test_lens_grid_checkpoints_equal_the_tape(cuda):
    """The lens grid (1024 x 1024, 147 bands), T=300, sqrt(T) segments."""
    N = 1024
    src = [(60 * N + y, -1) for y in range(200, 825)]
    prb = [(900 * N + 512, 1, 0)]
    res = _band_modes(cuda, N, N, 1, 300, src, prb, (18,), 0, 43)
    for a, t_ in zip(res[18], res[-1]):
        assert torch.equal(a, t_)
