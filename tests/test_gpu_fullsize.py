"""GPU checks at the benchmark configurations' full sizes: agreement with
the oracle on the batched training configuration (B=32, 120x120, T=3500),
the nonlinear configuration (B=64, 120x120, T=5000) and the large lens grid
(1024x1024, T=8000; the oracle keeps its 34 GB field history in host
memory), plain/fused agreement, and
size-independent properties (exact linearity under power-of-two input
scaling, silence for zero input)."""
import numpy as np
import pytest

from conftest import FUSED_DC_TOL
import torch

import oracle.oracle as o
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


def cfg1_problem(dev, B=32, N=120, steps=3500, seed=11):
    geom = wt.WaveGeometryFreeForm((N, N), 1.0, c0=1.0, c1=0.5, abs_N=20, abs_sig=3.0, abs_p=2,
                                   rho=torch.rand(N, N, generator=torch.Generator().manual_seed(seed)))
    geom = geom.to(dev)
    with torch.no_grad():
        c = geom.c.detach().contiguous()
    b = geom.b.contiguous()
    x, labels = vowel_like(B, steps, seed=seed)
    src = [(20 * N + 60, -1)]
    prb = [(80 * N + y, 1, i) for i, y in enumerate((35, 50, 65))]
    return b, c, torch.from_numpy(x).to(dev), labels, src, prb


def run(spec, sc, b, c, x, g=None):
    out, _, _, ws = seq_forward(spec, sc, b, c, x)
    gc = None
    if g is not None:
        gc, _ = seq_backward(spec, sc, b, c, x, g, ws, False)
    torch.cuda.synchronize()
    assert seq_device_status(spec, ws) == _lib.WT_OK
    return out, gc


def test_cfg1_batch_against_oracle(cuda):
    """The benchmark's batched training configuration at its full size (B=32,
    120x120, T=3500): plain form bit-exact with the oracle, fused form
    forward bit-exact and dL/dc within FUSED_DC_TOL."""
    B, N, steps = 32, 120, 3500
    b, c, x, _, src, prb = cfg1_problem(cuda, B, N, steps)
    g = torch.randn(B, steps, 3, generator=torch.Generator().manual_seed(5)).to(cuda)
    sc = scalars(0.707, 1.0, lap_order(B, N, N, 1.0))
    S = o.Seq(B, N, N, steps, 0.707, 1.0, src, prb)
    oout, hist = S.forward(b.cpu().numpy(), c.cpu().numpy(), x.cpu().numpy())
    ogc, _ = S.backward(b.cpu().numpy(), c.cpu().numpy(), hist, g.cpu().numpy())
    for form in (_lib.WT_FORM_PLAIN, _lib.WT_FORM_FUSED):
        spec = SeqSpec(B, N, N, steps, src, prb, form=form)
        out, gc = run(spec, sc, b, c, x, g)
        assert np.array_equal(out.cpu().numpy(), oout), form
        if form == _lib.WT_FORM_PLAIN:
            assert np.array_equal(gc.cpu().numpy(), ogc)
        else:
            assert rel(gc.cpu().numpy(), ogc) <= FUSED_DC_TOL


def test_cfg1_full_plain_vs_fused(cuda):
    """The benchmark workload (B=32, 120x120, T=3500): both forms agree."""
    b, c, x, _, src, prb = cfg1_problem(cuda)
    B, steps = x.shape
    N = 120
    g = torch.randn(B, steps, 3, generator=torch.Generator().manual_seed(6)).to(cuda)
    sc = scalars(0.707, 1.0, lap_order(B, N, N, 1.0))
    outs, gcs = {}, {}
    for form in (_lib.WT_FORM_PLAIN, _lib.WT_FORM_FUSED):
        spec = SeqSpec(B, N, N, steps, src, prb, form=form)
        outs[form], gcs[form] = run(spec, sc, b, c, x, g)
    assert torch.equal(outs[0], outs[1])
    # 3500 steps x 32 instances summed in a different order: within the
    # 1e-5 parity bar (measured 1.5e-6)
    assert rel(gcs[1].cpu().numpy(), gcs[0].cpu().numpy()) <= 1e-5
    assert torch.isfinite(gcs[1]).all()


@pytest.mark.parametrize("form", [_lib.WT_FORM_PLAIN, _lib.WT_FORM_FUSED])
def test_power_of_two_scaling_is_exact(cuda, form):
    """Scaling the input by 2 scales every field by 2 (a float32 multiply or
    add commutes exactly with a power of two except in the subnormal range,
    where rounding is absolute), so intensities scale by 4; dL/dc, the product
    of the doubled field's Laplacian and the doubled adjoint, scales by 4."""
    b, c, x, _, src, prb = cfg1_problem(cuda, B=32, N=120, steps=3500)
    B, steps = x.shape
    sc = scalars(0.707, 1.0, lap_order(B, 120, 120, 1.0))
    spec = SeqSpec(B, 120, 120, steps, src, prb, form=form)
    g = torch.randn(B, steps, 3, generator=torch.Generator().manual_seed(7)).to(cuda)
    o1, g1 = run(spec, sc, b, c, x, g)
    o2, g2 = run(spec, sc, b, c, 2 * x, g)
    assert rel(o2.cpu().numpy(), 4 * o1.cpu().numpy()) <= 1e-7
    # intensity seeds g * 2y double with y, so the adjoint doubles
    assert rel(g2.cpu().numpy(), 4 * g1.cpu().numpy()) <= 1e-7


def test_zero_input_is_silent(cuda):
    b, c, x, _, src, prb = cfg1_problem(cuda, B=4, N=120, steps=500)
    sc = scalars(0.707, 1.0, lap_order(4, 120, 120, 1.0))
    for form in (_lib.WT_FORM_PLAIN, _lib.WT_FORM_FUSED):
        spec = SeqSpec(4, 120, 120, 500, src, prb, form=form)
        out, _ = run(spec, sc, b, c, torch.zeros_like(x))
        assert torch.count_nonzero(out) == 0


def test_ragged_segments(cuda):
    """Checkpoint intervals that do not divide T, and the tape mode, give the
    same adjoint."""
    b, c, x, _, src, prb = cfg1_problem(cuda, B=3, N=120, steps=301)
    B, steps = x.shape
    sc = scalars(0.707, 1.0, lap_order(B, 120, 120, 1.0))
    g = torch.randn(B, steps, 3, generator=torch.Generator().manual_seed(8)).to(cuda)
    ref_spec = SeqSpec(B, 120, 120, steps, src, prb, form=_lib.WT_FORM_PLAIN)
    _, gref = run(ref_spec, sc, b, c, x, g)
    for seg in (1, 7, 64, 301, 1000, -1):   # -1: tape mode
        spec = SeqSpec(B, 120, 120, steps, src, prb, form=_lib.WT_FORM_FUSED, segment=seg)
        _, gf = run(spec, sc, b, c, x, g)
        assert rel(gf.cpu().numpy(), gref.cpu().numpy()) <= FUSED_DC_TOL, seg


@pytest.mark.parametrize("cluster", [1, 2, 4, 8])
def test_cluster_sizes_agree(cuda, cluster):
    N = 64
    geom = wt.WaveGeometryFreeForm((N, N), 1.0, c0=1.0, c1=0.5, abs_N=10, abs_sig=3.0, abs_p=2,
                                   rho=torch.rand(N, N, generator=torch.Generator().manual_seed(9))).to(cuda)
    with torch.no_grad():
        c = geom.c.contiguous()
    b = geom.b.contiguous()
    x = torch.from_numpy(vowel_like(2, 200, seed=9)[0]).to(cuda)
    src = [(10 * N + 32, -1)]
    prb = [(50 * N + 32, 1, 0), (50 * N + 20, 0, 1)]
    sc = scalars(0.707, 1.0, lap_order(2, N, N, 1.0))
    g = torch.randn(2, 200, 2, generator=torch.Generator().manual_seed(10)).to(cuda)
    p_out, p_gc = run(SeqSpec(2, N, N, 200, src, prb, form=_lib.WT_FORM_PLAIN), sc, b, c, x, g)
    f_out, f_gc = run(SeqSpec(2, N, N, 200, src, prb, form=_lib.WT_FORM_FUSED, cluster=cluster),
                      sc, b, c, x, g)
    assert torch.equal(p_out, f_out)
    assert rel(f_gc.cpu().numpy(), p_gc.cpu().numpy()) <= FUSED_DC_TOL


def test_tape_and_checkpoint_modes_agree_bitwise(cuda):
    """B=32, 120x120, first 700 steps: the adjoint that streams the stored
    Laplacians back and the one that recomputes segments from checkpoints do
    the same arithmetic on the same values, so dL/dc is identical."""
    b, c, x, _, src, prb = cfg1_problem(cuda, B=32, N=120, steps=3500)
    x = x[:, :700].contiguous()
    B, steps = x.shape
    sc = scalars(0.707, 1.0, lap_order(B, 120, 120, 1.0))
    g = torch.randn(B, steps, 3, generator=torch.Generator().manual_seed(12)).to(cuda)
    res = {}
    for seg in (-1, 0, 11, 50):
        spec = SeqSpec(B, 120, 120, steps, src, prb, form=_lib.WT_FORM_FUSED, segment=seg)
        res[seg] = run(spec, sc, b, c, x, g)
    for seg in (0, 11, 50):
        assert torch.equal(res[seg][0], res[-1][0]), seg
        assert torch.equal(res[seg][1], res[-1][1]), seg


@pytest.mark.parametrize("N", [200, 256])
def test_large_grids_fused_agree_with_plain(cuda, N):
    """Grids above 160x160 run on 16-CTA clusters: forward identical to the
    plain form (bit-exact with the reference), dL/dc within FUSED_DC_TOL."""
    geom = wt.WaveGeometryFreeForm((N, N), 1.0, c0=1.0, c1=0.5, abs_N=20, abs_sig=3.0, abs_p=2,
                                   rho=torch.rand(N, N, generator=torch.Generator().manual_seed(N))).to(cuda)
    with torch.no_grad():
        c = geom.c.contiguous()
    b = geom.b.contiguous()
    B, steps = 2, 300
    x = torch.from_numpy(vowel_like(B, steps, seed=N)[0]).to(cuda)
    src = [(20 * N + N // 2, -1)]
    prb = [((N - 20) * N + N // 2 + d, 1, i) for i, d in enumerate((-15, 0, 15))]
    sc = scalars(0.707, 1.0, lap_order(B, N, N, 1.0))
    g = torch.randn(B, steps, 3, generator=torch.Generator().manual_seed(1)).to(cuda)
    p_out, p_gc = run(SeqSpec(B, N, N, steps, src, prb, form=_lib.WT_FORM_PLAIN), sc, b, c, x, g)
    f_out, f_gc = run(SeqSpec(B, N, N, steps, src, prb, form=_lib.WT_FORM_FUSED), sc, b, c, x, g)
    assert torch.equal(p_out, f_out)
    assert rel(f_gc.cpu().numpy(), p_gc.cpu().numpy()) <= FUSED_DC_TOL


@pytest.mark.parametrize("N", [64, 150])
def test_per_instance_geometries(cuda, N):
    """coef_batched: three instances with their own rho (own c) in one fused
    launch agree with three separate single-instance runs of the plain form:
    outputs bit for bit, per-instance dL/dc within FUSED_DC_TOL."""
    B, steps = 3, 250
    cs, bs = [], None
    for i in range(B):
        geom = wt.WaveGeometryFreeForm((N, N), 1.0, c0=1.0, c1=0.5, abs_N=20, abs_sig=3.0, abs_p=2,
                                       rho=torch.rand(N, N, generator=torch.Generator().manual_seed(40 + i))).to(cuda)
        with torch.no_grad():
            cs.append(geom.c.contiguous())
        bs = geom.b.contiguous()
    c = torch.stack(cs).contiguous()
    b = bs.expand(B, N, N).contiguous()
    x = torch.from_numpy(vowel_like(B, steps, seed=N)[0]).to(cuda)
    src = [(20 * N + N // 2, -1)]
    prb = [((N - 20) * N + N // 2 + d, 1, i) for i, d in enumerate((-15, 0, 15))]
    sc = scalars(0.707, 1.0, lap_order(1, N, N, 1.0))      # each instance is a batch of one
    g = torch.randn(B, steps, 3, generator=torch.Generator().manual_seed(2)).to(cuda)
    spec = SeqSpec(B, N, N, steps, src, prb, form=_lib.WT_FORM_FUSED, coef_batched=True)
    out, gc = run(spec, sc, b, c, x, g)
    assert gc.shape == (B, N, N)
    for i in range(B):
        one = SeqSpec(1, N, N, steps, src, prb, form=_lib.WT_FORM_PLAIN)
        o1, g1 = run(one, sc, bs, cs[i], x[i:i + 1].contiguous(), g[i:i + 1].contiguous())
        assert torch.equal(out[i:i + 1], o1), i
        assert rel(gc[i].cpu().numpy(), g1.cpu().numpy()) <= FUSED_DC_TOL, i


@pytest.mark.parametrize("b0,cnl", [(0.05, 0.1), (0.05, 0.0), (0.0, 0.1)])
def test_nonlinear_fused_matches_step_form(cuda, b0, cnl):
    """B=4, 120x120, 400 steps, nonlinearity where rho > 0.5: the fused
    nonlinear sequence forms b and c with the same float32 operations as the
    per-step form, so the probe series agree bit for bit; dL/drho within 1e-5."""
    N, B, steps = 120, 4, 400
    rho0 = torch.rand(N, N, generator=torch.Generator().manual_seed(21))
    x = torch.from_numpy(vowel_like(B, steps, seed=21)[0] * np.float32(0.2)).to(cuda)
    labels = torch.tensor([0, 1, 2, 1], device=cuda)
    res = {}
    for form in ("step", "fused"):
        geom = wt.WaveGeometryFreeForm((N, N), 1.0, c0=1.0, c1=0.5, abs_N=20, abs_sig=3.0, abs_p=2,
                                       rho=rho0)
        cell = wt.WaveCell(0.707, geom, satdamp_b0=b0, satdamp_uth=float(np.sqrt(0.1)), c_nl=cnl)
        m = wt.WaveRNN(cell, wt.WaveSource(20, 60),
                       [wt.WaveIntensityProbe(80, y) for y in (35, 50, 65)], form=form).to(cuda)
        y = m(x)
        loss = torch.nn.CrossEntropyLoss()(wt.utils.normalize_power(y.sum(dim=1)), labels)
        loss.backward()
        res[form] = (y.detach(), m.cell.geom.rho.grad.detach())
    assert torch.equal(res["step"][0], res["fused"][0])
    assert rel(res["fused"][1].cpu().numpy(), res["step"][1].cpu().numpy()) <= 1e-5


def test_cfg2_nonlinear_full_size_against_oracle(cuda):
    """The nonlinear configuration at its full size: B=64, 120x120 (PML 20),
    T=5000, intensity-dependent speed (c_nl 0.1) and saturable damping (b0
    0.05, u_th sqrt(0.1)), inputs x 0.2 (inside the CFL limit).  The fused
    kernels' probe outputs are bit-exact with the oracle's on the same c; the
    training step's dL/drho (through the nonlinear adjoint and rho -> c) is
    within 1e-5."""
    N, B, T = 120, 64, 5000
    b0, uth, cnl = 0.05, float(np.sqrt(0.1)), 0.1
    rho0 = torch.rand(N, N, generator=torch.Generator().manual_seed(5))
    geom = wt.WaveGeometryFreeForm((N, N), 1.0, c0=1.0, c1=0.5, abs_N=20, abs_sig=3.0, abs_p=2,
                                   rho=rho0)
    m = wt.WaveRNN(wt.WaveCell(0.707, geom, satdamp_b0=b0, satdamp_uth=uth, c_nl=cnl),
                   wt.WaveSource(20, 60), [wt.WaveIntensityProbe(80, y) for y in (35, 50, 65)]
                   ).to(cuda)
    x_np, lab = vowel_like(B, T, seed=7)
    x_np = (x_np * np.float32(0.2)).astype(np.float32)
    y = m(torch.from_numpy(x_np).to(cuda))
    loss = torch.nn.CrossEntropyLoss()(wt.utils.normalize_power(y.sum(dim=1)),
                                       torch.from_numpy(lab).to(cuda))
    loss.backward()
    got_out = y.detach().cpu().numpy()
    got_grad = m.cell.geom.rho.grad.cpu().numpy()
    g = m.cell.geom
    b, rho = g.b.cpu().numpy(), g.rho.detach().cpu().numpy()
    c_lin = g.c.detach().cpu().numpy()
    S = o.Seq(B, N, N, T, 0.707, 1.0, [(20 * N + 60, -1)],
              [(80 * N + yy, 1, i) for i, yy in enumerate((35, 50, 65))])
    out, hist = o.seq_forward_nl(S, b, c_lin, rho, x_np, b0, uth, cnl)
    assert np.array_equal(got_out, out)
    yo = torch.from_numpy(out).requires_grad_()
    lo = torch.nn.CrossEntropyLoss()(wt.utils.normalize_power(yo.sum(dim=1)),
                                     torch.from_numpy(lab))
    (gout,) = torch.autograd.grad(lo, [yo])
    gc, gr = o.seq_backward_nl(S, b, c_lin, rho, hist, gout.numpy(), b0, uth, cnl)
    del hist
    kern = g.blur_kernel[0, 0].cpu().numpy()
    _, th = o.rho_to_c(rho, kern, 1, 0.5, 100.0, 1.0, 0.5)
    want = gr + o.rho_to_c_bwd(th, kern, 1, 0.5, 100.0, 1.0, 0.5, gc)
    assert rel(got_grad, want) <= 1e-5


def test_cfg3_lens_against_oracle(cuda):
    """The large-grid lens configuration: 1024x1024 (PML 40), line source at
    x=60 over y=200..824 driven by sin(2 pi 0.02 t), intensity probe at
    (900, 512), all 8000 steps (the wave reaches the focal point after about
    1200).  The fused form runs it in the band layout; its probe outputs are
    bit-exact with the oracle and dL/dc (objective -sum_t I) is within
    FUSED_DC_TOL."""
    from wavetorch_gb300.data import sinusoid
    N, T = 1024, 8000
    geom = wt.WaveGeometryFreeForm((N, N), 1.0, c0=1.0, c1=0.5, abs_N=40, abs_sig=3.0, abs_p=2,
                                   rho=torch.rand(N, N, generator=torch.Generator().manual_seed(3)))
    geom = geom.to(cuda)
    with torch.no_grad():
        c = geom.c.detach().contiguous()
    b = geom.b.contiguous()
    src = [(cell, -1) for cell in
           [x_ * N + y_ for x_, y_ in wt.WaveLineSource(60, 200, 60, 824).cells()]]
    prb = [(900 * N + 512, 1, 0)]
    x = torch.from_numpy(sinusoid(T, 0.02)).to(cuda)
    g = torch.full((1, T, 1), -1.0, device=cuda)          # d(-sum_t I)/dI_t
    spec = SeqSpec(1, N, N, T, src, prb, form=_lib.WT_FORM_FUSED)
    sc = scalars(0.707, 1.0, lap_order(1, N, N, 1.0))
    out, gc = run(spec, sc, b, c, x, g)
    S = o.Seq(1, N, N, T, 0.707, 1.0, src, prb)
    oout, hist = S.forward(b.cpu().numpy(), c.cpu().numpy(), x.cpu().numpy())
    assert np.abs(oout).max() > 0            # the wave has reached the probe
    assert np.array_equal(out.cpu().numpy(), oout)
    ogc, _ = S.backward(b.cpu().numpy(), c.cpu().numpy(), hist, g.cpu().numpy())
    del hist
    assert rel(gc.cpu().numpy(), ogc) <= FUSED_DC_TOL


@pytest.mark.parametrize("B,N,steps", [(560, 120, 12), (128, 256, 10), (37, 132, 20)])
def test_plain_large_batches_against_oracle(cuda, B, N, steps):
    """Large batches in the plain form (the batch reduction over 35, 8 and
    three blocks of 16 instances, the last one short, formed in the adjoint
    step's kernel; probes on the vector kernels' tile edges):
    outputs and dL/dc bit-exact with the oracle, i.e. with the reference's
    batch reduction order; the forward reads its coefficients from planes
    formed once per sequence."""
    b, c, x, _, _, _ = cfg1_problem(cuda, B=B, N=N, steps=steps, seed=17)
    src = [(20 * N + N // 2, -1)]
    # probes on tile edges: rows 7/8 (tiles of 8 rows), column 127/128
    prb = [(7 * N + N // 2, 1, 0), (8 * N + min(N - 1, 127), 1, 1), ((N - 20) * N + N // 2, 0, 2)]
    g = torch.randn(B, steps, 3, generator=torch.Generator().manual_seed(18)).to(cuda)
    sc = scalars(0.707, 1.0, lap_order(B, N, N, 1.0))
    S = o.Seq(B, N, N, steps, 0.707, 1.0, src, prb)
    oout, hist = S.forward(b.cpu().numpy(), c.cpu().numpy(), x.cpu().numpy())
    ogc, _ = S.backward(b.cpu().numpy(), c.cpu().numpy(), hist, g.cpu().numpy())
    out, gc = run(SeqSpec(B, N, N, steps, src, prb, form=_lib.WT_FORM_PLAIN), sc, b, c, x, g)
    assert np.array_equal(out.cpu().numpy(), oout)
    assert np.array_equal(gc.cpu().numpy(), ogc)
