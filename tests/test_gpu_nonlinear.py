"""The fused nonlinear sequence (saturable damping and Kerr term,
wavetorch/cell.py:8-9, :79-107) against the oracle, which reproduces the
reference's probe outputs and dL/dc_lin bit for bit (golden `nonlinear`), on a
rectangular grid and batch the fixture does not cover.  Probe outputs
bit-exact (the oracle is fed the kernels' own c, so the projection's tanh
ulps do not enter); dL/drho within 1e-5 (the kernels' adjoint sums each
instance over time before the batch, and forms the field gradient's terms
in its own order)."""
import numpy as np
import pytest
import torch

import oracle.oracle as o
import wavetorch_gb300 as wt
from wavetorch_gb300.data import vowel_like

pytestmark = pytest.mark.gpu


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("b0,cnl", [(0.05, 0.1), (0.05, 0.0), (0.0, 0.1)])
def test_fused_nonlinear_against_oracle(cuda, b0, cnl):
    nx, ny, B, T = 48, 40, 3, 50
    uth = float(np.sqrt(0.1))
    rho0 = torch.rand(nx, ny, generator=torch.Generator().manual_seed(31))
    geom = wt.WaveGeometryFreeForm((nx, ny), 1.0, c0=1.0, c1=0.5, abs_N=8, abs_sig=3.0, abs_p=2,
                                   rho=rho0)
    cell = wt.WaveCell(0.707, geom, satdamp_b0=b0, satdamp_uth=uth, c_nl=cnl)
    probes = [(36, 10), (36, 20), (30, 31)]
    m = wt.WaveRNN(cell, wt.WaveSource(10, 20),
                   [wt.WaveIntensityProbe(px, py) for px, py in probes]).to(cuda)
    x_np, lab = vowel_like(B, T, seed=31)
    x_np = (x_np * np.float32(0.2)).astype(np.float32)
    y = m(torch.from_numpy(x_np).to(cuda))
    loss = torch.nn.CrossEntropyLoss()(wt.utils.normalize_power(y.sum(dim=1)),
                                       torch.from_numpy(lab).to(cuda))
    loss.backward()
    got_out = y.detach().cpu().numpy()
    got_grad = m.cell.geom.rho.grad.cpu().numpy()

    g = m.cell.geom
    b = g.b.cpu().numpy()
    c_lin = g.c.detach().cpu().numpy()
    rho = g.rho.detach().cpu().numpy()
    S = o.Seq(B, nx, ny, T, 0.707, 1.0, [(10 * ny + 20, -1)],
              [(px * ny + py, 1, i) for i, (px, py) in enumerate(probes)])
    out, hist = o.seq_forward_nl(S, b, c_lin, rho, x_np, b0, uth, cnl)
    assert np.array_equal(got_out, out)

    yo = torch.from_numpy(out).requires_grad_()
    lo = torch.nn.CrossEntropyLoss()(wt.utils.normalize_power(yo.sum(dim=1)), torch.from_numpy(lab))
    (gout,) = torch.autograd.grad(lo, [yo])
    gc, gr = o.seq_backward_nl(S, b, c_lin, rho, hist, gout.numpy(), b0, uth, cnl)
    kern = g.blur_kernel[0, 0].cpu().numpy()
    _, th = o.rho_to_c(rho, kern, 1, 0.5, 100.0, 1.0, 0.5)
    want = gr + o.rho_to_c_bwd(th, kern, 1, 0.5, 100.0, 1.0, 0.5, gc)
    assert rel(got_grad, want) <= 1e-5
