"""The hole geometry's kernels (wt_holey_fwd/bwd) against the reference's
golden vectors and the oracle, and inside a training step."""
import numpy as np
import pytest
import torch

from conftest import golden
import oracle.oracle as o
import wavetorch_gb300 as wt

pytestmark = pytest.mark.gpu

ETA, BETA, C0, C1 = 0.5, 100.0, 1.0, 0.5


def holey(shape, x, y, r, dev):
    return wt.WaveGeometryHoley(shape, 1.0, c0=C0, c1=C1, abs_N=10, abs_sig=3.0, abs_p=2,
                                x=list(map(float, x)), y=list(map(float, y)),
                                r=list(map(float, r))).to(dev)


def close(got, ref, tol):
    """Largest difference within tol times the largest magnitude."""
    return np.abs(got - ref).max() <= tol * max(np.abs(ref).max(), 1e-30)


def test_matches_reference_golden(cuda):
    """rho, c and the gradients of sum(c * w) with respect to the holes'
    centres and radii against the reference run on the CPU (64x48, three
    holes).  exp and tanh differ from the reference's by an ulp at most, which
    the projection (beta = 100) turns into a few 1e-6 in a few cells."""
    d = golden("holey")
    geom = holey((64, 48), d["x"], d["y"], d["r"], cuda)
    c = geom.c
    loss = (c * torch.from_numpy(d["w"]).to(cuda)).sum()
    gx, gy, gr = torch.autograd.grad(loss, [geom.x, geom.y, geom.r])
    rho = geom.rho.detach().cpu().numpy()
    assert np.abs(rho - d["rho"]).max() <= 5e-6
    assert np.count_nonzero(rho != d["rho"]) <= 0.005 * rho.size
    assert np.abs(c.detach().cpu().numpy() - d["c"]).max() <= 5e-6
    for got, key in ((gx, "grad_x"), (gy, "grad_y"), (gr, "grad_r")):
        assert close(got.cpu().numpy(), d[key], 2e-5), key


@pytest.mark.parametrize("shape,nh", [((150, 110), 12), ((64, 64), 1), ((333, 257), 40)])
def test_matches_oracle(cuda, shape, nh):
    """Random holes (centres off the grid points) on grids of several shapes,
    gradients through both outputs: rho and c equal to the oracle's, the
    gradients within 1e-6 of the largest."""
    rng = np.random.default_rng(nh)
    x = rng.uniform(0, shape[0] - 1, nh).astype(np.float32) + np.float32(0.25)
    y = rng.uniform(0, shape[1] - 1, nh).astype(np.float32) + np.float32(0.375)
    r = rng.uniform(2.0, 12.0, nh).astype(np.float32)
    wr = rng.standard_normal(shape).astype(np.float32)
    wc = rng.standard_normal(shape).astype(np.float32)
    geom = holey(shape, x, y, r, cuda)
    rho, c = geom._rho_c()
    loss = (rho * torch.from_numpy(wr).to(cuda)).sum() + (c * torch.from_numpy(wc).to(cuda)).sum()
    gx, gy, gr = torch.autograd.grad(loss, [geom.x, geom.y, geom.r])
    orho, oc, th = o.holey(shape[0], shape[1], x, y, r, ETA, BETA, C0, C1)
    assert np.count_nonzero(rho.detach().cpu().numpy() != orho) <= 2
    assert np.abs(rho.detach().cpu().numpy() - orho).max() <= 5e-6
    assert np.abs(c.detach().cpu().numpy() - oc).max() <= 5e-6
    ogx, ogy, ogr = o.holey_bwd(x, y, r, th, ETA, BETA, C0, C1, grad_rho=wr, grad_c=wc)
    for got, ref in ((gx, ogx), (gy, ogy), (gr, ogr)):
        assert close(got.cpu().numpy(), ref, 1e-6)


def test_no_holes_and_shortest_list(cuda):
    """No holes: rho = P(0) everywhere.  Lists of different lengths: the
    holes are the shortest list's (the reference zips them), and the extra
    entries get zero gradients."""
    geom = holey((40, 30), [], [], [], cuda)
    orho, oc, _ = o.holey(40, 30, [], [], [], ETA, BETA, C0, C1)
    assert np.array_equal(geom.rho.detach().cpu().numpy(), orho)
    assert np.array_equal(geom.c.detach().cpu().numpy(), oc)

    geom = holey((40, 30), [10.5, 20.5, 30.5, 5.5], [7.25, 15.25, 22.25, 3.25], [3.0, 4.0, 2.5], cuda)
    c = geom.c
    gx, = torch.autograd.grad(c.sum(), [geom.x])
    orho, oc, th = o.holey(40, 30, [10.5, 20.5, 30.5], [7.25, 15.25, 22.25], [3.0, 4.0, 2.5],
                           ETA, BETA, C0, C1)
    assert np.abs(c.detach().cpu().numpy() - oc).max() <= 5e-6
    assert gx.shape == (4,) and gx[3].item() == 0.0


def test_training_step_through_holes(cuda):
    """A fused-form training step of a model on a hole geometry: the
    gradient with respect to the holes' centres and radii equals the
    oracle's sequence adjoint (dL/dc) carried through the oracle's hole
    adjoint, within 1e-5 of the largest."""
    N, B, T = 64, 2, 160
    hx, hy, hr = [20.5, 40.25, 31.75], [30.5, 22.25, 44.5], [4.0, 3.0, 5.0]
    geom = holey((N, N), hx, hy, hr, cuda)
    model = wt.WaveRNN(wt.WaveCell(0.707, geom), wt.WaveSource(12, 32),
                       [wt.WaveIntensityProbe(52, y) for y in (20, 32, 44)]).to(cuda)
    x = torch.from_numpy(np.sin(0.3 * np.arange(T, dtype=np.float32))[None].repeat(B, 0)).to(cuda)
    x[1] *= 0.5
    w = torch.randn(B, T, 3, generator=torch.Generator().manual_seed(5)).to(cuda)
    loss = (model(x) * w).sum()
    loss.backward()

    orho, oc, th = o.holey(N, N, hx, hy, hr, ETA, BETA, C0, C1)
    b = geom.b.cpu().numpy()
    S = o.Seq(B, N, N, T, 0.707, 1.0, [(12 * N + 32, -1)],
              [((52 * N + y), 1, k) for k, y in enumerate((20, 32, 44))])
    out, hist = S.forward(b, oc, x.cpu().numpy())
    gc, _ = S.backward(b, oc, hist, w.cpu().numpy())
    ogx, ogy, ogr = o.holey_bwd(hx, hy, hr, th, ETA, BETA, C0, C1, grad_c=gc)
    for p, ref in ((geom.x, ogx), (geom.y, ogy), (geom.r, ogr)):
        assert np.isfinite(p.grad.cpu().numpy()).all()
        assert close(p.grad.cpu().numpy(), ref, 1e-5)
