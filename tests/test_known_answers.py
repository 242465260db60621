"""Known-answer tests of the leapfrog (wavetorch/cell.py:12-17) and its
hand-written backward (wavetorch/cell.py:20-44) that need no golden file:

  * one step on an 8 x 8 grid against the update written out in float64;
  * the backward against float64 autograd of that update (the idea of the
    reference's study/utils/test_grad.py, with asserts);
  * a centred impulse on a homogeneous grid without PML keeps the grid's
    four-fold symmetry;
  * the scheme's discrete energy
        E_t = ||(y_t - y_{t-1}) / dt||^2 - c^2 <y_t, Lap y_{t-1}>
    is conserved without damping and never grows with damping b >= 0
    (multiply the update by y_{t+1} - y_{t-1} and sum over cells: the change
    of E is -(1/dt) sum b (y_{t+1} - y_{t-1})^2).

The CPU tests check the oracle; the GPU tests check the fields the CUDA
sequence kernels write (plain and fused forms) for the same properties and
against the oracle bit for bit."""
import numpy as np
import pytest
import torch

import oracle.oracle as o
from wavetorch_gb300.geom import pml_profile

DT = 0.707


def lap64(y, h):
    """Zero-padded 5-point Laplacian of [B, nx, ny] in float64."""
    p = np.pad(np.asarray(y, np.float64), [(0, 0), (1, 1), (1, 1)])
    return (p[:, :-2, 1:-1] + p[:, 2:, 1:-1] + p[:, 1:-1, :-2] + p[:, 1:-1, 2:]
            - 4 * p[:, 1:-1, 1:-1]) / (h * h)


def energy(F, dt, c, h):
    """E_t for t = 1 .. T-1 of the fields F [T, nx, ny] (uniform c)."""
    F = np.asarray(F, np.float64)
    dt = np.float64(np.float32(dt))
    E = []
    for t in range(1, F.shape[0]):
        v = (F[t] - F[t - 1]) / dt
        E.append((v * v).sum() - c * c * (F[t] * lap64(F[t - 1][None], h)[0]).sum())
    return np.array(E)


def symmetry_defect(F):
    """Largest deviation of [T, n, n] fields from their mirror images and
    transpose, relative to the largest field value."""
    d = max(np.abs(F - F[:, ::-1]).max(), np.abs(F - F[:, :, ::-1]).max(),
            np.abs(F - F.transpose(0, 2, 1)).max())
    return d / np.abs(F).max()


def impulse(T):
    x = np.zeros((1, T), np.float32)
    x[0, 0] = 1.0
    return x


def damping(kind, n):
    if kind == "none":
        return np.zeros((n, n), np.float32)
    if kind == "pml":
        return pml_profile((n, n), 8, 3.0, 2).numpy()
    return np.full((n, n), 0.02, np.float32)


def check_energy(kind, E):
    if kind == "none":      # conserved up to float32 rounding of the fields
        assert np.abs(E - E[0]).max() <= 1e-4 * E[0]
    else:                   # never grows (beyond rounding), and really decays
        assert np.diff(E).max() <= 1e-6 * E.max()
        assert E[-1] < 0.05 * E[0]


# ---------------------------------------------------------------------------
# oracle (CPU)

@pytest.mark.parametrize("h,dt", [(1.0, DT), (0.5, 0.35)])
def test_one_step_8x8_by_hand(h, dt):
    rng = np.random.default_rng(5)
    y1, y2 = (rng.standard_normal((2, 8, 8)).astype(np.float32) for _ in range(2))
    b = (0.5 * rng.random((8, 8))).astype(np.float32)
    c = (0.5 + 0.5 * rng.random((8, 8))).astype(np.float32)
    got = o.step_fwd(b, c, y1, y2, dt, h)
    bb, cc, a1, a2 = (v.astype(np.float64) for v in (b, c, y1, y2))
    t = np.float64(np.float32(dt))
    want = (t ** -2 + bb / t) ** -1 * (2 * t ** -2 * a1 - (t ** -2 - bb / t) * a2
                                       + cc ** 2 * lap64(a1, h))
    assert np.abs(got - want).max() <= 1e-6 * np.abs(want).max()


@pytest.mark.parametrize("h,dt", [(1.0, DT), (0.5, 0.35)])
def test_backward_matches_float64_autograd(h, dt):
    rng = np.random.default_rng(6)
    y1, y2, g = (rng.standard_normal((2, 8, 8)).astype(np.float32) for _ in range(3))
    b = (0.5 * rng.random((8, 8))).astype(np.float32)
    c = (0.5 + 0.5 * rng.random((8, 8))).astype(np.float32)
    got = o.step_bwd(b, c, y1, y2, g, dt, h)
    leaves = [torch.tensor(v, dtype=torch.float64, requires_grad=True) for v in (b, c, y1, y2)]
    tb, tc, t1, t2 = leaves
    t = float(np.float32(dt))
    k = torch.tensor([[0., 1, 0], [1, -4, 1], [0, 1, 0]], dtype=torch.float64)[None, None] / (h * h)
    lap = torch.nn.functional.conv2d(t1[:, None], k, padding=1)[:, 0]
    y = (t ** -2 + tb / t) ** -1 * (2 * t ** -2 * t1 - (t ** -2 - tb / t) * t2 + tc ** 2 * lap)
    want = torch.autograd.grad(y, leaves, torch.tensor(g, dtype=torch.float64))
    for name, a, w in zip(("b", "c", "y1", "y2"), got, want):
        w = w.numpy()
        assert np.linalg.norm(a - w) / np.linalg.norm(w) <= 1e-6, name


def test_centred_impulse_keeps_four_fold_symmetry():
    N, T = 33, 60
    S = o.Seq(1, N, N, T, DT, 1.0, [(16 * N + 16, -1)], [(16 * N + 16, 0, 0)])
    _, hist = S.forward(np.zeros((N, N), np.float32), np.ones((N, N), np.float32), impulse(T))
    assert np.abs(hist[0, -1]).max() > 0
    assert symmetry_defect(hist[0]) <= 1e-6


@pytest.mark.parametrize("kind", ["none", "pml", "uniform"])
def test_discrete_energy(kind):
    N, T = 48, 400
    S = o.Seq(1, N, N, T, DT, 1.0, [(20 * N + 27, -1)], [(30 * N + 20, 0, 0)])
    _, hist = S.forward(damping(kind, N), np.ones((N, N), np.float32), impulse(T))
    check_energy(kind, energy(hist[0], DT, 1.0, 1.0))


# ---------------------------------------------------------------------------
# CUDA kernels

def gpu_fields(cuda, form, b, c, x, src):
    from wavetorch_gb300 import _lib
    from wavetorch_gb300.functional import SeqSpec, lap_order, scalars, seq_forward
    n = c.shape[0]
    T = x.shape[1]
    spec = SeqSpec(1, n, n, T, src, [], form=form, output_fields=True)
    sc = scalars(DT, 1.0, lap_order(1, n, n, 1.0))
    tb, tc, tx = (torch.from_numpy(v).to(cuda) for v in (b, c, x))
    _, fields, _, _ = seq_forward(spec, sc, tb, tc, tx)
    torch.cuda.synchronize()
    return fields.cpu().numpy()[0]


FORMS = ["plain", "fused"]


@pytest.mark.gpu
@pytest.mark.parametrize("form", FORMS)
def test_gpu_centred_impulse_keeps_four_fold_symmetry(cuda, form):
    from wavetorch_gb300 import _lib
    N, T = 33, 60
    b, c = np.zeros((N, N), np.float32), np.ones((N, N), np.float32)
    src = [(16 * N + 16, -1)]
    F = gpu_fields(cuda, {"plain": _lib.WT_FORM_PLAIN, "fused": _lib.WT_FORM_FUSED}[form],
                   b, c, impulse(T), src)
    assert symmetry_defect(F) <= 1e-6
    _, hist = o.Seq(1, N, N, T, DT, 1.0, src, [(16 * N + 16, 0, 0)]).forward(b, c, impulse(T))
    assert np.array_equal(F, hist[0])


@pytest.mark.gpu
@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("kind", ["none", "pml", "uniform"])
def test_gpu_discrete_energy(cuda, form, kind):
    from wavetorch_gb300 import _lib
    N, T = 48, 400
    b, c = damping(kind, N), np.ones((N, N), np.float32)
    src = [(20 * N + 27, -1)]
    F = gpu_fields(cuda, {"plain": _lib.WT_FORM_PLAIN, "fused": _lib.WT_FORM_FUSED}[form],
                   b, c, impulse(T), src)
    check_energy(kind, energy(F, DT, 1.0, 1.0))
    _, hist = o.Seq(1, N, N, T, DT, 1.0, src, [(30 * N + 20, 0, 0)]).forward(b, c, impulse(T))
    assert np.array_equal(F, hist[0])
