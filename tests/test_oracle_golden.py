"""Pin the CPU oracle against golden vectors produced by the reference itself.

Expected agreement (see oracle/wave_oracle.c):
  * sequence forward outputs and fields, and dL/dc: bit-exact (linear and
    nonlinear cells);
  * one-step backward: bit-exact except a few cells where torch's own
    kernels take a tail path (the last plane%16 cells of a batch sum over
    more than 16 instances; im2col+GEMM tail cells of single-instance grids);
  * rho -> c: the blur of small grids and tanh differ by ulps.
"""
import numpy as np
import pytest

from conftest import golden
import oracle.oracle as o

SEQ_CASES = ["cfg0_small", "cfg1_small", "multi", "line"]


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def seq_of(d):
    B, N, T = int(d["B"]), int(d["N"]), int(d["T"])
    return o.Seq(B, N, N, T, float(d["dt"]), float(d["h"]), [tuple(s) for s in d["sources"]],
                 [tuple(p) for p in d["probes"]])


@pytest.mark.parametrize("name", SEQ_CASES)
def test_seq_forward_bit_exact(name):
    d = golden(name)
    S = seq_of(d)
    out, hist = S.forward(d["b"], d["c"], d["x"])
    assert np.array_equal(out, d["out"])
    for k in d.files:
        if k.startswith("field_"):
            t = int(k.split("_")[1])
            assert np.array_equal(hist[:, t], d[k]), k


@pytest.mark.parametrize("name", SEQ_CASES)
def test_seq_backward_bit_exact(name):
    d = golden(name)
    S = seq_of(d)
    _, hist = S.forward(d["b"], d["c"], d["x"])
    gc, _ = S.backward(d["b"], d["c"], hist, d["grad_out"])
    assert np.array_equal(gc, d["grad_c"])


def test_lap_order_rule():
    # oneDNN for batch > 1 or > 20480 cells, else im2col+GEMM
    assert o.lap_order(1, 100, 100) == o.ORD_PAIRED
    assert o.lap_order(1, 143, 143) == o.ORD_PAIRED
    assert o.lap_order(1, 144, 144) == o.ORD_SEQ
    assert o.lap_order(2, 16, 16) == o.ORD_SEQ


@pytest.mark.parametrize("name", ["step_b2_h025", "step_b1_h1", "step_b20_h1"])
def test_timestep(name):
    d = golden(name)
    dt, h = float(d["dt"]), float(d["h"])
    y = o.step_fwd(d["b"], d["c"], d["y1"], d["y2"], dt, h)
    assert np.array_equal(y, d["y"])
    gb, gc, gy1, gy2 = o.step_bwd(d["b"], d["c"], d["y1"], d["y2"], d["grad_y"], dt, h)
    assert np.array_equal(gy1, d["grad_y1"])
    assert np.array_equal(gy2, d["grad_y2"])
    for got, ref in ((gb, d["grad_b"]), (gc, d["grad_c"])):
        assert np.count_nonzero(got != ref) <= 4
        assert rel(got, ref) < 1e-7


@pytest.mark.parametrize("name", ["cfg0_small", "geom_n100", "geom_n160"])
def test_rho_to_c(name):
    d = golden(name)
    c, th = o.rho_to_c(d["rho"], d["blur_kernel"], 1, 0.5, 100.0, 1.0, 0.5)
    assert rel(c, d["c"]) < 3e-7
    gr = o.rho_to_c_bwd(th, d["blur_kernel"], 1, 0.5, 100.0, 1.0, 0.5, d["grad_c"])
    assert rel(gr, d["grad_rho"]) < 5e-6


def test_nonlinear_cell():
    """The nonlinear cell (saturable damping and Kerr term, wavetorch/cell.py:
    8-9, :79-107; golden `nonlinear`: B=2, 40x40, T=60): probe outputs and
    dL/dc_lin bit-exact (the adjoint replays autograd's node order); dL/drho,
    the direct part plus the projection's, within 5e-6 (ulps of tanh in the
    projection, as in test_rho_to_c)."""
    d = golden("nonlinear")
    S = seq_of(d)
    nl = (float(d["satdamp_b0"]), float(d["satdamp_uth"]), float(d["c_nl"]))
    out, hist = o.seq_forward_nl(S, d["b"], d["c"], d["rho"], d["x"], *nl)
    assert np.array_equal(out, d["out"])
    gc, gr = o.seq_backward_nl(S, d["b"], d["c"], d["rho"], hist, d["grad_out"], *nl)
    assert np.array_equal(gc, d["grad_c"])
    _, th = o.rho_to_c(d["rho"], d["blur_kernel"], 1, 0.5, 100.0, 1.0, 0.5)
    total = gr + o.rho_to_c_bwd(th, d["blur_kernel"], 1, 0.5, 100.0, 1.0, 0.5, gc)
    assert rel(total, d["grad_rho"]) < 5e-6


def test_fp32_vs_fp64_floor():
    """The reference's own float32 error against its float64 run (the noise
    floor every float32 implementation sits on)."""
    d = golden("cfg0_small")
    assert rel(d["out"], d["out64"]) < 1e-4
    assert rel(d["grad_rho"], d["grad_rho64"]) < 1e-4
    for t in (99, 199):
        assert rel(d[f"field_{t}"], d[f"field64_{t}"]) < 1e-4
    assert not d["field64_0"].any()       # x_0 = sin(0): nothing injected yet


@pytest.mark.parametrize("name", ["fd64_linear", "fd64_nonlinear"])
def test_fp64_finite_difference_fixtures_match_reference_autograd(name):
    """The central differences (float64, eps 1e-5) that pin the GPU gradients
    agree with the reference's own float64 autograd gradient."""
    d = golden(name)
    fd, ag = d["fd_grad"], d["grad_rho64"]
    assert fd.shape == (16,)
    assert np.abs(fd - ag).max() <= 1e-7 * np.abs(fd).max()


@pytest.mark.parametrize("name", ["fd64_linear", "fd64_nonlinear"])
def test_oracle_gradient_against_fp64_central_differences(name):
    """The oracle's whole adjoint (sequence, nonlinear terms, projection) at
    16 design cells against central differences of the reference run in
    float64: within 1e-5 of the largest derivative (measured 2.6e-6 linear,
    1.2e-6 nonlinear).  This pins the adjoint's algebra independently of
    autograd's order."""
    import torch
    from wavetorch_gb300.geom import pml_profile
    from wavetorch_gb300.utils import normalize_power
    d = golden(name)
    B, N, T, abs_N = int(d["B"]), int(d["N"]), int(d["T"]), int(d["abs_N"])
    b = pml_profile((N, N), abs_N, 3.0, 2).numpy()
    kern = np.full((3, 3), np.float32(1.0) / np.float32(9.0), np.float32)
    rho = d["rho"]
    c, th = o.rho_to_c(rho, kern, 1, 0.5, 100.0, 1.0, 0.5)
    S = seq_of(d)
    nl = (float(d["satdamp_b0"]), float(d["satdamp_uth"]), float(d["c_nl"]))
    nonlinear = nl[0] > 0 or nl[2] != 0
    if nonlinear:
        out, hist = o.seq_forward_nl(S, b, c, rho, d["x"], *nl)
    else:
        out, hist = S.forward(b, c, d["x"])
    y = torch.from_numpy(out).requires_grad_()
    loss = torch.nn.CrossEntropyLoss()(normalize_power(y.sum(dim=1)), torch.from_numpy(d["labels"]))
    (g,) = torch.autograd.grad(loss, [y])
    if nonlinear:
        gc, direct = o.seq_backward_nl(S, b, c, rho, hist, g.numpy(), *nl)
    else:
        (gc, _), direct = S.backward(b, c, hist, g.numpy()), 0.0
    total = direct + o.rho_to_c_bwd(th, kern, 1, 0.5, 100.0, 1.0, 0.5, gc)
    ours = total.reshape(-1).astype(np.float64)[d["fd_index"]]
    fd = d["fd_grad"]
    assert np.abs(ours - fd).max() <= 1e-5 * np.abs(fd).max()


def test_holey_geometry():
    """The oracle's hole geometry against the reference's (golden `holey`:
    64x48, three holes, gradients of sum(c * w)).  A one-ulp difference in
    exp moves the projected density by up to beta/2 ulps, so a few cells
    differ by a few 1e-6."""
    d = golden("holey")
    rho, c, th = o.holey(64, 48, d["x"], d["y"], d["r"], 0.5, 100.0, 1.0, 0.5)
    assert np.abs(rho - d["rho"]).max() <= 5e-6
    assert np.abs(c - d["c"]).max() <= 5e-6
    assert np.count_nonzero(rho != d["rho"]) <= 0.005 * rho.size
    g = o.holey_bwd(d["x"], d["y"], d["r"], th, 0.5, 100.0, 1.0, 0.5, grad_c=d["w"])
    for got, key in zip(g, ("grad_x", "grad_y", "grad_r")):
        ref = d[key]
        assert np.abs(got - ref).max() <= 2e-5 * np.abs(ref).max(), key
