"""Ragged batches: models of different grid sizes and step counts advanced
together (packed: one forward and one adjoint launch for all models; grouped:
one launch per group of equal grids), as one captured CUDA graph, give each
model the loss and dL/drho it gets when run alone through WaveRNN (tolerance
1e-5, the parity bar: the ragged step forms the loss gradient in closed
form, autograd op by op); the packed launch's probe outputs are bit-exact
with the oracle and its dL/dc within FUSED_DC_TOL."""
import numpy as np
import pytest
import torch

from conftest import FUSED_DC_TOL
import oracle.oracle as o
import wavetorch_gb300 as wt
from wavetorch_gb300 import _lib
from wavetorch_gb300.data import vowel_like
from wavetorch_gb300.ragged import RaggedBatch

pytestmark = pytest.mark.gpu


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def make(N, seed, dev):
    geom = wt.WaveGeometryFreeForm((N, N), 1.0, c0=1.0, c1=0.5, abs_N=20, abs_sig=3.0, abs_p=2,
                                   rho=torch.rand(N, N, generator=torch.Generator().manual_seed(seed)))
    cell = wt.WaveCell(0.707, geom)
    return wt.WaveRNN(cell, wt.WaveSource(20, N // 2),
                      [wt.WaveIntensityProbe(N - 20, N // 2 + d) for d in (-15, 0, 15)]).to(dev)


def _ragged_case(cuda):
    # enough steps for the wave to reach the probes (N - 40 cells away at
    # about 0.7 cells per step), else every intensity is 0 and the loss 0/0
    sizes = [64, 64, 100, 150, 200, 256]
    steps = [150, 120, 200, 260, 330, 400]
    models = [make(N, 100 + i, cuda) for i, N in enumerate(sizes)]
    inputs, labels = [], []
    for i, T in enumerate(steps):
        x, lab = vowel_like(1, T, seed=200 + i)
        inputs.append(torch.from_numpy(x[0]).to(cuda))
        labels.append(int(lab[0]))
    return models, inputs, labels


def _check_against_alone(cuda, rb, models, inputs, labels):
    for _ in range(2):                       # replays are repeatable
        losses = rb.step().clone()
    torch.cuda.synchronize()
    assert rb.device_status() == _lib.WT_OK
    grads = [m.cell.geom.rho.grad.clone() for m in models]
    for i, m in enumerate(models):
        m.cell.geom.rho.grad = None
        y = m(inputs[i][None])
        loss = torch.nn.CrossEntropyLoss()(wt.utils.normalize_power(y.sum(dim=1)),
                                           torch.tensor([labels[i]], device=cuda))
        loss.backward()
        assert abs(losses[i].item() - loss.item()) <= 1e-5 * abs(loss.item()), i
        assert rel(grads[i].cpu().numpy(), m.cell.geom.rho.grad.cpu().numpy()) <= 1e-5, i


@pytest.mark.parametrize("packed,strip", [(True, 0), (True, 4), (False, 0)])
@pytest.mark.parametrize("graph", [False, True])
def test_ragged_step_matches_models_run_alone(cuda, graph, packed, strip):
    models, inputs, labels = _ragged_case(cuda)
    rb = RaggedBatch(models, inputs, labels, graph=graph, packed=packed, strip=strip)
    if packed and strip:
        assert rb.strip == strip
    _check_against_alone(cuda, rb, models, inputs, labels)


def test_packed_launch_against_the_oracle(cuda):
    """Each model of a packed step (one forward launch for all six models,
    one adjoint launch) against the oracle run on that model alone, on the
    c the step computed: probe outputs bit-exact, dL/dc within
    FUSED_DC_TOL; the models' Laplacian orders differ (a batch of one:
    im2col order below 20,481 cells, oneDNN order above)."""
    models, inputs, labels = _ragged_case(cuda)
    rb = RaggedBatch(models, inputs, labels, graph=False, autotune=False)
    launches = _lib.kernel_launches()
    rb.step()
    torch.cuda.synchronize()
    assert rb.device_status() == _lib.WT_OK
    # rho -> c (blur + projection) and its adjoint (blur + projection) per
    # model, and the two sequence launches
    assert _lib.kernel_launches() - launches == 4 * len(models) + 2
    for i, m in enumerate(models):
        N = m.cell.geom.domain_shape[0]
        b = rb._b[i].cpu().numpy()
        c = rb._c[i].cpu().numpy()
        S = o.Seq(1, N, N, rb.T[i], 0.707, 1.0, m.source_table(1), m.probe_table()[0])
        out, hist = S.forward(b, c, rb._x[i][None].cpu().numpy())
        assert np.array_equal(rb._outs[i].cpu().numpy()[None], out), i
        gc, _ = S.backward(b, c, hist, rb._gouts[i].cpu().numpy()[None])
        assert rel(rb._gc[i].cpu().numpy(), gc) <= FUSED_DC_TOL, i


@pytest.mark.parametrize("graph", [False, True])
def test_ragged_groups_in_band_layout(cuda, graph):
    """Groups of the larger grids run in the band layout (at most 12 CTAs
    per instance, cooperative launches, captured in the step's CUDA graph
    too): same losses and gradients as the models run alone."""
    models, inputs, labels = _ragged_case(cuda)
    rb = RaggedBatch(models, inputs, labels, graph=False, autotune=False, packed=False)
    banded = 0
    for grp in rb.groups:
        if grp.N >= 200:
            grp.spec.cluster, grp.spec.sm_count = -1, 12 * len(grp.idx)
            banded += 1
    assert banded == 2
    if graph:
        rb._capture()
    _check_against_alone(cuda, rb, models, inputs, labels)
