"""Host-side behaviour of the drop-in modules (CPU only: no kernels run)."""
import json
import os

import numpy as np
import pytest
import torch

from conftest import GOLDEN, golden
import wavetorch_gb300 as wt
from wavetorch_gb300.functional import lap_order
from wavetorch_gb300 import _lib


def model_cfg0(N=100):
    geom = wt.WaveGeometryFreeForm((N, N), 1.0, c0=1.0, c1=0.5, abs_N=20, abs_sig=3.0, abs_p=2,
                                   rho=torch.rand(N, N, generator=torch.Generator().manual_seed(0)))
    cell = wt.WaveCell(0.707, geom)
    return wt.WaveRNN(cell, wt.WaveSource(20, 50), [wt.WaveIntensityProbe(80, y) for y in (35, 50, 65)])


def test_pml_profile_matches_reference_bit_exact():
    for name in ["cfg0_small", "cfg1_small", "geom_n160"]:
        d = golden(name)
        N = d["b"].shape[0]
        abs_N = 20 if name != "multi" else 10
        g = wt.WaveGeometryFreeForm((N, N), 1.0, c0=1.0, c1=0.5, abs_N=abs_N, abs_sig=3.0, abs_p=2)
        assert np.array_equal(g.b.numpy(), d["b"]), name


def test_blur_kernel_matches_reference():
    d = golden("cfg0_small")
    g = wt.WaveGeometryFreeForm((50, 50), 1.0, c0=1.0, c1=0.5, abs_N=10)
    assert np.array_equal(g.blur_kernel[0, 0].numpy(), d["blur_kernel"])


def test_state_dict_keys_match_reference():
    ref = json.load(open(os.path.join(GOLDEN, "state_keys.json")))
    geom = wt.WaveGeometryFreeForm((50, 50), 1.0, c0=1.0, c1=0.5, abs_N=10, abs_sig=3.0, abs_p=2,
                                   rho='half')
    model = wt.WaveRNN(wt.WaveCell(0.707, geom), [wt.WaveSource(10, 25)],
                       [wt.WaveIntensityProbe(40, y) for y in (15, 25, 35)])
    ours = {k: [list(v.shape), str(v.dtype)] for k, v in model.state_dict().items()}
    assert ours == ref


def test_cfl_violation_raises_value_error():
    geom = wt.WaveGeometryFreeForm((50, 50), 1.0, c0=1.0, c1=0.5, abs_N=10)
    with pytest.raises(ValueError, match="CFL"):
        wt.WaveCell(0.8, geom)
    wt.WaveCell(0.707, geom)   # 0.707 <= 1/sqrt(2)


def test_pml_must_fit():
    with pytest.raises(AssertionError):
        wt.WaveGeometryFreeForm((40, 40), 1.0, c0=1.0, c1=0.5, abs_N=20)


def test_rho_init_modes():
    for mode in ("half", "blank", "rand"):
        wt.WaveGeometryFreeForm((30, 30), 1.0, c0=1.0, c1=0.5, abs_N=5, rho=mode)
    with pytest.raises(ValueError):
        wt.WaveGeometryFreeForm((30, 30), 1.0, c0=1.0, c1=0.5, abs_N=5, rho='bogus')


def test_constrain_to_design_region_zeroes_pml():
    g = wt.WaveGeometryFreeForm((40, 40), 1.0, c0=1.0, c1=0.5, abs_N=8, rho='half')
    assert torch.all(g.rho[g.b > 0] == 0)
    assert torch.all(g.rho[g.b == 0] == 0.5)


def test_parameters_are_only_rho():
    m = model_cfg0(60)
    names = [p.shape for p in m.parameters()]
    assert names == [torch.Size([60, 60])]


def test_no_cpu_fallback():
    m = model_cfg0(60)
    with pytest.raises((RuntimeError, _lib.WaveKernelError), match="CUDA|cuda"):
        m(torch.zeros(1, 5))


def test_lap_order_rule():
    assert lap_order(1, 100, 100, 1.0) == _lib.WT_LAP_PAIRED
    assert lap_order(32, 120, 120, 1.0) == _lib.WT_LAP_SEQ
    assert lap_order(1, 1024, 1024, 1.0) == _lib.WT_LAP_SEQ
    assert lap_order(1, 100, 100, 1.43) == _lib.WT_LAP_SEQ


def test_source_table_broadcast_rules():
    geom = wt.WaveGeometryFreeForm((64, 64), 1.0, c0=1.0, c1=0.5, abs_N=10)
    line = wt.WaveLineSource(14, 12, 14, 50)
    m = wt.WaveRNN(wt.WaveCell(0.707, geom), [wt.WaveSource(20, 30), line],
                   [wt.WaveIntensityProbe(50, 20)])
    t1 = m.source_table(1)
    assert t1[0] == (20 * 64 + 30, -1)
    assert len(t1) == 1 + 39 and all(r == -1 for _, r in t1)
    with pytest.raises(RuntimeError, match="shape mismatch"):
        m.source_table(3)
    # batch == number of line cells: cell l takes instance l's input
    t39 = m.source_table(39)
    assert [r for _, r in t39[1:]] == list(range(39))


def test_line_cells_match_golden():
    d = golden("line")
    N = int(d["N"])
    cells = [cc for cc, _ in d["sources"]]
    a = wt.WaveLineSource(14, 12, 14, 50).cells()
    b = wt.WaveLineSource(20, 15, 31, 40).cells()
    assert [x * N + y for x, y in a + b] == cells


def test_probe_table_order():
    geom = wt.WaveGeometryFreeForm((48, 48), 1.0, c0=1.0, c1=0.5, abs_N=10)
    probes = [wt.WaveIntensityProbe(30, 20), wt.WaveProbe(30, 24), wt.WaveProbe(30, 20)]
    m = wt.WaveRNN(wt.WaveCell(0.707, geom), wt.WaveSource(12, 24), probes)
    table, L = m.probe_table()
    assert L == 1
    assert table == [(30 * 48 + 20, 1, 0), (30 * 48 + 24, 0, 1), (30 * 48 + 20, 0, 2)]


def test_save_load_roundtrip(tmp_path):
    m = model_cfg0(60)
    wt.io.save_model(m, "m", savedir=str(tmp_path) + "/", cfg={"dtype": "float32"}, verbose=False)
    m2, hist, geo_hist, cfg = wt.io.load_model(str(tmp_path / "m.pt"))
    for (k, v), (k2, v2) in zip(m.state_dict().items(), m2.state_dict().items()):
        assert k == k2 and torch.equal(v, v2)


def test_load_model_file_written_by_the_reference():
    """tests/golden/ref_model.pt was written by the reference's own
    io.save_model (wavetorch/io.py:13-40).  load_model rebuilds the same
    geometry (density, PML, class), the two sources and three probes in
    module order, and dt; probes come back as intensity probes, the
    reference loader's rule for files without probe kinds."""
    d = golden("ref_model")
    m, hist, geo_hist, cfg = wt.io.load_model(os.path.join(GOLDEN, "ref_model.pt"))
    assert cfg == {"dtype": "float32"} and hist is None and len(geo_hist) == 1
    g = m.cell.geom
    assert isinstance(g, wt.WaveGeometryFreeForm)
    assert np.array_equal(g.rho.detach().numpy(), d["rho"])
    assert np.array_equal(g.b.numpy(), d["b"])
    assert [s.cells() for s in m.sources] == [[(10, 20)], [(12, 14)]]
    assert [p.cells() for p in m.probes] == [[(30, 12)], [(30, 20)], [(30, 28)]]
    assert all(type(p) is wt.WaveIntensityProbe for p in m.probes)
    assert abs(m.cell.dt.item() - 0.707) < 1e-7
    ref_keys = set(torch.load(os.path.join(GOLDEN, "ref_model.pt"), weights_only=False)["model_state"])
    assert set(m.state_dict()) == ref_keys


def test_model_file_keeps_probe_kinds_and_line_sources(tmp_path):
    """Files written here record the probe classes (a key the reference's
    loader ignores), so amplitude probes stay amplitude probes; a line
    source comes back as a source over the same cells."""
    geom = wt.WaveGeometryFreeForm((48, 48), 1.0, c0=1.0, c1=0.5, abs_N=10)
    m = wt.WaveRNN(wt.WaveCell(0.707, geom), [wt.WaveLineSource(14, 12, 14, 30), wt.WaveSource(20, 20)],
                   [wt.WaveProbe(30, 20), wt.WaveIntensityProbe(30, 24)])
    wt.io.save_model(m, "k", savedir=str(tmp_path) + "/", cfg={"dtype": "float32"}, verbose=False)
    m2, _, _, _ = wt.io.load_model(str(tmp_path / "k.pt"))
    assert [type(p) for p in m2.probes] == [wt.WaveProbe, wt.WaveIntensityProbe]
    assert [s.cells() for s in m2.sources] == [s.cells() for s in m.sources]
    assert m2.source_table(1) == m.source_table(1)
    for (k, v), (k2, v2) in zip(m.state_dict().items(), m2.state_dict().items()):
        assert k == k2 and torch.equal(v, v2)


def test_synthetic_vowels_shape_and_norm():
    from wavetorch_gb300.data import vowel_like
    x, y = vowel_like(8, 3500, seed=3)
    assert x.shape == (8, 3500) and x.dtype == np.float32
    assert np.allclose(np.abs(x).max(axis=1), 1.0)
    assert set(np.unique(y)) <= {0, 1, 2}


def _holey(d, dev="cpu"):
    import wavetorch_gb300 as wt
    return wt.WaveGeometryHoley((64, 48), 1.0, c0=1.0, c1=0.5, abs_N=10, abs_sig=3.0, abs_p=2,
                                x=d["x"].tolist(), y=d["y"].tolist(), r=d["r"].tolist()).to(dev)


def test_holey_geometry_on_cpu_raises():
    """Hole geometries have no CPU path: reading rho or c of CPU-held holes
    raises, as every wave operation on CPU tensors does (the oracle, not the
    product, evaluates them on the CPU: tests/test_oracle_golden.py)."""
    d = golden("holey")
    geom = _holey(d)
    for name in ("rho", "c"):
        with pytest.raises((RuntimeError, TypeError, ValueError)):
            getattr(geom, name)


def test_ragged_cluster_choice():
    """The ragged autotuner's choice from measured times: the size of least
    SM-time per group (groups share the SMs), unless a group alone would
    then outlast the whole batch; a group of G instances takes G x size SMs."""
    from wavetorch_gb300.ragged import pick_cluster_sizes
    small = {1: 1.8, 2: 1.1, 4: 0.8, 8: 0.6}          # seconds per size
    # many groups: the cheapest size (1 SM x 1.8) everywhere
    assert pick_cluster_sizes([(small, 1.0, 1)] * 200 + [({16: 1.0}, 1.0, 1)], 152) == [1] * 200 + [16]
    # one long group on an idle machine: alone it would set the step -> faster sizes
    assert pick_cluster_sizes([(small, 10.0, 1), ({16: 0.5}, 1.0, 1)], 152) == [8, 16]
    # a group of 40 instances at size 2 already fills the machine's SM-time bound
    assert pick_cluster_sizes([(small, 1.0, 40)], 80) == [2]


def test_ragged_layout_choice_with_band_options():
    """Options may be (cluster, bands) pairs: a band option with at most p
    CTAs per model counts p SMs per model; the least SM-time wins."""
    from wavetorch_gb300.ragged import _option_spec, pick_cluster_sizes
    big = {(16, 0): 2.0, (-1, 8): 2.9, (-1, 12): 2.2}      # SM-times 32, 23.2, 26.4
    assert pick_cluster_sizes([(big, 1.0, 1)] * 100, 152) == [(-1, 8)] * 100
    # alone on the machine it would set the step: the fastest option instead
    assert pick_cluster_sizes([(big, 1.0, 1)], 152) == [(16, 0)]
    assert _option_spec((-1, 8), 3) == (-1, 24) and _option_spec((4, 0), 3) == (4, 0)


def test_ragged_strip_trial_keeps_the_step_ratios():
    """The packed batch's strip-height trial runs every model on one scaled
    step count: the longest gets exactly `steps`, the others keep their
    ratio to it (rounded up, at least one step, never more than their own)."""
    from wavetorch_gb300.ragged import trial_steps
    T = [4000, 2000, 500, 3999, 7]
    got = trial_steps(T, 256)
    assert got[0] == 256 and got[1] == 128 and got[2] == 32 and got[3] == 256
    assert got[4] == 1
    assert trial_steps([100, 50], 256) == [100, 50]          # short runs: their own counts
    ratios = [g / t for g, t in zip(trial_steps(T[:4], 256), T[:4])]
    assert max(ratios) - min(ratios) < 1e-3 * 5


def test_save_load_roundtrip_hole_geometry(tmp_path):
    """A model on a hole geometry round-trips through the model file: the
    geometry class is rebuilt by name from its reconstruction arguments
    (holes' centres and radii, eta, beta), as in the reference's io."""
    geom = wt.WaveGeometryHoley((48, 40), 1.0, c0=1.0, c1=0.5, abs_N=8, abs_sig=3.0, abs_p=2,
                                x=[20.5, 30.25], y=[10.5, 25.75], r=[3.0, 4.5])
    m = wt.WaveRNN(wt.WaveCell(0.707, geom), wt.WaveSource(10, 20),
                   [wt.WaveIntensityProbe(38, 20)])
    wt.io.save_model(m, "h", savedir=str(tmp_path) + "/", cfg={"dtype": "float32"}, verbose=False)
    m2, _, _, _ = wt.io.load_model(str(tmp_path / "h.pt"))
    g2 = m2.cell.geom
    assert isinstance(g2, wt.WaveGeometryHoley)
    for name in ("x", "y", "r", "eta", "beta", "b"):
        assert torch.equal(getattr(g2, name), getattr(geom, name)), name


def test_utils_match_the_reference_formulas():
    """wavetorch/utils.py:23-36: the centred window (int() truncation of
    len/2 -/+ w/2), the argmax accuracy, and the row normalisation of
    time-summed intensities that feeds the loss."""
    from wavetorch_gb300 import utils
    x = np.arange(11)
    assert list(utils.window_data(x, 4)) == [3, 4, 5, 6]         # [int(3.5):int(7.5)]
    assert list(utils.window_data(x, 5)) == [3, 4, 5, 6, 7]      # [int(3.0):int(8.0)]
    assert list(utils.window_data(np.arange(10), 3)) == [3, 4, 5]
    pred = torch.tensor([[0.1, 0.7, 0.2], [0.5, 0.3, 0.2], [0.2, 0.2, 0.6], [0.9, 0.05, 0.05]])
    assert utils.accuracy_onehot(pred, torch.tensor([1, 0, 1, 0])) == 0.75
    X = torch.tensor([[1.0, 3.0], [2.0, 2.0]])
    P = utils.normalize_power(X)
    assert torch.equal(P, torch.tensor([[0.25, 0.75], [0.5, 0.5]]))
    with pytest.raises(ValueError):
        utils.set_dtype("float16")
