"""The C-ABI library builds, loads and exports every symbol the header
declares; host-side argument validation (no GPU needed for any of this)."""
import ctypes as C
import os
import re
import shutil

import numpy as np
import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "wavetorch_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(wt_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    if not (shutil.which("nvcc") or os.path.exists("/usr/local/cuda/bin/nvcc")):
        pytest.skip("nvcc not available")
    from wavetorch_gb300 import _lib
    return _lib.load()


def declared_arity():
    """{function: number of parameters} from the header's prototypes."""
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    out = {}
    for name, params in re.findall(r"\b(wt_[a-z0-9_]+)\s*\(([^)]*)\)\s*;", text):
        params = params.strip()
        out[name] = 0 if params in ("", "void") else params.count(",") + 1
    return out


def test_ctypes_binding_matches_the_header(lib):
    """Every function the Python binding declares argument types for takes
    as many arguments as its prototype in the header (a mismatch would pass
    pointers in the wrong slots)."""
    from wavetorch_gb300 import _lib
    arity = declared_arity()
    checked = 0
    for name in _lib.EXPORTED:
        argtypes = getattr(lib, name).argtypes
        if argtypes is None:
            continue
        assert name in arity, name
        assert len(argtypes) == arity[name], (name, len(argtypes), arity[name])
        checked += 1
    assert checked >= 20


def test_header_declares_the_api():
    names = declared_functions()
    for n in ["wt_step_fwd", "wt_step_bwd", "wt_seq_fwd", "wt_seq_bwd", "wt_seq_workspace_bytes",
              "wt_rho_to_c_fwd", "wt_rho_to_c_bwd"]:
        assert n in names


def test_every_declared_symbol_is_exported(lib):
    from wavetorch_gb300 import _lib
    names = declared_functions()
    assert set(names) == set(_lib.EXPORTED)
    for n in names:
        assert hasattr(lib, n), n


def test_test_hooks_are_exported(lib):
    """The test hooks' header (outside the drop-in ABI) is exported too."""
    text = open(os.path.join(ROOT, "include", "wavetorch_gb300_testing.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = sorted(set(re.findall(r"\b(wt_[a-z0-9_]+)\s*\(", text)))
    assert names == ["wt_test_band_missing_arrival", "wt_test_cluster_missing_arrival",
                     "wt_test_device_peaks", "wt_test_device_peaks_scratch_floats",
                     "wt_test_tape_missing_slice"]
    for n in names:
        assert hasattr(lib, n), n


def test_version_and_status_strings(lib):
    assert b"sm_103a" in lib.wt_version()
    assert lib.wt_status_string(1) == b"invalid argument"


def _desc(B=2, N=32, T=10, sources=((5 * 32 + 16, -1),), probes=((20 * 32 + 16, 1, 0),),
          form=1, cluster=0):
    from wavetorch_gb300 import _lib
    src = (_lib.SourceEntry * max(1, len(sources)))(*[_lib.SourceEntry(*s) for s in sources])
    prb = (_lib.ProbeEntry * max(1, len(probes)))(*[_lib.ProbeEntry(*p) for p in probes])
    d = _lib.SeqDesc(B, N, N, T, len(sources), C.cast(src, C.POINTER(_lib.SourceEntry)),
                     len(probes), C.cast(prb, C.POINTER(_lib.ProbeEntry)), form, 0, cluster, 0, 0, 0)
    return d, (src, prb)


def test_workspace_query(lib):
    from wavetorch_gb300 import _lib
    for form in (0, 1):
        d, keep = _desc(form=form)
        n = C.c_size_t(0)
        assert lib.wt_seq_workspace_bytes(C.byref(d), C.byref(n)) == _lib.WT_OK
        assert n.value > 0
    # the plain form keeps every field: at least T * B * N * N floats
    d, keep = _desc(form=0, B=2, N=32, T=10)
    n = C.c_size_t(0)
    lib.wt_seq_workspace_bytes(C.byref(d), C.byref(n))
    assert n.value >= 10 * 2 * 32 * 32 * 4


@pytest.mark.parametrize("bad", [
    dict(sources=((32 * 32, -1),)),          # cell out of range
    dict(sources=((5, 2),)),                  # input row >= batch
    dict(probes=((5, 2, 0),)),                # unknown probe kind
    dict(probes=((-1, 1, 0),)),
    dict(B=0), dict(T=0), dict(form=7),
])
def test_invalid_descriptors_rejected(lib, bad):
    from wavetorch_gb300 import _lib
    d, keep = _desc(**bad)
    n = C.c_size_t(0)
    assert lib.wt_seq_workspace_bytes(C.byref(d), C.byref(n)) == _lib.WT_ERR_INVALID


def test_planner_on_random_valid_descriptors(lib):
    """The workspace planner (host code; it launches nothing) on 600 random
    valid descriptors,
    from 1x1 grids to 2048x2048, T up to 1e5, every form, adjoint mode,
    cluster request and flag: it answers OK or UNSUPPORTED, never INVALID,
    and an OK plan holds at least the probe amplitudes (and, for the plain
    form, every field)."""
    from wavetorch_gb300 import _lib
    rng = np.random.default_rng(0)
    sizes = [1, 2, 7, 16, 33, 64, 120, 160, 200, 256, 257, 300, 512, 1024, 2048]
    for _ in range(600):
        B = int(rng.choice([1, 2, 3, 32, 64, 200]))
        nx, ny = int(rng.choice(sizes)), int(rng.choice(sizes))
        T = int(rng.choice([1, 2, 3, 50, 3500, 100000]))
        srcs = tuple((int(rng.integers(0, nx * ny)), int(rng.choice([-1, 0, B - 1])))
                     for _ in range(int(rng.integers(0, 4))))
        prbs = tuple((int(rng.integers(0, nx * ny)), int(rng.integers(0, 2)), i)
                     for i in range(int(rng.integers(0, 5))))
        src = (_lib.SourceEntry * max(1, len(srcs)))(*[_lib.SourceEntry(*v) for v in srcs])
        prb = (_lib.ProbeEntry * max(1, len(prbs)))(*[_lib.ProbeEntry(*v) for v in prbs])
        form = int(rng.integers(0, 2))
        d = _lib.SeqDesc(B, nx, ny, T, len(srcs), C.cast(src, C.POINTER(_lib.SourceEntry)),
                         len(prbs), C.cast(prb, C.POINTER(_lib.ProbeEntry)), form,
                         int(rng.choice([-2, -1, 0, 1, 7, T])), int(rng.choice([-1, 0, 1, 2, 4, 16])),
                         int(rng.integers(0, 2)), int(rng.integers(0, 2)), 0)
        n = C.c_size_t(0)
        st = lib.wt_seq_workspace_bytes(C.byref(d), C.byref(n))
        assert st in (_lib.WT_OK, _lib.WT_ERR_UNSUPPORTED), (B, nx, ny, T, form)
        if st == _lib.WT_OK:
            assert n.value >= B * T * len(prbs) * 4
            if form == 0:
                assert n.value >= B * T * nx * ny * 4
        st = lib.wt_seq_workspace_bytes_nl(C.byref(d), C.byref(n))
        assert st in (_lib.WT_OK, _lib.WT_ERR_UNSUPPORTED)


def test_fused_tap_capacity(lib):
    """More than 4 source entries on one thread's cells is refused (the plain
    form serves it)."""
    from wavetorch_gb300 import _lib
    srcs = tuple((r * 32 + 16, -1) for r in range(1, 6))   # one column, 5 rows of one strip
    d, keep = _desc(sources=srcs, form=1)
    n = C.c_size_t(0)
    assert lib.wt_seq_workspace_bytes(C.byref(d), C.byref(n)) == _lib.WT_ERR_UNSUPPORTED
    d, keep = _desc(sources=srcs, form=0)
    assert lib.wt_seq_workspace_bytes(C.byref(d), C.byref(n)) == _lib.WT_OK


def test_fused_plan_size_limit(lib):
    """The cluster layout plans instances that fit one cluster (up to
    256x256, with 16-CTA clusters above 160); larger grids need the band
    layout, which needs the SMs for batch x bands CTAs (with one SM, none)."""
    from wavetorch_gb300.functional import SeqSpec, fused_supported
    for n in (160, 161, 200, 256):
        assert fused_supported(SeqSpec(2, n, n, 100, [(5, -1)], [(7, 1, 0)], sm_count=1)), n
    assert not fused_supported(SeqSpec(2, 257, 257, 100, [(5, -1)], [(7, 1, 0)], sm_count=1))
    assert not fused_supported(SeqSpec(1, 1024, 1024, 100, [(5, -1)], [(7, 1, 0)], sm_count=1))
    # the plain form takes any grid
    spec = SeqSpec(1, 1024, 1024, 100, [(5, -1)], [(7, 1, 0)], form=0)
    d, keep = spec.desc()
    n = C.c_size_t(0)
    assert lib.wt_seq_workspace_bytes(C.byref(d), C.byref(n)) == 0


def test_band_layout_plan(lib):
    """Grids no cluster holds run in bands of rows, one CTA per band and SM:
    1024x1024 on 152 SMs takes 147 bands of 7 rows (1024 threads), and its
    workspace is the tape (T x 147 x 1024 x 7 floats), the exchange words,
    dL/dc and the tables; a batch whose bands outnumber the SMs runs in
    rounds.  From checkpoints (segment > 0 or -2, or automatically past a
    64 GiB tape) it keeps the pairs of fields every `segment` steps, one
    segment's stash of Laplacians and the adjoint's per-cell state.  Refused
    (the caller uses the plain form): more than 1024 columns, field outputs,
    an explicit cluster size, more than two sources on one thread's cells."""
    from wavetorch_gb300 import _lib
    from wavetorch_gb300.functional import SeqSpec, fused_supported, seq_workspace_bytes
    N, T = 1024, 100
    src = [(60 * N + y, -1) for y in range(200, 825)]
    prb = [(900 * N + 512, 1, 0)]
    spec = SeqSpec(1, N, N, T, src, prb, sm_count=152)
    assert fused_supported(spec)
    tape = T * 147 * 1024 * 7 * 4
    halo = 147 * 4 * 1024 * 8
    ws = seq_workspace_bytes(spec)
    assert tape + halo + N * N * 4 < ws < tape + halo + N * N * 4 + 16 * 2**20
    assert seq_workspace_bytes(SeqSpec(1, N, N, T, src, prb, sm_count=152, segment=-1)) == ws

    def status(**kw):
        args = dict(batch=1, nx=N, ny=N, steps=T, sources=src, probes=prb, sm_count=152)
        args.update(kw)
        d, keep = SeqSpec(**args).desc()
        n = C.c_size_t(0)
        return lib.wt_seq_workspace_bytes(C.byref(d), C.byref(n))

    U = _lib.WT_ERR_UNSUPPORTED
    # 2 x 147 bands > 152 SMs: the bands run in rounds (a work list), with
    # both instances' tapes and a list of 2 x 147 items
    assert status(batch=2) == _lib.WT_OK
    ws2 = seq_workspace_bytes(SeqSpec(2, N, N, T, src, prb, sm_count=152))
    assert 2 * tape + 2 * halo < ws2 < 2 * ws + 16 * 2**20
    assert status(ny=1056, sources=[(61, -1)], probes=[(70, 1, 0)]) == U   # > 1024 columns
    assert status(output_fields=True, probes=[]) == U
    assert status(segment=50) == _lib.WT_OK
    assert status(segment=-2) == _lib.WT_OK
    slice_ = 147 * 1024 * 7 * 4                      # one step of tape
    ckpt = lambda seg: -(-T // seg) * 2 * N * N * 4 + seg * slice_ + 3 * slice_
    ws50 = seq_workspace_bytes(SeqSpec(1, N, N, T, src, prb, sm_count=152, segment=50))
    assert ckpt(50) + halo < ws50 < ckpt(50) + halo + N * N * 4 + 16 * 2**20
    ws_auto = seq_workspace_bytes(SeqSpec(1, N, N, T, src, prb, sm_count=152, segment=-2))
    assert ckpt(10) + halo < ws_auto < ckpt(10) + halo + N * N * 4 + 16 * 2**20   # ceil(sqrt(100))
    # a tape past 64 GiB: checkpoints in the automatic mode
    long_T = 20000
    assert seq_workspace_bytes(SeqSpec(1, N, N, long_T, src, prb, sm_count=152)) < 8 * 2**30
    assert status(cluster=4) == U
    assert status(sources=[(60 * N + 5, -1), (61 * N + 5, -1), (62 * N + 5, -1)]) == U
    assert status(sources=[(60 * N + 5, -1), (61 * N + 5, -1)]) == _lib.WT_OK
    assert status(sm_count=-1) == _lib.WT_ERR_INVALID
    many = [((900 + k // 1000) * N + k % 1000, 1, k) for k in range(1024)]
    assert status(probes=many) == U                  # probe columns beyond the tap words
    # several strips per band when bands of one strip would need too many SMs
    assert status(nx=300, ny=300, sources=[(61, -1)], probes=[(70, 1, 0)], sm_count=20) == _lib.WT_OK
    # cluster -1 asks for bands where a cluster would hold the grid; below -1 invalid
    small = dict(nx=120, ny=120, sources=[(20 * 120 + 60, -1)], probes=[(80 * 120 + 50, 1, 0)])
    assert status(cluster=-1, sm_count=16, **small) == _lib.WT_OK
    assert status(cluster=-1, sm_count=16, segment=-2, **small) == _lib.WT_OK
    assert status(cluster=-2, **small) == _lib.WT_ERR_INVALID
    sz = lambda **kw: seq_workspace_bytes(SeqSpec(1, 120, 120, T, [(20 * 120 + 60, -1)],
                                                  [(80 * 120 + 50, 1, 0)], **kw))
    assert sz(cluster=-1, sm_count=16) != sz(sm_count=16)   # a different layout


def test_fused_adjoint_modes(lib):
    """segment -1: tape (T x batch x nx x ny floats plus strip padding); > 0:
    checkpoints; 0: the tape up to 16 GiB, else checkpoints; -2: checkpoints
    at the automatic interval; below -2 invalid."""
    from wavetorch_gb300 import _lib
    from wavetorch_gb300.functional import SeqSpec, seq_workspace_bytes
    prb = [(80 * 120 + y, 1, i) for i, y in enumerate((35, 50, 65))]
    sz = lambda B, seg: seq_workspace_bytes(SeqSpec(B, 120, 120, 3500, [(2460, -1)], prb, segment=seg))
    tape = 3500 * 32 * 120 * 120 * 4
    assert tape <= sz(32, -1) < 1.1 * tape
    assert sz(32, 0) == sz(32, -1)
    assert sz(32, 11) < 2 * 2**30
    assert sz(128, 0) < 8 * 2**30         # a 25.8 GB tape: checkpoints instead
    assert sz(128, -1) > 4 * tape
    assert sz(32, -2) < 2 * 2**30            # -2: checkpoints at the automatic interval
    d, keep = SeqSpec(32, 120, 120, 3500, [(2460, -1)], prb, segment=-3).desc()
    n = C.c_size_t(0)
    assert lib.wt_seq_workspace_bytes(C.byref(d), C.byref(n)) == _lib.WT_ERR_INVALID


def test_checkpoint_workspace_is_a_small_fraction_of_the_tape(lib):
    """At the benchmark size (B=32, 120x120, T=3500) the checkpoints at
    sqrt(T) intervals and the two-segment recompute stash take hundreds of
    MB, against the tape's 6.9 GB."""
    from wavetorch_gb300.functional import SeqSpec, seq_workspace_bytes
    prb = [(80 * 120 + y, 1, i) for i, y in enumerate((35, 50, 65))]
    sz = lambda seg: seq_workspace_bytes(SeqSpec(32, 120, 120, 3500, [(2460, -1)], prb, segment=seg))
    assert sz(-1) > 6e9
    assert sz(60) < 6e8
    assert sz(-2) == sz(60)              # the automatic interval: ceil(sqrt(3500))


def test_per_instance_geometry_flag(lib):
    """coef_batched: fused form only; anything but 0/1 is invalid."""
    from wavetorch_gb300 import _lib
    n = C.c_size_t(0)
    d, keep = _desc(form=1)
    d.coef_batched = 1
    assert lib.wt_seq_workspace_bytes(C.byref(d), C.byref(n)) == _lib.WT_OK
    d, keep = _desc(form=0)
    d.coef_batched = 1
    assert lib.wt_seq_workspace_bytes(C.byref(d), C.byref(n)) == _lib.WT_ERR_UNSUPPORTED
    d.coef_batched = 2
    assert lib.wt_seq_workspace_bytes(C.byref(d), C.byref(n)) == _lib.WT_ERR_INVALID


def test_step_entry_points_validate_before_touching_the_device(lib):
    from wavetorch_gb300 import _lib
    sc = _lib.Scalars(0.707, 1.0, 0)
    assert lib.wt_step_fwd(C.byref(sc), 1, 8, 8, 0, None, None, None, None, None, None) == _lib.WT_ERR_INVALID
    bad = _lib.Scalars(-1.0, 1.0, 0)
    p = C.c_void_p(16)
    assert lib.wt_step_fwd(C.byref(bad), 1, 8, 8, 0, p, p, p, p, C.c_void_p(32), None) == _lib.WT_ERR_INVALID
    assert lib.wt_step_fwd(C.byref(sc), 1, 8, 8, 0, p, p, p, p, p, None) == _lib.WT_ERR_INVALID  # y aliases y1


def test_other_entry_points_validate_before_touching_the_device(lib):
    """Every compute entry point refuses missing buffers, a too-small
    workspace or bad descriptors with WT_ERR_INVALID before any device work
    (all buffer arguments here are NULL, so nothing can reach a device)."""
    from wavetorch_gb300 import _lib
    INV = _lib.WT_ERR_INVALID
    sc = _lib.Scalars(0.707, 1.0, 0)
    for form in (0, 1):
        d, keep = _desc(form=form)
        assert lib.wt_seq_fwd(C.byref(sc), C.byref(d), *([None] * 7), 0, None) == INV
        assert lib.wt_seq_bwd(C.byref(sc), C.byref(d), *([None] * 7), 0, None) == INV
        assert lib.wt_seq_device_status(C.byref(d), None, 0, None) == INV
    bad = _lib.Scalars(0.0, 1.0, 0)
    d, keep = _desc(form=1)
    assert lib.wt_seq_fwd(C.byref(bad), C.byref(d), *([None] * 7), 0, None) == INV
    assert lib.wt_seq_bwd_sum(C.byref(sc), C.byref(d), *([None] * 6), 0, None) == INV
    d0, keep0 = _desc(form=0)    # the probe-sum adjoint exists only in the fused form
    assert lib.wt_seq_bwd_sum(C.byref(sc), C.byref(d0), *([None] * 6), 0, None) == \
        _lib.WT_ERR_UNSUPPORTED
    nl = _lib.NonLinear(0.05, 0.3, 0.1)
    assert lib.wt_seq_fwd_nl(C.byref(sc), C.byref(d), C.byref(nl), *([None] * 7), 0, None) == INV
    assert lib.wt_seq_bwd_nl(C.byref(sc), C.byref(d), C.byref(nl), *([None] * 9), 0, None) == INV
    assert lib.wt_loss_ce_normalize_power(0, 3, None, None, None, None, None) == INV
    assert lib.wt_loss_ce_normalize_power(2, 3, None, None, None, None, None) == INV
    g = _lib.GeomDesc(10, 12, 1, 1, 0.5, 100.0, 1.0, 0.5)
    assert lib.wt_rho_to_c_fwd(C.byref(g), None, None, None, None, None) == INV
    assert lib.wt_rho_to_c_bwd(C.byref(g), None, None, None, None, None, None) == INV
    assert lib.wt_rho_to_c_fwd_noalloc(C.byref(g), None, None, None, None) == INV
    gbad = _lib.GeomDesc(0, 12, 1, 1, 0.5, 100.0, 1.0, 0.5)
    n = C.c_size_t(0)
    assert lib.wt_rho_to_c_work_bytes(C.byref(gbad), C.byref(n)) == INV
    h = _lib.HoleyDesc(64, 48, 3, 0.5, 100.0, 1.0, 0.5)
    assert lib.wt_holey_fwd(C.byref(h), *([None] * 7)) == INV
    assert lib.wt_holey_bwd(C.byref(h), *([None] * 10)) == INV
    assert lib.wt_holey_work_bytes(C.byref(h), None) == INV
    hbad = _lib.HoleyDesc(64, 0, 3, 0.5, 100.0, 1.0, 0.5)
    assert lib.wt_holey_work_bytes(C.byref(hbad), C.byref(n)) == INV


def test_geom_work_bytes(lib):
    from wavetorch_gb300 import _lib
    g = _lib.GeomDesc(10, 12, 1, 1, 0.5, 100.0, 1.0, 0.5)
    n = C.c_size_t(0)
    assert lib.wt_rho_to_c_work_bytes(C.byref(g), C.byref(n)) == 0
    assert n.value == 2 * 10 * 12 * 4


def test_ragged_plan_validates_arguments(lib):
    """wt_ragged_plan: no SMs, a group without options or instances, or a
    negative time is an invalid argument; an empty batch is fine."""
    from wavetorch_gb300 import _lib
    opt = (_lib.RaggedOption * 1)(_lib.RaggedOption(4, 4, 1.0))
    grp = (_lib.RaggedGroup * 1)(_lib.RaggedGroup(1, 1.0, 1, C.cast(opt, C.POINTER(_lib.RaggedOption))))
    out = (C.c_int32 * 1)()
    assert lib.wt_ragged_plan(grp, 1, 152, out) == _lib.WT_OK and out[0] == 0
    assert lib.wt_ragged_plan(grp, 1, 0, out) == _lib.WT_ERR_INVALID
    assert lib.wt_ragged_plan(grp, 0, 152, out) == _lib.WT_OK
    bad = (_lib.RaggedGroup * 1)(_lib.RaggedGroup(0, 1.0, 1, C.cast(opt, C.POINTER(_lib.RaggedOption))))
    assert lib.wt_ragged_plan(bad, 1, 152, out) == _lib.WT_ERR_INVALID
    neg = (_lib.RaggedOption * 1)(_lib.RaggedOption(4, 4, -1.0))
    grp2 = (_lib.RaggedGroup * 1)(_lib.RaggedGroup(1, 1.0, 1, C.cast(neg, C.POINTER(_lib.RaggedOption))))
    assert lib.wt_ragged_plan(grp2, 1, 152, out) == _lib.WT_ERR_INVALID


def _ragged_plan_restated(groups, n_sm):
    """wt_ragged_plan's rule as its header states it, in double precision:
    least SM-time per group (ties: fewer CTAs, then the earlier option); then,
    while the longest group outlasts total SM-time / n_sm, move it to the
    faster option of least SM-time (ties: the slower)."""
    t = lambda g, k: groups[g][2][k][1] * groups[g][1]          # noqa: E731
    sms = lambda g, k: float(groups[g][2][k][0])                # noqa: E731
    pick = []
    for g in range(len(groups)):
        best = 0
        for k in range(1, len(groups[g][2])):
            if (sms(g, k) * t(g, k), sms(g, k)) < (sms(g, best) * t(g, best), sms(g, best)):
                best = k
        pick.append(best)
    for _ in range(4 * len(groups) + 1):
        if not groups:
            break
        bound = 0.0
        for g in range(len(groups)):
            bound += groups[g][0] * sms(g, pick[g]) * t(g, pick[g])
        bound /= n_sm
        kg = 0
        for g in range(1, len(groups)):
            if t(g, pick[g]) > t(kg, pick[kg]):
                kg = g
        tk = t(kg, pick[kg])
        if tk <= bound:
            break
        cand = [k for k in range(len(groups[kg][2])) if t(kg, k) < tk]
        if not cand:
            break
        best = cand[0]
        for k in cand[1:]:
            if (sms(kg, k) * t(kg, k), -t(kg, k)) < (sms(kg, best) * t(kg, best), -t(kg, best)):
                best = k
        pick[kg] = best
    return pick


def test_ragged_plan_matches_its_stated_rule(lib):
    """wt_ragged_plan against a restatement of its documented rule on 400
    random batches (1-20 groups, 1-6 options, tied times included)."""
    from wavetorch_gb300 import _lib
    rng = np.random.default_rng(3)
    for _ in range(400):
        groups = []
        for _ in range(int(rng.integers(1, 21))):
            opts = [(int(rng.choice([1, 2, 4, 8, 12, 16])),
                     float(rng.choice([0.5, 1.0, 2.0])) if rng.random() < 0.3
                     else float(rng.uniform(0.01, 3.0)))
                    for _ in range(int(rng.integers(1, 7)))]
            groups.append((int(rng.integers(1, 31)), float(rng.uniform(0.5, 8.0)), opts))
        n_sm = int(rng.choice([8, 152]))
        arrs = [(_lib.RaggedOption * len(o))(*[_lib.RaggedOption(c, c, s) for c, s in o])
                for _, _, o in groups]
        grp = (_lib.RaggedGroup * len(groups))(*[
            _lib.RaggedGroup(n, sc, len(o), C.cast(a, C.POINTER(_lib.RaggedOption)))
            for (n, sc, o), a in zip(groups, arrs)])
        out = (C.c_int32 * len(groups))()
        assert lib.wt_ragged_plan(grp, len(groups), n_sm, out) == _lib.WT_OK
        assert list(out) == _ragged_plan_restated(groups, n_sm)


def _ragged_models(sizes, steps, in_row=-1):
    from wavetorch_gb300 import _lib
    keep, arr = [], (_lib.RaggedModel * len(sizes))()
    for i, (N, T) in enumerate(zip(sizes, steps)):
        src = (_lib.SourceEntry * 1)(_lib.SourceEntry(20 * N + N // 2, in_row))
        prb = (_lib.ProbeEntry * 3)(*[_lib.ProbeEntry((N - 20) * N + N // 2 + d, 1, k)
                                      for k, d in enumerate((-15, 0, 15))])
        keep += [src, prb]
        arr[i] = _lib.RaggedModel(N, N, T, 1, C.cast(src, C.POINTER(_lib.SourceEntry)), 3,
                                  C.cast(prb, C.POINTER(_lib.ProbeEntry)),
                                  *([C.c_void_p(256)] * 6))
    return arr, keep


def test_ragged_workspace_query(lib):
    """The packed ragged plan on the host (an SM count given, so no device is
    needed): its workspace holds every model's Laplacian tape (steps x bands
    x 1024 threads x strip cells), so it grows with the steps; strips of 4
    cut the larger grids into more bands than strips of 8; bad requests are
    refused before any device work."""
    from wavetorch_gb300 import _lib
    sc = _lib.Scalars(0.707, 1.0, 0)
    arr, keep = _ragged_models([64, 100, 256], [100, 200, 300])
    n4, n8 = C.c_size_t(0), C.c_size_t(0)
    assert lib.wt_ragged_workspace_bytes(C.byref(sc), arr, 3, 152, 4, C.byref(n4)) == _lib.WT_OK
    assert lib.wt_ragged_workspace_bytes(C.byref(sc), arr, 3, 152, 0, C.byref(n8)) == _lib.WT_OK
    assert n4.value > 4 * 1024 * (100 + 200 + 300) and n8.value > 0
    longer, keep2 = _ragged_models([64, 100, 256], [200, 400, 600])
    n = C.c_size_t(0)
    assert lib.wt_ragged_workspace_bytes(C.byref(sc), longer, 3, 152, 4, C.byref(n)) == _lib.WT_OK
    assert n.value > n4.value
    bad, keep3 = _ragged_models([64], [100], in_row=0)
    assert lib.wt_ragged_workspace_bytes(C.byref(sc), bad, 1, 152, 0, C.byref(n)) == \
        _lib.WT_ERR_UNSUPPORTED
    assert lib.wt_ragged_workspace_bytes(C.byref(sc), arr, 3, 152, 5, C.byref(n)) == \
        _lib.WT_ERR_INVALID
    assert lib.wt_ragged_workspace_bytes(C.byref(sc), arr, 0, 152, 0, C.byref(n)) == \
        _lib.WT_ERR_INVALID
    # a model wider than 1024 columns: no band layout serves it
    wide, keep4 = _ragged_models([1100], [10])
    assert lib.wt_ragged_workspace_bytes(C.byref(sc), wide, 1, 152, 0, C.byref(n)) == \
        _lib.WT_ERR_UNSUPPORTED
