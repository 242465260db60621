"""Ragged batches: many single-instance wave models of different grid sizes
and step counts, advanced together.

The reference trains one ``WaveRNN`` at a time; a user with many models (a
sweep over grid sizes, an ensemble) runs them one after another.

Packed form (the default): every model's forward runs in ONE persistent,
cooperative launch and every adjoint in ONE more (``wt_ragged_fwd`` /
``wt_ragged_bwd``, include/wavetorch_gb300.h section 5).  Each model is cut
into bands of rows; one CTA per SM walks a list of (model, band) items in a
global order the host's schedule fixes, each item that band's whole time
loop, so a model runs its own step count with no padding.  A small
autotuner times the strip heights the models' shared memory admits (4 or 8
cells per thread) on a short horizon and keeps the faster.

Grouped form (``packed=False``): models grouped by grid size and
source/probe layout; a group runs as one fused sequence launch with one
geometry per instance (``coef_batched``), its shorter inputs zero-padded to
the group's longest step count and the loss masked to each instance's own
steps; every group runs on its own stream, and the layout of each group
(clusters of 1-16 CTAs per instance, or bands) is autotuned by SM-time.

In both, one training step (rho -> c for every model, the forwards, the
losses and their gradients, the adjoints, c -> rho) is captured once into a
CUDA graph and replayed.  Loss per model: ``CrossEntropy(normalize_power(
sum_t I), label)``, the reference's training loss (wavetorch/train.py:61-62,
utils.py:35-36); its gradient with respect to the probe series is formed in
closed form.
"""
from __future__ import annotations

import ctypes as C
import time
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Sequence

import torch

from . import _lib
from .functional import (SeqSpec, _ptr, _stream, fused_supported, lap_order, scalars,
                         seq_backward, seq_forward, seq_workspace_bytes)
from .geom import WaveGeometryFreeForm
from .probe import WaveProbe
from .source import WaveSource

# measured seconds per layout option, per (grid, source/probe layout)
_TUNED: Dict[tuple, Dict[tuple, float]] = {}


@dataclass
class _Group:
    key: tuple
    idx: List[int]
    N: int
    T: int
    spec: SeqSpec
    sc: _lib.Scalars
    b: torch.Tensor                 # [G, N, N]
    c: torch.Tensor                 # [G, N, N] (rho -> c writes each slice)
    x: torch.Tensor                 # [G, T] zero-padded inputs
    mask: torch.Tensor              # [G, T, 1] 1 for t < T_i
    labels: torch.Tensor            # [G]
    onehot: torch.Tensor            # [G, P]
    work: List[torch.Tensor] = field(default_factory=list)   # rho -> c scratch per instance
    stream: Optional[torch.cuda.Stream] = None
    ws: Optional[torch.Tensor] = None   # the sequence workspace of the last step


def _option_spec(opt: tuple, G: int) -> tuple:
    """(cluster, sm_count) of a layout option for a group of G instances:
    (c, 0) a cluster of c CTAs per instance; (-1, p) bands, at most p CTAs
    per instance."""
    cl, per = opt
    return (cl, 0) if cl > 0 else (-1, per * G)


def _option_sms(opt) -> int:
    """SMs one instance occupies under a layout option (a cluster size, or
    a (cluster, bands) pair as `_option_spec` takes)."""
    if isinstance(opt, tuple):
        return opt[0] if opt[0] > 0 else opt[1]
    return opt


def pick_cluster_sizes(timings: Sequence[tuple], n_sm: int) -> List:
    """Layout option per group from measured times (the library's
    wt_ragged_plan).

    timings: per group (times, scale, G): times maps a layout option (a
    cluster size, or a (cluster, bands) pair) -> seconds of the group's
    measured run (its G instances side by side), scale the factor to the
    group's full step count.  An option using c SMs per instance occupies
    G x c SMs for the group's time.  The choice minimises SM-time unless the
    group alone would outlast the batch (see wt_ragged_plan)."""
    keep, groups, order = [], [], []
    for times, scale, G in timings:
        opts = sorted(times, key=lambda o: (_option_sms(o), str(o)))
        arr = (_lib.RaggedOption * len(opts))(*[
            _lib.RaggedOption(o[0] if isinstance(o, tuple) else int(o), _option_sms(o),
                              float(times[o])) for o in opts])
        keep.append(arr)
        order.append(opts)
        groups.append(_lib.RaggedGroup(int(G), float(scale), len(opts),
                                       C.cast(arr, C.POINTER(_lib.RaggedOption))))
    n = len(groups)
    garr = (_lib.RaggedGroup * max(n, 1))(*groups)
    choice = (C.c_int32 * max(n, 1))()
    _lib.check(_lib.load().wt_ragged_plan(garr, n, int(n_sm), choice), "wt_ragged_plan")
    return [order[g][choice[g]] for g in range(n)]


def _check_model(m) -> None:
    if not isinstance(m.cell.geom, WaveGeometryFreeForm):
        raise TypeError("ragged batches need WaveGeometryFreeForm geometries")
    if not m.cell.is_linear():
        raise TypeError("ragged batches need linear cells (no saturable damping or Kerr term)")
    if not all(isinstance(s, WaveSource) for s in m.sources) or \
            not all(isinstance(p, WaveProbe) for p in m.probes):
        raise TypeError("ragged batches need point sources and probes")


def trial_steps(T, steps: int):
    """Step counts of the strip-height trial: every model's count scaled by
    one factor (rounded up, at least 1, at most its own) so that the longest
    runs `steps`; the models keep their ratios and so the schedule its shape."""
    top = max(T)
    return [max(1, min(t, -(-t * steps // top))) for t in T]


class RaggedBatch:
    """One training step over many models.

    models: single-instance ``WaveRNN`` models (FreeForm geometry, linear
    cell, point sources and probes), on one CUDA device.
    inputs: one 1-D float32 input series per model (lengths may differ).
    labels: one class index per model.

    ``step()`` runs rho -> c, the forwards, the losses and the adjoints of all
    models and leaves each model's ``cell.geom.rho.grad`` (overwritten, not
    accumulated) and returns the per-model losses [n_models].
    """

    def __init__(self, models: Sequence, inputs: Sequence[torch.Tensor], labels, *,
                 autotune: bool = True, graph: bool = True, segment: int = 0,
                 packed: bool = True, strip: int = 0):
        if not (len(models) == len(inputs) == len(labels)) or not models:
            raise ValueError("models, inputs and labels must be non-empty and of equal length")
        self.models = list(models)
        dev = self.models[0].cell.geom.rho.device
        if dev.type != "cuda":
            raise RuntimeError("ragged batches run on CUDA devices only")
        self.device = dev
        for m in self.models:
            _check_model(m)
        self.T = [int(v.numel()) for v in inputs]
        self.n = len(self.models)
        self.packed = packed
        self.groups: List[_Group] = []
        self.losses: Optional[torch.Tensor] = None
        self.graph: Optional[torch.cuda.CUDAGraph] = None
        if packed:
            self._init_packed(inputs, labels, autotune, strip)
            for m in self.models:
                m.cell.geom.rho.grad = torch.zeros_like(m.cell.geom.rho)
            if graph:
                self._capture()
            return
        # group by grid, physics scalars and source/probe layout
        keys = {}
        for i, m in enumerate(self.models):
            nx, ny = m.cell.geom.domain_shape
            if nx != ny:
                raise ValueError("ragged batches take square grids")
            dt, h = m.cell.scalars()[:2]
            ptab, L = m.probe_table()
            if L != 1:
                raise ValueError("ragged batches take single-cell probes")
            key = (nx, dt, h, tuple(m.source_table(1)), tuple(ptab), tuple(m.cell.geom.b.shape))
            keys.setdefault(key, []).append(i)
        for key, idx in sorted(keys.items(), key=lambda kv: -kv[0][0]):
            N, dt, h, src, prb = key[0], key[1], key[2], list(key[3]), list(key[4])
            G, T = len(idx), max(self.T[i] for i in idx)
            x = torch.zeros(G, T, device=dev)
            mask = torch.zeros(G, T, 1, device=dev)
            for j, i in enumerate(idx):
                x[j, :self.T[i]] = inputs[i].to(dev, torch.float32).reshape(-1)
                mask[j, :self.T[i]] = 1.0
            b = torch.stack([self.models[i].cell.geom.b for i in idx]).contiguous()
            spec = SeqSpec(G, N, N, T, src, prb, form=_lib.WT_FORM_FUSED, segment=segment,
                           coef_batched=True)
            if not fused_supported(spec):
                raise ValueError(f"the fused form does not plan a {N}x{N} grid")
            # each model is an instance of its own: the Laplacian order of a batch of one
            sc = scalars(dt, h, lap_order(1, N, N, h))
            lab = torch.as_tensor([int(labels[i]) for i in idx], device=dev)
            onehot = torch.nn.functional.one_hot(lab, len(prb)).to(torch.float32)
            grp = _Group(key, idx, N, T, spec, sc, b, torch.empty(G, N, N, device=dev), x, mask,
                         lab, onehot)
            nwork = C.c_size_t(0)
            for i in idx:
                gd = self.models[i].cell.geom.geom_desc()
                _lib.check(_lib.load().wt_rho_to_c_work_bytes(C.byref(gd), C.byref(nwork)),
                           "wt_rho_to_c_work_bytes")
                grp.work.append(torch.empty(nwork.value // 4, device=dev))
            grp.stream = torch.cuda.Stream(device=dev)
            self.groups.append(grp)
        if segment == 0:
            self._fit_memory()
        for m in self.models:
            m.cell.geom.rho.grad = torch.zeros_like(m.cell.geom.rho)
        if autotune:
            self._autotune()
        if graph:
            self._capture()

    # -- packed form ----------------------------------------------------------
    def _packed_models(self, steps, x, out, gout, gc):
        """The C-ABI descriptors of every model (host arrays kept alive)."""
        keep, arr = [], (_lib.RaggedModel * self.n)()
        for i, m in enumerate(self.models):
            nx, ny = m.cell.geom.domain_shape
            src = m.source_table(1)
            prb, _ = m.probe_table()
            sa = (_lib.SourceEntry * max(1, len(src)))(*[_lib.SourceEntry(c, r) for c, r in src])
            pa = (_lib.ProbeEntry * max(1, len(prb)))(*[_lib.ProbeEntry(c, k, o) for c, k, o in prb])
            keep += [sa, pa]
            arr[i] = _lib.RaggedModel(nx, ny, steps[i], len(src), C.cast(sa, C.POINTER(_lib.SourceEntry)),
                                      len(prb), C.cast(pa, C.POINTER(_lib.ProbeEntry)),
                                      _ptr(self._b[i]), _ptr(self._c[i]), _ptr(x[i]), _ptr(out[i]),
                                      _ptr(gout[i]), _ptr(gc[i]))
        return arr, keep

    def _prepare(self, steps, x, out, gout, gc, strip):
        """Workspace and plan of a packed run over the given buffers."""
        lib = _lib.load()
        arr, keep = self._packed_models(steps, x, out, gout, gc)
        n = C.c_size_t(0)
        _lib.check(lib.wt_ragged_workspace_bytes(C.byref(self._sc), arr, self.n, 0, strip,
                                                 C.byref(n)), "wt_ragged_workspace_bytes")
        ws = torch.empty(n.value, dtype=torch.uint8, device=self.device)
        plan = _lib.RaggedPlan()
        _lib.check(lib.wt_ragged_prepare(C.byref(self._sc), arr, self.n, 0, strip, _ptr(ws),
                                         n.value, C.byref(plan)), "wt_ragged_prepare")
        return ws, plan

    def _init_packed(self, inputs, labels, autotune: bool, strip: int) -> None:
        dev = self.device
        scal = {m.cell.scalars()[:2] for m in self.models}
        if len(scal) != 1:
            raise ValueError("a packed ragged batch needs one dt and one h for all models")
        dt, h = scal.pop()
        self._sc = scalars(dt, h, _lib.WT_LAP_SEQ)     # each model's order is planned per model
        nprb = set()
        for m in self.models:
            ptab, L = m.probe_table()
            if L != 1:
                raise ValueError("ragged batches take single-cell probes")
            nprb.add(len(ptab))
            if any(r != -1 for _, r in m.source_table(1)):
                raise ValueError("ragged batches take sources driven by the model's own input")
        if len(nprb) != 1 or 0 in nprb:
            raise ValueError("a packed ragged batch needs the same number of probes in every model")
        P = nprb.pop()
        self._P = P
        self._b = [m.cell.geom.b.contiguous() for m in self.models]
        self._c = [torch.empty_like(b) for b in self._b]
        self._x = [inputs[i].to(dev, torch.float32).reshape(-1).contiguous() for i in range(self.n)]
        rows = sum(self.T)
        self._out = torch.empty(rows, P, device=dev)
        self._gout = torch.empty(rows, P, device=dev)
        offs = [0]
        for t in self.T:
            offs.append(offs[-1] + t)
        self._outs = [self._out[offs[i]:offs[i + 1]] for i in range(self.n)]
        self._gouts = [self._gout[offs[i]:offs[i + 1]] for i in range(self.n)]
        self._gc = [torch.empty_like(b) for b in self._b]
        self._seg = torch.repeat_interleave(torch.arange(self.n, device=dev),
                                            torch.as_tensor(self.T, device=dev))
        self._labels = torch.as_tensor([int(v) for v in labels], device=dev)
        self._onehot = torch.nn.functional.one_hot(self._labels, P).to(torch.float32)
        nwork = C.c_size_t(0)
        self._work = []
        for m in self.models:
            gd = m.cell.geom.geom_desc()
            _lib.check(_lib.load().wt_rho_to_c_work_bytes(C.byref(gd), C.byref(nwork)),
                       "wt_rho_to_c_work_bytes")
            self._work.append(torch.empty(nwork.value // 4, device=dev))
        self.strip = strip or (self._tune_strip() if autotune else 0)
        self._ws, self._plan = self._prepare(self.T, self._x, self._outs, self._gouts, self._gc,
                                             self.strip)
        self.strip = self._plan.strip

    def _tune_strip(self, steps: int = 256) -> int:
        """The strip height (4 or 8 cells per thread) of the faster forward +
        adjoint on the first steps of every model, each model's count scaled
        by one factor so that the longest runs `steps` (the schedule keeps
        its shape: equal counts would balance the CTAs differently); the one
        that fits when only one does, 0 when neither does."""
        dev = self.device
        T = trial_steps(self.T, steps)
        x = [v[:t].contiguous() for v, t in zip(self._x, T)]
        out = [torch.zeros(t, self._P, device=dev) for t in T]
        gout = [torch.ones(t, self._P, device=dev) for t in T]
        gc = [torch.empty_like(b) for b in self._b]
        for i in range(self.n):
            self._c[i].fill_(0.75)
        best, best_t = 0, None
        for strip in (8, 4):
            try:
                ws, plan = self._prepare(T, x, out, gout, gc, strip)
            except _lib.WaveKernelError:
                continue
            st = _stream(dev)
            ts = []
            for r in range(3):
                torch.cuda.synchronize(dev)
                t0 = time.perf_counter()
                _lib.check(_lib.load().wt_ragged_fwd(C.byref(plan), _ptr(ws), st), "wt_ragged_fwd")
                _lib.check(_lib.load().wt_ragged_bwd(C.byref(plan), _ptr(ws), st), "wt_ragged_bwd")
                torch.cuda.synchronize(dev)
                if r:
                    ts.append(time.perf_counter() - t0)
            del ws
            if best_t is None or min(ts) < best_t:
                best, best_t = strip, min(ts)
        self.tuned = {"strip": best, "seconds": best_t, "steps": steps}
        return best

    def _run_packed(self) -> torch.Tensor:
        lib = _lib.load()
        st = _stream(self.device)
        for i, m in enumerate(self.models):                     # rho -> c
            geom = m.cell.geom
            _lib.check(lib.wt_rho_to_c_fwd(C.byref(geom.geom_desc()), _ptr(geom.rho),
                                           _ptr(geom.blur_kernel[0, 0]), _ptr(self._c[i]),
                                           _ptr(self._work[i]), st), "wt_rho_to_c_fwd")
        _lib.check(lib.wt_ragged_fwd(C.byref(self._plan), _ptr(self._ws), st), "wt_ragged_fwd")
        # loss = CE(normalize_power(sum over each model's own steps))
        I = torch.zeros(self.n, self._P, device=self.device).index_add_(0, self._seg, self._out)
        S = I.sum(dim=1, keepdim=True)
        p = I / S
        loss = -torch.log_softmax(p, dim=1).gather(1, self._labels[:, None])[:, 0]
        dp = torch.softmax(p, dim=1) - self._onehot
        dI = (dp - (dp * p).sum(dim=1, keepdim=True)) / S          # dloss/dI per model
        self._gout.copy_(dI.index_select(0, self._seg))
        _lib.check(lib.wt_ragged_bwd(C.byref(self._plan), _ptr(self._ws), st), "wt_ragged_bwd")
        for i, m in enumerate(self.models):                     # c -> rho
            geom = m.cell.geom
            _lib.check(lib.wt_rho_to_c_bwd(C.byref(geom.geom_desc()), _ptr(geom.rho),
                                           _ptr(geom.blur_kernel[0, 0]), _ptr(self._gc[i]),
                                           _ptr(geom.rho.grad), _ptr(self._work[i]), st),
                       "wt_rho_to_c_bwd")
        return loss

    def _fit_memory(self, share: float = 0.6) -> None:
        """Groups whose tapes would take the workspaces past `share` of the
        device memory free now (largest first) use checkpoints instead
        (segment -2).  The graph keeps one workspace per group for its whole
        life, so the budget is what is free when the batch is built."""
        free, _ = torch.cuda.mem_get_info(self.device)
        sizes = [seq_workspace_bytes(g.spec) for g in self.groups]
        total = sum(sizes)
        for k in sorted(range(len(self.groups)), key=lambda k: -sizes[k]):
            if total <= share * free:
                break
            g = self.groups[k]
            g.spec.segment = -2
            new = seq_workspace_bytes(g.spec)
            total += new - sizes[k]

    def workspace_bytes(self) -> int:
        """Device bytes the sequence workspaces of one step take."""
        if self.packed:
            return int(self._plan.workspace_bytes)
        return sum(seq_workspace_bytes(g.spec) for g in self.groups)

    # -- one step, eagerly ------------------------------------------------
    def _run(self) -> torch.Tensor:
        lib = _lib.load()
        main = torch.cuda.current_stream(self.device)
        start = torch.cuda.Event()
        start.record(main)
        parts = [None] * self.n
        done = []
        for grp in self.groups:
            grp.stream.wait_event(start)
            with torch.cuda.stream(grp.stream):
                st = _stream(self.device)
                for j, i in enumerate(grp.idx):            # rho -> c into the group's stack
                    geom = self.models[i].cell.geom
                    _lib.check(lib.wt_rho_to_c_fwd(C.byref(geom.geom_desc()), _ptr(geom.rho),
                                                   _ptr(geom.blur_kernel[0, 0]), _ptr(grp.c[j]),
                                                   _ptr(grp.work[j]), st), "wt_rho_to_c_fwd")
                out, _, _, ws = seq_forward(grp.spec, grp.sc, grp.b, grp.c, grp.x)
                grp.ws = ws
                # loss = CE(normalize_power(sum over the instance's own steps))
                I = (out * grp.mask).sum(dim=1)                     # [G, P]
                S = I.sum(dim=1, keepdim=True)
                p = I / S
                lp = torch.log_softmax(p, dim=1)
                loss = -lp.gather(1, grp.labels[:, None])[:, 0]     # [G]
                dp = torch.softmax(p, dim=1) - grp.onehot
                dI = (dp - (dp * p).sum(dim=1, keepdim=True)) / S   # dloss/dI
                gout = (dI[:, None, :] * grp.mask).contiguous()     # dloss/d out, [G, T, P]
                gc, _ = seq_backward(grp.spec, grp.sc, grp.b, grp.c, grp.x, gout, ws, False)
                for j, i in enumerate(grp.idx):            # c -> rho
                    geom = self.models[i].cell.geom
                    _lib.check(lib.wt_rho_to_c_bwd(C.byref(geom.geom_desc()), _ptr(geom.rho),
                                                   _ptr(geom.blur_kernel[0, 0]), _ptr(gc[j]),
                                                   _ptr(geom.rho.grad), _ptr(grp.work[j]), st),
                               "wt_rho_to_c_bwd")
                for j, i in enumerate(grp.idx):
                    parts[i] = loss[j:j + 1]
                ev = torch.cuda.Event()
                ev.record(grp.stream)
                done.append(ev)
        for ev in done:
            main.wait_event(ev)
        return torch.cat(parts)

    def _capture(self) -> None:
        run = self._run_packed if self.packed else self._run
        side = torch.cuda.Stream(device=self.device)
        side.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(side):
            for _ in range(2):
                run()
        torch.cuda.current_stream(self.device).wait_stream(side)
        torch.cuda.synchronize(self.device)
        torch.cuda.empty_cache()   # the warm-up's workspaces: the graph gets its own pool
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph):
            self.losses = run()

    def device_status(self) -> int:
        """The sequence kernels' status words of the last step (synchronises):
        WT_OK, or WT_ERR_TIMEOUT when a bounded wait gave up."""
        from .functional import seq_device_status
        if self.packed:
            return int(_lib.load().wt_ragged_status(C.byref(self._plan), _ptr(self._ws),
                                                    _stream(self.device)))
        worst = _lib.WT_OK
        for grp in self.groups:
            if grp.ws is not None:
                st = seq_device_status(grp.spec, grp.ws)
                worst = st if st != _lib.WT_OK else worst
        return worst

    def step(self) -> torch.Tensor:
        """One training step of every model; returns the losses [n_models]."""
        if self.graph is not None:
            self.graph.replay()
            return self.losses
        return self._run_packed() if self.packed else self._run()

    # -- autotuner ----------------------------------------------------------
    def _autotune(self, steps: int = 96) -> None:
        """Pick each group's layout: a cluster of 1, 2, 4 or 8 CTAs per
        instance, or bands of rows (at most 8 or 12 CTAs per instance, any
        SMs); a 16-CTA cluster only where no band layout plans (clusters that
        large must each fit within one GPC, which limits how many run at
        once).  Every option is timed on a short forward + adjoint (cached per
        layout); the groups share the GPU's SMs, so the choice minimises
        SM-time (CTAs x time), except where a group alone would then outlast
        the whole batch."""
        for grp in self.groups:
            if grp.key not in _TUNED:
                _TUNED[grp.key] = self._time_options(grp, min(grp.T, steps))
        n_sm = torch.cuda.get_device_properties(self.device).multi_processor_count
        choice = pick_cluster_sizes(
            [(_TUNED[g.key], g.T / min(g.T, steps), len(g.idx)) for g in self.groups], n_sm)
        for grp, opt in zip(self.groups, choice):
            grp.spec.cluster, grp.spec.sm_count = _option_spec(opt, len(grp.idx))

    def _time_options(self, grp: _Group, T: int) -> Dict[tuple, float]:
        """Seconds of a T-step forward + adjoint of the group's instances per
        layout option (see `_option_spec`)."""
        out: Dict[tuple, float] = {}
        x = grp.x[:, :T].contiguous()
        g = torch.ones(len(grp.idx), T, len(grp.spec.probes), device=self.device)
        c = torch.ones_like(grp.c) * 0.75
        G = len(grp.idx)
        options = [(1, 0), (2, 0), (4, 0), (8, 0)]
        if grp.spec.segment in (0, -1):
            options += [(-1, 8), (-1, 12)]
        for opt in options + [(16, 0)]:
            if opt == (16, 0) and any(o[0] == -1 for o in out):
                continue
            cl, per = _option_spec(opt, G)
            spec = SeqSpec(G, grp.N, grp.N, T, grp.spec.sources, grp.spec.probes,
                           form=_lib.WT_FORM_FUSED, segment=grp.spec.segment, cluster=cl,
                           coef_batched=True, sm_count=per)
            if not fused_supported(spec):
                continue
            try:
                ts = []
                for r in range(3):
                    torch.cuda.synchronize(self.device)
                    t0 = time.perf_counter()
                    _, _, _, ws = seq_forward(spec, grp.sc, grp.b, c, x)
                    seq_backward(spec, grp.sc, grp.b, c, x, g, ws, False)
                    torch.cuda.synchronize(self.device)
                    if r:
                        ts.append(time.perf_counter() - t0)
            except _lib.WaveKernelError:
                continue
            out[opt] = min(ts)
        if not out:
            raise ValueError(f"no fused layout serves a {grp.N}x{grp.N} grid")
        return out

    def cell_steps(self) -> int:
        """Cell-steps of one training step (each model's N^2 x T_i)."""
        return sum(self.models[i].cell.geom.domain_shape[0] ** 2 * self.T[i] for i in range(self.n))
