#!/usr/bin/env python
"""Benchmark: one training step of the batched wave RNN on a GB300.

Workload (the reference's batched training configuration): batch 32 of
vowel-like waveforms (3 formants, 10 kHz, Hann envelope, peak 1), T = 3500
steps, 120 x 120 grid with a 20-cell PML (order 2, max 3.0), dt = 0.707,
c0 = 1, c1 = 0.5, free-form rho ~ U(0,1) with 1-cell blur and projection
(beta 100, eta 0.5), one point source at (20, 60), intensity probes at
(80, {35, 50, 65}), loss CE(normalize_power(sum_t I), label).

A step is rho -> c, the forward time loop, the loss, the hand-written adjoint
back to dL/drho.  Metric: cell-steps/s = batch * 120^2 * 3500 / step time
(the adjoint is not counted again).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints ONE JSON line (rank 0).
"""
from __future__ import annotations

import argparse
import contextlib
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = "cell-steps/s fwd+adjoint, fused vs plain per-step on GB300, grad rel err <=1e-5"
WORKLOAD = dict(workload="batched training step: B=32, 120x120 (PML 20), T=3500, linear, "
                         "fwd + hand-written adjoint to dL/drho",
                batch=32, nx=120, ny=120, steps=3500, abs_N=20)
BYTES_FWD = 12     # algorithmic bytes per forward cell-step (read y_t, y_{t-1}; write y_{t+1})
BYTES_ADJ = 20     # per adjoint cell-step (read lam_{t+1}, lam_{t+2}, h_{t-1}; write lam_t; + y)
L2_FLUSH_BYTES = 512 << 20


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--form", choices=["fused", "plain"], default="fused")
    p.add_argument("--no-plain", action="store_true", help="skip the plain-form comparison")
    p.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    p.add_argument("--no-workloads", action="store_true",
                   help="skip the compact pass over the other workloads after the headline")
    p.add_argument("--batch", type=int, default=WORKLOAD["batch"])
    p.add_argument("--T", type=int, default=WORKLOAD["steps"])
    p.add_argument("--kernels-only", action="store_true",
                   help="run only the sequence kernels (forward + adjoint) -- the profiling case")
    p.add_argument("--workload", choices=["batched", "ragged", "nonlinear", "lens", "fields", "holey"],
                   default="batched",
                   help="ragged: many models of different grid sizes / step counts in one graph; "
                        "nonlinear: B=64, 120x120, T=5000 with saturable damping and Kerr term; "
                        "lens: 1024x1024, T=8000; fields: the benchmark's forward with every "
                        "field written; holey: the benchmark's step through 16 holes")
    p.add_argument("--instances", type=int, default=256, help="models in the ragged workload")
    p.add_argument("--cluster", type=int, default=0,
                   help="--kernels-only: CTAs per instance (0: the planner's choice, -1: bands)")
    p.add_argument("--segment", type=int, default=0,
                   help="--kernels-only: adjoint mode (0 auto, -1 tape, >0 checkpoint interval)")
    return p.parse_args()


# ---------------------------------------------------------------------------
def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def max_over_ranks(v: float, world: int, device=None) -> float:
    """Largest value of v over all ranks (identity for one process)."""
    if world <= 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world: int, device=None):
    if world > 1:
        import torch.distributed as dist
        if device is not None and device.type == "cuda":
            dist.barrier(device_ids=[device.index])
        else:
            dist.barrier()


class ClockSampler:
    """SM clock and clock-event (throttle) reasons sampled while the timed
    region runs: every 2 ms through NVML (libnvidia-ml, which comes with the
    NVIDIA display driver; read-only queries), else from nvidia-smi at 100 ms.  The sampler is running before
    __enter__ returns, so the samples cover the region even when it lasts only
    a few tens of milliseconds."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    # nvmlClocksEventReasons bits reported (the rest: idle, application or
    # display clock settings, sync boost)
    NVML_REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown",
                    0x40: "hw_thermal_slowdown", 0x80: "hw_power_brake_slowdown"}
    PERIOD_S = 0.002

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []
        self.samples = []        # NVML: (sm MHz, reason bits)
        self.max_mhz = None
        self.source = None
        self._stop = threading.Event()
        self._thread = None

    def _nvml_handle(self):
        import ctypes
        nv = ctypes.CDLL("libnvidia-ml.so.1")
        if nv.nvmlInit_v2() != 0:
            raise OSError("nvmlInit failed")
        h = ctypes.c_void_p()
        ok = False
        try:
            import torch
            uuid = str(torch.cuda.get_device_properties(self.index).uuid)
            ok = nv.nvmlDeviceGetHandleByUUID(("GPU-" + uuid).encode(), ctypes.byref(h)) == 0
        except Exception:
            ok = False
        if not ok:
            vis = os.environ.get("CUDA_VISIBLE_DEVICES", "").split(",")
            idx = int(vis[self.index]) if vis[0].strip().isdigit() else self.index
            if nv.nvmlDeviceGetHandleByIndex_v2(idx, ctypes.byref(h)) != 0:
                raise OSError("no NVML handle for the device")
        get_reasons = getattr(nv, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            nv.nvmlDeviceGetCurrentClocksThrottleReasons
        mx = ctypes.c_uint()
        if nv.nvmlDeviceGetMaxClockInfo(h, 1, ctypes.byref(mx)) == 0:   # NVML_CLOCK_SM
            self.max_mhz = float(mx.value)
        return nv, h, get_reasons

    def _nvml_loop(self, nv, h, get_reasons):
        import ctypes
        clk, rs = ctypes.c_uint(), ctypes.c_ulonglong()
        while True:
            if nv.nvmlDeviceGetClockInfo(h, 1, ctypes.byref(clk)) == 0 and \
                    get_reasons(h, ctypes.byref(rs)) == 0:
                self.samples.append((float(clk.value), int(rs.value)))
            if self._stop.wait(self.PERIOD_S):
                return

    def __enter__(self):
        try:
            nv, h, get_reasons = self._nvml_handle()
            self.source = "nvml"
            self._thread = threading.Thread(target=self._nvml_loop, args=(nv, h, get_reasons),
                                            daemon=True)
            self._thread.start()
            t0 = time.perf_counter()
            while not self.samples and time.perf_counter() - t0 < 1.0:
                time.sleep(self.PERIOD_S)
            return self
        except (OSError, AttributeError, ValueError, IndexError):
            self.source = None
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.source = "nvidia-smi"
            threading.Thread(target=self._read, daemon=True).start()
            t0 = time.perf_counter()
            while not self.lines and time.perf_counter() - t0 < 3.0:
                time.sleep(0.01)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self._thread is not None:
            self._stop.set()
            self._thread.join(timeout=5)
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if self.samples:
            sm = [c for c, _ in self.samples]
            bits = 0
            for _, r in self.samples:
                bits |= r
            reasons = sorted(n for b, n in self.NVML_REASONS.items() if bits & b)
            return {"sm_mhz": statistics.median(sm), "sm_max_mhz": self.max_mhz or max(sm),
                    "reasons": reasons, "samples": len(sm), "source": "nvml, every 2 ms"}
        if not self.lines:
            return None
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm), "source": "nvidia-smi, every 100 ms"}


def measured_peaks():
    p = os.path.join(HERE, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def committed_traffic(kernel: str):
    """Per-launch DRAM bytes of `kernel` from the committed ncu summary
    (`profiles/traffic.txt`: `name bytes` lines, `#` comments)."""
    p = os.path.join(HERE, "profiles", "traffic.txt")
    if not os.path.exists(p):
        return None
    with open(p) as fh:
        for line in fh:
            f = line.split("#", 1)[0].split()
            if len(f) == 2 and f[0] == kernel:
                return int(f[1])
    return None


def committed_count(kernel: str, name: str = "instructions.txt"):
    """`kernel count` lines of a committed ncu summary under profiles/ (`#` comments)."""
    p = os.path.join(HERE, "profiles", name)
    if not os.path.exists(p):
        return None
    with open(p) as fh:
        for line in fh:
            f = line.split("#", 1)[0].split()
            if len(f) == 2 and f[0] == kernel:
                return float(f[1])
    return None


def device_peaks(dev):
    """FP32 FFMA issue rate and shared-memory load bandwidth of the device,
    measured by the library's wt_test_device_peaks (two kernels on every SM,
    CUDA events): the denominators of the fused kernels' roofline."""
    import ctypes as C
    import torch
    from wavetorch_gb300 import _lib

    class Peaks(C.Structure):
        _fields_ = [("ffma_per_s", C.c_double), ("warp_inst_per_s", C.c_double),
                    ("smem_bytes_per_s", C.c_double), ("sm_mhz", C.c_double),
                    ("sm_count", C.c_int32)]

    lib = _lib.load()
    nfn = lib.wt_test_device_peaks_scratch_floats
    nfn.argtypes, nfn.restype = [C.POINTER(C.c_size_t)], C.c_int
    fn = lib.wt_test_device_peaks
    fn.argtypes = [C.POINTER(Peaks), C.c_void_p, C.c_size_t, C.c_void_p]
    fn.restype = C.c_int
    n = C.c_size_t(0)
    _lib.check(nfn(C.byref(n)), "wt_test_device_peaks_scratch_floats")
    scratch = torch.empty(n.value, dtype=torch.float32, device=dev)
    pk = Peaks()
    _lib.check(fn(C.byref(pk), C.c_void_p(scratch.data_ptr()), n.value,
                  C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)), "wt_test_device_peaks")
    return {"ffma_per_s": pk.ffma_per_s, "warp_inst_per_s": pk.warp_inst_per_s,
            "smem_bytes_per_s": pk.smem_bytes_per_s, "sm_mhz": pk.sm_mhz, "sm_count": pk.sm_count}


# Algorithmic work of one cell-step in the fused kernels at h == 1 (the
# reference's float32 operations, unfused, in its order): forward 4 for the
# Laplacian + 6 for the update; adjoint 1 (c^2 g) + 4 (Laplacian) + 4 (grad_y1)
# + 1 (grad_y2) + 1 (lambda) + 1 (dL/dc sum).  Shared-memory bytes: each step a
# cell's new value is stored once and both horizontal neighbours loaded (12 B);
# the adjoint also lands its tape value in shared memory by bulk copy and reads
# it back (8 B).
FP32_FWD, FP32_ADJ = 10, 12
# steps of the workload the unmodified reference is timed on (its rate is flat in T)
REFERENCE_SAMPLE_T = 350
SMEM_FWD, SMEM_ADJ = 12, 20


# ---------------------------------------------------------------------------
def build_model(dev, B, T, seed, form):
    import numpy as np
    import torch
    import wavetorch_gb300 as wt
    from wavetorch_gb300.data import vowel_like
    N = WORKLOAD["nx"]
    rho = torch.rand(N, N, generator=torch.Generator().manual_seed(seed))
    geom = wt.WaveGeometryFreeForm((N, N), 1.0, c0=1.0, c1=0.5, abs_N=WORKLOAD["abs_N"],
                                   abs_sig=3.0, abs_p=2, eta=0.5, beta=100.0, rho=rho)
    cell = wt.WaveCell(0.707, geom)
    model = wt.WaveRNN(cell, wt.WaveSource(20, 60),
                       [wt.WaveIntensityProbe(80, y) for y in (35, 50, 65)], form=form).to(dev)
    x, labels = vowel_like(B, T, seed=seed)
    return model, np.ascontiguousarray(x), labels


def train_step(model, x, labels):
    import torch
    import wavetorch_gb300 as wt
    model.cell.geom.rho.grad = None
    y = model(x)
    loss = torch.nn.CrossEntropyLoss()(wt.utils.normalize_power(y.sum(dim=1)), labels)
    loss.backward()
    return loss


def run_ours(args):
    import numpy as np
    import torch
    import torch.distributed as dist
    from wavetorch_gb300 import _lib
    from wavetorch_gb300.functional import (SeqSpec, fused_uses_tape, lap_order, scalars,
                                            seq_backward, seq_forward)

    world, rank, local = dist_env()
    if world > 1:
        dist.init_process_group("nccl", init_method="env://")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    B, T, N = args.batch, args.T, WORKLOAD["nx"]
    cell_steps = B * N * N * T

    model, x_np, lab_np = build_model(dev, B, T, seed=1234 + rank, form=args.form)
    x = torch.from_numpy(x_np).to(dev)
    labels = torch.from_numpy(lab_np).to(dev)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)

    for _ in range(args.warmup):
        train_step(model, x, labels)
    torch.cuda.synchronize(dev)

    # ---- device-resident timed region: K steps, L2 flushed before each ----
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(args.steps)]
    launches0 = _lib.kernel_launches()
    barrier(world, dev)
    torch.cuda.synchronize(dev)
    with ClockSampler(local) as clk:
        for k in range(args.steps):
            flush.zero_()
            evs[k][0].record(stream)
            loss_t = train_step(model, x, labels)
            evs[k][1].record(stream)
        torch.cuda.synchronize(dev)
    loss_fused = float(loss_t.item())
    barrier(world, dev)
    launches = (_lib.kernel_launches() - launches0) // max(1, args.steps)
    t_step = sum(a.elapsed_time(b) for a, b in evs) / 1e3 / args.steps
    t_step = max_over_ranks(t_step, world, dev)
    value = world * cell_steps / t_step
    grad_fused = model.cell.geom.rho.grad.detach().clone()

    # ---- the same step with the loss fused into the sequence ----
    from wavetorch_gb300.losses import cross_entropy_normalize_power

    def fused_loss_step():
        model.cell.geom.rho.grad = None
        loss, _ = cross_entropy_normalize_power(model, x, labels)
        loss.backward()

    fused_loss = None
    if args.form == "fused":
        for _ in range(2):
            fused_loss_step()
        torch.cuda.synchronize(dev)
        tl = []
        for k in range(args.steps):
            flush.zero_()
            e = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
            e[0].record(stream)
            fused_loss_step()
            e[1].record(stream)
            torch.cuda.synchronize(dev)
            tl.append(e[0].elapsed_time(e[1]) / 1e3)
        t_fl = max_over_ranks(statistics.mean(tl), world, dev)
        g_fl = model.cell.geom.rho.grad.detach()
        fused_loss = {"value": world * cell_steps / t_fl, "ms_per_step": t_fl * 1e3,
                      "grad_rel_diff": float((g_fl - grad_fused).norm() / grad_fused.norm()),
                      "note": "wavetorch_gb300.losses.cross_entropy_normalize_power: the "
                              "reference's loss computed from the forward's probe sums"}

    # ---- end to end through the public API with host buffers ----
    x_host = torch.from_numpy(x_np).pin_memory()
    l_host = torch.from_numpy(lab_np).pin_memory()
    g_host = torch.empty((N, N), dtype=torch.float32).pin_memory()
    loss_host = torch.empty((), dtype=torch.float32).pin_memory()
    for _ in range(2):
        xd = x_host.to(dev, non_blocking=True)
        ld = l_host.to(dev, non_blocking=True)
        loss = train_step(model, xd, ld)
        g_host.copy_(model.cell.geom.rho.grad, non_blocking=True)
        loss_host.copy_(loss.detach(), non_blocking=True)
    barrier(world, dev)
    torch.cuda.synchronize(dev)
    e0 = time.perf_counter()
    for k in range(args.steps):
        xd = x_host.to(dev, non_blocking=True)
        ld = l_host.to(dev, non_blocking=True)
        loss = train_step(model, xd, ld)
        g_host.copy_(model.cell.geom.rho.grad, non_blocking=True)
        loss_host.copy_(loss.detach(), non_blocking=True)
        torch.cuda.synchronize(dev)
    t_e2e = (time.perf_counter() - e0) / args.steps
    t_e2e = max_over_ranks(t_e2e, world, dev)
    h2d = x_host.numel() * 4 + l_host.numel() * 8
    d2h = g_host.numel() * 4 + 4

    # ---- the kernels alone (roofline of the dominant kernel) ----
    geom = model.cell.geom
    with torch.no_grad():
        c = geom.c.contiguous()
    b = geom.b.contiguous()
    sc = scalars(0.707, 1.0, lap_order(B, N, N, 1.0))
    src = model.source_table(B)
    prb, _ = model.probe_table()
    form_id = _lib.WT_FORM_FUSED if args.form == "fused" else _lib.WT_FORM_PLAIN
    spec = SeqSpec(B, N, N, T, src, prb, form=form_id)
    gout = torch.randn(B, T, len(prb), generator=torch.Generator().manual_seed(3)).to(dev)
    kf, kb = [], []
    for k in range(args.warmup + args.steps):
        flush.zero_()
        e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        e[0].record(stream)
        out, _, _, ws = seq_forward(spec, sc, b, c, x)
        e[1].record(stream)
        seq_backward(spec, sc, b, c, x, gout, ws, False)
        e[2].record(stream)
        torch.cuda.synchronize(dev)
        if k >= args.warmup:
            kf.append(e[0].elapsed_time(e[1]) / 1e3)
            kb.append(e[1].elapsed_time(e[2]) / 1e3)
        del ws
    t_f, t_b = statistics.mean(kf), statistics.mean(kb)
    bwd_name = "seq_bwd_tape_kernel" if fused_uses_tape(spec) else "seq_bwd_fused_kernel"
    dom, t_dom, bpc = (bwd_name, t_b, BYTES_ADJ) if t_b >= t_f else \
        ("seq_fwd_fused_kernel", t_f, BYTES_FWD)
    if args.form == "plain":
        dom = "seq_adj_step_kernel" if t_b >= t_f else "step_fwd_kernel"
    peak, peak_src = measured_peaks()
    achieved = bpc * cell_steps / t_dom / 1e9
    traffic = committed_traffic(dom)

    # ---- the adjoint's two modes: the tape against sqrt(T) checkpoints ----
    adjoint_modes = None
    if args.form == "fused":
        from wavetorch_gb300.functional import seq_workspace_bytes
        seg = int(math.ceil(math.sqrt(T)))
        modes = {}
        for name, segment in (("tape", -1), ("checkpoint", seg)):
            mspec = SeqSpec(B, N, N, T, src, prb, form=form_id, segment=segment)
            tb_ = []
            for k in range(1 + max(2, min(args.steps, 3))):
                flush.zero_()
                _, _, _, ws = seq_forward(mspec, sc, b, c, x)
                e = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
                e[0].record(stream)
                seq_backward(mspec, sc, b, c, x, gout, ws, False)
                e[1].record(stream)
                torch.cuda.synchronize(dev)
                if k:
                    tb_.append(e[0].elapsed_time(e[1]))
                del ws
            modes[name] = {"adjoint_ms": statistics.mean(tb_),
                           "workspace_bytes": seq_workspace_bytes(mspec)}
        modes["checkpoint"]["segment"] = seg
        adjoint_modes = {**modes, "forward_ms": t_f * 1e3,
                         "checkpoint_over_tape_step": (t_f * 1e3 + modes["checkpoint"]["adjoint_ms"]) /
                                                      (t_f * 1e3 + modes["tape"]["adjoint_ms"]),
                         "note": "tape: every step's Laplacian kept in HBM; checkpoint: the pair "
                                 "(h_{t-1}, h_{t-2}) every ceil(sqrt(T)) steps, one thread group "
                                 "recomputing segment s-1 while a second runs the adjoint steps "
                                 "of segment s (two segments' Laplacians staged in HBM)"}
        torch.cuda.empty_cache()

    # ---- fused form: the on-chip resources that bound it ----
    fused_roofline = None
    if args.form == "fused":
        pk = device_peaks(dev)
        ipstep = committed_count(dom)            # warp instructions per time step (ncu)
        fp32 = (FP32_FWD * cell_steps / t_f, FP32_ADJ * cell_steps / t_b)
        smem = (SMEM_FWD * cell_steps / t_f, SMEM_ADJ * cell_steps / t_b)
        fused_roofline = {
            "device_peaks": pk,
            "fp32_fwd_frac": fp32[0] / pk["ffma_per_s"], "fp32_adj_frac": fp32[1] / pk["ffma_per_s"],
            "smem_fwd_frac": smem[0] / pk["smem_bytes_per_s"],
            "smem_adj_frac": smem[1] / pk["smem_bytes_per_s"],
            "issue_inst_per_step": ipstep,
            "note": "fp32: the reference's float32 operations per cell-step (forward 10, "
                    "adjoint 12 at h = 1) over the FFMA rate of all SMs; smem: 12 B (forward) "
                    "and 20 B (adjoint) of shared-memory traffic per cell-step over the "
                    "measured load bandwidth; issue: ncu-counted warp instructions per time "
                    "step of the launch (profiles/instructions.txt) over the FFMA loop's "
                    "issue rate"}
        if ipstep:
            inst_rate = ipstep * T / t_dom
            roofline = {"bound": "issue", "kernel": dom, "achieved": inst_rate / 1e9,
                        "peak": pk["warp_inst_per_s"] / 1e9, "unit": "Gwarp-inst/s",
                        "frac": inst_rate / pk["warp_inst_per_s"], "traffic": traffic,
                        "peak_source": "wt_test_device_peaks (FFMA-only loop on all SMs, "
                                       f"{pk['sm_mhz']:.0f} MHz), measured in this run"}
        else:
            roofline = {"bound": "fp32", "kernel": dom, "achieved": fp32[1] / 1e12,
                        "peak": pk["ffma_per_s"] / 1e12, "unit": "TFFMA/s",
                        "frac": fp32[1] / pk["ffma_per_s"], "traffic": traffic,
                        "peak_source": "wt_test_device_peaks, measured in this run"}
        roofline.update({"hbm_equivalent_frac": achieved / peak,
                         "hbm_equivalent_note": "the per-step form's HBM bytes (12 B fwd / 20 B "
                                                "adjoint per cell-step) over the fused kernel's "
                                                f"time, against hbm_gbs of {peak_src}",
                         "dram_frac": (traffic / t_dom / 1e9 / peak) if traffic else None,
                         "ms_fwd_kernel": t_f * 1e3, "ms_bwd_kernels": t_b * 1e3})
    else:
        roofline = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak,
                    "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
                    "peak_source": f"hbm_gbs of {peak_src}",
                    "algorithmic_bytes_per_cell_step": bpc,
                    "note": "per-step kernels: algorithmic bytes = HBM bytes per step",
                    "ms_fwd_kernel": t_f * 1e3, "ms_bwd_kernels": t_b * 1e3}

    # ---- plain per-step form: the metric's comparison arm ----
    plain = None
    if not args.no_plain and args.form == "fused":
        pm = model
        pm.form = "plain"
        train_step(pm, x, labels)
        torch.cuda.synchronize(dev)
        pe = []
        for k in range(max(2, min(args.steps, 3))):
            flush.zero_()
            a, z = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            train_step(pm, x, labels)
            z.record(stream)
            torch.cuda.synchronize(dev)
            pe.append(a.elapsed_time(z) / 1e3)
        grad_plain = pm.cell.geom.rho.grad.detach().clone()
        pm.form = "fused"
        t_plain = max_over_ranks(statistics.mean(pe), world, dev)
        g_rel = float(torch.linalg.norm((grad_fused - grad_plain).double()) /
                      torch.linalg.norm(grad_plain.double()))
        # the plain form's kernels without their launch cost: its forward and
        # adjoint sequences (3 launches per time step) replayed from a CUDA graph
        pspec = SeqSpec(B, N, N, T, src, prb, form=_lib.WT_FORM_PLAIN)
        side = torch.cuda.Stream(device=dev)
        side.wait_stream(stream)
        with torch.cuda.stream(side):
            _, _, _, pws = seq_forward(pspec, sc, b, c, x)
            seq_backward(pspec, sc, b, c, x, gout, pws, False)
            del pws
        stream.wait_stream(side)
        torch.cuda.synchronize(dev)
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph):
            _, _, _, pws = seq_forward(pspec, sc, b, c, x)
            seq_backward(pspec, sc, b, c, x, gout, pws, False)
        graph.replay()
        torch.cuda.synchronize(dev)
        pg = []
        for k in range(2):
            flush.zero_()
            a, z = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            graph.replay()
            z.record(stream)
            torch.cuda.synchronize(dev)
            pg.append(a.elapsed_time(z) / 1e3)
        del graph, pws
        torch.cuda.empty_cache()
        t_pgraph = max_over_ranks(statistics.mean(pg), world, dev)
        plain = {"value": world * cell_steps / t_plain, "ms_per_step": t_plain * 1e3,
                 "fused_over_plain": t_plain / t_step,
                 "grad_rel_err_fused_vs_plain": g_rel,
                 "kernels_graph_ms": t_pgraph * 1e3,
                 "fused_kernels_over_plain_kernels_graph": t_pgraph / (t_f + t_b),
                 "note": "plain = one kernel per step, every field kept; bit-exact with the "
                         "reference's float32 CPU path. Run as a user runs it, it is partly "
                         "bound by the host's launch rate (3 launches per time step); "
                         "kernels_graph_ms is its forward + adjoint kernels replayed from a "
                         "CUDA graph, compared with the fused kernels' own time"}

    cpu = None
    parity = parity_vs_reference(dev) if rank == 0 else None
    if rank == 0 and world == 1 and not args.no_cpu:
        full = oracle_workload(1234, B, T) if (B, T) == (WORKLOAD["batch"], WORKLOAD["steps"]) \
            else None
        cpu = cpu_baseline(sample_T=T, batch=B, res=full)
        if full is not None and args.form == "fused":
            parity["cfg1_full/fused"] = parity_full_size(dev, full, model, x, loss_fused, grad_fused)
        del full

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "cell-steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_step * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp32",
            "data": "synthetic (seeded vowel-like waveforms, random-init rho)",
            "config": {**WORKLOAD, "batch": B, "steps": T, "form": args.form,
                       "l2": "flushed (512 MiB write) before every timed step",
                       "parallelism": "replicas" if world > 1 else "single GPU"},
            "e2e": {"value": world * cell_steps / t_e2e, "unit": "cell-steps/s",
                    "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "ms_per_step": t_e2e * 1e3},
            "roofline": roofline,
            "fused_roofline": fused_roofline,
            "adjoint_modes": adjoint_modes,
            "cpu_baseline": cpu,
            "plain_form": plain,
            "fused_loss": fused_loss,
            "parity": parity,
            "clocks": clk.summary(),
            "gpu_launches": int(launches),
        }
        if world == 1 and args.form == "fused" and not args.no_workloads and \
                (B, T) == (WORKLOAD["batch"], WORKLOAD["steps"]):
            del model
            torch.cuda.empty_cache()
            line["workloads"] = other_workloads(args)
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def other_workloads(args):
    """The other workloads of this benchmark, each run once in compact form
    after the headline (3 warm-up and 2 timed steps each) so that their
    numbers come from the same run: the lens grid (band layout, tape and
    sqrt(T) checkpoints), the nonlinear cell, the ragged batch in one packed
    launch, field streaming and the hole geometry.  Each one's JSON line
    (what `--workload NAME` prints) goes under its name; a workload that fails
    records its error instead and the others still run."""
    import copy
    import io
    import torch
    out = {}
    for name, fn in (("lens", run_lens), ("nonlinear", run_nonlinear), ("ragged", run_ragged),
                     ("fields", run_fields), ("holey", run_holey)):
        a = copy.copy(args)
        a.workload, a.steps, a.warmup = name, 2, 3
        buf = io.StringIO()
        t0 = time.time()
        try:
            with contextlib.redirect_stdout(buf):
                fn(a)
            lines = [ln for ln in buf.getvalue().splitlines() if ln.startswith("{")]
            out[name] = json.loads(lines[-1]) if lines else {"error": "no result line"}
        except Exception as e:   # keep the headline and the other workloads
            out[name] = {"error": f"{type(e).__name__}: {e}"[:400]}
        out[name]["wall_s"] = round(time.time() - t0, 2)
        if torch.cuda.is_available():
            torch.cuda.synchronize()
            torch.cuda.empty_cache()
    return out


# ---------------------------------------------------------------------------
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tests", "golden")


def parity_vs_reference(dev):
    """Rel. L2 of our probe outputs, fields, loss and dL/drho against the reference's
    own results on the committed fixtures (made by running the reference in
    float32 and, for the configuration-0 case, float64): configuration-0
    physics (B=1, 100x100, T=200) and configuration-1 physics at a reduced
    size (B=4, 120x120, T=150), fused and plain forms."""
    import numpy as np
    import torch
    import wavetorch_gb300 as wt

    def rel(a, b):
        a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
        return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))

    res = {}
    for name in ("cfg0_small", "cfg1_small"):
        path = os.path.join(GOLDEN, name + ".npz")
        if not os.path.exists(path):
            continue
        d = np.load(path)
        N = int(d["N"])
        for form in ("fused", "plain"):
            geom = wt.WaveGeometryFreeForm((N, N), 1.0, c0=1.0, c1=0.5, abs_N=int(d["abs_N"]),
                                           abs_sig=3.0, abs_p=2, rho=torch.from_numpy(d["rho"]))
            srcs = [wt.WaveSource(int(cc) // N, int(cc) % N) for cc, _ in d["sources"]]
            prbs = [(wt.WaveIntensityProbe if k else wt.WaveProbe)(int(cc) // N, int(cc) % N)
                    for cc, k, _ in d["probes"]]
            m = wt.WaveRNN(wt.WaveCell(0.707, geom), srcs, prbs, form=form).to(dev)
            y = m(torch.from_numpy(d["x"]).to(dev))
            loss = torch.nn.CrossEntropyLoss()(wt.utils.normalize_power(y.sum(dim=1)),
                                               torch.from_numpy(d["labels"]).to(dev))
            loss.backward()
            out = y.detach().cpu().numpy()
            g = m.cell.geom.rho.grad.cpu().numpy()
            # field snapshots the fixture holds (steps named field_<t>)
            snaps = sorted(int(k.split("_")[1]) for k in d.files if k.startswith("field_"))
            with torch.no_grad():
                f = m(torch.from_numpy(d["x"]).to(dev), output_fields=True)
            f = np.stack([f[:, t].cpu().numpy() for t in snaps])
            f32 = np.stack([d[f"field_{t}"] for t in snaps])
            r = {"out_vs_ref_fp32": rel(out, d["out"]),
                 "fields_vs_ref_fp32": rel(f, f32),
                 "loss_vs_ref_fp32": rel(loss.item(), float(d["loss"])),
                 "grad_rho_vs_ref_fp32": rel(g, d["grad_rho"]),
                 "field_steps": snaps}
            if "out64" in d.files:
                f64 = np.stack([d[f"field64_{t}"] for t in snaps])
                r["out_vs_ref_fp64"] = rel(out, d["out64"])
                r["fields_vs_ref_fp64"] = rel(f, f64)
                r["grad_rho_vs_ref_fp64"] = rel(g, d["grad_rho64"])
                r["ref_fp32_out_vs_ref_fp64"] = rel(d["out"], d["out64"])
                r["ref_fp32_fields_vs_ref_fp64"] = rel(f32, f64)
                r["ref_fp32_grad_rho_vs_ref_fp64"] = rel(d["grad_rho"], d["grad_rho64"])
            res[f"{name}/{form}"] = r
    return res


def oracle_workload(seed: int, batch: int = WORKLOAD["batch"], T: int = WORKLOAD["steps"]):
    """The oracle port (plain C, OpenMP over all host threads) on the
    benchmark's training step with the inputs of `seed`: rho -> c, the
    forward, the loss and its gradient (torch on the CPU), the adjoint and
    dL/drho.  Returns the arrays and the forward + adjoint time."""
    import numpy as np
    import oracle.oracle as o
    import torch
    import wavetorch_gb300 as wt
    from wavetorch_gb300.data import vowel_like
    from wavetorch_gb300.geom import pml_profile
    N = WORKLOAD["nx"]
    b = pml_profile((N, N), WORKLOAD["abs_N"], 3.0, 2).numpy()
    rho = torch.rand(N, N, generator=torch.Generator().manual_seed(seed)).numpy()
    rho[b > 0] = 0
    kern = np.full((3, 3), np.float32(1.0) / np.float32(9.0), np.float32)
    c, th = o.rho_to_c(rho, kern, 1, 0.5, 100.0, 1.0, 0.5)
    x, labels = vowel_like(batch, T, seed=seed)
    S = o.Seq(batch, N, N, T, 0.707, 1.0, [(20 * N + 60, -1)],
              [(80 * N + y, 1, i) for i, y in enumerate((35, 50, 65))])
    t0 = time.perf_counter()
    out, hist = S.forward(b, c, x)
    t_f = time.perf_counter() - t0
    yo = torch.from_numpy(out).requires_grad_()
    loss = torch.nn.CrossEntropyLoss()(wt.utils.normalize_power(yo.sum(dim=1)),
                                       torch.from_numpy(labels))
    (g,) = torch.autograd.grad(loss, [yo])
    g = np.ascontiguousarray(g.numpy())
    t0 = time.perf_counter()
    gc, _ = S.backward(b, c, hist, g)
    t_b = time.perf_counter() - t0
    del hist
    grho = o.rho_to_c_bwd(th, kern, 1, 0.5, 100.0, 1.0, 0.5, gc)
    return {"b": b, "c": c, "x": x, "labels": labels, "out": out, "loss": float(loss.item()),
            "grad_out": g, "gc": gc, "grad_rho": grho, "seconds": t_f + t_b,
            "threads": o.num_threads()}


def cpu_baseline(sample_T: int, batch: int = WORKLOAD["batch"], res=None):
    """The oracle port on a bounded sample of the workload (the full batch
    and grid, the first sample_T steps): cell-steps/s of its forward +
    adjoint on all host threads."""
    N, T = WORKLOAD["nx"], sample_T
    r = res or oracle_workload(1234, batch, T)
    dt = r["seconds"]
    return {"value": batch * N * N * T / dt, "unit": "cell-steps/s", "cores": r["threads"],
            "kind": "port",
            "sample": f"batch {batch}, {N}x{N}, first {T} of {WORKLOAD['steps']} steps, "
                      f"fwd + adjoint, {dt:.2f} s"}


def parity_full_size(dev, r, model, x, loss_gpu: float, grad_rho_gpu):
    """The timed workload (B=32, 120x120, T=3500) against the oracle on the
    same inputs: the fused kernels on the oracle's c (probe outputs bit for
    bit, dL/dc) and the whole training step through WaveRNN (loss, dL/drho;
    c differs from the oracle's by ulps of tanh)."""
    import numpy as np
    import torch
    from wavetorch_gb300 import _lib
    from wavetorch_gb300.functional import SeqSpec, lap_order, scalars, seq_backward, seq_forward

    def rel(a, b_):
        a, b_ = np.asarray(a, np.float64), np.asarray(b_, np.float64)
        return float(np.linalg.norm(a - b_) / max(np.linalg.norm(b_), 1e-300))

    B, T = r["x"].shape
    N = WORKLOAD["nx"]
    spec = SeqSpec(B, N, N, T, model.source_table(B), model.probe_table()[0],
                   form=_lib.WT_FORM_FUSED)
    sc = scalars(0.707, 1.0, lap_order(B, N, N, 1.0))
    tb, tc = (torch.from_numpy(np.ascontiguousarray(v)).to(dev) for v in (r["b"], r["c"]))
    out, _, _, ws = seq_forward(spec, sc, tb, tc, x)
    gc, _ = seq_backward(spec, sc, tb, tc, x, torch.from_numpy(r["grad_out"]).to(dev), ws, False)
    torch.cuda.synchronize(dev)
    out = out.cpu().numpy()
    with torch.no_grad():
        c_gpu = model.cell.geom.c.cpu().numpy()
    return {"out_bit_exact": bool(np.array_equal(out, r["out"])), "out_rel": rel(out, r["out"]),
            "grad_c_rel": rel(gc.cpu().numpy(), r["gc"]),
            "c_rel": rel(c_gpu, r["c"]),
            "loss_rel": rel(loss_gpu, r["loss"]),
            "grad_rho_rel": rel(grad_rho_gpu.cpu().numpy(), r["grad_rho"]),
            "workload": f"B={B}, {N}x{N}, T={T}: the timed inputs, oracle on the host"}


def reference_cpu_path(batch: int, sample_T: int):
    """The unmodified reference (the pip install under baseline/_ref, imported
    through tests/golden/ref_shim.py's stand-ins for its plotting and data
    imports) on the benchmark's model: forward and autograd backward of the
    training loss on the CPU with all host threads, on the first sample_T
    steps of the workload.  None when the install is absent."""
    ref_root = os.path.join(HERE, "baseline", "_ref")
    if not os.path.isdir(os.path.join(ref_root, "wavetorch")):
        return None
    os.environ["WAVETORCH_REFERENCE"] = ref_root
    sys.path.insert(0, os.path.join(HERE, "tests", "golden"))
    import torch
    import ref_shim
    from wavetorch_gb300.data import vowel_like
    wt = ref_shim.import_reference()
    torch.set_num_threads(os.cpu_count() or 1)
    N = WORKLOAD["nx"]
    geom = wt.WaveGeometryFreeForm((N, N), 1.0, c0=1.0, c1=0.5, abs_N=WORKLOAD["abs_N"],
                                   abs_sig=3.0, abs_p=2,
                                   rho=torch.rand(N, N, generator=torch.Generator().manual_seed(1234)))
    model = wt.WaveRNN(wt.WaveCell(0.707, geom), [wt.WaveSource(20, 60)],
                       [wt.WaveIntensityProbe(80, y) for y in (35, 50, 65)])
    x, labels = vowel_like(batch, sample_T, seed=1234)
    xt, lt = torch.from_numpy(x), torch.from_numpy(labels)

    def step():
        geom.rho.grad = None
        y = model(xt)
        loss = torch.nn.CrossEntropyLoss()(wt.utils.normalize_power(y.sum(dim=1)), lt)
        loss.backward()

    step()                                 # warm-up
    t0 = time.perf_counter()
    step()
    dt = time.perf_counter() - t0
    return {"value": batch * N * N * sample_T / dt, "unit": "cell-steps/s",
            "cores": torch.get_num_threads(), "kind": "reference",
            "sample": f"batch {batch}, {N}x{N}, first {sample_T} of {WORKLOAD['steps']} steps, "
                      f"forward + autograd backward of the unmodified reference (torch "
                      f"{torch.__version__}, CPU), {dt:.2f} s"}


def run_reference(args):
    world, rank, _ = dist_env()
    if rank != 0:
        return
    import oracle.oracle as o
    o.build()
    B = args.batch
    sample_T = WORKLOAD["steps"]
    for _ in range(args.warmup):
        cpu_baseline(sample_T, B)
    vals = [cpu_baseline(sample_T, B) for _ in range(args.steps)]
    v = statistics.mean(r["value"] for r in vals)
    N = WORKLOAD["nx"]
    ms = B * N * N * args.T / v * 1e3
    line = {"metric": METRIC, "value": v, "unit": "cell-steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp32",
            "data": "synthetic (seeded vowel-like waveforms, random-init rho)",
            "config": {**WORKLOAD, "batch": B, "form": "reference CPU path (oracle port)"},
            "impl": "reference",
            "cpu_baseline": {"value": v, "unit": "cell-steps/s", "kind": "port",
                             "cores": vals[0]["cores"], "sample": vals[0]["sample"]},
            "cpu_baseline_reference": reference_cpu_path(B, REFERENCE_SAMPLE_T),
            "e2e": {"value": v, "unit": "cell-steps/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_kernels_only(args):
    """seq forward + adjoint on the workload shape, no training glue: the
    command the ncu captures run (small T keeps a capture short)."""
    import torch
    from wavetorch_gb300 import _lib
    from wavetorch_gb300.functional import SeqSpec, lap_order, scalars, seq_backward, seq_forward
    dev = torch.device("cuda", 0)
    B, T, N = args.batch, args.T, WORKLOAD["nx"]
    model, x_np, _ = build_model(dev, B, T, seed=1234, form=args.form)
    x = torch.from_numpy(x_np).to(dev)
    with torch.no_grad():
        c = model.cell.geom.c.contiguous()
    b = model.cell.geom.b.contiguous()
    prb, _ = model.probe_table()
    spec = SeqSpec(B, N, N, T, model.source_table(B), prb,
                   form=_lib.WT_FORM_FUSED if args.form == "fused" else _lib.WT_FORM_PLAIN,
                   cluster=args.cluster, segment=args.segment)
    sc = scalars(0.707, 1.0, lap_order(B, N, N, 1.0))
    g = torch.randn(B, T, len(prb), generator=torch.Generator().manual_seed(3)).to(dev)
    t = []
    for k in range(args.warmup + args.steps):
        e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        e[0].record()
        out, _, _, ws = seq_forward(spec, sc, b, c, x)
        e[1].record()
        seq_backward(spec, sc, b, c, x, g, ws, False)
        e[2].record()
        torch.cuda.synchronize()
        if k >= args.warmup:
            t.append((e[0].elapsed_time(e[1]), e[1].elapsed_time(e[2])))
    f = sum(a for a, _ in t) / len(t)
    bw = sum(b_ for _, b_ in t) / len(t)
    print(json.dumps({"kernels_only": True, "batch": B, "T": T, "form": args.form,
                      "cluster": args.cluster, "segment": args.segment, "ms_fwd": f, "ms_bwd": bw,
                      "cell_steps_per_s": B * N * N * T / ((f + bw) / 1e3)}))


def layout_counts(rb):
    """How many groups of a ragged batch run in each fused layout."""
    counts = {}
    for g in rb.groups:
        c = g.spec.cluster
        key = f"cluster {c}" if c > 0 else f"bands <= {g.spec.sm_count // len(g.idx)} per model"
        counts[key] = counts.get(key, 0) + 1
    return counts


def run_ragged(args):
    """Ragged workload: `instances` single-instance models, grid side
    U{64..256} (PML 20), step count U{500..4000}, the vowel-like generator
    with independent seeds, source (20, N/2), intensity probes (N-20,
    N/2 + {-15, 0, 15}); one training step of all models as one CUDA graph
    holding one forward and one adjoint launch for all models (packed form).
    Compared with the per-model loops a user of the reference would run:
    each model alone through WaveRNN, plain form and fused form, timed on a
    16-model subsample and scaled by cell-steps."""
    import numpy as np
    import torch
    import wavetorch_gb300 as wt
    from wavetorch_gb300.data import vowel_like
    from wavetorch_gb300.ragged import RaggedBatch
    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    rng = np.random.default_rng(4321 + rank)
    n = args.instances
    sizes = rng.integers(64, 257, n)
    steps = rng.integers(500, 4001, n)
    models, inputs, labels = [], [], []
    for i in range(n):
        N = int(sizes[i])
        geom = wt.WaveGeometryFreeForm((N, N), 1.0, c0=1.0, c1=0.5, abs_N=20, abs_sig=3.0, abs_p=2,
                                       rho=torch.rand(N, N, generator=torch.Generator().manual_seed(i)))
        models.append(wt.WaveRNN(wt.WaveCell(0.707, geom), wt.WaveSource(20, N // 2),
                                 [wt.WaveIntensityProbe(N - 20, N // 2 + d) for d in (-15, 0, 15)]
                                 ).to(dev))
        x, lab = vowel_like(1, int(steps[i]), seed=1000 + i)
        inputs.append(torch.from_numpy(x[0]).to(dev))
        labels.append(int(lab[0]))
    t0 = time.perf_counter()
    rb = RaggedBatch(models, inputs, labels)
    t_setup = time.perf_counter() - t0
    cell_steps = rb.cell_steps()
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)
    for _ in range(args.warmup):
        rb.step()
    torch.cuda.synchronize(dev)
    ts = []
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            flush.zero_()
            e = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
            e[0].record(stream)
            rb.step()
            e[1].record(stream)
            torch.cuda.synchronize(dev)
            ts.append(e[0].elapsed_time(e[1]) / 1e3)
    t_step = statistics.mean(ts)
    # per-model loops on a 16-model subsample
    sub = list(range(min(16, n)))
    sub_cells = sum(int(sizes[i]) ** 2 * int(steps[i]) for i in sub)
    loops = {}
    for form in ("plain", "fused"):
        tot = 0.0
        for i in sub:
            m = models[i]
            m.form = form
            lab = torch.tensor([labels[i]], device=dev)
            for r in range(2):
                torch.cuda.synchronize(dev)
                a = time.perf_counter()
                m.cell.geom.rho.grad = None
                y = m(inputs[i][None])
                loss = torch.nn.CrossEntropyLoss()(wt.utils.normalize_power(y.sum(dim=1)), lab)
                loss.backward()
                torch.cuda.synchronize(dev)
                if r:
                    tot += time.perf_counter() - a
        loops[form] = sub_cells / tot
    line = {
        "metric": "cell-steps/s fwd+adjoint, ragged batch of models in one CUDA graph",
        "value": cell_steps / t_step, "unit": "cell-steps/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_step * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "fp32",
        "data": "synthetic (seeded vowel-like waveforms, random-init rho)",
        "config": {"workload": f"ragged: {n} models, N ~ U{{64..256}} (PML 20), T ~ U{{500..4000}}, "
                               "fwd + adjoint to dL/drho per model",
                   "instances": n, "cell_steps": cell_steps,
                   "launch": ({"form": "packed: one cooperative forward launch and one adjoint "
                                       "launch over (model, band) work items",
                               "ctas": rb._plan.ctas, "strip": rb._plan.strip,
                               "work_items": rb._plan.n_items,
                               "autotune": getattr(rb, "tuned", None),
                               "workspace_GB": rb._plan.workspace_bytes / 1e9}
                              if rb.packed else
                              {"form": "grouped", "groups": len(rb.groups),
                               "layouts": layout_counts(rb)}),
                   "l2": "flushed (512 MiB write) before every timed step",
                   "setup_s": t_setup},
        "per_model_loop": {"plain_cell_steps_per_s": loops["plain"],
                           "fused_cell_steps_per_s": loops["fused"],
                           "ragged_over_plain_loop": (cell_steps / t_step) / loops["plain"],
                           "ragged_over_fused_loop": (cell_steps / t_step) / loops["fused"],
                           "sample": f"{len(sub)} models, {sub_cells} cell-steps, each alone "
                                     "through WaveRNN (forward, CE loss, backward)"},
        "clocks": clk.summary(),
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_nonlinear(args):
    """Nonlinear workload: B=64 vowel-like inputs (scaled by 0.2 so the Kerr
    term stays inside the CFL limit), 120x120 (PML 20), T=5000, intensity-
    dependent speed c^2 = (c_lin + 0.1 rho h^2)^2 and saturable damping
    b = b_pml + rho 0.05 / (1 + |h|^2/0.1), rho the free-form density;
    forward + adjoint to dL/drho, fused.  Compared with the per-step form
    (torch ops for b and c every step, autograd through them), timed on the
    first 200 steps (its tape would not fit at T=5000) and compared per
    cell-step."""
    import numpy as np
    import torch
    import wavetorch_gb300 as wt
    from wavetorch_gb300.data import vowel_like
    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    B, T, N = 64, 5000, 120

    def make(form, steps):
        rho0 = torch.rand(N, N, generator=torch.Generator().manual_seed(5 + rank))
        geom = wt.WaveGeometryFreeForm((N, N), 1.0, c0=1.0, c1=0.5, abs_N=20, abs_sig=3.0,
                                       abs_p=2, rho=rho0)
        cell = wt.WaveCell(0.707, geom, satdamp_b0=0.05, satdamp_uth=float(np.sqrt(0.1)),
                           c_nl=0.1)
        m = wt.WaveRNN(cell, wt.WaveSource(20, 60),
                       [wt.WaveIntensityProbe(80, y) for y in (35, 50, 65)], form=form).to(dev)
        x, lab = vowel_like(B, steps, seed=7 + rank)
        return m, torch.from_numpy(x * np.float32(0.2)).to(dev), torch.from_numpy(lab).to(dev)

    def timed(form, steps, reps, warm, clk=None):
        m, x, lab = make(form, steps)
        flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
        stream = torch.cuda.current_stream(dev)
        for _ in range(warm):
            train_step(m, x, lab)
        torch.cuda.synchronize(dev)
        ts = []
        with clk or contextlib.nullcontext():
            for _ in range(reps):
                flush.zero_()
                e = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
                e[0].record(stream)
                train_step(m, x, lab)
                e[1].record(stream)
                torch.cuda.synchronize(dev)
                ts.append(e[0].elapsed_time(e[1]) / 1e3)
        return statistics.mean(ts)

    clk = ClockSampler(local)
    t_fused = timed("fused", T, args.steps, args.warmup, clk)
    t_step = timed("step", 200, 2, 1)
    value = B * N * N * T / t_fused
    step_rate = B * N * N * 200 / t_step
    line = {
        "metric": "cell-steps/s fwd+adjoint, nonlinear cell (saturable damping + Kerr), fused",
        "value": value, "unit": "cell-steps/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_fused * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "fp32",
        "data": "synthetic (seeded vowel-like waveforms x 0.2, random-init rho)",
        "config": {"workload": "nonlinear training step: B=64, 120x120 (PML 20), T=5000, "
                               "c_nl 0.1, satdamp b0 0.05 uth sqrt(0.1), fwd + adjoint to dL/drho",
                   "l2": "flushed (512 MiB write) before every timed step"},
        "step_form": {"cell_steps_per_s": step_rate, "fused_over_step_form": value / step_rate,
                      "sample": "first 200 of 5000 steps (B=64, 120x120)"},
        "clocks": clk.summary(),
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_lens(args):
    """Large-grid lens design: 1024x1024 (PML 40), one instance, line source
    along x=60 from y=200 to 824 driven by sin(2 pi 0.02 t), T=8000, loss
    -sum_t I(900, 512), gradient w.r.t. a full-grid rho ~ U(0,1).  The fused
    form runs it in bands of 7 rows, one CTA per band and SM (the forward
    stores a 31 GiB Laplacian tape); the plain per-step form (every field
    kept: 33.5 GB) is timed beside it."""
    import numpy as np
    import torch
    import wavetorch_gb300 as wt
    from wavetorch_gb300.data import sinusoid
    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    N, T = 1024, args.T if args.T != WORKLOAD["steps"] else 8000
    x = torch.from_numpy(sinusoid(T, 0.02)).to(dev)          # [1, T]

    def make(form, segment=0):
        geom = wt.WaveGeometryFreeForm((N, N), 1.0, c0=1.0, c1=0.5, abs_N=40, abs_sig=3.0,
                                       abs_p=2,
                                       rho=torch.rand(N, N, generator=torch.Generator().manual_seed(3)))
        return wt.WaveRNN(wt.WaveCell(0.707, geom), wt.WaveLineSource(60, 200, 60, 824),
                          [wt.WaveIntensityProbe(900, 512)], form=form, segment=segment).to(dev)

    def timed(model, steps, warmup, clk=None):
        def step():
            model.cell.geom.rho.grad = None
            loss = -model(x).sum()
            loss.backward()
        for _ in range(warmup):
            step()
        torch.cuda.synchronize(dev)
        stream = torch.cuda.current_stream(dev)
        ts = []
        with clk or contextlib.nullcontext():
            for _ in range(steps):
                e = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
                e[0].record(stream)
                step()
                e[1].record(stream)
                torch.cuda.synchronize(dev)
                ts.append(e[0].elapsed_time(e[1]) / 1e3)
        return statistics.mean(ts), model.cell.geom.rho.grad.clone()

    fused = make("fused")
    clk = ClockSampler(local)
    t, g_fused = timed(fused, args.steps, args.warmup, clk)
    del fused
    torch.cuda.empty_cache()
    # the same step from sqrt(T) checkpoints (segment -2): each segment
    # recomputed by one launch, its adjoint steps run by the next
    from wavetorch_gb300.functional import SeqSpec, seq_workspace_bytes
    ck = make("fused", segment=-2)
    t_ck, g_ck = timed(ck, 1, 1)
    del ck
    torch.cuda.empty_cache()
    ws_spec = lambda seg: SeqSpec(1, N, N, T, [(60 * N + y, -1) for y in range(200, 825)],
                                  [(900 * N + 512, 1, 0)], segment=seg)
    t_plain, g_plain = timed(make("plain"), 1, 1) if not args.no_plain else (None, None)
    alg_bytes = (12 + 20) * N * N * T   # per-step form's algorithmic HBM bytes, fwd + adjoint
    line = {
        "metric": "cell-steps/s fwd+adjoint, 1024x1024 lens design (fused form, band layout)",
        "value": N * N * T / t, "unit": "cell-steps/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "fp32",
        "data": "synthetic (sinusoidal line source, random-init rho)",
        "config": {"workload": f"lens: 1024x1024 (PML 40), line source x=60 y=200..824, T={T}, "
                               "objective -sum_t I(900,512), fwd + adjoint to dL/drho",
                   "layout": "147 bands of 7 rows x 1024 columns, one CTA (1024 threads) per SM, "
                             "cooperative launch; Laplacian tape in HBM",
                   "l2": "inputs (tape 31 GiB) larger than L2"},
        "algorithmic_GBps": alg_bytes / t / 1e9,
        "tape_GBps": 8 * N * N * T / t / 1e9,
        "adjoint_modes": {"tape": {"ms_per_step": t * 1e3,
                                   "workspace_bytes": seq_workspace_bytes(ws_spec(-1))},
                          "checkpoint": {"ms_per_step": t_ck * 1e3,
                                         "workspace_bytes": seq_workspace_bytes(ws_spec(-2)),
                                         "segment": int(math.ceil(math.sqrt(T))),
                                         "grad_rel_diff_vs_tape":
                                             float((g_ck - g_fused).norm() / g_fused.norm())}},
        "clocks": clk.summary(),
    }
    if t_plain is not None:
        line["plain_form"] = {"ms_per_step": t_plain * 1e3, "cell_steps_per_s": N * N * T / t_plain,
                              "fused_over_plain": t_plain / t,
                              "grad_rel_diff_fused_vs_plain":
                                  float((g_fused - g_plain).norm() / g_plain.norm())}
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_fields(args):
    """Field streaming (WaveRNN.forward(x, output_fields=True), the reference's
    rnn.py:59-67): the benchmark's model and inputs (B=32, 120x120, T=3500),
    forward only, every field [B, T, 120, 120] written to HBM (6.45 GB).  The
    fused kernel writes each step's fields straight from registers; the plain
    form computes its field history and copies it out.  Both results are
    compared bit for bit."""
    import torch
    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    B, T, N = args.batch, args.T, WORKLOAD["nx"]
    field_bytes = 4 * B * T * N * N
    peak, peak_src = measured_peaks()
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)

    def timed(form, steps, warmup, clk=None):
        model, x_np, _ = build_model(dev, B, T, seed=1234, form=form)
        x = torch.from_numpy(x_np).to(dev)
        stream = torch.cuda.current_stream(dev)
        with torch.no_grad():
            for _ in range(warmup):
                model(x, output_fields=True)
            torch.cuda.synchronize(dev)
            ts = []
            with clk or contextlib.nullcontext():
                for _ in range(steps):
                    flush.zero_()
                    e = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
                    e[0].record(stream)
                    f = model(x, output_fields=True)
                    e[1].record(stream)
                    torch.cuda.synchronize(dev)
                    ts.append(e[0].elapsed_time(e[1]) / 1e3)
        return statistics.mean(ts), f

    clk = ClockSampler(local)
    t, f_fused = timed("fused", args.steps, args.warmup, clk)
    line = {
        "metric": "cell-steps/s forward with every field written (output_fields), fused form",
        "value": B * N * N * T / t, "unit": "cell-steps/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "fp32",
        "data": "synthetic (seeded vowel-like waveforms, random-init rho)",
        "config": {"workload": f"field streaming: B={B}, {N}x{N} (PML 20), T={T}, forward only, "
                               "fields [B, T, N, N] written to HBM",
                   "l2": "flushed (512 MiB write) before every timed step; output 6.45 GB"},
        "fields_GBps": field_bytes / t / 1e9,
        "fields_frac_of_hbm_peak": field_bytes / t / 1e9 / peak,
        "peak_source": f"hbm_gbs of {peak_src}",
        "clocks": clk.summary(),
    }
    if not args.no_plain:
        t_plain, f_plain = timed("plain", 1, 1)
        line["plain_form"] = {"ms_per_step": t_plain * 1e3,
                              "cell_steps_per_s": B * N * N * T / t_plain,
                              "fused_over_plain": t_plain / t,
                              "fields_bit_identical": bool(torch.equal(f_fused, f_plain))}
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_holey(args):
    """Training step through the hole geometry (wavetorch/geom.py:88-132): the
    benchmark's model and inputs (B=32, 120x120, T=3500) with c from 16 holes
    (seeded centres in the design region, radii 2..6) instead of the
    free-form density; the gradients reach the holes' centres and radii.
    Also times the geometry alone: rho and c from the holes and the adjoint
    back to (x, y, r)."""
    import numpy as np
    import torch
    import wavetorch_gb300 as wt
    from wavetorch_gb300.data import vowel_like
    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    B, T, N, nh = args.batch, args.T, WORKLOAD["nx"], 16
    rng = np.random.default_rng(7)
    hx, hy = (30.0 + 60.0 * rng.random(nh)).tolist(), (30.0 + 60.0 * rng.random(nh)).tolist()
    hr = (2.0 + 4.0 * rng.random(nh)).tolist()
    geom = wt.WaveGeometryHoley((N, N), 1.0, c0=1.0, c1=0.5, abs_N=WORKLOAD["abs_N"], abs_sig=3.0,
                                abs_p=2, x=hx, y=hy, r=hr)
    model = wt.WaveRNN(wt.WaveCell(0.707, geom), wt.WaveSource(20, 60),
                       [wt.WaveIntensityProbe(80, y) for y in (35, 50, 65)]).to(dev)
    x_np, lab = vowel_like(B, T, seed=1234)
    x = torch.from_numpy(np.ascontiguousarray(x_np)).to(dev)
    labels = torch.from_numpy(lab).to(dev)
    holes = [model.cell.geom.x, model.cell.geom.y, model.cell.geom.r]
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)

    def train():
        for p in holes:
            p.grad = None
        y = model(x)
        loss = torch.nn.CrossEntropyLoss()(wt.utils.normalize_power(y.sum(dim=1)), labels)
        loss.backward()

    w = torch.randn(N, N, generator=torch.Generator().manual_seed(8)).to(dev)

    def geometry():
        for p in holes:
            p.grad = None
        (model.cell.geom.c * w).sum().backward()

    def timed(fn, steps, warmup, flush_l2, clk=None):
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize(dev)
        ts = []
        with clk or contextlib.nullcontext():
            for _ in range(steps):
                if flush_l2:
                    flush.zero_()
                e = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
                e[0].record(stream)
                fn()
                e[1].record(stream)
                torch.cuda.synchronize(dev)
                ts.append(e[0].elapsed_time(e[1]) / 1e3)
        return statistics.mean(ts)

    clk = ClockSampler(local)
    t = timed(train, args.steps, args.warmup, True, clk)
    grads_finite = all(bool(torch.isfinite(p.grad).all()) for p in holes)
    t_geo = timed(geometry, 50, 5, False)
    line = {
        "metric": "cell-steps/s fwd+adjoint, hole geometry (16 holes), fused form",
        "value": B * N * N * T / t, "unit": "cell-steps/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "fp32",
        "data": "synthetic (seeded vowel-like waveforms, 16 seeded holes)",
        "config": {"workload": f"training step through the hole geometry: B={B}, {N}x{N} "
                               f"(PML 20), T={T}, 16 holes, fwd + adjoint to dL/d(x, y, r)",
                   "l2": "flushed (512 MiB write) before every timed step"},
        "geometry_ms": t_geo * 1e3,
        "geometry_note": "rho and c from the holes plus the adjoint to (x, y, r) through "
                         "autograd, one call at a time (50 calls, warm); at 120x120 its kernels "
                         "are short, so this includes the host's launch time",
        "hole_grads_finite": grads_finite,
        "clocks": clk.summary(),
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.workload == "holey" and args.impl == "ours":
        run_holey(args)
        return
    if args.workload == "fields" and args.impl == "ours":
        run_fields(args)
        return
    if args.workload == "lens" and args.impl == "ours":
        run_lens(args)
        return
    if args.workload == "ragged" and args.impl == "ours":
        run_ragged(args)
        return
    if args.workload == "nonlinear" and args.impl == "ours":
        run_nonlinear(args)
        return
    if args.kernels_only:
        run_kernels_only(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
