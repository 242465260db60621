"""Generate the golden fixtures in this directory by running the unmodified
reference (fancompute/wavetorch v0.2.1) on the CPU.

Run from the repository root where the reference sources are available:

    WAVETORCH_REFERENCE=/path/to/wavetorch python tests/golden/gen_golden.py

Each case is saved as ``<name>.npz`` (float32 arrays plus a few scalars).  The
inputs are seeded synthetic data; nothing from the reference's dataset is
stored.  The fixtures pin the oracle (tests/test_oracle_golden.py) and the GPU
kernels (tests/test_gpu_parity.py).
"""
from __future__ import annotations

import os
import sys

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import ref_shim  # noqa: E402
from wavetorch_gb300.data import sinusoid, vowel_like  # noqa: E402

torch.set_num_threads(max(1, os.cpu_count() or 1))


def _np(t):
    return t.detach().cpu().numpy()


def fixed_c(geom):
    """Make geom.c return one tensor (so its gradient can be read) while
    keeping the reference's own rho -> c computation."""
    cls = type(geom)
    orig = cls.c
    c = orig.fget(geom)
    cls.c = property(lambda self: c)
    return c, lambda: setattr(cls, 'c', orig)


def run_model(wt, *, N, abs_N, B, T, x, labels, sources, probes, rho0, dt=0.707, h=1.0,
              abs_sig=3.0, abs_p=2, c0=1.0, c1=0.5, satdamp_b0=0.0, satdamp_uth=0.0, c_nl=0.0,
              field_steps=(), dtype=torch.float32):
    """Forward + CE(normalize_power(sum_t I)) backward through the reference."""
    geom = wt.WaveGeometryFreeForm((N, N), h, c0=c0, c1=c1, abs_N=abs_N, abs_sig=abs_sig,
                                   abs_p=abs_p, rho=rho0.to(dtype))
    cell = wt.WaveCell(dt, geom, satdamp_b0=satdamp_b0, satdamp_uth=satdamp_uth, c_nl=c_nl)
    model = wt.WaveRNN(cell, [s() for s in sources], [p() for p in probes])
    c, restore = fixed_c(geom)
    try:
        xt = torch.from_numpy(x).to(dtype)
        y = model(xt)
        I = y.sum(dim=1)
        loss = torch.nn.CrossEntropyLoss()(wt.utils.normalize_power(I), torch.from_numpy(labels))
        gy, gc = torch.autograd.grad(loss, [y, c], retain_graph=True)
        loss.backward()
        out = {"out": _np(y), "loss": np.array(loss.item()), "grad_out": _np(gy),
               "grad_c": _np(gc), "grad_rho": _np(geom.rho.grad), "c": _np(c), "b": _np(geom.b),
               "rho": _np(geom.rho), "blur_kernel": _np(geom.blur_kernel[0, 0])}
        if field_steps:
            with torch.no_grad():
                f = model(xt, output_fields=True)
            for t in field_steps:
                out[f"field_{t}"] = _np(f[:, t])
        return out
    finally:
        restore()


def as32(d):
    return {k: (v.astype(np.float32) if isinstance(v, np.ndarray) and v.dtype == np.float64 else v)
            for k, v in d.items()}


def case_cfg0(wt):
    """Configuration-0 physics at reduced T: B=1, 100x100, PML 20 (p=2, 3.0)."""
    N, T = 100, 200
    g = torch.Generator().manual_seed(0)
    rho0 = torch.rand(N, N, generator=g)
    x = sinusoid(T, 0.05)
    labels = np.array([0])
    kw = dict(N=N, abs_N=20, B=1, T=T, x=x, labels=labels,
              sources=[lambda: wt.WaveSource(20, 50)],
              probes=[lambda y=y: wt.WaveIntensityProbe(80, y) for y in (35, 50, 65)], rho0=rho0)
    r32 = run_model(wt, field_steps=(0, 99, T - 1), **kw)
    wt.utils.set_dtype('float64')
    try:
        r64 = run_model(wt, dtype=torch.float64, field_steps=(0, 99, T - 1), **kw)
    finally:
        wt.utils.set_dtype('float32')
    res = dict(r32)
    res.update({"x": x, "labels": labels, "out64": r64["out"], "grad_c64": r64["grad_c"],
                "grad_rho64": r64["grad_rho"], "c64": r64["c"]})
    res.update({f"field64_{t}": r64[f"field_{t}"] for t in (0, 99, T - 1)})
    res.update(meta(N=N, T=T, B=1, abs_N=20, sources=[(20 * N + 50, -1)],
                    probes=[(80 * N + y, 1, i) for i, y in enumerate((35, 50, 65))]))
    return as32(res)


def case_cfg1(wt):
    """Configuration-1 physics at reduced batch and T: B=4, 120x120, PML 20."""
    N, T, B = 120, 150, 4
    g = torch.Generator().manual_seed(1)
    rho0 = torch.rand(N, N, generator=g)
    x, labels = vowel_like(B, T, seed=1)
    r = run_model(wt, N=N, abs_N=20, B=B, T=T, x=x, labels=labels,
                  sources=[lambda: wt.WaveSource(20, 60)],
                  probes=[lambda y=y: wt.WaveIntensityProbe(80, y) for y in (35, 50, 65)],
                  rho0=rho0, field_steps=(T - 1,))
    r.update({"x": x, "labels": labels})
    r.update(meta(N=N, T=T, B=B, abs_N=20, sources=[(20 * N + 60, -1)],
                  probes=[(80 * N + y, 1, i) for i, y in enumerate((35, 50, 65))]))
    return as32(r)


def case_multi(wt):
    """Two point sources (one cell shared), mixed probe kinds, a repeated probe cell."""
    N, T, B = 48, 80, 3
    g = torch.Generator().manual_seed(2)
    rho0 = torch.rand(N, N, generator=g)
    x, labels = vowel_like(B, T, seed=2)
    P = [(30, 20, 1), (30, 24, 0), (30, 20, 0), (33, 28, 1)]
    r = run_model(wt, N=N, abs_N=10, B=B, T=T, x=x, labels=labels,
                  sources=[lambda: wt.WaveSource(12, 24), lambda: wt.WaveSource(12, 24),
                           lambda: wt.WaveSource(14, 20)],
                  probes=[(lambda px=px, py=py, k=k: (wt.WaveIntensityProbe if k else wt.WaveProbe)(px, py))
                          for px, py, k in P],
                  rho0=rho0, field_steps=(T - 1,))
    r.update({"x": x, "labels": labels})
    r.update(meta(N=N, T=T, B=B, abs_N=10,
                  sources=[(12 * N + 24, -1), (12 * N + 24, -1), (14 * N + 20, -1)],
                  probes=[(px * N + py, k, i) for i, (px, py, k) in enumerate(P)]))
    return as32(r)


def case_line(wt):
    """B=1 line sources (horizontal and diagonal), 64x64, PML 10."""
    N, T = 64, 70
    g = torch.Generator().manual_seed(3)
    rho0 = torch.rand(N, N, generator=g)
    x = sinusoid(T, 0.02)
    labels = np.array([1])
    r = run_model(wt, N=N, abs_N=10, B=1, T=T, x=x, labels=labels,
                  sources=[lambda: wt.WaveLineSource(14, 12, 14, 50),
                           lambda: wt.WaveLineSource(20, 15, 31, 40)],
                  probes=[lambda y=y: wt.WaveIntensityProbe(50, y) for y in (20, 32, 44)],
                  rho0=rho0, field_steps=(T - 1,))
    r.update({"x": x, "labels": labels})
    l1 = ref_shim._line(14, 12, 14, 50)
    l2 = ref_shim._line(20, 15, 31, 40)
    cells = [int(a) * N + int(b) for a, b in zip(*l1)] + [int(a) * N + int(b) for a, b in zip(*l2)]
    r.update(meta(N=N, T=T, B=1, abs_N=10, sources=[(cc, -1) for cc in cells],
                  probes=[(50 * N + y, 1, i) for i, y in enumerate((20, 32, 44))]))
    return as32(r)


def case_nonlinear(wt):
    """Configuration-2 physics (c_nl and saturable damping) at small size."""
    N, T, B = 40, 60, 2
    g = torch.Generator().manual_seed(4)
    rho0 = torch.rand(N, N, generator=g)
    x, labels = vowel_like(B, T, seed=4)
    x = (x * np.float32(0.2)).astype(np.float32)   # keeps the Kerr term inside the CFL limit
    r = run_model(wt, N=N, abs_N=8, B=B, T=T, x=x, labels=labels,
                  sources=[lambda: wt.WaveSource(10, 20)],
                  probes=[lambda y=y: wt.WaveIntensityProbe(30, y) for y in (12, 20, 28)],
                  rho0=rho0, satdamp_b0=0.05, satdamp_uth=float(np.sqrt(0.1)), c_nl=0.1)
    r.update({"x": x, "labels": labels, "satdamp_b0": np.array(0.05),
              "satdamp_uth": np.array(np.sqrt(0.1)), "c_nl": np.array(0.1)})
    r.update(meta(N=N, T=T, B=B, abs_N=8, sources=[(10 * N + 20, -1)],
                  probes=[(30 * N + y, 1, i) for i, y in enumerate((12, 20, 28))]))
    return as32(r)


def loss64(wt, kw, rho):
    """Loss of the model of `kw` at density `rho`, run in float64."""
    geom = wt.WaveGeometryFreeForm((kw["N"], kw["N"]), 1.0, c0=1.0, c1=0.5, abs_N=kw["abs_N"],
                                   abs_sig=3.0, abs_p=2, rho=rho)
    with torch.no_grad():
        geom.rho.copy_(rho)        # keep the perturbed entry (the ctor constrains)
    cell = wt.WaveCell(0.707, geom, satdamp_b0=kw["satdamp_b0"], satdamp_uth=kw["satdamp_uth"],
                       c_nl=kw["c_nl"])
    model = wt.WaveRNN(cell, [s() for s in kw["sources"]], [p() for p in kw["probes"]])
    with torch.no_grad():
        y = model(torch.from_numpy(kw["x"]).to(torch.float64))
        return torch.nn.CrossEntropyLoss()(wt.utils.normalize_power(y.sum(dim=1)),
                                           torch.from_numpy(kw["labels"])).item()


def case_fd64(wt, nonlinear):
    """Central finite differences of the loss in float64 at 16 random design
    entries of rho (eps = 1e-5), next to the float64 autograd gradient."""
    N, T, B, abs_N = 40, 60, 2, 8
    g = torch.Generator().manual_seed(13 if nonlinear else 14)
    rho0 = torch.rand(N, N, generator=g)
    x, labels = vowel_like(B, T, seed=13 if nonlinear else 14)
    x = (x * np.float32(0.2)).astype(np.float32)
    kw = dict(N=N, abs_N=abs_N, x=x, labels=labels,
              sources=[lambda: wt.WaveSource(10, 20)],
              probes=[lambda y=y: wt.WaveIntensityProbe(30, y) for y in (12, 20, 28)],
              satdamp_b0=0.05 if nonlinear else 0.0,
              satdamp_uth=float(np.sqrt(0.1)) if nonlinear else 0.0,
              c_nl=0.1 if nonlinear else 0.0)
    wt.utils.set_dtype('float64')
    try:
        r64 = run_model(wt, N=N, abs_N=abs_N, B=B, T=T, x=x, labels=labels,
                        sources=kw["sources"], probes=kw["probes"], rho0=rho0,
                        satdamp_b0=kw["satdamp_b0"], satdamp_uth=kw["satdamp_uth"],
                        c_nl=kw["c_nl"], dtype=torch.float64)
        rho = torch.from_numpy(r64["rho"])                 # constrained density
        design = np.argwhere((r64["b"] == 0).reshape(-1)).reshape(-1)
        pick = np.random.default_rng(15).choice(design, 16, replace=False)
        eps = 1e-5
        fd = []
        for i in pick:
            rp, rm = rho.clone(), rho.clone()
            rp.view(-1)[i] += eps
            rm.view(-1)[i] -= eps
            fd.append((loss64(wt, kw, rp) - loss64(wt, kw, rm)) / (2 * eps))
    finally:
        wt.utils.set_dtype('float32')
    res = {"rho": r64["rho"].astype(np.float32), "x": x, "labels": labels,
           "fd_index": pick.astype(np.int64), "fd_grad": np.array(fd, np.float64),
           "grad_rho64": r64["grad_rho"].reshape(-1)[pick], "eps": np.array(eps),
           "satdamp_b0": np.array(kw["satdamp_b0"]), "satdamp_uth": np.array(kw["satdamp_uth"]),
           "c_nl": np.array(kw["c_nl"])}
    res.update(meta(N=N, T=T, B=B, abs_N=abs_N, sources=[(10 * N + 20, -1)],
                    probes=[(30 * N + y, 1, i) for i, y in enumerate((12, 20, 28))]))
    return res


def case_step(wt, B, N, dt, h, seed):
    """One TimeStep forward/backward on random inputs (the check of
    study/utils/test_grad.py, with stored values)."""
    g = torch.Generator().manual_seed(seed)
    b = torch.rand(N, N, generator=g).requires_grad_()
    c = torch.rand(N, N, generator=g).requires_grad_()
    y1 = torch.rand(B, N, N, generator=g).requires_grad_()
    y2 = torch.rand(B, N, N, generator=g).requires_grad_()
    gout = torch.randn(B, N, N, generator=g)
    dtt, ht = torch.tensor(dt), torch.tensor(h)
    y = wt.cell.TimeStep.apply(b, c, y1, y2, dtt, ht)
    gb, gc, gy1, gy2 = torch.autograd.grad(y, [b, c, y1, y2], gout)
    return {"b": _np(b), "c": _np(c), "y1": _np(y1), "y2": _np(y2), "grad_y": _np(gout),
            "y": _np(y), "grad_b": _np(gb), "grad_c": _np(gc), "grad_y1": _np(gy1),
            "grad_y2": _np(gy2), "dt": np.array(dt, np.float32), "h": np.array(h, np.float32)}


def case_geom(wt, N, seed):
    g = torch.Generator().manual_seed(seed)
    geom = wt.WaveGeometryFreeForm((N, N), 1.0, c0=1.0, c1=0.5, abs_N=20, abs_sig=3.0, abs_p=2,
                                   rho=torch.rand(N, N, generator=g))
    c = geom.c
    gc = torch.randn(N, N, generator=g)
    (gr,) = torch.autograd.grad(c, [geom.rho], gc)
    return {"rho": _np(geom.rho), "blur_kernel": _np(geom.blur_kernel[0, 0]), "c": _np(c),
            "grad_c": _np(gc), "grad_rho": _np(gr), "b": _np(geom.b)}


def case_holey(wt):
    """WaveGeometryHoley (wavetorch/geom.py:88-132): rho and c of three
    exponential holes on a 64x48 grid, and the gradient of a random linear
    functional of c with respect to the holes' x, y, r."""
    g = torch.Generator().manual_seed(16)
    geom = wt.WaveGeometryHoley((64, 48), 1.0, c0=1.0, c1=0.5, abs_N=10, abs_sig=3.0, abs_p=2,
                                x=[20.3, 35.5, 44.0], y=[12.0, 30.0, 24.5], r=[3.0, 5.5, 2.5])
    c = geom.c
    w = torch.randn(64, 48, generator=g)
    gx, gy, gr = torch.autograd.grad((c * w).sum(), [geom.x, geom.y, geom.r])
    return {"rho": _np(geom.rho), "c": _np(c), "w": _np(w), "grad_x": _np(gx), "grad_y": _np(gy),
            "grad_r": _np(gr), "x": np.array([20.3, 35.5, 44.0], np.float32),
            "y": np.array([12.0, 30.0, 24.5], np.float32), "r": np.array([3.0, 5.5, 2.5], np.float32)}


def ref_model_file(wt):
    """A model file written by the reference's own ``io.save_model``
    (wavetorch/io.py:13-40): free-form geometry 40x40 (PML 8) with a seeded
    density, two point sources, three intensity probes; plus the model's
    float32 outputs on a short seeded input, for a load-and-run check."""
    N, T, B = 40, 50, 2
    g = torch.Generator().manual_seed(17)
    geom = wt.WaveGeometryFreeForm((N, N), 1.0, c0=1.0, c1=0.5, abs_N=8, abs_sig=3.0, abs_p=2,
                                   rho=torch.rand(N, N, generator=g))
    cell = wt.WaveCell(0.707, geom)
    model = wt.WaveRNN(cell, [wt.WaveSource(10, 20), wt.WaveSource(12, 14)],
                       [wt.WaveIntensityProbe(30, y) for y in (12, 20, 28)])
    wt.io.save_model(model, "ref_model", savedir=HERE + "/", cfg={"dtype": "float32"},
                     verbose=False)
    x, _ = vowel_like(B, T, seed=17)
    with torch.no_grad():
        out = model(torch.from_numpy(x))
    return {"x": x, "out": _np(out), "c": _np(geom.c), "b": _np(geom.b), "rho": _np(geom.rho)}


def state_keys(wt):
    """state_dict keys, shapes and dtypes of a reference model (drop-in check)."""
    geom = wt.WaveGeometryFreeForm((50, 50), 1.0, c0=1.0, c1=0.5, abs_N=10, abs_sig=3.0, abs_p=2,
                                   rho='half')
    cell = wt.WaveCell(0.707, geom)
    model = wt.WaveRNN(cell, [wt.WaveSource(10, 25)],
                       [wt.WaveIntensityProbe(40, y) for y in (15, 25, 35)])
    return {k: [list(v.shape), str(v.dtype)] for k, v in model.state_dict().items()}


def meta(N, T, B, abs_N, sources, probes):
    return {"N": np.array(N), "T": np.array(T), "B": np.array(B), "abs_N": np.array(abs_N),
            "dt": np.array(0.707, np.float32), "h": np.array(1.0, np.float32),
            "sources": np.array(sources, np.int32).reshape(-1, 2),
            "probes": np.array(probes, np.int32).reshape(-1, 3)}


def main():
    wt = ref_shim.import_reference()
    torch.set_default_dtype(torch.float32)
    cases = {
        "cfg0_small": lambda: case_cfg0(wt),
        "cfg1_small": lambda: case_cfg1(wt),
        "multi": lambda: case_multi(wt),
        "line": lambda: case_line(wt),
        "nonlinear": lambda: case_nonlinear(wt),
        "fd64_linear": lambda: case_fd64(wt, False),
        "fd64_nonlinear": lambda: case_fd64(wt, True),
        "step_b2_h025": lambda: case_step(wt, 2, 16, 0.1, 0.25, 5),
        "step_b1_h1": lambda: case_step(wt, 1, 14, 0.5, 1.0, 6),
        "step_b20_h1": lambda: case_step(wt, 20, 10, 0.707, 1.0, 7),
        "geom_n100": lambda: case_geom(wt, 100, 8),
        "geom_n160": lambda: case_geom(wt, 160, 9),
        "holey": lambda: case_holey(wt),
        "ref_model": lambda: ref_model_file(wt),
    }
    only = set(sys.argv[1:])
    if not only or "state_keys" in only:
        import json
        with open(os.path.join(HERE, "state_keys.json"), "w") as fh:
            json.dump(state_keys(wt), fh, indent=1, sort_keys=True)
    for name, fn in cases.items():
        if only and name not in only:
            continue
        d = fn()
        d["reference_version"] = np.array(wt.__version__)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **d)
        print("wrote", name, sum(v.nbytes for v in d.values() if isinstance(v, np.ndarray)), "bytes")


if __name__ == "__main__":
    main()
