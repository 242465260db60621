"""ORACLE -- test infrastructure only (tests, smoke check, CPU baseline).

numpy/ctypes front end of ``wave_oracle.c``, the plain-C float32 restatement
of fancompute/wavetorch v0.2.1's time-stepping path (wavetorch/cell.py:8-44,
:79-107, wavetorch/operators.py:5-11, wavetorch/rnn.py:36-72,
wavetorch/geom.py:63-85, 109-132, 207-233).  Pinned against golden vectors produced by running the reference
(tests/golden/).  Nothing in the product imports this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libwave_oracle.so")
ORD_SEQ, ORD_PAIRED = 0, 1
ONEDNN_MIN_CELLS = 20480

_lock = threading.Lock()
_lib = None


def build(force: bool = False) -> str:
    src = os.path.join(HERE, "wave_oracle.c")
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB


class Desc(C.Structure):
    _fields_ = [("batch", C.c_int32), ("nx", C.c_int32), ("ny", C.c_int32), ("steps", C.c_int32),
                ("dt", C.c_float), ("h", C.c_float), ("order", C.c_int32),
                ("n_src", C.c_int32), ("src_cell", C.c_void_p), ("src_row", C.c_void_p),
                ("n_prb", C.c_int32), ("prb_cell", C.c_void_p), ("prb_kind", C.c_void_p),
                ("prb_order", C.c_void_p)]


def load():
    global _lib
    with _lock:
        if _lib is None:
            _lib = C.CDLL(build())
            _lib.or_num_threads.restype = C.c_int
        return _lib


def lap_order(batch, nx, ny, h=1.0):
    """torch CPU conv2d's algorithm choice (oneDNN vs im2col+GEMM)."""
    return ORD_SEQ if (batch > 1 or nx * ny > ONEDNN_MIN_CELLS or h != 1.0) else ORD_PAIRED


def _f(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _i(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def step_fwd(b, c, y1, y2, dt, h, order=None):
    y1, y2, b, c = _f(y1), _f(y2), _f(b), _f(c)
    B, nx, ny = y1.shape
    cb = int(b.ndim == 3)
    order = lap_order(B, nx, ny, h) if order is None else order
    y = np.empty_like(y1)
    load().or_step_fwd(B, nx, ny, C.c_float(dt), C.c_float(h), order, cb, _p(b), _p(c), _p(y1),
                       _p(y2), _p(y))
    return y


def step_bwd(b, c, y1, y2, g, dt, h, order=None, need=(True, True, True, True)):
    y1, y2, b, c, g = _f(y1), _f(y2), _f(b), _f(c), _f(g)
    B, nx, ny = y1.shape
    cb = int(b.ndim == 3)
    order = lap_order(B, nx, ny, h) if order is None else order
    cs = y1.shape if cb else (nx, ny)
    gb = np.empty(cs, np.float32) if need[0] else None
    gc = np.empty(cs, np.float32) if need[1] else None
    gy1 = np.empty_like(y1) if need[2] else None
    gy2 = np.empty_like(y1) if need[3] else None
    load().or_step_bwd(B, nx, ny, C.c_float(dt), C.c_float(h), order, cb, _p(b), _p(c), _p(y1),
                       _p(y2), _p(g), _p(gb), _p(gc), _p(gy1), _p(gy2))
    return gb, gc, gy1, gy2


class Seq:
    """One sequence problem: sources [(cell, in_row)], probes [(cell, kind, order)]."""

    def __init__(self, batch, nx, ny, steps, dt, h, sources, probes, order=None):
        self.batch, self.nx, self.ny, self.steps = batch, nx, ny, steps
        self.dt, self.h = float(dt), float(h)
        self.order = lap_order(batch, nx, ny, h) if order is None else order
        self.sc = _i([s[0] for s in sources] or [0])
        self.sr = _i([s[1] for s in sources] or [0])
        self.pc = _i([p[0] for p in probes] or [0])
        self.pk = _i([p[1] for p in probes] or [0])
        self.po = _i([p[2] for p in probes] or [0])
        self.ns, self.np = len(sources), len(probes)

    def desc(self):
        return Desc(self.batch, self.nx, self.ny, self.steps, self.dt, self.h, self.order,
                    self.ns, _p(self.sc), _p(self.sr), self.np, _p(self.pc), _p(self.pk),
                    _p(self.po))

    def forward(self, b, c, x):
        """Returns (out [B,T,Q], hist [B,T,nx,ny])."""
        b, c, x = _f(b), _f(c), _f(x)
        out = np.empty((self.batch, self.steps, self.np), np.float32)
        hist = np.empty((self.batch, self.steps, self.nx, self.ny), np.float32)
        d = self.desc()
        load().or_seq_fwd(C.byref(d), _p(b), _p(c), _p(x), _p(out), _p(hist))
        return out, hist

    def backward(self, b, c, hist, grad_out, want_x=False):
        b, c, hist, g = _f(b), _f(c), _f(hist), _f(grad_out)
        gc = np.empty((self.nx, self.ny), np.float32)
        gx = np.empty((self.batch, self.steps), np.float32) if want_x else None
        d = self.desc()
        load().or_seq_bwd(C.byref(d), _p(b), _p(c), _p(hist), _p(g), _p(gc), _p(gx))
        return gc, gx


class NL(C.Structure):
    _fields_ = [("b0", C.c_float), ("uth", C.c_float), ("cnl", C.c_float)]


def seq_forward_nl(S, b, c_lin, rho, x, b0, uth, cnl):
    """Nonlinear cell (wavetorch/cell.py:8-9, :79-107) over the sequence S:
    returns (out [B,T,Q], hist [B,T,nx,ny])."""
    b, c_lin, rho, x = _f(b), _f(c_lin), _f(rho), _f(x)
    out = np.empty((S.batch, S.steps, S.np), np.float32)
    hist = np.empty((S.batch, S.steps, S.nx, S.ny), np.float32)
    d, n = S.desc(), NL(b0, uth, cnl)
    load().or_seq_fwd_nl(C.byref(d), C.byref(n), _p(b), _p(c_lin), _p(rho), _p(x), _p(out),
                         _p(hist))
    return out, hist


def seq_backward_nl(S, b, c_lin, rho, hist, grad_out, b0, uth, cnl):
    """Returns (dL/dc_lin, the direct dL/drho of the nonlinear terms)."""
    b, c_lin, rho, hist, g = _f(b), _f(c_lin), _f(rho), _f(hist), _f(grad_out)
    gc = np.empty((S.nx, S.ny), np.float32)
    gr = np.empty((S.nx, S.ny), np.float32)
    d, n = S.desc(), NL(b0, uth, cnl)
    load().or_seq_bwd_nl(C.byref(d), C.byref(n), _p(b), _p(c_lin), _p(rho), _p(hist), _p(g),
                         _p(gc), _p(gr))
    return gc, gr


def rho_to_c(rho, kernel, blur_n, eta, beta, c0, c1):
    """Returns (c, tanh values)."""
    rho, k = _f(rho), _f(kernel)
    nx, ny = rho.shape
    rad = (k.shape[-1] - 1) // 2
    c = np.empty_like(rho)
    th = np.empty_like(rho)
    load().or_rho_to_c(nx, ny, rad, blur_n, C.c_float(eta), C.c_float(beta), C.c_float(c0),
                       C.c_float(c1), _p(k), _p(rho), _p(c), _p(th))
    return c, th


def rho_to_c_bwd(th, kernel, blur_n, eta, beta, c0, c1, grad_c):
    th, k, g = _f(th), _f(kernel), _f(grad_c)
    nx, ny = th.shape
    rad = (k.shape[-1] - 1) // 2
    gr = np.empty_like(th)
    load().or_rho_to_c_bwd(nx, ny, rad, blur_n, C.c_float(eta), C.c_float(beta), C.c_float(c0),
                           C.c_float(c1), _p(k), _p(th), _p(g), _p(gr))
    return gr


def holey(nx, ny, x, y, r, eta, beta, c0, c1):
    """Hole geometry (wavetorch/geom.py:109-132): returns (rho, c, tanh values)
    for holes at (x_k, y_k) of radius r_k (the shortest of the three sets)."""
    x, y, r = _f(x).ravel(), _f(y).ravel(), _f(r).ravel()
    nh = min(len(x), len(y), len(r))
    rho = np.empty((nx, ny), np.float32)
    c = np.empty_like(rho)
    th = np.empty_like(rho)
    load().or_holey(nx, ny, nh, C.c_float(eta), C.c_float(beta), C.c_float(c0), C.c_float(c1),
                    _p(x), _p(y), _p(r), _p(rho), _p(c), _p(th))
    return rho, c, th


def holey_bwd(x, y, r, th, eta, beta, c0, c1, grad_rho=None, grad_c=None):
    """Gradients (x, y, r) of <grad_rho, rho> + <grad_c, c> for the holes."""
    x, y, r, th = _f(x).ravel(), _f(y).ravel(), _f(r).ravel(), _f(th)
    nh = min(len(x), len(y), len(r))
    nx, ny = th.shape
    grho = None if grad_rho is None else _f(grad_rho)
    gc = None if grad_c is None else _f(grad_c)
    gx, gy, gr = (np.zeros(nh, np.float32) for _ in range(3))
    load().or_holey_bwd(nx, ny, nh, C.c_float(eta), C.c_float(beta), C.c_float(c0),
                        C.c_float(c1), _p(x), _p(y), _p(r), _p(th), _p(grho), _p(gc), _p(gx),
                        _p(gy), _p(gr))
    return gx, gy, gr


def num_threads() -> int:
    return int(load().or_num_threads())
