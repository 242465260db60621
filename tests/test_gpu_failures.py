"""Failure detection of the cluster layout without a GPU fault: host-forced
missing arrivals through the test hooks of include/wavetorch_gb300_testing.h.
A CTA that never sends its boundary rows (distributed shared memory), and a
tape ring whose producer stops issuing slices: the bounded waits give up
after about 2 s, the status word reads WT_ERR_TIMEOUT, nothing faults or
hangs, and the next sequence on the same context is correct."""
import ctypes as C
import time

import numpy as np
import pytest
import torch

from wavetorch_gb300 import _lib
from wavetorch_gb300.data import vowel_like
from wavetorch_gb300.functional import (SeqSpec, _ptr, _stream, lap_order, scalars,
                                        seq_backward, seq_device_status, seq_forward,
                                        seq_workspace_bytes)
from wavetorch_gb300.geom import pml_profile

pytestmark = pytest.mark.gpu

N, B, T = 120, 2, 100
SRC = [(20 * N + 60, -1)]
PRB = [(80 * N + y, 1, i) for i, y in enumerate((35, 50, 65))]


def problem(dev):
    rng = np.random.default_rng(12)
    b = pml_profile((N, N), 20, 3.0, 2).numpy()
    c = (0.5 + 0.5 * rng.random((N, N))).astype(np.float32)
    x = vowel_like(B, T, seed=12)[0]
    g = rng.standard_normal((B, T, 3)).astype(np.float32)
    return tuple(torch.from_numpy(v).to(dev) for v in (b, c, x, g))


def reference_run(_unused, sc, b, c, x, g):
    """The same sequence in the plain form (bit-exact with the reference)."""
    spec = SeqSpec(B, N, N, T, SRC, PRB, form=_lib.WT_FORM_PLAIN)
    out, _, _, ws = seq_forward(spec, sc, b, c, x)
    gc, _ = seq_backward(spec, sc, b, c, x, g, ws, False)
    torch.cuda.synchronize()
    return out, gc


def rel(a, b):
    a, b = a.double().cpu(), b.double().cpu()
    return float((a - b).norm() / b.norm())


def test_cluster_missing_arrival_times_out_and_the_context_survives(cuda):
    b, c, x, g = problem(cuda)
    sc = scalars(0.707, 1.0, lap_order(B, N, N, 1.0))
    spec = SeqSpec(B, N, N, T, SRC, PRB, form=_lib.WT_FORM_FUSED, cluster=4)
    d, keep = spec.desc()
    n = seq_workspace_bytes(spec)
    ws = torch.empty(n, dtype=torch.uint8, device=cuda)
    out = torch.empty(B, T, 3, device=cuda)
    fn = _lib.load().wt_test_cluster_missing_arrival
    fn.argtypes = [C.POINTER(_lib.Scalars), C.POINTER(_lib.SeqDesc)] + [C.c_void_p] * 5 + \
                  [C.c_size_t, C.c_int32, C.c_void_p]
    fn.restype = C.c_int
    torch.cuda.synchronize()
    t0 = time.time()
    assert fn(C.byref(sc), C.byref(d), _ptr(b), _ptr(c), _ptr(x), _ptr(out), _ptr(ws), n, 1,
              _stream(cuda)) == _lib.WT_OK
    torch.cuda.synchronize()
    elapsed = time.time() - t0
    assert seq_device_status(spec, ws) == _lib.WT_ERR_TIMEOUT
    assert 1.0 < elapsed < 60.0
    # the context is usable: the next fused sequence agrees with the plain form
    fout, _, _, ws2 = seq_forward(spec, sc, b, c, x)
    fgc, _ = seq_backward(spec, sc, b, c, x, g, ws2, False)
    torch.cuda.synchronize()
    assert seq_device_status(spec, ws2) == _lib.WT_OK
    pout, pgc = reference_run(None, sc, b, c, x, g)
    assert torch.equal(fout, pout)
    assert rel(fgc, pgc) <= 5e-6


@pytest.mark.parametrize("segment", [-1, 7])
def test_tape_missing_slice_times_out_and_the_context_survives(cuda, segment):
    """The adjoint's ring of Laplacian slices (from the tape, or from the
    checkpoint mode's two-segment stash, segment 7) loses every slice from
    the middle step down: the waits give up after 2 s, nothing faults."""
    b, c, x, g = problem(cuda)
    sc = scalars(0.707, 1.0, lap_order(B, N, N, 1.0))
    spec = SeqSpec(B, N, N, T, SRC, PRB, form=_lib.WT_FORM_FUSED, segment=segment)
    d, keep = spec.desc()
    n = seq_workspace_bytes(spec)
    out, _, _, ws = seq_forward(spec, sc, b, c, x)
    gc = torch.empty(N, N, device=cuda)
    fn = _lib.load().wt_test_tape_missing_slice
    fn.argtypes = [C.POINTER(_lib.Scalars), C.POINTER(_lib.SeqDesc)] + [C.c_void_p] * 6 + \
                  [C.c_size_t, C.c_int32, C.c_void_p]
    fn.restype = C.c_int
    torch.cuda.synchronize()
    t0 = time.time()
    assert fn(C.byref(sc), C.byref(d), _ptr(b), _ptr(c), _ptr(x), _ptr(g), _ptr(gc), _ptr(ws), n,
              T // 2, _stream(cuda)) == _lib.WT_OK
    torch.cuda.synchronize()
    elapsed = time.time() - t0
    assert seq_device_status(spec, ws) == _lib.WT_ERR_TIMEOUT
    assert 1.0 < elapsed < 60.0
    # the context is usable: the next fused sequence agrees with the plain form
    fout, _, _, ws2 = seq_forward(spec, sc, b, c, x)
    fgc, _ = seq_backward(spec, sc, b, c, x, g, ws2, False)
    torch.cuda.synchronize()
    assert seq_device_status(spec, ws2) == _lib.WT_OK
    pout, pgc = reference_run(None, sc, b, c, x, g)
    assert torch.equal(out, pout) and torch.equal(fout, pout)
    assert rel(fgc, pgc) <= 5e-6
