"""wt_rho_to_c_fwd_noalloc: the rho -> c forward for callers that cannot
hand the library a work buffer (C or ctypes code with no allocator at hand,
or a loop whose device memory was budgeted up front).  Its scratch lives in
the library's static device memory.

It runs the same kernels as wt_rho_to_c_fwd, so its c must be identical
(bit for bit) to that entry point's on consecutive calls that share the
scratch, for 0, 1 and 2 blur passes and at the largest grid the scratch
holds (1024 x 1024); once it is also checked against the reference's own c
(golden geom_n100, within the rho -> c tests' 3e-7: tanh differs from the
reference's by ulps).  Grids larger than its scratch are refused before the
device is touched.  This file runs last so that a failure here leaves every
other test already run."""
import ctypes as C

import numpy as np
import pytest
import torch

from conftest import golden
from wavetorch_gb300 import _lib

GOLDEN_TOL = 3e-7


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def desc(nx, ny, blur_n=1):
    return _lib.GeomDesc(nx, ny, 1, blur_n, 0.5, 100.0, 1.0, 0.5)


def stream(dev):
    return C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)


def ptr(t):
    return C.c_void_p(t.data_ptr())


def test_noalloc_refuses_grids_beyond_its_scratch():
    lib = _lib.load()
    g = desc(1025, 1024)
    p = C.c_void_p(256)
    assert lib.wt_rho_to_c_fwd_noalloc(C.byref(g), p, p, C.c_void_p(512), None) == _lib.WT_ERR_UNSUPPORTED
    assert lib.wt_rho_to_c_fwd_noalloc(C.byref(desc(0, 8)), p, p, p, None) == _lib.WT_ERR_INVALID


@pytest.mark.gpu
@pytest.mark.parametrize("blur_n", [0, 1, 2])
@pytest.mark.parametrize("shape", [(120, 120), (300, 170), (1024, 1024)])
def test_noalloc_matches_the_work_buffer_entry_point(cuda, shape, blur_n):
    lib = _lib.load()
    nx, ny = shape
    g = desc(nx, ny, blur_n)
    kern = torch.full((3, 3), 1.0 / 9.0, dtype=torch.float32, device=cuda)
    n = C.c_size_t(0)
    assert lib.wt_rho_to_c_work_bytes(C.byref(g), C.byref(n)) == _lib.WT_OK
    work = torch.empty(n.value // 4, dtype=torch.float32, device=cuda)
    gen = torch.Generator().manual_seed(nx * 1000 + ny + blur_n)
    for call in range(2):              # two calls in a row share the scratch
        rho = torch.rand(nx, ny, generator=gen).to(cuda)
        c_ref = torch.empty_like(rho)
        c_new = torch.full_like(rho, float("nan"))
        s = stream(rho.device)
        assert lib.wt_rho_to_c_fwd(C.byref(g), ptr(rho), ptr(kern), ptr(c_ref), ptr(work),
                                   s) == _lib.WT_OK
        assert lib.wt_rho_to_c_fwd_noalloc(C.byref(g), ptr(rho), ptr(kern), ptr(c_new),
                                           s) == _lib.WT_OK
        torch.cuda.synchronize()
        a, b = c_new.cpu().numpy(), c_ref.cpu().numpy()
        assert np.isfinite(a).all(), call
        assert np.array_equal(a, b), call


@pytest.mark.gpu
def test_noalloc_matches_the_reference_c(cuda):
    """c of the reference's free-form geometry (100 x 100, one 3x3 blur
    pass), twice in a row through the shared scratch."""
    lib = _lib.load()
    d = golden("geom_n100")
    g = desc(100, 100, 1)
    rho = torch.from_numpy(d["rho"]).to(cuda)
    kern = torch.from_numpy(np.ascontiguousarray(d["blur_kernel"])).to(cuda)
    for call in range(2):
        c = torch.full_like(rho, float("nan"))
        assert lib.wt_rho_to_c_fwd_noalloc(C.byref(g), ptr(rho), ptr(kern), ptr(c),
                                           stream(cuda)) == _lib.WT_OK
        torch.cuda.synchronize()
        assert rel(c.cpu().numpy(), d["c"]) <= GOLDEN_TOL, call
