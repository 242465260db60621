"""wt_rho_to_c_fwd_noalloc: the rho -> c forward with its scratch in the
library's static device memory.  It must write the same c as wt_rho_to_c_fwd
(given a caller-owned work buffer) on consecutive calls that share the
scratch, and refuse grids larger than its scratch before touching the
device.  Tolerance: the rho -> c tests' 3e-7 (the two calls run the same
kernels, so the results are expected to be identical)."""
import ctypes as C

import numpy as np
import pytest
import torch

from wavetorch_gb300 import _lib

TOL = 3e-7


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def desc(nx, ny):
    return _lib.GeomDesc(nx, ny, 1, 1, 0.5, 100.0, 1.0, 0.5)


def stream(dev):
    return C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)


def test_noalloc_refuses_grids_beyond_its_scratch():
    lib = _lib.load()
    g = desc(1025, 1024)
    p = C.c_void_p(256)
    assert lib.wt_rho_to_c_fwd_noalloc(C.byref(g), p, p, C.c_void_p(512), None) == _lib.WT_ERR_UNSUPPORTED
    assert lib.wt_rho_to_c_fwd_noalloc(C.byref(desc(0, 8)), p, p, p, None) == _lib.WT_ERR_INVALID


@pytest.mark.gpu
@pytest.mark.parametrize("shape", [(120, 120), (300, 170)])
def test_noalloc_matches_the_work_buffer_entry_point(cuda, shape):
    lib = _lib.load()
    nx, ny = shape
    g = desc(nx, ny)
    kern = torch.full((3, 3), 1.0 / 9.0, dtype=torch.float32, device=cuda)
    n = C.c_size_t(0)
    assert lib.wt_rho_to_c_work_bytes(C.byref(g), C.byref(n)) == _lib.WT_OK
    work = torch.empty(n.value // 4, dtype=torch.float32, device=cuda)
    gen = torch.Generator().manual_seed(nx * 1000 + ny)
    for call in range(2):              # two calls in a row share the scratch
        rho = torch.rand(nx, ny, generator=gen).to(cuda)
        c_ref = torch.empty_like(rho)
        c_new = torch.full_like(rho, float("nan"))
        s = stream(rho.device)
        assert lib.wt_rho_to_c_fwd(C.byref(g), C.c_void_p(rho.data_ptr()),
                                   C.c_void_p(kern.data_ptr()), C.c_void_p(c_ref.data_ptr()),
                                   C.c_void_p(work.data_ptr()), s) == _lib.WT_OK
        assert lib.wt_rho_to_c_fwd_noalloc(C.byref(g), C.c_void_p(rho.data_ptr()),
                                           C.c_void_p(kern.data_ptr()),
                                           C.c_void_p(c_new.data_ptr()), s) == _lib.WT_OK
        torch.cuda.synchronize()
        a, b = c_new.cpu().numpy(), c_ref.cpu().numpy()
        assert np.isfinite(a).all(), call
        assert rel(a, b) <= TOL, call
