"""ctypes binding of the C ABI in ``include/wavetorch_gb300.h``.

The shared library is built in-tree by :mod:`wavetorch_gb300.build`.  There is
no CPU fallback: every entry point that computes raises
:class:`WaveKernelError` when the library is missing or a call fails.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

from . import build as _build

WT_OK = 0
WT_ERR_INVALID = 1
WT_ERR_CUDA = 2
WT_ERR_TIMEOUT = 3
WT_ERR_UNSUPPORTED = 4

WT_LAP_SEQ = 0
WT_LAP_PAIRED = 1

WT_FORM_PLAIN = 0
WT_FORM_FUSED = 1

# Every symbol the header declares, in header order.
EXPORTED = [
    "wt_version", "wt_status_string", "wt_last_error", "wt_kernel_launches",
    "wt_step_fwd", "wt_step_bwd",
    "wt_seq_workspace_bytes", "wt_seq_fwd", "wt_seq_bwd", "wt_seq_device_status",
    "wt_loss_ce_normalize_power", "wt_seq_bwd_sum",
    "wt_seq_workspace_bytes_nl", "wt_seq_fwd_nl", "wt_seq_bwd_nl",
    "wt_rho_to_c_fwd", "wt_rho_to_c_bwd", "wt_rho_to_c_work_bytes", "wt_rho_to_c_fwd_noalloc",
    "wt_holey_fwd", "wt_holey_bwd", "wt_holey_work_bytes",
    "wt_ragged_plan",
    "wt_ragged_workspace_bytes", "wt_ragged_prepare", "wt_ragged_fwd", "wt_ragged_bwd",
    "wt_ragged_status",
]


class WaveKernelError(RuntimeError):
    """A wavetorch_gb300 C-ABI call failed (or the library is unavailable)."""


class Scalars(C.Structure):
    _fields_ = [("dt", C.c_float), ("h", C.c_float), ("lap_order", C.c_int32)]


class SourceEntry(C.Structure):
    _fields_ = [("cell", C.c_int32), ("in_row", C.c_int32)]


class ProbeEntry(C.Structure):
    _fields_ = [("cell", C.c_int32), ("kind", C.c_int32), ("order", C.c_int32)]


class SeqDesc(C.Structure):
    _fields_ = [
        ("batch", C.c_int32), ("nx", C.c_int32), ("ny", C.c_int32), ("steps", C.c_int32),
        ("n_sources", C.c_int32), ("sources_host", C.POINTER(SourceEntry)),
        ("n_probes", C.c_int32), ("probes_host", C.POINTER(ProbeEntry)),
        ("form", C.c_int32), ("segment", C.c_int32), ("cluster", C.c_int32),
        ("output_fields", C.c_int32), ("coef_batched", C.c_int32), ("sm_count", C.c_int32),
    ]


class NonLinear(C.Structure):
    _fields_ = [("satdamp_b0", C.c_float), ("satdamp_uth", C.c_float), ("c_nl", C.c_float)]


class GeomDesc(C.Structure):
    _fields_ = [
        ("nx", C.c_int32), ("ny", C.c_int32), ("blur_radius", C.c_int32), ("blur_n", C.c_int32),
        ("eta", C.c_float), ("beta", C.c_float), ("c0", C.c_float), ("c1", C.c_float),
    ]


class HoleyDesc(C.Structure):
    _fields_ = [
        ("nx", C.c_int32), ("ny", C.c_int32), ("n_holes", C.c_int32),
        ("eta", C.c_float), ("beta", C.c_float), ("c0", C.c_float), ("c1", C.c_float),
    ]


class RaggedOption(C.Structure):
    _fields_ = [("cluster", C.c_int32), ("ctas", C.c_int32), ("seconds", C.c_double)]


class RaggedGroup(C.Structure):
    _fields_ = [("instances", C.c_int32), ("scale", C.c_double), ("n_options", C.c_int32),
                ("options", C.POINTER(RaggedOption))]


class RaggedModel(C.Structure):
    _fields_ = [("nx", C.c_int32), ("ny", C.c_int32), ("steps", C.c_int32),
                ("n_sources", C.c_int32), ("sources_host", C.POINTER(SourceEntry)),
                ("n_probes", C.c_int32), ("probes_host", C.POINTER(ProbeEntry)),
                ("b", C.c_void_p), ("c", C.c_void_p), ("x", C.c_void_p), ("out", C.c_void_p),
                ("grad_out", C.c_void_p), ("grad_c", C.c_void_p)]


class RaggedPlan(C.Structure):
    _fields_ = [("n_models", C.c_int32), ("ctas", C.c_int32), ("strip", C.c_int32),
                ("n_items", C.c_int32), ("smem_fwd", C.c_size_t), ("smem_bwd", C.c_size_t),
                ("workspace_bytes", C.c_size_t), ("off_params", C.c_size_t),
                ("off_first", C.c_size_t), ("off_items", C.c_size_t), ("off_halo", C.c_size_t),
                ("halo_bytes", C.c_size_t), ("off_err", C.c_size_t),
                ("est_steps_per_cta", C.c_double)]


_VP = C.c_void_p
_lock = threading.Lock()
_lib = None


def _declare(lib):
    P = C.POINTER
    lib.wt_version.restype = C.c_char_p
    lib.wt_status_string.restype = C.c_char_p
    lib.wt_status_string.argtypes = [C.c_int]
    lib.wt_last_error.restype = C.c_char_p
    lib.wt_kernel_launches.restype = C.c_uint64
    lib.wt_kernel_launches.argtypes = []
    i32 = C.c_int32
    lib.wt_step_fwd.argtypes = [P(Scalars), i32, i32, i32, i32, _VP, _VP, _VP, _VP, _VP, _VP]
    lib.wt_step_bwd.argtypes = [P(Scalars), i32, i32, i32, i32, _VP, _VP, _VP, _VP, _VP,
                                _VP, _VP, _VP, _VP, _VP]
    lib.wt_seq_workspace_bytes.argtypes = [P(SeqDesc), P(C.c_size_t)]
    lib.wt_seq_fwd.argtypes = [P(Scalars), P(SeqDesc), _VP, _VP, _VP, _VP, _VP, _VP, _VP,
                               C.c_size_t, _VP]
    lib.wt_seq_bwd.argtypes = [P(Scalars), P(SeqDesc), _VP, _VP, _VP, _VP, _VP, _VP, _VP,
                               C.c_size_t, _VP]
    lib.wt_seq_device_status.argtypes = [P(SeqDesc), _VP, C.c_size_t, _VP]
    lib.wt_loss_ce_normalize_power.argtypes = [i32, i32, _VP, _VP, _VP, _VP, _VP]
    lib.wt_seq_bwd_sum.argtypes = [P(Scalars), P(SeqDesc), _VP, _VP, _VP, _VP, _VP, _VP,
                                   C.c_size_t, _VP]
    lib.wt_seq_workspace_bytes_nl.argtypes = [P(SeqDesc), P(C.c_size_t)]
    lib.wt_seq_fwd_nl.argtypes = [P(Scalars), P(SeqDesc), P(NonLinear), _VP, _VP, _VP, _VP, _VP,
                                  _VP, _VP, C.c_size_t, _VP]
    lib.wt_seq_bwd_nl.argtypes = [P(Scalars), P(SeqDesc), P(NonLinear), _VP, _VP, _VP, _VP, _VP,
                                  _VP, _VP, _VP, _VP, C.c_size_t, _VP]
    lib.wt_rho_to_c_fwd.argtypes = [P(GeomDesc), _VP, _VP, _VP, _VP, _VP]
    lib.wt_rho_to_c_bwd.argtypes = [P(GeomDesc), _VP, _VP, _VP, _VP, _VP, _VP]
    lib.wt_rho_to_c_work_bytes.argtypes = [P(GeomDesc), P(C.c_size_t)]
    lib.wt_rho_to_c_fwd_noalloc.argtypes = [P(GeomDesc), _VP, _VP, _VP, _VP]
    lib.wt_holey_fwd.argtypes = [P(HoleyDesc), _VP, _VP, _VP, _VP, _VP, _VP, _VP]
    lib.wt_holey_bwd.argtypes = [P(HoleyDesc)] + [_VP] * 10
    lib.wt_holey_work_bytes.argtypes = [P(HoleyDesc), P(C.c_size_t)]
    lib.wt_ragged_plan.argtypes = [P(RaggedGroup), C.c_int32, C.c_int32, P(C.c_int32)]
    lib.wt_ragged_workspace_bytes.argtypes = [P(Scalars), P(RaggedModel), C.c_int32, C.c_int32,
                                              C.c_int32, P(C.c_size_t)]
    lib.wt_ragged_prepare.argtypes = [P(Scalars), P(RaggedModel), C.c_int32, C.c_int32,
                                      C.c_int32, _VP, C.c_size_t, P(RaggedPlan)]
    lib.wt_ragged_fwd.argtypes = [P(RaggedPlan), _VP, _VP]
    lib.wt_ragged_bwd.argtypes = [P(RaggedPlan), _VP, _VP]
    lib.wt_ragged_status.argtypes = [P(RaggedPlan), _VP, _VP]
    for name in EXPORTED:
        if name not in ("wt_version", "wt_status_string", "wt_last_error", "wt_kernel_launches"):
            getattr(lib, name).restype = C.c_int
    return lib


def library_path() -> str:
    return _build.LIB_PATH


def load(build_if_missing: bool = True):
    """Load (building first if needed) and return the ctypes library."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.LIB_PATH
        if build_if_missing and (not os.path.exists(path) or _build._stale()):
            try:
                path = _build.build()
            except Exception as e:  # pragma: no cover - depends on toolchain
                raise WaveKernelError(f"cannot build {_build.LIB_NAME}: {e}") from e
        if not os.path.exists(path):
            raise WaveKernelError(f"{path} is missing; run wavetorch_gb300.build.build()")
        _lib = _declare(C.CDLL(path))
        return _lib


def check(status: int, what: str) -> None:
    if status != WT_OK:
        lib = load()
        msg = lib.wt_status_string(status).decode()
        detail = lib.wt_last_error().decode() if status == WT_ERR_CUDA else ""
        raise WaveKernelError(f"{what} failed: {msg}" + (f" ({detail})" if detail else ""))


def kernel_launches() -> int:
    """Kernels launched by the library so far (all threads)."""
    return int(load().wt_kernel_launches())
