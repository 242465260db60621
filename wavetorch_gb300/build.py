"""Build the CUDA C-ABI library ``libwavetorch_gb300.so`` in-tree.

Each translation unit under ``csrc/`` is compiled for sm_103a in parallel and
linked into one shared library next to this file.  The library has a plain C
ABI (``include/wavetorch_gb300.h``) and no torch dependency; the Python side
loads it with ctypes.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB_NAME = "libwavetorch_gb300.so"
LIB_PATH = os.path.join(HERE, LIB_NAME)
# (source, object name, extra flags): seq_fused.cu builds as four parts (its
# kernels per Laplacian order) so that they compile in parallel
SOURCES = [("api.cu", "api", []), ("step.cu", "step", []), ("seq_band.cu", "seq_band", []),
           ("geom.cu", "geom", []), ("holey.cu", "holey", []), ("ragged.cu", "ragged", []), ("peaks.cu", "peaks", []), ("ragged_seq.cu", "ragged_seq", [])] + \
          [("seq_fused.cu", f"seq_fused_{k}", [f"-DWT_FUSED_PART={k}"]) for k in range(4)]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
    "-Xcompiler", "-fPIC,-ffp-contract=off,-O2",
    "-Xptxas", "-v",
]


def nvcc_path() -> str:
    p = shutil.which("nvcc")
    if p:
        return p
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build wavetorch_gb300")


def _compile(unit, verbose: bool) -> tuple[str, str]:
    src, name, extra = unit
    obj = os.path.join(BUILD, name + ".o")
    cmd = [nvcc_path(), *ARCH, *NVCC_FLAGS, *extra, "-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def _stale() -> bool:
    if not os.path.exists(LIB_PATH):
        return True
    t = os.path.getmtime(LIB_PATH)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps.append(os.path.join(HERE, "..", "include", "wavetorch_gb300.h"))
    deps.append(os.path.abspath(__file__))
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile (if stale) and return the path of the shared library."""
    if not force and not _stale():
        return LIB_PATH
    os.makedirs(BUILD, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    objs = [o for o, _ in results]
    if verbose:
        for _, log in results:
            sys.stderr.write(log)
    tmp = LIB_PATH + ".tmp"
    cmd = [nvcc_path(), *ARCH, "-shared", "-cudart", "shared", *objs, "-o", tmp,
           "-Xlinker", "-rpath,/usr/local/cuda/lib64"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


def ptxas_report() -> str:
    """Compile every unit again and return the ptxas resource report."""
    os.makedirs(BUILD, exist_ok=True)
    return "\n".join(_compile(s, True)[1] for s in SOURCES)


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
