"""Import shim for the unmodified reference package (fancompute/wavetorch v0.2.1).

The reference's ``wavetorch/__init__.py`` eagerly imports its plotting, data and
training modules, which need librosa, pandas, seaborn, matplotlib, skimage and
(where it is not installed) scikit-learn.
None of those are installed here and none of them is on the time-stepping path.
This shim registers inert stand-in modules for them (each with a real
``__spec__`` so that ``importlib.util.find_spec`` keeps working) and a small
project-written ``skimage.draw`` with the two functions the path calls:

* ``circle(r, c, radius)`` -- the open-disk rule ``(i-r)^2 + (j-c)^2 < radius^2``,
  clipped at 0 (used by ``wavetorch/geom.py:149`` to build the blur kernel; for
  ``blur_radius=1`` it yields the full 3x3 box).
* ``line(r0, c0, r1, c1)`` -- integer Bresenham (used by
  ``wavetorch/source.py:31``).

The golden-fixture generator imports this module where the reference
sources exist, and ``bench.py --impl reference`` to time the reference's own
CPU path from its pip install (``baseline/_ref``).
"""
import importlib.machinery
import os
import sys
import types

import numpy as np

REFERENCE_ROOT = os.environ.get("WAVETORCH_REFERENCE", "")


def _stub(name, **attrs):
    mod = types.ModuleType(name)
    mod.__spec__ = importlib.machinery.ModuleSpec(name, loader=None)
    mod.__path__ = []
    for k, v in attrs.items():
        setattr(mod, k, v)
    sys.modules[name] = mod
    return mod


def _circle(r, c, radius):
    rr, cc = [], []
    rad = int(np.ceil(radius))
    for i in range(int(r) - rad, int(r) + rad + 1):
        for j in range(int(c) - rad, int(c) + rad + 1):
            if i < 0 or j < 0:
                continue
            if (i - r) ** 2 + (j - c) ** 2 < radius ** 2:
                rr.append(i)
                cc.append(j)
    return np.array(rr, dtype=np.int64), np.array(cc, dtype=np.int64)


def _line(r0, c0, r1, c1):
    """Integer Bresenham line from (r0, c0) to (r1, c1), both ends included."""
    r0, c0, r1, c1 = int(r0), int(c0), int(r1), int(c1)
    rr, cc = [], []
    dr, dc = abs(r1 - r0), abs(c1 - c0)
    sr = 1 if r1 >= r0 else -1
    sc = 1 if c1 >= c0 else -1
    steep = dr > dc
    if steep:
        err = dr // 2
        c = c0
        for r in range(r0, r1 + sr, sr):
            rr.append(r)
            cc.append(c)
            err -= dc
            if err < 0:
                c += sc
                err += dr
    else:
        err = dc // 2
        r = r0
        for c in range(c0, c1 + sc, sc):
            rr.append(r)
            cc.append(c)
            err -= dr
            if err < 0:
                r += sr
                err += dc
    return np.array(rr, dtype=np.int64), np.array(cc, dtype=np.int64)


def import_reference():
    """Return the reference ``wavetorch`` package, imported unmodified from
    the directory named by the WAVETORCH_REFERENCE environment variable (the
    directory that holds the ``wavetorch`` package)."""
    if not REFERENCE_ROOT or not os.path.isdir(os.path.join(REFERENCE_ROOT, "wavetorch")):
        raise RuntimeError("set WAVETORCH_REFERENCE to the directory holding the reference's "
                           "wavetorch package")
    if "wavetorch" in sys.modules and getattr(sys.modules["wavetorch"], "__file__", "").startswith(REFERENCE_ROOT):
        return sys.modules["wavetorch"]
    for name in ["librosa", "pandas", "seaborn", "matplotlib", "matplotlib.pyplot",
                 "matplotlib.animation", "matplotlib.colors", "matplotlib.gridspec",
                 "mpl_toolkits", "mpl_toolkits.axes_grid1",
                 "mpl_toolkits.axes_grid1.axes_divider", "yaml"]:
        if name not in sys.modules:
            _stub(name)
    sys.modules["mpl_toolkits.axes_grid1.axes_divider"].make_axes_locatable = lambda *a, **k: None
    sys.modules["mpl_toolkits.axes_grid1"].make_axes_locatable = lambda *a, **k: None
    try:
        import skimage  # noqa: F401
        import skimage.draw as _d
        if not hasattr(_d, "circle"):
            _d.circle = _circle
    except ImportError:
        sk = _stub("skimage")
        draw = _stub("skimage.draw", circle=_circle, line=_line)
        sk.draw = draw
    try:
        import sklearn.metrics  # noqa: F401
    except ImportError:
        # utils.py / train.py import confusion_matrix for their accuracy
        # reports (off the time-stepping path); machines without scikit-learn
        # get a stand-in that raises if it is ever called
        def _no_sklearn(*a, **k):
            raise RuntimeError("scikit-learn is not available")
        skl = _stub("sklearn")
        skl.metrics = _stub("sklearn.metrics", confusion_matrix=_no_sklearn)
    if not os.path.isdir(os.path.join(REFERENCE_ROOT, "wavetorch", "data")):
        # the reference's setup.py packages `wavetorch` alone, so a pip install
        # of it lacks the `wavetorch.data` subpackage (the vowel dataset
        # loader, librosa-based, off the time-stepping path) that its
        # __init__ imports: stand in for it as for the other data imports
        def _no_dataset(*a, **k):
            raise RuntimeError("the vowel dataset loader is not available")
        _stub("wavetorch.data", load_all_vowels=_no_dataset, select_vowel_sample=_no_dataset)
    if REFERENCE_ROOT not in sys.path:
        sys.path.insert(0, REFERENCE_ROOT)
    import wavetorch  # noqa: E402
    return wavetorch
