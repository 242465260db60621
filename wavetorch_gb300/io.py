"""Model files in the reference's format (wavetorch/io.py:13-87).

A model file is one ``torch.save`` of a dictionary whose keys the reference
reads by name: ``model_geom_class_str`` (the geometry's class name),
``model_state`` (the WaveRNN ``state_dict``), ``history``,
``history_geom_state`` (constructor arguments of the geometry, one entry per
saved iteration) and ``cfg`` (whose ``dtype`` entry selects float32/float64).
Files written here add one key the reference never reads, ``probe_kinds``,
so a reload keeps amplitude probes apart from intensity probes; files
without it (every file the reference writes) get intensity probes, which is
what the reference's loader builds.

Sources and probes are rebuilt from the ``sources.<i>.x`` / ``probes.<i>.y``
entries of the state dict, in module order ``i``.  A source entry holding
several cells (a line source) comes back as a multi-cell
:class:`~wavetorch_gb300.source.WaveSource` over the same cells.
"""
from __future__ import annotations

import copy
import os
import re

import torch

from . import geom as _geom
from .cell import WaveCell
from .probe import WaveIntensityProbe, WaveProbe
from .rnn import WaveRNN
from .source import WaveSource
from .utils import set_dtype

_MODULE_KEY = re.compile(r"^(sources|probes)\.(\d+)\.(x|y)$")
_PROBE_CLASSES = {"WaveProbe": WaveProbe, "WaveIntensityProbe": WaveIntensityProbe}


def save_model(model, name, savedir='./study/', history=None, history_geom_state=None, cfg=None,
               verbose=True):
    """Write ``savedir + name + '.pt'`` (the reference's file layout)."""
    os.makedirs(savedir, exist_ok=True)
    target = savedir + name + '.pt'
    geom_hist = history_geom_state
    if geom_hist is None:
        geom_hist = [model.cell.geom.state_reconstruction_args()]
    payload = dict(
        model_geom_class_str=type(model.cell.geom).__name__,
        model_state=model.state_dict(),
        history=history,
        history_geom_state=geom_hist,
        cfg=cfg,
        probe_kinds=[type(p).__name__ for p in model.probes],
    )
    if verbose:
        print(f"Saving model to {target}")
    torch.save(payload, target)


def new_geometry(class_str, state):
    """Construct geometry class ``class_str`` from saved constructor arguments."""
    try:
        cls = getattr(_geom, class_str)
    except AttributeError:
        raise ValueError(f"unknown geometry class {class_str!r} in model file") from None
    return cls(**copy.deepcopy(state))


def _coords(state):
    """{'sources': {i: (xs, ys)}, 'probes': {i: (xs, ys)}} from the state dict."""
    found = {"sources": {}, "probes": {}}
    for key, val in state.items():
        m = _MODULE_KEY.match(key)
        if m is None:
            continue
        group, idx, axis = m.group(1), int(m.group(2)), m.group(3)
        cells = torch.as_tensor(val).reshape(-1).tolist()
        found[group].setdefault(idx, {})[axis] = cells
    out = {}
    for group, entries in found.items():
        pairs = []
        for idx in sorted(entries):
            e = entries[idx]
            if "x" not in e or "y" not in e or len(e["x"]) != len(e["y"]):
                raise ValueError(f"model file: {group}.{idx} needs x and y of equal length")
            pairs.append((e["x"], e["y"]))
        out[group] = pairs
    return out


def _point_or_cells(xs, ys):
    return (xs[0], ys[0]) if len(xs) == 1 else (xs, ys)


def load_model(str_filename, which_iteration=-1):
    """Rebuild ``(model, history, history_geom_state, cfg)`` from a model file."""
    print(f"Loading model from {str_filename}")
    data = torch.load(str_filename, weights_only=False)
    set_dtype(data['cfg']['dtype'])
    geometry = new_geometry(data['model_geom_class_str'],
                            data['history_geom_state'][which_iteration])
    state = data['model_state']
    coords = _coords(state)
    kinds = data.get('probe_kinds') or ['WaveIntensityProbe'] * len(coords['probes'])
    if len(kinds) != len(coords['probes']):
        raise ValueError("model file: probe_kinds does not match the probes in model_state")
    probes = [_PROBE_CLASSES[k](*_point_or_cells(xs, ys)) for k, (xs, ys) in zip(kinds, coords['probes'])]
    sources = [WaveSource(*_point_or_cells(xs, ys)) for xs, ys in coords['sources']]
    cell = WaveCell(torch.as_tensor(state['cell.dt']).item(), geometry)
    model = WaveRNN(cell, sources, probes)
    model.eval()
    return model, data['history'], data['history_geom_state'], data['cfg']
