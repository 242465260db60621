"""Model files (wavetorch/io.py:13-87): the same dictionary layout and
state_dict keys, so files written by either implementation load in both."""
from __future__ import annotations

import copy
import os

import torch

from . import geom
from .cell import WaveCell
from .probe import WaveIntensityProbe
from .rnn import WaveRNN
from .source import WaveSource
from .utils import set_dtype


def save_model(model, name, savedir='./study/', history=None, history_geom_state=None, cfg=None,
               verbose=True):
    """Save the model state and history to ``savedir + name + '.pt'``."""
    path = savedir + name + '.pt'
    if not os.path.exists(savedir):
        os.makedirs(savedir)
    if history_geom_state is None:
        history_geom_state = [model.cell.geom.state_reconstruction_args()]
    data = {'model_geom_class_str': model.cell.geom.__class__.__name__,
            'model_state': model.state_dict(),
            'history': history,
            'history_geom_state': history_geom_state,
            'cfg': cfg}
    if verbose:
        print("Saving model to %s" % path)
    torch.save(data, path)


def new_geometry(class_str, state):
    cls = getattr(geom, class_str)
    return cls(**copy.deepcopy(state))


def load_model(str_filename, which_iteration=-1):
    """Rebuild (model, history, history_geom_state, cfg) from a saved file."""
    print("Loading model from %s" % str_filename)
    data = torch.load(str_filename, weights_only=False)
    set_dtype(data['cfg']['dtype'])
    new_geom = new_geometry(data['model_geom_class_str'], data['history_geom_state'][which_iteration])
    state = copy.deepcopy(data['model_state'])
    # probe / source coordinates come back from the state_dict keys
    px = [state[k].item() for k in state if 'probes' in k and 'x' in k]
    py = [state[k].item() for k in state if 'probes' in k and 'y' in k]
    sx = [state[k].item() for k in state if 'sources' in k and 'x' in k]
    sy = [state[k].item() for k in state if 'sources' in k and 'y' in k]
    probes = [WaveIntensityProbe(x, y) for x, y in zip(px, py)]
    sources = [WaveSource(x, y) for x, y in zip(sx, sy)]
    cell = WaveCell(state['cell.dt'].item(), new_geom)
    model = WaveRNN(cell, sources, probes)
    model.eval()
    return model, data['history'], data['history_geom_state'], data['cfg']
