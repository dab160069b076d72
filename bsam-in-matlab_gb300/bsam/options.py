"""Solver options, mirroring the reference's name-value option parsers.

``ebOptions`` follows ``EllipticBSAM/src/ebOptions.m:44-73`` (same names,
same defaults, same normalisation of ``BaseCells`` and ``GhostInterp``);
``ebtOptions`` is the identical tree-variant parser
(``EllipticBSAMTree/src/ebtOptions.m``).  Two options are new and have no
counterpart in the reference:

  Device     CUDA device ordinal that runs the solve path (default 0).  The
             solve path has no CPU implementation: a missing CUDA library is
             an error.
  Precision  'fp64' (default; the drop-in, identical arithmetic to the
             reference) or 'mixed' (FP32 smoothing / ghost fill /
             prolongation inside an FP64 defect-correction loop).
"""
from __future__ import annotations

import copy

_DEFAULTS = {
    'BaseCells': [64, 64],
    'MaxLevels': 1,
    'CoarsestCells': 16,
    'GhostInterp': 'qif',
    'MassCorrection': True,
    'NPre': 3,
    'NPost': 3,
    'Omega': 1.0,
    'MaxVCycles': 60,
    'RelTol': 1e-9,
    'Indicator': 'ulap',
    'TagFunction': None,
    'TagThreshold': 1e-3,
    'TagBuffer': 2,
    'MinBoxWidth': 4,
    'MinFillRatio': 0.70,
    'Verbose': 1,
    'InitialGuess': None,
    'MeanZero': 'auto',
    'SourceQuad': 1,
    # device-path options (new)
    'Device': 0,
    'Precision': 'fp64',
}


class Options(dict):
    """Attribute-access dict so host code reads like ``opts.RelTol``."""

    def __getattr__(self, name):
        try:
            return self[name]
        except KeyError as e:
            raise AttributeError(name) from e

    def __setattr__(self, name, value):
        self[name] = value

    def copy(self):
        return Options(copy.copy(dict(self)))


def _parse(args, kwargs, known):
    """Name-value parsing like MATLAB's inputParser (case-insensitive names)."""
    if len(args) % 2:
        raise ValueError('eb_options:pairs: options must be name-value pairs')
    pairs = list(zip(args[0::2], args[1::2])) + list(kwargs.items())
    lower = {k.lower(): k for k in known}
    out = Options(copy.deepcopy(known))
    for name, val in pairs:
        key = lower.get(str(name).lower())
        if key is None:
            raise ValueError(f"eb_options:unknown: '{name}' is not a recognised option")
        out[key] = val
    return out


def ebOptions(*args, **kwargs) -> Options:
    """Parse elliptic solver options (``ebOptions.m:44-73``)."""
    if len(args) == 1 and isinstance(args[0], dict) and not kwargs:
        base = Options(copy.deepcopy(_DEFAULTS))
        base.update(args[0])
        opts = base
    else:
        opts = _parse(args, kwargs, _DEFAULTS)
    bc = opts['BaseCells']
    if isinstance(bc, (int, float)):
        bc = [bc, bc]
    bc = [int(round(v)) for v in list(bc)]
    if len(bc) == 1:
        bc = [bc[0], bc[0]]
    opts['BaseCells'] = bc
    opts['GhostInterp'] = str(opts['GhostInterp']).lower()
    if opts['GhostInterp'] not in ('qif', 'lif'):
        raise ValueError('eb_options:ghost: GhostInterp must be qif or lif')
    opts['Precision'] = str(opts['Precision']).lower()
    if opts['Precision'] not in ('fp64', 'mixed'):
        raise ValueError("eb_options:precision: Precision must be 'fp64' or 'mixed'")
    return opts


def ebtOptions(*args, **kwargs) -> Options:
    """``ebtOptions`` (``EllipticBSAMTree/src/ebtOptions.m``): the same
    options; its errors carry the tree identifiers (``ebt_options:*``)."""
    try:
        return ebOptions(*args, **kwargs)
    except ValueError as e:
        m = str(e)
        if m.startswith('eb_options:'):
            raise ValueError('ebt_' + m[3:]) from None
        raise
