"""GB300-native BSAM adaptive FAS V-cycle: host side of the drop-in.

The reference (BSAM-in-MATLAB) keeps problem definition, options, tagging,
Berger-Rigoutsos clustering and the hierarchy build on the host and spends
its time in ``ebSolveCycles``.  This package mirrors that host side in
Python (same entry-point names, option names and error identifiers) and
sends every ``ebSolveCycles`` to the CUDA library ``libbsam_dev.so``
through its C-ABI (``include/bsam_dev.h``).  There is no CPU solve path.
"""
from .options import ebOptions, ebtOptions, Options
from .problem import ebProblem, ebtProblem
from .solve import ebSolve, ebtSolve, ebSolveCycles, ebtSolveCycles, build_hierarchy, error_norms, ebSample, ebtSample
from .treecheck import ebtTreeCheck
from .ddsolve import ddGeometry, ddProblem, ddSolve, ddErrorInside, ddToUniform
from . import hierarchy, tagcluster, flat

__all__ = ['ebOptions', 'ebtOptions', 'Options', 'ebProblem', 'ebtProblem', 'ebSolve', 'ebtSolve',
           'ebSolveCycles', 'ebtSolveCycles', 'build_hierarchy', 'error_norms', 'ebSample', 'ebtSample', 'hierarchy', 'tagcluster',
           'flat', 'ddGeometry', 'ddProblem', 'ddSolve', 'ddErrorInside', 'ddToUniform', 'ebtTreeCheck']
