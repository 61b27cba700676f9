"""mrhyde_gb300: GB300-native (sm_103a) implementation of MrHyDE's workset finite-element assembly path.

The compute path is libmrhyde_gb.so (hand-written CUDA behind the C ABI of include/mrhyde_gb300.h);
this package is its host-side mirror of the reference's AssemblyManager / SolverManager interface.
"""
from . import _lib
from .assembly import AssemblyManager, Problem
from .buildlib import build
from .solver import SolverManager, SolveResult

__all__ = ["AssemblyManager", "Problem", "SolverManager", "SolveResult", "build", "load"]


def load():
    """Build (if needed) and load libmrhyde_gb.so; raises if it cannot be loaded."""
    return _lib.lib()
