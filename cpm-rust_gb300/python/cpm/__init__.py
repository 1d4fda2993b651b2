"""Cellular Potts Model simulator on GB300: a drop-in for the Python API of
DebajyotiS/cpm-rust (`cpm.CPM`, `cells_for_density`, the warning classes),
running the Monte Carlo hot loop as sm_103a kernels through libcpm_gpu.so."""

from .model import CPM, Server, run_many
from .parameters import cells_for_density
from .warnings import CPMInitializationWarning, CPMLowResolutionWarning

__all__ = [
    "CPM",
    "run_many",
    "Server",
    "cells_for_density",
    "CPMInitializationWarning",
    "CPMLowResolutionWarning",
]
