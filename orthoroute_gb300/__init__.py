"""orthoroute_gb300 — GB300-native PathFinder negotiated-congestion routing.

A drop-in for the hot path of OrthoRoute's ``PathFinderRouter``
(orthoroute/algorithms/manhattan/unified_pathfinder.py): the lattice CSR,
the per-net ROI shortest path, the present/history cost update, the overuse
and barrel tallies, and backtrace / rip-up run as hand-written sm_103a CUDA
kernels behind the C ABI in ``include/orthoroute_gb300.h``.
"""
from .lattice import Lattice, default_layer_dirs

__all__ = ["Lattice", "default_layer_dirs"]
__version__ = "0.1.0"
