"""GB300-native first-arrival traveltime engine (fast-sweeping eikonal solver
of phbastosa/SeisFAT2D, rebuilt for sm_103a).

The compute path is ``libseisfat2d.so`` (hand-written CUDA behind a C ABI,
``include/seisfat2d.h``); this package is its Python mirror.
"""
from .engine import Engine, EngineError  # noqa: F401

__all__ = ["Engine", "EngineError"]
