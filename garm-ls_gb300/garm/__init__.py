"""GB300-native GARM-LS per-timestep grid pipeline (Python harness over libgarm.so)."""
from . import capi, scenes  # noqa: F401
from .capi import Simulation, default_config, grid_desc, load  # noqa: F401
