"""GB300-native per-timestep fluid update (drop-in for the step API of
mdushkoff/Probabilistic_Fluid_Simulation, includes/fluid.hpp)."""
from . import synthetic  # noqa: F401

__all__ = ["synthetic", "fluid", "build"]
