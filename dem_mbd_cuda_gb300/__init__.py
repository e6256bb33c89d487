"""GB300-native DEM step engine (drop-in for the reference's CudaDemSolver)."""
from .scene import Mech, Scene  # noqa: F401
