"""GB300-native coupled SPH-DEM seepage-flow substep (sph_seepage_flows drop-in)."""

from . import params, scenes  # noqa: F401

__version__ = "0.1.0"
