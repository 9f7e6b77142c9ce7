"""Utilities of the layered simulator (the items of pyxopto_gb300.mcbase.mcutil,
as xopto/mcml/mcutil re-exports xopto/mcbase/mcutil)."""
from ...mcbase.mcutil import *  # noqa: F401,F403
from ...mcbase.mcutil import Axis, RadialAxis  # noqa: F401
from . import fiber, lut, fourier, interp  # noqa: F401
