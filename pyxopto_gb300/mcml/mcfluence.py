"""Fluence accumulators (re-exported from pyxopto_gb300.mcbase.mcfluence)."""
from ..mcbase.mcfluence import Fluence
from ..mcbase.mcutil import Axis
FLUENCE_TYPE = Fluence
