"""Sampling volume (xopto/mcvox/mcsv.py re-exports xopto/mcbase/mcsv.py)."""
from ..mcbase.mcsv import SamplingVolume, Axis  # noqa: F401
