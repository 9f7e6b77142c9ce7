"""Interpolation (xopto/mcml/mcutil re-exports xopto/mcbase/mcutil/interp.py)."""
from ...mcbase.mcutil.interp import interp2  # noqa: F401
