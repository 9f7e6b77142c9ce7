"""Fourier transforms (xopto/mcml/mcutil re-exports xopto/mcbase/mcutil/fourier.py)."""
from ...mcbase.mcutil.fourier import discreteSimpson  # noqa: F401
