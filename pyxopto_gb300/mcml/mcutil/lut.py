"""Look-up tables (xopto/mcml/mcutil/lut.py re-exports xopto/mcbase/mcutil/lut.py)."""
from ...mcbase.mcutil.lut import LinearLut, EmissionLut, CollectionLut  # noqa: F401
