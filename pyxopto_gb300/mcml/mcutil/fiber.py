"""Optical fibres (xopto/mcml/mcutil/fiber.py re-exports xopto/mcbase/mcutil/fiber.py)."""
from ...mcbase.mcutil.fiber import *  # noqa: F401,F403
from ...mcbase.mcutil.fiber import MultimodeFiber, FiberLayout, MultimodeFiberLut  # noqa: F401
