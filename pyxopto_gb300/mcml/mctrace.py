"""Packet trace and trace filter (re-exported from pyxopto_gb300.mcbase.mctrace)."""
from ..mcbase.mctrace import *  # noqa: F401,F403
from ..mcbase.mctrace import Trace, Filter  # noqa: F401
