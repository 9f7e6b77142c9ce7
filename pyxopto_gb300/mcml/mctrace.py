"""Packet trace (re-exported from pyxopto_gb300.mcbase.mctrace)."""
from ..mcbase.mctrace import Trace
