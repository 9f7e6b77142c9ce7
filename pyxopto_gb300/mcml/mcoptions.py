"""Simulator options (re-exported from pyxopto_gb300.mcbase.mcoptions)."""
from ..mcbase.mcoptions import *
