"""Data types (re-exported from pyxopto_gb300.mcbase.mctypes)."""
from ..mcbase.mctypes import *
