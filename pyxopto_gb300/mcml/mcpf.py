"""Scattering phase functions (re-exported from pyxopto_gb300.mcbase.mcpf)."""
from ..mcbase.mcpf import PfBase, Hg, Gk, Lut, pf_fromdict
