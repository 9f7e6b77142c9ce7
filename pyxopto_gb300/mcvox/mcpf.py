"""Scattering phase functions (re-exported from pyxopto_gb300.mcbase.mcpf)."""
from ..mcbase.mcpf import PfBase, Hg, Gk, Lut, Hg2, MHg, Pc, MPc, MGk, Gk2, Hga, HgDir, pf_fromdict
