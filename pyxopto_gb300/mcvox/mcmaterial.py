"""Materials (re-exported from pyxopto_gb300.mcbase.mcmaterial)."""
from ..mcbase.mcmaterial import Material, Materials
