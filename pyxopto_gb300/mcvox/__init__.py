"""Voxelized-medium simulator (drop-in for xopto.mcvox)."""
from . import mcdetector, mcpf, mcfluence, mctrace, mcoptions, mctypes, mcgeometry, mcsource, mcmaterial, mcsv, mcsurface
