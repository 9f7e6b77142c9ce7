"""Layered-medium simulator (drop-in for xopto.mcml)."""
from . import mcdetector, mcpf, mcfluence, mctrace, mcoptions, mctypes, mclayer, mcsource, mcsurface, mcsv
