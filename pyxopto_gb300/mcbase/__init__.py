"""Plugins shared by the layered and voxelized simulators."""
