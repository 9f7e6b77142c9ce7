"""Surface detectors (re-exported from pyxopto_gb300.mcbase.mcdetector).
The voxelized simulator has no TotalLutPl and no FiberLutArray in the
reference (xopto/mcvox/mcdetector/__init__.py)."""
from ..mcbase.mcdetector import (Axis, RadialAxis, SymmetricAxis, Detector, DetectorDefault,
                                 Total, Radial, TotalPl, RadialPl, Cartesian, CartesianPl,
                                 SymmetricX, TotalLut, Detectors)
from ..mcbase.mcdetector_probe import (LinearArray, LinearArrayPl, SixAroundOne, SixAroundOnePl,
                                       FiberArray, FiberArrayPl)
from ..mcbase.mcutil.lut import CollectionLut
