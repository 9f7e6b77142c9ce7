"""Surface detectors (re-exported from pyxopto_gb300.mcbase.mcdetector)."""
from ..mcbase.mcdetector import (Axis, RadialAxis, SymmetricAxis, Detector, DetectorDefault,
                                 Total, Radial, TotalPl, RadialPl, Cartesian, CartesianPl,
                                 SymmetricX, TotalLut, TotalLutPl, Detectors)
from ..mcbase.mcdetector_probe import (LinearArray, LinearArrayPl, SixAroundOne, SixAroundOnePl,
                                       FiberArray, FiberArrayPl, FiberLutArray)
from ..mcbase.mcutil.lut import CollectionLut
