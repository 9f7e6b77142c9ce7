"""Surface detectors (re-exported from pyxopto_gb300.mcbase.mcdetector)."""
from ..mcbase.mcdetector import (Axis, RadialAxis, Detector, DetectorDefault, Total, Radial,
                                 TotalPl, RadialPl,
                                 Detectors)
