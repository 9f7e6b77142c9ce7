"""Run helpers of the voxelized simulator (xopto/mcvox/mcrun/mcrun.py:32-257):
the same run-until-weight/packets classes as the layered simulator; the
voxelized reference has no McRunHelper."""
from ..mcml.mcrun import (RunMinWeightTop, RunMinWeightBottom, RunMinWeightSpecular,  # noqa: F401
                          RunMinWeightTrace, RunMinPacketsTrace)

__all__ = ['RunMinWeightTop', 'RunMinWeightBottom', 'RunMinWeightSpecular', 'RunMinWeightTrace',
           'RunMinPacketsTrace']
