"""Surface layouts of the voxelized simulator (xopto/mcvox/mcsurface).

The classes are those of the layered simulator, so configurations import
and round-trip.  None of the reference's voxelized layouts builds into its
kernel, so ``mcvox.Mc`` accepts only the default (empty) layouts:
  - LambertianReflector and SixAroundOne define a handler with a critical
    cosine argument that the voxel boundary does not pass
    (xopto/mcvox/mcsurface/lambertian.py:79-80, probe/sixaroundone.py:143-144
    against xopto/mcvox/kernel/mcvox.template.c:337,347);
  - LinearArray transforms an undeclared variable ``cutout_pos``
    (probe/lineararray.py:196);
  - FiberArray's handler takes no ``n2`` but assigns it
    (probe/fiberarray.py:126-127).
"""
from ..mcml.mcsurface import (SurfaceLayoutBase, SurfaceLayoutAny, SurfaceLayoutDefault,  # noqa: F401
                              LambertianReflector, LinearArray, SixAroundOne, FiberArray,
                              SurfaceLayouts)


def check_supported(surface):
    """Raises ValueError unless every layout of ``surface`` is the default."""
    if surface is None:
        return
    layouts = (surface.top, surface.bottom) if isinstance(surface, SurfaceLayouts) else (surface,)
    for layout in layouts:
        if layout is not None and not isinstance(layout, SurfaceLayoutDefault):
            raise ValueError(
                "Surface layout {} is not available for voxelized media: the reference's "
                "voxelized surface layouts do not build into its kernel.".format(type(layout).__name__))
