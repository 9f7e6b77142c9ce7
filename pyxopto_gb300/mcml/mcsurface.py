"""Layouts of the top and bottom sample surfaces of the layered simulator
(xopto/mcml/mcsurface): a Lambertian reflector and optical-fibre probe faces
(LinearArray, SixAroundOne, FiberArray) that change the refractive index and
critical angle of the boundary under each fibre core, cladding or cutout, or
reflect the packet from the probe's metal face.

Each layout packs its parameters as a float table appended to the simulator's
float lookup buffer (the layout of each table is documented with
McgbSurface in include/xopto_gb300.h).
"""
import numpy as np

from .. import _abi
from ..mcbase import mcutil
from ..mcbase.mcutil.fiber import MultimodeFiber, FiberLayout

TOP, BOTTOM, NONE = 'top', 'bottom', 'none'


def _n_sample(mc, location):
    return mc.layers[1].n if location == TOP else mc.layers[-2].n


def _transform_to_fiber(direction):
    d = np.asarray(direction, dtype=np.float64)
    adir = (d[0], d[1], abs(d[2]))
    return np.asarray(mcutil.transform_base(adir, (0.0, 0.0, 1.0)), dtype=np.float64)


class SurfaceLayoutBase:
    """A layout of the top or bottom sample surface
    (xopto/mcml/mcsurface/base.py:36-92)."""
    kind = _abi.SURFACE_NONE

    def __init__(self, location: str = NONE):
        if location not in (TOP, BOTTOM, NONE):
            raise ValueError('Surface layout location must be "none", "top" or "bottom"!')
        self._location = location

    def _set_location(self, location):
        if location not in (NONE, TOP, BOTTOM):
            raise ValueError('Surface layout location must be "none", "top" or "bottom"!')
        if location != self._location and self._location != NONE:
            raise RuntimeError('Surface layout cannot be changed!')
        self._location = str(location)

    location = property(lambda self: self._location, _set_location)

    def table(self, mc) -> np.ndarray:
        raise NotImplementedError

    def n_fibers(self) -> int:
        return 0

    def pack(self, mc, target: _abi.McgbSurface):
        data = np.asarray(self.table(mc), dtype=np.float32)
        target.kind = self.kind
        target.n_fibers = self.n_fibers()
        target.table_offset = mc.append_r_lut(data)
        target.table_size = data.size
        return target


class SurfaceLayoutAny(SurfaceLayoutBase):
    pass


class SurfaceLayoutDefault(SurfaceLayoutAny):
    """No layout: the plain boundary (xopto/mcml/mcsurface/base.py:110-196)."""

    def pack(self, mc, target):
        target.kind = _abi.SURFACE_NONE
        target.n_fibers = target.table_offset = target.table_size = 0
        return target

    def todict(self):
        return {'type': 'SurfaceLayoutDefault'}


class LambertianReflector(SurfaceLayoutAny):
    """Reflector of the given total reflectance; a fraction ``specular`` of
    the reflections is specular, the rest Lambertian
    (xopto/mcml/mcsurface/lambertian.py:31-196)."""
    kind = _abi.SURFACE_LAMBERTIAN

    def __init__(self, reflectance: float = 1.0, specular: float = 0.0):
        super().__init__()
        self._reflectance = min(max(float(reflectance), 0.0), 1.0)
        self._specular = min(max(float(specular), 0.0), 1.0)

    def _set_reflectance(self, v):
        self._reflectance = min(max(float(v), 0.0), 1.0)

    def _set_specular(self, v):
        self._specular = min(max(float(v), 0.0), 1.0)

    reflectance = property(lambda self: self._reflectance, _set_reflectance)
    specular = property(lambda self: self._specular, _set_specular)

    def table(self, mc):
        """lambertian.py:170-181.  The reference packs the attribute
        ``_specular``, which its constructor sets to 0 while the setter stores
        the fraction in ``_specular_fraction``; the kernel therefore always
        sees a specular fraction of 0, and so does this table."""
        return [self._reflectance, 0.0]

    def todict(self):
        return {'type': 'LambertianReflector', 'reflectance': self._reflectance,
                'specular': self._specular}


class LinearArray(SurfaceLayoutAny):
    """Probe face with a linear array of n identical fibres, optionally
    tilted, a rectangular cutout and a metal face of the given diameter and
    reflectivity (xopto/mcml/mcsurface/probe/lineararray.py:33-620)."""
    kind = _abi.SURFACE_LINEAR_ARRAY

    def __init__(self, fiber: MultimodeFiber, n=1, spacing: float = None,
                 orientation=(1.0, 0.0), diameter: float = 0.0, reflectivity: float = 0.0,
                 cutout=(0.0, 0.0), cutoutn=1.0, position=(0.0, 0.0), direction=(0.0, 0.0, 1.0)):
        super().__init__()
        if isinstance(fiber, LinearArray):
            la = fiber
            fiber, n, spacing, orientation = la.fiber, la.n, la.spacing, la.orientation
            diameter, reflectivity, cutout, cutoutn = la.diameter, la.reflectivity, la.cutout, la.cutoutn
            position, direction = la.position, la.direction
        self._fiber = fiber
        self._n = max(int(n), 1)
        self._spacing = float(fiber.dcladding if spacing is None else spacing)
        o = np.asarray(orientation, dtype=np.float64)
        self._orientation = o / np.linalg.norm(o)
        self._diameter = float(diameter)
        self._reflectivity = min(max(float(reflectivity), 0.0), 1.0)
        self._cutout = np.zeros((2,))
        self._cutout[:] = cutout
        self._cutout_n = float(cutoutn)
        self._position = np.zeros((2,))
        self._position[:] = position
        d = np.asarray(direction, dtype=np.float64)
        self._direction = d / np.linalg.norm(d)

    fiber = property(lambda self: self._fiber)
    n = property(lambda self: self._n)
    spacing = property(lambda self: self._spacing)
    orientation = property(lambda self: self._orientation)
    diameter = property(lambda self: self._diameter)
    reflectivity = property(lambda self: self._reflectivity)
    cutout = property(lambda self: self._cutout)
    cutoutn = property(lambda self: self._cutout_n)
    position = property(lambda self: self._position)
    direction = property(lambda self: self._direction)

    def n_fibers(self):
        return self._n

    def fiber_position(self, index: int):
        """Centre of fibre ``index`` (lineararray.py:fiber_position)."""
        if index >= self._n or index < -self._n:
            raise IndexError('The fiber index is out of valid range!')
        left = self._position - self._orientation * self._spacing * (self._n - 1) * 0.5
        return tuple(left + self._spacing * self._orientation * int(index))

    def table(self, mc):
        """lineararray.py:492-552."""
        n_sample = _n_sample(mc, self.location)
        f = self._fiber
        T = _transform_to_fiber(self._direction)
        C = mcutil.rotation_matrix_2d(self._orientation, [1.0, 0.0])
        return np.concatenate([
            T.ravel(), self._position, self.fiber_position(0), self._orientation * self._spacing,
            [0.25 * f.dcore ** 2, f.ncore, mcutil.cos_critical(n_sample, f.ncore),
             0.25 * f.dcladding ** 2, f.ncladding, mcutil.cos_critical(n_sample, f.ncladding),
             0.25 * self._diameter ** 2, self._reflectivity],
            C.ravel(),
            [self._cutout[0] * 0.5, self._cutout[1] * 0.5, self._cutout_n,
             mcutil.cos_critical(n_sample, self._cutout_n)]])

    def todict(self):
        return {'type': 'LinearArray', 'fiber': self._fiber.todict(), 'n': self._n,
                'spacing': self._spacing, 'orientation': self._orientation.tolist(),
                'diameter': self._diameter, 'reflectivity': self._reflectivity,
                'cutout': self._cutout.tolist(), 'cutoutn': self._cutout_n,
                'position': self._position.tolist(), 'direction': self._direction.tolist()}


class SixAroundOne(SurfaceLayoutAny):
    """Probe face with a central fibre surrounded by six, a circular cutout
    and a metal face (xopto/mcml/mcsurface/probe/sixaroundone.py:33-600)."""
    kind = _abi.SURFACE_SIX_AROUND_ONE

    def __init__(self, fiber: MultimodeFiber, spacing: float = None, diameter: float = 0.0,
                 reflectivity: float = 1.0, cutout: float = 0.0, cutoutn: float = 1.0,
                 position=(0.0, 0.0), direction=(0.0, 0.0, 1.0)):
        super().__init__()
        if isinstance(fiber, SixAroundOne):
            o = fiber
            fiber, spacing, diameter, reflectivity = o.fiber, o.spacing, o.diameter, o.reflectivity
            cutout, cutoutn, position, direction = o.cutout, o.cutoutn, o.position, o.direction
        self._fiber = fiber
        self._spacing = float(fiber.dcladding if spacing is None else spacing)
        self._diameter = float(diameter)
        self._reflectivity = min(max(float(reflectivity), 0.0), 1.0)
        self._cutout = float(cutout)
        self._cutout_n = float(cutoutn)
        self._position = np.zeros((2,))
        self._position[:] = position
        d = np.asarray(direction, dtype=np.float64)
        self._direction = d / np.linalg.norm(d)

    fiber = property(lambda self: self._fiber)
    spacing = property(lambda self: self._spacing)
    diameter = property(lambda self: self._diameter)
    reflectivity = property(lambda self: self._reflectivity)
    cutout = property(lambda self: self._cutout)
    cutoutn = property(lambda self: self._cutout_n)
    position = property(lambda self: self._position)
    direction = property(lambda self: self._direction)

    def table(self, mc):
        """sixaroundone.py:495-545."""
        n_sample = _n_sample(mc, self.location)
        f = self._fiber
        T = _transform_to_fiber(self._direction)
        return np.concatenate([
            T.ravel(), self._position,
            [self._spacing, 0.25 * f.dcore ** 2, f.ncore, mcutil.cos_critical(n_sample, f.ncore),
             0.25 * f.dcladding ** 2, f.ncladding, mcutil.cos_critical(n_sample, f.ncladding),
             0.25 * self._cutout ** 2, self._cutout_n, mcutil.cos_critical(n_sample, self._cutout_n),
             0.25 * self._diameter ** 2, self._reflectivity]])

    def todict(self):
        return {'type': 'SixAroundOne', 'fiber': self._fiber.todict(), 'spacing': self._spacing,
                'diameter': self._diameter, 'reflectivity': self._reflectivity,
                'cutout': self._cutout, 'cutoutn': self._cutout_n,
                'position': self._position.tolist(), 'direction': self._direction.tolist()}


class FiberArray(SurfaceLayoutAny):
    """Probe face with an arbitrary array of fibres (FiberLayout) and a metal
    face (xopto/mcml/mcsurface/probe/fiberarray.py:33-470)."""
    kind = _abi.SURFACE_FIBER_ARRAY

    def __init__(self, fibers, diameter: float = 0.0, reflectivity: float = 0.0,
                 position=(0.0, 0.0)):
        super().__init__()
        if isinstance(fibers, FiberArray):
            o = fibers
            fibers, diameter, reflectivity, position = o.fibers, o.diameter, o.reflectivity, o.position
        self._fibers = [FiberLayout(f) for f in fibers]
        self._diameter = float(diameter)
        self._reflectivity = min(max(float(reflectivity), 0.0), 1.0)
        self._position = np.zeros((2,))
        self._position[:] = position

    fibers = property(lambda self: self._fibers)
    diameter = property(lambda self: self._diameter)
    reflectivity = property(lambda self: self._reflectivity)
    position = property(lambda self: self._position)

    def n_fibers(self):
        return len(self._fibers)

    def table(self, mc):
        """fiberarray.py:330-390."""
        n_sample = _n_sample(mc, self.location)
        # The reference assigns target.probe_reflectivity, a name that its
        # ctypes structure does not have (the field is "reflectivity"), so
        # the kernel always sees a probe reflectivity of 0; so does this table.
        out = [self._position[0], self._position[1], 0.25 * self._diameter ** 2, 0.0]
        for fl in self._fibers:
            f = fl.fiber
            out.extend(_transform_to_fiber(fl.direction).ravel())
            out.extend([fl.position[0], fl.position[1]])
            out.extend([0.25 * f.dcladding ** 2, f.ncladding, mcutil.cos_critical(n_sample, f.ncladding),
                        0.25 * f.dcore ** 2, f.ncore, mcutil.cos_critical(n_sample, f.ncore)])
        return np.asarray(out, dtype=np.float64)

    def todict(self):
        return {'type': 'FiberArray', 'fibers': [f.todict() for f in self._fibers],
                'diameter': self._diameter, 'reflectivity': self._reflectivity,
                'position': self._position.tolist()}


class SurfaceLayouts:
    """Layouts of the top and bottom sample surfaces
    (xopto/mcml/mcsurface/base.py:199-426)."""

    def __init__(self, top=None, bottom=None):
        if isinstance(top, SurfaceLayouts):
            top, bottom = top.top, top.bottom
        self._top = top if top is not None else SurfaceLayoutDefault()
        self._bottom = bottom if bottom is not None else SurfaceLayoutDefault()
        if not isinstance(self._top, SurfaceLayoutDefault):
            self._top.location = TOP
        if not isinstance(self._bottom, SurfaceLayoutDefault):
            self._bottom.location = BOTTOM

    top = property(lambda self: self._top)
    bottom = property(lambda self: self._bottom)

    def pack(self, mc, cfg):
        self._top.pack(mc, cfg.surface_top)
        self._bottom.pack(mc, cfg.surface_bottom)

    def todict(self):
        return {'type': 'SurfaceLayouts', 'top': self._top.todict(), 'bottom': self._bottom.todict()}

    def __str__(self):
        return 'SurfaceLayouts(top={}, bottom={})'.format(self._top, self._bottom)

    __repr__ = __str__
