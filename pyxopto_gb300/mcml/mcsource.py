"""Photon packet sources of the layered simulator: Line, GaussianBeam,
UniformBeam, IsotropicPoint and the fibre sources UniformFiberNI,
LambertianFiberNI, UniformFiber and LambertianFiber
(xopto/mcml/mcsource/line.py, gaussianbeam.py, uniformbeam.py, point.py,
fiberni.py, fiber.py)."""
import numpy as np

from .. import _abi
from ..mcbase import mcutil
from ..mcbase.mcutil.fiber import MultimodeFiber


def _unit(v):
    v = np.asarray(v, dtype=np.float64).copy()
    n = np.linalg.norm(v)
    if n == 0.0:
        raise ValueError('The norm/length of the propagation direction vector must not be 0!')
    return v / n


class Source:
    def todict(self):
        raise NotImplementedError


class Line(Source):
    """Infinitely thin beam (xopto/mcml/mcsource/line.py:31-237)."""

    def __init__(self, position=(0.0, 0.0, 0.0), direction=(0.0, 0.0, 1.0)):
        if isinstance(position, Line):
            position, direction = position.position, position.direction
        self._position = np.zeros((3,))
        self._position[:] = position
        self._direction = _unit(direction)

    def _set_position(self, p):
        self._position[:] = p

    def _set_direction(self, d):
        self._direction = _unit(d)

    position = property(lambda self: self._position, _set_position)
    direction = property(lambda self: self._direction, _set_direction)

    def pack(self, mc, target: _abi.McgbSource):
        """line.py:181-228: move to the surface, refract, specular reflectance."""
        t = -self._position[2] / self._direction[2]
        position = self._position + self._direction * t
        position[2] = 0.0
        n1, n2 = mc.layers[0].n, mc.layers[1].n
        reflectance = mcutil.reflectance(n1, n2, self._direction[2])
        if reflectance >= 1.0:
            raise ValueError('The line source is fully reflected from the top surface of the sample!')
        sin1 = (1.0 - self._direction[2] ** 2) ** 0.5
        sin2 = max(min(n1 * sin1 / n2, 1.0), -1.0)
        d = (self._direction[0] * n1 / n2, self._direction[1] * n1 / n2,
             np.sign(self._direction[2]) * (1 - sin2 ** 2) ** 0.5)
        target.kind = _abi.SRC_LINE
        target.position[:] = [float(v) for v in position]
        target.direction[:] = [float(v) for v in d]
        target.direction_reflected[:] = [self._direction[0], self._direction[1], -self._direction[2]]
        target.reflectance = reflectance
        return target

    def todict(self):
        return {'type': 'Line', 'position': self._position.tolist(),
                'direction': self._direction.tolist()}

    def __str__(self):
        return 'Line(position=({}, {}, {}), direction=({}, {}, {}))'.format(
            *self._position, *self._direction)

    __repr__ = __str__


class GaussianBeam(Source):
    """Collimated Gaussian beam (xopto/mcml/mcsource/gaussianbeam.py:33-374)."""

    def __init__(self, sigma, clip=5.0, position=(0.0, 0.0, 0.0), direction=(0.0, 0.0, 1.0)):
        if isinstance(sigma, GaussianBeam):
            o = sigma
            sigma, clip, position, direction = o.sigma, o.clip, o.position, o.direction
        self._sigma = np.zeros((2,))
        self._sigma[:] = sigma
        if np.any(self._sigma < 0.0):
            raise ValueError('Beam diameter/sigma must not be negative!')
        self._clip = float(clip)
        if self._clip < 0.0:
            raise ValueError('Clip diameter/sigma must be greater than zero!')
        self._position = np.zeros((3,))
        self._position[:] = position
        self._direction = _unit(direction)

    sigma = property(lambda self: self._sigma)
    clip = property(lambda self: self._clip)
    position = property(lambda self: self._position)
    direction = property(lambda self: self._direction)

    @staticmethod
    def fwhm2sigma(fwhm: float) -> float:
        return fwhm / (8.0 * np.log(2.0)) ** 0.5

    @staticmethod
    def sigma2fwhm(sigma: float) -> float:
        return sigma * (8.0 * np.log(2.0)) ** 0.5

    def pack(self, mc, target: _abi.McgbSource):
        """gaussianbeam.py:300-362."""
        k = (0.0 - self._position[2]) / self._direction[2]
        position = self._position + k * self._direction
        position[2] = 0.0
        n1, n2 = mc.layers[0].n, mc.layers[1].n
        direction = mcutil.refract(self._direction, (0.0, 0.0, 1.0), n1, n2)
        reflectance = mcutil.reflectance(n1, n2, abs(self._direction[-1]))
        T = mcutil.transform_base((0.0, 0.0, 1.0), self._direction)
        target.kind = _abi.SRC_GAUSSIAN_BEAM
        target.transformation[:] = [float(v) for v in np.asarray(T).ravel()]
        target.position[:] = [float(v) for v in position]
        target.direction[:] = [float(v) for v in direction]
        target.sigma[:] = [float(v) for v in self._sigma]
        target.clip = self._clip
        target.reflectance = reflectance
        return target

    def todict(self):
        return {'type': 'GaussianBeam', 'sigma': self._sigma.tolist(), 'clip': self._clip,
                'position': self._position.tolist(), 'direction': self._direction.tolist()}

    def __str__(self):
        return 'GaussianBeam(sigma=({}, {}), clip={})'.format(*self._sigma, self._clip)

    __repr__ = __str__


class UniformFiberNI(Source):
    """Optical fibre source with normal incidence: packets start uniformly
    over the core and uniformly in solid angle within the acceptance cone
    (xopto/mcml/mcsource/fiberni.py:180-438)."""

    def __init__(self, fiber: MultimodeFiber, position=(0.0, 0.0, 0.0)):
        if isinstance(fiber, UniformFiberNI):
            fiber, position = fiber.fiber, fiber.position
        self._fiber = fiber
        self._position = np.zeros((3,))
        self._set_position(position)

    def _set_fiber(self, fib):
        self._fiber = fib

    def _set_position(self, p):
        self._position[:] = p
        self._position[2] = 0.0

    fiber = property(lambda self: self._fiber, _set_fiber, None, 'Multimode optical fiber.')
    position = property(lambda self: self._position, _set_position, None, 'Source position.')

    def update(self, other):
        if isinstance(other, UniformFiberNI):
            self.fiber, self.position = other.fiber, other.position
        elif isinstance(other, dict):
            self.fiber = other.get('fiber', self.fiber)
            self.position = other.get('position', self.position)

    def pack(self, mc, target: _abi.McgbSource):
        """fiberni.py:383-412: core radius, acceptance cosine in air,
        core refractive index."""
        target.kind = _abi.SRC_UNIFORM_FIBER_NI
        target.position[:] = [float(v) for v in self._position]
        target.sigma[0] = self._fiber.dcore * 0.5
        target.sigma[1] = (1.0 - self._fiber.na ** 2) ** 0.5
        target.clip = self._fiber.ncore
        return target

    def todict(self):
        return {'type': 'UniformFiberNI', 'fiber': self._fiber.todict(),
                'position': self._position.tolist()}

    def __str__(self):
        return 'UniformFiberNI(fiber={}, position=({}, {}, {}))'.format(self._fiber, *self._position)

    __repr__ = __str__


class LambertianFiberNI(UniformFiberNI):
    """Fibre source with normal incidence and a Lambertian angular
    distribution, sin(theta) = sqrt(u)*NA (xopto/mcml/mcsource/fiberni.py:422-578)."""

    def pack(self, mc, target: _abi.McgbSource):
        """fiberni.py:562-573: core radius, NA, core refractive index."""
        UniformFiberNI.pack(self, mc, target)
        target.kind = _abi.SRC_LAMBERTIAN_FIBER_NI
        target.sigma[1] = self._fiber.na
        return target

    def todict(self):
        d = UniformFiberNI.todict(self)
        d['type'] = 'LambertianFiberNI'
        return d

    def __str__(self):
        return 'LambertianFiberNI(fiber={}, position=({}, {}, {}))'.format(self._fiber, *self._position)

    __repr__ = __str__


class UniformFiber(Source):
    """Fibre source tilted along ``direction`` (z component positive):
    packets start uniformly over the core projected onto the surface,
    uniformly in solid angle within the acceptance cone around the fibre axis
    (xopto/mcml/mcsource/fiber.py:190-496)."""
    _kind = _abi.SRC_UNIFORM_FIBER

    def __init__(self, fiber: MultimodeFiber, position=(0.0, 0.0, 0.0), direction=(0.0, 0.0, 1.0)):
        if isinstance(fiber, UniformFiber):
            fiber, position, direction = fiber.fiber, fiber.position, fiber.direction
        self._fiber = fiber
        self._position = np.zeros((3,))
        self._direction = np.zeros((3,))
        self._set_position(position)
        self._set_direction(direction)

    def _set_fiber(self, fib):
        self._fiber = fib

    def _set_position(self, p):
        self._position[:] = p
        self._position[2] = 0.0

    def _set_direction(self, d):
        d = _unit(d)
        if d[-1] <= 0.0:
            raise ValueError('Z component of the propagation direction must be positive!')
        self._direction[:] = d

    fiber = property(lambda self: self._fiber, _set_fiber, None, 'Multimode optical fiber.')
    position = property(lambda self: self._position, _set_position, None, 'Source position.')
    direction = property(lambda self: self._direction, _set_direction, None, 'Source direction.')

    def _angular(self):
        return (1.0 - self._fiber.na ** 2) ** 0.5

    def pack(self, mc, target: _abi.McgbSource):
        """fiber.py:429-470: rotation onto the fibre axis, core refractive
        index, angular parameter, position, axis, core radius."""
        T = mcutil.transform_base((0.0, 0.0, 1.0), self._direction)
        target.kind = self._kind
        target.transformation[:] = [float(v) for v in np.asarray(T).ravel()]
        target.position[:] = [float(v) for v in self._position]
        target.direction[:] = [float(v) for v in self._direction]
        target.sigma[0] = self._fiber.dcore * 0.5
        target.sigma[1] = self._angular()
        target.clip = self._fiber.ncore
        return target

    def todict(self):
        return {'type': type(self).__name__, 'fiber': self._fiber.todict(),
                'position': self._position.tolist(), 'direction': self._direction.tolist()}

    def __str__(self):
        return '{}(fiber={}, position=({}, {}, {}), direction=({}, {}, {}))'.format(
            type(self).__name__, self._fiber, *self._position, *self._direction)

    __repr__ = __str__


class LambertianFiber(UniformFiber):
    """Tilted fibre source with a Lambertian angular distribution
    (xopto/mcml/mcsource/fiber.py:499-687)."""
    _kind = _abi.SRC_LAMBERTIAN_FIBER

    def _angular(self):
        return self._fiber.na


class UniformBeam(Source):
    """Collimated beam of uniform intensity over an ellipse of the given
    diameters (xopto/mcml/mcsource/uniformbeam.py:32-330)."""

    def __init__(self, diameter, position=(0.0, 0.0, 0.0), direction=(0.0, 0.0, 1.0)):
        if isinstance(diameter, UniformBeam):
            o = diameter
            diameter, position, direction = o.diameter, o.position, o.direction
        self._diameter = np.zeros((2,))
        self._diameter[:] = diameter
        if np.any(self._diameter < 0.0):
            raise ValueError('Beam diameter must not be negative!')
        self._position = np.zeros((3,))
        self._position[:] = position
        self._direction = _unit(direction)
        if self._direction[-1] <= 0.0:
            raise ValueError('Z component of the propagation direction must be positive!')

    diameter = property(lambda self: self._diameter)
    position = property(lambda self: self._position)
    direction = property(lambda self: self._direction)

    def pack(self, mc, target: _abi.McgbSource):
        """uniformbeam.py:243-292: move to the surface, refract, specular
        reflectance, rotation of the beam plane."""
        k = (0.0 - self._position[2]) / self._direction[2]
        position = self._position + k * self._direction
        position[2] = 0.0
        n1, n2 = mc.layers[0].n, mc.layers[1].n
        direction = mcutil.refract(self._direction, (0.0, 0.0, 1.0), n1, n2)
        reflectance = mcutil.reflectance(n1, n2, abs(self._direction[-1]))
        T = mcutil.transform_base((0.0, 0.0, 1.0), self._direction)
        target.kind = _abi.SRC_UNIFORM_BEAM
        target.transformation[:] = [float(v) for v in np.asarray(T).ravel()]
        target.position[:] = [float(v) for v in position]
        target.direction[:] = [float(v) for v in direction]
        target.sigma[:] = [float(v) * 0.5 for v in self._diameter]
        target.reflectance = reflectance
        return target

    def todict(self):
        return {'type': 'UniformBeam', 'diameter': self._diameter.tolist(),
                'position': self._position.tolist(), 'direction': self._direction.tolist()}

    def __str__(self):
        return 'UniformBeam(diameter=({}, {}), position=({}, {}, {}), direction=({}, {}, {}))'.format(
            *self._diameter, *self._position, *self._direction)

    __repr__ = __str__


class IsotropicPoint(Source):
    """Isotropic point source above (z <= 0) or inside the sample
    (xopto/mcml/mcsource/point.py:31-260)."""

    def __init__(self, position=(0.0, 0.0, 0.0)):
        if isinstance(position, IsotropicPoint):
            position = position.position
        self._position = np.zeros((3,))
        self._position[:] = position

    def _set_position(self, p):
        self._position[:] = p

    position = property(lambda self: self._position, _set_position)

    def pack(self, mc, target: _abi.McgbSource):
        """point.py:188-226: position and the index of the layer holding it."""
        if self._position[2] >= mc.layers.thickness():
            raise ValueError('The source must be located above or within the sample but not '
                             'under the sample!')
        target.kind = _abi.SRC_ISOTROPIC_POINT
        target.position[:] = [float(v) for v in self._position]
        target.layer_index = 1 if self._position[2] <= 0.0 else mc.layer_index(self._position[2])
        return target

    def todict(self):
        return {'type': 'IsotropicPoint', 'position': self._position.tolist()}

    def __str__(self):
        return 'IsotropicPoint(position=({}, {}, {}))'.format(*self._position)

    __repr__ = __str__


class UniformRectangular(Source):
    """Rectangular source whose emission is uniform in the cosine of the
    angle up to the numerical aperture in air, refracted into the layer that
    holds the source; the Fresnel reflectance at the source face is taken
    from the initial weight (xopto/mcml/mcsource/rectangular.py:32-316)."""
    _kind = _abi.SRC_UNIFORM_RECTANGULAR

    def __init__(self, width: float, height: float = None, n: float = 1.0, na: float = 0.0,
                 position=(0.0, 0.0, 0.0)):
        if isinstance(width, UniformRectangular):
            o = width
            width, height, n, na, position = o.width, o.height, o.n, o.na, o.position
        self._width = float(width)
        self._height = float(height)
        self._n = max(1.0, float(n))
        self._na = max(0.0, float(na))
        self._position = np.zeros((3,))
        self._position[:] = position

    def _set_width(self, v):
        self._width = float(v)

    def _set_height(self, v):
        self._height = float(v)

    def _set_n(self, v):
        self._n = max(1.0, float(v))

    def _set_na(self, v):
        self._na = max(0.0, float(v))

    def _set_position(self, p):
        self._position[:] = p

    width = property(lambda self: self._width, _set_width, None, 'Source width (m).')
    height = property(lambda self: self._height, _set_height, None, 'Source height (m).')
    n = property(lambda self: self._n, _set_n, None, 'Source refractive index.')
    na = property(lambda self: self._na, _set_na, None, 'Source numerical aperture.')
    position = property(lambda self: self._position, _set_position)

    def _angular(self) -> float:
        return (1.0 - self._na ** 2) ** 0.5

    def pack(self, mc, target: _abi.McgbSource):
        """rectangular.py:246-300: a source at z <= 0 sits on the surface in
        layer 1, otherwise in the layer that contains its depth."""
        if self._position[2] <= 0.0:
            position = (self._position[0], self._position[1], 0.0)
            layer_index = 1
        else:
            position = self._position
            layer_index = mc.layer_index(self._position[2])
        target.kind = self._kind
        target.position[:] = [float(v) for v in position]
        target.sigma[:] = [self._width, self._height]
        target.clip = self._n
        target.angular = self._angular()
        target.layer_index = layer_index
        return target

    def todict(self):
        return {'type': type(self).__name__, 'width': self._width, 'height': self._height,
                'n': self._n, 'na': self._na, 'position': self._position.tolist()}

    def __str__(self):
        return '{}(width={}, height={}, n={}, na={}, position=({}, {}, {}))'.format(
            type(self).__name__, self._width, self._height, self._n, self._na, *self._position)

    __repr__ = __str__


class LambertianRectangular(UniformRectangular):
    """Rectangular source with Lambertian emission up to the numerical
    aperture in air (xopto/mcml/mcsource/rectangular.py:317-529)."""
    _kind = _abi.SRC_LAMBERTIAN_RECTANGULAR

    def _angular(self) -> float:
        return self._na


def _pack_emission(mc, target, emission):
    """Appends an EmissionLut to the float table (LinearLut.cl_pack,
    xopto/mcbase/mcutil/lut.py:164-193); the device samples it by a uniform
    random number (fp_linear_lut_rel_sample)."""
    if emission is None:
        raise ValueError('The source needs an emission look-up table!')
    _, _, n, offset = emission.pack(mc)
    target.lut_offset = offset
    target.lut_size = n


class UniformFiberLutNI(UniformFiberNI):
    """Fibre source with normal incidence whose emission-angle cosine in air
    is drawn from the fibre's EmissionLut (a MultimodeFiberLut), refracted
    into the sample (xopto/mcml/mcsource/fiberni.py:581-760)."""

    def pack(self, mc, target: _abi.McgbSource):
        """fiberni.py:796-830: position, core radius, core index, LUT."""
        target.kind = _abi.SRC_UNIFORM_FIBER_LUT_NI
        target.position[:] = [float(v) for v in self._position]
        target.sigma[0] = self._fiber.dcore * 0.5
        target.sigma[1] = 0.0
        target.clip = self._fiber.ncore
        _pack_emission(mc, target, self._fiber.emission)
        return target

    def todict(self):
        return {'type': 'UniformFiberLutNI', 'fiber': self._fiber.todict(),
                'position': self._position.tolist()}

    def __str__(self):
        return 'UniformFiberLutNI(fiber={}, position=({}, {}, {}))'.format(self._fiber, *self._position)

    __repr__ = __str__


class UniformFiberLut(UniformFiber):
    """Tilted fibre source whose emission-angle cosine in air is drawn from
    the fibre's EmissionLut; unlike UniformFiber, the launch direction is
    refracted into the sample (xopto/mcml/mcsource/fiber.py:690-1010)."""
    _kind = _abi.SRC_UNIFORM_FIBER_LUT

    def _angular(self):
        return 0.0

    def pack(self, mc, target: _abi.McgbSource):
        """fiber.py:970-990: rotation onto the fibre axis, position, axis,
        core radius, core index, LUT."""
        UniformFiber.pack(self, mc, target)
        _pack_emission(mc, target, self._fiber.emission)
        return target


class UniformRectangularLut(Source):
    """Rectangular source whose emission-angle cosine in air is drawn from
    an EmissionLut (xopto/mcml/mcsource/rectangular.py:530-854)."""

    def __init__(self, lut, width: float = None, height: float = None, n: float = 1.0,
                 position=(0.0, 0.0, 0.0)):
        if isinstance(lut, UniformRectangularLut):
            o = lut
            lut, width, height, n, position = o.lut, o.width, o.height, o.n, o.position
        self._lut = lut
        self._width = float(width)
        self._height = float(height)
        self._n = max(1.0, float(n))
        self._position = np.zeros((3,))
        self._position[:] = position

    def _set_position(self, p):
        self._position[:] = p

    lut = property(lambda self: self._lut)
    width = property(lambda self: self._width)
    height = property(lambda self: self._height)
    n = property(lambda self: self._n)
    position = property(lambda self: self._position, _set_position)

    def pack(self, mc, target: _abi.McgbSource):
        """rectangular.py:780-830, with the layer rule of UniformRectangular."""
        if self._position[2] <= 0.0:
            position = (self._position[0], self._position[1], 0.0)
            layer_index = 1
        else:
            position = self._position
            layer_index = mc.layer_index(self._position[2])
        _pack_emission(mc, target, self._lut)
        target.kind = _abi.SRC_UNIFORM_RECTANGULAR_LUT
        target.position[:] = [float(v) for v in position]
        target.sigma[:] = [self._width, self._height]
        target.clip = self._n
        target.angular = 0.0
        target.layer_index = layer_index
        return target

    def todict(self):
        return {'type': 'UniformRectangularLut', 'lut': self._lut.todict(), 'width': self._width,
                'height': self._height, 'n': self._n, 'position': self._position.tolist()}

    def __str__(self):
        return 'UniformRectangularLut(lut={}, width={}, height={}, n={}, position=({}, {}, {}))'.format(
            self._lut, self._width, self._height, self._n, *self._position)

    __repr__ = __str__
