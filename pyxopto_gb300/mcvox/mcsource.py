"""Photon packet sources of the voxelized simulator: Line, GaussianBeam,
UniformBeam, IsotropicPoint, UniformFiber, LambertianFiber and IsotropicVoxel
(xopto/mcvox/mcsource/line.py, gaussianbeam.py, uniformbeam.py, point.py,
fiber.py, voxel.py)."""
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


class Line:
    """Infinitely thin beam entering the voxel box
    (xopto/mcvox/mcsource/line.py)."""

    def __init__(self, position=(0.0, 0.0, 0.0), direction=(0.0, 0.0, 1.0)):
        if isinstance(position, Line):
            position, direction = position.position, position.direction
        self._position = np.zeros((3,))
        self._position[:] = position
        self._direction = _unit(direction)

    position = property(lambda self: self._position)
    direction = property(lambda self: self._direction)

    def pack(self, mc, target: _abi.McgbSource):
        vox = mc.voxels
        search = -self._direction if vox.contains(self._position) else self._direction
        position, normal = vox.intersect(self._position, search)
        if position is None:
            raise ValueError('The line source does not intersect the voxelized sample!')
        m_out = mc.materials[0]
        m_in = mc.material(position)
        reflectance = mcutil.reflectance(m_out.n, m_in.n, np.abs(np.dot(normal, self._direction)))
        if reflectance >= 1.0:
            raise ValueError('The line source is fully reflected from the surface of the '
                             'voxelized sample!')
        sample_direction = mcutil.refract(self._direction, normal, m_out.n, m_in.n)
        dir_reflected = mcutil.reflect(self._direction, normal)
        target.kind = _abi.SRC_LINE
        target.position[:] = [float(v) for v in position]
        target.direction[:] = [float(v) for v in sample_direction]
        target.direction_reflected[:] = [float(v) for v in dir_reflected]
        target.reflectance = reflectance
        return target

    def todict(self):
        return {'type': 'Line', 'position': self._position.tolist(),
                'direction': self._direction.tolist()}

    def __str__(self):
        return 'Line(position=({}, {}, {}), direction=({}, {}, {}))'.format(
            *self._position, *self._direction)

    __repr__ = __str__


class GaussianBeam:
    """Collimated Gaussian beam entering the voxel box
    (xopto/mcvox/mcsource/gaussianbeam.py:33-353)."""

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

    def pack(self, mc, target: _abi.McgbSource):
        """gaussianbeam.py:296-336."""
        T = mcutil.transform_base((0.0, 0.0, 1.0), self._direction)
        target.kind = _abi.SRC_GAUSSIAN_BEAM
        target.transformation[:] = [float(v) for v in np.asarray(T).ravel()]
        target.position[:] = [float(v) for v in self._position]
        target.direction[:] = [float(v) for v in self._direction]
        target.sigma[:] = [float(v) for v in self._sigma]
        target.clip = self._clip
        target.reflectance = 0.0
        return target

    def todict(self):
        return {'type': 'GaussianBeam', 'sigma': self._sigma.tolist(), 'clip': self._clip,
                'position': self._position.tolist(), 'direction': self._direction.tolist()}

    def __str__(self):
        return 'GaussianBeam(sigma=({}, {}), clip={})'.format(*self._sigma, self._clip)

    __repr__ = __str__


class UniformBeam:
    """Collimated beam of uniform intensity over an ellipse, entering the
    voxel box (xopto/mcvox/mcsource/uniformbeam.py:32-340)."""

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

    diameter = property(lambda self: self._diameter)
    position = property(lambda self: self._position)
    direction = property(lambda self: self._direction)

    def pack(self, mc, target: _abi.McgbSource):
        """uniformbeam.py:271-310."""
        T = mcutil.transform_base((0.0, 0.0, 1.0), self._direction)
        target.kind = _abi.SRC_UNIFORM_BEAM
        target.transformation[:] = [float(v) for v in np.asarray(T).ravel()]
        target.position[:] = [float(v) for v in self._position]
        target.direction[:] = [float(v) for v in self._direction]
        target.sigma[:] = [float(v) * 0.5 for v in self._diameter]
        return target

    def todict(self):
        return {'type': 'UniformBeam', 'diameter': self._diameter.tolist(),
                'position': self._position.tolist(), 'direction': self._direction.tolist()}

    def __str__(self):
        return 'UniformBeam(diameter=({}, {}))'.format(*self._diameter)

    __repr__ = __str__


class IsotropicPoint:
    """Isotropic point source inside or outside the voxel box
    (xopto/mcvox/mcsource/point.py:31-230)."""

    def __init__(self, position=(0.0, 0.0, 0.0)):
        if isinstance(position, IsotropicPoint):
            position = position.position
        self._position = np.zeros((3,))
        self._position[:] = position

    position = property(lambda self: self._position)

    def pack(self, mc, target: _abi.McgbSource):
        target.kind = _abi.SRC_ISOTROPIC_POINT
        target.position[:] = [float(v) for v in self._position]
        return target

    def todict(self):
        return {'type': 'IsotropicPoint', 'position': self._position.tolist()}

    def __str__(self):
        return 'IsotropicPoint(position=({}, {}, {}))'.format(*self._position)

    __repr__ = __str__


class UniformFiber:
    """Optical fibre source with its axis along ``direction``, launching
    onto the voxel box; uniform over the core and in solid angle within the
    acceptance cone (xopto/mcvox/mcsource/fiber.py:178-520)."""
    _kind = _abi.SRC_UNIFORM_FIBER

    def __init__(self, fiber: MultimodeFiber, position=(0.0, 0.0, 0.0), direction=(0.0, 0.0, 1.0)):
        if isinstance(fiber, UniformFiber):
            fiber, position, direction = fiber.fiber, fiber.position, fiber.direction
        self._fiber = fiber
        self._position = np.zeros((3,))
        self._position[:] = position
        self._direction = _unit(direction)

    fiber = property(lambda self: self._fiber)
    position = property(lambda self: self._position)
    direction = property(lambda self: self._direction)

    def _angular(self):
        return (1.0 - self._fiber.na ** 2) ** 0.5

    def pack(self, mc, target: _abi.McgbSource):
        """fiber.py:455-493 (UniformFiber), 700-740 (LambertianFiber)."""
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
        return '{}(fiber={})'.format(type(self).__name__, self._fiber)

    __repr__ = __str__


class LambertianFiber(UniformFiber):
    """Fibre source with a Lambertian angular distribution
    (xopto/mcvox/mcsource/fiber.py:523-744)."""
    _kind = _abi.SRC_LAMBERTIAN_FIBER

    def _angular(self):
        return self._fiber.na


class IsotropicVoxel:
    """Isotropic source uniformly distributed within one voxel
    (xopto/mcvox/mcsource/voxel.py:31-192)."""

    def __init__(self, voxel):
        if isinstance(voxel, IsotropicVoxel):
            voxel = voxel.voxel
        self._voxel = np.zeros((3,), dtype=np.int64)
        self._voxel[:] = voxel

    voxel = property(lambda self: self._voxel)

    def pack(self, mc, target: _abi.McgbSource):
        shape = mc.voxels.shape          # (nz, ny, nx)
        nx, ny, nz = shape[2], shape[1], shape[0]
        x, y, z = (int(v) for v in self._voxel)
        if not (0 <= x < nx and 0 <= y < ny and 0 <= z < nz):
            raise ValueError('Voxel index ({}, {}, {}) is not valid!'.format(x, y, z))
        target.kind = _abi.SRC_ISOTROPIC_VOXEL
        target.direction[:] = [float(x), float(y), float(z)]
        target.position[:] = [float(v) for v in mc.voxels.center(self._voxel)]
        return target

    def todict(self):
        return {'type': 'IsotropicVoxel', 'voxel': self._voxel.tolist()}

    def __str__(self):
        return 'IsotropicVoxel(voxel=({}, {}, {}))'.format(*self._voxel)

    __repr__ = __str__


class IsotropicVoxels:
    """Isotropic source spread over a set of voxels, each with a weight in
    [0, 1]; a packet starts uniformly within one voxel chosen uniformly
    (xopto/mcvox/mcsource/voxel.py:195-380)."""

    def __init__(self, voxels, weights=None):
        if isinstance(voxels, IsotropicVoxels):
            voxels, weights = voxels.voxels, voxels.weights
        voxels = np.asarray(voxels)
        if voxels.shape[-1] != 3 or voxels.ndim > 2:
            raise ValueError('Shape of the voxel array must be (n, 3)!')
        voxels = np.reshape(voxels, (-1, 3))
        self._data = np.ones((voxels.shape[0], 4))
        self._data[:, 1:] = voxels
        if weights is not None:
            weights = np.asarray(weights, dtype=np.float64)
            if weights.size != self._data.shape[0]:
                raise ValueError('The number of weights must equal the number of voxels!')
            self._data[:, 0] = np.clip(weights, 0.0, 1.0)

    voxels = property(lambda self: self._data[:, 1:])
    weights = property(lambda self: self._data[:, 0])

    def pack(self, mc, target: _abi.McgbSource):
        """voxel.py:340-380: the (weight, x, y, z) rows go to the float
        table; position is the centre of the mean voxel index."""
        for v in self._data[:, 1:]:
            if not mc.voxels.isvalid([int(i) for i in v]):
                raise ValueError('Voxel index ({}, {}, {}) is not valid!'.format(*v))
        target.kind = _abi.SRC_ISOTROPIC_VOXELS
        target.lut_offset = mc.append_r_lut(np.asarray(self._data, dtype=np.float32).ravel())
        target.lut_size = self._data.shape[0]
        target.position[:] = [float(v) for v in mc.voxels.center(np.mean(self._data[:, 1:], 0))]
        return target

    def todict(self):
        return {'type': 'IsotropicVoxels', 'voxels': self._data[:, 1:].tolist(),
                'weights': self._data[:, 0].tolist()}

    def __str__(self):
        return 'IsotropicVoxels(n={})'.format(self._data.shape[0])

    __repr__ = __str__


class UniformFiberLut(UniformFiber):
    """Tilted fibre source of the voxelized medium whose emission-angle
    cosine in air is drawn from the fibre's EmissionLut (a
    MultimodeFiberLut); launched onto the voxel box like UniformFiber
    (xopto/mcvox/mcsource/fiber.py:770-960)."""
    _kind = _abi.SRC_UNIFORM_FIBER_LUT

    def _angular(self):
        return 0.0

    def pack(self, mc, target: _abi.McgbSource):
        """fiber.py:930-960: the UniformFiber fields and the emission LUT."""
        UniformFiber.pack(self, mc, target)
        emission = self._fiber.emission
        if emission is None:
            raise ValueError('The source needs an emission look-up table!')
        _, _, n, offset = emission.pack(mc)
        target.lut_offset = offset
        target.lut_size = n
        return target
