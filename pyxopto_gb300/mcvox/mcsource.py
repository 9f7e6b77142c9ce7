"""Photon packet sources of the voxelized simulator: Line and GaussianBeam
(xopto/mcvox/mcsource/line.py, gaussianbeam.py)."""
import numpy as np

from .. import _abi
from ..mcbase import mcutil


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
