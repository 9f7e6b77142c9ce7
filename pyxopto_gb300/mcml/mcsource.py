"""Photon packet sources of the layered simulator: Line and GaussianBeam
(xopto/mcml/mcsource/line.py, gaussianbeam.py)."""
import numpy as np

from .. import _abi
from ..mcbase import mcutil


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
