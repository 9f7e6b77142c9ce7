"""Axes, boundary optics and geometry helpers of the plugin objects.

Host-side (float64) counterparts of xopto/mcbase/mcutil/axis.py,
xopto/mcbase/mcutil/boundary.py and xopto/mcbase/mcutil/geometry.py, with
the same names and argument meaning.
"""
from typing import Tuple
import numpy as np


class Axis:
    """Linearly or logarithmically spaced accumulator axis
    (xopto/mcbase/mcutil/axis.py:33-197)."""

    def __init__(self, start=0.0, stop: float = 1.0, n: int = 1, logscale: bool = False):
        if isinstance(start, Axis):
            ax = start
            start, stop, n, logscale = ax.start, ax.stop, ax.n, ax.logscale
        start, stop, n, logscale = float(start), float(stop), int(n), bool(logscale)
        if n < 1:
            raise ValueError('An axis needs at least one bin!')
        self._logscale = logscale
        self._n = n
        if logscale:
            start = max(start, float(np.finfo(np.float64).eps))
            self._edges = np.logspace(np.log(start), np.log(stop), n + 1, base=np.e)
            self._step = (np.log(stop) - np.log(start)) / n
        else:
            self._edges = np.linspace(start, stop, n + 1)
            self._step = (stop - start) / n
        self._span = np.array((start, stop), dtype=np.float64)
        self._scaled_span = np.log(self._span) if logscale else self._span
        self._centers = 0.5 * (self._edges[:-1] + self._edges[1:])

    logscale = property(lambda self: self._logscale)
    step = property(lambda self: self._step)
    n = property(lambda self: self._n)
    span = property(lambda self: self._span)
    start = property(lambda self: self._span[0])
    stop = property(lambda self: self._span[1])
    scaled_span = property(lambda self: self._scaled_span)
    scaled_start = property(lambda self: self._scaled_span[0])
    scaled_stop = property(lambda self: self._scaled_span[1])
    edges = property(lambda self: self._edges)
    centers = property(lambda self: self._centers)

    def todict(self):
        return {'start': self.start, 'stop': self.stop, 'n': self.n,
                'logscale': self.logscale, 'type': type(self).__name__}

    @classmethod
    def fromdict(cls, data: dict):
        data = dict(data)
        data.pop('type', None)
        return cls(**data)

    def __str__(self):
        return '{}(start={}, stop={}, n={}, logscale={})'.format(
            type(self).__name__, self.start, self.stop, self.n, self.logscale)

    __repr__ = __str__


class RadialAxis(Axis):
    """Radial axis with area-corrected bin centers
    (xopto/mcbase/mcutil/axis.py:200-262)."""

    def __init__(self, start=0.0, stop: float = 1.0, n: int = 1, logscale: bool = False):
        Axis.__init__(self, start, stop, n, logscale)
        e = self.edges
        self._centers = (2.0 / 3.0) * (e[:-1] ** 2 + e[:-1] * e[1:] + e[1:] ** 2) / (e[:-1] + e[1:])


class SymmetricAxis:
    """Accumulator axis with 2*n_half bins placed symmetrically about a
    center, linear or logarithmic in the distance from the center
    (xopto/mcbase/mcutil/axis.py:267-480)."""

    def __init__(self, center: float = 0.0, range: float = 1.0, n_half: int = 1000,
                 logscale: bool = False):
        if isinstance(center, SymmetricAxis):
            ax = center
            center, range, n_half, logscale = ax.center, ax.range, ax.n_half, ax.logscale
        self._center, self._range = float(center), float(range)
        self._n_half, self._logscale = int(n_half), bool(logscale)
        self._n = 2 * self._n_half
        if self._logscale:
            eps = np.finfo(np.float64).eps
            right = (self._center + np.logspace(np.log(eps), np.log(self._range), self._n_half + 1,
                                                base=np.e))[1:]
            self._offset = eps
            self._edges = np.hstack((-right[::-1], [self._center], right))
            self._step = (np.log(self._range) - np.log(eps)) / self._n_half
            self._scaled_offset = np.log(self._offset)
        else:
            self._offset = 0.0
            self._edges = np.linspace(self._center - self._range, self._center + self._range,
                                      self._n + 1)
            self._step = (self._edges[-1] - self._edges[0]) / self._n
            self._scaled_offset = 0.0
        self._span = np.array((self._center + self._offset, self._center + self._range))
        self._centers = 0.5 * (self._edges[:-1] + self._edges[1:])

    center = property(lambda self: self._center)
    range = property(lambda self: self._range)
    n_half = property(lambda self: self._n_half)
    n = property(lambda self: self._n)
    logscale = property(lambda self: self._logscale)
    step = property(lambda self: self._step)
    span = property(lambda self: self._span)
    start = property(lambda self: self._span[0])
    stop = property(lambda self: self._span[1])
    offset = property(lambda self: self._offset)
    scaled_offset = property(lambda self: self._scaled_offset)
    edges = property(lambda self: self._edges)
    centers = property(lambda self: self._centers)

    def todict(self):
        return {'range': self._range, 'center': self._center, 'n_half': self._n_half,
                'logscale': self._logscale, 'type': 'SymmetricAxis'}

    def __str__(self):
        return 'SymmetricAxis(center={}, range={}, n_half={}, logscale={})'.format(
            self._center, self._range, self._n_half, self._logscale)

    __repr__ = __str__


def rotation_matrix_2d(a, b) -> np.ndarray:
    """2-D rotation matrix taking the direction of a onto the direction of b
    (xopto/mcbase/mcutil/geometry.py:33-59; the sine is taken as
    non-negative, as there)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    a = a / np.linalg.norm(a)
    b = b / np.linalg.norm(b)
    cos_theta = np.dot(a, b)
    sin_theta = np.sqrt(1.0 - cos_theta ** 2)
    return np.array([[cos_theta, -sin_theta], [sin_theta, cos_theta]])


def cos_critical(n1: float, n2: float) -> float:
    """Cosine of the critical incidence angle at the n1 -> n2 boundary
    (xopto/mcbase/mcutil/boundary.py:25-41)."""
    return (1.0 - (n2 / n1) ** 2) ** 0.5 if n1 > n2 else 0.0


def reflectance(n1: float, n2: float, costheta: float = 1.0) -> float:
    """Fresnel reflectance of unpolarized light
    (xopto/mcbase/mcutil/boundary.py:43-71)."""
    if costheta < 0.0:
        raise ValueError('The incidence angle cosine must not be negative!')
    n1, n2 = float(n1), float(n2)
    sintheta = (1.0 - costheta ** 2) ** 0.5
    if n1 > n2 and sintheta >= n2 / n1:
        return 1.0
    a1, a2 = n1 * costheta, n2 * (1.0 - (n1 / n2 * sintheta) ** 2) ** 0.5
    rs = abs((a1 - a2) / (a1 + a2)) ** 2
    b1, b2 = n1 * (1.0 - (n1 / n2 * sintheta) ** 2) ** 0.5, n2 * costheta
    rp = abs((b1 - b2) / (b1 + b2)) ** 2
    return 0.5 * (rs + rp)


def refract(direction, normal, n1: float, n2: float) -> np.ndarray:
    """Direction of the refracted beam (xopto/mcbase/mcutil/boundary.py:74-108)."""
    d = np.asarray(direction, dtype=np.float64)
    dl = np.linalg.norm(d)
    nn = np.asarray(normal, dtype=np.float64)
    nl = np.linalg.norm(nn)
    cos1 = np.dot(d, nn) / (dl * nl)
    if abs(cos1) < cos_critical(n1, n2):
        raise ValueError('Cannot refract, the incidence angle exceeds the critical angle!')
    k_n = n1 / n2
    sin2_squared = k_n * k_n * (1.0 - cos1 * cos1)
    k = k_n * abs(cos1) - np.sqrt(1.0 - sin2_squared)
    return k_n * d / dl - np.sign(cos1) * k * nn / nl


def reflect(direction, normal) -> np.ndarray:
    """Direction of the reflected beam (xopto/mcbase/mcutil/boundary.py:111-136)."""
    d = np.asarray(direction, dtype=np.float64)
    if np.linalg.norm(d) > 0:
        d = d / np.linalg.norm(d)
    nn = np.asarray(normal, dtype=np.float64)
    if np.linalg.norm(nn) > 0:
        nn = nn / np.linalg.norm(nn)
    return d - 2.0 * np.dot(d, nn) * nn


def rotation_matrix(a, b) -> np.ndarray:
    """Rotation taking unit vector a onto unit vector b (Rodrigues' formula
    R = I + [v]x + [v]x^2/(1 + a.b), v = a x b), as used by
    xopto/mcbase/mcutil/geometry.py:63-97."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    a = a / np.linalg.norm(a)
    b = b / np.linalg.norm(b)
    v = np.cross(a, b)
    c = float(np.dot(a, b))
    vx = np.array([[0.0, -v[2], v[1]], [v[2], 0.0, -v[0]], [-v[1], v[0], 0.0]])
    return np.identity(3) + vx + np.dot(vx, vx) * (1.0 / (1.0 + c))


def transform_base(vfrom, vto) -> np.ndarray:
    """xopto/mcbase/mcutil/geometry.py:100-133."""
    return rotation_matrix(vfrom, vto)
