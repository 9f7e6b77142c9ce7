"""Surface detectors: Total, Radial, Cartesian and SymmetricX, the optical
path-length variants TotalPl, RadialPl and CartesianPl, grouped by
Detectors into the top, bottom and specular slots
(xopto/mcml/mcdetector/base.py, total.py, radial.py, cartesian.py,
symmetric.py, totalpl.py, radialpl.py, cartesianpl.py; the mcvox package uses
the same classes).

Tallies come back from the device as uint64 fixed-point integers and are
converted with the reference's rule raw += accumulator/K
(xopto/mcml/mcdetector/base.py:269-292).
"""
from typing import Tuple
import numpy as np

from .. import _abi
from .mcutil import Axis, RadialAxis, SymmetricAxis


class Detector:
    kind = _abi.DET_NONE

    def __init__(self, raw_data: np.ndarray, nphotons: int):
        self._raw_data = raw_data
        self._nphotons = int(nphotons)

    raw = property(lambda self: self._raw_data, None, None, 'Raw accumulator data.')
    nphotons = property(lambda self: self._nphotons)
    shape = property(lambda self: self._raw_data.shape)
    total = property(lambda self: self._raw_data.sum())

    def set_raw_data(self, data, nphotons):
        self._raw_data[:] = np.asarray(data, dtype=self._raw_data.dtype)
        self._nphotons = int(nphotons)

    def update_data(self, mc, accumulators, nphotons: int, **kwargs):
        new_data = np.reshape(accumulators[0], self.shape)
        self._raw_data += new_data * (1.0 / _abi.ACCU_K)
        self._nphotons += int(nphotons)

    def pack(self, mc, target: _abi.McgbDetector):
        target.kind = _abi.DET_NONE
        return target

    def copy(self):
        raise NotImplementedError


class DetectorDefault(Detector):
    """Empty detector slot (xopto/mcml/mcdetector/base.py:140-200)."""

    def __init__(self, *args, **kwargs):
        super().__init__(np.zeros((0,)), 0)

    def copy(self):
        return DetectorDefault()

    def __str__(self):
        return 'DetectorDefault()'


class Total(Detector):
    """Total reflectance/transmittance (xopto/mcml/mcdetector/total.py:32-239)."""
    kind = _abi.DET_TOTAL

    def __init__(self, cosmin=0.0, direction=(0.0, 0.0, 1.0)):
        if isinstance(cosmin, Total):
            other = cosmin
            super().__init__(np.copy(other.raw), other.nphotons)
            cosmin, direction = other.cosmin, other.direction
        else:
            super().__init__(np.zeros((1,)), 0)
        self._cosmin = 0.0
        self._direction = np.zeros((3,))
        self.cosmin = cosmin
        self.direction = direction

    def _set_cosmin(self, v):
        self._cosmin = min(max(float(v), 0.0), 1.0)

    cosmin = property(lambda self: self._cosmin, _set_cosmin)

    def _set_direction(self, d):
        self._direction[:] = d
        n = np.linalg.norm(self._direction)
        if n == 0.0:
            raise ValueError('Direction vector norm/length must not be 0!')
        self._direction *= 1.0 / n

    direction = property(lambda self: self._direction, _set_direction)

    def _get_normalized(self):
        return self.raw * (1.0 / max(self.nphotons, 1.0))

    normalized = property(_get_normalized)
    reflectance = property(_get_normalized)
    transmittance = property(_get_normalized)

    def pack(self, mc, target):
        target.kind = _abi.DET_TOTAL
        target.offset = mc.cl_allocate_rw_accumulator_buffer(self, self.shape)
        target.cos_min = self._cosmin
        target.direction[:] = [float(v) for v in self._direction]
        return target

    def copy(self):
        return Total(self)

    def todict(self):
        return {'type': 'Total', 'cosmin': self._cosmin, 'direction': self._direction.tolist()}

    def __str__(self):
        return 'Total(cosmin={}, direction=({}, {}, {}))'.format(self._cosmin, *self._direction)


class Radial(Detector):
    """Radial (concentric ring) detector; radii beyond the axis are clipped
    into the last bin (xopto/mcml/mcdetector/radial.py:32-337)."""
    kind = _abi.DET_RADIAL

    def __init__(self, raxis, position=(0.0, 0.0), cosmin=0.0, direction=(0.0, 0.0, 1.0)):
        if isinstance(raxis, Radial):
            other = raxis
            super().__init__(np.copy(other.raw), other.nphotons)
            position, cosmin, direction = other.position, other.cosmin, other.direction
            raxis = type(other.raxis)(other.raxis)
        else:
            super().__init__(np.zeros((raxis.n,)), 0)
        self._r_axis = raxis
        self._position = np.zeros((2,))
        self._direction = np.zeros((3,))
        self._cosmin = 0.0
        self.position = position
        self.cosmin = cosmin
        self.direction = direction
        e = self._r_axis.edges
        self._inv_accumulators_area = 1.0 / (np.pi * (e[1:] ** 2 - e[:-1] ** 2))

    raxis = property(lambda self: self._r_axis)

    def _set_position(self, v):
        self._position[:] = v

    position = property(lambda self: self._position, _set_position)

    def _set_cosmin(self, v):
        self._cosmin = min(max(float(v), 0.0), 1.0)

    cosmin = property(lambda self: self._cosmin, _set_cosmin)

    def _set_direction(self, d):
        self._direction[:] = d
        n = np.linalg.norm(self._direction)
        if n == 0.0:
            raise ValueError('Direction vector norm/length must not be 0!')
        self._direction *= 1.0 / n

    direction = property(lambda self: self._direction, _set_direction)
    r = property(lambda self: self._r_axis.centers)
    edges = property(lambda self: self._r_axis.edges)
    n = property(lambda self: self._r_axis.n)
    logscale = property(lambda self: self._r_axis.logscale)

    def _get_normalized(self):
        return self.raw * self._inv_accumulators_area * (1.0 / max(self.nphotons, 1))

    normalized = property(_get_normalized)
    reflectance = property(_get_normalized)
    transmittance = property(_get_normalized)

    def pack(self, mc, target):
        target.kind = _abi.DET_RADIAL
        target.offset = mc.cl_allocate_rw_accumulator_buffer(self, self.shape)
        target.position[:] = [float(v) for v in self._position]
        target.r_min = self._r_axis.scaled_start
        target.inv_dr = 1.0 / self._r_axis.step if self._r_axis.step != 0.0 else 0.0
        target.log_scale = int(self._r_axis.logscale)
        target.n = self._r_axis.n
        target.cos_min = self._cosmin
        target.direction[:] = [float(v) for v in self._direction]
        return target

    def copy(self):
        return Radial(self)

    def todict(self):
        return {'type': 'Radial', 'r_axis': self._r_axis.todict(),
                'position': self._position.tolist(), 'cosmin': self._cosmin,
                'direction': self._direction.tolist()}

    def __str__(self):
        return 'Radial(raxis={}, position=({}, {}), cosmin={})'.format(
            self._r_axis, *self._position, self._cosmin)


def _pack_pl_axis(axis, target):
    target.pl_min = axis.scaled_start
    target.inv_dpl = 1.0 / axis.step if axis.step != 0.0 else 0.0
    target.pl_log_scale = int(axis.logscale)
    target.n_pl = axis.n


class TotalPl(Total):
    """Total reflectance/transmittance resolved by optical path length
    (xopto/mcml/mcdetector/totalpl.py:30-300); raw has shape (n_pl, 1).
    Turns on optical path-length tracking."""
    kind = _abi.DET_TOTAL_PL
    tracks_pathlength = True

    def __init__(self, plaxis=None, cosmin=0.0, direction=(0.0, 0.0, 1.0)):
        if isinstance(plaxis, TotalPl):
            other = plaxis
            Total.__init__(self, cosmin=other.cosmin, direction=other.direction)
            self._pl_axis = type(other.plaxis)(other.plaxis)
            self._raw_data = np.copy(other.raw)
            self._nphotons = other.nphotons
            return
        Total.__init__(self, cosmin=cosmin, direction=direction)
        self._pl_axis = plaxis if plaxis is not None else Axis(0.0, 1.0, 1)
        self._raw_data = np.zeros((self._pl_axis.n, 1))

    plaxis = property(lambda self: self._pl_axis)
    pl = property(lambda self: self._pl_axis.centers)
    pledges = property(lambda self: self._pl_axis.edges)
    npl = property(lambda self: self._pl_axis.n)

    def pack(self, mc, target):
        Total.pack(self, mc, target)
        target.kind = _abi.DET_TOTAL_PL
        _pack_pl_axis(self._pl_axis, target)
        return target

    def copy(self):
        return TotalPl(self)

    def todict(self):
        return {'type': 'TotalPl', 'pl_axis': self._pl_axis.todict(), 'cosmin': self._cosmin,
                'direction': self._direction.tolist()}

    def __str__(self):
        return 'TotalPl(plaxis={}, cosmin={})'.format(self._pl_axis, self._cosmin)


class RadialPl(Radial):
    """Radial reflectance/transmittance resolved by optical path length
    (xopto/mcml/mcdetector/radialpl.py:30-470); raw has shape (n_pl, n_r),
    path length first.  Turns on optical path-length tracking."""
    kind = _abi.DET_RADIAL_PL
    tracks_pathlength = True

    def __init__(self, raxis, plaxis=None, position=(0.0, 0.0), cosmin=0.0,
                 direction=(0.0, 0.0, 1.0)):
        if isinstance(raxis, RadialPl):
            other = raxis
            Radial.__init__(self, type(other.raxis)(other.raxis), position=other.position,
                            cosmin=other.cosmin, direction=other.direction)
            self._pl_axis = type(other.plaxis)(other.plaxis)
            self._raw_data = np.copy(other.raw)
            self._nphotons = other.nphotons
        else:
            Radial.__init__(self, raxis, position=position, cosmin=cosmin, direction=direction)
            self._pl_axis = plaxis if plaxis is not None else Axis(0.0, 1.0, 1)
            self._raw_data = np.zeros((self._pl_axis.n, raxis.n))
        self._inv_accumulators_area = self._inv_accumulators_area.reshape(1, -1)

    plaxis = property(lambda self: self._pl_axis)
    pl = property(lambda self: self._pl_axis.centers)
    pledges = property(lambda self: self._pl_axis.edges)
    npl = property(lambda self: self._pl_axis.n)
    nr = property(lambda self: self._r_axis.n)

    def pack(self, mc, target):
        Radial.pack(self, mc, target)
        target.kind = _abi.DET_RADIAL_PL
        _pack_pl_axis(self._pl_axis, target)
        return target

    def copy(self):
        return RadialPl(self)

    def todict(self):
        return {'type': 'RadialPl', 'r_axis': self._r_axis.todict(),
                'pl_axis': self._pl_axis.todict(), 'position': self._position.tolist(),
                'cosmin': self._cosmin, 'direction': self._direction.tolist()}

    def __str__(self):
        return 'RadialPl(raxis={}, plaxis={}, cosmin={})'.format(self._r_axis, self._pl_axis,
                                                                 self._cosmin)


class _Directional(Detector):
    """Acceptance cosine and reference direction shared by the detectors."""

    def _init_direction(self, cosmin, direction):
        self._cosmin = 0.0
        self._direction = np.zeros((3,))
        self.cosmin = cosmin
        self.direction = direction

    def _set_cosmin(self, v):
        self._cosmin = min(max(float(v), 0.0), 1.0)

    cosmin = property(lambda self: self._cosmin, _set_cosmin)

    def _set_direction(self, d):
        self._direction[:] = d
        n = np.linalg.norm(self._direction)
        if n == 0.0:
            raise ValueError('Direction vector norm/length must not be 0!')
        self._direction *= 1.0 / n

    direction = property(lambda self: self._direction, _set_direction)


class Cartesian(_Directional):
    """Reflectance/transmittance on a 2-D x-y grid; raw has shape (n_y, n_x)
    and positions beyond the grid are clipped into the edge bins
    (xopto/mcml/mcdetector/cartesian.py:33-420)."""
    kind = _abi.DET_CARTESIAN

    def __init__(self, xaxis, yaxis=None, cosmin=0.0, direction=(0.0, 0.0, 1.0)):
        if isinstance(xaxis, Cartesian):
            other = xaxis
            xaxis, yaxis = type(other.xaxis)(other.xaxis), type(other.yaxis)(other.yaxis)
            cosmin, direction = other.cosmin, other.direction
            raw, nphotons = np.copy(other.raw), other.nphotons
        else:
            if yaxis is None:
                yaxis = Axis(xaxis)
            raw, nphotons = np.zeros((yaxis.n, xaxis.n)), 0
        super().__init__(raw, nphotons)
        self._x_axis, self._y_axis = xaxis, yaxis
        self._init_direction(cosmin, direction)
        self._accumulators_area = self._x_axis.step * self._y_axis.step

    xaxis = property(lambda self: self._x_axis)
    yaxis = property(lambda self: self._y_axis)
    x = property(lambda self: self._x_axis.centers)
    y = property(lambda self: self._y_axis.centers)

    def _get_normalized(self):
        return self.raw * (1.0 / (max(self.nphotons, 1.0) * self._accumulators_area))

    normalized = property(_get_normalized)
    reflectance = property(_get_normalized)
    transmittance = property(_get_normalized)

    def radial(self, raxis, order=2, nfi=360, center=(0.0, 0.0)) -> 'Radial':
        """A Radial detector resampled from this one: the per-area data is
        interpolated at nfi azimuths on every ring of ``raxis`` around
        ``center`` and summed with the ring areas
        (xopto/mcml/mcdetector/cartesian.py:289-327)."""
        from .mcutil.interp import interp2
        nfi = int(nfi)
        dfi = 2.0 * np.pi / nfi
        fi = np.linspace(0.5 * dfi, 2.0 * np.pi - 0.5 * dfi, nfi)
        area = self._x_axis.step * self._y_axis.step
        a = np.pi * (raxis.edges[1:] ** 2 - raxis.edges[:-1] ** 2)
        w = np.reshape(a / (nfi * area), (1, raxis.n))
        R, Fi = np.meshgrid(raxis.centers, fi)
        Xi, Yi = R * np.cos(Fi) + center[0], R * np.sin(Fi) + center[1]
        raw = interp2(Xi, Yi, self.x, self.y, self.raw, order=order)
        raw = (raw * w).sum(0)
        out = Radial(raxis, cosmin=self._cosmin)
        out.set_raw_data(raw, self.nphotons)
        return out

    def pack(self, mc, target):
        """cartesian.py:340-372."""
        target.kind = self.kind
        target.offset = mc.cl_allocate_rw_accumulator_buffer(self, self.shape)
        target.direction[:] = [float(v) for v in self._direction]
        target.r_min = self._x_axis.start
        target.inv_dr = 1.0 / self._x_axis.step if self._x_axis.n > 1 else 0.0
        target.y_min = self._y_axis.start
        target.inv_dy = 1.0 / self._y_axis.step if self._y_axis.n > 1 else 0.0
        target.cos_min = self._cosmin
        target.n = self._x_axis.n
        target.n_y = self._y_axis.n
        return target

    def copy(self):
        return type(self)(self)

    def todict(self):
        return {'type': 'Cartesian', 'x_axis': self._x_axis.todict(),
                'y_axis': self._y_axis.todict(), 'cosmin': self._cosmin,
                'direction': self._direction.tolist()}

    def __str__(self):
        return 'Cartesian(xaxis={}, yaxis={}, cosmin={})'.format(self._x_axis, self._y_axis,
                                                                self._cosmin)


class CartesianPl(Cartesian):
    """Cartesian detector resolved by optical path length; raw has shape
    (n_pl, n_y, n_x) (xopto/mcml/mcdetector/cartesianpl.py:33-470).  Turns
    on optical path-length tracking."""
    kind = _abi.DET_CARTESIAN_PL
    tracks_pathlength = True

    def __init__(self, xaxis, yaxis=None, plaxis=None, cosmin=0.0, direction=(0.0, 0.0, 1.0)):
        if isinstance(xaxis, CartesianPl):
            other = xaxis
            Cartesian.__init__(self, type(other.xaxis)(other.xaxis), type(other.yaxis)(other.yaxis),
                               other.cosmin, other.direction)
            self._pl_axis = type(other.plaxis)(other.plaxis)
            self._raw_data = np.copy(other.raw)
            self._nphotons = other.nphotons
            return
        Cartesian.__init__(self, xaxis, yaxis, cosmin, direction)
        self._pl_axis = plaxis if plaxis is not None else Axis(0.0, 1.0, 1)
        self._raw_data = np.zeros((self._pl_axis.n, self._y_axis.n, self._x_axis.n))

    plaxis = property(lambda self: self._pl_axis)
    pl = property(lambda self: self._pl_axis.centers)

    def pack(self, mc, target):
        Cartesian.pack(self, mc, target)
        _pack_pl_axis(self._pl_axis, target)
        return target

    def todict(self):
        d = Cartesian.todict(self)
        d.update(type='CartesianPl', pl_axis=self._pl_axis.todict())
        return d


class SymmetricX(_Directional):
    """Reflectance/transmittance in 2*n_half bins symmetric about
    x = center, linear or logarithmic in |x - center|
    (xopto/mcml/mcdetector/symmetric.py:33-320)."""
    kind = _abi.DET_SYMMETRIC_X

    def __init__(self, xaxis: SymmetricAxis, cosmin=0.0, direction=(0.0, 0.0, 1.0)):
        if isinstance(xaxis, SymmetricX):
            other = xaxis
            xaxis, cosmin, direction = SymmetricAxis(other.xaxis), other.cosmin, other.direction
            raw, nphotons = np.copy(other.raw), other.nphotons
        else:
            raw, nphotons = np.zeros((xaxis.n,)), 0
        super().__init__(raw, nphotons)
        self._x_axis = xaxis
        self._init_direction(cosmin, direction)
        self._inv_dx = 1.0 / (self._x_axis.edges[1:] - self._x_axis.edges[:-1])

    xaxis = property(lambda self: self._x_axis)
    x = property(lambda self: self._x_axis.centers)

    def _get_normalized(self):
        return self.raw * self._inv_dx * (1.0 / max(self.nphotons, 1.0))

    normalized = property(_get_normalized)
    reflectance = property(_get_normalized)
    transmittance = property(_get_normalized)

    def pack(self, mc, target):
        """symmetric.py:260-285."""
        target.kind = self.kind
        target.offset = mc.cl_allocate_rw_accumulator_buffer(self, self.shape)
        target.direction[:] = [float(v) for v in self._direction]
        target.position[0] = self._x_axis.center
        target.r_min = self._x_axis.scaled_offset
        target.inv_dr = 1.0 / self._x_axis.step if self._x_axis.step != 0.0 else 0.0
        target.log_scale = int(self._x_axis.logscale)
        target.n = self._x_axis.n_half
        target.cos_min = self._cosmin
        return target

    def copy(self):
        return SymmetricX(self)

    def todict(self):
        return {'type': 'SymmetricX', 'x_axis': self._x_axis.todict(), 'cosmin': self._cosmin,
                'direction': self._direction.tolist()}

    def __str__(self):
        return 'SymmetricX(xaxis={}, cosmin={})'.format(self._x_axis, self._cosmin)


class TotalLut(Detector):
    """Total reflectance/transmittance weighted by a CollectionLut of the
    |cosine| between the exit direction and ``direction``
    (xopto/mcml/mcdetector/total.py:240-460); one bin."""
    kind = _abi.DET_TOTAL_LUT

    def __init__(self, lut, direction=(0.0, 0.0, 1.0)):
        if isinstance(lut, TotalLut):
            other = lut
            super().__init__(np.copy(other.raw), other.nphotons)
            lut, direction = other.lut, other.direction
        else:
            super().__init__(np.zeros((1,)), 0)
        self._lut = lut
        self._direction = np.zeros((3,))
        self.direction = direction

    def _set_direction(self, d):
        self._direction[:] = d
        n = np.linalg.norm(self._direction)
        if n == 0.0:
            raise ValueError('Direction vector norm/length must not be 0!')
        self._direction *= 1.0 / n

    lut = property(lambda self: self._lut, None, None, 'Collection look-up table.')
    direction = property(lambda self: self._direction, _set_direction)

    def _get_normalized(self):
        return self.raw * (1.0 / max(self.nphotons, 1.0))

    normalized = property(_get_normalized)
    reflectance = property(_get_normalized)
    transmittance = property(_get_normalized)

    def pack(self, mc, target):
        first, inv_span, n, offset = self._lut.pack(mc)
        target.kind = self.kind
        target.offset = mc.cl_allocate_rw_accumulator_buffer(self, self.shape)
        target.direction[:] = [float(v) for v in self._direction]
        target.r_min, target.inv_dr, target.n_y, target.table_offset = first, inv_span, n, offset
        target.n = 1
        return target

    def copy(self):
        return TotalLut(self)

    def todict(self):
        return {'type': 'TotalLut', 'lut': self._lut.todict(), 'direction': self._direction.tolist()}

    def __str__(self):
        return 'TotalLut(lut={}, direction=({}, {}, {}))'.format(self._lut, *self._direction)


class TotalLutPl(TotalLut):
    """TotalLut resolved by optical path length
    (xopto/mcml/mcdetector/totalpl.py, TotalLutPl); raw has shape (n_pl, 1)."""
    kind = _abi.DET_TOTAL_LUT_PL
    tracks_pathlength = True

    def __init__(self, lut, plaxis=None, direction=(0.0, 0.0, 1.0)):
        if isinstance(lut, TotalLutPl):
            other = lut
            TotalLut.__init__(self, other.lut, other.direction)
            self._pl_axis = type(other.plaxis)(other.plaxis)
            self._raw_data = np.copy(other.raw)
            self._nphotons = other.nphotons
            return
        TotalLut.__init__(self, lut, direction)
        self._pl_axis = plaxis if plaxis is not None else Axis(0.0, 1.0, 1)
        self._raw_data = np.zeros((self._pl_axis.n, 1))

    plaxis = property(lambda self: self._pl_axis)
    pl = property(lambda self: self._pl_axis.centers)

    def pack(self, mc, target):
        TotalLut.pack(self, mc, target)
        _pack_pl_axis(self._pl_axis, target)
        return target

    def copy(self):
        return TotalLutPl(self)


class Detectors:
    """Top, bottom and specular detectors
    (xopto/mcml/mcdetector/base.py:295-568)."""

    def __init__(self, top=None, bottom=None, specular=None):
        if isinstance(top, Detectors):
            other = top
            top, bottom, specular = other.top.copy(), other.bottom.copy(), other.specular.copy()
        self._top = top if top is not None else DetectorDefault()
        self._bottom = bottom if bottom is not None else DetectorDefault()
        self._specular = specular if specular is not None else DetectorDefault()

    top = property(lambda self: self._top)
    bottom = property(lambda self: self._bottom)
    specular = property(lambda self: self._specular)

    def types(self):
        return type(self._top), type(self._bottom), type(self._specular)

    def __iter__(self):
        return iter([d for d in (self._top, self._bottom, self._specular)
                     if not isinstance(d, DetectorDefault)])

    def tracks_pathlength(self) -> bool:
        """True if a detector needs the packets' optical path length."""
        return any(getattr(d, 'tracks_pathlength', False)
                   for d in (self._top, self._bottom, self._specular))

    def pack(self, mc, cfg):
        self._top.pack(mc, cfg.top)
        self._bottom.pack(mc, cfg.bottom)
        self._specular.pack(mc, cfg.specular)

    def slots(self):
        return (('top', self._top), ('bottom', self._bottom), ('specular', self._specular))

    def todict(self) -> dict:
        """Configuration of the three slots (xopto/mcml/mcdetector/base.py:
        Detectors.todict); an empty slot is None."""
        def one(d):
            if isinstance(d, DetectorDefault) or not hasattr(d, 'todict'):
                return None
            return d.todict()
        return {'type': 'Detectors', 'top': one(self._top), 'bottom': one(self._bottom),
                'specular': one(self._specular)}

    def __str__(self):
        return 'Detectors(top={}, bottom={}, specular={})'.format(
            self._top, self._bottom, self._specular)

    __repr__ = __str__


__all__ = ['Axis', 'RadialAxis', 'SymmetricAxis', 'Detector', 'DetectorDefault', 'Total', 'Radial',
           'TotalPl', 'RadialPl', 'Cartesian', 'CartesianPl', 'SymmetricX', 'TotalLut', 'TotalLutPl',
           'Detectors']
