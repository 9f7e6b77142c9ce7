"""Optical-fibre probe detectors: the weight of a packet leaving the sample
through the core of a probe fibre, within the fibre's acceptance, goes to
that fibre's bin (xopto/mcml/mcdetector/probe: lineararray.py,
sixaroundone.py, fiberarray.py and the path-length variants
lineararraypl.py, sixaroundonepl.py, fiberarraypl.py; the voxelized
simulator uses the same classes).

Each detector packs its geometry as a float table appended to the
simulator's float lookup buffer (layouts documented with McgbDetector in
include/xopto_gb300.h).  The raw data has one value per fibre, or
(path-length bins, fibres) for the _Pl variants.
"""
import numpy as np

from .. import _abi
from . import mcutil
from .mcdetector import Detector, _pack_pl_axis
from .mcutil import Axis
from .mcutil.fiber import MultimodeFiber, FiberLayout


def _fiber_transform(direction):
    d = np.asarray(direction, dtype=np.float64)
    adir = (d[0], d[1], abs(d[2]))
    return np.asarray(mcutil.transform_base(adir, (0.0, 0.0, 1.0)), dtype=np.float64).ravel()


def _cos_min(fiber):
    return (1.0 - (fiber.na / fiber.ncore) ** 2) ** 0.5


class _Probe(Detector):
    kind = _abi.DET_NONE
    kind_pl = _abi.DET_NONE

    def _init_pl(self, plaxis, n):
        self._pl_axis = plaxis
        if plaxis is not None:
            self._raw_data = np.zeros((plaxis.n, n))
            self.tracks_pathlength = True

    plaxis = property(lambda self: getattr(self, '_pl_axis', None))

    def _get_normalized(self):
        return self.raw * (1.0 / max(self.nphotons, 1.0))

    normalized = property(_get_normalized)
    reflectance = property(_get_normalized)
    transmittance = property(_get_normalized)

    def pack(self, mc, target: _abi.McgbDetector):
        table = np.asarray(self.table(), dtype=np.float32)
        target.kind = self.kind_pl if self.plaxis is not None else self.kind
        target.offset = mc.cl_allocate_rw_accumulator_buffer(self, self.shape)
        target.n = self.n_fibers()
        target.table_offset = mc.append_r_lut(table)
        if self.plaxis is not None:
            _pack_pl_axis(self.plaxis, target)
        return target


class LinearArray(_Probe):
    """Linear array of n identical, optionally tilted fibres
    (xopto/mcml/mcdetector/probe/lineararray.py:33-420); with ``plaxis`` the
    path-length resolved LinearArrayPl."""
    kind, kind_pl = _abi.DET_LINEAR_ARRAY, _abi.DET_LINEAR_ARRAY_PL

    def __init__(self, fiber: MultimodeFiber, n=1, spacing: float = None, orientation=(1.0, 0.0),
                 position=(0.0, 0.0), direction=(0.0, 0.0, 1.0), plaxis: Axis = None):
        if isinstance(fiber, LinearArray):
            o = fiber
            fiber, n, spacing, orientation = o.fiber, o.n, o.spacing, o.orientation
            position, direction, plaxis = o.position, o.direction, o.plaxis
        n = max(int(n), 1)
        super().__init__(np.zeros((n,)), 0)
        self._fiber = fiber
        self._n = n
        self._spacing = float(fiber.dcladding if spacing is None else spacing)
        o = np.asarray(orientation, dtype=np.float64)
        self._orientation = o / np.linalg.norm(o)
        self._position = np.zeros((2,))
        self._position[:] = position
        d = np.asarray(direction, dtype=np.float64)
        self._direction = d / np.linalg.norm(d)
        self._init_pl(plaxis, n)

    fiber = property(lambda self: self._fiber)
    n = property(lambda self: self._n)
    spacing = property(lambda self: self._spacing)
    orientation = property(lambda self: self._orientation)
    position = property(lambda self: self._position)
    direction = property(lambda self: self._direction)

    def n_fibers(self):
        return self._n

    def fiber_position(self, index: int):
        if index >= self._n or index < -self._n:
            raise IndexError('The fiber index is out of valid range!')
        left = self._position - self._orientation * self._spacing * (self._n - 1) * 0.5
        return tuple(left + self._spacing * self._orientation * int(index))

    def table(self):
        """lineararray.py:341-380."""
        return np.concatenate([_fiber_transform(self._direction), self.fiber_position(0),
                               self._orientation * self._spacing,
                               [0.25 * self._fiber.dcore ** 2, _cos_min(self._fiber)]])

    def copy(self):
        return LinearArray(self)


class LinearArrayPl(LinearArray):
    """LinearArray resolved by optical path length
    (xopto/mcml/mcdetector/probe/lineararraypl.py)."""

    def __init__(self, fiber, n=1, spacing=None, plaxis=None, orientation=(1.0, 0.0),
                 position=(0.0, 0.0), direction=(0.0, 0.0, 1.0)):
        LinearArray.__init__(self, fiber, n, spacing, orientation, position, direction,
                             plaxis if plaxis is not None else Axis(0.0, 1.0, 1))


class SixAroundOne(_Probe):
    """Central fibre and six around it, optionally tilted
    (xopto/mcml/mcdetector/probe/sixaroundone.py:33-440)."""
    kind, kind_pl = _abi.DET_SIX_AROUND_ONE, _abi.DET_SIX_AROUND_ONE_PL

    def __init__(self, fiber: MultimodeFiber, spacing: float = None, position=(0.0, 0.0),
                 direction=(0.0, 0.0, 1.0), plaxis: Axis = None):
        if isinstance(fiber, SixAroundOne):
            o = fiber
            fiber, spacing, position, direction, plaxis = o.fiber, o.spacing, o.position, o.direction, o.plaxis
        super().__init__(np.zeros((7,)), 0)
        self._fiber = fiber
        self._spacing = float(fiber.dcladding if spacing is None else spacing)
        self._position = np.zeros((2,))
        self._position[:] = position
        d = np.asarray(direction, dtype=np.float64)
        self._direction = d / np.linalg.norm(d)
        self._init_pl(plaxis, 7)

    fiber = property(lambda self: self._fiber)
    spacing = property(lambda self: self._spacing)
    position = property(lambda self: self._position)
    direction = property(lambda self: self._direction)

    def n_fibers(self):
        return 7

    def table(self):
        """sixaroundone.py:346-386."""
        return np.concatenate([_fiber_transform(self._direction), self._position,
                               [0.25 * self._fiber.dcore ** 2, self._spacing,
                                _cos_min(self._fiber)]])

    def copy(self):
        return SixAroundOne(self)


class SixAroundOnePl(SixAroundOne):
    """SixAroundOne resolved by optical path length
    (xopto/mcml/mcdetector/probe/sixaroundonepl.py)."""

    def __init__(self, fiber, spacing=None, plaxis=None, position=(0.0, 0.0),
                 direction=(0.0, 0.0, 1.0)):
        SixAroundOne.__init__(self, fiber, spacing, position, direction,
                              plaxis if plaxis is not None else Axis(0.0, 1.0, 1))


class FiberArray(_Probe):
    """Arbitrary array of fibres (FiberLayout list)
    (xopto/mcml/mcdetector/probe/fiberarray.py:33-360)."""
    kind, kind_pl = _abi.DET_FIBER_ARRAY, _abi.DET_FIBER_ARRAY_PL

    def __init__(self, fibers, plaxis: Axis = None):
        if isinstance(fibers, FiberArray):
            fibers, plaxis = fibers.fibers, fibers.plaxis
        self._fibers = [FiberLayout(f) for f in fibers]
        super().__init__(np.zeros((len(self._fibers),)), 0)
        self._init_pl(plaxis, len(self._fibers))

    fibers = property(lambda self: self._fibers)

    def n_fibers(self):
        return len(self._fibers)

    def table(self):
        """fiberarray.py:270-312."""
        out = []
        for fl in self._fibers:
            out.extend(_fiber_transform(fl.direction))
            out.extend([fl.position[0], fl.position[1], 0.25 * fl.fiber.dcore ** 2,
                        _cos_min(fl.fiber)])
        return np.asarray(out, dtype=np.float64)

    def copy(self):
        return FiberArray(self)


class FiberArrayPl(FiberArray):
    """FiberArray resolved by optical path length
    (xopto/mcml/mcdetector/probe/fiberarraypl.py)."""

    def __init__(self, fibers, plaxis=None):
        FiberArray.__init__(self, fibers, plaxis if plaxis is not None else Axis(0.0, 1.0, 1))


class FiberLutArray(_Probe):
    """Array of fibres (FiberLayout of MultimodeFiberLut) whose collection
    is weighted by each fibre's CollectionLut at the |cosine| of the exit
    direction to the fibre axis (xopto/mcml/mcdetector/probe/fiberlutarray.py:
    30-366).  The float table holds, per fibre, transformation, position,
    core r^2, LUT first position and 1/span, and the LUT size and offset
    (relative to the table) as uint32 bit patterns, then the LUT data."""
    kind = kind_pl = _abi.DET_FIBER_LUT_ARRAY

    def __init__(self, fibers):
        if isinstance(fibers, FiberLutArray):
            fibers = fibers.fibers
        self._fibers = [FiberLayout(f) for f in fibers]
        super().__init__(np.zeros((len(self._fibers),)), 0)

    fibers = property(lambda self: self._fibers)

    def n_fibers(self):
        return len(self._fibers)

    def table(self):
        """fiberlutarray.py:305-324."""
        n = len(self._fibers)
        head = np.zeros((n, _abi.DET_LUT_FIBER_FLOATS), dtype=np.float32)
        data = []
        rel = n * _abi.DET_LUT_FIBER_FLOATS
        for i, fl in enumerate(self._fibers):
            lut = fl.fiber.collection
            head[i, :9] = _fiber_transform(fl.direction)
            head[i, 9:11] = fl.position[:2]
            head[i, 11] = 0.25 * fl.fiber.dcore ** 2
            head[i, 12] = lut.first
            head[i, 13] = 1.0 / (lut.last - lut.first)
            head[i, 14:16] = np.array([lut.data.size, rel], dtype=np.uint32).view(np.float32)
            data.append(np.asarray(lut.data, dtype=np.float32))
            rel += lut.data.size
        return np.concatenate([head.ravel()] + data)

    def pack(self, mc, target: _abi.McgbDetector):
        table = self.table()
        target.kind = self.kind
        target.offset = mc.cl_allocate_rw_accumulator_buffer(self, self.shape)
        target.n = self.n_fibers()
        target.n_y = table.size
        target.table_offset = mc.append_r_lut(table)
        return target

    def copy(self):
        return FiberLutArray(self)


__all__ = ['LinearArray', 'LinearArrayPl', 'SixAroundOne', 'SixAroundOnePl', 'FiberArray',
           'FiberArrayPl', 'FiberLutArray']
