"""Cartesian fluence / energy-deposition accumulator
(xopto/mcbase/mcfluence/fluence.py:33-592)."""
import numpy as np

from .. import _abi
from .mcutil import Axis


class Fluence:
    """Fluence(xaxis, yaxis, zaxis, mode='deposition'|'fluence', k=ACCU_K).

    The accumulator is a (nz, ny, nx) grid addressed (z*ny + y)*nx + x
    (fluence.py:103-143); deposits are uint32(w*k + 0.5) added into 64-bit
    integers."""

    def __init__(self, xaxis, yaxis=None, zaxis=None, mode: str = 'deposition',
                 k: int = _abi.ACCU_K):
        if isinstance(xaxis, Fluence):
            other = xaxis
            self._x_axis, self._y_axis, self._z_axis = Axis(other.xaxis), Axis(other.yaxis), Axis(other.zaxis)
            self._mode = other.mode
            self._k = other.k
            self._data = np.copy(other.raw) if other.raw is not None else None
            self._nphotons = other.nphotons
            return
        self._x_axis, self._y_axis, self._z_axis = xaxis, yaxis, zaxis
        if mode not in ('deposition', 'fluence'):
            raise ValueError('Fluence mode must be "deposition" or "fluence"!')
        self._mode = mode
        self._k = max(1, min(int(k), 2 ** 31 - 1))
        self._data = None
        self._nphotons = 0

    xaxis = property(lambda self: self._x_axis)
    yaxis = property(lambda self: self._y_axis)
    zaxis = property(lambda self: self._z_axis)
    mode = property(lambda self: self._mode)
    k = property(lambda self: self._k)
    nphotons = property(lambda self: self._nphotons)
    shape = property(lambda self: (self._z_axis.n, self._y_axis.n, self._x_axis.n))
    dx = property(lambda self: self._x_axis.step)
    dy = property(lambda self: self._y_axis.step)
    dz = property(lambda self: self._z_axis.step)
    x = property(lambda self: self._x_axis.centers)
    y = property(lambda self: self._y_axis.centers)
    z = property(lambda self: self._z_axis.centers)
    raw = property(lambda self: self._data)

    def _get_data(self):
        if self._data is None:
            return None
        return self._data * (1.0 / (max(self._nphotons, 1) * self.dx * self.dy * self.dz))

    data = property(_get_data, None, None, 'Deposition or fluence rate per packet and volume.')

    def update_data(self, mc, accumulators, nphotons: int, **kwargs):
        acc = np.asarray(accumulators[0]).reshape(self.shape)
        if self._data is not None:
            self._data += acc * (1.0 / self._k)
            self._nphotons += int(nphotons)
        else:
            self._data = acc * (1.0 / self._k)
            self._nphotons = int(nphotons)

    def update(self, obj: 'Fluence'):
        if self._data is not None:
            if self.shape != obj.shape:
                raise TypeError('Cannot update with fluence data of incompatible shape!')
            self._data += obj.raw
            self._nphotons += obj.nphotons
        else:
            self._data = np.copy(obj.raw)
            self._nphotons = obj.nphotons

    def pack(self, mc, target: _abi.McgbFluence):
        n = self._x_axis.n * self._y_axis.n * self._z_axis.n
        target.kind = _abi.FLUENCE_DEPOSITION if self._mode == 'deposition' else _abi.FLUENCE_RATE
        target.offset = mc.cl_allocate_rw_accumulator_buffer(self, (n,))
        target.inv_step[:] = [1.0 / self._x_axis.step, 1.0 / self._y_axis.step, 1.0 / self._z_axis.step]
        target.top_left[:] = [self._x_axis.start, self._y_axis.start, self._z_axis.start]
        target.shape[:] = [self._x_axis.n, self._y_axis.n, self._z_axis.n]
        target.k = self._k
        return target

    def todict(self):
        return {'type': 'Fluence', 'xaxis': self._x_axis.todict(), 'yaxis': self._y_axis.todict(),
                'zaxis': self._z_axis.todict(), 'mode': self._mode, 'k': self._k}

    def __str__(self):
        return 'Fluence(xaxis={}, yaxis={}, zaxis={}, mode={})'.format(
            self._x_axis, self._y_axis, self._z_axis, self._mode)
