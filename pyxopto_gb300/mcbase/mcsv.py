"""Sampling volume of photon packet traces (xopto/mcbase/mcsv.py:30-409).

The voxel grid is given by three axes; ``Mc.sampling_volume(trace, sv)``
walks every traced packet through it on the GPU and adds, for each voxel it
crosses, the packet's end value times the path length inside the voxel.
The raw integer tallies are scaled back by 1/(k * multiplier) in
``update_data``; ``weight`` sums the end values.
"""
from typing import Tuple

import numpy as np

from .. import _abi
from .mcutil import Axis


class SamplingVolume:
    K = 0x7FFFFF        # McFloat32.mc_fp_maxint, xopto/mcbase/mctypes.py:575

    def __init__(self, xaxis, yaxis: Axis = None, zaxis: Axis = None):
        data, weight = None, 0.0
        if isinstance(xaxis, SamplingVolume):
            sv = xaxis
            xaxis, yaxis, zaxis = Axis(sv.xaxis), Axis(sv.yaxis), Axis(sv.zaxis)
            if sv.data is not None:
                data = np.copy(sv.data)
            weight = sv.weight
        self._x_axis, self._y_axis, self._z_axis = xaxis, yaxis, zaxis
        self._data = data
        self._weight = weight
        self._k = self.K
        if self._x_axis.n * self._y_axis.n * self._z_axis.n <= 0:
            raise ValueError('Sampling volume accumulator array has one or '
                             'dimensions equal to zero!')

    def todict(self) -> dict:
        return {'type': 'SamplingVolume', 'xaxis': self._x_axis.todict(),
                'yaxis': self._y_axis.todict(), 'zaxis': self._z_axis.todict()}

    @classmethod
    def fromdict(cls, data: dict) -> 'SamplingVolume':
        d = dict(data)
        t = d.pop('type')
        if t != cls.__name__:
            raise TypeError('Expected data for type "{}" but got "{}"!'.format(cls.__name__, t))
        return cls(Axis.fromdict(d.pop('xaxis')), Axis.fromdict(d.pop('yaxis')),
                   Axis.fromdict(d.pop('zaxis')), **d)

    shape = property(lambda self: (self._z_axis.n, self._y_axis.n, self._x_axis.n),
                     None, None, 'Sampling volume array shape (z, y, x).')
    x = property(lambda self: self._x_axis.centers)
    y = property(lambda self: self._y_axis.centers)
    z = property(lambda self: self._z_axis.centers)
    xaxis = property(lambda self: self._x_axis)
    yaxis = property(lambda self: self._y_axis)
    zaxis = property(lambda self: self._z_axis)
    k = property(lambda self: self._k)

    def _get_data(self):
        return self._data

    def _set_data(self, data):
        self._data = data

    data = property(_get_data, _set_data, None, 'Sampling volume data if any.')

    def _get_weight(self):
        return self._weight

    def _set_weight(self, w):
        self._weight = w

    weight = property(_get_weight, _set_weight, None, 'Total end value of the processed packets.')

    def clear(self):
        if self._data is not None:
            self._data.fill(0)

    def _multiplier(self, mc=None) -> float:
        """1 / the smallest voxel size (mcsv.py:344-351)."""
        step = min(self._x_axis.step, self._y_axis.step, self._z_axis.step)
        if step <= 0.0:
            step = 1.0 / self._k
        return 1.0 / step

    def update_data(self, mc, accumulators, total_weight, **kwargs):
        """Adds the raw tallies scaled by 1/(k * multiplier) (mcsv.py:313-342)."""
        multiplier = self._multiplier(mc)
        new = np.reshape(np.asarray(accumulators[0], dtype=np.float64), self.shape) * \
            (1.0 / (self._k * multiplier))
        w = float(np.asarray(total_weight).ravel()[0]) / self._k
        if self._data is not None:
            self._data += new
            self._weight += w
        else:
            self._data = new
            self._weight = w

    def pack(self, mc, target: _abi.McgbSamplingVolume = None) -> _abi.McgbSamplingVolume:
        """The C-ABI form of the grid (ClSamplingVolume, mcsv.py:354-395)."""
        if target is None:
            target = _abi.McgbSamplingVolume()
        axes = (self._x_axis, self._y_axis, self._z_axis)
        for i, a in enumerate(axes):
            target.top_left[i] = a.start
            target.voxel_size[i] = a.step
            target.shape[i] = a.n
        target.multiplier = self._multiplier(mc)
        target.k = self._k
        target.offset = 0
        return target

    def __str__(self):
        return 'SamplingVolume(xaxis={}, yaxis={}, zaxis={})'.format(
            self._x_axis, self._y_axis, self._z_axis)

    __repr__ = __str__


__all__ = ['SamplingVolume', 'Axis']
