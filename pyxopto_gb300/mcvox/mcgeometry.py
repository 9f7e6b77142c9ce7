"""Voxelized sample volume (xopto/mcvox/mcgeometry/voxel.py:88-729).

Each voxel holds a uint8 index into the material list (material 0 is the
surrounding medium); the array is addressed [z, y, x]."""
from typing import Tuple
import numpy as np

from .. import _abi
from ..mcbase.mcutil import Axis


class Voxels:
    def __init__(self, xaxis: Axis, yaxis: Axis, zaxis: Axis, voxel=None):
        if xaxis.logscale or yaxis.logscale or zaxis.logscale:
            raise ValueError('Logarithmic scale is not supported!')
        self._x_axis, self._y_axis, self._z_axis = xaxis, yaxis, zaxis
        self._voxel_size = (abs(xaxis.step), abs(yaxis.step), abs(zaxis.step))
        self._top_left = (min(xaxis.span), min(yaxis.span), min(zaxis.span))
        self._bottom_right = (max(xaxis.span), max(yaxis.span), max(zaxis.span))
        self._data = np.zeros((zaxis.n, yaxis.n, xaxis.n), dtype=np.uint8)

    xaxis = property(lambda self: self._x_axis)
    yaxis = property(lambda self: self._y_axis)
    zaxis = property(lambda self: self._z_axis)
    x = property(lambda self: self._x_axis.centers)
    y = property(lambda self: self._y_axis.centers)
    z = property(lambda self: self._z_axis.centers)
    dx = property(lambda self: self._voxel_size[0])
    dy = property(lambda self: self._voxel_size[1])
    dz = property(lambda self: self._voxel_size[2])
    voxel_size = property(lambda self: self._voxel_size)
    shape = property(lambda self: self._data.shape, None, None, 'Voxel array shape (z, y, x).')
    size = property(lambda self: self._data.size)
    top_left = property(lambda self: self._top_left)
    bottom_right = property(lambda self: self._bottom_right)

    def data(self, mc=None) -> np.ndarray:
        """The (nz, ny, nx) uint8 material-index array."""
        return self._data

    def _get_material(self):
        return self._data

    def _set_material(self, value):
        v = np.asarray(value)
        if v.min(initial=0) < 0 or v.max(initial=0) > 255:
            raise ValueError('Material indices must fit uint8 (0..255)!')
        self._data[...] = v

    material = property(_get_material, _set_material, None, '3D array of material indices.')

    def __getitem__(self, item):
        return self._data[item]

    def __setitem__(self, item, value):
        self._data[item] = value

    def meshgrid(self):
        return np.meshgrid(self._z_axis.centers, self._y_axis.centers, self._x_axis.centers,
                           indexing='ij')

    def index(self, position) -> Tuple[int, int, int]:
        return tuple(int((position[k] - self._top_left[k]) // self._voxel_size[k]) for k in range(3))

    def center(self, index):
        return tuple(self._top_left[k] + (index[k] + 0.5) * self._voxel_size[k] for k in range(3))

    def isvalid(self, index) -> bool:
        return 0 <= index[0] < self._x_axis.n and 0 <= index[1] < self._y_axis.n and \
            0 <= index[2] < self._z_axis.n

    def contains(self, position) -> bool:
        return self._x_axis.start <= position[0] < self._x_axis.stop and \
            self._y_axis.start <= position[1] < self._y_axis.stop and \
            self._z_axis.start <= position[2] < self._z_axis.stop

    def intersect(self, pos, dir):
        """Ray / box intersection with the outward normal
        (xopto/mcvox/mcgeometry/voxel.py:317-378)."""
        invdir = [np.inf, np.inf, np.inf]
        for ax in (0, 1, 2):
            if dir[ax] != 0.0:
                invdir[ax] = 1.0 / dir[ax]
        xmin, xmax = self._x_axis.edges[[0, -1]]
        ymin, ymax = self._y_axis.edges[[0, -1]]
        zmin, zmax = self._z_axis.edges[[0, -1]]
        t1, t2 = (xmin - pos[0]) * invdir[0], (xmax - pos[0]) * invdir[0]
        t3, t4 = (ymin - pos[1]) * invdir[1], (ymax - pos[1]) * invdir[1]
        t5, t6 = (zmin - pos[2]) * invdir[2], (zmax - pos[2]) * invdir[2]
        txmin, txmax = min(t1, t2), max(t1, t2)
        tymin, tymax = min(t3, t4), max(t3, t4)
        tzmin, tzmax = min(t5, t6), max(t5, t6)
        tmin = max(txmin, tymin, tzmin)
        tmax = min(txmax, tymax, tzmax)
        if tmax < tmin or tmax < 0.0:
            return None, None
        t = tmin if tmin >= 0.0 else tmax
        intersection = (pos[0] + t * dir[0], pos[1] + t * dir[1], pos[2] + t * dir[2])
        normal = [0.0, 0.0, 0.0]
        normal[0] = int(txmin >= tymin and txmin >= tzmin) * np.sign(dir[0])
        normal[1] = int(not normal[0] and tymin >= tzmin) * np.sign(dir[1])
        normal[2] = int(not (normal[0] or normal[1])) * np.sign(dir[2])
        return intersection, normal

    def pack_geometry(self, cfg):
        cfg.top_left[:] = [float(v) for v in self._top_left]
        cfg.bottom_right[:] = [float(v) for v in self._bottom_right]
        cfg.voxel_size[:] = [float(v) for v in self._voxel_size]
        cfg.shape[:] = [self._x_axis.n, self._y_axis.n, self._z_axis.n]
        return cfg

    def todict(self):
        return {'type': 'Voxels', 'xaxis': self._x_axis.todict(), 'yaxis': self._y_axis.todict(),
                'zaxis': self._z_axis.todict()}

    def __str__(self):
        return 'Voxels(xaxis={}, yaxis={}, zaxis={})'.format(self._x_axis, self._y_axis, self._z_axis)

    __repr__ = __str__
