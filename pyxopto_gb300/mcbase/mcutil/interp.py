"""Interpolation of functions sampled on uniform grids
(xopto/mcbase/mcutil/interp.py:82-160), used to resample Cartesian
detector data."""
import numpy as np


def interp2(xi, yi, x, y, f, order: int = 1, **kwargs) -> np.ndarray:
    """Values of f (shape (y.size, x.size), sampled at the uniform points x
    and y) at the points (xi, yi), by spline interpolation of the given
    order (scipy.ndimage.map_coordinates; 0 nearest, 1 linear, ...)."""
    from scipy.ndimage import map_coordinates
    f = np.asarray(f)
    if x is not None:
        x = np.asarray(x)
        if x.size != f.shape[1]:
            raise IndexError('Length of vector x must match the number of columns of f.')
        indx = (np.asarray(xi) - x[0]) * ((x.size - 1) / (x[-1] - x[0]))
    else:
        indx = np.asarray(xi)
    if y is not None:
        y = np.asarray(y)
        if y.size != f.shape[0]:
            raise IndexError('Length of vector y must match the number of rows of f.')
        indy = (np.asarray(yi) - y[0]) * ((y.size - 1) / (y[-1] - y[0]))
    else:
        indy = np.asarray(yi)
    return map_coordinates(f, np.asarray([indy, indx]), order=order, **kwargs)


__all__ = ['interp2']
