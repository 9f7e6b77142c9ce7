"""Linear look-up tables for emission and collection characteristics
(xopto/mcbase/mcutil/lut.py:33-364).

A ``LinearLut`` holds samples spread uniformly from ``first`` to ``last``.
``EmissionLut`` turns a radiance profile into the inverse cumulative
distribution of the emission-angle cosine (sampled on the device with a
uniform random number); ``CollectionLut`` resamples a detector sensitivity
over the incidence-angle cosine.  ``pack(mc)`` appends the table to the
simulator's float table and returns (first, 1/span, size, offset).
"""
import numpy as np


class LinearLut:
    def __init__(self, lut_data, first: float = 0.0, last: float = 1.0):
        if isinstance(lut_data, LinearLut):
            self._first, self._last = lut_data.first, lut_data.last
            self._lut_data = np.copy(lut_data.data)
        elif isinstance(lut_data, str):
            d = np.load(lut_data)
            self._first, self._last = float(d['first']), float(d['last'])
            self._lut_data = np.asarray(d['lut_data'], dtype=np.float64)
        else:
            self._first, self._last = float(first), float(last)
            self._lut_data = np.asarray(lut_data, dtype=np.float64)

    @staticmethod
    def fromfile(filename: str) -> 'LinearLut':
        d = np.load(filename)
        return LinearLut(d['lut_data'], d['first'], d['last'])

    first = property(lambda self: self._first, None, None, 'Position of the first entry.')
    last = property(lambda self: self._last, None, None, 'Position of the last entry.')
    span = property(lambda self: self._last - self._first)
    data = property(lambda self: self._lut_data, None, None, 'Table as a flat array.')

    def __call__(self, x):
        """Linear interpolation at x (lut.py:155-162)."""
        n = self._lut_data.size
        fp_ind = (np.asarray(x) - self._first) / (self._last - self._first) * (n - 1)
        i1 = np.clip(np.floor(fp_ind), 0, n - 1).astype(np.intp)
        i2 = np.clip(i1 + 1, 0, n - 1)
        w = fp_ind - i1
        return (1.0 - w) * self._lut_data[i1] + w * self._lut_data[i2]

    def pack(self, mc):
        """Appends the table to the simulator's float table; returns
        (first, 1/span, size, offset) (lut.py:164-193)."""
        offset = mc.append_r_lut(self._lut_data)
        return self._first, 1.0 / (self._last - self._first), int(self._lut_data.size), offset

    def todict(self, np2list: bool = True) -> dict:
        return {'type': type(self).__name__, 'first': self._first, 'last': self._last,
                'lut_data': self._lut_data.tolist() if np2list else self._lut_data}

    @staticmethod
    def fromdict(data: dict) -> 'LinearLut':
        d = dict(data)
        d.pop('type', None)
        return LinearLut(d['lut_data'], d['first'], d['last'])

    def save(self, filename: str):
        np.savez(filename, first=self._first, last=self._last, lut_data=self._lut_data)

    def __str__(self):
        return '{}(first={}, last={}, n={})'.format(type(self).__name__, self._first, self._last,
                                                   self._lut_data.size)

    __repr__ = __str__


class EmissionLut(LinearLut):
    """Inverse cumulative distribution of the emission-angle cosine for a
    radiance profile over cos(theta), assuming azimuthal symmetry
    (lut.py:240-325).  The density in cos(theta) is radiance *
    sin(theta); its cumulative integral is evaluated with composite
    Simpson's rule on an odd number of points ('simps') or adaptively
    ('quad'), normalised, and inverted by linear interpolation at n uniform
    probabilities."""

    def __init__(self, radiance, costheta=None, n: int = 2000, npts: int = 10000,
                 meth: str = 'simps'):
        from scipy.interpolate import interp1d
        lut_random = np.linspace(0.0, 1.0, n)
        if isinstance(radiance, (str, EmissionLut)):
            super().__init__(radiance)
            return
        radiance = np.asarray(radiance, dtype=np.float64)
        costheta = np.linspace(0.0, 1.0, radiance.size) if costheta is None \
            else np.asarray(costheta, dtype=np.float64)
        if radiance.size != costheta.size:
            raise ValueError('The sizes of the radiance and costheta array must be equal!')
        density = interp1d(costheta, radiance * np.sqrt(1.0 - costheta ** 2))
        lo, hi = costheta.min(), costheta.max()
        if meth == 'simps':
            npts = max(int((max(2 * n, npts) // 2)) * 2 + 1, 3)
            ct = np.linspace(lo, hi, max(n, npts))
            f = density(ct)
            h = (ct[-1] - ct[0]) / (ct.size - 1)
            cdf = np.zeros([int(ct.size // 2) + 1])
            cdf[1:] = h / 3.0 * (f[:-2:2] + 4.0 * f[1:-1:2] + f[2::2])
            cdf = cdf.cumsum()
            cdf /= cdf[-1]
            lut = interp1d(cdf, ct[::2])(lut_random)
        elif meth == 'quad':
            from scipy.integrate import quad
            ct = np.linspace(lo, hi, max(n, npts))
            cdf = np.array([quad(density, lo, c)[0] for c in ct])
            cdf /= cdf[-1]
            lut = interp1d(cdf, ct)(lut_random)
        else:
            raise ValueError('Unknown integration method "{}"!'.format(meth))
        super().__init__(lut, 0.0, 1.0)


class CollectionLut(LinearLut):
    """Detector sensitivity over the incidence-angle cosine, resampled to n
    uniform points by linear interpolation (lut.py:327-362)."""

    def __init__(self, sensitivity, costheta=None, n: int = 1000):
        from scipy.interpolate import interp1d
        if isinstance(sensitivity, (str, CollectionLut)):
            super().__init__(sensitivity)
            return
        sensitivity = np.asarray(sensitivity, dtype=np.float64)
        costheta = np.linspace(0.0, 1.0, sensitivity.size) if costheta is None \
            else np.asarray(costheta)
        ct = np.linspace(costheta.min(), costheta.max(), n)
        lut = interp1d(costheta, sensitivity)(ct)
        super().__init__(lut, ct[0], ct[-1])


__all__ = ['LinearLut', 'EmissionLut', 'CollectionLut']
