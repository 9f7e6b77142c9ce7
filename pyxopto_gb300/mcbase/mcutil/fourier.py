"""Fourier transform of a sampled 1-D profile (xopto/mcbase/mcutil/fourier.py:33-110),
used to turn spatially resolved reflectance into spatial-frequency-domain
amplitude and phase."""
import numpy as np


def discreteSimpson(frequency, xpts: np.ndarray, fpts: np.ndarray, uneven: bool = False) -> np.ndarray:
    """F(f) = integral of fpts(x) * exp(-2 pi i f x) dx by Simpson's rule over
    the sample points xpts (uneven spacing when ``uneven``), for every f in
    ``frequency``.  fpts may hold several profiles as rows."""
    from scipy.integrate import simpson
    freqs = np.asarray(frequency, dtype=np.float64)
    xpts = np.asarray(xpts, dtype=np.float64)
    fpts = np.asarray(fpts)
    if uneven is None:
        d = np.diff(xpts.ravel())
        uneven = not np.allclose(d, d[0])
    if fpts.ndim > 1:
        out = np.empty((fpts.shape[0], freqs.size), dtype=np.complex128)
        xr = np.reshape(xpts, (1, xpts.size))
    else:
        out = np.empty((freqs.size,), dtype=np.complex128)
        xr = xpts
    for i, f in enumerate(freqs):
        y = fpts * np.exp(-2.0 * np.pi * 1j * xr * f)
        if uneven:
            out[..., i] = simpson(y, x=xpts.ravel(), axis=-1)
        else:
            out[..., i] = simpson(y, dx=xpts.flat[1] - xpts.flat[0], axis=-1)
    return out


__all__ = ['discreteSimpson']
