"""Reflectance collected through optical fibres from a radial reflectance
profile (xopto/util/convolve.py:27-133, fiber_reflectance).

For a fibre of radius r_c centred at distance sds from the source, the
collected reflectance is

    2 * integral_{max(sds - r_c, 0)}^{sds + r_c}
          arccos((r^2 + sds^2 - r_c^2) / (2 r sds)) R(r) r dr

(2*pi*integral R(r) r dr over [0, r_c] for sds = 0), evaluated with
Simpson's rule on an even grid of ``nsimps`` points and the profile
interpolated linearly (or in log space) from its sample points.
"""
import numpy as np
from scipy.integrate import simpson
from scipy.interpolate import interp1d


def fiber_reflectance(r: np.ndarray, reflectance: np.ndarray, sds, dcore: float,
                      nsimps: int = 1000, loginterp: bool = False, uneven: bool = False,
                      **kwargs) -> np.ndarray:
    """Reflectance through fibres at source-detector separations ``sds``.

    r: sorted sample points of the radial profile (covering
    [sds - dcore/2, sds + dcore/2]); reflectance: the profile, or a 2-D array
    with one profile per row.  Returns (num_profiles, len(sds))."""
    if isinstance(sds, (float, int)):
        sds = (float(sds),)
    rfib = 0.5 * dcore
    nsimps = max(nsimps // 2 * 2 + 1, 3)
    reflectance = np.asarray(reflectance)
    nrefl = reflectance.shape[0] if reflectance.ndim > 1 else 1
    values = np.log(reflectance) if loginterp else reflectance
    f = interp1d(r, values, assume_sorted=True, bounds_error=False, fill_value='extrapolate',
                 **kwargs)
    out = np.zeros((nrefl, len(sds)))
    for i, d in enumerate(sds):
        rs = np.linspace(max(d - rfib, 0.0), max(d + rfib, 0.0), nsimps)
        kw = {'x': rs} if uneven else {'dx': rs[1] - rs[0]}
        fs = f(rs)
        if loginterp:
            fs = np.exp(fs)
        if d == 0.0:
            out[:, i] = 2.0 * np.pi * simpson(fs * rs, **kw)
        else:
            d_rs = rs * d
            d_rs[d_rs == 0.0] = np.finfo(np.float64).tiny
            cos_a = np.clip((rs ** 2 + d ** 2 - rfib ** 2) / (2.0 * d_rs), -1.0, 1.0)
            out[:, i] = 2.0 * simpson(np.arccos(cos_a) * fs * rs, **kw)
    return out
