"""Scattering phase functions: Henyey-Greenstein, Gegenbauer kernel, lookup
table, the analytic mixtures Hg2, MHg, Pc, MPc, MGk and Gk2, the
anisotropic Hga and the directional HgDir, with the reference's names and
parameters (xopto/mcbase/mcpf/hg.py, gk.py, lut.py, hg2.py, mhg.py, pc.py,
mpc.py, mgk.py, gk2.py, hga.py, hgdir.py).

Each object packs itself into the ``McgbPf`` struct that the GB300 kernels
read from their shared-memory layer/material table.
"""
import numpy as np

from .. import _abi


class PfBase:
    kind = None

    def pack(self, mc, target: _abi.McgbPf):
        raise NotImplementedError

    def todict(self) -> dict:
        raise NotImplementedError

    @classmethod
    def fromdict(cls, data: dict):
        data = dict(data)
        data.pop('type', None)
        return cls(**data)

    def __repr__(self):
        return str(self)


class Hg(PfBase):
    """Henyey-Greenstein phase function (xopto/mcbase/mcpf/hg.py:25-167)."""
    kind = _abi.PF_HG

    def __init__(self, g: float):
        self._g = 0.0
        self.g = g

    def _get_g(self):
        return self._g

    def _set_g(self, g):
        self._g = min(max(float(g), -1.0), 1.0)

    g = property(_get_g, _set_g, None, 'Anisotropy factor.')

    def pack(self, mc, target):
        target.p[0] = self._g
        return target

    def todict(self):
        return {'g': self._g, 'type': 'Hg'}

    def __str__(self):
        return 'Hg(g={})'.format(self._g)


class Gk(PfBase):
    """Gegenbauer kernel phase function (xopto/mcbase/mcpf/gk.py:30-243).
    The sampling constants inv_a, a1, a2 are precomputed on the host as in
    gk.py:153-178."""
    kind = _abi.PF_GK

    def __init__(self, g: float, a: float):
        self._g = min(max(float(g), -1.0), 1.0)
        self._a = max(float(a), -0.5)
        self._recalculate()

    def _recalculate(self):
        g, a = self._g, self._a
        if g == 0:
            inv_a = a1 = a2 = 0.0
        elif a == 0:
            a1 = (1 + g ** 2) / (2 * g)
            a2 = (1 + 2 * g + g ** 2) / (2 * g)
            inv_a = 0.0
        else:
            temp = a * g * (1.0 - g * g) ** (2.0 * a)
            temp = temp / (np.pi * ((1.0 + g) ** (2.0 * a) - (1.0 - g) ** (2.0 * a)))
            a1 = 2.0 * a * g / (2.0 * np.pi * temp)
            a2 = (1 + g) ** (-2.0 * a)
            inv_a = 1.0 / a
        self._precalculated = [inv_a, a1, a2]

    def _get_g(self):
        return self._g

    def _set_g(self, g):
        self._g = min(max(float(g), -1.0), 1.0)
        self._recalculate()

    g = property(_get_g, _set_g, None, 'Anisotropy factor when a=0.5.')

    def _get_a(self):
        return self._a

    def _set_a(self, a):
        self._a = max(float(a), -0.5)
        self._recalculate()

    a = property(_get_a, _set_a, None, 'Parameter alpha.')

    def pack(self, mc, target):
        target.p[0] = self._g
        target.p[1] = self._a
        target.p[2] = self._precalculated[0]
        target.p[3] = self._precalculated[1]
        target.p[4] = self._precalculated[2]
        return target

    def todict(self):
        return {'g': self._g, 'a': self._a, 'type': 'Gk'}

    def __str__(self):
        return 'Gk(g={}, a={})'.format(self._g, self._a)


class Lut(PfBase):
    """Lookup-table phase function with the nonlinear index transform
    index = (a/(xi - c) - b + 1)*(N - 1)/2 (xopto/mcbase/mcpf/lut.py:31-260).
    The table is appended to the simulator's floating-point LUT buffer."""
    kind = _abi.PF_LUT

    def __init__(self, params, lut):
        self._params = np.zeros((3,))
        self._params[:] = params
        self._lut = np.asarray(lut, dtype=np.float64).ravel()
        if self._lut.size < 2:
            raise ValueError('A lookup table needs at least two entries!')
        self._offset = 0

    params = property(lambda self: self._params)
    lut = property(lambda self: self._lut)
    size = property(lambda self: self._lut.size)
    offset = property(lambda self: self._offset)

    def pack(self, mc, target):
        self._offset = mc.append_r_lut(self._lut)
        target.p[0] = self._params[0]
        target.p[1] = self._params[1]
        target.p[2] = self._params[2]
        target.lut_offset = self._offset
        target.lut_size = self._lut.size
        return target

    def todict(self):
        return {'params': list(self._params), 'lut': self._lut.tolist(), 'type': 'Lut'}

    def __str__(self):
        return 'Lut(params=({}, {}, {}), size={})'.format(*self._params, self._lut.size)


def _clip_g(g):
    return min(max(float(g), -1.0), 1.0)


class _Ext(PfBase):
    """Analytic samplers that share the MCGB_PF_EXT kernels; ``ext_kind``
    selects the sampler and ``_params`` fills McgbPf.p in order."""
    kind = _abi.PF_EXT
    ext_kind = None
    _names = ()

    def _params(self):
        return [getattr(self, name) for name in self._names]

    def pack(self, mc, target):
        for i, value in enumerate(self._params()):
            target.p[i] = value
        target.ext_kind = self.ext_kind
        return target

    def todict(self):
        d = {name: getattr(self, name) for name in self._names}
        d['type'] = type(self).__name__
        return d

    def __str__(self):
        return '{}({})'.format(type(self).__name__, ', '.join(
            '{}={}'.format(name, getattr(self, name)) for name in self._names))


class Hg2(_Ext):
    """Mixture of two Henyey-Greenstein phase functions,
    (1 - b)*Hg(g1) + b*Hg(g2) (xopto/mcbase/mcpf/hg2.py:25-231)."""
    ext_kind = _abi.PF_EXT_HG2
    _names = ('g1', 'g2', 'b')

    def __init__(self, g1: float, g2: float, b: float):
        self.g1, self.g2, self.b = g1, g2, b

    g1 = property(lambda self: self._g1, lambda self, g: setattr(self, '_g1', _clip_g(g)),
                  None, 'Anisotropy factor of the first component.')
    g2 = property(lambda self: self._g2, lambda self, g: setattr(self, '_g2', _clip_g(g)),
                  None, 'Anisotropy factor of the second component.')
    b = property(lambda self: self._b, lambda self, b: setattr(self, '_b', float(b)),
                 None, 'Contribution of the second component.')


class MHg(_Ext):
    """Modified Henyey-Greenstein phase function,
    b*Hg(g) + (1 - b)*(3/2)cos^2 (xopto/mcbase/mcpf/mhg.py:25-195)."""
    ext_kind = _abi.PF_EXT_MHG
    _names = ('g', 'b')

    def __init__(self, g: float, b: float):
        self.g, self.b = g, b

    g = property(lambda self: self._g, lambda self, g: setattr(self, '_g', _clip_g(g)),
                 None, 'Anisotropy factor of the Henyey-Greenstein component.')
    b = property(lambda self: self._b, lambda self, b: setattr(self, '_b', float(b)),
                 None, 'Contribution of the Henyey-Greenstein component.')


class Pc(_Ext):
    """Power of cosines phase function, cos(theta/2)^(2n)
    (xopto/mcbase/mcpf/pc.py:25-186)."""
    ext_kind = _abi.PF_EXT_PC
    _names = ('n',)

    def __init__(self, n: float):
        self.n = n

    n = property(lambda self: self._n, lambda self, n: setattr(self, '_n', float(n)),
                 None, 'Power of the cosine.')


class MPc(_Ext):
    """Modified power of cosines phase function,
    b*Pc(n) + (1 - b)*(3/2)cos^2 (xopto/mcbase/mcpf/mpc.py:25-196)."""
    ext_kind = _abi.PF_EXT_MPC
    _names = ('n', 'b')

    def __init__(self, n: float, b: float):
        self.n, self.b = n, b

    n = property(lambda self: self._n, lambda self, n: setattr(self, '_n', float(n)),
                 None, 'Power of the cosine.')
    b = property(lambda self: self._b, lambda self, b: setattr(self, '_b', float(b)),
                 None, 'Contribution of the power of cosines component.')


class MGk(Gk):
    """Modified Gegenbauer kernel phase function,
    b*Gk(g, a) + (1 - b)*(3/2)cos^2 (xopto/mcbase/mcpf/mgk.py:31-270).  The
    constants inv_a, a1, a2 are the Gk ones (mgk.py:195-215).  The sampler
    tells a == 0 by inv_a == 0, which is the same test for |a| >= 1.2e-38."""
    kind = _abi.PF_EXT
    ext_kind = _abi.PF_EXT_MGK

    def __init__(self, g: float, a: float, b: float):
        self._b = float(b)
        super().__init__(g, a)

    b = property(lambda self: self._b, lambda self, b: setattr(self, '_b', float(b)),
                 None, 'Contribution of the Gegenbauer kernel component.')

    def pack(self, mc, target):
        inv_a, a1, a2 = self._precalculated
        for i, value in enumerate((self.g, self._b, inv_a, a1, a2)):
            target.p[i] = value
        target.ext_kind = self.ext_kind
        return target

    def todict(self):
        return {'g': self.g, 'a': self.a, 'b': self._b, 'type': 'MGk'}

    def __str__(self):
        return 'MGk(g={}, a={}, b={})'.format(self.g, self.a, self._b)


class Gk2(PfBase):
    """Mixture of two Gegenbauer kernel phase functions,
    (1 - b)*Gk(g1, a1) + b*Gk(g2, a2), the first forward (0 <= g1 <= 1), the
    second backward (-1 <= g2 <= 0) (xopto/mcbase/mcpf/gk2.py:30-300).  The
    eleven packed floats (each term's g, a and its Gk sampling constants,
    then b) go to the simulator's float LUT."""
    kind = _abi.PF_EXT
    ext_kind = _abi.PF_EXT_GK2

    def __init__(self, g1: float, a1: float, g2: float, a2: float, b: float):
        self._gk1 = Gk(min(max(float(g1), 0.0), 1.0), a1)
        self._gk2 = Gk(min(max(float(g2), -1.0), 0.0), a2)
        self._b = min(max(float(b), 0.0), 1.0)

    g1 = property(lambda self: self._gk1.g,
                  lambda self, g: setattr(self._gk1, 'g', min(max(float(g), 0.0), 1.0)),
                  None, 'Parameter g of the first (forward) term.')
    a1 = property(lambda self: self._gk1.a, lambda self, a: setattr(self._gk1, 'a', a),
                  None, 'Parameter alpha of the first term.')
    g2 = property(lambda self: self._gk2.g,
                  lambda self, g: setattr(self._gk2, 'g', min(max(float(g), -1.0), 0.0)),
                  None, 'Parameter g of the second (backward) term.')
    a2 = property(lambda self: self._gk2.a, lambda self, a: setattr(self._gk2, 'a', a),
                  None, 'Parameter alpha of the second term.')
    b = property(lambda self: self._b,
                 lambda self, b: setattr(self, '_b', min(max(float(b), 0.0), 1.0)),
                 None, 'Relative contribution of the second term.')

    def params(self):
        out = []
        for gk in (self._gk1, self._gk2):
            out += [gk.g, gk.a] + list(gk._precalculated)
        return out + [self._b]

    def pack(self, mc, target):
        target.lut_offset = mc.append_r_lut(np.asarray(self.params(), dtype=np.float32))
        target.lut_size = _abi.PF_GK2_FLOATS
        target.ext_kind = self.ext_kind
        return target

    def todict(self):
        return {'g1': self.g1, 'a1': self.a1, 'g2': self.g2, 'a2': self.a2, 'b': self._b,
                'type': 'Gk2'}

    def __str__(self):
        return 'Gk2(g1={}, a1={}, g2={}, a2={}, b={})'.format(self.g1, self.a1, self.g2, self.a2,
                                                            self._b)


class Hga(PfBase):
    """Anisotropic Henyey-Greenstein phase function: the anisotropy factor
    is the projection p^T G p of the 3x3 tensor G on the propagation
    direction p (xopto/mcbase/mcpf/hga.py:25-200).  A scalar g gives
    G = g I; three values the diagonal.  The nine tensor floats go to the
    simulator's float LUT."""
    kind = _abi.PF_EXT
    ext_kind = _abi.PF_EXT_HGA

    def __init__(self, g):
        self._g = np.zeros((3, 3))
        self.g = g

    def _get_g(self):
        return self._g

    def _set_g(self, g):
        if isinstance(g, (float, int)):
            v = min(max(float(g), -1.0), 1.0)
            self._g[0, 0] = self._g[1, 1] = self._g[2, 2] = v
        else:
            g = np.asarray(g, dtype=float)
            if g.size == 3:
                g = np.clip(g, -1.0, 1.0)
                self._g[0, 0], self._g[1, 1], self._g[2, 2] = g.ravel()
            else:
                self._g[:] = np.clip(g.reshape(3, 3), -1.0, 1.0)

    g = property(_get_g, _set_g, None, 'Anisotropy tensor.')

    def pack(self, mc, target):
        target.lut_offset = mc.append_r_lut(np.asarray(self._g, dtype=np.float32).ravel())
        target.lut_size = _abi.PF_HGA_FLOATS
        target.ext_kind = self.ext_kind
        return target

    def todict(self):
        return {'g': self._g.tolist(), 'type': 'Hga'}

    def __str__(self):
        return 'Hga(g={})'.format(self._g.tolist())


class HgDir(PfBase):
    """Directional Henyey-Greenstein phase function: with probability p the
    packet scatters about the fixed unit ``direction`` (the polar angle
    turned so that the new direction stays on the side of the packet's
    current one), otherwise about its current direction
    (xopto/mcbase/mcpf/hgdir.py:25-230)."""
    kind = _abi.PF_EXT
    ext_kind = _abi.PF_EXT_HGDIR

    def __init__(self, g: float, direction=(0.0, 0.0, 1.0), p: float = 1.0):
        self._direction = np.array((0.0, 0.0, 1.0))
        self.direction = direction
        self.g = g
        self.p = p

    g = property(lambda self: self._g,
                 lambda self, g: setattr(self, '_g', min(max(float(g), -1.0), 1.0)),
                 None, 'Anisotropy factor.')
    p = property(lambda self: self._p,
                 lambda self, p: setattr(self, '_p', min(max(float(p), 0.0), 1.0)),
                 None, 'Probability of directional scattering.')

    def _get_direction(self):
        return self._direction

    def _set_direction(self, direction):
        d = np.asarray(direction, dtype=float).ravel()
        norm = np.linalg.norm(d)
        if norm == 0.0:
            raise ValueError('The norm/length of the scattering direction vector must not be 0!')
        self._direction[:] = d / norm

    direction = property(_get_direction, _set_direction, None, 'Scattering direction.')

    def pack(self, mc, target):
        for i, value in enumerate(list(self._direction) + [self._g, self._p]):
            target.p[i] = value
        target.ext_kind = self.ext_kind
        return target

    def todict(self):
        return {'g': self._g, 'direction': self._direction.tolist(), 'p': self._p, 'type': 'HgDir'}

    def __str__(self):
        return 'HgDir(g={}, direction={}, p={})'.format(self._g, self._direction.tolist(), self._p)


def pf_fromdict(data: dict) -> PfBase:
    kinds = {'Hg': Hg, 'Gk': Gk, 'Lut': Lut, 'Hg2': Hg2, 'MHg': MHg, 'Pc': Pc, 'MPc': MPc,
             'MGk': MGk, 'Gk2': Gk2, 'Hga': Hga, 'HgDir': HgDir}
    return kinds[data['type']].fromdict(data)
