"""Sample layers (xopto/mcml/mclayer/layer.py:35-1065)."""
import numpy as np

from .. import _abi
from ..mcbase import mcpf
from ..mcbase.mcutil import cos_critical


class Layer:
    """Layer(d, n, mua, mus, pf): thickness d (m), refractive index n,
    absorption mua and scattering mus coefficients (1/m)."""

    def __init__(self, d, n=None, mua=None, mus=None, pf=None):
        if isinstance(d, Layer):
            other = d
            d, n, mua, mus, pf = other.d, other.n, other.mua, other.mus, other.pf
        self._d, self._n, self._mua, self._mus = float(d), float(n), float(mua), float(mus)
        self._pf = pf

    def _set_d(self, v):
        self._d = float(v)

    def _set_n(self, v):
        self._n = float(v)

    def _set_mua(self, v):
        self._mua = float(v)

    def _set_mus(self, v):
        self._mus = float(v)

    def _set_pf(self, pf):
        if type(self._pf) != type(pf):
            raise ValueError('The scattering phase function type of the layer must not change!')
        self._pf = pf

    d = property(lambda self: self._d, _set_d, None, 'Layer thickness (m).')
    n = property(lambda self: self._n, _set_n, None, 'Refractive index.')
    mua = property(lambda self: self._mua, _set_mua, None, 'Absorption coefficient (1/m).')
    mus = property(lambda self: self._mus, _set_mus, None, 'Scattering coefficient (1/m).')
    pf = property(lambda self: self._pf, _set_pf, None, 'Phase function object.')

    def pack(self, mc, target: _abi.McgbLayer):
        """Fields that do not depend on the neighbours (layer.py:304-354)."""
        mut = self._mua + self._mus
        inv_mut = 1.0 / mut if mut > 0.0 else float('inf')
        mua_inv_mut = 1.0 if self._mus == 0.0 else self._mua * inv_mut
        target.thickness = self._d
        target.n = self._n
        target.mua = self._mua
        target.mus = self._mus
        target.inv_mut = inv_mut
        target.mua_inv_mut = mua_inv_mut
        self._pf.pack(mc, target.pf)
        return target

    def todict(self):
        return {'d': self._d, 'n': self._n, 'mua': self._mua, 'mus': self._mus,
                'pf': self._pf.todict(), 'type': 'Layer'}

    @classmethod
    def fromdict(cls, data):
        data = dict(data)
        data.pop('type', None)
        pf = mcpf.pf_fromdict(data.pop('pf'))
        return cls(pf=pf, **data)

    def __str__(self):
        return 'Layer(d={}, n={}, mua={}, mus={}, pf={})'.format(
            self._d, self._n, self._mua, self._mus, self._pf)

    __repr__ = __str__


class Layers:
    """Layer stack; the first and last layers are the surrounding half-spaces
    (xopto/mcml/mclayer/layer.py:793-1065)."""

    def __init__(self, layers):
        if isinstance(layers, Layers):
            layers = [Layer(l) for l in layers]
        self._layers = list(layers)

    def check(self):
        if len(self._layers) < 3:
            raise ValueError('The layer stack must include at least 3 layers (two '
                             'surrounding media and one sample layer)!')
        if len(self._layers) > _abi.MAX_LAYERS:
            raise ValueError('At most {} layers are supported!'.format(_abi.MAX_LAYERS))
        pf_type = type(self._layers[0].pf)
        for l in self._layers:
            if type(l.pf) != pf_type:
                raise ValueError('All layers must use the same scattering phase function type!')
        return True

    def __getitem__(self, i):
        return self._layers[i]

    def __len__(self):
        return len(self._layers)

    def __iter__(self):
        return iter(self._layers)

    def thickness(self) -> float:
        return float(np.sum([l.d for l in self._layers[1:-1]]))

    def pack(self, mc, targets):
        """Top/bottom z and critical cosines (layer.py:944-1007).  The running
        z is read back from the float32 field, as the reference does."""
        n_layers = len(self._layers)
        for i, layer in enumerate(self._layers):
            t = targets[i]
            layer.pack(mc, t)
            cc_top = cc_bottom = 0.0
            if i > 0:
                cc_top = cos_critical(layer.n, self._layers[i - 1].n)
            if i + 1 < n_layers:
                cc_bottom = cos_critical(layer.n, self._layers[i + 1].n)
            if i == 0:
                t.top = -float('inf')
                t.bottom = 0.0
                t.thickness = float('inf')
            elif i == n_layers - 1:
                t.top = targets[i - 1].bottom
                t.bottom = float('inf')
                t.thickness = float('inf')
            else:
                t.top = targets[i - 1].bottom
                t.bottom = targets[i - 1].bottom + layer.d
            t.cos_critical_top = cc_top
            t.cos_critical_bottom = cc_bottom
        return targets

    def __str__(self):
        return 'Layers([\n    {}\n])'.format(',\n    '.join(str(l) for l in self._layers))

    __repr__ = __str__
