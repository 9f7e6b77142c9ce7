"""Materials of a voxelized sample (xopto/mcbase/mcmaterial.py:32-309,
656-878).  Material 0 is the medium surrounding the voxel box."""
from .. import _abi
from . import mcpf


class Material:
    def __init__(self, n=1.0, mua=0.0, mus=0.0, pf=None):
        if isinstance(n, Material):
            other = n
            n, mua, mus, pf = other.n, other.mua, other.mus, other.pf
        self._n, self._mua, self._mus = float(n), float(mua), float(mus)
        self._pf = pf if pf is not None else mcpf.Hg(0.0)

    def _set_n(self, v):
        self._n = float(v)

    def _set_mua(self, v):
        self._mua = float(v)

    def _set_mus(self, v):
        self._mus = float(v)

    def _set_pf(self, pf):
        if type(pf) != type(self._pf):
            raise ValueError('The scattering phase function type of the material must not change!')
        self._pf = pf

    n = property(lambda self: self._n, _set_n)
    mua = property(lambda self: self._mua, _set_mua)
    mus = property(lambda self: self._mus, _set_mus)
    pf = property(lambda self: self._pf, _set_pf)

    def pack(self, mc, target: _abi.McgbMaterial):
        """mcmaterial.py:240-276: inv_mut = 1/(mua+mus) (inf when 0) and
        mua_inv_mut = mua*inv_mut (1 when mus is 0)."""
        mut = self._mua + self._mus
        inv_mut = 1.0 / mut if mut > 0.0 else float('inf')
        mua_inv_mut = 1.0 if self._mus == 0.0 else self._mua * inv_mut
        target.n = self._n
        target.mua = self._mua
        target.mus = self._mus
        target.inv_mut = inv_mut
        target.mua_inv_mut = mua_inv_mut
        self._pf.pack(mc, target.pf)
        return target

    def todict(self):
        return {'n': self._n, 'mua': self._mua, 'mus': self._mus,
                'pf': self._pf.todict(), 'type': 'Material'}

    def __str__(self):
        return 'Material(n={}, mua={}, mus={}, pf={})'.format(self._n, self._mua, self._mus, self._pf)

    __repr__ = __str__


class Materials:
    def __init__(self, materials):
        if isinstance(materials, Materials):
            materials = [Material(m) for m in materials]
        materials = list(materials)
        if len(materials) < 2:
            raise ValueError('At least two materials (surrounding medium and one sample '
                             'material) are required!')
        if len(materials) > _abi.MAX_MATERIALS:
            raise ValueError('At most {} materials are supported (uint8 voxel '
                             'indices)!'.format(_abi.MAX_MATERIALS))
        pf_type = type(materials[0].pf)
        for m in materials:
            if type(m.pf) != pf_type:
                raise ValueError('All materials must use the same scattering phase function type!')
        self._materials = materials

    def __getitem__(self, i):
        return self._materials[i]

    def __len__(self):
        return len(self._materials)

    def __iter__(self):
        return iter(self._materials)

    def material(self, index):
        return self._materials[index]

    def surrounding(self):
        return self._materials[0]

    def __str__(self):
        return 'Materials([{}])'.format(', '.join(str(m) for m in self._materials))
