"""Optical fibre parameters (xopto/mcbase/mcutil/fiber.py:38-224,
MultimodeFiber) and the placement of a fibre in a probe (fiber.py:381-470,
FiberLayout)."""
import numpy as np


class MultimodeFiber:
    """Multimode fibre: core and cladding diameters (m), core refractive
    index and numerical aperture; the cladding index follows from
    NA = sqrt(ncore^2 - ncladding^2)."""

    @staticmethod
    def compute_na(ncore: float, ncladding: float) -> float:
        return (ncore ** 2 - ncladding ** 2) ** 0.5

    @staticmethod
    def compute_ncladding(ncore: float, na: float) -> float:
        return (ncore ** 2 - na ** 2) ** 0.5

    def __init__(self, dcore: float, dcladding: float, ncore: float, na: float):
        self._dcore = float(dcore)
        self._dcladding = float(dcladding)
        self._ncore = float(ncore)
        self._na = float(na)

    def validate(self):
        if self._dcore > self._dcladding:
            raise ValueError('Fiber core diameter must be smaller than the fiber cladding diameter!')

    def _set_dcore(self, v):
        self._dcore = float(v)

    def _set_dcladding(self, v):
        self._dcladding = float(v)

    def _set_ncore(self, v):
        self._ncore = float(v)

    def _set_na(self, v):
        self._na = float(v)

    dcore = property(lambda self: self._dcore, _set_dcore, None, 'Diameter (m) of the fiber core.')
    dcladding = property(lambda self: self._dcladding, _set_dcladding, None,
                         'Diameter (m) of the fiber cladding.')
    ncore = property(lambda self: self._ncore, _set_ncore, None, 'Refractive index of the fiber core.')
    ncladding = property(lambda self: self.compute_ncladding(self._ncore, self._na), None, None,
                         'Refractive index of the fiber cladding.')
    na = property(lambda self: self._na, _set_na, None, 'Numerical aperture of the fiber core.')

    def todict(self) -> dict:
        return {'type': 'MultimodeFiber', 'dcore': self._dcore, 'dcladding': self._dcladding,
                'ncore': self._ncore, 'na': self._na}

    @staticmethod
    def fromdict(data: dict) -> 'MultimodeFiber':
        data = dict(data)
        data.pop('type', None)
        return MultimodeFiber(**data)

    def __str__(self):
        return 'MultimodeFiber(dcore={}, dcladding={}, ncore={}, na={})'.format(
            self._dcore, self._dcladding, self._ncore, self._na)

    __repr__ = __str__


class FiberLayout:
    """A fibre of a probe: the fibre, the position of its tip centre and its
    direction (xopto/mcbase/mcutil/fiber.py:381-470)."""

    def __init__(self, fiber, position=(0.0, 0.0, 0.0), direction=(0.0, 0.0, 1.0)):
        if isinstance(fiber, FiberLayout):
            fiber, position, direction = fiber.fiber, fiber.position, fiber.direction
        self._fiber = fiber
        self._position = np.zeros((3,))
        self._direction = np.array((0.0, 0.0, 1.0))
        self.position = position
        self.direction = direction

    def _set_position(self, p):
        self._position[:] = p

    def _set_direction(self, d):
        self._direction[:] = d
        n = np.linalg.norm(self._direction)
        if n == 0.0:
            raise ValueError('Fiber direction vector norm/length must not be 0!')
        self._direction *= 1.0 / n

    fiber = property(lambda self: self._fiber)
    position = property(lambda self: self._position, _set_position)
    direction = property(lambda self: self._direction, _set_direction)

    def todict(self):
        return {'type': 'FiberLayout', 'fiber': self._fiber.todict(),
                'position': self._position.tolist(), 'direction': self._direction.tolist()}

    def __str__(self):
        return 'FiberLayout(fiber={}, position=({}, {}, {}), direction=({}, {}, {}))'.format(
            self._fiber, *self._position, *self._direction)

    __repr__ = __str__


class MultimodeFiberLut:
    """Multimode fibre whose emission and collection are given by look-up
    tables (xopto/mcbase/mcutil/fiber.py:224-420)."""

    def __init__(self, dcore: float, dcladding: float, ncore: float, ncladding: float = None,
                 emission=None, collection=None):
        from .lut import EmissionLut, CollectionLut
        if isinstance(dcore, MultimodeFiberLut):
            o = dcore
            dcore, dcladding, ncore, ncladding = o.dcore, o.dcladding, o.ncore, o.ncladding
            emission, collection = o.emission, o.collection
        self._dcore = float(dcore)
        self._dcladding = float(dcladding)
        self._ncore = float(ncore)
        self._ncladding = self._ncore if ncladding is None else float(ncladding)
        if isinstance(emission, str):
            emission = EmissionLut(emission)
        elif isinstance(emission, np.ndarray):
            emission = EmissionLut(emission)
        if isinstance(collection, str):
            collection = CollectionLut(collection)
        self._emission = emission
        self._collection = collection

    def validate(self):
        if self._dcore > self._dcladding:
            raise ValueError('Fiber core diameter must be smaller than the fiber cladding diameter!')

    def _set_dcore(self, v):
        self._dcore = float(v)

    def _set_dcladding(self, v):
        self._dcladding = float(v)

    def _set_ncore(self, v):
        self._ncore = float(v)

    dcore = property(lambda self: self._dcore, _set_dcore, None, 'Core diameter (m).')
    dcladding = property(lambda self: self._dcladding, _set_dcladding, None, 'Cladding diameter (m).')
    ncore = property(lambda self: self._ncore, _set_ncore, None, 'Core refractive index.')
    ncladding = property(lambda self: self._ncladding, None, None, 'Cladding refractive index.')
    emission = property(lambda self: self._emission, None, None, 'Emission look-up table.')
    collection = property(lambda self: self._collection, None, None, 'Collection look-up table.')

    def todict(self) -> dict:
        return {'type': 'MultimodeFiberLut', 'dcore': self._dcore, 'dcladding': self._dcladding,
                'ncore': self._ncore, 'emission': self._emission, 'collection': self._collection}

    def __repr__(self):
        return 'MultimodeFiberLut(dcore={:f}, dcladding={:f}, ncore={:f}, emission={}, ' \
               'collection={})'.format(self._dcore, self._dcladding, self._ncore, self._emission,
                                       self._collection)

    __str__ = __repr__
