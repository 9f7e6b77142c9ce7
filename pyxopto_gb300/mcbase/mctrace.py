"""Photon packet trace and trace filter (xopto/mcbase/mctrace.py:53-1234).

Each packet records up to ``maxlen`` events of 8 floats
(x, y, z, px, py, pz, w, optical path length); when the trace is full the
last slot is overwritten, and the per-packet event count is stored in the
integer buffer (mctrace.py:541-583).  Results of successive runs with
``out=`` are appended; a ``Filter`` keeps only the packets whose final
state matches it (mctrace.py:216-330)."""
from typing import Tuple

import numpy as np

from .. import _abi


def _range(value) -> Tuple[float, float]:
    if not isinstance(value, (list, tuple)) or len(value) != 2:
        raise TypeError('Range must be specified as a tuple of two float: (low, high)!')
    return float(value[0]), float(value[1])


def _origin2(value) -> Tuple[float, float]:
    if not isinstance(value, (list, tuple)) or len(value) != 2:
        raise TypeError('Origin must be specified as a tuple of two float: (x, y)!')
    return float(value[0]), float(value[1])


def _dir3(value, k: float = 1.0) -> Tuple[float, float, float]:
    if not isinstance(value, (list, tuple)) or len(value) != 3:
        raise TypeError('Direction must be specified as a tuple of three float: (x, y, z)!')
    k = float(k)
    return float(value[0]) * k, float(value[1]) * k, float(value[2]) * k


class Filter:
    """Selects traced packets by their final state; the criteria are joined
    by a logical and, the intervals of one criterion by a logical or
    (xopto/mcbase/mctrace.py:53-441).  Interval bounds are inclusive."""

    def __init__(self, x=None, y=None, z=None, pz=None, r=None, dir=None, pl=None):
        if isinstance(x, Filter):
            f = x
            x, y, z, pz, r, dir, pl = f.x, f.y, f.z, f.pz, f.r, f.dir, f.pl
        self._x = self._check_range('x', x) if x is not None else None
        self._y = self._check_range('y', y) if y is not None else None
        self._z = self._check_range('z', z) if z is not None else None
        self._pz = self._check_range('pz', pz) if pz is not None else None
        self._r = self._check_r(r) if r is not None else None
        self._dir = self._check_dir(dir) if dir is not None else None
        self._pl = self._check_range('pl', pl) if pl is not None else None

    x = property(lambda self: self._x)
    y = property(lambda self: self._y)
    z = property(lambda self: self._z)
    pz = property(lambda self: self._pz)
    r = property(lambda self: self._r)
    dir = property(lambda self: self._dir)
    pl = property(lambda self: self._pl)

    def todict(self) -> dict:
        return {'type': 'Filter', 'x': self._x, 'y': self._y, 'z': self._z, 'pz': self._pz,
                'r': self._r, 'dir': self._dir, 'pl': self._pl}

    @classmethod
    def fromdict(cls, data: dict) -> 'Filter':
        d = dict(data)
        t = d.pop('type')
        if t != cls.__name__:
            raise TypeError('Expected data for type "{}" but got "{}"!'.format(cls.__name__, t))
        return cls(**d)

    def __call__(self, trace_obj: 'Trace', update: bool = True) -> Tuple['Trace', int]:
        """Returns (filtered trace, number of matching packets dropped
        because their trace overflowed).  The optical path-length criterion
        applies only to traces with ``plon``; like the reference
        (mctrace.py:302-309) it does not reset the or-mask of the criterion
        before it."""
        if not isinstance(trace_obj, Trace):
            raise TypeError('Trace filter can be applied only to Trace objects!')
        term = trace_obj.terminal
        too_long = trace_obj.overflow
        valid = np.ones_like(too_long)
        var = np.zeros_like(valid)

        def apply(intervals, test, reset=True):
            nonlocal valid
            if reset:
                var.fill(0)
            for item in intervals:
                np.logical_or(np.logical_and(test(item), valid), var, out=var)
            np.logical_and(var, valid, out=valid)

        if self._x is not None:
            apply(self._x, lambda rg: (term['x'] >= rg[0]) & (term['x'] <= rg[1]), reset=False)
        if self._y is not None:
            apply(self._y, lambda rg: (term['y'] >= rg[0]) & (term['y'] <= rg[1]))
        if self._z is not None:
            apply(self._z, lambda rg: (term['z'] >= rg[0]) & (term['z'] <= rg[1]))
        if self._pz is not None:
            apply(self._pz, lambda rg: (term['pz'] >= rg[0]) & (term['pz'] <= rg[1]))
        if self._r is not None:
            def r_test(item):
                x = term['x'] - item[2][0]
                y = term['y'] - item[2][1]
                rr = x ** 2 + y ** 2
                return (rr >= item[0] ** 2) & (rr <= item[1] ** 2)
            apply(self._r, r_test)
        if self._dir is not None:
            def dir_test(item):
                v = item[2]
                c = term['px'] * v[0] + term['py'] * v[1] + term['pz'] * v[2]
                return (c >= item[0]) & (c <= item[1])
            apply(self._dir, dir_test)
        if self._pl is not None and trace_obj.plon:
            apply(self._pl, lambda rg: (term['pl'] >= rg[0]) & (term['pl'] <= rg[1]), reset=False)
        selected = np.logical_and(valid, np.logical_not(too_long))
        n_dropped = int(np.count_nonzero(np.logical_and(valid, too_long)))
        out = trace_obj if update else Trace(trace_obj)
        out.data = trace_obj.data[selected, :]
        out.n = trace_obj.n[selected]
        return out, n_dropped

    @staticmethod
    def _check_range(param, value):
        if not isinstance(value, (list, tuple)):
            raise TypeError('Filter parameter {} must be a tuple of two float values (low, high), '
                            'or a list of such tuples!'.format(param))
        if isinstance(value[0], (list, tuple)):
            return [_range(item) for item in value]
        return (_range(value),)

    @staticmethod
    def _check_r(r):
        if not isinstance(r, (list, tuple)):
            raise TypeError('Filter parameter r must be a tuple (rmin, rmax, (x_origin, y_origin)) '
                            'or a list or tuple of such tuples!')

        def one(item):
            origin = _origin2(item[2]) if len(item) > 2 else (0.0, 0.0)
            return float(item[0]), float(item[1]), origin
        if isinstance(r[0], (list, tuple)):
            return [one(item) for item in r]
        return (one(r),)

    @staticmethod
    def _check_dir(d):
        if not isinstance(d, (list, tuple)):
            raise TypeError('Filter parameter dir must be a tuple (cosmin, cosmax, (px, py, pz)) '
                            'or a list or tuple of such tuples!')

        def one(item):
            p = item[2]
            n = float(np.sqrt(p[0] ** 2 + p[1] ** 2 + p[2] ** 2))
            if n == 0.0:
                raise ValueError('Direction vector length must not be 0!')
            return float(item[0]), float(item[1]), _dir3(p, 1.0 / n)
        if isinstance(d[0], (list, tuple)):
            return [one(item) for item in d]
        return (one(d),)

    def __str__(self):
        return 'Filter(x={}, y={}, z={}, pz={}, dir={}, r={}, pl={})'.format(
            self._x, self._y, self._z, self._pz, self._dir, self._r, self._pl)

    __repr__ = __str__


class Trace:
    TRACE_ENTRY_LEN = _abi.TRACE_ENTRY_LEN
    TRACE_NONE = _abi.TRACE_NONE
    TRACE_START = _abi.TRACE_START
    TRACE_END = _abi.TRACE_END
    TRACE_ALL = _abi.TRACE_ALL

    TRACE_EVENT_REFLECTION = 1
    TRACE_EVENT_REFRACTION = 2
    TRACE_EVENT_BOUNDARY_HIT = 4
    TRACE_EVENT_LAUNCH = 8
    TRACE_EVENT_ABSORPTION = 16
    TRACE_EVENT_SCATTERING = 32
    TRACE_EVENT_TERMINATION = 64
    TRACE_EVENT_ESCAPE = 128
    TRACE_EVENT_ALL = -1

    def __init__(self, maxlen=500, options: int = TRACE_ALL, filter: Filter = None,
                 event_mask: int = None, plon: bool = True):
        if isinstance(maxlen, Trace):
            other = maxlen
            self._maxlen, self._options, self._event_mask = other.maxlen, other.options, other.event_mask
            self._plon = other.plon
            self._filter = other.filter
            self._data, self._n = other.data, other.n
            self._n_dropped = other.dropped
        else:
            self._options = int(options) & 7
            self._set_maxlen(maxlen)
            self._event_mask = None if event_mask is None else int(event_mask)
            self._plon = bool(plon)
            self._filter = filter
            self._data = None
            self._n = None
            self._n_dropped = 0
        self._terminal = None
        self._overflow = None

    def _set_maxlen(self, maxlen):
        """TRACE_START or TRACE_END alone record one event, both two
        (mctrace.py:848-857)."""
        if self._options == self.TRACE_ALL:
            pass
        elif self._options == (self.TRACE_START | self.TRACE_END):
            maxlen = 2
        else:
            maxlen = 1
        if int(maxlen) < 1:
            raise ValueError('Maximum trace length must be at least 1!')
        self._maxlen = int(maxlen)

    maxlen = property(lambda self: self._maxlen, _set_maxlen)
    options = property(lambda self: self._options)
    event_mask = property(lambda self: self._event_mask)
    plon = property(lambda self: self._plon)
    dropped = property(lambda self: self._n_dropped, None, None,
                       'Packets that matched the filter but overflowed the trace.')

    def _get_filter(self):
        return self._filter

    def _set_filter(self, f):
        self._filter = f

    filter = property(_get_filter, _set_filter)

    def _get_data(self):
        return self._data

    def _set_data(self, data):
        self._data = data
        self._terminal = self._overflow = None

    data = property(_get_data, _set_data, None, 'Structured array (packets, maxlen) of events.')

    def _get_n(self):
        return self._n

    def _set_n(self, n):
        self._n = n
        self._terminal = self._overflow = None

    n = property(_get_n, _set_n, None, 'Number of events recorded per packet.')

    nphotons = property(lambda self: 0 if self._n is None else int(self._n.size), None, None,
                        'Number of photon packets in the trace.')

    @property
    def terminal(self) -> np.ndarray:
        """Last recorded event of every packet (mctrace.py:707-712)."""
        if self._terminal is None and self._data is not None:
            last = np.minimum(self._n - 1, self._maxlen - 1)
            self._terminal = self._data[np.arange(self._n.size), last]
        return self._terminal

    @property
    def overflow(self) -> np.ndarray:
        """Packets with more events than the trace holds."""
        if self._overflow is None and self._data is not None:
            self._overflow = self._n >= self._maxlen
        return self._overflow

    def _get_dtype(self):
        return np.dtype([('x', np.float32), ('y', np.float32), ('z', np.float32),
                         ('px', np.float32), ('py', np.float32), ('pz', np.float32),
                         ('w', np.float32), ('pl', np.float32)])

    dtype = property(_get_dtype)

    def pack(self, mc, target: _abi.McgbTrace, nphotons: int):
        target.flags = self._options
        target.max_events = self._maxlen
        target.event_mask = int(self._event_mask or 0) & 0xFFFFFFFF
        target.data_offset = mc.cl_allocate_rw_float_buffer(
            self, (int(nphotons) * self._maxlen * self.TRACE_ENTRY_LEN,))
        target.count_offset = mc.cl_allocate_rw_int_buffer(self, (int(nphotons),))
        return target

    def apply_filter(self):
        if self._filter is not None:
            self._n_dropped = self._filter(self, update=True)[1]
            self._terminal = None

    def update_data(self, mc, floats, ints, nphotons: int):
        """Adds the events of a run; a filter is applied to the new packets
        (mctrace.py:1120-1172)."""
        events = np.asarray(floats, dtype=np.float32).reshape(int(nphotons), self._maxlen,
                                                               self.TRACE_ENTRY_LEN)
        data = np.ascontiguousarray(events).view(self.dtype).reshape(int(nphotons), self._maxlen)
        n = np.asarray(ints, dtype=np.int32).copy()
        self._terminal = self._overflow = None
        if self._data is not None:
            tmp = Trace(self)
            tmp._data = tmp._n = None
            tmp.update_data(mc, floats, ints, nphotons)
            self._n = np.hstack([self._n, tmp.n])
            self._data = np.vstack([self._data, tmp.data])
        else:
            self._data, self._n = data, n
            self.apply_filter()

    def update(self, obj: 'Trace'):
        """Appends the packets of another trace, filtered by this trace's
        filter (mctrace.py:1089-1118)."""
        if self._maxlen != obj.maxlen:
            raise ValueError('Cannot update the trace with trace data of different maximum length!')
        self._terminal = self._overflow = None
        if self._data is not None:
            if self._filter is not None:
                obj = self._filter(obj, update=False)[0]
            self._n = np.hstack([self._n, obj.n])
            self._data = np.vstack([self._data, obj.data])
        else:
            self._data, self._n = obj.data, obj.n

    def __len__(self):
        return 0 if self._n is None else int(self._n.size)

    def todict(self):
        return {'type': 'Trace', 'maxlen': self._maxlen, 'options': self._options,
                'filter': None if self._filter is None else self._filter.todict(),
                'event_mask': self._event_mask, 'plon': self._plon}

    @classmethod
    def fromdict(cls, data: dict) -> 'Trace':
        d = dict(data)
        t = d.pop('type')
        if t != cls.__name__:
            raise TypeError('Expected data for type "{}" but got "{}"!'.format(cls.__name__, t))
        f = d.pop('filter', None)
        if f is not None:
            f = Filter.fromdict(f)
        return cls(filter=f, **d)

    def __str__(self):
        return 'Trace(maxlen={}, options={}, filter={}, plon={})'.format(
            self._maxlen, self._options, self._filter, self._plon)

    __repr__ = __str__


TRACE_EVENT_REFLECTION = Trace.TRACE_EVENT_REFLECTION
TRACE_EVENT_REFRACTION = Trace.TRACE_EVENT_REFRACTION
TRACE_EVENT_BOUNDARY_HIT = Trace.TRACE_EVENT_BOUNDARY_HIT
TRACE_EVENT_LAUNCH = Trace.TRACE_EVENT_LAUNCH
TRACE_EVENT_ABSORPTION = Trace.TRACE_EVENT_ABSORPTION
TRACE_EVENT_SCATTERING = Trace.TRACE_EVENT_SCATTERING
TRACE_EVENT_TERMINATION = Trace.TRACE_EVENT_TERMINATION
TRACE_EVENT_ESCAPE = Trace.TRACE_EVENT_ESCAPE
TRACE_EVENT_ALL = Trace.TRACE_EVENT_ALL

__all__ = ['Filter', 'Trace', 'TRACE_EVENT_REFLECTION', 'TRACE_EVENT_REFRACTION',
           'TRACE_EVENT_BOUNDARY_HIT', 'TRACE_EVENT_LAUNCH', 'TRACE_EVENT_ABSORPTION',
           'TRACE_EVENT_SCATTERING', 'TRACE_EVENT_TERMINATION', 'TRACE_EVENT_ESCAPE',
           'TRACE_EVENT_ALL']
