"""Photon packet trace (xopto/mcbase/mctrace.py:444-1234).

Each packet records up to ``maxlen`` events of 8 floats
(x, y, z, px, py, pz, w, optical path length); when the trace is full the
last slot is overwritten, and the per-packet event count is stored in the
integer buffer (mctrace.py:541-583)."""
import numpy as np

from .. import _abi


class Trace:
    TRACE_ENTRY_LEN = _abi.TRACE_ENTRY_LEN
    TRACE_NONE = _abi.TRACE_NONE
    TRACE_START = _abi.TRACE_START
    TRACE_END = _abi.TRACE_END
    TRACE_ALL = _abi.TRACE_ALL

    def __init__(self, maxlen=500, options: int = TRACE_ALL, filter=None,
                 event_mask: int = None, plon: bool = True):
        if isinstance(maxlen, Trace):
            other = maxlen
            self._maxlen, self._options, self._event_mask = other.maxlen, other.options, other.event_mask
            self._plon = other.plon
            self._filter = other.filter
        else:
            self._maxlen = max(int(maxlen), 1)
            self._options = int(options)
            self._event_mask = event_mask
            self._plon = bool(plon)
            self._filter = filter
        self._data = None
        self._n = None
        self._nphotons = 0

    maxlen = property(lambda self: self._maxlen)
    options = property(lambda self: self._options)
    event_mask = property(lambda self: self._event_mask)
    plon = property(lambda self: self._plon)
    filter = property(lambda self: self._filter)
    data = property(lambda self: self._data, None, None,
                    'Structured array (nphotons, maxlen) of events.')
    n = property(lambda self: self._n, None, None, 'Number of events per packet.')
    nphotons = property(lambda self: self._nphotons)

    def _get_dtype(self):
        return np.dtype([('x', np.float32), ('y', np.float32), ('z', np.float32),
                         ('px', np.float32), ('py', np.float32), ('pz', np.float32),
                         ('w', np.float32), ('pl', np.float32)])

    dtype = property(_get_dtype)

    def pack(self, mc, target: _abi.McgbTrace, nphotons: int):
        target.flags = self._options
        target.max_events = self._maxlen
        target.event_mask = int(self._event_mask or 0)
        target.data_offset = mc.cl_allocate_rw_float_buffer(
            self, (int(nphotons) * self._maxlen * self.TRACE_ENTRY_LEN,))
        target.count_offset = mc.cl_allocate_rw_int_buffer(self, (int(nphotons),))
        return target

    def update_data(self, mc, floats, ints, nphotons: int):
        events = np.asarray(floats, dtype=np.float32).reshape(int(nphotons), self._maxlen,
                                                               self.TRACE_ENTRY_LEN)
        self._data = np.ascontiguousarray(events).view(self.dtype).reshape(int(nphotons), self._maxlen)
        self._n = np.asarray(ints, dtype=np.int32).copy()
        self._nphotons = int(nphotons)
        if self._filter is not None:
            self._data, self._n = self._filter(self._data, self._n)

    def __len__(self):
        return 0 if self._n is None else self._n.size

    def todict(self):
        return {'type': 'Trace', 'maxlen': self._maxlen, 'options': self._options,
                'event_mask': self._event_mask, 'plon': self._plon}

    def __str__(self):
        return 'Trace(maxlen={}, options={}, plon={})'.format(self._maxlen, self._options, self._plon)
