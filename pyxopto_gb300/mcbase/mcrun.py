"""Run a simulator until a detector has collected enough weight or enough
packets (xopto/mcbase/mcrun.py:28-263).  Each batch is one ``Mc.run`` of
``batch_size`` packets accumulating into the same results."""
from typing import Tuple

import numpy as np


class RunMinWeightBase:
    def __init__(self, min_weight: float, batch_size: int, selection=None):
        self._min_weight = float(min_weight)
        self._batch_size = int(batch_size)
        self._num_packets = 0
        self._total_weight = 0.0
        self._selection = slice(None) if selection is None else selection

    def run(self, mc_obj, min_packets: int = None, out: tuple = None, *args, **kwargs) -> tuple:
        """Runs batches until the selected weight reaches ``min_weight`` and
        at least ``min_packets`` packets were launched (mcrun.py:49-91)."""
        min_packets = 0 if min_packets is None else int(min_packets)
        total_packets, total_weight = 0, 0.0
        while out is None or self._min_weight > total_weight or total_packets < min_packets:
            out = mc_obj.run(self._batch_size, *args, out=out, **kwargs)
            total_weight, _, out = self.process_batch(out)
            total_packets += self._batch_size
        self._num_packets = total_packets
        self._total_weight = total_weight
        return out

    def process_batch(self, result: tuple) -> Tuple[float, int, tuple]:
        return 0.0, 0, result

    selection = property(lambda self: self._selection)
    batch_size = property(lambda self: self._batch_size)
    min_weight = property(lambda self: self._min_weight)
    n = property(lambda self: self._num_packets, None, None, 'Packets launched by the last run.')
    weight = property(lambda self: self._total_weight, None, None, 'Weight collected in the last run.')


class RunMinPacketsBase:
    """Runs batches until at least ``min_packets`` packets were collected by
    the selected detector (mcrun.py:145-263; the reference's loop tests an
    undefined min_weight, restated here with the number of collected
    packets)."""

    def __init__(self, min_packets: float, batch_size: int, selection=None):
        self._min_packets = int(min_packets)
        self._batch_size = int(batch_size)
        self._num_packets = 0
        self._total_weight = 0.0
        self._selection = slice(None) if selection is None else selection

    def run(self, mc_obj, min_packets: int = None, out: tuple = None, *args, **kwargs) -> tuple:
        min_launched = 0 if min_packets is None else int(min_packets)
        total_packets, collected, total_weight = 0, 0, 0.0
        while out is None or collected < self._min_packets or total_packets < min_launched:
            out = mc_obj.run(self._batch_size, *args, out=out, **kwargs)
            total_weight, collected, out = self.process_batch(out)
            total_packets += self._batch_size
        self._num_packets = total_packets
        self._total_weight = total_weight
        return out

    def process_batch(self, result: tuple) -> Tuple[float, int, tuple]:
        return 0.0, 0, result

    selection = property(lambda self: self._selection)
    batch_size = property(lambda self: self._batch_size)
    min_packets = property(lambda self: self._min_packets)
    n = property(lambda self: self._num_packets)
    weight = property(lambda self: self._total_weight)


__all__ = ['RunMinWeightBase', 'RunMinPacketsBase']
