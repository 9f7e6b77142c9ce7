"""Run helpers of the layered simulator (xopto/mcml/mcrun): run until a
detector or the trace has collected enough weight or packets
(mcrun/mcrun.py:31-257), and McRunHelper, the customisable loop over
configurations that dataset generators subclass (mcrun/helper.py:32-686)."""
import time
from typing import Callable, Dict, List

import numpy as np

from ..mcbase.mcrun import RunMinWeightBase, RunMinPacketsBase
from . import mc as _mc


class _RunMinWeightDetector(RunMinWeightBase):
    def __init__(self, location: str, min_weight: float, batch_size: int, selection=None):
        self._location = location
        super().__init__(min_weight, batch_size, selection)

    def process_batch(self, result):
        """Weight in the selected part of the detector (mcrun.py:54-96)."""
        detectors = result[2]
        if detectors is None or isinstance(getattr(detectors, self._location),
                                           _mc.mcdetector.DetectorDefault):
            raise RuntimeError('This MC simulator instance does not use the configured ("{}") '
                               'detector!'.format(self._location))
        raw = getattr(detectors, self._location).raw
        return float(np.sum(raw[self.selection])), None, result

    location = property(lambda self: self._location)


class RunMinWeightTop(_RunMinWeightDetector):
    def __init__(self, min_weight: float, batch_size: int, selection=None):
        super().__init__('top', min_weight, batch_size, selection)


class RunMinWeightBottom(_RunMinWeightDetector):
    def __init__(self, min_weight: float, batch_size: int, selection=None):
        super().__init__('bottom', min_weight, batch_size, selection)


class RunMinWeightSpecular(_RunMinWeightDetector):
    def __init__(self, min_weight: float, batch_size: int, selection=None):
        super().__init__('specular', min_weight, batch_size, selection)


class RunMinWeightTrace(RunMinWeightBase):
    """Until the terminal weight of the traced packets reaches min_weight
    (mcrun.py:161-208)."""

    def process_batch(self, result):
        trace = result[0]
        if trace is None:
            raise RuntimeError('This MC simulator instance does not use a trace!')
        w = trace.terminal['w'] if len(trace) else np.zeros((0,))
        return float(np.sum(w[self.selection])), len(trace), result


class RunMinPacketsTrace(RunMinPacketsBase):
    """Until min_packets packets are in the (filtered) trace
    (mcrun.py:211-257)."""

    def process_batch(self, result):
        trace = result[0]
        if trace is None:
            raise RuntimeError('This MC simulator instance does not use a trace!')
        w = trace.terminal['w'] if len(trace) else np.zeros((0,))
        return float(np.sum(w)), len(trace), result


class McRunHelper:
    """Creates a simulator from overridable ``create_*`` hooks, updates it
    before every run through ``update_*`` hooks and collects the results as
    dicts (xopto/mcml/mcrun/helper.py:32-686)."""

    def __init__(self, *args, **kwargs):
        self._mc_obj = self.create_mc(*args, **kwargs)

    def create_layers(self):
        return _mc.mclayer.Layers([
            _mc.mclayer.Layer(d=float('inf'), mua=0.0, mus=0.0, n=1.0, pf=_mc.mcpf.Hg(0.8))
            for _ in range(3)])

    def create_source(self):
        return _mc.mcsource.Line()

    def create_surface(self):
        return None

    def create_detectors(self):
        return _mc.mcdetector.Detectors(
            top=_mc.mcdetector.Radial(_mc.mcdetector.Axis(0.0, 5.0, 500)),
            bottom=_mc.mcdetector.Radial(_mc.mcdetector.Axis(0.0, 5.0, 500)),
            specular=_mc.mcdetector.Total())

    def create_fluence(self):
        return None

    def create_trace(self):
        return None

    def create_mc(self, *args, **kwargs):
        """Source, surface, layers, detectors, fluence, trace, in the
        reference's order (helper.py:278-318)."""
        source = self.create_source()
        surface = self.create_surface()
        layers = self.create_layers()
        detectors = self.create_detectors()
        fluence = self.create_fluence()
        trace = self.create_trace()
        return _mc.Mc(layers, source, detectors, *args, trace=trace, fluence=fluence,
                      surface=surface, **kwargs)

    def update_layers(self):
        pass

    def update_source(self):
        pass

    def update_surface(self):
        pass

    def update_detectors(self):
        pass

    def update_fluence(self):
        pass

    def update_trace(self):
        pass

    def update_rmax(self):
        pass

    def verbose_print(self):
        pass

    def update(self):
        self.update_layers()
        self.update_source()
        self.update_surface()
        self.update_detectors()
        self.update_fluence()
        self.update_trace()
        self.update_rmax()

    mc_obj = property(lambda self: self._mc_obj, None, None, 'Monte Carlo simulator instance')

    def collect_mc_config(self) -> dict:
        m = self._mc_obj

        def d(obj):
            return obj.todict() if obj is not None and hasattr(obj, 'todict') else None
        return {'source': d(m.source), 'surface': d(m.surface), 'layers': d(m.layers),
                'detectors': d(m.detectors), 'fluence': d(m.fluence), 'trace': d(m.trace),
                'rmax': m.rmax, 'run_report': dict(m.run_report)}

    def collect_detectors(self, result) -> dict:
        data = {'reflectance': None, 'transmittance': None, 'specular': None}
        if result is not None:
            D = _mc.mcdetector.DetectorDefault
            if not isinstance(result.top, D):
                data['reflectance'] = result.top.reflectance
            if not isinstance(result.bottom, D):
                data['transmittance'] = result.bottom.reflectance
            if not isinstance(result.specular, D):
                data['specular'] = result.specular.reflectance
        return data

    def collect_fluence(self, result) -> dict:
        return {'data': None if result is None else result.data}

    def collect_trace(self, result):
        return None if result is None else {'data': result.data, 'n': result.n}

    def run_one(self, nphotons, verbose: bool = False, *args, **kwargs) -> dict:
        if not isinstance(nphotons, (int, float, np.integer)):
            nphotons = nphotons(self)
        self.update()
        if verbose:
            self.verbose_print()
        trace_res, fluence_res, detectors_res = self._mc_obj.run(nphotons, *args, **kwargs)
        return self.collect_one(nphotons, trace_res, fluence_res, detectors_res)

    def collect_one(self, nphotons, trace_res=None, fluence_res=None, detectors_res=None) -> dict:
        return {'epoch_timestamp': time.time(), 'mc': self.collect_mc_config(),
                'num_packets': nphotons, 'detectors': self.collect_detectors(detectors_res),
                'fluence': self.collect_fluence(fluence_res), 'trace': self.collect_trace(trace_res)}

    def run_batch(self, size: int, nphotons, first: int = 0, verbose: bool = False,
                  *args, **kwargs) -> List[Dict]:
        out = []
        t0 = time.perf_counter()
        rate = float('nan')
        for i in range(size):
            if verbose:
                print('{}-{}: {}/{} - {:.1f} samples/h'.format(first, first + size, i + 1, size, rate))
            data = self.run_one(nphotons, verbose, *args, **kwargs)
            data['index'] = first + i
            out.append(data)
            rate = (i + 1) / (time.perf_counter() - t0) * 3600
        return out


__all__ = ['RunMinWeightTop', 'RunMinWeightBottom', 'RunMinWeightSpecular', 'RunMinWeightTrace',
           'RunMinPacketsTrace', 'McRunHelper']
