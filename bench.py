"""Throughput benchmark of the GB300 photon-packet transport engine.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                    [--workload c2_skin_gk_fluence|c1_slab_hg_radial] [--math fast|exact]

Workload (default): the 3-layer skin-like stack with the Gegenbauer phase
function (alpha 0.5), a normal Line source and a 100x100x100 Cartesian
fluence grid over 10x10x10 mm; one step = one run of 1e8 photon packets.
Metric: packets/s.  Inputs (layer table, seeds, tallies) are resident on the
device before the timed region; the 8 MB fluence tally fits in L2, so L2 is
flushed by writing a 256 MB buffer between steps.

Reported on one JSON line: the device-timed value, the end-to-end value
through Mc.run (host packing, host<->device copies, tally download), the
roofline of the transport kernel, the reference CPU build timed on this
host's cores, and the SM clocks sampled during the timed region.

--impl reference times the reference's own McKernel (rendered by PyXOpto's
plugins and compiled for the CPU, oracle/_ref/) on all host cores, on
bounded samples of the same workload.

Multi-GPU (torchrun): every rank runs an independent replica of the full
workload with its own random-number streams (weak scaling); integer tallies
are summed across ranks after the timed region.
"""
import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (ROOT, os.path.join(ROOT, 'oracle'), os.path.join(ROOT, 'tests', 'golden')):
    if _p not in sys.path:
        sys.path.insert(0, _p)

# FP32-equivalent operations per interaction step of the albedo-weight loop
# (log, boundary tests, move, absorption, phase-function sample, direction
# update and renormalisation, rmax test, 3 RNG draws), frozen for the
# roofline figure.
OPS_PER_STEP = 91
L2_FLUSH_BYTES = 256 << 20
METRIC = 'packets/s (1 GB300)'


def measured_peaks():
    path = os.path.join(ROOT, 'MEASURED_PEAKS.json')
    try:
        with open(path) as f:
            return json.load(f)
    except Exception:
        return {}


class ClockSampler:
    """Samples nvidia-smi SM clocks and throttle reasons in the background."""
    QUERY = ('index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,'
             'clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,'
             'clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap')

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ['nvidia-smi', '-i', str(self.index), '--query-gpu=' + self.QUERY,
                 '--format=csv,noheader,nounits', '-lms', '200'],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {'sm_mhz': None, 'sm_max_mhz': None, 'reasons': ['nvidia-smi unavailable']}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        for line in self.lines:
            parts = [p.strip() for p in line.split(',')]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for name, v in zip(names, parts[5:9]):
                if v.lower() == 'active':
                    reasons.add(name)
        return {'sm_mhz': float(np.median(sm)) if sm else None,
                'sm_max_mhz': float(max(smax)) if smax else None,
                'reasons': sorted(reasons), 'samples': len(sm)}


def dist_env():
    return int(os.environ.get('RANK', 0)), int(os.environ.get('WORLD_SIZE', 1)), \
        int(os.environ.get('LOCAL_RANK', 0))


# --------------------------------------------------------------- CPU side
def reference_cpu(workload, seconds=12.0, threads=None, max_packets=None):
    """Times the reference CPU build (or the oracle port when the reference
    build is absent) on a bounded sample; returns (packets/s, meta)."""
    import mcoracle
    import scenarios
    import render_ref
    from pyxopto_gb300.rng import Random
    threads = threads or os.cpu_count() or 1
    so = os.path.join(render_ref.REF_DIR, workload + '.so')
    kind = 'reference' if os.path.exists(so) else 'port'
    streams = 4096
    seeds = Random().seeds(streams, 1)
    mc = scenarios.build_mc(workload) if kind == 'port' else None

    def run(n):
        t0 = time.perf_counter()
        if kind == 'reference':
            render_ref.run_ref(workload, n, streams, seeds, nthreads=threads)
        else:
            mcoracle.run(mc, n, streams, mcoracle.LIBM, nthreads=threads, seeds=seeds)
        return time.perf_counter() - t0

    n = 2 * streams
    dt = run(n)
    while dt < seconds / 4 and (max_packets is None or n < max_packets):
        n = int(n * min(8.0, max(2.0, seconds / 4 / max(dt, 1e-3))))
        if max_packets:
            n = min(n, max_packets)
        dt = run(n)
    total_n, total_t = n, dt
    while total_t < seconds and (max_packets is None or total_n < max_packets):
        total_t += run(n)
        total_n += n
    rate = total_n / total_t
    return rate, {'kind': kind, 'cores': threads,
                  'sample': '{} packets of {} on {} streams in {:.1f} s'.format(
                      total_n, workload, streams, total_t)}


# --------------------------------------------------------------- GPU side
def gpu_bench(args, rank, world, local_rank):
    import torch
    import scenarios
    from pyxopto_gb300 import _abi, _lib
    torch.cuda.set_device(local_rank)
    dev = torch.device('cuda', local_rank)
    lib = _lib.load()
    spec = scenarios.ALL[args.workload]
    nphotons = int(args.packets or spec['nphotons'])
    fast = args.math == 'fast'
    mc = scenarios.build_mc(args.workload, fast=fast)
    mc._rnginit = 1 + 7919 * rank
    math = _abi.MATH_FAST if fast else _abi.MATH_EXACT
    streams = mc.suggested_streams(math)
    cfg = mc.pack(nphotons, streams)
    mc._ensure_streams(torch, streams, dev)
    bufs = mc._device_buffers(torch, dev, mc._lut_array(), {})
    stream = torch.cuda.current_stream()
    sptr = C.c_void_p(stream.cuda_stream)
    flush = torch.empty((L2_FLUSH_BYTES // 4,), dtype=torch.float32, device=dev)
    accu = mc._dev['accu']
    counters = mc._dev['counters']
    host_counters = (C.c_uint64 * _abi.NUM_COUNTERS)()

    def step():
        accu.zero_()
        counters.zero_()
        _lib.check(lib.mcgb_mcml_run(C.byref(cfg), C.byref(bufs), sptr))

    barrier = (lambda: torch.distributed.barrier()) if world > 1 else (lambda: None)

    for _ in range(args.warmup):
        flush.fill_(1.0)
        step()
    torch.cuda.synchronize()
    _lib.check(lib.mcgb_check_counters(C.c_void_p(counters.data_ptr()), sptr, host_counters))
    steps_per_launch = int(host_counters[_abi.CNT_STEPS])

    sampler = ClockSampler(local_rank)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    barrier()
    torch.cuda.synchronize()
    sampler.start()
    t_start = torch.cuda.Event(enable_timing=True)
    t_end = torch.cuda.Event(enable_timing=True)
    t_start.record(stream)
    for k in range(args.steps):
        flush.fill_(float(k))
        accu.zero_()
        counters.zero_()
        ev[k][0].record(stream)
        _lib.check(lib.mcgb_mcml_run(C.byref(cfg), C.byref(bufs), sptr))
        ev[k][1].record(stream)
    t_end.record(stream)
    torch.cuda.synchronize()
    barrier()
    clocks = sampler.stop()
    _lib.check(lib.mcgb_check_counters(C.c_void_p(counters.data_ptr()), sptr, host_counters))
    total_ms = t_start.elapsed_time(t_end)
    kernel_ms = [a.elapsed_time(b) for a, b in ev]
    if world > 1:
        t = torch.tensor([total_ms], device=dev, dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(t.item())
        # exact integer tally reduction across the replicas
        torch.distributed.all_reduce(accu, op=torch.distributed.ReduceOp.SUM)

    # ---- end-to-end through the public API (host buffers, copies inside)
    e2e = None
    if not args.no_e2e:
        api = scenarios.build_mc(args.workload, fast=fast)
        api._rnginit = 2 + 7919 * rank
        api.run(nphotons, maxthreads=streams)        # warm-up (seeds, buffers)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.e2e_steps):
            api.run(nphotons, maxthreads=streams)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        h2d = C.sizeof(_abi.McgbMcmlConfig) + 4 * int(api._lut_size)
        d2h = 8 * int(api._acc.size) + 4 * int(api._flt.size) + 4 * int(api._int.size) + \
            8 * _abi.NUM_COUNTERS
        e2e = {'value': nphotons * args.e2e_steps * world / dt, 'unit': 'packets/s',
               'h2d_bytes_per_step': h2d, 'd2h_bytes_per_step': d2h,
               'path': 'pyxopto_gb300.mcml.mc.Mc.run'}
    return dict(total_ms=total_ms, kernel_ms=kernel_ms, steps_per_launch=steps_per_launch,
                clocks=clocks, e2e=e2e, nphotons=nphotons, streams=streams,
                packets_done=int(host_counters[_abi.CNT_PACKETS]))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=5)
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--impl', default='gb300', choices=['gb300', 'reference'])
    ap.add_argument('--workload', default='c2_skin_gk_fluence')
    ap.add_argument('--math', default='fast', choices=['fast', 'exact'])
    ap.add_argument('--e2e-steps', type=int, default=2)
    ap.add_argument('--no-e2e', action='store_true')
    ap.add_argument('--no-cpu-baseline', action='store_true')
    ap.add_argument('--cpu-seconds', type=float, default=12.0)
    ap.add_argument('--packets', type=int, default=None,
                    help='override the packets per step (small profiling cases only; '
                         'a headline number uses the workload size)')
    args = ap.parse_args()
    rank, world, local_rank = dist_env()
    import scenarios
    spec = scenarios.ALL[args.workload]
    config = {'workload': args.workload, 'packets_per_step': int(args.packets or spec['nphotons']),
              'medium': spec['medium'], 'math': args.math,
              'l2': 'flushed between steps (256 MB write); fluence tally 8 MB fits L2'}

    if args.impl == 'reference':
        if rank != 0:
            return
        threads = os.cpu_count() or 1
        for _ in range(args.warmup):
            reference_cpu(args.workload, seconds=1.0, threads=threads, max_packets=20000)
        rates, meta = [], None
        t0 = time.perf_counter()
        for _ in range(args.steps):
            r, meta = reference_cpu(args.workload, seconds=args.cpu_seconds / max(args.steps, 1) * 2,
                                    threads=threads)
            rates.append(r)
        wall = time.perf_counter() - t0
        value = float(np.mean(rates))
        line = {'metric': METRIC, 'value': value, 'unit': 'packets/s', 'n_gpus': 0,
                'steps': args.steps, 'warmup': args.warmup,
                'ms_per_step': 1e3 * wall / max(args.steps, 1), 'higher_is_better': True,
                'scaling': 'none', 'vs_baseline': None, 'dtype': 'f32', 'impl': 'reference',
                'data': 'synthetic (seeded streams, rnginit=1)', 'config': config,
                'cpu_baseline': dict(meta, value=value, unit='packets/s'),
                'e2e': {'value': value, 'unit': 'packets/s', 'h2d_bytes_per_step': 0,
                        'd2h_bytes_per_step': 0}}
        print(json.dumps(line))
        return

    if world > 1:
        import torch
        torch.distributed.init_process_group('nccl')
    res = gpu_bench(args, rank, world, local_rank)
    if rank != 0:
        if world > 1:
            import torch
            torch.distributed.destroy_process_group()
        return
    n = res['nphotons']
    ms_per_step = res['total_ms'] / args.steps
    value = n * args.steps * world / (res['total_ms'] / 1e3)
    kern_ms = float(np.mean(res['kernel_ms']))
    peaks = measured_peaks()
    sm_max = peaks.get('sm_max_mhz') or 2070.0
    fp32_peak = 152 * 128 * 2 * sm_max * 1e6 / 1e12
    achieved = res['steps_per_launch'] * OPS_PER_STEP / (kern_ms / 1e3) / 1e12
    roofline = {'bound': 'fp32', 'achieved': achieved, 'peak': fp32_peak, 'unit': 'TFLOP/s',
                'frac': achieved / fp32_peak, 'traffic': None,
                'peak_source': 'derived: 152 SMs x 128 FP32 lanes x 2 x sm_max_mhz {} '
                               '(MEASURED_PEAKS.json); no FP32 peak is measured there'.format(sm_max),
                'ops_per_step': OPS_PER_STEP, 'steps_per_launch': res['steps_per_launch'],
                'kernel_ms': kern_ms, 'steps_per_s': res['steps_per_launch'] / (kern_ms / 1e3)}
    line = {'metric': METRIC, 'value': value, 'unit': 'packets/s', 'n_gpus': world,
            'steps': args.steps, 'warmup': args.warmup, 'ms_per_step': ms_per_step,
            'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f32',
            'data': 'synthetic (seeded RNG streams; no dataset)', 'config': config,
            'roofline': roofline, 'clocks': res['clocks'], 'e2e': res['e2e'],
            'gpu_launches': args.steps, 'streams': res['streams'],
            'packets_checked': res['packets_done'] == n}
    if not args.no_cpu_baseline and world == 1:
        rate, meta = reference_cpu(args.workload, seconds=args.cpu_seconds)
        line['cpu_baseline'] = dict(meta, value=rate, unit='packets/s')
    print(json.dumps(line))
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == '__main__':
    main()
