"""Throughput benchmark of the GB300 photon-packet transport engine.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                    [--workload c2_skin_gk_fluence|c1_slab_hg_radial|c3_vox_skin_vessel|
                                batched_4096|surrogate|mlp_train_step|fiber_sweep|fiber_sweep_vox]
                    [--math fast|exact] [--no-others]

Workload (default): the 3-layer skin-like stack with the Gegenbauer phase
function (alpha 0.5), a normal Line source and a 100x100x100 Cartesian
fluence grid over 10x10x10 mm; one step = one run of 1e8 photon packets.
Metric: packets/s.  Inputs (layer table, seeds, tallies) are resident on the
device before the timed region; the 8 MB fluence tally fits in L2, so L2 is
flushed by writing a 256 MB buffer between steps.

Reported on one JSON line: the device-timed value, the end-to-end value
through Mc.run (host packing, host<->device copies, tally download), the
roofline of the transport kernel, the reference CPU build timed on this
host's cores, and the SM clocks sampled during the timed region.  The
default run also measures the other configurations (the 10 mm slab, the
200^3 voxel grid, the batched engine, the surrogate) and reports them under
"other_workloads" in the same line.

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
# From ncu captures of the transport kernel (the summary file named beside
# each entry): DRAM bytes (read + write) per launch, one-pass capture of the
# full workload, mean of three launches -- the one-time fill of the tallies
# and tables into L2, which does not grow with the packet count -- and the
# fraction of issue slots in use (smsp__issue_active), the resource that
# bounds this kernel.
PROFILED_TRAFFIC = {
    ('c2_skin_gk_fluence', 'fast', 'dynamic'): (7.74e6, 'profiles/mcml_dynamic_kernel_c2_skin_gk_fluence.md'),
    ('c3_vox_skin_vessel', 'fast', 'dynamic'): (1.80e10, 'profiles/mcvox_dynamic_kernel_c3_skin_vessel_200cubed.md'),
}
PROFILED_ISSUE_ACTIVE = {
    ('c2_skin_gk_fluence', 'fast', 'dynamic'): (0.875, 'profiles/mcml_dynamic_kernel_c2_skin_gk_fluence.md'),
    ('c3_vox_skin_vessel', 'fast', 'dynamic'): (0.867, 'profiles/mcvox_dynamic_kernel_c3_skin_vessel_200cubed.md'),
}
# L2 atomic-unit use of the transport kernel's 64-bit tally atomics, from a
# medium-case ncu capture (one kernel, one launch, 2e7 packets): the share of
# L2 cycles in which the atomic unit's input was active
# (lts__d_atomic_input_cycles_active), the reduction requests per packet and
# per interaction step (lts__t_requests_op_red), and the L2 throughput.
PROFILED_L2_ATOMICS = {
    ('c2_skin_gk_fluence', 'fast', 'dynamic'): (
        {'atomic_unit_active_pct': 14.66, 'red_requests_per_packet': 436.6,
         'red_requests_per_ref_step': 0.484, 'lts_throughput_pct': 21.98},
        'profiles/mcml_dynamic_kernel_c2_skin_gk_fluence.md'),
    ('c3_vox_skin_vessel', 'fast', 'dynamic'): (
        {'atomic_unit_active_pct': 12.22, 'red_requests_per_packet': 300.1,
         'red_requests_per_ref_step': 0.370, 'lts_throughput_pct': 24.04},
        'profiles/mcvox_dynamic_kernel_c3_skin_vessel_200cubed.md'),
}
# DRAM traffic of the voxel fluence (same capture): dram__bytes_read +
# dram__bytes_write over the kernel's duration (L2 evictions of the 64 MB
# fluence tally's atomics; the tally itself is read once).
PROFILED_HBM = {
    ('c3_vox_skin_vessel', 'fast', 'dynamic'): (
        {'gbs': 41.7, 'bytes_per_packet': 180.2},
        'profiles/mcvox_dynamic_kernel_c3_skin_vessel_200cubed.md'),
}
HBM_FALLBACK_GBS = 6800.0
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
def reference_seeds():
    """Stream seeds of the reference's own initialiser (clrng.Random().seeds
    (4096, 1)), stored as a fixture so that the CPU arms load no library of
    this package: tests/golden/ref_seeds.npz."""
    d = np.load(os.path.join(ROOT, 'tests', 'golden', 'ref_seeds.npz'))
    return d['x'].copy(), d['a'].copy()


def reference_cpu(workload, seconds=12.0, threads=None, max_packets=None):
    """Times the reference CPU build (or the oracle port when the reference
    build is absent) on a bounded sample; returns (packets/s, meta)."""
    import render_ref
    threads = threads or os.cpu_count() or 1
    so = os.path.join(render_ref.REF_DIR, workload + '.so')
    kind = 'reference' if os.path.exists(so) else 'port'
    seeds = reference_seeds()
    streams = len(seeds[0])
    mc = None
    if kind == 'port':
        import mcoracle
        import scenarios
        mc = scenarios.build_mc(workload)

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
def fp32_peak_tflops(torch, lib, dev):
    """FP32 FMA throughput of this GPU, measured with the library's probe
    kernel (16 independent FMA chains per thread, full occupancy): best of
    three launches of about 30 ms, timed with CUDA events.  This is the
    denominator of the transport kernels' roofline figure."""
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    blocks, threads = 2 * sms, 1024
    out = torch.zeros((blocks,), dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream()
    sptr = C.c_void_p(stream.cuda_stream)

    def timed(iters):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        from pyxopto_gb300 import _lib
        _lib.check(lib.mcgb_fp32_fma_rate(blocks, threads, iters, C.c_void_p(out.data_ptr()), sptr))
        b.record(stream)
        torch.cuda.synchronize()
        return a.elapsed_time(b)

    ms = timed(200)
    iters = max(200, int(200 * 30.0 / max(ms, 1e-3)))
    best = min(timed(iters) for _ in range(3))
    flops = float(blocks) * threads * iters * 256
    return flops / (best / 1e3) / 1e12, {'blocks': blocks, 'threads': threads, 'iters': iters,
                                         'ms': best}


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
    mc = scenarios.build_mc(args.workload, fast=fast, scheduling=args.scheduling)
    mc._rnginit = 1 + 7919 * rank
    run_fn, cfg, bufs = mc._prepare(nphotons)
    streams = cfg.num_streams
    stream = torch.cuda.current_stream()
    sptr = C.c_void_p(stream.cuda_stream)
    flush = torch.empty((L2_FLUSH_BYTES // 4,), dtype=torch.float32, device=dev)
    accu = mc._dev['accu']
    counters = mc._dev['counters']
    host_counters = (C.c_uint64 * _abi.NUM_COUNTERS)()

    def step():
        accu.zero_()
        counters.zero_()
        _lib.check(run_fn(C.byref(cfg), C.byref(bufs), sptr))

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
        _lib.check(run_fn(C.byref(cfg), C.byref(bufs), sptr))
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
        api = scenarios.build_mc(args.workload, fast=fast, scheduling=args.scheduling)
        api._rnginit = 2 + 7919 * rank
        api.run(nphotons, maxthreads=streams)        # warm-up (seeds, buffers)
        torch.cuda.synchronize()
        barrier()
        t0 = time.perf_counter()
        for _ in range(args.e2e_steps):
            api.run(nphotons, maxthreads=streams)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        barrier()
        if world > 1:
            # the slowest rank's wall time, as for the device-timed value
            t = torch.tensor([dt], device=dev, dtype=torch.float64)
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            dt = float(t.item())
        h2d = C.sizeof(cfg) + 4 * int(api._lut_size)
        if spec['medium'] == 'mcvox':
            # the voxel grid stays on the device between runs; the material
            # table is uploaded with every run
            h2d += C.sizeof(_abi.McgbMaterial) * len(api.materials)
        d2h = 8 * int(api._acc.size) + 4 * int(api._flt.size) + 4 * int(api._int.size) + \
            8 * _abi.NUM_COUNTERS
        e2e = {'value': nphotons * args.e2e_steps * world / dt, 'unit': 'packets/s',
               'h2d_bytes_per_step': h2d, 'd2h_bytes_per_step': d2h,
               'path': 'pyxopto_gb300.{}.mc.Mc.run'.format(spec['medium'])}
    # reference steps per packet: the reference's loop iterations for this
    # workload, the unit of the algorithmic work.  The layered kernels run
    # the reference's loop step for step; voxelized FAST runs take free
    # flights through same-material voxels, so their reference step count is
    # measured on a calibration run that walks every wall (2e6 packets).
    ref_spp = steps_per_launch / float(nphotons)
    ref_spp_source = 'device step counter of the timed launches (the reference loop, step for step)'
    if spec['medium'] == 'mcvox' and fast:
        from pyxopto_gb300.mcvox import mcoptions
        cal = scenarios.build_mc(args.workload, fast=True, scheduling=args.scheduling)
        cal._mc_options.append(mcoptions.McVoxelFreeFlight(False))
        cal._rnginit = 3 + 7919 * rank
        ncal = min(nphotons, 2_000_000)
        cal.run(ncal)
        ref_spp = cal.run_report['steps'] / float(ncal)
        ref_spp_source = ('calibration run of {} packets walking every voxel wall as the reference '
                          'does (McVoxelFreeFlight off)'.format(ncal))
    fp32_peak, fp32_probe = fp32_peak_tflops(torch, lib, dev)
    return dict(total_ms=total_ms, kernel_ms=kernel_ms, steps_per_launch=steps_per_launch,
                clocks=clocks, e2e=e2e, nphotons=nphotons, streams=streams,
                packets_done=int(host_counters[_abi.CNT_PACKETS]),
                fp32_peak=fp32_peak, fp32_probe=fp32_probe, ref_spp=ref_spp,
                ref_spp_source=ref_spp_source)


def batched_bench(args):
    """4096 single-layer simulations (the batched benchmark ranges) in one
    persistent launch replayed from a CUDA graph; metric profiles/s."""
    import torch
    from pyxopto_gb300.batched import BatchedMc
    nsims = args.sims
    sims = BatchedMc.sample_sims(nsims, seed=1)
    b = BatchedMc(sims, fast=args.math == 'fast')
    tune = b.autotune()
    for _ in range(args.warmup):
        b.run_raw(graph=True)
    stream = torch.cuda.current_stream()
    sampler = ClockSampler(0)
    t0e, t1e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    sampler.start()
    t0e.record(stream)
    for _ in range(args.steps):
        b._graph.replay()
    t1e.record(stream)
    torch.cuda.synchronize()
    clocks = sampler.stop()
    dev_s = t0e.elapsed_time(t1e) / 1e3 / args.steps
    npk = int(b.packets.sum())
    t0 = time.perf_counter()
    for _ in range(args.e2e_steps):
        b.run(graph=True)
    e2e_s = (time.perf_counter() - t0) / args.e2e_steps
    steps = b.last_report['steps']
    # the same simulations as sequential plain Mc.run calls (a sample of
    # the first 64, each with its own packet count, plus one warm-up)
    from pyxopto_gb300.surrogate import sequential_plain_mc
    nseq = min(64, nsims - 1)
    sample = {k: np.asarray(v)[list(range(nseq)) + [nseq]] for k, v in sims.items()}
    seq_rate = sequential_plain_mc(sample)
    seq_packets = int(np.asarray(sims['num_packets'])[:nseq].sum())
    return {'metric': 'profiles/s (batched MC, {} single-layer simulations)'.format(nsims),
            'value': nsims / dev_s, 'unit': 'profiles/s', 'ms_per_step': dev_s * 1e3,
            'packets_per_s': npk / dev_s, 'steps_per_s': steps / dev_s,
            'sequential_plain_mc': {'profiles_per_s': seq_rate, 'packets_per_s':
                                    seq_rate * seq_packets / nseq, 'sample_sims': nseq},
            'config': {'workload': 'batched_4096', 'sims': nsims, 'packets_total': npk,
                       'radial_bins': 30, 'r_max_m': 3e-3, 'autotuned': {
                           k: tune[k] for k in ('block_size', 'packets_per_item')},
                       'graph': True},
            'clocks': clocks, 'gpu_launches': 2 * args.steps,
            'e2e': {'value': nsims / e2e_s, 'unit': 'profiles/s',
                    'h2d_bytes_per_step': 40 * nsims, 'd2h_bytes_per_step': 8 * 30 * nsims + 64,
                    'path': 'pyxopto_gb300.batched.BatchedMc.run(graph=True)'}}


def surrogate_bench(args):
    """The shipped surrogate (trained on the GPU by pyxopto_gb300.train_surrogate
    on 2^18 profiles of 1e6 packets) serving 65536 queries with its 1 % Monte
    Carlo judge and the library's default fallback (max_fail 0.1), against
    sequential plain Mc.run calls at the judge's packet count (1e6 packets,
    whose own Monte Carlo noise is about 1 % RMS relative); metric profiles/s."""
    from pyxopto_gb300 import _lib
    from pyxopto_gb300.batched import BatchedMc
    from pyxopto_gb300.surrogate import Surrogate, default_weights, sequential_plain_mc
    _lib.load().mcgb_mlp_gemm_path(0 if args.mlp_gemm == 'tcgen05' else 1)
    path = default_weights()
    sur = Surrogate.load(path)
    train_log = None
    log_path = os.path.splitext(path)[0] + '.log.json'
    if os.path.exists(log_path):
        with open(log_path) as f:
            train_log = json.load(f)
    # accuracy against high-accuracy Monte Carlo (independent of the judge):
    # two 2e6-packet halves per test profile, noise-corrected
    test = BatchedMc.sample_sims(256, seed=1099, packets=(1, 2))
    a, b = sur.simulate_halves(test, 4_000_000, seed=77)
    pred = sur.predict(test['mua'], test['mus'] * (1 - test['g']), test['g'], test['n'])
    err, raw, noise = Surrogate.judge_error(pred, a, b)
    queries = BatchedMc.sample_sims(65536, seed=5, packets=(1, 2))
    serve_kw = dict(judge_fraction=0.01, judge_packets=1_000_000, tol=0.01)
    for _ in range(args.warmup):
        sur.serve(queries, **serve_kw)
    sampler = ClockSampler(0)
    sampler.start()
    reps = []
    for k in range(args.steps):
        _, rep = sur.serve(queries, seed=7 + k, **serve_kw)
        reps.append(rep)
    clocks = sampler.stop()
    sec = float(np.mean([r['seconds'] for r in reps]))
    seq = BatchedMc.sample_sims(args.seq_profiles + 1, seed=31, packets=(1, 2))
    seq_rate = sequential_plain_mc(seq, 1_000_000)
    value = 65536 / sec
    launches_per_serve = 4 * ((65536 + sur.mlp.batch - 1) // sur.mlp.batch) + 2
    stat = lambda v: {'median': float(np.median(v)), 'mean': float(np.mean(v)),
                      'p90': float(np.percentile(v, 90))}
    return {'metric': 'profiles/s (surrogate + 1% MC judge, 65536 queries)', 'value': value,
            'unit': 'profiles/s', 'ms_per_step': sec * 1e3,
            'sequential_plain_mc_profiles_per_s': seq_rate,
            'gain_vs_sequential_plain_mc': value / seq_rate,
            'surrogate_rms_rel_vs_mc': dict(stat(err), raw=stat(raw), mc_noise=stat(noise),
                                            share_above_1pct=float(np.mean(err > 0.01)),
                                            reference='2 x 2e6-packet batched MC per profile, '
                                                      '256 profiles, noise-corrected'),
            'held_out_at_training': (train_log or {}).get('held_out'),
            'judge': {k: float(np.mean([r[k] for r in reps]))
                      for k in ('judge_rms_rel_mean', 'judge_rms_rel_median', 'judge_rms_rel_p90',
                                'judge_raw_rms_rel_median', 'judge_noise_rms_rel_median',
                                'judge_noise_rms_rel_p90', 'judge_estimate_se_median',
                                'judge_fail_fraction', 'judge_point_estimate_above_tol',
                                'infer_seconds', 'judge_seconds', 'fallback_seconds')},
            'fallback_all': [bool(r['fallback_all']) for r in reps],
            'config': {'workload': 'surrogate', 'mlp': '4-256-256-256-30 GELU bf16/fp32',
                       'weights': os.path.relpath(path, ROOT),
                       'train_profiles': (train_log or {}).get('train_profiles'),
                       'train_packets': (train_log or {}).get('train_packets'),
                       'train_profiles_note': '2^18 profiles, a quarter of the 2^20 of the '
                                              'benchmark definition',
                       'judge_fraction': 0.01, 'judge_packets': 1_000_000, 'tol': 0.01,
                       'max_fail': 0.1, 'judge_confidence_se': 2.0,
                       'sequential_profiles_timed': args.seq_profiles,
                       'sequential_packets': 1_000_000},
            'clocks': clocks, 'gpu_launches': launches_per_serve * args.steps,
            'e2e': {'value': value, 'unit': 'profiles/s',
                    'h2d_bytes_per_step': 65536 * 16 * 2 + 655 * 2 * 40,
                    'd2h_bytes_per_step': 65536 * 32 * 4 + 655 * 2 * 30 * 8,
                    'path': 'pyxopto_gb300.surrogate.Surrogate.serve'}}


def mlp_train_bench(args):
    """One training step of the surrogate network 4-256-256-256-30 at batch
    4096 on the library's kernels (forward, loss gradient, backward, tied
    input columns, AdamW), timed with CUDA events over 50 steps per step of
    the bench; metric training profiles/s."""
    import torch
    from pyxopto_gb300 import _lib
    from pyxopto_gb300.surrogate import Mlp, split_bf16, features
    _lib.load().mcgb_mlp_gemm_path(0 if args.mlp_gemm == 'tcgen05' else 1)
    rng = np.random.default_rng(0)
    m = 4096
    x = features(np.exp(rng.uniform(0, 6.9, m)), np.exp(rng.uniform(6.2, 8.5, m)),
                 rng.uniform(0.6, 0.95, m), rng.uniform(1.33, 1.5, m))
    t = np.zeros((m, 32), np.float32)
    t[:, :30] = rng.normal(0, 1, (m, 30))
    net = Mlp(sizes=(4, 256, 256, 256, 30), batch=m)
    xd = split_bf16(x)
    td = torch.from_numpy(t).cuda()
    inner = 50
    for _ in range(args.warmup * inner):
        net.train_step(xd, td, 30, 1e-4)
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(args.steps * inner):
        net.train_step(xd, td, 30, 1e-4)
    b.record()
    torch.cuda.synchronize()
    ms = a.elapsed_time(b) / (args.steps * inner)
    # launches per step: the layers' forward GEMMs, the loss gradient, per
    # layer the activation backward + bias sum and the weight gradient + slice
    # sum, the input gradients below the top layer, the tied input columns and
    # one AdamW over every tensor
    nl = len(net.w)
    launches = nl + 1 + 4 * nl + (nl - 1) + (1 if net.split else 0) + 1
    flops = 3 * 2 * m * (16 * 256 + 256 * 256 * 2 + 256 * 32)
    return {'metric': 'training profiles/s (MLP 4-256-256-256-30, batch 4096)', 'value': m / (ms / 1e3),
            'unit': 'profiles/s', 'ms_per_step': ms, 'tflops_dense': flops / (ms / 1e3) / 1e12,
            'config': {'workload': 'mlp_train_step', 'batch': m, 'layers': '4-256-256-256-30 (16/32 padded)',
                       'steps_per_bench_step': inner, 'gemm': args.mlp_gemm},
            'gpu_launches': args.steps * inner * launches}


def fiber_sweep_bench(args):
    """The reference's own performance workload (test/performance.py running
    xopto/mcml/test/validate.py:348-511): 400 sequential Mc.run calls of
    1e7 packets each (a 20 x 20 mua/mus' sweep, UniformFiberNI source),
    timed through the public API; one step = one sweep.  The reference
    prints 5.7 s per sweep for an RTX A6000 (OpenCL, fast relaxed math).
    Workload 'fiber_sweep_vox' is the voxelized version
    (test/mcvox/performance.py running xopto/mcvox/test/validate.py:357-536:
    the layer as one voxel, UniformFiber source), 8.3 s on an RTX A6000."""
    import torch
    import fiber_sweep
    from pyxopto_gb300 import _abi
    vox = args.workload == 'fiber_sweep_vox'
    data = fiber_sweep.load()
    nphotons = int(args.packets or 10_000_000)
    builder = fiber_sweep.build_vox if vox else fiber_sweep.build
    sim = builder(data, fast=args.math == 'fast', scheduling=args.scheduling)
    for _ in range(args.warmup):
        fiber_sweep.run(sim, data, nphotons)
    torch.cuda.synchronize()
    sampler = ClockSampler(0)
    sampler.start()
    times, errs = [], []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        refl, _ = fiber_sweep.run(sim, data, nphotons)
        torch.cuda.synchronize()
        times.append(time.perf_counter() - t0)
        errs.append(float(fiber_sweep.relative_error(data, refl).mean()))
    clocks = sampler.stop()
    sweep_s = float(np.mean(times))
    npk = nphotons * data['reflectance'].shape[0] * data['reflectance'].shape[1]
    return {'metric': 'packets/s (fibre sweep through Mc.run, 400 x {:.0e} packets)'.format(nphotons),
            'value': npk / sweep_s, 'unit': 'packets/s', 'ms_per_step': sweep_s * 1e3,
            'seconds_per_sweep': sweep_s,
            'reference_published_seconds_per_sweep': (
                {'RTX A6000': 8.3, 'RTX 2080 Ti': 9.9, 'source': 'test/mcvox/performance.py:138-141'}
                if vox else {'RTX A6000': 5.7, 'RTX 2080 Ti': 7.4, 'source': 'test/performance.py:122-125'}),
            'mean_rel_error_vs_cuda_mcml_pct': float(np.mean(errs)),
            'config': {'workload': args.workload, 'simulations': 400, 'packets_per_sim': nphotons,
                       'medium': 'mcvox (one voxel)' if vox else 'mcml',
                       'source': ('UniformFiber' if vox else 'UniformFiberNI') + ' 200 um, NA 0.22',
                       'layer_mm': 8, 'rmax_m': 5e-3,
                       'detector': 'Radial 0-1.7 mm / 340 bins, fibre acceptance',
                       'math': args.math, 'scheduling': args.scheduling},
            'clocks': clocks, 'gpu_launches': 400 * args.steps,
            'e2e': {'value': npk / sweep_s, 'unit': 'packets/s',
                    'h2d_bytes_per_step': 400 * (C.sizeof(_abi.McgbMcvoxConfig) + 2 * C.sizeof(_abi.McgbMaterial) if vox else C.sizeof(_abi.McgbMcmlConfig)),
                    'd2h_bytes_per_step': 400 * (8 * 340 + 8 * _abi.NUM_COUNTERS),
                    'path': 'pyxopto_gb300.{}.mc.Mc.run, 400 calls'.format('mcvox' if vox else 'mcml')}}


DEFAULT_WORKLOAD = 'c2_skin_gk_fluence'


def _transport_summary(args, workload):
    """The 10 mm slab or the 200^3 skin and vessel voxels, measured like the
    default workload, compactly."""
    import copy
    a = copy.copy(args)
    a.workload, a.steps, a.warmup, a.e2e_steps = workload, 3, 2, 2
    res = gpu_bench(a, 0, 1, 0)
    n = res['nphotons']
    kern_s = float(np.mean(res['kernel_ms'])) / 1e3
    achieved = res['ref_spp'] * n * OPS_PER_STEP / kern_s / 1e12
    out = {'value': n * a.steps / (res['total_ms'] / 1e3), 'unit': 'packets/s',
           'e2e': res['e2e']['value'] if res['e2e'] else None, 'kernel_ms': kern_s * 1e3,
           'roofline_frac': achieved / res['fp32_peak'], 'achieved_tflops': achieved,
           'ref_steps_per_packet': res['ref_spp'],
           'executed_steps_per_packet': res['steps_per_launch'] / float(n),
           'clocks': res['clocks']}
    if not args.no_cpu_baseline:
        rate, meta = reference_cpu(workload, seconds=args.cpu_seconds / 2)
        out['cpu_baseline'] = dict(meta, value=rate, unit='packets/s')
    return out


def other_workloads(args, fp32_peak):
    """The other benchmark configurations, measured in the same run as the
    headline line: the 10 mm slab (1e6 packets), the 200^3 skin and vessel
    voxels (1e8 packets), the batched engine (4096 simulations) and the
    surrogate with its Monte Carlo judge (65536 queries).  Each entry has its
    own timing (CUDA events for the device values); failures are recorded,
    not raised."""
    import copy
    out = {}
    for name in ('c1_slab_hg_radial', 'c3_vox_skin_vessel'):
        try:
            out[name] = _transport_summary(args, name)
        except Exception as e:          # keep the headline line
            out[name] = {'error': repr(e)}
    try:
        a = copy.copy(args)
        a.steps, a.warmup, a.e2e_steps, a.sims = 2, 1, 1, 4096
        r = batched_bench(a)
        out['batched_4096'] = {k: r[k] for k in ('value', 'unit', 'ms_per_step', 'packets_per_s',
                                                 'steps_per_s', 'sequential_plain_mc', 'clocks')}
        out['batched_4096']['e2e'] = r['e2e']['value']
        out['batched_4096']['roofline_frac'] = r['steps_per_s'] * OPS_PER_STEP / 1e12 / fp32_peak
    except Exception as e:
        out['batched_4096'] = {'error': repr(e)}
    try:
        a = copy.copy(args)
        a.steps, a.warmup, a.seq_profiles = 2, 1, 16
        r = surrogate_bench(a)
        out['surrogate'] = {k: r[k] for k in ('value', 'unit', 'ms_per_step', 'gain_vs_sequential_plain_mc',
                                              'sequential_plain_mc_profiles_per_s', 'fallback_all',
                                              'surrogate_rms_rel_vs_mc', 'clocks')}
        out['surrogate']['judge'] = {k: r['judge'][k] for k in (
            'judge_fail_fraction', 'judge_rms_rel_median', 'judge_rms_rel_p90', 'judge_noise_rms_rel_median')}
        out['surrogate']['held_out_at_training'] = (r['held_out_at_training'] or {}).get('error')
    except Exception as e:
        out['surrogate'] = {'error': repr(e)}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=5)
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--impl', default='gb300', choices=['gb300', 'reference'])
    ap.add_argument('--workload', default=DEFAULT_WORKLOAD)
    ap.add_argument('--math', default='fast', choices=['fast', 'exact'])
    ap.add_argument('--scheduling', default='dynamic', choices=['dynamic', 'static'])
    ap.add_argument('--e2e-steps', type=int, default=2)
    ap.add_argument('--no-e2e', action='store_true')
    ap.add_argument('--no-cpu-baseline', action='store_true')
    ap.add_argument('--no-others', action='store_true',
                    help='default workload only: skip the other configurations in the same line')
    ap.add_argument('--cpu-seconds', type=float, default=12.0)
    ap.add_argument('--sims', type=int, default=4096, help='batched workload: simulations')
    ap.add_argument('--seq-profiles', type=int, default=16)
    ap.add_argument('--mlp-gemm', choices=['tcgen05', 'mma_sync'], default='tcgen05',
                    help='GEMM implementation of the surrogate kernels (mlp_train_step, surrogate)')
    ap.add_argument('--packets', type=int, default=None,
                    help='override the packets per step (small profiling cases only; '
                         'a headline number uses the workload size)')
    args = ap.parse_args()
    rank, world, local_rank = dist_env()
    if args.workload in ('batched_4096', 'surrogate', 'fiber_sweep', 'fiber_sweep_vox',
                         'mlp_train_step') and args.impl == 'gb300':
        import torch
        torch.cuda.set_device(local_rank)
        res = {'batched_4096': batched_bench, 'surrogate': surrogate_bench,
               'fiber_sweep': fiber_sweep_bench, 'fiber_sweep_vox': fiber_sweep_bench,
               'mlp_train_step': mlp_train_bench}[args.workload](args)
        line = dict({'n_gpus': 1, 'steps': args.steps, 'warmup': args.warmup, 'higher_is_better': True,
                     'scaling': 'none', 'vs_baseline': None, 'dtype': 'f32',
                     'data': 'synthetic (seeded parameter draws and RNG streams)'}, **res)
        if rank == 0:
            print(json.dumps(line))
        return
    import scenarios
    spec = scenarios.ALL[args.workload]
    config = {'workload': args.workload, 'packets_per_step': int(args.packets or spec['nphotons']),
              'medium': spec['medium'], 'math': args.math, 'scheduling': args.scheduling,
              'l2': 'flushed between steps (256 MB write); fluence tally {:.0f} MB'.format(
                  8.0 * np.prod([a[2] for a in (spec['fluence']['x'], spec['fluence']['y'],
                                                spec['fluence']['z'])]) / 1e6 if spec.get('fluence') else 0.0)}

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
    fp32_derived = 152 * 128 * 2 * sm_max * 1e6 / 1e12
    fp32_peak = res['fp32_peak']
    ref_steps = res['ref_spp'] * n
    achieved = ref_steps * OPS_PER_STEP / (kern_ms / 1e3) / 1e12
    executed = res['steps_per_launch'] * OPS_PER_STEP / (kern_ms / 1e3) / 1e12
    key = (args.workload, args.math, args.scheduling)
    traffic = PROFILED_TRAFFIC.get(key)
    roofline = {'bound': 'fp32', 'achieved': achieved, 'peak': fp32_peak, 'unit': 'TFLOP/s',
                'frac': achieved / fp32_peak, 'traffic': traffic[0] if traffic else None,
                'traffic_source': traffic[1] if traffic else None,
                'issue_active': (PROFILED_ISSUE_ACTIVE.get(key) or (None,))[0],
                'peak_source': 'measured in this run: FP32 FMA throughput of the library probe kernel '
                               '(mcgb_fp32_fma_rate, {blocks} blocks x {threads} threads, best of 3 '
                               'launches of {ms:.1f} ms); MEASURED_PEAKS.json holds no FP32 '
                               'peak'.format(**res['fp32_probe']),
                'peak_derived': fp32_derived,
                'peak_derived_source': '152 SMs x 128 FP32 lanes x 2 flops x sm_max_mhz {}'.format(sm_max),
                'ops_per_step': OPS_PER_STEP, 'ref_steps_per_packet': res['ref_spp'],
                'ref_steps_source': res['ref_spp_source'], 'ref_steps_per_launch': ref_steps,
                'executed_steps_per_launch': res['steps_per_launch'],
                'executed_achieved': executed, 'executed_frac': executed / fp32_peak,
                'kernel_ms': kern_ms, 'steps_per_s': ref_steps / (kern_ms / 1e3)}
    l2 = PROFILED_L2_ATOMICS.get(key)
    if l2:
        roofline['l2_atomics'] = dict(l2[0], source=l2[1])
    hbm = PROFILED_HBM.get(key)
    if hbm:
        hbm_peak = peaks.get('hbm_gbs')
        roofline['hbm'] = dict(hbm[0], source=hbm[1], peak_gbs=hbm_peak or HBM_FALLBACK_GBS,
                               peak_source='MEASURED_PEAKS.json' if hbm_peak else
                               'fallback 6.8 TB/s (MEASURED_PEAKS.json absent)',
                               frac=hbm[0]['gbs'] / (hbm_peak or HBM_FALLBACK_GBS))
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
    if world == 1 and args.workload == DEFAULT_WORKLOAD and not args.packets and not args.no_others:
        line['other_workloads'] = other_workloads(args, fp32_peak)
    print(json.dumps(line))
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == '__main__':
    main()
