"""Failure detection without faulting the GPU: the kernels bound their own
run time (device clock deadline), poll a host-written abort word and cap the
steps of a packet, and report each as a status the host reads; the context
stays usable afterwards."""
import ctypes as C
import time

import numpy as np
import pytest

import scenarios

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize('scheduling', ['static', 'dynamic'])
def test_deadline_expiry_is_reported_and_device_stays_usable(cuda, lib, oracle, scheduling):
    from pyxopto_gb300 import _abi, _lib
    mc = scenarios.build_mc('c2_gk_fluence', fast=True, scheduling=scheduling)
    mc.deadline = 0.25
    t0 = time.perf_counter()
    with pytest.raises(_lib.McgbError) as ei:
        mc.run(10_000_000_000)                   # ~100 s of work
    assert ei.value.code == _abi.E_TIMEOUT
    assert time.perf_counter() - t0 < 30.0
    rep = mc.run_report
    assert rep['status'] & _abi.STATUS_TIMEOUT
    assert rep['packets_done'] < 10_000_000_000
    # a normal run afterwards is still bit-identical to the oracle
    ok = scenarios.build_mc('c1_line_hg_radial')
    ref = oracle.run(ok, 1000, 32, oracle.PORTABLE)
    ok.run(1000, maxthreads=32)
    got = oracle.tallies(ok, ok._dev['accu'].cpu().numpy().view(np.uint64))
    assert np.array_equal(got['top'], ref['top'])


def test_host_abort_word_stops_the_kernel(cuda, lib):
    from pyxopto_gb300 import _abi, _lib
    import torch
    mc = scenarios.build_mc('c2_gk_fluence', fast=True)
    n, t = 1_000_000_000, 4096
    cfg = mc.pack(n, t)
    mc._ensure_streams(torch, t, torch.device('cuda'))
    b = mc._device_buffers(torch, torch.device('cuda'), mc._lut_array(), {})
    mc._dev['counters'][_abi.CNT_ABORT] = 1
    code, counters = mc._launch(lib.mcgb_mcml_run, cfg, b, torch)
    assert code == _abi.E_TIMEOUT
    assert counters[_abi.CNT_STATUS] & _abi.STATUS_ABORTED
    assert counters[_abi.CNT_PACKETS] < n


def test_packet_step_limit_is_a_status_not_an_error(cuda, lib):
    from pyxopto_gb300 import _abi
    mc = scenarios.build_mc('semiinf_hg', fast=True)
    mc.max_steps_per_packet = 3
    mc.run(20000, maxthreads=512)
    rep = mc.run_report
    assert rep['status'] & _abi.STATUS_STEP_LIMIT
    assert rep['packets_done'] == 20000
    assert rep['steps'] <= 3 * 20000


def test_batched_deadline(cuda, lib):
    from pyxopto_gb300 import _abi, _lib
    from pyxopto_gb300.batched import BatchedMc
    sims = BatchedMc.sample_sims(256, seed=2, packets=(1e8, 1e8 + 1))
    b = BatchedMc(sims)
    cfg = b.config()
    cfg.deadline_s = 0.2
    import torch
    d = b._buffers(torch)
    with pytest.raises(_lib.McgbError) as ei:
        b._launch(torch, cfg, d, torch.cuda.current_stream().cuda_stream)
        counters = (C.c_uint64 * _abi.NUM_COUNTERS)()
        _lib.check(lib.mcgb_check_counters(C.c_void_p(d['counters'].data_ptr()),
                                           C.c_void_p(torch.cuda.current_stream().cuda_stream),
                                           counters))
    assert ei.value.code == _abi.E_TIMEOUT
