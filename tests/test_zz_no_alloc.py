"""The allocation-free batched entry point.

Callers that cannot allocate device memory (inside another framework's
memory pool, in a real-time loop where cudaMalloc is forbidden, or in a
plugin host that hands over only input and output buffers) call
mcgb_batched_run_noalloc, which keeps its scratch in a fixed array inside
the library.  This test calls it through the C ABI twice in a row and
checks both results against mcgb_batched_run with a caller-owned work
buffer.  The tallies are integers and independent of scheduling, so the
results must be identical.  The file is collected last so that a stopping
failure here comes after every other test has run."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_noalloc_batched_matches_caller_scratch_twice(cuda, lib):
    import torch
    from pyxopto_gb300 import _abi, _lib
    from pyxopto_gb300.batched import BatchedMc
    sims = BatchedMc.sample_sims(300, seed=17, packets=(2000, 20000))
    b = BatchedMc(sims, fast=True)
    cfg = b.config()
    d = b._buffers(torch)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)

    def read(code):
        _lib.check(code)
        counters = (C.c_uint64 * _abi.NUM_COUNTERS)()
        _lib.check(lib.mcgb_check_counters(C.c_void_p(d['counters'].data_ptr()), stream, counters))
        return d['tally'].cpu().numpy().view(np.uint64).copy()

    d['tally'].zero_()
    d['counters'].zero_()
    ref = read(lib.mcgb_batched_run(C.byref(cfg), C.c_void_p(d['sims'].data_ptr()),
                                    C.c_void_p(d['mult'].data_ptr()), C.c_void_p(d['tally'].data_ptr()),
                                    C.c_void_p(d['work'].data_ptr()), C.c_void_p(d['counters'].data_ptr()),
                                    stream))
    assert ref.sum() > 0
    for _ in range(2):
        d['tally'].zero_()
        d['counters'].zero_()
        got = read(lib.mcgb_batched_run_noalloc(C.byref(cfg), C.c_void_p(d['sims'].data_ptr()),
                                                C.c_void_p(d['mult'].data_ptr()),
                                                C.c_void_p(d['tally'].data_ptr()),
                                                C.c_void_p(d['counters'].data_ptr()), stream))
        assert np.array_equal(got, ref)


def test_noalloc_rejects_batches_beyond_its_array(cuda, lib):
    from pyxopto_gb300 import _abi
    cfg = _abi.McgbBatchConfig()
    cfg.num_sims = 8193
    assert lib.mcgb_batched_run_noalloc(C.byref(cfg), None, None, None, None, None) == _abi.E_SIZE
    assert b'8192' in lib.mcgb_last_error()
