"""Surrogate MLP kernels: forward pass and gradients against the float64 CPU
oracle (oracle/mlp_oracle.py) at the served network's shape
4-256-256-256-30, deterministic gradients, both loss modes, training
convergence, and the served surrogate with its Monte Carlo judge and
fallback."""
import numpy as np
import pytest

import mlp_oracle as mo

pytestmark = pytest.mark.gpu


def _net(torch, sizes, seed=0, batch=512):
    from pyxopto_gb300.surrogate import Mlp
    net = Mlp(sizes=sizes, seed=seed, batch=batch)
    rng = np.random.default_rng(seed + 1)
    for i in range(len(net.w)):
        w = net.w[i].cpu().numpy()
        w[:] = 0.0
        n, k = sizes[i + 1], sizes[i]
        w[:n, :k] = rng.normal(0, 1.0 / np.sqrt(k), (n, k))
        net.w[i].copy_(torch.from_numpy(w))
        net.b[i].copy_(torch.from_numpy(rng.normal(0, 0.1, net.b[i].shape[0]).astype(np.float32)))
    net.sync_copies()
    return net


@pytest.fixture(params=[0, 1], ids=['tcgen05', 'mma_sync'])
def gemm_path(request, lib):
    """Run a test on each GEMM implementation, restoring the default."""
    prev = lib.mcgb_mlp_gemm_path(request.param)
    assert prev in (0, 1)
    yield request.param
    lib.mcgb_mlp_gemm_path(prev)


@pytest.mark.parametrize('sizes', [(4, 256, 256, 256, 30), (4, 64, 64, 30)])
def test_forward_and_gradients_match_oracle(cuda, sizes, gemm_path):
    torch = cuda
    m = 512
    net = _net(torch, sizes, batch=m)
    rng = np.random.default_rng(5)
    x = np.zeros((m, 16), np.float32)
    x[:, :4] = rng.uniform(-1, 1, (m, 4))
    xb = torch.from_numpy(x).cuda().to(torch.bfloat16)
    y = net.forward(xb).cpu().numpy().astype(np.float64)
    dy = np.zeros((m, 32), np.float32)
    dy[:, :30] = rng.normal(0, 1e-2, (m, 30))
    dyb = torch.from_numpy(dy).cuda().to(torch.bfloat16)
    net.backward(dyb, m)
    dw = [d.cpu().numpy().astype(np.float64) for d in net.dw]
    db = [d.cpu().numpy().astype(np.float64) for d in net.db]
    # oracle on the same bf16 values
    ws = [mo.from_bits(w.view(torch.int16).cpu().numpy().view(np.uint16)) for w in net.wb]
    bs = [b.cpu().numpy().astype(np.float64) for b in net.b]
    xs = mo.from_bits(xb.view(torch.int16).cpu().numpy().view(np.uint16))
    acts = net.acts
    inputs, pres, yo = mo.forward(ws, bs, xs, acts)
    assert np.max(np.abs(y[:, :30] - yo[:, :30])) <= 1e-3 * max(1.0, np.max(np.abs(yo)))
    dyo = mo.from_bits(dyb.view(torch.int16).cpu().numpy().view(np.uint16))
    dwo, dbo = mo.backward(ws, inputs, pres, dyo, acts)
    for i in range(len(ws)):
        assert np.linalg.norm(dw[i] - dwo[i]) <= 2e-2 * np.linalg.norm(dwo[i]), i
        assert np.linalg.norm(db[i] - dbo[i]) <= 2e-2 * np.linalg.norm(dbo[i]) + 1e-6, i
    # deterministic: the same backward twice gives the same bits
    net.forward(xb)
    net.backward(dyb, m)
    assert all(np.array_equal(a.cpu().numpy(), b_) for a, b_ in zip(net.dw, [d.astype(np.float32) for d in dw]))


@pytest.mark.parametrize('m,n,k', [(4096, 256, 256), (4096, 32, 256), (4096, 256, 16), (136, 48, 32),
                                   (520, 256, 256), (264, 64, 80), (256, 64, 1024)])
def test_gemm_paths_agree_with_float64(cuda, lib, m, n, k):
    """The three GEMM entry points on the tcgen05 path and on the mma.sync
    path against float64 products of the same bf16 operands: partial tiles
    in every dimension (136 and 264 rows, 48 and 32 columns, 16- and 80-wide
    reductions) and a 1024-deep reduction that refills every shared-memory
    stage of the tcgen05 pipeline four times."""
    import ctypes as C
    from pyxopto_gb300 import _lib
    torch = cuda
    rng = np.random.default_rng(m + 3 * n + 7 * k)
    bf = lambda a: torch.from_numpy(a.astype(np.float32)).cuda().to(torch.bfloat16)
    x = bf(rng.normal(0, 1, (m, k)))
    w = bf(rng.normal(0, 1 / np.sqrt(k), (n, k)))
    wt = w.t().contiguous()
    b = torch.from_numpy(rng.normal(0, 0.1, n).astype(np.float32)).cuda()
    dpre = bf(rng.normal(0, 1e-2, (m, n)))
    X, W, DP = (t.float().cpu().numpy().astype(np.float64) for t in (x, w, dpre))
    ref = {'pre': X @ W.T + b.cpu().numpy().astype(np.float64), 'dx': DP @ W, 'dw': DP.T @ X}
    P = lambda t: C.c_void_p(t.data_ptr())
    out = {}
    for path in (0, 1):
        prev = lib.mcgb_mlp_gemm_path(path)
        try:
            y = torch.full((m, n), float('nan'), dtype=torch.bfloat16, device='cuda')
            pre = torch.full((m, n), float('nan'), device='cuda')
            _lib.check(lib.mcgb_mlp_linear_fwd(P(x), P(w), P(b), P(y), P(pre), m, n, k, 1, None))
            dx = torch.full((m, k), float('nan'), dtype=torch.bfloat16, device='cuda')
            _lib.check(lib.mcgb_mlp_linear_bwd_input(P(dpre), P(wt), P(dx), m, n, k, None))
            scratch = torch.empty(int(lib.mcgb_mlp_bwd_weight_scratch(m, n, k)), device='cuda')
            dw = torch.full((n, k), float('nan'), device='cuda')
            _lib.check(lib.mcgb_mlp_linear_bwd_weight(P(dpre), P(x), P(dw), P(scratch), m, n, k, None))
            torch.cuda.synchronize()
            out[path] = {'pre': pre, 'y': y, 'dx': dx, 'dw': dw}
            out[path] = {key: v.float().cpu().numpy().astype(np.float64) for key, v in out[path].items()}
        finally:
            lib.mcgb_mlp_gemm_path(prev)
    gelu = lambda v: 0.5 * v * (1 + np.tanh(0.7978845608028654 * (v + 0.044715 * v ** 3)))
    for path, o in out.items():
        for key in ('pre', 'dw'):             # FP32 results: accumulation order only
            assert np.max(np.abs(o[key] - ref[key])) <= 1e-4 * np.max(np.abs(ref[key])), (path, key)
        for key, r in (('y', gelu(ref['pre'])), ('dx', ref['dx'])):   # rounded to bf16
            assert np.all(np.abs(o[key] - r) <= 2.0 ** -8 * np.abs(r) + 1e-3 * np.max(np.abs(r))), (path, key)
    assert np.max(np.abs(out[0]['pre'] - out[1]['pre'])) <= 1e-5 * np.max(np.abs(ref['pre']))
    assert lib.mcgb_mlp_gemm_path(-1) == 0
    assert lib.mcgb_mlp_gemm_path(7) == -1


def test_adamw_multi_equals_per_tensor(cuda, lib):
    """The one-launch AdamW of every weight and bias gives the same bits as
    one launch per tensor (weights with weight decay and their transposed
    bf16 copies, biases without), over three steps."""
    from pyxopto_gb300.surrogate import Mlp
    torch = cuda
    a = Mlp(sizes=(4, 64, 64, 30), seed=3, batch=256)
    b = Mlp(sizes=(4, 64, 64, 30), seed=3, batch=256)
    rng = np.random.default_rng(9)
    for _ in range(3):
        for ga, gb in zip(a.dw + a.db, b.dw + b.db):
            g = torch.from_numpy(rng.normal(0, 1e-2, tuple(ga.shape)).astype(np.float32)).cuda()
            ga.copy_(g)
            gb.copy_(g)
        a.adamw(lr=1e-3, wd=1e-2)
        b.adamw_per_tensor(lr=1e-3, wd=1e-2)
    torch.cuda.synchronize()
    for name in ('w', 'b', 'wb', 'wt', 'm', 'v', 'bb', 'mb', 'vb'):
        for x, y in zip(getattr(a, name), getattr(b, name)):
            assert torch.equal(x, y), name


@pytest.mark.parametrize('mode', [0, 1])
def test_loss_gradient_matches_oracle(cuda, mode):
    torch = cuda
    from pyxopto_gb300.surrogate import Mlp
    net = Mlp(sizes=(4, 32, 30), batch=256)
    rng = np.random.default_rng(2)
    y = rng.normal(0, 1, (256, 32)).astype(np.float32)
    t = rng.normal(0, 1, (256, 32)).astype(np.float32)
    if mode == 1:
        t = np.exp(rng.normal(0, 0.5, (256, 32))).astype(np.float32) * np.exp(0.7 * y)
    dy = net.loss_grad(torch.from_numpy(y).cuda(), torch.from_numpy(t).cuda(), 256, 30, mode=mode,
                       scale=0.7)
    got = dy.float().cpu().numpy()
    ref, loss = mo.loss_grad(y.astype(np.float64), t.astype(np.float64), 30, mode=mode, scale=0.7)
    assert np.max(np.abs(got - ref)) <= 1e-2 * np.max(np.abs(ref))
    assert abs(net.loss_part[:1].sum().item() - loss) < 1e-3 * loss


def test_training_reduces_loss(cuda):
    torch = cuda
    from pyxopto_gb300.surrogate import Mlp
    rng = np.random.default_rng(0)
    m = 8192
    x = np.zeros((m, 16), np.float32)
    x[:, :4] = rng.uniform(-1, 1, (m, 4))
    r = np.linspace(0, 1, 30)
    t = np.zeros((m, 32), np.float32)
    t[:, :30] = np.sin(2 * x[:, :1] + r[None, :] * x[:, 1:2]) + 0.5 * x[:, 2:3] * x[:, 3:4]
    net = Mlp(sizes=(4, 256, 256, 256, 30), batch=1024)
    xd = torch.from_numpy(x).cuda().to(torch.bfloat16)
    td = torch.from_numpy(t).cuda()
    losses = []
    for step in range(400):
        s = (step * 1024) % m
        lp = net.train_step(xd[s:s + 1024], td[s:s + 1024], 30, 2e-3)
        losses.append(lp.sum().item())
    assert np.mean(losses[-20:]) < 0.05 * np.mean(losses[:5])


def test_surrogate_fit_reduces_loss(cuda, lib):
    """Both training stages run on the library's kernels: a short fit on
    low-packet profiles lowers the squared error of the first stage and
    the relative error of the second."""
    from pyxopto_gb300.batched import BatchedMc
    from pyxopto_gb300.surrogate import Surrogate
    sur = Surrogate()
    train = BatchedMc.sample_sims(8192, seed=21, packets=(20000, 20001))
    refl = sur.simulate(train)
    hist = sur.fit(train, refl, epochs=30, batch=1024, warm_epochs=10)
    assert hist[9] < 0.2 * hist[0]
    assert hist[-1] < hist[10]


def test_served_surrogate_meets_tolerance_with_fallback_live(cuda, lib):
    """The trained network shipped with the package (trained on the GPU by
    pyxopto_gb300.train_surrogate) served with its Monte Carlo judge at the
    1 % tolerance and the library's default fallback (max_fail 0.1): the
    batch is not re-simulated, the judged errors are low, and the service
    runs at least 100x the profiles/s of sequential plain Mc.run calls at the
    judge's packet count."""
    from pyxopto_gb300.batched import BatchedMc
    from pyxopto_gb300.surrogate import Surrogate, sequential_plain_mc, default_weights
    sur = Surrogate.load(default_weights())
    queries = BatchedMc.sample_sims(16384, seed=5, packets=(1, 2))
    sur.serve(queries, seed=3)                        # warm-up
    out, rep = sur.serve(queries, seed=7)
    assert out.shape == (16384, 30) and np.all(np.isfinite(out))
    assert not rep['fallback_all'], rep
    assert rep['judge_fail_fraction'] <= 0.1, rep
    assert rep['judge_rms_rel_median'] < 0.01, rep
    seq = BatchedMc.sample_sims(9, seed=23, packets=(1, 2))
    plain = sequential_plain_mc(seq, 1_000_000)
    assert rep['profiles_per_s'] > 100.0 * plain, (rep['profiles_per_s'], plain)


def test_split_inputs_keep_16_bits_and_tied_weights_stay_equal(cuda, lib):
    """The network input as high + low bf16 parts reproduces the FP32
    features to about 16 bits, and training keeps the first layer's two
    weight copies identical (mcgb_mlp_tie_columns + AdamW)."""
    torch = cuda
    from pyxopto_gb300.surrogate import Mlp, split_bf16, features
    rng = np.random.default_rng(3)
    x = features(np.exp(rng.uniform(0, 6.9, 512)), np.exp(rng.uniform(6.2, 8.5, 512)),
                 rng.uniform(0.6, 0.95, 512), rng.uniform(1.33, 1.5, 512))
    xs = split_bf16(x).float().cpu().numpy()
    rec = xs[:, :4] + xs[:, 4:8]
    assert np.max(np.abs(rec - x[:, :4])) < 2.0 ** -15
    assert np.max(np.abs(xs[:, :4] - x[:, :4])) > 2.0 ** -12      # bf16 alone is coarser
    net = Mlp(sizes=(4, 64, 30), batch=512)
    t = torch.from_numpy(rng.normal(0, 1, (512, 32)).astype(np.float32)).cuda()
    xd = split_bf16(x)
    for _ in range(5):
        net.train_step(xd, t, 30, 1e-2)
    w = net.w[0].cpu().numpy()
    assert np.array_equal(w[:, :4], w[:, 4:8])
