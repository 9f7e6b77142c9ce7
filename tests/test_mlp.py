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


@pytest.mark.parametrize('sizes', [(4, 256, 256, 256, 30), (4, 64, 64, 30)])
def test_forward_and_gradients_match_oracle(cuda, sizes):
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
