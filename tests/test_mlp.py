"""Surrogate MLP kernels: forward pass and gradients against the float64 CPU
oracle (oracle/mlp_oracle.py), deterministic gradients, training
convergence, and the end-to-end surrogate with its Monte Carlo judge."""
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


def test_forward_and_gradients_match_oracle(cuda):
    torch = cuda
    sizes = (4, 64, 64, 30)
    m = 512
    net = _net(torch, sizes, batch=m)
    rng = np.random.default_rng(5)
    x = np.zeros((m, 16), np.float32)
    x[:, :4] = rng.uniform(-1, 1, (m, 4))
    xb = torch.from_numpy(x).cuda().to(torch.bfloat16)
    y = net.forward(xb).float().cpu().numpy()
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
    assert np.max(np.abs(y - yo)) <= 2e-2 * max(1.0, np.max(np.abs(yo)))
    dyo = mo.from_bits(dyb.view(torch.int16).cpu().numpy().view(np.uint16))
    dwo, dbo = mo.backward(ws, inputs, pres, dyo, acts)
    for i in range(len(ws)):
        assert np.linalg.norm(dw[i] - dwo[i]) <= 2e-2 * np.linalg.norm(dwo[i]), i
        assert np.linalg.norm(db[i] - dbo[i]) <= 2e-2 * np.linalg.norm(dbo[i]) + 1e-6, i
    # deterministic: the same backward twice gives the same bits
    net.forward(xb)
    net.backward(dyb, m)
    assert all(np.array_equal(a.cpu().numpy(), b_) for a, b_ in zip(net.dw, [d.astype(np.float32) for d in dw]))


def test_mse_gradient_matches_oracle(cuda):
    torch = cuda
    from pyxopto_gb300.surrogate import Mlp
    net = Mlp(sizes=(4, 32, 30), batch=256)
    rng = np.random.default_rng(2)
    y = rng.normal(0, 1, (256, 32)).astype(np.float32)
    t = rng.normal(0, 1, (256, 32)).astype(np.float32)
    yb = torch.from_numpy(y).cuda().to(torch.bfloat16)
    dy = net.mse_grad(yb, torch.from_numpy(t).cuda(), 256, 30)
    got = dy.float().cpu().numpy()
    ref, loss = mo.mse_grad(mo.from_bits(yb.view(torch.int16).cpu().numpy().view(np.uint16)), t, 30)
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


def test_surrogate_end_to_end(cuda, lib):
    from pyxopto_gb300.batched import BatchedMc
    from pyxopto_gb300.surrogate import Surrogate, sequential_plain_mc
    sur = Surrogate()
    train = BatchedMc.sample_sims(8192, seed=21, packets=(20000, 20001))
    refl = sur.simulate(train)
    hist = sur.fit(train, refl, epochs=25, batch=1024)
    assert hist[-1] < 0.2 * hist[0]
    test = BatchedMc.sample_sims(2048, seed=22, packets=(1, 2))
    out, rep = sur.serve(test, judge_fraction=0.05, judge_packets=200000, tol=0.05, max_fail=1.0,
                         rel_floor=1e-3)
    assert out.shape == (2048, 30)
    assert rep['judge_rms_rel_median'] < 0.1, rep
    # what the network gains: the same 2048 profiles from sequential plain
    # Monte Carlo at the judge's packet count
    seq = BatchedMc.sample_sims(5, seed=23, packets=(1, 2))
    plain = sequential_plain_mc(seq, 200000)
    assert rep['profiles_per_s'] > 10.0 * plain, (rep['profiles_per_s'], plain)
