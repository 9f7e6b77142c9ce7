"""Training-set generation and training of the radial-reflectance surrogate.

    python -m pyxopto_gb300.train_surrogate generate --profiles 262144 \
        --packets 1000000 --test-profiles 2048 --test-packets 10000000 --out DIR
    python -m pyxopto_gb300.train_surrogate fit --data DIR --out WEIGHTS.npz

``generate`` draws the simulations from the batched benchmark's ranges
(mua log-uniform in [1, 1000] 1/m, mus' log-uniform in [500, 5000] 1/m, g
uniform in [0.6, 0.95], n uniform in [1.33, 1.5]) and runs them on the GPU
with the batched engine, every profile as two independent halves of
packets/2 packets (one launch per chunk).  It writes

  DIR/train.npz  the optical properties, the mean profile R (float32,
                 radial reflectance in 1/m^2 per packet, 30 bins of
                 0.1 mm; the last bin also holds the radii beyond 3 mm) and
                 the relative half difference (a - b)/(a + b) (float16),
                 an estimate of each bin's Monte Carlo noise;
  DIR/test.npz   a held-out set simulated the same way at a higher packet
                 count (both halves kept), the reference of the accuracy
                 figures;
  DIR/generate.json  sizes, seeds and timings.

``fit`` trains the network with the library's own kernels (Surrogate.fit),
evaluates it on the held-out set (noise-corrected relative RMS error per
profile) and writes the weights and a JSON training log.
"""
import argparse
import json
import os
import time

import numpy as np

from .batched import BatchedMc
from .surrogate import Surrogate


def _halves(sur, sims, packets, seed):
    a, b = sur.simulate_halves(sims, packets, seed=seed)
    return a.astype(np.float64), b.astype(np.float64)


def generate(out, profiles, packets, test_profiles, test_packets, seed=21, test_seed=99,
             chunk=16384, log=print):
    import torch
    os.makedirs(out, exist_ok=True)
    sur = Surrogate()
    nb = sur.raxis.n
    sims = BatchedMc.sample_sims(profiles, seed=seed, packets=(packets, packets + 1))
    R = np.empty((profiles, nb), np.float32)
    D = np.empty((profiles, nb), np.float16)
    t0 = time.perf_counter()
    for s in range(0, profiles, chunk):
        e = min(profiles, s + chunk)
        sub = {k: np.asarray(v)[s:e] for k, v in sims.items()}
        a, b = _halves(sur, sub, packets, seed=1000 + s // chunk)
        R[s:e] = 0.5 * (a + b)
        D[s:e] = np.where(a + b > 0, (a - b) / np.where(a + b > 0, a + b, 1.0), 0.0)
        torch.cuda.synchronize()
        log('train chunk {}-{}: {:.1f} s'.format(s, e, time.perf_counter() - t0))
    t_train = time.perf_counter() - t0
    f32 = lambda v: np.asarray(v, np.float32)
    np.savez(os.path.join(out, 'train.npz'), mua=f32(sims['mua']), mus=f32(sims['mus']),
             g=f32(sims['g']), n=f32(sims['n']), R=R, D=D, packets=np.array([packets]),
             seed=np.array([seed]))
    t1 = time.perf_counter()
    test = BatchedMc.sample_sims(test_profiles, seed=test_seed, packets=(1, 2))
    ta, tb = _halves(sur, test, test_packets, seed=777)
    torch.cuda.synchronize()
    t_test = time.perf_counter() - t1
    np.savez(os.path.join(out, 'test.npz'), mua=test['mua'], mus=test['mus'], g=test['g'],
             n=test['n'], a=ta.astype(np.float32), b=tb.astype(np.float32),
             packets=np.array([test_packets]), seed=np.array([test_seed]))
    info = {'profiles': profiles, 'packets': packets, 'seed': seed, 'train_seconds': t_train,
            'train_packets_per_s': profiles * packets / t_train, 'test_profiles': test_profiles,
            'test_packets': test_packets, 'test_seed': test_seed, 'test_seconds': t_test,
            'device': torch.cuda.get_device_name()}
    with open(os.path.join(out, 'generate.json'), 'w') as f:
        json.dump(info, f, indent=1)
    log(json.dumps(info))
    return info


def load_train(data):
    d = np.load(os.path.join(data, 'train.npz'))
    sims = {k: d[k].astype(np.float64) for k in ('mua', 'mus', 'g', 'n')}
    return sims, d['R'].astype(np.float64), d['D'].astype(np.float64), int(d['packets'][0])


def load_test(data):
    d = np.load(os.path.join(data, 'test.npz'))
    sims = {k: d[k].astype(np.float64) for k in ('mua', 'mus', 'g', 'n')}
    return sims, d['a'].astype(np.float64), d['b'].astype(np.float64)


def evaluate(sur, sims, a, b):
    """Noise-corrected relative RMS error of the surrogate per held-out
    profile, with the raw error and the reference's own noise."""
    musr = np.asarray(sims['mus']) * (1.0 - np.asarray(sims['g']))
    pred = sur.predict(sims['mua'], musr, sims['g'], sims['n'])
    err, raw, noise = Surrogate.judge_error(pred, a, b)
    stat = lambda v: {'mean': float(np.mean(v)), 'median': float(np.median(v)),
                      'p90': float(np.percentile(v, 90)), 'p99': float(np.percentile(v, 99)),
                      'max': float(np.max(v))}
    return {'profiles': int(len(err)), 'error': stat(err), 'raw': stat(raw),
            'reference_noise': stat(noise), 'share_above_1pct': float(np.mean(err > 0.01))}


def main(argv=None):
    ap = argparse.ArgumentParser()
    sub = ap.add_subparsers(dest='cmd', required=True)
    g = sub.add_parser('generate')
    g.add_argument('--out', required=True)
    g.add_argument('--profiles', type=int, default=1 << 18)
    g.add_argument('--packets', type=int, default=1_000_000)
    g.add_argument('--test-profiles', type=int, default=2048)
    g.add_argument('--test-packets', type=int, default=10_000_000)
    g.add_argument('--chunk', type=int, default=16384)
    f = sub.add_parser('fit')
    f.add_argument('--data', required=True)
    f.add_argument('--out', required=True)
    f.add_argument('--epochs', type=int, default=400)
    f.add_argument('--batch', type=int, default=4096)
    f.add_argument('--lr', type=float, default=2e-3)
    f.add_argument('--warm-epochs', type=int, default=10)
    args = ap.parse_args(argv)
    import torch
    torch.cuda.set_device(0)
    if args.cmd == 'generate':
        generate(args.out, args.profiles, args.packets, args.test_profiles, args.test_packets,
                 chunk=args.chunk, log=lambda s: print(s, flush=True))
        return
    sims, R, D, packets = load_train(args.data)
    sur = Surrogate()
    sur.fit(sims, R, epochs=args.epochs, batch=args.batch, lr=args.lr, warm_epochs=args.warm_epochs,
            verbose=True)
    tsims, ta, tb = load_test(args.data)
    ev = evaluate(sur, tsims, ta, tb)
    sur.save(args.out)
    log = {'train_profiles': int(len(R)), 'train_packets': packets, 'epochs': args.epochs,
           'batch': args.batch, 'lr': args.lr, 'warm_epochs': args.warm_epochs,
           'train_seconds': sur.report['train_seconds'], 'train_steps': sur.report['train_steps'],
           'loss_first': sur.report['loss'][0], 'loss_last': sur.report['loss'][-1], 'held_out': ev}
    with open(os.path.splitext(args.out)[0] + '.log.json', 'w') as fh:
        json.dump(log, fh, indent=1)
    print(json.dumps(log))


if __name__ == '__main__':
    main()
