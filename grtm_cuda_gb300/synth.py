"""Seeded synthetic layered models and receiver sets (the workloads of the
tests, the learned sampler's training sweeps and the benchmark).

Each generator returns ``(model_kwargs, dists)`` where ``model_kwargs`` feeds
``make_model(**model_kwargs)``: layer tops (km, first 0, last = half-space),
Vp, Vs (km/s), density (g/cm^3), Qp, Qs, source depth hs, receiver depth hr
and the source type (0 single force, 1 moment tensor).
"""
import numpy as np


def _off_interface(tops, hs):
    # a source exactly on an interface is moved 0.5 m down (the reference
    # inserts an interface at the source depth; one already there is ambiguous)
    if np.min(np.abs(np.asarray(tops) - hs)) < 1e-9:
        hs += 0.0005
    return hs


def crust(rng, n_layers, hs, src_type=1):
    """Crustal column of n_layers layers over a half-space: thickness
    U(0.5, 5) km, Vp rising linearly 2.5 -> 8.0 km/s plus N(0, 0.15),
    Vs = Vp / U(1.65, 1.85), Gardner density 1.74 Vp^0.25, Qs ~ U(50, 300),
    Qp = 2 Qs."""
    h = rng.uniform(0.5, 5.0, n_layers)
    tops = np.concatenate([[0.0], np.cumsum(h)])
    vp = np.linspace(2.5, 8.0, n_layers + 1) + rng.normal(0.0, 0.15, n_layers + 1)
    vs = vp / rng.uniform(1.65, 1.85, n_layers + 1)
    rho = 1.74 * vp ** 0.25
    qs = rng.uniform(50.0, 300.0, n_layers + 1)
    qp = 2.0 * qs
    hs = min(float(hs), float(tops[-1]) - 0.25)   # the source stays above the half-space
    return dict(ztop=tops, vp=vp, vs=vs, rho=rho, qp=qp, qs=qs, hs=_off_interface(tops, hs), hr=0.0,
                src_type=src_type)


def crust4_model(seed=0):
    """Four layers over a half-space (tops 0/2/10/20/35 km), Vp 3.0/5.8/6.5/7.0/8.0,
    Vs = Vp/1.73, rho = 1.74 Vp^0.25, Qp 200, Qs 100; source 10 km; 10
    receivers at 10..100 km."""
    tops = np.array([0.0, 2.0, 10.0, 20.0, 35.0])
    vp = np.array([3.0, 5.8, 6.5, 7.0, 8.0])
    m = dict(ztop=tops, vp=vp, vs=vp / 1.73, rho=1.74 * vp ** 0.25, qp=np.full(5, 200.0),
             qs=np.full(5, 100.0), hs=10.0, hr=0.0, src_type=1)
    return m, np.arange(10.0, 101.0, 10.0)


def crust20_model(seed):
    """20 layers + half-space, source 15 km, 200 receivers log-spaced 5-300 km."""
    rng = np.random.default_rng(seed)
    m = crust(rng, 20, 15.0)
    return m, np.logspace(np.log10(5.0), np.log10(300.0), 200)


def crust40_model(seed, n_receivers=1000, hs=None):
    """40 layers + half-space, receivers uniform in 1-500 km (sorted); source
    15 km unless given."""
    rng = np.random.default_rng(seed)
    m = crust(rng, 40, 15.0 if hs is None else hs)
    return m, np.sort(rng.uniform(1.0, 500.0, n_receivers))


def uneven_models(seed, n_models=256):
    """Uneven batch: layer counts U{3..60}, source depth U(1, 30) km, random
    double-couple (strike, dip, rake), 16-512 receivers in 5-400 km, N in
    {1024, 2048, 4096} samples at dt 0.05 s.  Yields dicts with keys model,
    dists, log2n, dc (strike, dip, rake in degrees)."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n_models):
        nl = int(rng.integers(3, 61))
        m = crust(rng, nl, rng.uniform(1.0, 30.0))
        nr = int(rng.integers(16, 513))
        dists = np.sort(rng.uniform(5.0, 400.0, nr))
        log2n = int(rng.choice([10, 11, 12]))
        dc = (rng.uniform(0, 360), rng.uniform(0, 90), rng.uniform(-180, 180))
        out.append(dict(model=m, dists=dists, log2n=log2n, dc=dc))
    return out
