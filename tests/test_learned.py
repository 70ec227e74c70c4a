"""Learned wavenumber sampler: the network's CUDA kernels against the FP64
numpy oracle, the convergence sweep, and the learned path against the plain
grid (its judge and fallback) and FP64."""
import math
import os

import numpy as np
import pytest

from oracle import mlp_oracle as MO

N_IN, N_OUT = 15, 2


def _data(n, seed=0):
    rng = np.random.default_rng(seed)
    x = rng.normal(size=(n, N_IN))
    t = np.stack([np.sin(x[:, 0]) + 0.5 * x[:, 1] * x[:, 2], np.tanh(x[:, 3] - x[:, 4])], axis=1)
    return x, t


# ---------------------------------------------------------------- CPU
def test_oracle_gradient_matches_finite_differences():
    _, n = MO.layout(N_IN, N_OUT)
    rng = np.random.default_rng(3)
    p = rng.normal(scale=0.2, size=n)
    x, t = _data(6)
    _, g = MO.loss_grad(p, x, t, N_IN, N_OUT)
    idx = rng.choice(n, 40, replace=False)
    h = 1e-6
    for i in idx:
        e = np.zeros(n)
        e[i] = h
        fd = (MO.loss(p + e, x, t, N_IN, N_OUT) - MO.loss(p - e, x, t, N_IN, N_OUT)) / (2 * h)
        assert abs(fd - g[i]) <= 1e-7 + 1e-5 * abs(fd)


def test_sampler_file_roundtrip(tmp_path):
    from grtm_cuda_gb300.learned import Sampler
    _, n = MO.layout(N_IN, N_OUT)
    rng = np.random.default_rng(1)
    s = Sampler(rng.normal(size=n), rng.normal(size=N_IN), rng.uniform(1, 2, N_IN), rng.normal(size=N_OUT),
                rng.uniform(1, 2, N_OUT), margin_k=1.3, margin_d=1.5, tol=2e-4)
    path = str(tmp_path / "k.bin")
    s.save(path)
    r = Sampler.load(path)
    assert np.array_equal(r.params, s.params.astype(np.float32))
    assert np.array_equal(r.x_std, s.x_std) and np.array_equal(r.y_mean, s.y_mean)
    assert (r.margin_k, r.margin_d, r.tol) == (1.3, 1.5, 2e-4) and r.kbands is None
    # per-band k margins: edges in log w, the outer bands open
    s.kbands = (np.array([0.0, 1.0, 2.5]), np.array([2.0, 1.1]))
    s.save(path)
    r = Sampler.load(path)
    assert np.array_equal(r.kbands[0], s.kbands[0]) and np.array_equal(r.kbands[1], s.kbands[1])
    assert np.array_equal(r.k_margin([-5.0, 0.5, 1.0, 2.0, 9.0]), [2.0, 2.0, 1.1, 1.1, 1.1])
    with pytest.raises(ValueError):
        Sampler(s.params, s.x_mean, s.x_std, s.y_mean, s.y_std, kbands=([1.0, 0.0], [1.0]))
    with open(path, "r+b") as f:
        f.write(b"XXXXXXXX")
    with pytest.raises(ValueError):
        Sampler.load(path)


def test_features_finite_on_generators():
    from grtm_cuda_gb300 import learned, synth
    for seed in range(5):
        for nl in (3, 20, 40, 60):
            m = synth.crust(np.random.default_rng(seed), nl, 1.0 + 5 * seed)
            f = learned.layer_features(m)
            assert f.shape == (12,) and np.all(np.isfinite(f))
    m, _ = synth.crust4_model()
    assert np.all(np.isfinite(learned.layer_features(m)))


def test_committed_weights_load():
    from grtm_cuda_gb300 import learned
    if not os.path.exists(learned.WEIGHTS):
        pytest.skip("no trained sampler in the tree")
    s = learned.Sampler.load()
    assert s.params.size == MO.layout(N_IN, N_OUT)[1]
    assert s.margin_k >= 1.0 and s.margin_d >= 1.0 and 0 < s.tol < 1e-2
    if s.kbands is not None:
        assert np.all(s.kbands[1] >= 1.0) and np.all(s.kbands[1] <= s.margin_k * 4)
    # the oracle's forward of the committed network gives finite outputs
    x = np.zeros((4, N_IN))
    y, _ = MO.forward(s.params, x, N_IN, N_OUT)
    assert np.all(np.isfinite(y))


# ---------------------------------------------------------------- GPU
@pytest.fixture(scope="module")
def ctx():
    import grtm_cuda_gb300 as g
    c = g.Context()
    yield c
    c.close()


@pytest.mark.gpu
def test_mlp_forward_matches_oracle(ctx):
    from grtm_cuda_gb300.learned import Mlp
    net = Mlp(ctx, seed=7)
    p = net.get_params().astype(np.float64)
    x, _ = _data(300, 1)
    y = net.forward(x)
    yo, _ = MO.forward(p, x.astype(np.float32), N_IN, N_OUT)
    assert np.max(np.abs(y - yo)) <= 1e-5 * (1 + np.max(np.abs(yo)))
    net.close()


@pytest.mark.gpu
def test_mlp_gradient_matches_oracle(ctx):
    from grtm_cuda_gb300.learned import Mlp
    net = Mlp(ctx, seed=11)
    p = net.get_params().astype(np.float64)
    for n in (1, 63, 64, 257):
        x, t = _data(n, n)
        loss, g = net.loss_grad(x, t)
        lo, go = MO.loss_grad(p, x.astype(np.float32), t.astype(np.float32), N_IN, N_OUT)
        assert abs(loss - lo) <= 1e-5 * abs(lo)
        assert np.linalg.norm(g - go) <= 1e-5 * np.linalg.norm(go)
    net.close()


@pytest.mark.gpu
def test_mlp_adam_step_matches_oracle(ctx):
    from grtm_cuda_gb300.learned import Mlp
    net = Mlp(ctx, seed=5)
    x, t = _data(128, 9)
    lr = 1e-3
    p0 = net.get_params().astype(np.float64)
    m = np.zeros_like(p0)
    v = np.zeros_like(p0)
    for step in (1, 2, 3):
        # one epoch with one batch of all samples is one full-batch Adam step
        p = net.get_params().astype(np.float64)
        _, g = MO.loss_grad(p, x.astype(np.float32), t.astype(np.float32), N_IN, N_OUT)
        po, m, v = MO.adam(p, g, m, v, step, lr)
        net.train(x, t, epochs=1, batch=128, lr=lr, seed=step)
        err = np.abs(net.get_params() - po)
        # Adam normalises by |g|: where the gradient is at rounding level its
        # sign, and so the step, is not defined to better than lr
        big = np.abs(g) > 1e-4 * np.abs(g).max()
        assert np.max(err[big]) <= 2e-6
        assert np.max(err) <= 2.5 * lr
    net.close()


@pytest.mark.gpu
def test_mlp_training_converges(ctx):
    from grtm_cuda_gb300.learned import Mlp
    net = Mlp(ctx, seed=2)
    x, t = _data(4096, 4)
    l0, _ = net.loss_grad(x, t)
    net.train(x, t, epochs=60, batch=128, lr=2e-3)
    l1, _ = net.loss_grad(x, t)
    assert l1 < 0.05 * l0
    net.close()


def _small_job():
    import grtm_cuda_gb300 as g
    from grtm_cuda_gb300 import synth
    m = synth.crust(np.random.default_rng(5), 12, 8.0)
    opts = g.make_opts(0.1, 10, sigma_factor=math.pi, k_mode=g.K_FIXED, nk_fixed=4096)
    return m, g.make_model(**m), opts


@pytest.mark.gpu
def test_sweep_properties(ctx):
    import grtm_cuda_gb300 as g
    m, model, opts = _small_job()
    gr = g.grid(model, opts)
    fi = np.array([1, 7, 40, 150, 400])
    br = np.array([2.0, 30.0, 300.0])
    s4 = g.sweep_kmax(model, opts, fi, br, 1e-4, ctx=ctx, env=True, alias=True)
    k4, k6 = s4["kmax"], g.sweep_kmax(model, opts, fi, br, 1e-6, ctx=ctx)["kmax"]
    top = 4096 * gr["dk"]
    assert np.all(k4 > 0) and np.all(k4 <= top) and np.all(k6 <= top)
    assert np.all(k6 >= k4)                                   # a tighter tolerance never cuts earlier
    # an absolute threshold equal to tol x total gives the same cutoff
    ka = g.sweep_kmax(model, opts, fi, br, 1.0, tol_abs=1e-4 * s4["env"], ctx=ctx)["kmax"]
    assert np.allclose(ka, k4)
    assert np.all(s4["alias"][..., 0] > 0) and np.all(np.isfinite(s4["alias"]))
    # judging the sweep's own cutoff finds a tail within the tolerance
    t1 = g.sweep_kmax(model, opts, fi, br, 1e-4, k_judge=k4, ctx=ctx)["tail"]
    assert np.all(t1 <= 1e-4 + 1e-12)
    t2 = g.sweep_kmax(model, opts, fi, br, 1e-4, k_judge=0.5 * k4, ctx=ctx)["tail"]
    assert np.all(t2 >= t1)


@pytest.mark.gpu
def test_custom_grid_equals_fixed_grid(ctx):
    """K_CUSTOM with every frequency at the fixed grid's size reproduces it."""
    import grtm_cuda_gb300 as g
    m, model, opts = _small_job()
    d = np.array([5.0, 50.0])
    t1, _, _ = g.run(model, opts, d, ctx=ctx)
    nw = g.grid(model, opts)["nw"]
    t2, _, _ = g.run(model, g.make_opts(0.1, 10, sigma_factor=math.pi, nk_custom=np.full(nw, 4096)), d, ctx=ctx)
    assert np.array_equal(t1, t2)


@pytest.mark.gpu
@pytest.mark.parametrize("impl", ["tc", "simt"])
def test_strided_grid_equals_scaled_step(ctx, impl, monkeypatch):
    """k_j = j m dk on a stride-m grid are the points of a unit-stride grid of
    step m dk: both give the same traces (to FP32 rounding of the points)."""
    import grtm_cuda_gb300 as g
    if impl == "simt":
        monkeypatch.setenv("GRT_KSUM", "simt")
    m, model, opts = _small_job()
    gr = g.grid(model, opts)
    nw, dk = gr["nw"], gr["dk"]
    d = np.array([3.0, 40.0, 250.0])
    nk = np.full(nw, 1024, np.int32)
    stride = np.repeat(np.array([1, 2, 4, 2, 8, 1, 2, 4]), 64)[:nw].astype(np.int32)
    # the same points frequency by frequency: one plan per stride value
    s1 = np.zeros((len(d), 20, 2 * nw), dtype=complex)
    for sv in np.unique(stride):
        _, s, _ = g.run(model, g.make_opts(0.1, 10, sigma_factor=math.pi, dk=dk * sv, nk_custom=nk), d, ctx=ctx,
                        spectra=True)
        sel = np.nonzero(stride == sv)[0]
        s1[..., sel] = s[..., sel]
    _, s0, _ = g.run(model, g.make_opts(0.1, 10, sigma_factor=math.pi, dk=dk, nk_custom=nk, k_stride=stride), d,
                     ctx=ctx, spectra=True)
    err = np.abs(s0[..., :nw] - s1[..., :nw]).max() / np.abs(s1[..., :nw]).max()
    assert err <= 2e-6


@pytest.mark.gpu
def test_stride_tile_rule(ctx, monkeypatch):
    """The tensor-core sum needs one stride per aligned tile of 64 frequencies;
    the SIMT sum takes any per-frequency stride."""
    import grtm_cuda_gb300 as g
    m, model, opts = _small_job()
    nw = g.grid(model, opts)["nw"]
    stride = np.ones(nw, np.int32)
    stride[5] = 2
    o = g.make_opts(0.1, 10, sigma_factor=math.pi, nk_custom=np.full(nw, 512), k_stride=stride)
    with pytest.raises(g.GrtError) as e:
        g.run(model, o, [10.0], ctx=ctx)
    assert e.value.status == g.ERR_ARG
    monkeypatch.setenv("GRT_KSUM", "simt")
    t, _, _ = g.run(model, o, [10.0], ctx=ctx)
    assert np.all(np.isfinite(t))


def _learned_case(seed=3007, n_rec=8):
    from grtm_cuda_gb300 import synth
    rng = np.random.default_rng(seed)
    m = synth.crust(rng, 40, rng.uniform(1.0, 30.0))
    return m, np.sort(rng.uniform(1.0, 500.0, n_rec))


@pytest.mark.gpu
def test_learned_batch_judge_overlap(ctx):
    """The batched learned path with its judge run beside the batch's graph (a
    second context on another host thread) gives the traces and verdicts of
    the judge run after it, and reports only the judge time the graph did
    not hide."""
    from grtm_cuda_gb300 import learned
    if not os.path.exists(learned.WEIGHTS):
        pytest.skip("no trained sampler in the tree")
    s = learned.Sampler.load()
    cases = [_learned_case(3007, 6), _learned_case(3011, 5)]
    ms, ds = [m for m, _ in cases], [d for _, d in cases]
    t1, i1 = learned.run_learned_batch(s, ms, ds, ctx=ctx, overlap=False)
    t2, i2 = learned.run_learned_batch(s, ms, ds, ctx=ctx, overlap=True)
    for a, b in zip(t1, t2):
        assert np.array_equal(a, b)
    assert i1["fallback"] == i2["fallback"] and i1["nkw_learned"] == i2["nkw_learned"]
    assert i2["judge_overlapped"] and not i1["judge_overlapped"]
    assert 0.0 <= i2["s_judge"] <= i2["s_judge_parts"]["total"] + 1e-6


@pytest.mark.gpu
def test_learned_stream_matches_batches(ctx):
    """The pipelined stream (batch i+1 predicted, built and judged beside
    batch i's graph; two contexts alternating) gives every batch the traces
    and verdicts of run_learned_batch, with and without page-locked outputs
    written by the graphs."""
    import grtm_cuda_gb300 as g
    from grtm_cuda_gb300 import learned
    if not os.path.exists(learned.WEIGHTS):
        pytest.skip("no trained sampler in the tree")
    s = learned.Sampler.load()
    work = [([m], [d]) for m, d in (_learned_case(3007, 6), _learned_case(3011, 5), _learned_case(3013, 4))]
    ref = [learned.run_learned_batch(s, ms, ds, ctx=ctx, autotune=False) for ms, ds in work]
    c1 = g.Context()
    try:
        n = 0
        for (tr, info), (rt, ri) in zip(learned.run_learned_stream(s, work, (ctx, c1), autotune=False), ref):
            assert np.array_equal(tr[0], rt[0])
            assert info["fallback"] == ri["fallback"] and info["nkw_learned"] == ri["nkw_learned"]
            n += 1
        assert n == len(work)
        # one batch repeated into two alternating sets of page-locked outputs
        ms, ds = work[0]
        gr = g.grid(g.make_model(**ms[0]), learned.plain_opts())
        outs = tuple([g.pinned_empty((len(ds[0]), gr["n_cols"], gr["n_samples"]))] for _ in range(2))
        got = [np.array(tr[0]) for tr, _ in learned.run_learned_stream(s, [work[0]] * 3, (ctx, c1), outs=outs,
                                                                         autotune=False)]
        assert len(got) == 3
        for t in got:
            assert np.array_equal(t, ref[0][0][0])
        assert learned.run_learned_stream(s, [], (ctx, c1)) is not None
        assert list(learned.run_learned_stream(s, [], (ctx, c1))) == []
    finally:
        c1.close()


@pytest.mark.gpu
def test_learned_path_gain_and_accuracy(ctx):
    """On a held-out model the trained sampler evaluates far fewer (w,k)
    points than the plain fixed grid and stays within 1e-3 of FP64."""
    import grtm_cuda_gb300 as g
    from grtm_cuda_gb300 import learned
    if not os.path.exists(learned.WEIGHTS):
        pytest.skip("no trained sampler in the tree")
    s = learned.Sampler.load()
    m, d = _learned_case()
    model = g.make_model(**m)
    t64, _, _ = g.run(model, learned.plain_opts(precision=g.FP64), d, ctx=ctx)
    tl, info = learned.run_learned(s, m, d, ctx=ctx)
    err = np.sqrt(np.sum((tl - t64) ** 2, axis=(1, 2)) / np.sum(t64 ** 2, axis=(1, 2)))
    # per-band k margins: 1.46x fewer points here (1.20x with one margin)
    assert info["nkw_plain"] / info["nkw_learned"] >= 1.35
    assert info["fallback"] == []                      # a sound grid passes its judge
    assert np.sqrt(np.sum((tl - t64) ** 2) / np.sum(t64 ** 2)) <= 1e-3
    assert np.median(err) <= 1e-3


@pytest.mark.gpu
def test_learned_judge_falls_back(ctx):
    """A sampler that cuts the integral far too early is caught by the judge
    and its receivers are recomputed on the plain grid."""
    import grtm_cuda_gb300 as g
    from grtm_cuda_gb300 import learned
    if not os.path.exists(learned.WEIGHTS):
        pytest.skip("no trained sampler in the tree")
    s = learned.Sampler.load()
    s.margin_k, s.kbands = 0.2, None
    m, d = _learned_case(3011, 4)
    tl, info = learned.run_learned(s, m, d, ctx=ctx)
    assert len(info["fallback"]) == len(d)
    tp, _, _ = g.run(g.make_model(**m), learned.plain_opts(), d, ctx=ctx)
    assert np.array_equal(tl, tp)


def test_sampler_network_per_context_without_gpu(monkeypatch):
    """The sampler keeps one network per live context (building one uploads
    the weights, freeing one waits for the whole device) and drops those of
    closed or collected contexts."""
    from grtm_cuda_gb300 import learned
    made, closed = [], []

    class FakeMlp:
        def __init__(self, ctx):
            self.ctx = ctx
            made.append(self)

        def set_params(self, p):
            pass

        def close(self):
            closed.append(self)

    class FakeCtx:
        def __init__(self):
            self.h = 1

    monkeypatch.setattr(learned, "Mlp", FakeMlp)
    s = learned.Sampler(np.zeros(4, np.float32), np.zeros(15), np.ones(15), np.zeros(2), np.ones(2))
    a, b = FakeCtx(), FakeCtx()
    na, nb = s.net(a), s.net(b)
    assert na is not nb and s.net(a) is na and s.net(b) is nb and len(made) == 2
    b.h = 0                                   # b closed: its network goes at the next lookup
    assert s.net(a) is na and closed == [nb]
    del b
    c = FakeCtx()
    assert s.net(c) is not na and len(made) == 3
