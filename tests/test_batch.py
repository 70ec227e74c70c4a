"""Batches of uneven jobs in one graph: the batched persistent GRT launch
and the per-job stages must give exactly what the jobs give one by one."""
import math

import numpy as np
import pytest


def _jobs(g, precision):
    from grtm_cuda_gb300 import synth
    out = []
    for seed, nl, log2n, nr in ((11, 3, 9, 5), (12, 17, 10, 23), (13, 41, 9, 2)):
        rng = np.random.default_rng(seed)
        m = synth.crust(rng, nl, rng.uniform(1.0, 30.0))
        d = np.sort(rng.uniform(5.0, 400.0, nr))
        o = g.make_opts(0.05, log2n, sigma_factor=math.pi, k_mode=g.K_FIXED, nk_fixed=600 + 37 * seed,
                        precision=precision, fix=g.FIX_ALL)
        out.append((g.make_model(**m), o, d))
    return out


@pytest.fixture(scope="module")
def ctx():
    import grtm_cuda_gb300 as g
    c = g.Context()
    yield c
    c.close()


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp32", "fp64"])
def test_batch_equals_single_jobs(ctx, prec):
    import grtm_cuda_gb300 as g
    jobs = _jobs(g, g.FP32 if prec == "fp32" else g.FP64)
    g.lib().grt_tune_clear()                           # the choices are kept per device for the process
    b = g.Batch(ctx, jobs, autotune=(prec == "fp32"))
    rep = b.execute()
    assert rep.n_wk == sum(g.grid(m, o)["n_wk"] for m, o, _ in jobs)
    first = [b.fetch(j)[0] for j in range(len(jobs))]
    for j in range(len(jobs)):
        assert np.array_equal(b.fetch_f32(j), first[j].astype(np.float32))
    b.execute()                                        # the graph replays
    for j, (m, o, d) in enumerate(jobs):
        # the single job with the batch's (tuned) tensor-core k split adds in the same order
        oj = g.with_precision(o, o.precision)
        oj.k_slice = b.info(j)[0]["k_slice"]
        t1, _, _ = g.run(m, oj, d, ctx=ctx)
        t2 = b.fetch(j)[0]
        assert np.array_equal(t2, first[j])
        assert np.array_equal(t1, t2)
    _, tune = b.info()
    if prec == "fp32":
        assert tune["tuned"] == 1 and len(tune["candidates"]) >= 3
        assert (tune["grt_threads"], tune["grt_blocks"]) in [(c[0], c[1]) for c in tune["candidates"]]
        assert 0 <= tune["grt_shape"] <= 4
        # the tensor-core k split was timed too, and the largest job runs the fastest candidate
        assert tune["tc_tuned"] == 1 and len(tune["tc_candidates"]) >= 2
        best = min(tune["tc_candidates"], key=lambda c: c[1])
        assert tune["tc_nsplit"] == best[0]
        # a second batch of the same kind, on another context of this device, reuses the shape
        c2 = g.Context()
        b2 = g.Batch(c2, jobs, autotune=True)
        _, t2 = b2.info()
        assert t2["tuned"] == 2 and (t2["grt_threads"], t2["grt_blocks"]) == (tune["grt_threads"], tune["grt_blocks"])
        assert t2["tc_tuned"] == 2 and t2["tc_nsplit"] == tune["tc_nsplit"]
        b2.execute()
        assert np.array_equal(b2.fetch(0)[0], first[0])
        b2.close()
        c2.close()
    b.close()


@pytest.mark.gpu
def test_batch_rejects_mixed_precision(ctx):
    import grtm_cuda_gb300 as g
    jobs = _jobs(g, g.FP32)
    m, o, d = jobs[1]
    o64 = g.make_opts(0.05, 10, sigma_factor=math.pi, k_mode=g.K_FIXED, nk_fixed=512, precision=g.FP64)
    with pytest.raises(g.GrtError) as e:
        g.Batch(ctx, [jobs[0], (m, o64, d)])
    assert e.value.status == g.ERR_ARG


@pytest.mark.gpu
def test_pinned_fetch_and_cached_memory(ctx):
    """Fetches into page-locked arrays equal ordinary ones; batches rebuilt on
    the context's cached memory, and after returning it to the driver, give
    the same traces."""
    import grtm_cuda_gb300 as g
    jobs = _jobs(g, g.FP32)
    b = g.Batch(ctx, jobs, autotune=False)
    b.execute()
    ref = [b.fetch_f32(j) for j in range(len(jobs))]
    outs = [g.pinned_empty(r.shape) for r in ref]
    for j, o in enumerate(outs):
        assert b.fetch_f32(j, out=o) is o
        assert np.array_equal(o, ref[j])
    with pytest.raises(ValueError):
        b.fetch_f32(0, out=np.empty(ref[0].shape, np.float64))
    b.close()
    for trim in (False, True):
        if trim:
            ctx.trim()
        b = g.Batch(ctx, jobs, autotune=False)
        b.execute()
        for j in range(len(jobs)):
            assert np.array_equal(b.fetch_f32(j), ref[j])
        b.close()


@pytest.mark.gpu
def test_async_fetch_matches(ctx):
    """Downloads started by fetch_f32_async equal synchronous ones after wait();
    the next execute waits for them."""
    import grtm_cuda_gb300 as g
    jobs = _jobs(g, g.FP32)
    b = g.Batch(ctx, jobs, autotune=False)
    b.execute()
    ref = [b.fetch_f32(j) for j in range(len(jobs))]
    outs = [g.pinned_empty(r.shape) for r in ref]
    for j, o in enumerate(outs):
        b.fetch_f32_async(j, o)
    b.execute()                      # waits for the downloads, then recomputes the same
    b.wait()
    for j, o in enumerate(outs):
        assert np.array_equal(o, ref[j])
    b.close()
    jobs64 = _jobs(g, g.FP64)
    b = g.Batch(ctx, jobs64, autotune=False)
    b.execute()
    with pytest.raises(g.GrtError) as e:
        b.fetch_f32_async(0, g.pinned_empty(b.fetch_f32(0).shape))
    assert e.value.status == g.ERR_UNSUPPORTED
    b.close()


@pytest.mark.gpu
def test_in_graph_downloads(ctx):
    """A batch given page-locked destinations downloads every job's traces
    inside its graph: after execute they equal the fetched ones, and the
    device time still covers the stages only."""
    import grtm_cuda_gb300 as g
    jobs = _jobs(g, g.FP32)
    b = g.Batch(ctx, jobs, autotune=False)
    b.execute()
    ref = [b.fetch_f32(j) for j in range(len(jobs))]
    b.close()
    outs = [g.pinned_empty(r.shape) for r in ref]
    outs[1] = None                                   # a job without a destination
    b = g.Batch(ctx, jobs, autotune=False, outs=outs)
    for _ in range(2):
        for o in outs:
            if o is not None:
                o[...] = -1.0
        b.execute()
        for j, o in enumerate(outs):
            if o is not None:
                assert np.array_equal(o, ref[j])
        assert np.array_equal(b.fetch_f32(1), ref[1])
    b.close()


@pytest.mark.gpu
def test_batch_execute_in_steps(ctx):
    """grt_batch_launch / grt_batch_wait_stages / grt_batch_finish give the
    traces and device time of grt_batch_execute (the last job's download
    drains between the last two steps); out of order they are refused."""
    import grtm_cuda_gb300 as g
    jobs = _jobs(g, g.FP32)
    b = g.Batch(ctx, jobs, autotune=False)
    b.execute()
    ref = [b.fetch_f32(j) for j in range(len(jobs))]
    b.close()
    outs = [g.pinned_empty(r.shape) for r in ref]
    b = g.Batch(ctx, jobs, autotune=False, outs=outs)
    try:
        for o in outs:
            o[...] = -1.0
        with pytest.raises(g.GrtError) as e:
            b.wait_stages()
        assert e.value.status == g.ERR_ARG
        b.launch()
        with pytest.raises(g.GrtError):
            b.finish()
        b.wait_stages()
        r = b.finish()
        assert r.ms_total > 0 and r.ms_grt > 0
        for j, o in enumerate(outs):
            assert np.array_equal(o, ref[j])
        for o in outs:
            o[...] = -1.0
        b.execute()                                  # the one-call form after the steps
        for j, o in enumerate(outs):
            assert np.array_equal(o, ref[j])
    finally:
        b.close()


@pytest.mark.gpu
def test_mixed_batch_runs_each_form(ctx):
    """A batch whose jobs do not all allow the specialised (two-pass) GRT form:
    those that do run it, the others (a receiver below the source's layer, a
    single force) the generic one, in separate launches over their own tiles;
    every job equals its single run bitwise."""
    import grtm_cuda_gb300 as g
    from grtm_cuda_gb300 import synth
    jobs = []
    for seed, nl, hs, hr, src in ((21, 9, 12.0, 0.0, 1), (22, 12, 3.0, 14.0, 1), (23, 7, 8.0, 0.0, 0),
                                  (24, 15, 20.0, 0.0, 1)):
        rng = np.random.default_rng(seed)
        m = dict(synth.crust(rng, nl, hs, src_type=src), hr=hr)
        d = np.sort(rng.uniform(5.0, 150.0, 4))
        o = g.make_opts(0.05, 9, sigma_factor=math.pi, k_mode=g.K_FIXED, nk_fixed=700 + 13 * seed,
                        precision=g.FP32, fix=g.FIX_ALL)
        jobs.append((g.make_model(**m), o, d))
    b = g.Batch(ctx, jobs, autotune=True)
    b.execute()
    for j, (m, o, d) in enumerate(jobs):
        oj = g.with_precision(o, o.precision)
        oj.k_slice = b.info(j)[0]["k_slice"]
        t1, _, _ = g.run(m, oj, d, ctx=ctx)
        assert np.array_equal(b.fetch(j)[0], t1), j
    b.close()
