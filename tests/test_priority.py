"""Stream priority of a context (grt_set_priority): the learned path's judge
runs on a second context whose streams take the device's greatest priority.
The priority changes only the order in which blocks are scheduled: a plan or
batch on such a context gives the same results as on a default one."""
import math

import numpy as np
import pytest


def _job(g, nk=600):
    from grtm_cuda_gb300 import synth
    rng = np.random.default_rng(5)
    m = synth.crust(rng, 7, 10.0)
    d = np.sort(rng.uniform(5.0, 250.0, 11))
    o = g.make_opts(0.05, 10, sigma_factor=math.pi, k_mode=g.K_FIXED, nk_fixed=nk, precision=g.FP32,
                    fix=g.FIX_ALL)
    return g.make_model(**m), o, d


@pytest.mark.gpu
def test_priority_context_gives_identical_results():
    import grtm_cuda_gb300 as g
    m, o, d = _job(g)
    c0 = g.Context(0)
    c1 = g.Context(0)
    try:
        c1.set_priority(True)
        c1.set_priority(True)          # unchanged: a no-op
        t0, _, _ = g.run(m, o, d, c0)
        t1, _, _ = g.run(m, o, d, c1)
        assert np.array_equal(t0, t1)
        jobs = [(m, o, d), (m, o, d[:5])]
        b0 = g.Batch(c0, jobs, autotune=False)
        b0.execute()
        ref = [b0.fetch(i)[0] for i in range(2)]
        b0.close()
        b = g.Batch(c1, jobs, autotune=False)
        b.execute()
        for i in range(2):
            assert np.array_equal(b.fetch(i)[0], ref[i])
        # a context that holds a batch keeps its streams
        with pytest.raises(g.GrtError) as e:
            c1.set_priority(False)
        assert e.value.status == g.ERR_ARG
        b.close()
        c1.set_priority(False)
        t2, _, _ = g.run(m, o, d, c1)
        assert np.array_equal(t2, t0)
        assert g.lib().grt_device_synchronize(0) == g.OK
    finally:
        c1.close()
        c0.close()


@pytest.mark.gpu
def test_judge_context_has_priority():
    import grtm_cuda_gb300 as g
    from grtm_cuda_gb300 import learned
    c = g.Context(0)
    try:
        j = learned.judge_context(c)
        assert j is learned.judge_context(c)
        m, o, d = _job(g, 300)
        t, _, _ = g.run(m, o, d, j)
        assert np.isfinite(t).all()
        with pytest.raises(g.GrtError):
            p = g.Plan(j, m, o, d)
            try:
                j.set_priority(False)
            finally:
                p.close()
    finally:
        c.close()
