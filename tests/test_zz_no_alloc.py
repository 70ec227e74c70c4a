"""grt_run_noalloc: the entry point for callers that cannot allocate device
memory (their GPU memory is reserved by another runtime, or cudaMalloc is not
permitted where they run).  Called through the C ABI twice in a row, each
call's traces must equal grt_run's for the same job within the FP32 parity
tolerance, and the calls must not change the free device memory.  This file
is collected last on purpose."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOPS = [0.0, 2.0, 10.0, 20.0, 35.0]
VP = [3.0, 5.8, 6.5, 7.0, 8.0]
VS = [v / 1.73 for v in VP]
RHO = [1.74 * v ** 0.25 for v in VP]
QP, QS = [200.0] * 5, [100.0] * 5
TOL = 5e-5   # FP32 tolerance used by the parity tests


def _free_bytes():
    torch = pytest.importorskip("torch")
    free, _ = torch.cuda.mem_get_info(0)
    return free


def _job(g, src_type, hs):
    m = g.make_model(TOPS, VP, VS, RHO, QP, QS, hs, 0.0, src_type)
    o = g.make_opts(0.1, 8, 0.0, 0.3, np.pi, g.K_FIXED, 1024, precision=g.FP32)
    return m, o


def test_noalloc_matches_grt_run_two_calls():
    import grtm_cuda_gb300 as g
    g.lib()
    jobs = [(_job(g, 1, 10.0005), [12.0, 47.0, 90.0]), (_job(g, 0, 5.0), [8.0, 33.0])]
    refs = []
    ctx = g.Context()
    for (m, o), d in jobs:
        t, _, _ = g.run(m, o, d, ctx)
        refs.append(t)
    ctx.close()
    # two calls in a row (moment tensor, then single force), each checked
    for call, ((m, o), d) in enumerate(jobs):
        out = g.run_noalloc(m, o, d)
        ref = refs[call]
        assert out.shape == ref.shape
        err = np.linalg.norm(out - ref) / np.linalg.norm(ref)
        assert err <= TOL, (call, err)
    # the same two calls again, now that set-up and kernel loading are done:
    # the free device memory must not move
    free_before = _free_bytes()
    for call, ((m, o), d) in enumerate(jobs):
        out = g.run_noalloc(m, o, d)
        err = np.linalg.norm(out - refs[call]) / np.linalg.norm(refs[call])
        assert err <= TOL, (call, err)
    assert _free_bytes() == free_before


def test_noalloc_rejects_jobs_beyond_its_scratch():
    import grtm_cuda_gb300 as g
    m = g.make_model(TOPS, VP, VS, RHO, QP, QS, 10.0005, 0.0, 1)
    o = g.make_opts(0.1, 12, 0.0, 0.3, np.pi, g.K_FIXED, 16384, precision=g.FP32)
    with pytest.raises(g.GrtError) as e:
        g.run_noalloc(m, o, [10.0])
    assert e.value.status == g.ERR_UNSUPPORTED
