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


SCRATCH = 32 << 20   # the entry point's device array


def _scratch_bytes(g, m, o, nd):
    """Device scratch a job needs: the buffer layout of grt_run_noalloc
    (grt_noalloc.cu), each buffer rounded up to 256 bytes.  FP32 layer rows of
    112 bytes, tiles of 128 wavenumbers, a fixed grid."""
    up = lambda n: (n + 255) & ~255
    gr = g.grid(m, o)
    L, nw, N, nk = gr["n_layer"], gr["nw"], gr["n_samples"], o.nk_fixed
    nq, nc = (10, 15) if m.src_type == 0 else (8, 20)
    ntiles = nw * ((nk + 127) // 128)
    sizes = [nw * L * 112, ntiles * 8, nw * 4, nw * 8, nd * 8, nw * 8, N * 8, N * 4,
             nq * nw * nk * 8, nk * 9 * nd * 4, nd * nc * nw * 8, nd * nc * N * 4, 4]
    return sum(up(x) for x in sizes)


def _edge_jobs(g):
    """Moment-tensor jobs on the 4-layer crust (N = 256, three receivers) whose
    scratch lands just under and just over the array: the largest fixed grid
    that fits, and the next one."""
    d = [12.0, 47.0, 90.0]
    m = g.make_model(TOPS, VP, VS, RHO, QP, QS, 10.0005, 0.0, 1)
    opts = lambda nk: g.make_opts(0.1, 8, 0.0, 0.3, np.pi, g.K_FIXED, nk, precision=g.FP32)
    nk = 1024
    while _scratch_bytes(g, m, opts(nk + 1), len(d)) <= SCRATCH:
        nk += 1
    return m, opts(nk), opts(nk + 1), d


def test_noalloc_jobs_at_the_edge_of_its_scratch():
    """The largest job the array holds (its buffers fill it to within a few
    KB) matches grt_run; one more wavenumber is refused."""
    import grtm_cuda_gb300 as g
    g.lib()
    m, o_in, o_over, d = _edge_jobs(g)
    need = _scratch_bytes(g, m, o_in, len(d))
    assert SCRATCH - 64 * 1024 < need <= SCRATCH, need
    ctx = g.Context()
    ref, _, _ = g.run(m, o_in, d, ctx)
    ctx.close()
    for _ in range(2):
        out = g.run_noalloc(m, o_in, d)
        err = np.linalg.norm(out - ref) / np.linalg.norm(ref)
        assert err <= TOL, err
    assert _scratch_bytes(g, m, o_over, len(d)) > SCRATCH
    with pytest.raises(g.GrtError) as e:
        g.run_noalloc(m, o_over, d)
    assert e.value.status == g.ERR_UNSUPPORTED


def test_noalloc_rejects_jobs_beyond_its_scratch():
    import grtm_cuda_gb300 as g
    m = g.make_model(TOPS, VP, VS, RHO, QP, QS, 10.0005, 0.0, 1)
    o = g.make_opts(0.1, 12, 0.0, 0.3, np.pi, g.K_FIXED, 16384, precision=g.FP32)
    with pytest.raises(g.GrtError) as e:
        g.run_noalloc(m, o, [10.0])
    assert e.value.status == g.ERR_UNSUPPORTED
