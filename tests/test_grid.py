"""Host-side job set-up without a GPU: the library's grid (grt_grid) against the
oracle's restatement of the reference's host code (green.cu:1989-2194) --
source-interface insertion, thickness table, source and receiver layers,
frequency step, imaginary frequency, wavenumber step and the ragged
per-frequency k_max rule -- on a matrix of geometries, in both the
bug-compatible and the corrected receiver-layer mode; and the status codes
of the inputs the method cannot take."""
import math

import numpy as np
import pytest

TOPS = [0.0, 2.0, 10.0, 20.0, 35.0]
VP = [3.0, 5.8, 6.5, 7.0, 8.0]
VS = [v / 1.73 for v in VP]
RHO = [1.74 * v ** 0.25 for v in VP]
QP, QS = [200.0] * 5, [100.0] * 5

# (hs, hr, src_type): surface and buried receivers, receiver above / below /
# in the source layer, source on and off an interface, single force and
# moment tensor
GEOMETRIES = [
    (10.0005, 0.0, 1),
    (10.0005, 0.0, 0),
    (1.0, 0.0, 0),
    (5.0, 15.0, 1),
    (15.0, 5.0, 0),
    (12.0, 14.0, 1),
    (0.5, 0.0, 1),
    (30.0, 3.0, 1),
]


def _seeded_crust(seed, n):
    from grtm_cuda_gb300 import synth
    return synth.crust(np.random.default_rng(seed), n, 12.0)


@pytest.mark.parametrize("fix", [0, 1])
@pytest.mark.parametrize("hs,hr,src", GEOMETRIES)
def test_grid_matches_oracle_reference_k_rule(oracle, hs, hr, src, fix):
    import grtm_cuda_gb300 as g
    dt, log2n, sf = 0.1, 9, 2.0
    m = g.make_model(TOPS, VP, VS, RHO, QP, QS, hs, hr, src)
    o = g.make_opts(dt, log2n, 0.0, 0.3, sf, g.K_REFERENCE, 0, fix=fix)
    try:
        rep = g.grid(m, o)
    except g.GrtError as e:
        # the reference's receiver search (quirk F11) can fail to find a layer;
        # the oracle must then refuse the job as well
        job = oracle.model(TOPS, VP, VS, RHO, QP, QS, hs, hr, src)
        with pytest.raises(RuntimeError):
            oracle.setup(job, dt, log2n, 0.0, 0.3, sf, oracle.K_REFERENCE, 0, fix=fix)
        assert e.status == g.ERR_MODEL
        return
    job = oracle.model(TOPS, VP, VS, RHO, QP, QS, hs, hr, src)
    oracle.setup(job, dt, log2n, 0.0, 0.3, sf, oracle.K_REFERENCE, 0, fix=fix)
    assert rep["n_layer"] == job.n_layer
    assert (rep["s_layer"], rep["r_layer"]) == (job.s_layer, job.r_layer)
    assert rep["zs"] == pytest.approx(job.zs, abs=1e-12)
    assert rep["zr"] == pytest.approx(job.zr, abs=1e-12)
    assert rep["nw"] == job.nw and rep["n_samples"] == 2 * job.nw
    assert rep["df"] == pytest.approx(job.df, rel=1e-15)
    assert rep["sigma"] == pytest.approx(job.sigma, rel=1e-15)
    assert rep["dk"] == pytest.approx(job.dk, rel=1e-15)
    nk = oracle.nk_list(job)
    assert rep["n_wk"] == int(nk.sum())
    assert rep["nk_max"] == int(nk.max())
    assert rep["n_cols"] == (15 if src == 0 else 20)


@pytest.mark.parametrize("seed,n", [(1, 3), (2, 20), (3, 40), (4, 60)])
def test_grid_matches_oracle_on_seeded_crusts(oracle, seed, n):
    """Deep stacks: the k_max rule sweeps every layer's slowness."""
    import grtm_cuda_gb300 as g
    mk = _seeded_crust(seed, n)
    m = g.make_model(**mk)
    o = g.make_opts(0.05, 10, 0.0, 0.3, math.pi, g.K_REFERENCE, 0, fix=g.FIX_ALL)
    rep = g.grid(m, o)
    job = oracle.model(mk["ztop"], mk["vp"], mk["vs"], mk["rho"], mk["qp"], mk["qs"], mk["hs"], mk["hr"],
                       mk["src_type"])
    oracle.setup(job, 0.05, 10, 0.0, 0.3, math.pi, oracle.K_REFERENCE, 0, fix=oracle.FIX_ALL)
    nk = oracle.nk_list(job)
    assert rep["n_layer"] == job.n_layer == n + 2      # the source interface is inserted
    assert (rep["s_layer"], rep["r_layer"]) == (job.s_layer, job.r_layer)
    assert rep["n_wk"] == int(nk.sum()) and rep["nk_max"] == int(nk.max())
    assert rep["dk"] == pytest.approx(job.dk, rel=1e-15)


def test_fixed_and_custom_grids(oracle):
    import grtm_cuda_gb300 as g
    m = g.make_model(TOPS, VP, VS, RHO, QP, QS, 10.0005, 0.0, 1)
    rep = g.grid(m, g.make_opts(0.1, 8, 0.0, 0.3, 2.0, g.K_FIXED, 300))
    assert rep["nw"] == 128 and rep["n_wk"] == 128 * 300 and rep["nk_max"] == 300
    nk = np.arange(128, dtype=np.int32) + 2
    rep = g.grid(m, g.make_opts(0.1, 8, 0.0, 0.3, 2.0, g.K_CUSTOM, 0, nk_custom=nk))
    assert rep["n_wk"] == int(nk.sum()) and rep["nk_max"] == int(nk.max())
    # a dk override applies to every mode
    rep = g.grid(m, g.make_opts(0.1, 8, 0.0, 0.3, 2.0, g.K_FIXED, 300, dk=0.01))
    assert rep["dk"] == 0.01


def _status(fn):
    import grtm_cuda_gb300 as g
    with pytest.raises(g.GrtError) as e:
        fn()
    return e.value.status


def test_models_the_method_cannot_take():
    import grtm_cuda_gb300 as g
    o = g.make_opts(0.1, 8, 0.0, 0.3, 2.0, g.K_FIXED, 64)

    def grid_of(tops=TOPS, vp=VP, vs=VS, rho=RHO, qp=QP, qs=QS, hs=10.0005, hr=0.0):
        return lambda: g.grid(g.make_model(tops, vp, vs, rho, qp, qs, hs, hr, 1), o)

    assert _status(grid_of(tops=[0.0], vp=[6.0], vs=[3.5], rho=[2.7], qp=[200.0], qs=[100.0], hs=1.0)) \
        == g.ERR_MODEL                                            # no half-space under a layer
    assert _status(grid_of(tops=[0.0, 2.0, 2.0, 20.0, 35.0])) == g.ERR_MODEL   # tops not increasing
    assert _status(grid_of(vs=[3.0] + VS[1:])) == g.ERR_MODEL    # vs = vp
    assert _status(grid_of(rho=[0.0] + RHO[1:])) == g.ERR_MODEL  # rho = 0
    assert _status(grid_of(qs=[-1.0] + QS[1:])) == g.ERR_MODEL   # Q < 0
    assert _status(grid_of(vp=[float("nan")] + VP[1:])) == g.ERR_MODEL
    assert _status(grid_of(hs=50.0)) == g.ERR_MODEL              # source in the half-space
    assert _status(grid_of(hr=-1.0)) == g.ERR_MODEL              # negative depth
    assert _status(grid_of(hs=-1.0)) == g.ERR_MODEL


def test_options_out_of_range():
    import grtm_cuda_gb300 as g
    m = g.make_model(TOPS, VP, VS, RHO, QP, QS, 10.0005, 0.0, 1)

    def grid_with(**kw):
        base = dict(dt=0.1, log2n=8, t0=0.0, taper=0.3, sigma_factor=2.0, k_mode=g.K_FIXED, nk_fixed=64)
        base.update(kw)
        return lambda: g.grid(m, g.make_opts(**base))

    for kw in (dict(dt=0.0), dict(dt=-0.1), dict(dt=float("nan")), dict(log2n=1), dict(log2n=16),
               dict(taper=1.5), dict(taper=-0.1), dict(sigma_factor=0.0), dict(k_mode=3),
               dict(nk_fixed=1), dict(nk_fixed=(1 << 24) + 2), dict(k_mode=g.K_CUSTOM)):
        assert _status(grid_with(**kw)) == g.ERR_ARG, kw
    bad_nk = np.full(128, 1, dtype=np.int32)
    assert _status(grid_with(k_mode=g.K_CUSTOM, nk_custom=bad_nk)) == g.ERR_ARG
    nk = np.full(128, 100, dtype=np.int32)
    for stride in (0, 65):
        st = np.full(128, stride, dtype=np.int32)
        assert _status(grid_with(k_mode=g.K_CUSTOM, nk_custom=nk, k_stride=st)) == g.ERR_ARG
    # a stride without a custom grid
    assert _status(grid_with(k_stride=np.ones(128, dtype=np.int32))) == g.ERR_ARG


def test_grid_matches_oracle_on_random_jobs(oracle):
    """200 seeded random jobs (2-60 layers, any source / receiver depth above the
    half-space, 2^6-2^13 samples, dt 0.01-0.5 s, both receiver-layer rules):
    the library's set-up and the oracle agree on every layer index, depth and
    step and on each frequency's wavenumber count (their sum and maximum)."""
    import grtm_cuda_gb300 as g
    from grtm_cuda_gb300 import synth
    rng = np.random.default_rng(77)
    checked = 0
    for _ in range(200):
        n = int(rng.integers(1, 60))
        mk = synth.crust(rng, n, 1.0)
        depth = float(mk["ztop"][-1])
        hs = float(rng.uniform(0.05, depth - 0.3))
        hr = float(rng.choice([0.0, rng.uniform(0.0, depth - 0.3)]))
        src = int(rng.integers(0, 2))
        dt, log2n = float(rng.uniform(0.01, 0.5)), int(rng.integers(6, 14))
        fix = int(rng.integers(0, 2))
        m = g.make_model(mk["ztop"], mk["vp"], mk["vs"], mk["rho"], mk["qp"], mk["qs"], hs, hr, src)
        o = g.make_opts(dt, log2n, 0.0, 0.3, 2.0, g.K_REFERENCE, 0, fix=fix)
        job = oracle.model(mk["ztop"], mk["vp"], mk["vs"], mk["rho"], mk["qp"], mk["qs"], hs, hr, src)
        try:
            rep = g.grid(m, o)
        except g.GrtError as e:
            # the reference's receiver search (fix 0) can leave the receiver
            # without a layer; the oracle refuses the same jobs
            with pytest.raises(RuntimeError):
                oracle.setup(job, dt, log2n, 0.0, 0.3, 2.0, oracle.K_REFERENCE, 0, fix=fix)
            assert e.status == g.ERR_MODEL and fix == 0
            continue
        oracle.setup(job, dt, log2n, 0.0, 0.3, 2.0, oracle.K_REFERENCE, 0, fix=fix)
        nk = oracle.nk_list(job)
        assert (rep["n_layer"], rep["s_layer"], rep["r_layer"]) == (job.n_layer, job.s_layer, job.r_layer)
        assert rep["zs"] == pytest.approx(job.zs, abs=1e-9) and rep["zr"] == pytest.approx(job.zr, abs=1e-9)
        assert rep["dk"] == pytest.approx(job.dk, rel=1e-14) and rep["sigma"] == pytest.approx(job.sigma, rel=1e-14)
        assert rep["n_wk"] == int(nk.sum()) and rep["nk_max"] == int(nk.max())
        checked += 1
    assert checked >= 150
