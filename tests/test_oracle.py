"""The FP64 CPU oracle pinned against the reference's own known-answer case.

The reference ships one golden case (demo/input.txt -> demo/oname_{w,t}.txt,
a single force at 8.005 km, surface receiver at 10000 km, N = 2048, dt = 2 s).
Its lowest three frequency bins are ill-conditioned in the reference's own
FP64 algorithm (the 4x4 eigenvector solve of green.cu:1810-1818 loses up to
13 digits as w -> 0; compared with an extended-precision run the reference is
off by up to 0.4 of the column peak at iw = 0).  Parity is therefore asserted
bin-wise above that noise floor and, in the time domain, on the de-damped
inverse DFT of the spectral difference with bins iw < 3 masked.
"""
import numpy as np
import pytest

IW_NOISE = 3


@pytest.fixture(scope="module")
def demo_run(oracle, demo_input):
    job = oracle.parse(demo_input)
    oracle.setup(job, job.dt, job.log2n, job.t0, job.taper)
    spec, sig = oracle.run(job, [job.dist0])
    return job, spec[0], sig[0]


def _damp(job):
    n = np.arange(2 * job.nw)
    return np.exp(n * job.dt * job.sigma) * np.exp(job.t0 * job.sigma)


def test_demo_parse_matches_reference_layout(oracle, demo_input):
    job = oracle.parse(demo_input)
    oracle.setup(job, job.dt, job.log2n, job.t0, job.taper)
    assert job.n_layer == 5 and job.inserted == 1
    assert (job.s_layer, job.r_layer) == (0, 0)
    assert job.zr == 0.0 and abs(job.zs - 8.00502696802798) < 1e-12
    assert job.nw == 1024 and job.src_type == 0
    assert abs(job.sigma - 2.0 / 4096.0) < 1e-18


def test_golden_fixture_structure(golden):
    # single force: columns 15-29 zero, Nyquist row zero, rows > N/2 conjugates
    assert golden["tail_max"].max() == 0.0
    assert golden["herm_err"][0] == 0.0 and golden["nyquist_max"][0] == 0.0


def test_golden_time_series_is_dedamped_idft_of_spectrum(oracle, golden, demo_input):
    job = oracle.parse(demo_input)
    oracle.setup(job, job.dt, job.log2n, job.t0, job.taper)
    half = golden["spec"]
    N = 2 * job.nw
    full = np.zeros((N, 15), complex)
    full[: job.nw + 1] = half
    full[job.nw + 1:] = np.conj(half[job.nw - 1:0:-1])
    rec = np.real(np.fft.ifft(full, axis=0)) * _damp(job)[:, None]
    err = np.linalg.norm(rec - golden["sig"]) / np.linalg.norm(golden["sig"])
    assert err < 1e-13


def test_oracle_spectrum_matches_golden_above_noise_floor(demo_run, golden):
    job, spec, _ = demo_run
    g = golden["spec"]
    for c in range(15):
        peak = np.abs(g[: job.nw, c]).max()
        err = np.abs(spec[IW_NOISE: job.nw, c] - g[IW_NOISE: job.nw, c]).max() / peak
        assert err < 5e-5, (c, err)
    assert np.abs(spec[:, 15:]).max() == 0.0
    assert np.abs(spec[job.nw]).max() == 0.0
    assert np.array_equal(spec[job.nw + 1:], np.conj(spec[job.nw - 1:0:-1]))


def test_oracle_time_series_matches_golden_masked(demo_run, golden):
    job, spec, sig = demo_run
    N = 2 * job.nw
    damp = _damp(job)
    g = golden["spec"]
    gfull = np.zeros((N, 15), complex)
    gfull[: job.nw + 1] = g
    gfull[job.nw + 1:] = np.conj(g[job.nw - 1:0:-1])
    for c in range(15):
        d = spec[:, c] - gfull[:, c]
        d[:IW_NOISE] = 0
        d[N - IW_NOISE + 1:] = 0
        t = np.real(np.fft.ifft(d)) * damp
        err = np.linalg.norm(t) / np.linalg.norm(golden["sig"][:, c])
        assert err < 5e-6, (c, err)
    # the unmasked comparison is dominated by the reference's own noise
    full_err = np.linalg.norm(sig[:, :15] - golden["sig"]) / np.linalg.norm(golden["sig"])
    assert full_err < 5e-2


def test_stable_formulation_agrees_with_reference_algorithm(oracle):
    """The well-conditioned basis reproduces the reference's E-matrix
    algorithm wherever the latter is well conditioned (iw >= 20)."""
    tops = [0, 2, 10, 20, 35]
    vp = [3.0, 5.8, 6.5, 7.0, 8.0]
    vs = [v / 1.73 for v in vp]
    rho = [1.74 * v ** 0.25 for v in vp]
    for hs, hr, fix, st in [(10.0005, 0.0, 0, 0), (10.0005, 0.0, 0, 1), (5.0, 3.0, 0, 1),
                            (5.0, 7.0, oracle.FIX_ALL, 0), (5.0, 7.0, oracle.FIX_ALL, 1)]:
        jobs = []
        for extra in (0, oracle.STABLE):
            j = oracle.model(tops, vp, vs, rho, [200] * 5, [100] * 5, hs, hr, st)
            oracle.setup(j, 0.1, 10, 0.0, 0.3, sigma_factor=np.pi, fix=fix | extra)
            jobs.append(j)
        for iw in (20, 100, 400):
            for k in (0.0, 0.05, 0.3, 1.0, 3.0):
                a, b = oracle.point(jobs[0], iw, k), oracle.point(jobs[1], iw, k)
                assert np.abs(a - b).max() <= 1e-10 * np.abs(a).max(), (hs, hr, fix, st, iw, k)


def test_bessel_restatement_against_scipy(oracle):
    sp = pytest.importorskip("scipy.special")
    xs = np.concatenate([np.linspace(0.01, 3.0, 40), np.linspace(3.0, 50.0, 40), [123.4, 5800.7]])
    for n in (0, 1, 2, 3):
        for x in xs:
            assert abs(oracle.besselj(x, n) - sp.jv(n, x)) < 2e-7, (n, x)
    # d/dx J_n: n J_n / x - J_{n+1}
    for x in (0.5, 2.0, 7.5):
        assert abs(oracle.d_besselj(x, 1) - sp.jvp(1, x)) < 1e-6
