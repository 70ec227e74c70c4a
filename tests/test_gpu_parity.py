"""Parity of the CUDA path with the FP64 oracle and the reference's golden case.

Tolerances (relative L2 over each output column's time series):
  FP64 GPU vs FP64 oracle (same method)         1e-10
  FP32 GPU vs FP64 oracle, regional distances   5e-5
  FP32 GPU vs FP64 oracle, the 10000 km demo    5e-4  (its k-sum cancels by ~1e3)
  judged FP32 (run_judged, tol 1e-4), the demo  1e-4
  vs the reference's golden demo output: above its own noise floor (bins
  iw >= 3; see test_oracle.py), 5e-6 masked time-domain for FP64.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

TOPS = [0.0, 2.0, 10.0, 20.0, 35.0]
VP = [3.0, 5.8, 6.5, 7.0, 8.0]
VS = [v / 1.73 for v in VP]
RHO = [1.74 * v ** 0.25 for v in VP]
QP, QS = [200.0] * 5, [100.0] * 5


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.fixture(scope="module")
def g():
    import grtm_cuda_gb300 as g
    g.lib()
    return g


@pytest.fixture(scope="module")
def ctx(g):
    c = g.Context()
    yield c
    c.close()


def _oracle_traces(oracle, hs, hr, st, fix, kw, dists):
    job = oracle.model(TOPS, VP, VS, RHO, QP, QS, hs, hr, st)
    oracle.setup(job, kw["dt"], kw["log2n"], kw["t0"], kw["taper"], kw["sigma_factor"], kw["k_mode"],
                 kw["nk_fixed"], fix=fix | oracle.STABLE)
    _, sig = oracle.run(job, dists, want_spec=False)
    nc = 15 if st == 0 else 20
    return np.transpose(sig[:, :, :nc], (0, 2, 1)), job


GEOMETRIES = [
    # (hs, hr, src_type, fix): receiver above / in / below the source layer
    (10.0005, 0.0, 1, 0),    # r < s, moment tensor (4-layer crust geometry)
    (10.0005, 0.0, 0, 0),    # r < s, single force
    (5.0, 3.0, 1, 0),        # same layer, receiver above the source
    (5.0, 4.0, 0, 7),        # same layer, receiver below the source
    (5.0, 7.0, 0, 7),        # r > s
    (5.0, 40.0, 1, 7),       # receiver in the half-space
]


@pytest.mark.parametrize("hs,hr,st,fix", GEOMETRIES)
def test_geometries_fp64_and_fp32(g, ctx, oracle, hs, hr, st, fix):
    kw = dict(dt=0.1, log2n=8, t0=0.0, taper=0.3, sigma_factor=np.pi, k_mode=g.K_FIXED, nk_fixed=1024)
    dists = [10.0, 35.0, 80.0]
    ref, job = _oracle_traces(oracle, hs, hr, st, fix, kw, dists)
    m = g.make_model(TOPS, VP, VS, RHO, QP, QS, hs, hr, st)
    t64, _, rep = g.run(m, g.make_opts(precision=g.FP64, fix=fix, **kw), dists, ctx)
    assert (rep["s_layer"], rep["r_layer"]) == (job.s_layer, job.r_layer)
    assert rep["n_wk"] == 128 * 1024 and rep["kernel_launches"] == 4
    for c in range(ref.shape[1]):
        assert rel(t64[:, c], ref[:, c]) < 1e-10, c
    t32, _, _ = g.run(m, g.make_opts(precision=g.FP32, fix=fix, **kw), dists, ctx)
    for c in range(ref.shape[1]):
        assert rel(t32[:, c], ref[:, c]) < 5e-5, c


# moment-tensor columns holding an SH term in the reference layout: b2 in
# 0, 4, 5 (5 reads b2 for b1) and their d/dr 10, 14, 15; b1 in 1 and 11
SH_B1_COLS, SH_B2_COLS = (1, 11), (0, 4, 5, 10, 14, 15)


@pytest.mark.parametrize("hs,hr", [(10.0005, 0.0), (14.0, 12.0), (5.0, 15.0), (12.0, 14.0)])
def test_sh_source_fix(g, ctx, oracle, hs, hr):
    """GRT_FIX_SHSRC on moment-tensor jobs, receiver above the source (surface,
    same layer) and below it (other layer, same layer): FP64 GPU equals the
    oracle, FP32 within the regional tolerance (whole job); against the run without the
    bit only the SH columns of the receiver's side move (b1 above, b2 below)."""
    kw = dict(dt=0.1, log2n=8, t0=0.0, taper=0.3, sigma_factor=np.pi, k_mode=g.K_FIXED, nk_fixed=1024)
    dists = [10.0, 35.0, 80.0]
    ref, job = _oracle_traces(oracle, hs, hr, 1, oracle.FIX_ALL | oracle.FIX_SHSRC, kw, dists)
    m = g.make_model(TOPS, VP, VS, RHO, QP, QS, hs, hr, 1)
    t64, _, rep = g.run(m, g.make_opts(precision=g.FP64, fix=g.FIX_ALL | g.FIX_SHSRC, **kw), dists, ctx)
    assert (rep["s_layer"], rep["r_layer"]) == (job.s_layer, job.r_layer)
    for c in range(20):
        assert rel(t64[:, c], ref[:, c]) < 1e-10, c
    t32, _, _ = g.run(m, g.make_opts(precision=g.FP32, fix=g.FIX_ALL | g.FIX_SHSRC, **kw), dists, ctx)
    assert rel(t32, ref) < 5e-5
    plain, _, _ = g.run(m, g.make_opts(precision=g.FP64, fix=g.FIX_ALL, **kw), dists, ctx)
    moved = SH_B1_COLS if hr < hs else SH_B2_COLS
    for c in range(20):
        if c in moved:
            assert rel(t64[:, c], plain[:, c]) > 1e-3, c
        else:
            assert rel(t64[:, c], plain[:, c]) < 1e-13, c


def test_crust4_double_couple_full_size(g, ctx, oracle):
    """4-layer crust, full grid: 10 receivers 10-100 km, nt 1024, dt 0.1, nk 4096,
    sigma = pi/T; the source is moved 0.5 m off the 10 km interface."""
    kw = dict(dt=0.1, log2n=10, t0=0.0, taper=0.3, sigma_factor=np.pi, k_mode=g.K_FIXED, nk_fixed=4096)
    dists = np.arange(10.0, 101.0, 10.0)
    ref, _ = _oracle_traces(oracle, 10.0005, 0.0, 1, 0, kw, dists)
    m = g.make_model(TOPS, VP, VS, RHO, QP, QS, 10.0005, 0.0, 1)
    t32, _, rep = g.run(m, g.make_opts(precision=g.FP32, **kw), dists, ctx)
    assert t32.shape == (10, 20, 1024)
    worst = max(rel(t32[:, c], ref[:, c]) for c in range(20))
    assert worst < 5e-5, worst


def _demo_model(g):
    toks = open(os.path.join(GOLDEN, "demo_input.txt")).read().split()
    n = int(toks[2])
    A = np.array([list(map(float, toks[3 + i].split(","))) for i in range(n)])
    rest = toks[3 + n:]
    dt, dist, log2n, t0, taper, st = float(rest[0]), float(rest[1]), int(rest[5]), float(rest[6]), float(rest[7]), int(rest[9])
    m = g.make_model(A[:, 0], A[:, 1], A[:, 2], A[:, 3], A[:, 4], A[:, 5], float(toks[0]), float(toks[1]), st)
    return m, dict(dt=dt, log2n=log2n, t0=t0, taper=taper, sigma_factor=2.0, k_mode=g.K_REFERENCE), dist


@pytest.fixture(scope="module")
def demo_oracle(oracle):
    job = oracle.parse(os.path.join(GOLDEN, "demo_input.txt"))
    oracle.setup(job, job.dt, job.log2n, job.t0, job.taper, fix=oracle.STABLE)
    _, sig = oracle.run(job, [job.dist0], want_spec=False)
    return job, sig[0]


def _masked_time_err(spec_gpu, gold_half, gold_sig, job, c, iw_noise=3):
    N = 2 * job.nw
    full = np.zeros(N, complex)
    full[: job.nw + 1] = gold_half[:, c]
    full[job.nw + 1:] = np.conj(gold_half[job.nw - 1:0:-1, c])
    d = spec_gpu - full
    d[:iw_noise] = 0
    d[N - iw_noise + 1:] = 0
    damp = np.exp(np.arange(N) * job.dt * job.sigma) * np.exp(job.t0 * job.sigma)
    return np.linalg.norm(np.real(np.fft.ifft(d)) * damp) / np.linalg.norm(gold_sig[:, c])


def test_demo_fp64_matches_oracle_and_golden(g, ctx, demo_oracle, golden):
    job, osig = demo_oracle
    m, kw, dist = _demo_model(g)
    tr, sp, rep = g.run(m, g.make_opts(precision=g.FP64, **kw), [dist], ctx, spectra=True)
    assert rep["n_wk"] == 8567889 and (rep["s_layer"], rep["r_layer"]) == (0, 0)
    for c in range(15):
        assert rel(tr[0, c], osig[:, c]) < 1e-10, c
        assert _masked_time_err(sp[0, c], golden["spec"], golden["sig"], job, c) < 5e-6, c


def test_demo_fp32_matches_oracle(g, ctx, demo_oracle):
    job, osig = demo_oracle
    m, kw, dist = _demo_model(g)
    tr, _, _ = g.run(m, g.make_opts(precision=g.FP32, **kw), [dist], ctx)
    for c in range(15):
        assert rel(tr[0, c], osig[:, c]) < 5e-4, c


def test_demo_judged_within_1e_4(g, ctx, demo_oracle):
    """The plain FP32 path misses 1e-4 on the 10 000 km demo (its k-sum
    cancels by ~1e3); the judged run at tolerance 1e-4 (error estimate, FP64
    for the receivers it flags) meets it against the oracle."""
    job, osig = demo_oracle
    m, kw, dist = _demo_model(g)
    tr, info = g.run_judged(m, g.make_opts(precision=g.FP32, **kw), [dist], ctx, tol=1e-4)
    for c in range(15):
        assert rel(tr[0, c], osig[:, c]) < 1e-4, c
    # the estimate is consistent with what it decided
    assert (len(info["fp64"]) > 0) == bool(g.JUDGE_SAFETY * info["est"][0] > 1e-4)


def test_green_file_interface(g, tmp_path, golden, demo_oracle):
    """The reference's entry point through the C ABI: same files, same layout."""
    job, _ = demo_oracle
    ow, ot = str(tmp_path / "w.txt"), str(tmp_path / "t.txt")
    os.environ["GRT_PRECISION"] = "fp64"
    try:
        g.green(os.path.join(GOLDEN, "demo_input.txt"), ow, ot)
    finally:
        del os.environ["GRT_PRECISION"]
    w = g.read_table(ow, complex_pairs=True)
    t = g.read_table(ot)
    assert w.shape == (2048, 30) and t.shape == (2048, 30)
    assert np.abs(w[:, 15:]).max() == 0 and np.abs(t[:, 15:]).max() == 0
    assert np.abs(w[job.nw]).max() == 0
    assert np.array_equal(w[job.nw + 1:], np.conj(w[job.nw - 1:0:-1]))
    for c in range(15):
        assert _masked_time_err(w[:, c], golden["spec"], golden["sig"], job, c) < 5e-6, c


def test_green_reports_bad_input(g, tmp_path):
    bad = tmp_path / "bad.txt"
    bad.write_text("8.0\n0.0\n3\n0,6,3.5\n")
    rc = g.lib().grt_green(str(bad).encode(), str(tmp_path / "w").encode(), str(tmp_path / "t").encode())
    assert rc == g.ERR_PARSE
    rc = g.lib().grt_green(str(tmp_path / "missing").encode(), b"w", b"t")
    assert rc == g.ERR_IO


@pytest.mark.parametrize("impl", ["tc", "simt"])
def test_reference_k_rule_grid(g, ctx, oracle, impl, monkeypatch):
    """Ragged per-frequency k_max grid (the reference's rule) on the 4-layer crust
    model: same (w,k) count as the oracle and the same traces, with the
    tensor-core sum and with the blocked SIMT sum (ragged k counts, 256
    frequencies, 11 receivers: partial frequency and receiver tiles)."""
    if impl == "simt":
        monkeypatch.setenv("GRT_KSUM", "simt")
    kw = dict(dt=0.1, log2n=9, t0=0.0, taper=0.3, sigma_factor=2.0, k_mode=g.K_REFERENCE, nk_fixed=0)
    dists = [15.0, 60.0, 3.0, 7.5, 22.0, 31.0, 44.0, 71.0, 90.0, 120.0, 150.0]
    ref, job = _oracle_traces(oracle, 10.0005, 0.0, 1, 0, kw, dists)
    m = g.make_model(TOPS, VP, VS, RHO, QP, QS, 10.0005, 0.0, 1)
    t32, _, rep = g.run(m, g.make_opts(precision=g.FP32, **kw), dists, ctx)
    assert rep["n_wk"] == int(oracle.nk_list(job).sum())
    assert rep["ksum_impl"] == (1 if impl == "tc" else 2)   # unit strides: the plain sum runs as SGEMMs
    for c in range(20):
        assert rel(t32[:, c], ref[:, c]) < 5e-5, c
