"""Seismogram synthesis: the fused combination + source-time convolution +
inverse DFT kernel against its numpy restatement on the same columns, and
the properties every moment-tensor combination must have."""
import math

import numpy as np
import pytest

from oracle import synth_oracle as SO


def test_source_forms_without_gpu():
    """A source is a moment tensor (6 values) or a force (3 values)."""
    import grtm_cuda_gb300 as g
    s = g.make_source([1.0, 2.0, 3.0], stf=np.ones(4))
    assert list(s.f) == [1.0, 2.0, 3.0] and list(s.m) == [0.0] * 6 and s.n_stf == 4
    s = g.make_source(np.arange(6.0))
    assert list(s.m) == list(np.arange(6.0)) and list(s.f) == [0.0] * 3 and s.n_stf == 0
    with pytest.raises(ValueError):
        g.make_source([1.0, 2.0])


def test_dc_moment_known_cases():
    # vertical strike-slip along north: pure Mxy; 45-degree thrust: Mzz = -Myy... traceless
    assert np.allclose(SO.dc_moment(0, 90, 0), [0, 0, 0, 1, 0, 0], atol=1e-12)
    for sdr in [(30, 60, 90), (123, 17, -45), (250, 80, 10)]:
        m = SO.dc_moment(*sdr)
        assert abs(m[0] + m[1] + m[2]) < 1e-12
        M = np.array([[m[0], m[3], m[4]], [m[3], m[1], m[5]], [m[4], m[5], m[2]]])
        ev = np.sort(np.linalg.eigvalsh(M))
        assert np.allclose(ev, [-1, 0, 1], atol=1e-12)       # a double couple of unit moment


def test_combination_rotation_invariance_cpu():
    # rotating the mechanism by d in strike and the receiver by d in azimuth leaves the weights unchanged
    rng = np.random.default_rng(0)
    for _ in range(10):
        s, d, r, phi, dl = rng.uniform(0, 360), rng.uniform(0, 90), rng.uniform(-180, 180), rng.uniform(0, 360), \
            rng.uniform(0, 360)
        w1 = SO.weights(SO.dc_moment(s, d, r), phi)
        w2 = SO.weights(SO.dc_moment(s + dl, d, r), phi + dl)
        assert np.allclose(w1, w2, atol=1e-12)


def test_dc_moment_library_matches_restatement():
    import grtm_cuda_gb300 as g
    for sdr in [(30, 60, 90), (123, 17, -45), (250, 80, 10)]:
        assert np.allclose(g.dc_moment(*sdr), SO.dc_moment(*sdr), atol=1e-14)


@pytest.fixture(scope="module")
def job():
    import grtm_cuda_gb300 as g
    from grtm_cuda_gb300 import synth
    ctx = g.Context()
    m, _ = synth.crust4_model()
    d = np.array([12.0, 40.0, 77.0])
    o = g.make_opts(0.1, 10, sigma_factor=math.pi, k_mode=g.K_FIXED, nk_fixed=2048, fix=g.FIX_ALL)
    p = g.Plan(ctx, g.make_model(**m), o, d)
    p.execute()
    tr, _ = p.fetch()
    yield g, p, tr, o
    p.close()
    ctx.close()


@pytest.mark.gpu
def test_fused_synthesis_matches_restatement(job):
    g, p, tr, o = job
    r = p.report
    m6 = g.dc_moment(30, 60, 90)
    az = np.array([10.0, 130.0, 250.0])
    stf = np.hanning(25)
    for s in (None, stf):
        out = p.synth(m6, az, stf=s)
        ref = SO.synth(tr, m6, az, o.dt, r.sigma, t0=o.t0, stf=s)
        err = np.linalg.norm(out - ref, axis=-1) / np.linalg.norm(ref, axis=-1)
        assert err.max() <= 2e-5


@pytest.mark.gpu
def test_synthesis_linear_and_rotation_invariant(job):
    g, p, tr, o = job
    m1, m2 = g.dc_moment(30, 60, 90), g.dc_moment(200, 35, -60)
    az = np.array([10.0, 130.0, 250.0])
    a = p.synth(m1, az) + 2.0 * p.synth(m2, az)
    b = p.synth(m1 + 2.0 * m2, az)
    assert np.linalg.norm(a - b) <= 1e-5 * np.linalg.norm(b)
    c = p.synth(g.dc_moment(30 + 40, 60, 90), az + 40)
    d = p.synth(m1, az)
    assert np.linalg.norm(c - d) <= 1e-5 * np.linalg.norm(d)


@pytest.mark.gpu
def test_single_force_synthesis(job):
    """A single-force job's seismograms are its displacement columns weighted
    by grt_sf_weights (the spectral stage is linear): fused synthesis equals
    that combination of the fetched traces, and is linear in the force."""
    import ctypes
    g, p, tr, o = job
    from grtm_cuda_gb300 import synth
    m, _ = synth.crust4_model()
    m = dict(m, src_type=0)
    d = np.array([12.0, 40.0, 77.0])
    ps = g.Plan(p.ctx, g.make_model(**m), o, d)
    try:
        ps.execute()
        t, _ = ps.fetch()
        f = np.array([0.3, -1.1, 0.7])
        az = np.array([10.0, 130.0, 250.0])
        out = ps.synth(f, az)
        dp = ctypes.POINTER(ctypes.c_double)
        for r in range(len(d)):
            w = np.zeros(3 * 15)
            g.lib().grt_sf_weights(f.ctypes.data_as(dp), float(az[r]), w.ctypes.data_as(dp))
            ref = w.reshape(3, 15) @ t[r][:15]
            assert np.linalg.norm(out[r] - ref) <= 1e-5 * np.linalg.norm(ref)
        f2 = np.array([-0.5, 0.2, 1.3])
        a = ps.synth(f, az) + 2.0 * ps.synth(f2, az)
        b = ps.synth(f + 2.0 * f2, az)
        assert np.linalg.norm(a - b) <= 1e-5 * np.linalg.norm(b)
        with pytest.raises(ValueError):
            ps.synth([1.0, 2.0], az)
    finally:
        ps.close()


@pytest.mark.gpu
def test_binary_output_roundtrip(job, tmp_path):
    g, p, tr, o = job
    path = tmp_path / "g.bin"
    p.write(path)
    b = g.read_bin(path)
    assert b["traces"].shape == tr.shape and np.array_equal(b["dist"], p.dists)
    assert b["dt"] == o.dt and b["sigma"] == p.report.sigma
    assert np.array_equal(b["traces"], tr.astype(np.float32))
