"""Parity with the oracle at the benchmark configurations' sizes (GB300).

The other GPU parity tests run small grids.  These run spectra-only plans
(opts.freq_sel: the selected frequencies of the full job, each with its full
wavenumber grid) on the two large configurations and compare every
receiver's spectra with the FP64 oracle's k-sums at the same frequencies
(grto_run_band; the reference's k-sum, green.cu:1878-1903, with the integrand
columns of green.cu:1558-1716, at each receiver distance):
  * a seeded 20-layer crust, 200 receivers log-spaced 5-300 km, nt 4096,
    dt 0.05 s, 16384 wavenumbers;
  * a seeded 40-layer crust, 1000 receivers uniform in 1-500 km, nt 8192,
    dt 0.05 s, 32768 wavenumbers.
Double-couple-type moment-tensor source, sigma = pi/T, the reference's
receiver-layer and d/dz quirks corrected (the synthetic workloads' setting),
its 20-column layout.  Eight frequencies spread over the band.  Per receiver,
the relative L2 error over the selected frequencies and the 20 columns:
FP64 within TOL_FP64 (reassociation), FP32 within TOL_FP32."""
import math

import numpy as np
import pytest

TOL_FP64 = 1e-9
TOL_FP32 = 1e-3


def config_job(g, name, precision, sel=None):
    """(model, opts, dists) of the named configuration."""
    from grtm_cuda_gb300 import synth
    if name == "crust20":
        mk, d = synth.crust20_model(1234)
        log2n, nk = 12, 16384
    else:
        mk, d = synth.crust40_model(1234, n_receivers=1000)
        log2n, nk = 13, 32768
    o = g.make_opts(0.05, log2n, 0.0, 0.3, math.pi, g.K_FIXED, nk, precision=precision, fix=g.FIX_ALL,
                    freq_sel=sel)
    return mk, g.make_model(**mk), o, d


def selection(nw):
    """Eight frequency indices: three spread geometrically over the lowest
    eighth of the band, five evenly over the rest up to the last (inside the
    taper)."""
    lo = np.geomspace(1, nw / 8, 3)
    hi = np.linspace(nw / 4, nw - 1, 5)
    return np.unique(np.round(np.concatenate([lo, hi])).astype(np.int32))


def post(job, iw):
    """Phase, taper and scale of the spectral stage (green.cu:1905-1921) at iw."""
    nw = job.nw
    wc = int(nw * (1 - job.taper))
    st0 = 0.5 * (1.0 + math.cos((iw - wc + 1) * math.pi / (nw - wc + 1))) if iw > wc else 1.0
    phi = 2 * math.pi * job.df * iw * job.t0
    return complex(math.cos(phi), math.sin(phi)) * st0 * job.df * nw / math.pi


def oracle_spectra(oracle, mk, o, d, sel):
    """[nd, 20, nsel] complex: the oracle's k-sums at the selected
    frequencies, times the spectral stage's post factor."""
    job = oracle.model(mk["ztop"], mk["vp"], mk["vs"], mk["rho"], mk["qp"], mk["qs"], mk["hs"], mk["hr"],
                       mk["src_type"])
    oracle.setup(job, o.dt, o.log2n, o.t0, o.taper, o.sigma_factor, oracle.K_FIXED, o.nk_fixed,
                 fix=oracle.FIX_ALL | oracle.STABLE)
    out = np.empty((len(d), 20, len(sel)), complex)
    for i, iw in enumerate(sel):
        s = oracle.run_band(job, d, int(iw), int(iw) + 1)[0]         # [nd, 30]
        out[:, :, i] = s[:, :20] * post(job, int(iw))
    return out


def per_receiver(a, ref):
    return np.linalg.norm(a - ref, axis=(1, 2)) / np.linalg.norm(ref, axis=(1, 2))


@pytest.fixture(scope="module")
def gctx():
    import grtm_cuda_gb300 as g
    g.lib()
    c = g.Context()
    yield g, c
    c.close()


@pytest.fixture(scope="module", params=["crust20", "crust40"])
def case(request, oracle, gctx):
    g, _ = gctx
    mk, _, o, d = config_job(g, request.param, g.FP64)
    sel = selection(1 << (o.log2n - 1))
    return request.param, sel, oracle_spectra(oracle, mk, o, d, sel)


def gpu_spectra(g, ctx, name, precision, sel):
    _, m, o, d = config_job(g, name, precision, sel)
    p = g.Plan(ctx, m, o, d)
    p.execute()
    s = p.fetch_freqs(sel)
    p.close()
    return s


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_spectra_match_oracle_at_config_size(gctx, case, prec):
    g, ctx = gctx
    name, sel, ref = case
    s = gpu_spectra(g, ctx, name, g.FP64 if prec == "fp64" else g.FP32, sel)
    e = per_receiver(s, ref)
    tol = TOL_FP64 if prec == "fp64" else TOL_FP32
    print(f"{name} {prec}: per-receiver rel-L2 max {e.max():.3e} median {np.median(e):.3e}")
    assert np.isfinite(e).all() and e.max() <= tol, (name, prec, float(e.max()), float(np.median(e)))
