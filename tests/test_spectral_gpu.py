"""The FP32 spectral stage (phase/taper/scale, Hermitian fill, inverse DFT,
de-damping: green.cu:1905-1938, 2222-2239) against numpy in double on the
plan's own spectra: the fetched full spectra Y (filled by a separate kernel
from the same wavenumber sums) give x[n] = Re IDFT(Y)[n] e^{sigma (n dt + t0)},
which the traces must reproduce to FP32 rounding at every length the job
accepts (log2 N = 2..15; the transform is a half-length complex FFT)."""
import math

import numpy as np
import pytest

TOL_REL_L2 = 3e-6      # per trace, against the trace's norm
TOL_MAX = 1e-5         # largest sample error, against the trace's largest sample


def _model(g):
    from grtm_cuda_gb300 import synth
    m, _ = synth.crust4_model()
    return g.make_model(**m)


@pytest.mark.gpu
@pytest.mark.parametrize("log2n", [2, 3, 4, 5, 6, 8, 9, 10, 11, 12, 13, 14, 15])
def test_spectral_stage_matches_numpy(log2n):
    import grtm_cuda_gb300 as g
    N = 1 << log2n
    dt = 0.05 * max(1.0, 4096 / N) if N < 4096 else 0.05
    t0 = 1.5
    o = g.make_opts(dt, log2n, t0=t0, sigma_factor=math.pi, k_mode=g.K_FIXED, nk_fixed=256, precision=g.FP32,
                    fix=g.FIX_ALL)
    d = np.array([10.0, 55.0])
    tr, sp, rep = g.run(_model(g), o, d, spectra=True)
    assert tr.shape[-1] == N and sp.shape[-1] == N
    n = np.arange(N)
    damp = np.exp(rep["sigma"] * (n * dt + t0))
    ref = np.real(np.fft.ifft(sp.astype(np.complex128), axis=-1)) * damp
    nrm = np.linalg.norm(ref, axis=-1)
    live = nrm > 0
    assert live.sum() >= 2
    err = np.linalg.norm(tr - ref, axis=-1)[live] / nrm[live]
    assert err.max() <= TOL_REL_L2, err.max()
    mx = np.abs(tr - ref).max(axis=-1)[live] / np.abs(ref).max(axis=-1)[live]
    assert mx.max() <= TOL_MAX, mx.max()
