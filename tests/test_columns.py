"""Corrected output columns (GRT_FIX_COLS): the derivative columns are the
derivatives of the displacement columns -- checked by central differences on
the FP64 oracle over the same wavenumber grid -- and the GPU reproduces the
oracle in this layout."""
import math

import numpy as np
import pytest

from oracle import oracle as O

FIXC = O.FIX_ALL | O.STABLE | O.FIX_COLS


def _model():
    from grtm_cuda_gb300 import synth
    m, _ = synth.crust4_model()
    return m


def _spec(src, hr, d, fix=FIXC, log2n=7, nk=1024, dk=0.0):
    m = _model()
    j = O.model(m["ztop"], m["vp"], m["vs"], m["rho"], m["qp"], m["qs"], m["hs"], hr, src)
    O.setup(j, 0.2, log2n, 0.0, 0.3, math.pi, O.K_FIXED, nk, dk, fix)
    s, t = O.run(j, np.atleast_1d(d), nthreads=0)
    return s, t


def _dk(src, hr):
    m = _model()
    j = O.model(m["ztop"], m["vp"], m["vs"], m["rho"], m["qp"], m["qs"], m["hs"], hr, src)
    O.setup(j, 0.2, 7, 0.0, 0.3, math.pi, O.K_FIXED, 1024, 0.0, FIXC)
    return j.dk


@pytest.mark.parametrize("src", [1, 0])
def test_derivative_columns_are_derivatives(src):
    hr, d, dz, dr = 3.0, 40.0, 1e-4, 1e-3
    # the wavenumber step follows |hs - hr| (green.cu:2077-2080): the shifted
    # receivers keep the unshifted job's grid, or the difference quotient would
    # also see the grid move (2.7e-5 tensor, 7.6e-4 single force)
    dk = _dk(src, hr)
    s0, _ = _spec(src, hr, d, dk=dk)
    sz = (_spec(src, hr + dz, d, dk=dk)[0] - _spec(src, hr - dz, d, dk=dk)[0]) / (2 * dz)
    sr = (_spec(src, hr, d + dr, dk=dk)[0] - _spec(src, hr, d - dr, dk=dk)[0]) / (2 * dr)
    nw = s0.shape[1] // 2
    disp, zoff, roff = (10, 10, 20) if src == 1 else (5, 5, 10)
    for c in range(disp):
        b = sz[0, :nw, c]
        e = np.abs(s0[0, :nw, zoff + c] - b).max() / np.abs(b).max()
        assert e <= 1e-6, (c, e)
        if src == 1 or c == 0:
            b = sr[0, :nw, c]
            e = np.abs(s0[0, :nw, roff + c] - b).max() / np.abs(b).max()
            assert e <= 1e-5, (c, e)


def test_reference_layout_unchanged_without_the_bit():
    s_ref, _ = _spec(1, 3.0, 40.0, fix=O.FIX_ALL | O.STABLE)
    s_fix, _ = _spec(1, 3.0, 40.0)
    # columns 0-9 agree except the m = 0 radial terms (2, 3: radial instead of
    # vertical coefficients) and the m = 1 transverse term (5); 10-19 of the
    # reference hold d/dr, 20-29 are empty there
    for c in (0, 1, 4, 6, 7, 8, 9):
        assert np.array_equal(s_ref[..., c], s_fix[..., c])
    for c in (2, 3, 5):
        assert not np.allclose(s_ref[..., c], s_fix[..., c])
    assert np.all(s_ref[..., 20:] == 0) and np.any(s_fix[..., 20:] != 0)


@pytest.mark.parametrize("src", [1, 0])
def test_free_surface_has_no_shear_traction(src):
    """At a surface receiver sigma_rz = mu (du_r/dz + du_z/dr) vanishes: in the
    corrected layout the d/dz of each radial column equals the d/dr of the
    vertical column of its azimuthal family (the SH parts' d/dz vanish there).
    Moment tensor: (radial, vertical) = (0, 6), (1, 7), (2, 9), (3, 8); single
    force (1, 4), (0, 3).  The reference's m = 0 radial columns 2 and 3, built
    from the vertical coefficients, fail it."""
    s, _ = _spec(src, 0.0, [15.0, 40.0], fix=FIXC | O.FIX_SHSRC)
    nw = s.shape[1] // 2
    pairs = [(10, 26), (11, 27), (12, 29), (13, 28)] if src == 1 else [(6, 14), (5, 13)]
    for dz_col, dr_col in pairs:
        a, b = s[:, :nw, dz_col], s[:, :nw, dr_col]
        assert np.abs(a - b).max() <= 1e-12 * np.abs(b).max(), (dz_col, dr_col)


@pytest.mark.gpu
@pytest.mark.parametrize("src", [1, 0])
def test_gpu_corrected_columns_match_oracle(src):
    import grtm_cuda_gb300 as g
    m = dict(_model(), hr=3.0, src_type=src)
    d = np.array([15.0, 40.0, 90.0])
    s_o, t_o = _spec(src, 3.0, d, log2n=8, nk=1536)
    ncol = 30 if src == 1 else 15
    for prec, tol in ((g.FP64, 1e-10), (g.FP32, 5e-5)):
        o = g.make_opts(0.2, 8, sigma_factor=math.pi, k_mode=g.K_FIXED, nk_fixed=1536, precision=prec,
                        fix=g.FIX_ALL | g.FIX_COLS)
        t, s, rep = g.run(g.make_model(**m), o, d, spectra=True)
        assert rep["n_cols"] == ncol
        t_ref = np.transpose(t_o, (0, 2, 1))[:, :ncol]
        err = np.linalg.norm(t - t_ref, axis=-1) / np.linalg.norm(t_ref, axis=-1).max(axis=-1, keepdims=True)
        assert err.max() <= tol, (prec, err.max())


@pytest.mark.gpu
@pytest.mark.parametrize("hr", [0.0, 3.0])
def test_gpu_corrected_20_column_layout_on_the_tensor_cores(hr):
    """GRT_FIX_COLS20: the corrected moment-tensor columns in the 20-column
    layout the tensor-core sum takes.  Its columns 0-9 and 10-19 are the
    oracle's corrected displacement (0-9) and d/dr (20-29) columns, with the
    SH source terms corrected too; FP32 runs on the tensor cores (3xTF32),
    FP64 on the SIMT sum."""
    import grtm_cuda_gb300 as g
    m = dict(_model(), hr=hr, src_type=1)
    d = np.array([15.0, 40.0, 90.0])
    _, t_o = _spec(1, hr, d, fix=FIXC | O.FIX_SHSRC, log2n=8, nk=1536)
    t_ref = np.transpose(t_o, (0, 2, 1))
    t_ref = np.concatenate([t_ref[:, :10], t_ref[:, 20:30]], axis=1)
    for prec, tol, impl in ((g.FP64, 1e-10, 0), (g.FP32, 5e-5, 1)):
        o = g.make_opts(0.2, 8, sigma_factor=math.pi, k_mode=g.K_FIXED, nk_fixed=1536, precision=prec,
                        fix=g.FIX_PHYSICAL_TC)
        t, _, rep = g.run(g.make_model(**m), o, d)
        assert rep["n_cols"] == 20 and rep["ksum_impl"] == impl
        err = np.linalg.norm(t - t_ref, axis=-1) / np.linalg.norm(t_ref, axis=-1).max(axis=-1, keepdims=True)
        assert err.max() <= tol, (prec, err.max())
