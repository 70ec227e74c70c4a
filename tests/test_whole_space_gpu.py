"""The CUDA path against the exact whole-space solutions (GB300).

The configuration of test_analytic.py -- a uniform, nearly elastic medium,
source and receivers 60-80 km deep, the first 20 s holding only the direct
waves -- run through the library with every correction of the reference
(FIX_PHYSICAL: the corrected 30-column layout and GRT_FIX_SHSRC), in FP64
and FP32: combined by grt_mt_weights / grt_sf_weights, the traces must equal
Aki & Richards eq. 4.29 and Stokes' solution with no fitted constant."""
import math

import numpy as np
import pytest

import test_analytic as A

pytestmark = pytest.mark.gpu

TOL = {"fp64": A.TOL, "fp32": 2e-3}


def _gpu_traces(g, ctx, hs, hr, src, precision):
    q = [1e6, 1e6]
    m = g.make_model(A.TOPS, [A.ALPHA] * 2, [A.BETA] * 2, [A.RHO] * 2, q, q, hs, hr, src)
    o = g.make_opts(A.DT, A.LOG2N, 0.0, 0.3, math.pi, g.K_FIXED, A.NK, precision=precision, fix=g.FIX_PHYSICAL)
    traces, _, rep = g.run(m, o, [A.DIST], ctx)
    assert rep["n_cols"] == (30 if src == 1 else 15)
    return traces[0]                                   # [n_cols, N]


@pytest.fixture(scope="module")
def gctx():
    import grtm_cuda_gb300 as g
    g.lib()
    c = g.Context()
    yield g, c
    c.close()


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
@pytest.mark.parametrize("hs,hr", [(60.0, 80.0), (80.0, 60.0)])
def test_gpu_moment_tensor_equals_aki_richards(gctx, hs, hr, prec):
    g, ctx = gctx
    tr = _gpu_traces(g, ctx, hs, hr, 1, g.FP64 if prec == "fp64" else g.FP32)
    cases = dict(A.MOMENTS, dc=list(g.dc_moment(30, 60, 90)))
    for name, m6 in cases.items():
        m6 = np.array(m6, float)
        ours = A._convolve(g.mt_weights(m6, A.PHI) @ tr)
        assert A._rel(ours, A._aki_richards(A._tensor(m6), hs, hr)) <= TOL[prec], name


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
@pytest.mark.parametrize("hs,hr", [(60.0, 80.0), (80.0, 60.0)])
def test_gpu_single_force_equals_stokes(gctx, hs, hr, prec):
    g, ctx = gctx
    tr = _gpu_traces(g, ctx, hs, hr, 0, g.FP64 if prec == "fp64" else g.FP32)
    for F in ([0.0, 0.0, 1.0], [1.0, 0.0, 0.0], [0.3, -0.7, 0.5]):
        ours = A._convolve(g.sf_weights(F, A.PHI) @ tr)
        assert A._rel(ours, A._stokes(np.array(F), hs, hr)) <= TOL[prec], F
