"""Earth flattening: the library's transform reproduces the reference's own
flattened demo input (demo/input.txt is crust1.0 with an 8 km source,
flattened by greent.py:13-47, 65-67)."""
import os

import numpy as np

from conftest import GOLDEN


def _read_input(path):
    lines = [ln.strip() for ln in open(path) if ln.strip()]
    hs, hr, n = float(lines[0]), float(lines[1]), int(lines[2])
    layers = np.array([[float(x) for x in lines[3 + i].split(",") if x.strip()] for i in range(n)])
    return hs, hr, layers


def test_flatten_reproduces_demo_input():
    import grtm_cuda_gb300 as g
    hs, hr, lay = _read_input(os.path.join(GOLDEN, "example_crust1.0_input.txt"))
    hs_f, hr_f, lay_f = _read_input(os.path.join(GOLDEN, "demo_input.txt"))
    m = dict(ztop=lay[:, 0], vp=lay[:, 1], vs=lay[:, 2], rho=lay[:, 3], qp=lay[:, 4], qs=lay[:, 5], hs=hs, hr=hr,
             src_type=0)
    f = g.flatten(m)
    assert abs(f["hs"] - hs_f) < 1e-12 and abs(f["hr"] - hr_f) < 1e-12
    assert np.allclose(f["ztop"], lay_f[:, 0], rtol=0, atol=1e-12)
    assert np.allclose(f["vp"], lay_f[:, 1], rtol=1e-14) and np.allclose(f["vs"], lay_f[:, 2], rtol=1e-14)
    assert np.array_equal(f["rho"], lay[:, 3]) and np.array_equal(f["qs"], lay[:, 5])


def test_flatten_rejects_bad_models():
    import pytest
    import grtm_cuda_gb300 as g
    m = dict(ztop=[0.0, 10.0, 5.0], vp=[5, 6, 7], vs=[3, 3.5, 4], rho=[2, 2, 2], qp=[1, 1, 1], qs=[1, 1, 1], hs=1.0)
    with pytest.raises(g.GrtError):
        g.flatten(m)
