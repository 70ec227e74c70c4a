"""The roofline's algorithmic work: the frozen per-point flop constants of
bench.py are the operation-counting oracle's (oracle/op_count.py), and the
counting type counts by its stated convention."""
import ctypes

import numpy as np


def test_bench_constants_are_the_counted_ones():
    import bench
    from oracle import op_count
    mt, sf = op_count.count(1), op_count.count(0)
    assert round(mt["F_layer"]) == bench.F_LAYER == round(sf["F_layer"])
    assert round(mt["F_src"]) == bench.F_SRC_TENSOR and round(sf["F_src"]) == bench.F_SRC_SINGLE
    # linear in the layer count, and the fit holds on the benchmark's models
    assert mt["fit_max_rel_residual"] < 0.02
    assert all(b["fit_rel_err"] < 0.02 for b in mt["bench_models"])


def test_counting_convention_on_a_half_space():
    """A surface receiver above a source in the top layer of a half-space
    model: the count is deterministic, independent of the values at one
    branch, and grows by the same per-layer amount when a layer is split."""
    from oracle import op_count
    from grtm_cuda_gb300 import synth
    mk = synth.crust(np.random.default_rng(7), 6, 3.0)
    J = op_count.job(mk, log2n=10, nk=4096)
    L = op_count.lib()
    c1 = L.grto_count_point(ctypes.byref(J), 100, 0.3)
    c2 = L.grto_count_point(ctypes.byref(J), 100, 0.3)
    assert c1 == c2 > 0
    # one layer more below the source: the same branches, one F_layer more
    mk2 = dict(mk)
    z = mk["ztop"]
    mk2["ztop"] = np.concatenate([z[:-1], [0.5 * (z[-2] + z[-1])], z[-1:]])
    for key in ("vp", "vs", "rho", "qp", "qs"):
        mk2[key] = np.concatenate([mk[key][:-1], mk[key][-2:-1], mk[key][-1:]])
    J2 = op_count.job(mk2, log2n=10, nk=4096)
    assert J2.n_layer == J.n_layer + 1
    d = L.grto_count_point(ctypes.byref(J2), 100, 0.3) - c1
    assert 1000 < d < 2000, d
