"""Algorithmic flop count of the per-(w,k) GRT evaluation (test infrastructure:
the roofline's work figure).

Runs the oracle built as C++ with the operation-counting complex type
(oracle/grt_count.hpp, library _build/libgrt_oracle_count.so) over sampled
(w, k) points of seeded crustal models and reports complex operations per
point by the convention cmul 6, cadd 2, cdiv 11, cexp / csqrt / clog 20
(the full list is in grt_count.hpp).  The evaluation counted is the oracle's
well-conditioned formulation of the reference's per-(w,k) pipeline
(set_pars, interface R/T, get_grt, get_src_*, get_ypars_a_*:
green.cu:164-1413) over every layer; per-frequency quantities ((w/alpha)^2,
(w/beta)^2, the shear moduli) are excluded, and so are the redundant (L-1)
repetitions of the reference's batched 4x4 solves (green.cu:1810-1818).

The count per point is linear in the layer count L (after source-interface
insertion): F(L) = L F_layer + F_src.  F_layer and F_src are fitted over
models of 10-60 layers, and the fit is checked against the exact mean count
of the benchmark's held-out models.

    python oracle/op_count.py            # prints a JSON summary
"""
import ctypes
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

from oracle import oracle as O  # noqa: E402

COUNT_LIB = os.path.join(HERE, "_build", "libgrt_oracle_count.so")
_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(COUNT_LIB):
            O.build()
        L = ctypes.CDLL(COUNT_LIB)
        P = ctypes.POINTER
        dp = P(ctypes.c_double)
        L.grto_model.argtypes = [P(O.Job), ctypes.c_int, dp, dp, dp, dp, dp, dp,
                                 ctypes.c_double, ctypes.c_double, ctypes.c_int]
        L.grto_setup.argtypes = [P(O.Job), ctypes.c_double, ctypes.c_int, ctypes.c_double,
                                 ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                 ctypes.c_double, ctypes.c_int]
        L.grto_nk.argtypes = [P(O.Job), ctypes.c_int]
        L.grto_count_point.argtypes = [P(O.Job), ctypes.c_int, ctypes.c_double]
        L.grto_count_point.restype = ctypes.c_longlong
        _lib = L
    return _lib


def job(mk, dt=0.05, log2n=13, nk=32768, fix=O.FIX_ALL | O.STABLE):
    """A counting-library job of model mk (synth.crust keys) on a fixed grid."""
    arrs = [np.ascontiguousarray(mk[k], dtype=np.float64) for k in ("ztop", "vp", "vs", "rho", "qp", "qs")]
    J = O.Job()
    rc = lib().grto_model(ctypes.byref(J), len(arrs[0]), *[a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
                                                           for a in arrs], float(mk["hs"]), float(mk["hr"]),
                          int(mk["src_type"]))
    assert rc == 0, rc
    rc = lib().grto_setup(ctypes.byref(J), dt, log2n, 0.0, 0.3, np.pi, O.K_FIXED, nk, 0.0, fix)
    assert rc == 0, rc
    J._keep = arrs
    return J


def mean_count(J, nfreq=24, nkpts=48):
    """Mean complex-operation count per (w,k) point over nfreq frequencies x
    nkpts wavenumbers spread evenly over the grid."""
    nk = lib().grto_nk(ctypes.byref(J), 0)
    tot, n = 0, 0
    for iw in np.linspace(1, J.nw - 1, nfreq).astype(int):
        for ik in np.linspace(0, nk - 1, nkpts).astype(int):
            tot += lib().grto_count_point(ctypes.byref(J), int(iw), float(ik * J.dk))
            n += 1
    return tot / n


def count(src_type=1):
    """Fit F(L) = L F_layer + F_src over seeded crusts of 10-60 layers (source
    at 15 km, surface receiver, the synthetic workloads' corrections) and
    compare with the benchmark's two held-out 40-layer models."""
    from grtm_cuda_gb300 import synth
    Ls, Fs = [], []
    for n in (10, 20, 30, 40, 50, 60):
        mk = synth.crust(np.random.default_rng(500 + n), n, 15.0, src_type=src_type)
        J = job(mk)
        Ls.append(J.n_layer)
        Fs.append(mean_count(J))
    a, b = np.polyfit(Ls, Fs, 1)
    resid = float(np.max(np.abs(np.polyval([a, b], Ls) - Fs) / np.asarray(Fs)))
    bench = []
    for i in range(2):   # bench.py's held-out models (seeds 3000 + i)
        rng = np.random.default_rng(3000 + i)
        mk = synth.crust(rng, 40, rng.uniform(1.0, 30.0), src_type=src_type)
        J = job(mk)
        f = mean_count(J)
        bench.append({"n_layer": J.n_layer, "s_layer": J.s_layer, "count": f,
                      "fit": float(a * J.n_layer + b), "fit_rel_err": float(abs(a * J.n_layer + b - f) / f)})
    return {"F_layer": float(a), "F_src": float(b), "fit_max_rel_residual": resid,
            "layers": Ls, "counts": [float(x) for x in Fs], "bench_models": bench}


def main():
    out = {"convention": "cmul 6, cadd 2, cdiv 11, cexp/csqrt/clog 20, real*complex 2, complex/real 2, "
                         "real+-complex 1; per (w,k) point of the oracle's stable formulation, all layers",
           "moment_tensor": count(1), "single_force": count(0)}
    print(json.dumps(out, indent=1))


if __name__ == "__main__":
    main()
