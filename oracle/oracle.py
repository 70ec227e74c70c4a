"""ctypes front-end of the FP64 CPU oracle (test infrastructure only).

The oracle is the checker of the CUDA product: only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py``'s cpu_baseline / reference arm
may import this module.  It restates the reference's GRT path
(cusrc/popm/func/green.cu) in plain FP64 C; see grt_oracle.c for the
line-by-line citations.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libgrt_oracle.so")

K_REFERENCE = 0
K_FIXED = 1
FIX_RLAYER = 1
FIX_REXUT = 2
FIX_DZ = 4
FIX_ALL = FIX_RLAYER | FIX_REXUT | FIX_DZ
STABLE = 8
FIX_COLS = 16   # corrected output columns (not the reference layout)
FIX_SHSRC = 32  # moment-tensor SH source terms with the jump structure of their order
ATTEN_MU = 64   # standard viscoelastic shear modulus rho beta(w)^2 (oracle only)
MAXL = 256


class Job(ctypes.Structure):
    _fields_ = [
        ("n_layer", ctypes.c_int),
        ("h", ctypes.c_double * MAXL),
        ("a0", ctypes.c_double * MAXL),
        ("b0", ctypes.c_double * MAXL),
        ("rho", ctypes.c_double * MAXL),
        ("qp", ctypes.c_double * MAXL),
        ("qs", ctypes.c_double * MAXL),
        ("mu", ctypes.c_double * MAXL),
        ("inserted", ctypes.c_int),
        ("hs", ctypes.c_double),
        ("hr", ctypes.c_double),
        ("s_layer", ctypes.c_int),
        ("r_layer", ctypes.c_int),
        ("zs", ctypes.c_double),
        ("zr", ctypes.c_double),
        ("src_type", ctypes.c_int),
        ("dt", ctypes.c_double),
        ("t0", ctypes.c_double),
        ("taper", ctypes.c_double),
        ("twin", ctypes.c_double),
        ("nf1", ctypes.c_int),
        ("nf2", ctypes.c_int),
        ("n_ptam", ctypes.c_int),
        ("log2n", ctypes.c_int),
        ("nw", ctypes.c_int),
        ("df", ctypes.c_double),
        ("sigma", ctypes.c_double),
        ("dk", ctypes.c_double),
        ("vmax", ctypes.c_double),
        ("vmin", ctypes.c_double),
        ("k_mode", ctypes.c_int),
        ("nk_fixed", ctypes.c_int),
        ("fix", ctypes.c_int),
        ("n_dist", ctypes.c_int),
        ("dist", ctypes.POINTER(ctypes.c_double)),
        ("dist0", ctypes.c_double),
    ]


_lib = None


def build():
    """Compile the oracle with its Makefile (gcc, OpenMP)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.POINTER
        dp = P(ctypes.c_double)
        L.grto_parse.argtypes = [ctypes.c_char_p, P(Job)]
        L.grto_model.argtypes = [P(Job), ctypes.c_int, dp, dp, dp, dp, dp, dp,
                                 ctypes.c_double, ctypes.c_double, ctypes.c_int]
        L.grto_setup.argtypes = [P(Job), ctypes.c_double, ctypes.c_int, ctypes.c_double,
                                 ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                 ctypes.c_double, ctypes.c_int]
        L.grto_nk.argtypes = [P(Job), ctypes.c_int]
        L.grto_nkw.argtypes = [P(Job)]
        L.grto_nkw.restype = ctypes.c_longlong
        L.grto_run.argtypes = [P(Job), dp, dp, ctypes.c_int]
        L.grto_run_band.argtypes = [P(Job), ctypes.c_int, ctypes.c_int, dp, ctypes.c_int]
        L.grto_point.argtypes = [P(Job), ctypes.c_int, ctypes.c_double, dp]
        L.grto_integrand.argtypes = [P(Job), ctypes.c_int, ctypes.c_double, ctypes.c_double, dp]
        L.grto_green.argtypes = [ctypes.c_char_p] * 3 + [ctypes.c_int]
        for n in ("grto_besselj", "grto_d_besselj", "grto_dd_besselj"):
            getattr(L, n).argtypes = [ctypes.c_double, ctypes.c_int]
            getattr(L, n).restype = ctypes.c_double
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _check(rc, what):
    if rc != 0:
        raise RuntimeError(f"oracle {what} failed with status {rc}")


def parse(path):
    job = Job()
    _check(lib().grto_parse(path.encode(), ctypes.byref(job)), "parse")
    return job


def model(ztop, vp, vs, rho, qp, qs, hs, hr, src_type):
    arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (ztop, vp, vs, rho, qp, qs)]
    job = Job()
    _check(lib().grto_model(ctypes.byref(job), len(arrs[0]), *[_dp(a) for a in arrs],
                            float(hs), float(hr), int(src_type)), "model")
    job._keep = arrs
    return job


def setup(job, dt, log2n, t0, taper, sigma_factor=2.0, k_mode=K_REFERENCE, nk_fixed=0,
          dk=0.0, fix=0):
    _check(lib().grto_setup(ctypes.byref(job), dt, log2n, t0, taper, sigma_factor, k_mode,
                            nk_fixed, dk, fix), "setup")
    return job


def nk_list(job):
    return np.array([lib().grto_nk(ctypes.byref(job), i) for i in range(job.nw)], dtype=np.int64)


def run(job, dists, nthreads=0, want_spec=True, want_sig=True):
    """Returns (spec [nd, N, 30] complex128, sig [nd, N, 30] float64)."""
    d = np.ascontiguousarray(np.atleast_1d(dists), dtype=np.float64)
    job.n_dist = len(d)
    job.dist = _dp(d)
    N = 2 * job.nw
    spec = np.zeros((len(d), N, 30, 2)) if want_spec else None
    sig = np.zeros((len(d), N, 30)) if want_sig else None
    rc = lib().grto_run(ctypes.byref(job), _dp(spec) if want_spec else None,
                        _dp(sig) if want_sig else None, int(nthreads))
    job.dist = ctypes.POINTER(ctypes.c_double)()
    _check(rc, "run")
    if want_spec:
        spec = spec[..., 0] + 1j * spec[..., 1]
    return spec, sig


def run_band(job, dists, iw0, iw1, nthreads=0):
    """k-sums of frequencies [iw0, iw1) for all receivers: [iw1-iw0, nd, 30] complex."""
    d = np.ascontiguousarray(np.atleast_1d(dists), dtype=np.float64)
    job.n_dist = len(d)
    job.dist = _dp(d)
    out = np.zeros((iw1 - iw0, len(d), 30, 2))
    rc = lib().grto_run_band(ctypes.byref(job), iw0, iw1, _dp(out), int(nthreads))
    job.dist = ctypes.POINTER(ctypes.c_double)()
    _check(rc, "run_band")
    return out[..., 0] + 1j * out[..., 1]


def point(job, iw, k):
    out = np.zeros(32)
    _check(lib().grto_point(ctypes.byref(job), iw, k, _dp(out)), "point")
    return out[0::2] + 1j * out[1::2]


def integrand(job, iw, k, r):
    out = np.zeros(60)
    _check(lib().grto_integrand(ctypes.byref(job), iw, k, r, _dp(out)), "integrand")
    return out[0::2] + 1j * out[1::2]


def green(iname, oname_w, oname_t, nthreads=0):
    _check(lib().grto_green(iname.encode(), oname_w.encode(), oname_t.encode(), nthreads), "green")


def besselj(x, n):
    return lib().grto_besselj(x, n)


def d_besselj(x, n):
    return lib().grto_d_besselj(x, n)


def dd_besselj(x, n):
    return lib().grto_dd_besselj(x, n)


def read_table(path, complex_pairs=False):
    """Read an output file of the reference writers (rows of 'v,' fields)."""
    rows = []
    with open(path) as f:
        for line in f:
            vals = [float(x) for x in line.strip().split(",") if x.strip()]
            if vals:
                rows.append(vals)
    a = np.array(rows)
    if complex_pairs:
        a = a[:, 0::2] + 1j * a[:, 1::2]
    return a
