"""GB300 layered-medium Green's functions by the generalized
reflection-transmission method.

Python front-end over the library's C ABI (include/grtm_gb300.h), loaded with
ctypes exactly as the reference's scripts load theirs
(``ctypes.cdll.LoadLibrary("build/libpopm.so").green(iname, oname_w, oname_t)``,
greent.py:94-98).  All computation runs in the CUDA library; if it is missing
this module raises instead of falling back to anything else.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.environ.get("GRTM_GB300_LIB", os.path.join(HERE, "_lib", "libgrtm_gb300.so"))

OK, ERR_ARG, ERR_IO, ERR_PARSE, ERR_MODEL, ERR_CUDA, ERR_NOMEM, ERR_TIMEOUT, ERR_UNSUPPORTED = range(9)
K_REFERENCE, K_FIXED, K_CUSTOM = 0, 1, 2
FP32, FP64 = 0, 1
TC_3XTF32, TC_3XBF16 = 0, 1   # split forms of the tensor-core wavenumber sum
FIX_RLAYER, FIX_REXUT, FIX_DZ, FIX_COLS = 1, 2, 4, 8
FIX_SHSRC = 16   # moment-tensor SH source terms with the jump structure of their order
FIX_ALL = FIX_RLAYER | FIX_REXUT | FIX_DZ
# every correction of the reference: the receiver layer and d/dz terms, the corrected
# column layouts and the moment tensor's SH source terms (0 reproduces the reference)
FIX_PHYSICAL = FIX_ALL | FIX_COLS | FIX_SHSRC
# the same corrections in the 20-column layout (displacement and d/dr, no d/dz):
# physical moment-tensor output on the tensor-core wavenumber sum
FIX_COLS20 = 32
FIX_PHYSICAL_TC = FIX_ALL | FIX_COLS20 | FIX_SHSRC

_dp = ctypes.POINTER(ctypes.c_double)


class Model(ctypes.Structure):
    _fields_ = [("n_layer", ctypes.c_int), ("ztop", _dp), ("vp", _dp), ("vs", _dp), ("rho", _dp),
                ("qp", _dp), ("qs", _dp), ("hs", ctypes.c_double), ("hr", ctypes.c_double),
                ("src_type", ctypes.c_int)]


class Opts(ctypes.Structure):
    _fields_ = [("dt", ctypes.c_double), ("log2n", ctypes.c_int), ("t0", ctypes.c_double),
                ("taper", ctypes.c_double), ("sigma_factor", ctypes.c_double), ("k_mode", ctypes.c_int),
                ("nk_fixed", ctypes.c_int), ("dk", ctypes.c_double), ("precision", ctypes.c_int),
                ("fix", ctypes.c_int), ("nk_custom", ctypes.POINTER(ctypes.c_int)),
                ("k_stride", ctypes.POINTER(ctypes.c_int)), ("n_freq_sel", ctypes.c_int),
                ("freq_sel", ctypes.POINTER(ctypes.c_int)), ("k_slice", ctypes.c_int), ("tc_split", ctypes.c_int)]


class Report(ctypes.Structure):
    _fields_ = [("n_layer", ctypes.c_int), ("s_layer", ctypes.c_int), ("r_layer", ctypes.c_int),
                ("zs", ctypes.c_double), ("zr", ctypes.c_double), ("nw", ctypes.c_int),
                ("n_samples", ctypes.c_int), ("n_cols", ctypes.c_int), ("n_wk", ctypes.c_longlong),
                ("nk_max", ctypes.c_int), ("dk", ctypes.c_double), ("df", ctypes.c_double),
                ("sigma", ctypes.c_double), ("ms_grt", ctypes.c_float), ("ms_bessel", ctypes.c_float),
                ("ms_ksum", ctypes.c_float), ("ms_spectral", ctypes.c_float), ("ms_total", ctypes.c_float),
                ("kernel_launches", ctypes.c_int), ("h2d_bytes", ctypes.c_longlong),
                ("d2h_bytes", ctypes.c_longlong), ("ksum_impl", ctypes.c_int), ("k_slice", ctypes.c_int),
                ("n_layer_evals", ctypes.c_longlong)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class Source(ctypes.Structure):
    _fields_ = [("m", ctypes.c_double * 6), ("n_stf", ctypes.c_int), ("stf", _dp), ("f", ctypes.c_double * 3)]


def make_source(m6, stf=None):
    """A source with an optional source-time function sampled at the job's
    dt: a moment tensor (Mxx, Myy, Mzz, Mxy, Mxz, Myz) for moment-tensor
    jobs, or a force (Fx, Fy, Fz; x north, y east, z down) for single-force
    jobs."""
    s = Source()
    v = np.asarray(m6, dtype=np.float64).ravel()
    if v.size == 3:
        for i in range(3):
            s.f[i] = float(v[i])
    elif v.size == 6:
        for i in range(6):
            s.m[i] = float(v[i])
    else:
        raise ValueError("a source is a moment tensor (6 values) or a force (3 values)")
    if stf is not None:
        a = _arr(stf)
        s.n_stf = len(a)
        s.stf = _ptr(a)
        s._keep = a
    return s


class _HostBuf:
    """Page-locked host memory from grt_host_alloc, freed when the last
    array over it goes (numpy keeps this object as the arrays' base)."""

    def __init__(self, nbytes, dtype, shape):
        self.p = ctypes.c_void_p()
        rc = lib().grt_host_alloc(max(1, nbytes), ctypes.byref(self.p))
        if rc:
            raise GrtError(rc, "grt_host_alloc")
        self.__array_interface__ = {"shape": tuple(shape), "typestr": np.dtype(dtype).str,
                                    "data": (self.p.value, False), "version": 3}

    def __del__(self):
        if self.p:
            try:
                lib().grt_host_free(self.p)
            except Exception:      # interpreter shutdown: the process frees it
                pass
            self.p = ctypes.c_void_p()


def pinned_empty(shape, dtype=np.float32):
    """An uninitialised array in page-locked host memory: the destination of
    fetches that should run at the host link's full rate."""
    shape = tuple(int(x) for x in np.atleast_1d(shape))
    return np.asarray(_HostBuf(int(np.prod(shape)) * np.dtype(dtype).itemsize, dtype, shape))


R_EARTH = 6371.0


def flatten(model, r_earth=R_EARTH):
    """Earth-flattened copy of a model dict (ztop, vp, vs, rho, qp, qs, hs,
    hr, src_type): grt_flatten."""
    zt, vp, vs = (_arr(model[k]) for k in ("ztop", "vp", "vs"))
    n = len(zt)
    zf, vpf, vsf = np.empty(n), np.empty(n), np.empty(n)
    hs, hr = ctypes.c_double(), ctypes.c_double()
    rc = lib().grt_flatten(n, _ptr(zt), _ptr(vp), _ptr(vs), float(model["hs"]), float(model.get("hr", 0.0)),
                           float(r_earth), _ptr(zf), _ptr(vpf), _ptr(vsf), ctypes.byref(hs), ctypes.byref(hr))
    if rc:
        raise GrtError(rc, "grt_flatten (details on stderr)")
    out = dict(model)
    out.update(ztop=zf, vp=vpf, vs=vsf, hs=hs.value, hr=hr.value)
    return out


def dc_moment(strike, dip, rake, m0=1.0):
    """Moment tensor (Mxx, Myy, Mzz, Mxy, Mxz, Myz) of a double couple."""
    m = (ctypes.c_double * 6)()
    lib().grt_dc_moment(float(strike), float(dip), float(rake), float(m0), m)
    return np.array(list(m))


def mt_weights(m6, azimuth):
    """Weights [3 (Z up, R away, T clockwise), 30] of the moment-tensor columns
    for moment tensor m6 (Mxx, Myy, Mzz, Mxy, Mxz, Myz; x north, y east, z down)
    at the receiver's azimuth from the source (degrees clockwise from north)."""
    m = np.ascontiguousarray(m6, dtype=np.float64)
    w = np.zeros((3, 30))
    lib().grt_mt_weights(_ptr(m), float(azimuth), _ptr(w))
    return w


def sf_weights(force, azimuth):
    """Weights [3 (Z up, R away, T clockwise), 15] of the single-force columns
    for force (Fx, Fy, Fz; x north, y east, z down) at the receiver's azimuth
    from the source (degrees clockwise from north)."""
    f = np.ascontiguousarray(force, dtype=np.float64)
    w = np.zeros((3, 15))
    lib().grt_sf_weights(_ptr(f), float(azimuth), _ptr(w))
    return w


class Job(ctypes.Structure):
    _fields_ = [("model", ctypes.POINTER(Model)), ("opts", ctypes.POINTER(Opts)), ("n_dist", ctypes.c_int),
                ("dist", _dp), ("out_f32", ctypes.POINTER(ctypes.c_float))]


TUNE_MAX = 16


class Tune(ctypes.Structure):
    _fields_ = [("tuned", ctypes.c_int), ("grt_shape", ctypes.c_int), ("grt_threads", ctypes.c_int),
                ("grt_blocks", ctypes.c_int),
                ("n_cand", ctypes.c_int), ("cand_threads", ctypes.c_int * TUNE_MAX),
                ("cand_blocks", ctypes.c_int * TUNE_MAX), ("cand_ms", ctypes.c_float * TUNE_MAX),
                ("sample_fraction", ctypes.c_double), ("tc_tuned", ctypes.c_int), ("tc_nsplit", ctypes.c_int),
                ("tc_n_cand", ctypes.c_int), ("tc_cand_split", ctypes.c_int * 4), ("tc_cand_ms", ctypes.c_float * 4)]

    def as_dict(self):
        n = self.n_cand
        return {"tuned": self.tuned, "grt_shape": self.grt_shape, "grt_threads": self.grt_threads,
                "grt_blocks": self.grt_blocks,
                "candidates": [(self.cand_threads[i], self.cand_blocks[i], self.cand_ms[i]) for i in range(n)],
                "sample_fraction": self.sample_fraction, "tc_tuned": self.tc_tuned, "tc_nsplit": self.tc_nsplit,
                "tc_candidates": [(self.tc_cand_split[i], self.tc_cand_ms[i]) for i in range(self.tc_n_cand)]}


# every symbol the public header declares
EXPORTS = ("grt_create", "grt_destroy", "grt_last_error", "grt_status_string", "grt_plan_create",
           "grt_plan_execute", "grt_plan_fetch", "grt_plan_fetch_freqs", "grt_plan_info", "grt_plan_destroy", "grt_grid", "grt_run",
           "grt_green", "green", "grt_run_noalloc", "grt_sweep_kmax", "grt_mlp_create", "grt_mlp_destroy",
           "grt_mlp_n_params", "grt_mlp_get_params", "grt_mlp_set_params", "grt_mlp_forward",
           "grt_mlp_loss_grad", "grt_mlp_train", "grt_batch_create", "grt_batch_execute", "grt_batch_fetch",
           "grt_batch_fetch_freqs", "grt_batch_info", "grt_batch_destroy", "grt_dc_moment", "grt_mt_weights",
           "grt_sf_weights",
           "grt_plan_synth",
           "grt_batch_synth", "grt_flatten", "grt_plan_write", "grt_plan_fetch_f32", "grt_batch_fetch_f32",
           "grt_host_alloc", "grt_host_free", "grt_trim", "grt_batch_fetch_f32_async", "grt_batch_wait",
           "grt_plan_error_estimate", "grt_batch_error_estimate", "grt_set_priority",
           "grt_tune_clear", "grt_device_synchronize", "grt_batch_launch", "grt_batch_wait_stages",
           "grt_batch_finish")

_lib = None


def build():
    from . import buildlib
    return buildlib.build()


def lib():
    """Load the CUDA library (building it first when only sources exist)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        build()
    L = ctypes.CDLL(LIB_PATH)
    P = ctypes.POINTER
    vp = ctypes.c_void_p
    L.grt_create.argtypes = [P(vp), ctypes.c_int]
    L.grt_destroy.argtypes = [vp]
    L.grt_destroy.restype = None
    L.grt_last_error.argtypes = [vp]
    L.grt_last_error.restype = ctypes.c_char_p
    L.grt_status_string.argtypes = [ctypes.c_int]
    L.grt_status_string.restype = ctypes.c_char_p
    L.grt_plan_create.argtypes = [vp, P(Model), P(Opts), ctypes.c_int, _dp, P(vp)]
    L.grt_plan_execute.argtypes = [vp, P(Report)]
    L.grt_plan_fetch.argtypes = [vp, _dp, _dp]
    L.grt_plan_fetch_freqs.argtypes = [vp, ctypes.c_int, P(ctypes.c_int), _dp]
    L.grt_plan_info.argtypes = [vp, P(Report)]
    L.grt_plan_destroy.argtypes = [vp]
    L.grt_plan_destroy.restype = None
    L.grt_grid.argtypes = [P(Model), P(Opts), P(Report)]
    L.grt_run.argtypes = [vp, P(Model), P(Opts), ctypes.c_int, _dp, _dp, _dp, P(Report)]
    L.grt_green.argtypes = [ctypes.c_char_p] * 3
    L.green.argtypes = [ctypes.c_char_p] * 3
    L.green.restype = None
    L.grt_run_noalloc.argtypes = [ctypes.c_int, P(Model), P(Opts), ctypes.c_int, _dp, _dp]
    ip = P(ctypes.c_int)
    fp = P(ctypes.c_float)
    L.grt_sweep_kmax.argtypes = [vp, P(Model), P(Opts), ctypes.c_int, ip, ctypes.c_int, _dp, ctypes.c_double,
                                 _dp, _dp, _dp, _dp, _dp, _dp]
    L.grt_mlp_create.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_ulonglong, P(vp)]
    L.grt_mlp_destroy.argtypes = [vp]
    L.grt_mlp_destroy.restype = None
    L.grt_mlp_n_params.argtypes = [vp]
    L.grt_mlp_get_params.argtypes = [vp, fp]
    L.grt_mlp_set_params.argtypes = [vp, fp]
    L.grt_mlp_forward.argtypes = [vp, ctypes.c_int, fp, fp]
    L.grt_mlp_loss_grad.argtypes = [vp, ctypes.c_int, fp, fp, fp, fp]
    L.grt_mlp_train.argtypes = [vp, ctypes.c_int, fp, fp, ctypes.c_int, ctypes.c_int, ctypes.c_float,
                                ctypes.c_ulonglong, fp]
    L.grt_batch_create.argtypes = [vp, ctypes.c_int, P(Job), ctypes.c_int, P(vp)]
    L.grt_batch_execute.argtypes = [vp, P(Report)]
    L.grt_batch_finish.argtypes = [vp, P(Report)]
    L.grt_batch_fetch.argtypes = [vp, ctypes.c_int, _dp, _dp]
    L.grt_batch_fetch_freqs.argtypes = [vp, ctypes.c_int, ctypes.c_int, ip, _dp]
    L.grt_batch_info.argtypes = [vp, ctypes.c_int, P(Report), P(Tune)]
    L.grt_batch_destroy.argtypes = [vp]
    L.grt_batch_destroy.restype = None
    L.grt_plan_write.argtypes = [vp, ctypes.c_char_p]
    L.grt_plan_fetch_f32.argtypes = [vp, P(ctypes.c_float)]
    L.grt_batch_fetch_f32.argtypes = [vp, ctypes.c_int, P(ctypes.c_float)]
    L.grt_host_alloc.argtypes = [ctypes.c_size_t, P(vp)]
    L.grt_host_free.argtypes = [vp]
    L.grt_host_free.restype = None
    L.grt_batch_fetch_f32_async.argtypes = [vp, ctypes.c_int, P(ctypes.c_float)]
    L.grt_batch_wait.argtypes = [vp]
    L.grt_trim.argtypes = [vp]
    L.grt_trim.restype = None
    L.grt_set_priority.argtypes = [vp, ctypes.c_int]
    L.grt_tune_clear.argtypes = []
    L.grt_device_synchronize.argtypes = [ctypes.c_int]
    L.grt_batch_launch.argtypes = [vp]
    L.grt_batch_wait_stages.argtypes = [vp]
    L.grt_tune_clear.restype = None
    L.grt_flatten.argtypes = [ctypes.c_int, _dp, _dp, _dp, ctypes.c_double, ctypes.c_double, ctypes.c_double, _dp,
                              _dp, _dp, _dp, _dp]
    L.grt_dc_moment.argtypes = [ctypes.c_double] * 4 + [_dp]
    L.grt_dc_moment.restype = None
    L.grt_mt_weights.argtypes = [_dp, ctypes.c_double, _dp]
    L.grt_mt_weights.restype = None
    L.grt_sf_weights.argtypes = [_dp, ctypes.c_double, _dp]
    L.grt_sf_weights.restype = None
    L.grt_plan_synth.argtypes = [vp, P(Source), _dp, _dp]
    L.grt_plan_error_estimate.argtypes = [vp, ctypes.c_double, _dp]
    L.grt_batch_error_estimate.argtypes = [vp, ctypes.c_int, ctypes.c_double, _dp]
    L.grt_batch_synth.argtypes = [vp, ctypes.c_int, P(Source), _dp, _dp]
    _lib = L
    return L


class GrtError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{lib().grt_status_string(status).decode()}: {msg}")
        self.status = status


def _arr(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _ptr(a):
    return a.ctypes.data_as(_dp)


class Context:
    """One CUDA stream on one device (grt_create / grt_destroy)."""

    def __init__(self, device=0):
        self.h = ctypes.c_void_p()
        self.device = int(device)
        rc = lib().grt_create(ctypes.byref(self.h), device)
        if rc:
            raise GrtError(rc, "grt_create failed")

    def error(self):
        return lib().grt_last_error(self.h).decode()

    def trim(self):
        """Return the device memory cached for reuse by later plans."""
        if self.h:
            lib().grt_trim(self.h)

    def set_priority(self, high=True):
        """The device's greatest stream priority for this context's work
        (grt_set_priority); only while it holds no plan or batch."""
        rc = lib().grt_set_priority(self.h, int(bool(high)))
        if rc:
            raise GrtError(rc, self.error())

    def close(self):
        if self.h:
            lib().grt_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def make_model(ztop, vp, vs, rho, qp, qs, hs, hr=0.0, src_type=0):
    arrs = [_arr(a) for a in (ztop, vp, vs, rho, qp, qs)]
    m = Model(len(arrs[0]), *[_ptr(a) for a in arrs], float(hs), float(hr), int(src_type))
    m._keep = arrs
    return m


def make_opts(dt, log2n, t0=0.0, taper=0.3, sigma_factor=2.0, k_mode=K_REFERENCE, nk_fixed=0, dk=0.0,
              precision=FP32, fix=0, nk_custom=None, k_stride=None, freq_sel=None, k_slice=0, tc_split=0):
    """nk_custom: points per frequency (N/2 ints) for K_CUSTOM grids;
    k_stride: optional per-frequency stride m (k_j = j m dk);
    freq_sel: evaluate only these frequency indices (a spectra-only plan);
    k_slice: wavenumbers per split-K slice of the tensor-core sum (0: auto);
    tc_split: TC_3XTF32 (default) or TC_3XBF16, the split form of the tensor-core sum."""
    o = Opts(float(dt), int(log2n), float(t0), float(taper), float(sigma_factor), int(k_mode),
             int(nk_fixed), float(dk), int(precision), int(fix), None, None, 0, None, int(k_slice), int(tc_split))
    o._keep = []
    if nk_custom is not None:
        arr = np.ascontiguousarray(nk_custom, dtype=np.int32)
        o.nk_custom = arr.ctypes.data_as(ctypes.POINTER(ctypes.c_int))
        o._keep.append(arr)
        o.k_mode = K_CUSTOM
    if k_stride is not None:
        arr = np.ascontiguousarray(k_stride, dtype=np.int32)
        o.k_stride = arr.ctypes.data_as(ctypes.POINTER(ctypes.c_int))
        o._keep.append(arr)
    if freq_sel is not None:
        arr = np.ascontiguousarray(freq_sel, dtype=np.int32)
        o.freq_sel = arr.ctypes.data_as(ctypes.POINTER(ctypes.c_int))
        o.n_freq_sel = len(arr)
        o._keep.append(arr)
    return o


class Plan:
    """A model, its grids, its receivers and their device buffers."""

    def __init__(self, ctx, model, opts, dists):
        self.ctx = ctx
        self.dists = _arr(np.atleast_1d(dists))
        self.h = ctypes.c_void_p()
        rc = lib().grt_plan_create(ctx.h, ctypes.byref(model), ctypes.byref(opts), len(self.dists),
                                   _ptr(self.dists), ctypes.byref(self.h))
        if rc:
            raise GrtError(rc, ctx.error())
        self.report = Report()
        lib().grt_plan_info(self.h, ctypes.byref(self.report))

    def execute(self):
        rc = lib().grt_plan_execute(self.h, ctypes.byref(self.report))
        if rc:
            raise GrtError(rc, self.ctx.error())
        return self.report

    def fetch(self, traces=True, spectra=False):
        r = self.report
        shape = (len(self.dists), r.n_cols, r.n_samples)
        t = np.empty(shape) if traces else None
        s = np.empty(shape + (2,)) if spectra else None
        rc = lib().grt_plan_fetch(self.h, _ptr(t) if traces else None, _ptr(s) if spectra else None)
        if rc:
            raise GrtError(rc, self.ctx.error())
        if spectra:
            s = s[..., 0] + 1j * s[..., 1]
        return t, s

    def write(self, path):
        """Traces to a binary file (grt_plan_write); read back with read_bin."""
        rc = lib().grt_plan_write(self.h, str(path).encode())
        if rc:
            raise GrtError(rc, self.ctx.error())

    def synth(self, m6, azimuth, stf=None):
        """Seismograms [n_dist, 3 (Z, R, T), N] for moment tensor m6 (or, for
        a single-force job, a force of 3 components) at the receivers'
        azimuths (degrees), convolved with stf (samples at dt)."""
        src = make_source(m6, stf)
        az = _arr(np.broadcast_to(azimuth, self.dists.shape))
        out = np.empty((len(self.dists), 3, self.report.n_samples))
        rc = lib().grt_plan_synth(self.h, ctypes.byref(src), _ptr(az), _ptr(out))
        if rc:
            raise GrtError(rc, self.ctx.error())
        return out

    def error_estimate(self, eps=0.0):
        """Predicted relative L2 error of each receiver's traces against the
        FP64 path (grt_plan_error_estimate; eps 0: the coefficients' noise
        measured against FP64 at spot frequencies)."""
        est = np.empty(len(self.dists))
        rc = lib().grt_plan_error_estimate(self.h, float(eps), _ptr(est))
        if rc:
            raise GrtError(rc, self.ctx.error())
        return est

    def fetch_freqs(self, freq_idx):
        """Spectra at selected frequency indices: complex [n_dist, n_cols, n_freq]."""
        fi = np.ascontiguousarray(freq_idx, dtype=np.int32)
        s = np.empty((len(self.dists), self.report.n_cols, len(fi), 2))
        rc = lib().grt_plan_fetch_freqs(self.h, len(fi), fi.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), _ptr(s))
        if rc:
            raise GrtError(rc, self.ctx.error())
        return s[..., 0] + 1j * s[..., 1]

    def close(self):
        if self.h:
            lib().grt_plan_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def grid(model, opts):
    """Layer, frequency and wavenumber grid of a job (no device work)."""
    r = Report()
    rc = lib().grt_grid(ctypes.byref(model), ctypes.byref(opts), ctypes.byref(r))
    if rc:
        raise GrtError(rc, "grt_grid (details on stderr)")
    return r.as_dict()


def sweep_kmax(model, opts, freq_idx, band_r, tol=1e-4, tol_abs=None, k_judge=None, ctx=None, env=False,
               alias=False):
    """Convergence sweep of the plain grid at selected frequencies and
    distances (grt_sweep_kmax).  Returns a dict of [n_freq, n_band] arrays:
    kmax, and tail (with k_judge), env, alias ([..., 6]) when asked."""
    fi = np.ascontiguousarray(freq_idx, dtype=np.int32)
    br = _arr(np.atleast_1d(band_r))
    shape = (len(fi), len(br))
    out = {"kmax": np.empty(shape)}
    if k_judge is not None:
        out["tail"] = np.empty(shape)
    if env:
        out["env"] = np.empty(shape)
    if alias:
        out["alias"] = np.empty(shape + (6,))
    kj = _arr(np.broadcast_to(k_judge, shape)) if k_judge is not None else None
    ta = _arr(np.broadcast_to(tol_abs, shape)) if tol_abs is not None else None
    own = ctx is None
    ctx = ctx or Context()
    opt = lambda k: _ptr(out[k]) if k in out else None
    try:
        rc = lib().grt_sweep_kmax(ctx.h, ctypes.byref(model), ctypes.byref(opts), len(fi),
                                  fi.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), len(br), _ptr(br), float(tol),
                                  _ptr(ta) if ta is not None else None, _ptr(kj) if kj is not None else None,
                                  _ptr(out["kmax"]), opt("tail"), opt("env"), opt("alias"))
        if rc:
            raise GrtError(rc, ctx.error())
    finally:
        if own:
            ctx.close()
    return out


class Batch:
    """Many jobs (model, opts, distances) executed as one CUDA graph with a
    single persistent GRT launch (grt_batch_*)."""

    def __init__(self, ctx, jobs, autotune=True, outs=None):
        """outs: optional list (per job) of float32 pinned_empty arrays of shape
        [n_dist, n_cols, N] (or None): each execute downloads the job's traces
        into its array inside the graph, beside the later jobs' work."""
        self.ctx = ctx
        self._keep = []
        self._pending = []
        arr = (Job * len(jobs))()
        self.dists = []
        for i, (model, opts, dists) in enumerate(jobs):
            d = _arr(np.atleast_1d(dists))
            self._keep += [model, opts, d]
            self.dists.append(d)
            o = None if outs is None else outs[i]
            op = None
            if o is not None:
                if o.dtype != np.float32 or not o.flags.c_contiguous or o.shape[0] != len(d):
                    raise ValueError("outs: C-contiguous float32 arrays [n_dist, n_cols, N]")
                self._keep.append(o)
                op = o.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
            arr[i] = Job(ctypes.pointer(model), ctypes.pointer(opts), len(d), _ptr(d), op)
        self.h = ctypes.c_void_p()
        rc = lib().grt_batch_create(ctx.h, len(jobs), arr, int(bool(autotune)), ctypes.byref(self.h))
        if rc:
            raise GrtError(rc, ctx.error())
        self.report = Report()

    def execute(self):
        rc = lib().grt_batch_execute(self.h, ctypes.byref(self.report))
        if rc:
            raise GrtError(rc, self.ctx.error())
        return self.report

    def launch(self):
        """execute() in three steps (grt_batch_launch, grt_batch_wait_stages,
        grt_batch_finish): start the graph."""
        rc = lib().grt_batch_launch(self.h)
        if rc:
            raise GrtError(rc, self.ctx.error())

    def wait_stages(self):
        """Block until every job's device stages are done; the last job's
        download into its out array is then still draining."""
        rc = lib().grt_batch_wait_stages(self.h)
        if rc:
            raise GrtError(rc, self.ctx.error())

    def finish(self):
        """Wait for the last download; the execution's report."""
        rc = lib().grt_batch_finish(self.h, ctypes.byref(self.report))
        if rc:
            raise GrtError(rc, self.ctx.error())
        return self.report

    def info(self, job=-1):
        r, t = Report(), Tune()
        rc = lib().grt_batch_info(self.h, int(job), ctypes.byref(r), ctypes.byref(t))
        if rc:
            raise GrtError(rc, "grt_batch_info")
        return r.as_dict(), t.as_dict()

    def fetch_f32(self, job, out=None):
        """Traces of one job as float32 [n_dist, n_cols, N], into `out` when
        given (e.g. a pinned_empty array, reused from call to call)."""
        r, _ = self.info(job)
        shape = (len(self.dists[job]), r["n_cols"], r["n_samples"])
        t = np.empty(shape, dtype=np.float32) if out is None else out
        if t.shape != shape or t.dtype != np.float32 or not t.flags.c_contiguous:
            raise ValueError(f"out must be a C-contiguous float32 array of shape {shape}")
        rc = lib().grt_batch_fetch_f32(self.h, int(job), t.ctypes.data_as(ctypes.POINTER(ctypes.c_float)))
        if rc:
            raise GrtError(rc, self.ctx.error())
        return t

    def fetch_f32_async(self, job, out):
        """Start downloading one job's float32 traces into `out` (a
        pinned_empty array of shape [n_dist, n_cols, N]); returns at once.
        `out` must not be read before wait()."""
        r, _ = self.info(job)
        shape = (len(self.dists[job]), r["n_cols"], r["n_samples"])
        if out.shape != shape or out.dtype != np.float32 or not out.flags.c_contiguous:
            raise ValueError(f"out must be a C-contiguous float32 array of shape {shape}")
        rc = lib().grt_batch_fetch_f32_async(self.h, int(job), out.ctypes.data_as(ctypes.POINTER(ctypes.c_float)))
        if rc:
            raise GrtError(rc, self.ctx.error())
        self._pending.append(out)
        return out

    def wait(self):
        """Wait for the downloads fetch_f32_async started."""
        rc = lib().grt_batch_wait(self.h)
        self._pending = []
        if rc:
            raise GrtError(rc, self.ctx.error())

    def fetch(self, job, traces=True, spectra=False):
        r, _ = self.info(job)
        shape = (len(self.dists[job]), r["n_cols"], r["n_samples"])
        t = np.empty(shape) if traces else None
        s = np.empty(shape + (2,)) if spectra else None
        rc = lib().grt_batch_fetch(self.h, int(job), _ptr(t) if traces else None, _ptr(s) if spectra else None)
        if rc:
            raise GrtError(rc, self.ctx.error())
        if spectra:
            s = s[..., 0] + 1j * s[..., 1]
        return t, s

    def synth(self, job, m6, azimuth, stf=None):
        """Seismograms of one job [n_dist, 3 (Z, R, T), N]."""
        r, _ = self.info(job)
        src = make_source(m6, stf)
        az = _arr(np.broadcast_to(azimuth, self.dists[job].shape))
        out = np.empty((len(self.dists[job]), 3, r["n_samples"]))
        rc = lib().grt_batch_synth(self.h, int(job), ctypes.byref(src), _ptr(az), _ptr(out))
        if rc:
            raise GrtError(rc, self.ctx.error())
        return out

    def error_estimate(self, job, eps=0.0):
        """grt_batch_error_estimate: predicted per-receiver error of a job's traces."""
        est = np.empty(len(self.dists[job]))
        rc = lib().grt_batch_error_estimate(self.h, int(job), float(eps), _ptr(est))
        if rc:
            raise GrtError(rc, self.ctx.error())
        return est

    def fetch_freqs(self, job, freq_idx):
        r, _ = self.info(job)
        fi = np.ascontiguousarray(freq_idx, dtype=np.int32)
        s = np.empty((len(self.dists[job]), r["n_cols"], len(fi), 2))
        rc = lib().grt_batch_fetch_freqs(self.h, int(job), len(fi), fi.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                         _ptr(s))
        if rc:
            raise GrtError(rc, self.ctx.error())
        return s[..., 0] + 1j * s[..., 1]

    def close(self):
        if self.h:
            lib().grt_batch_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def run(model, opts, dists, ctx=None, spectra=False):
    """Green's functions for one model at all distances.

    Returns (traces [n_dist, n_cols, N], spectra or None, report dict)."""
    own = ctx is None
    ctx = ctx or Context()
    try:
        p = Plan(ctx, model, opts, dists)
        p.execute()
        t, s = p.fetch(True, spectra)
        rep = p.report.as_dict()
        p.close()
        return t, s, rep
    finally:
        if own:
            ctx.close()


def with_precision(opts, precision):
    """A copy of opts at another working precision (arrays shared)."""
    o = Opts.from_buffer_copy(opts)
    o.precision = int(precision)
    o._keep = getattr(opts, "_keep", [])
    return o


# The judge's margin.  Over the 63 359 traces of the 256-model uneven set, a
# receiver recomputed in FP64 when m times its estimate exceeds 1e-3 left
# 179 traces above 1e-3 at m = 1, 16 at m = 1.5 and none from m = 2; 3 keeps
# a factor 1.5 beyond that.
JUDGE_SAFETY = 3.0


def run_judged(model, opts, dists, ctx=None, tol=1e-3, eps=0.0, safety=JUDGE_SAFETY):
    """FP32 traces, judged: every receiver whose predicted error against FP64
    (grt_plan_error_estimate) exceeds tol / safety is recomputed by the FP64
    path.

    Returns (traces [n_dist, n_cols, N], info) with info["est"] the predicted
    errors, info["fp64"] the receivers recomputed."""
    own = ctx is None
    ctx = ctx or Context()
    try:
        d = _arr(np.atleast_1d(dists))
        p = Plan(ctx, model, with_precision(opts, FP32), d)
        p.execute()
        t, _ = p.fetch(True, False)
        est = p.error_estimate(eps)
        p.close()
        bad = np.nonzero(est * safety > tol)[0]
        if bad.size:
            t64, _, _ = run(model, with_precision(opts, FP64), d[bad], ctx)
            t[bad] = t64
        return t, {"est": est, "fp64": bad}
    finally:
        if own:
            ctx.close()


def run_noalloc(model, opts, dists, device=0):
    """grt_run_noalloc: the same traces as run() for small FP32 jobs, with no
    device allocation (library-owned scratch; see the C header).  The C call
    writes 15 columns for a single force and 20 for a moment tensor (it
    refuses the corrected 30-column layout), so the output is sized from the
    source type."""
    d = _arr(np.atleast_1d(dists))
    n_cols = 15 if model.src_type == 0 else 20
    out = np.empty((len(d), n_cols, 1 << opts.log2n))
    rc = lib().grt_run_noalloc(int(device), ctypes.byref(model), ctypes.byref(opts), len(d), _ptr(d), _ptr(out))
    if rc:
        raise GrtError(rc, "grt_run_noalloc (details on stderr)")
    return out


def green(iname, oname_w, oname_t):
    """The reference's entry point: input file in, two text files out."""
    rc = lib().grt_green(str(iname).encode(), str(oname_w).encode(), str(oname_t).encode())
    if rc:
        raise GrtError(rc, f"green({iname})")


def read_bin(path):
    """A file written by grt_plan_write: dict with dt, t0, sigma, dist and
    traces float32 [n_dist, n_cols, N]."""
    with open(path, "rb") as f:
        b = f.read()
    if b[:8] != b"GRTMBIN1":
        raise ValueError(f"{path}: not a GRTMBIN1 file")
    ver, nd, nc, n = np.frombuffer(b, "<i4", 4, 8)
    if ver != 1:
        raise ValueError(f"{path}: version {ver}")
    dt, t0, sigma = np.frombuffer(b, "<f8", 3, 24)
    dist = np.frombuffer(b, "<f8", nd, 48).copy()
    o = 48 + 8 * nd
    tr = np.frombuffer(b, "<f4", nd * nc * n, o).reshape(nd, nc, n).copy()
    if o + 4 * tr.size != len(b):
        raise ValueError(f"{path}: size mismatch")
    return {"dt": float(dt), "t0": float(t0), "sigma": float(sigma), "dist": dist, "traces": tr}


def read_table(path, complex_pairs=False):
    """Read a file written by green() (rows of comma-terminated fields)."""
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
