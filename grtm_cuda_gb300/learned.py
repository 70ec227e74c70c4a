"""Learned wavenumber sampling.

The plain method integrates every frequency over a fixed wavenumber grid
(k_j = j dk, j < nk, dk = 2 pi / L with the reference's aperture rule
green.cu:2072-2077).  Most of that grid is wasted: at low frequencies the
integrand has died out long before the top of the grid, and the step is often
finer than the receivers' distances need.  A small network, trained on
convergence sweeps that the plain method runs on the GPU, predicts for each
(model, frequency, distance) the cutoff k_max and the step dk; the GRT kernel
then evaluates a ragged grid of nk(w) = k_max(w)/dk points (grid mode
K_CUSTOM).

Network: 15 inputs (12 layer statistics of the model, log w, log r, log zs),
three hidden layers of 64 SiLU units, 2 outputs (log k_max, log2 of the step
multiple dk / dk_plain), trained and evaluated by the library's own CUDA
kernels (grt_mlp_*).  Inputs and targets are standardised with statistics
stored beside the weights.

The plain fixed grid is both fallback and judge of every prediction: before
its result is used, the integrand tail beyond the predicted k_max is measured
on the plain grid at a few spot frequencies and distances, and the spectra of
every receiver at the spot frequencies (which carry any aliasing of a coarser
step at that receiver's distance) are compared with the plain grid's.  A
receiver that fails is recomputed on the plain grid.

No counterpart in the reference.
"""
import ctypes
import math
import os
import struct
import threading
import time
import weakref

import numpy as np

from . import FIX_ALL, K_FIXED, Context, GrtError, Plan, grid, lib, make_model, make_opts, sweep_kmax, synth

HERE = os.path.dirname(os.path.abspath(__file__))
WEIGHTS = os.path.join(HERE, "data", "ksampler.bin")
N_FEAT, N_IN, N_OUT = 12, 15, 2
MAGIC = b"GRTKSMP1"      # one k margin for every frequency
MAGIC2 = b"GRTKSMP2"     # k margins per band of log w

# the plain grid the sampler is trained against and judged by.  Synthetic
# models run with the reference's receiver-layer and d/dz quirks corrected
# (FIX_ALL, the 20-column layout of the tensor-core sums): with its
# receiver-layer search (green.cu:2092-2101) a surface receiver whose source
# sits deeper in its layer than the top layer is thick lands at a negative
# depth in a deeper layer, and the field grows like e^{nu |z|} (overflow).
PLAIN = dict(dt=0.05, log2n=13, nk=32768, sigma_factor=math.pi, taper=0.3, t0=0.0, fix=FIX_ALL)


def plain_opts(plain=PLAIN, **over):
    """Options of the plain fixed grid (keyword overrides, e.g. precision)."""
    kw = dict(t0=plain["t0"], taper=plain["taper"], sigma_factor=plain["sigma_factor"], k_mode=K_FIXED,
              nk_fixed=plain["nk"], fix=plain["fix"])
    kw.update(over)
    return make_opts(plain["dt"], plain["log2n"], **kw)


def custom_opts(nk, dk, plain=PLAIN, **over):
    """Options of a ragged grid nk[w] with step dk, otherwise as the plain grid."""
    kw = dict(t0=plain["t0"], taper=plain["taper"], sigma_factor=plain["sigma_factor"], dk=dk, nk_custom=nk,
              fix=plain["fix"])
    kw.update(over)
    return make_opts(plain["dt"], plain["log2n"], **kw)


def spot_opts(nw, dk, spots, k_slice, plain=PLAIN):
    """The plain grid (step dk) at the judge's spot frequencies alone: a
    spectra-only plan whose frequency tiles hold nothing but spots.  With the
    learned plan's k_slice both add a frequency's wavenumbers in the same
    order, so their difference is the learned grid's own error and not the
    FP32 rounding of two differently split sums."""
    return custom_opts(np.full(nw, plain["nk"], np.int32), dk, plain, freq_sel=np.asarray(spots, np.int32),
                       k_slice=int(k_slice))


def layer_features(m):
    """12 statistics of a layered model (dict as from synth): depth of the
    half-space, min/max Vs, max Vp, thickness-weighted mean Vs, Vs of the
    source and receiver layers, min Vs between them, layer count, thinnest
    layer, mean Qs, thickness of the source layer -- all as logs."""
    tops = np.asarray(m["ztop"], dtype=np.float64)
    vp, vs, qs = (np.asarray(m[k], dtype=np.float64) for k in ("vp", "vs", "qs"))
    h = np.diff(tops)
    s = int(np.searchsorted(tops, m["hs"], side="right") - 1)
    r = int(np.searchsorted(tops, m.get("hr", 0.0), side="right") - 1)
    lo, hi = min(s, r), max(s, r)
    hsrc = h[s] if s < len(h) else 10.0
    f = [tops[-1], vs.min(), vs.max(), vp.max(), float(np.sum(h * vs[:-1]) / max(np.sum(h), 1e-9)), vs[s], vs[r],
         vs[lo:hi + 1].min(), float(len(vs)), h.min() if len(h) else 1.0, qs.mean(), hsrc]
    return np.log(np.maximum(np.asarray(f, dtype=np.float64), 1e-6))


def net_inputs(feat, omega, r, zs):
    """Rows of the 15 network inputs for frequencies omega (rad/s) and
    distances r (km), broadcast together."""
    omega, r = np.broadcast_arrays(np.atleast_1d(omega).astype(np.float64), np.atleast_1d(r).astype(np.float64))
    n = omega.size
    x = np.empty((n, N_IN), dtype=np.float64)
    x[:, :N_FEAT] = feat
    x[:, 12] = np.log(omega.ravel())
    x[:, 13] = np.log(r.ravel())
    x[:, 14] = math.log(zs + 0.1)
    return x


class Mlp:
    """The network on the GPU (grt_mlp_*): forward, loss gradient, Adam."""

    def __init__(self, ctx, n_in=N_IN, n_out=N_OUT, seed=1):
        self.ctx, self.n_in, self.n_out = ctx, n_in, n_out
        self.h = ctypes.c_void_p()
        rc = lib().grt_mlp_create(ctx.h, n_in, n_out, seed, ctypes.byref(self.h))
        if rc:
            raise GrtError(rc, ctx.error())
        self.n_params = lib().grt_mlp_n_params(self.h)

    @staticmethod
    def _f(a, cols):
        a = np.ascontiguousarray(a, dtype=np.float32)
        assert a.ndim == 2 and a.shape[1] == cols
        return a

    @staticmethod
    def _fp(a):
        return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))

    def _check(self, rc):
        if rc:
            raise GrtError(rc, self.ctx.error())

    def get_params(self):
        p = np.empty(self.n_params, dtype=np.float32)
        self._check(lib().grt_mlp_get_params(self.h, self._fp(p)))
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.size == self.n_params
        self._check(lib().grt_mlp_set_params(self.h, self._fp(p)))

    def forward(self, x):
        x = self._f(x, self.n_in)
        y = np.empty((x.shape[0], self.n_out), dtype=np.float32)
        self._check(lib().grt_mlp_forward(self.h, x.shape[0], self._fp(x), self._fp(y)))
        return y

    def loss_grad(self, x, t):
        x, t = self._f(x, self.n_in), self._f(t, self.n_out)
        loss = ctypes.c_float()
        g = np.empty(self.n_params, dtype=np.float32)
        self._check(lib().grt_mlp_loss_grad(self.h, x.shape[0], self._fp(x), self._fp(t), ctypes.byref(loss),
                                            self._fp(g)))
        return loss.value, g

    def train(self, x, t, epochs, batch=256, lr=1e-3, seed=1):
        x, t = self._f(x, self.n_in), self._f(t, self.n_out)
        loss = ctypes.c_float()
        self._check(lib().grt_mlp_train(self.h, x.shape[0], self._fp(x), self._fp(t), int(epochs), int(batch),
                                        float(lr), int(seed), ctypes.byref(loss)))
        return loss.value

    def close(self):
        if self.h:
            lib().grt_mlp_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------- training data
def taper_weight(iw, nw, taper):
    """The cosine taper the spectral stage applies at frequency index iw
    (green.cu:1909-1921)."""
    iw = np.asarray(iw, np.float64)
    wc = int(nw * (1 - taper))
    w = 0.5 * (1 + np.cos((iw - wc + 1) * math.pi / (nw - wc + 1)))
    return np.where(iw > wc, w, 1.0)


def sweep_targets(ctx, model, opts, fi, br, tol, nw, taper):
    """Targets of the sampler at frequencies fi and distances br.

    The cutoff k_c(w, r) keeps the envelope tail beyond it below tol times
    the envelope's peak over the sampled frequencies at that distance,
    relative to the taper weight of w (a frequency the taper removes needs
    no integral); the step multiple 2^s(w, r) is the coarsest whose
    aliasing error stays below tol times that frequency's own k-sum
    magnitude (aliasing is not averaged away across frequencies: it shifts
    energy in time).  Two sweeps: totals and aliasing, then the cutoffs at
    those absolute thresholds."""
    s1 = sweep_kmax(model, opts, fi, br, tol, ctx=ctx, env=True, alias=True)
    w = np.maximum(taper_weight(fi, nw, taper), 1e-6)[:, None]
    thr = tol * s1["env"].max(0)[None, :] / w
    kmax = sweep_kmax(model, opts, fi, br, tol, tol_abs=thr, ctx=ctx)["kmax"]
    al = s1["alias"]
    ok = al[..., 1:] <= tol * al[..., :1]                       # [f, b, 5]
    # coarsest s with every finer stride passing too
    l2 = np.cumprod(ok, axis=2).sum(axis=2)
    return kmax, l2, s1


def sweep_dataset(ctx, seeds, n_freq=8, n_band=8, tol=1e-4, plain=PLAIN, rng_seed=0, n_layers=40):
    """Convergence sweeps of the plain grid on seeded crustal models
    (n_layers layers, source depth U(1, 30) km), n_freq frequencies (log-
    uniform) x n_band distances (log-uniform in 1-500 km) per model.
    Returns inputs [n, 15] and targets [n, 2] = (log k_max, log2(dk/dk_plain))."""
    rng = np.random.default_rng(rng_seed)
    X, Y = [], []
    for seed in seeds:
        m = synth.crust(np.random.default_rng(seed), n_layers, rng.uniform(1.0, 30.0))
        model = make_model(**m)
        opts = plain_opts(plain)
        gr = grid(model, opts)
        nw, dkp, df = gr["nw"], gr["dk"], gr["df"]
        fi = np.unique(np.round(np.exp(rng.uniform(0.0, math.log(nw - 1), 4 * n_freq))).astype(np.int64))
        fi = np.sort(rng.choice(fi, size=min(n_freq, len(fi)), replace=False))
        br = np.exp(rng.uniform(math.log(1.0), math.log(500.0), n_band))
        kmax, l2, _ = sweep_targets(ctx, model, opts, fi, br, tol, nw, plain["taper"])
        feat = layer_features(m)
        om = (2 * math.pi * df * fi)[:, None] * np.ones((1, n_band))
        rr = np.ones((len(fi), 1)) * br[None, :]
        X.append(net_inputs(feat, om.ravel(), rr.ravel(), m["hs"]))
        Y.append(np.stack([np.log(np.maximum(kmax.ravel(), 4 * dkp)), l2.ravel().astype(np.float64)], axis=1))
    return np.concatenate(X), np.concatenate(Y)


# ---------------------------------------------------------------- the sampler
class Sampler:
    """Trained network parameters with their input/output standardisation
    and the safety margins measured on held-out sweeps.

    The k_max margin is either one factor (margin_k) or, when kbands is set,
    a factor per band of log w: kbands = (edges [nb + 1], margins [nb]),
    frequencies below the first edge or above the last take the end bands.
    The network's relative error differs with frequency (at low frequencies
    k_max is a few grid steps and its log is coarse); one margin sized by the
    worst band lifts every high frequency to the top of the plain grid."""

    def __init__(self, params, x_mean, x_std, y_mean, y_std, margin_k=1.25, margin_d=1.0, tol=1e-4, kbands=None):
        self.params = np.ascontiguousarray(params, dtype=np.float32)
        self.x_mean, self.x_std = np.asarray(x_mean, np.float64), np.asarray(x_std, np.float64)
        self.y_mean, self.y_std = np.asarray(y_mean, np.float64), np.asarray(y_std, np.float64)
        self.margin_k, self.margin_d, self.tol = float(margin_k), float(margin_d), float(tol)
        self.kbands = None
        if kbands is not None:
            e, mg = (np.asarray(a, np.float64) for a in kbands)
            if e.ndim != 1 or mg.shape != (e.size - 1,) or e.size < 2 or np.any(np.diff(e) <= 0):
                raise ValueError("kbands: edges [nb + 1] ascending and margins [nb]")
            self.kbands = (e, mg)
        self._nets = {}

    def k_margin(self, log_w):
        """The k_max margin at log angular frequencies log_w."""
        log_w = np.asarray(log_w, np.float64)
        if self.kbands is None:
            return np.full(log_w.shape, self.margin_k)
        e, mg = self.kbands
        return mg[np.clip(np.searchsorted(e, log_w, side="right") - 1, 0, mg.size - 1)]

    # tiny binary file: magic, n_in, n_out, n_params (int32), margins and tol
    # (float64), [MAGIC2: the band count (int32), edges and margins (float64)],
    # then standardisation (float64) and parameters (float32)
    def save(self, path):
        os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
        with open(path, "wb") as f:
            f.write(MAGIC if self.kbands is None else MAGIC2)
            f.write(struct.pack("<3i", N_IN, N_OUT, self.params.size))
            f.write(struct.pack("<3d", self.margin_k, self.margin_d, self.tol))
            if self.kbands is not None:
                e, mg = self.kbands
                f.write(struct.pack("<i", mg.size))
                f.write(np.asarray(e, "<f8").tobytes())
                f.write(np.asarray(mg, "<f8").tobytes())
            for a in (self.x_mean, self.x_std, self.y_mean, self.y_std):
                f.write(np.asarray(a, "<f8").tobytes())
            f.write(self.params.astype("<f4").tobytes())

    @classmethod
    def load(cls, path=WEIGHTS):
        with open(path, "rb") as f:
            b = f.read()
        if b[:8] not in (MAGIC, MAGIC2):
            raise ValueError(f"{path}: not a sampler file")
        n_in, n_out, n_p = struct.unpack_from("<3i", b, 8)
        if (n_in, n_out) != (N_IN, N_OUT):
            raise ValueError(f"{path}: network {n_in}->{n_out}, expected {N_IN}->{N_OUT}")
        mk, md, tol = struct.unpack_from("<3d", b, 20)
        o = 44
        kb = None
        if b[:8] == MAGIC2:
            nb, = struct.unpack_from("<i", b, o)
            o += 4
            if not 0 < nb < 1024:
                raise ValueError(f"{path}: bad band count {nb}")
            e = np.frombuffer(b, "<f8", nb + 1, o).copy()
            o += 8 * (nb + 1)
            mg = np.frombuffer(b, "<f8", nb, o).copy()
            o += 8 * nb
            kb = (e, mg)
        arrs = []
        for n in (n_in, n_in, n_out, n_out):
            arrs.append(np.frombuffer(b, "<f8", n, o).copy())
            o += 8 * n
        p = np.frombuffer(b, "<f4", n_p, o).copy()
        if o + 4 * n_p != len(b):
            raise ValueError(f"{path}: size mismatch")
        return cls(p, *arrs, margin_k=mk, margin_d=md, tol=tol, kbands=kb)

    def net(self, ctx):
        """The network on ctx's device, one per context (kept while the
        context lives: building one allocates and uploads the weights, and
        freeing one waits for the whole device)."""
        for k in [k for k, (r, _) in self._nets.items() if r() is None or not r().h]:
            self._nets.pop(k)[1].close()
        e = self._nets.get(id(ctx))
        if e is None or e[0]() is not ctx:
            net = Mlp(ctx)
            net.set_params(self.params)
            self._nets[id(ctx)] = (weakref.ref(ctx), net)
            return net
        return e[1]

    def predict(self, ctx, x):
        """Un-standardised outputs (log k_max, log2 step multiple) for raw inputs."""
        z = (np.asarray(x, np.float64) - self.x_mean) / self.x_std
        y = self.net(ctx).forward(z.astype(np.float32)).astype(np.float64)
        return y * self.y_std + self.y_mean

    @staticmethod
    def train_new(ctx, X, Y, epochs=(200, 100, 100), lrs=(2e-3, 5e-4, 1e-4), batch=256, seed=1, val=None):
        """Fit a fresh network with the library's CUDA kernels.  Returns the
        sampler and the loss history [(epochs, lr, train loss, val loss)]."""
        xm, xs = X.mean(0), X.std(0) + 1e-9
        ym, ys = Y.mean(0), Y.std(0) + 1e-9
        net = Mlp(ctx, seed=seed)
        zx, zy = ((X - xm) / xs).astype(np.float32), ((Y - ym) / ys).astype(np.float32)
        hist = []
        for i, (ep, lr) in enumerate(zip(epochs, lrs)):
            tl = net.train(zx, zy, ep, batch, lr, seed + i)
            vl = None
            if val is not None:
                vl, _ = net.loss_grad(((val[0] - xm) / xs).astype(np.float32), ((val[1] - ym) / ys).astype(np.float32))
            hist.append((ep, lr, tl, vl))
        s = Sampler(net.get_params(), xm, xs, ym, ys)
        net.close()
        return s, hist

    def calibrate(self, ctx, X, Y, q_k=0.995, q_d=0.95, n_bands=0, min_per_band=256):
        """Margins from held-out sweeps: k_max is scaled by the q_k-quantile of
        the under-prediction ratio; the step multiple is lowered by the
        q_d-quantile of its over-prediction (the judge catches the rest).
        n_bands > 0: one k margin per band of log w, the bands holding equal
        numbers of sweeps (at least min_per_band each), the outer edges open."""
        y = self.predict(ctx, X)
        under_k = np.exp(Y[:, 0] - y[:, 0])            # > 1 where the net predicts too small
        self.margin_k = float(max(1.0, np.quantile(under_k, q_k)))
        over_d = 2.0 ** (y[:, 1] - Y[:, 1])            # > 1 where the net predicts too coarse
        self.margin_d = float(max(1.0, np.quantile(over_d, q_d)))
        self.kbands = None
        nb = min(int(n_bands), len(X) // max(1, int(min_per_band)))
        if nb >= 2:
            lw = X[:, 12]
            e = np.quantile(lw, np.linspace(0.0, 1.0, nb + 1))
            e[0], e[-1] = lw.min() - 1.0, lw.max() + 1.0
            e = np.unique(e)
            band = np.clip(np.searchsorted(e, lw, side="right") - 1, 0, e.size - 2)
            mg = np.array([max(1.0, np.quantile(under_k[band == i], q_k)) if np.any(band == i) else self.margin_k
                           for i in range(e.size - 1)])
            self.kbands = (e, mg)
        return self.margin_k, self.margin_d

    # ------------------------------------------------------------ inference
    def grid(self, ctx, m, dists, plain=PLAIN, tile=64, use_stride=True):
        """Learned ragged grid for one model and receiver set: (nk[nw],
        stride[nw], kmax[nw], plain grid report).  Frequency iw takes
        nk[iw] points k_j = j stride[iw] dk_plain.  k_max per frequency is
        the prediction at the nearest receiver (the cutoff falls with
        distance); the stride the finest prediction at the farthest receiver
        over each aligned tile of `tile` frequencies (the tensor-core sum
        multiplies a tile by one Bessel operand), floored to a power of two."""
        model = make_model(**m)
        gr = grid(model, plain_opts(plain))
        nk_plain = plain["nk"]
        nw, dkp, df = gr["nw"], gr["dk"], gr["df"]
        om = 2 * math.pi * df * np.maximum(np.arange(nw), 1)
        d = np.asarray(dists, np.float64)
        feat = layer_features(m)
        y = self.predict(ctx, np.concatenate([net_inputs(feat, om, d.min(), m["hs"]),
                                              net_inputs(feat, om, d.max(), m["hs"])]))
        kmax = np.minimum(np.exp(y[:nw, 0]) * self.k_margin(np.log(om)), (nk_plain - 1) * dkp)
        # one octave below the prediction (aliasing errors do not average out over frequencies)
        l2 = np.clip(y[nw:, 1] - math.log2(self.margin_d) - 1.0, 0.0, 5.0) if use_stride else np.zeros(nw)
        nt = (nw + tile - 1) // tile
        l2t = np.full(nt * tile, np.inf)
        l2t[:nw] = l2
        l2t = np.floor(l2t.reshape(nt, tile).min(1))
        stride = np.repeat((2 ** l2t).astype(np.int64), tile)[:nw]
        nk_top = (nk_plain - 1) // stride + 1                 # stay inside the plain grid
        nk = np.clip(np.ceil(kmax / (dkp * stride)).astype(np.int64) + 2, 8, nk_top)
        return nk.astype(np.int32), stride.astype(np.int32), (nk - 1) * stride * dkp, gr


def spot_frequencies(nw):
    """Judge frequencies: log-spaced from the lowest bin, then spread over
    the band (indices >= 1)."""
    f = np.array([1, 2, 4, 8, 16, 32]) * max(1, nw // 4096)
    f = np.concatenate([f, np.round(np.array([0.02, 0.05, 0.12, 0.25, 0.45, 0.65, 0.85]) * nw)])
    return np.unique(np.clip(f.astype(np.int64), 1, nw - 1))


def judge_spots(nw, stride, tile=64):
    """Spot frequencies of the judge: the fixed spread, plus the middle
    frequency of every tile that uses a coarser step (its aliasing shows
    there)."""
    extra = [t * tile + tile // 2 for t in range((nw + tile - 1) // tile) if stride[min(nw - 1, t * tile)] > 1]
    return np.unique(np.clip(np.concatenate([spot_frequencies(nw), np.asarray(extra, np.int64)]), 1, nw - 1))


def spectral_verdict(s_learn, s_plain, tol, floor=0.05):
    """Per receiver: the worst spot frequency's error ||dS(w)|| / ||S(w)||
    over the columns, with ||S(w)|| floored at `floor` times the receiver's
    largest spot level (a frequency with next to no energy cannot fail it).
    Returns (error per receiver, rejected mask)."""
    num = np.sqrt(np.sum(np.abs(s_learn - s_plain) ** 2, axis=1))          # [receiver, spot]
    lev = np.sqrt(np.sum(np.abs(s_plain) ** 2, axis=1))
    den = np.maximum(lev, floor * lev.max(axis=1, keepdims=True)) + 1e-300
    err = (num / den).max(axis=1)
    return err, ~(err <= tol)


def run_learned(sampler, m, dists, ctx=None, plain=PLAIN, tail_tol=None, spec_tol=3e-3, judge=True, use_stride=True):
    """Traces of one model on the learned grid, judged against the plain grid.

    Returns (traces [n_dist, n_cols, N], info).  info: learned and plain (w,k)
    counts, step multiple, the judge's tail and spectral figures, the
    receivers recomputed on the plain grid and the wall time of each part."""
    own = ctx is None
    ctx = ctx or Context()
    try:
        t_start = time.perf_counter()
        dists = np.asarray(dists, np.float64)
        nk_plain = plain["nk"]
        nk, stride, kmax, gr = sampler.grid(ctx, m, dists, plain, use_stride=use_stride)
        nw, dkp = gr["nw"], gr["dk"]
        t_pred = time.perf_counter()
        model = make_model(**m)
        plan = Plan(ctx, model, custom_opts(nk, dkp, plain, k_stride=stride), dists)
        plan.execute()
        traces, _ = plan.fetch(True, False)
        info = dict(nkw_learned=int(nk.sum()), nkw_plain=int(nw) * int(nk_plain),
                    stride_mean=float(np.mean(stride)), ms_learned_gpu=plan.report.ms_total, fallback=[],
                    tail_max=0.0, spec_err_max=0.0)
        t_run = time.perf_counter()
        if judge:
            spot = judge_spots(nw, stride)
            popts = plain_opts(plain)
            bands = np.unique(np.array([dists.min(), math.sqrt(dists.min() * dists.max()), dists.max()]))
            tol = sampler.tol if tail_tol is None else tail_tol
            sw = sweep_kmax(model, popts, spot, bands, sampler.tol,
                            k_judge=np.repeat(kmax[spot][:, None], len(bands), 1), ctx=ctx, env=True)
            # the tail beyond the prediction, against the threshold the
            # targets were made with (peak envelope over the spot frequencies)
            w = np.maximum(taper_weight(spot, nw, plain["taper"]), 1e-6)[:, None]
            excess = sw["tail"] * sw["env"] * w / (tol * sw["env"].max(0)[None, :])
            info["tail_max"] = float(excess.max())
            tail_bad = excess.max(0) > 10.0                                         # per band
            # plain grid at the spot frequencies only (a spectra-only plan)
            sp_plan = Plan(ctx, model, spot_opts(nw, dkp, spot, plan.report.k_slice, plain), dists)
            sp_plan.execute()
            s_plain = sp_plan.fetch_freqs(spot)
            s_learn = plan.fetch_freqs(spot)
            sp_plan.close()
            err, bad = spectral_verdict(s_learn, s_plain, spec_tol)
            info["spec_err_max"] = float(err.max())
            # the cutoff falls with distance: a band's tail verdict covers the
            # receivers beyond it (the step is judged by the spectra above,
            # at each receiver's own distance)
            below = np.clip(np.searchsorted(bands, dists * (1 + 1e-12), side="right") - 1, 0, len(bands) - 1)
            bad |= tail_bad[below]
            if bad.any():
                idx = np.nonzero(bad)[0]
                pplan = Plan(ctx, model, popts, dists[idx])
                pplan.execute()
                traces[idx], _ = pplan.fetch(True, False)
                pplan.close()
                info["fallback"] = idx.tolist()
        plan.close()
        t_end = time.perf_counter()
        info.update(s_predict=t_pred - t_start, s_learned=t_run - t_pred, s_judge=t_end - t_run,
                    s_total=t_end - t_start)
        return traces, info
    finally:
        if own:
            ctx.close()


_JUDGE_CTX = {}


def judge_context(ctx):
    """A second context on ctx's device for the judge's work, kept for the
    process (its cached memory serves every later judge).  Its streams have
    the greatest priority: the judge's small kernels (its plans' set-up, the
    spot sums, the sweeps) are scheduled ahead of the batch graph's pending
    blocks instead of after each of its long kernels."""
    dev = getattr(ctx, "device", 0)
    jc = _JUDGE_CTX.get(dev)
    if jc is None or not jc.h:
        jc = Context(dev)
        jc.set_priority(True)
        _JUDGE_CTX[dev] = jc
    return jc


class _LearnedBatch:
    """One learned batch in stages: prepare (prediction, the batch and its
    judge's spot jobs), start (the batch's graph in a host thread), judge_pre
    (the judge's work that does not need the batch: the plain grid at the
    spot frequencies and the tail sweeps, on the judge's context), join
    (the graph done) and finish (the comparison, fallbacks, the info).
    run_learned_batch runs them back to back; run_learned_stream interleaves
    consecutive batches."""

    def __init__(self, sampler, models, dists_list, ctx, plain, spec_tol, autotune, use_stride, out):
        from . import Batch
        self.sampler, self.plain, self.spec_tol, self.out = sampler, plain, spec_tol, out
        self.ctx, self.dists_list = ctx, dists_list
        self.t = [time.perf_counter()]
        self.grids = [sampler.grid(ctx, m, d, plain, use_stride=use_stride) for m, d in zip(models, dists_list)]
        self.t.append(time.perf_counter())
        self.mods = [make_model(**m) for m in models]
        jobs = [(mo, custom_opts(nk, gr["dk"], plain, k_stride=st), d)
                for mo, (nk, st, _, gr), d in zip(self.mods, self.grids, dists_list)]
        # with page-locked destinations the graph itself downloads each model's
        # traces as soon as its stages finish, beside the next model's sums
        # (downloads started after the graph held up the judge's own small
        # copies behind them on the copy engine: 20 -> 83 ms of judge)
        self.b = Batch(ctx, jobs, autotune=autotune, outs=out)
        self.t.append(time.perf_counter())
        self.spots = [judge_spots(gr["nw"], st) for (nk, st, kmax, gr) in self.grids]
        self.spot_jobs = [(mo, spot_opts(gr["nw"], gr["dk"], sp, self.b.info(j)[0]["k_slice"], plain), d)
                          for j, (mo, (nk, st, kmax, gr), d, sp) in
                          enumerate(zip(self.mods, self.grids, dists_list, self.spots))]
        self.done, self.runner, self.pre = {}, None, None
        self.t_sw = self.t_ff = 0.0
        self.n_judge_launches = 0

    def _execute(self):
        # the batch's execute in its three steps; `staged` is set once the
        # device stages are done (the last model's download then drains
        # beside whatever the caller starts next), or when a step failed
        try:
            self.b.launch()
            self.b.wait_stages()
            self.done["t_staged"] = time.perf_counter()
            self.staged.set()
            self.done["rep"] = self.b.finish()
        except BaseException as e:   # re-raised on the calling thread
            self.done["exc"] = e
        finally:
            self.staged.set()
        self.done["t"] = time.perf_counter()

    def wait_stages(self):
        """Block until the batch's device stages are done (its graph thread
        may still be waiting for the last download)."""
        self.staged.wait()
        if "exc" in self.done:
            self.join()

    def start(self, threaded=True):
        self.t_start = time.perf_counter()
        self.staged = threading.Event()
        if threaded:
            self.runner = threading.Thread(target=self._execute)
            self.runner.start()
        else:
            self._execute()

    def judge_pre(self, jctx):
        """The judge's part that does not need the batch's spectra."""
        self.tj = [time.perf_counter()]
        from . import Batch
        sb = Batch(jctx, self.spot_jobs, autotune=False)
        self.tj.append(time.perf_counter())
        self.n_judge_launches = sb.execute().kernel_launches
        self.tj.append(time.perf_counter())
        pre = []
        try:
            for j, (mo, (nk, st, kmax, gr), d) in enumerate(zip(self.mods, self.grids, self.dists_list)):
                d = np.asarray(d, np.float64)
                sp = self.spots[j]
                bands = np.unique(np.array([d.min(), math.sqrt(d.min() * d.max()), d.max()]))
                t_a = time.perf_counter()
                sw = sweep_kmax(mo, plain_opts(self.plain), sp, bands, self.sampler.tol,
                                k_judge=np.repeat(kmax[sp][:, None], len(bands), 1), ctx=jctx, env=True)
                t_b = time.perf_counter()
                w = np.maximum(taper_weight(sp, gr["nw"], self.plain["taper"]), 1e-6)[:, None]
                excess = sw["tail"] * sw["env"] * w / (self.sampler.tol * sw["env"].max(0)[None, :])
                s_plain = sb.fetch_freqs(j, sp)
                self.t_sw += t_b - t_a
                self.t_ff += time.perf_counter() - t_b
                pre.append((d, bands, excess, s_plain))
        finally:
            sb.close()
        self.pre = pre
        self.t_pre = time.perf_counter()

    def join(self):
        """Wait for the graph's thread (always, before anything of the batch's
        context may be used again); re-raise its error."""
        if self.runner is not None:
            self.runner.join()
            self.runner = None
        if "exc" in self.done:
            raise self.done["exc"]
        self.t_exec = self.done["t"]

    def finish(self, overlap):
        b, ctx = self.b, self.ctx
        t = self.t
        rep = self.done["rep"]
        traces = list(self.out) if self.out is not None else [b.fetch_f32(j) for j in range(len(self.mods))]
        t.append(time.perf_counter())
        # judge, the part that needs the batch: each receiver's spectra at the
        # spot frequencies against the plain grid's
        t_c = time.perf_counter()
        n_fb = 0
        fallback = []
        for j, (d, bands, excess, s_plain) in enumerate(self.pre):
            sp = self.spots[j]
            t_a = time.perf_counter()
            s_learn = b.fetch_freqs(j, sp)
            self.t_ff += time.perf_counter() - t_a
            _, bad = spectral_verdict(s_learn, s_plain, self.spec_tol)
            below = np.clip(np.searchsorted(bands, d * (1 + 1e-12), side="right") - 1, 0, len(bands) - 1)
            bad |= (excess.max(0) > 10.0)[below]
            fallback.append(np.nonzero(bad)[0].tolist())
            n_fb += int(bad.sum())
        tj = self.tj
        tj.append(time.perf_counter())
        t_wait = time.perf_counter()
        b.wait()
        t.append(time.perf_counter())
        for j, idx in enumerate(fallback):
            if idx:
                p = Plan(ctx, self.mods[j], plain_opts(self.plain), np.asarray(self.dists_list[j], np.float64)[idx])
                p.execute()
                traces[j][idx] = p.fetch(True, False)[0].astype(np.float32)
                p.close()
        t.append(time.perf_counter())
        _, tune = b.info()
        grids, t_exec, t_pre = self.grids, self.t_exec, self.t_pre
        # the judge's time beyond the graph: its part before the graph ended
        # (when it outlasted the graph) and its part after
        exposed_pre = max(0.0, t_pre - t_exec) if overlap else t_pre - tj[0]
        info = dict(nkw_learned=int(sum(int(g_[0].sum()) for g_ in grids)),
                    nkw_plain=int(sum(int(g_[3]["nw"]) * self.plain["nk"] for g_ in grids)),
                    stride_mean=float(np.mean([g_[1].mean() for g_ in grids])), fallback=fallback,
                    n_fallback=n_fb, ms_batch_gpu=rep.ms_total, ms_batch_grt=rep.ms_grt,
                    n_layer_evals=int(rep.n_layer_evals),
                    gpu_launches=rep.kernel_launches,
                    # the judge's: its spot batch, per model a sweep (GRT and sweep kernels) and two gathers
                    judge_launches=int(self.n_judge_launches) + 4 * len(self.mods), tune=tune,
                    s_predict=t[1] - t[0], s_build=t[2] - t[1],
                    s_execute=t[3] - t[2], s_fetch=t[3] - t_exec, s_fetch_wait=t[4] - t_wait,
                    s_judge=exposed_pre + (t_wait - t_c), s_fallback=t[5] - t[4],
                    s_total=t[5] - t[0], judge_overlapped=bool(overlap),
                    s_judge_parts=dict(spot_build=tj[1] - tj[0], spot_exec=tj[2] - tj[1],
                                       sweeps_compare=(t_pre - tj[2]) + (tj[3] - t_c), sweeps=self.t_sw,
                                       fetch_spots=self.t_ff, before_graph_end=max(0.0, t_exec - tj[0]) if overlap
                                       else 0.0, total=(t_pre - tj[0]) + (t_wait - t_c)))
        t_close = time.perf_counter()
        b.close()
        info["s_close"] = time.perf_counter() - t_close
        info["s_graph_call"] = t_exec - self.t_start   # the batch's execute call (graph launch to results)
        info["t_graph_start"], info["t_graph_end"] = self.t_start, self.done.get("t_staged", t_exec)
        info["s_call"] = time.perf_counter() - t[0]
        return traces, info

    def abandon(self):
        """After an error: the graph's thread ends before the batch goes."""
        try:
            if self.runner is not None:
                self.runner.join()
                self.runner = None
        finally:
            self.b.close()


def run_learned_batch(sampler, models, dists_list, ctx=None, plain=PLAIN, spec_tol=3e-3, autotune=True,
                      use_stride=True, out=None, overlap=True):
    """run_learned for many models at once: one batch (one CUDA graph, one
    GRT launch) on the learned grids, the judge's spot evaluations as a
    second batch, sweeps per model, and the plain grid for any receiver the
    judge rejects.  Returns (list of float32 traces, info); with `out` (one
    float32 [n_dist, n_cols, N] array per model, e.g. pinned_empty ones) the
    traces are fetched into those arrays.

    overlap: the judge's own GPU work (the plain grid at the spot
    frequencies, the tail sweeps) needs only the models and the batch's k
    split, so it runs on a second context while the batch's graph runs on
    this one (the graph in a host thread; both share the GPU); only the
    comparison with the batch's spectra waits for the graph.  info's s_judge
    is the judge's time not hidden behind the graph."""
    own = ctx is None
    ctx = ctx or Context()
    try:
        lb = _LearnedBatch(sampler, models, dists_list, ctx, plain, spec_tol, autotune, use_stride, out)
        try:
            lb.start(threaded=overlap)
            lb.judge_pre(judge_context(ctx) if overlap else ctx)
        except BaseException:
            lb.abandon()
            raise
        try:
            lb.join()
        except BaseException:
            lb.abandon()
            raise
        return lb.finish(overlap)
    finally:
        if own:
            ctx.close()


def run_learned_stream(sampler, work, ctxs, outs=None, plain=PLAIN, spec_tol=3e-3, autotune=True,
                       use_stride=True):
    """run_learned_batch over a sequence of batches, pipelined: while batch
    i's graph runs, batch i+1 is predicted and built and its judge's own GPU
    work runs; batch i+1's graph starts as soon as batch i's device stages
    end (batch i's last download drains beside it), and batch i's
    comparison, fallbacks and clean-up run beside it.  Yields
    (traces, info) per batch, in order.

    work: iterable of (models, dists_list); ctxs: two contexts on one device
    (consecutive batches alternate between them: a context is used by one
    host thread at a time); outs: optional pair of per-model page-locked
    output lists, alternating the same way (the graph of batch i+2 writes
    into batch i's arrays: use or copy a batch's traces before asking for
    the next batch)."""
    if len(ctxs) != 2:
        raise ValueError("run_learned_stream needs two contexts")
    jctx = judge_context(ctxs[0])
    it = iter(work)

    def make(i, item):
        models, dists_list = item
        out = outs[i % 2] if outs is not None else None
        return _LearnedBatch(sampler, models, dists_list, ctxs[i % 2], plain, spec_tol, autotune, use_stride, out)

    item = next(it, None)
    if item is None:
        return
    cur, i = make(0, item), 0
    nxt = None
    try:
        cur.start()
        cur.judge_pre(jctx)
        while cur is not None:
            item = next(it, None)
            nxt = make(i + 1, item) if item is not None else None
            if nxt is not None:
                nxt.judge_pre(jctx)
            cur.wait_stages()
            if nxt is not None:
                nxt.start()
            cur.join()
            res = cur.finish(True)
            cur, nxt, i = nxt, None, i + 1
            yield res
    except BaseException:
        for lb in (cur, nxt):
            if lb is not None:
                try:
                    lb.abandon()
                except Exception:
                    pass
        raise
