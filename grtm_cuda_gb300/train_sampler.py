"""Train the learned wavenumber sampler on convergence sweeps of the plain
grid, and evaluate it on held-out models.

    python -m grtm_cuda_gb300.train_sampler --out grtm_cuda_gb300/data/ksampler.bin
    python -m grtm_cuda_gb300.train_sampler --eval --weights ... --eval-models 8
    python -m grtm_cuda_gb300.train_sampler --recalibrate --weights ... --out ...

Training data: 320 seeded 40-layer crustal models (source depth U(1, 30) km),
8 frequencies x 8 distances each (20480 sweeps) on the plain grid of
N = 8192 samples at dt = 0.05 s with nk = 32768; 64 further models for
validation and the safety margins.  Everything runs on the GPU through the
library (sweeps: grt_sweep_kmax; training: grt_mlp_train).
"""
import argparse
import json
import sys
import time

import numpy as np

from . import FP64, Context, Plan, make_model, synth
from .learned import PLAIN, WEIGHTS, Sampler, plain_opts, run_learned, sweep_dataset

TRAIN_SEEDS = range(1000, 1320)
VAL_SEEDS = range(2000, 2064)
HELD_OUT_SEEDS = range(3000, 3256)
CAL_SEEDS = range(5000, 5256)      # further sweeps for the per-band margins


def recalibrate(weights, out, n_bands=8, n_cal=256, tol=1e-4, log=sys.stdout, dump=None, q_k=0.995):
    """Keep a trained network and measure its k_max margins per band of log w
    on the validation sweeps and n_cal further models (the bands need more
    sweeps than one global quantile)."""
    s = Sampler.load(weights)
    ctx = Context()
    t0 = time.perf_counter()
    Xv, Yv = sweep_dataset(ctx, list(VAL_SEEDS), tol=tol, rng_seed=2)
    Xc, Yc = sweep_dataset(ctx, list(CAL_SEEDS)[:n_cal], tol=tol, rng_seed=3)
    X, Y = np.concatenate([Xv, Xc]), np.concatenate([Yv, Yc])
    t1 = time.perf_counter()
    if dump:
        np.savez_compressed(dump, X=X, Y=Y, pred=s.predict(ctx, X))
    mk, md = s.calibrate(ctx, X, Y, q_k=q_k, n_bands=n_bands)
    s.save(out)
    ctx.close()
    e, mg = s.kbands if s.kbands is not None else ([], [])
    res = dict(n_sweeps=len(X), s_sweeps=t1 - t0, q_k=q_k, margin_k=mk, margin_d=md,
               band_edges_hz=[float(np.exp(x) / (2 * np.pi)) for x in e], band_margins=[float(x) for x in mg])
    print(json.dumps(res), file=log)
    return s, res


def train(out, n_models=320, n_val=64, tol=1e-4, log=sys.stdout, dump=None):
    ctx = Context()
    t0 = time.perf_counter()
    X, Y = sweep_dataset(ctx, list(TRAIN_SEEDS)[:n_models], tol=tol, rng_seed=1)
    Xv, Yv = sweep_dataset(ctx, list(VAL_SEEDS)[:n_val], tol=tol, rng_seed=2)
    t1 = time.perf_counter()
    if dump:
        np.savez_compressed(dump, X=X.astype(np.float32), Y=Y.astype(np.float32), Xv=Xv.astype(np.float32),
                            Yv=Yv.astype(np.float32))
    s, hist = Sampler.train_new(ctx, X, Y, val=(Xv, Yv))
    t2 = time.perf_counter()
    s.tol = tol
    mk, md = s.calibrate(ctx, Xv, Yv)
    yv = s.predict(ctx, Xv)
    res = dict(n_train=len(X), n_val=len(Xv), s_sweeps=t1 - t0, s_train=t2 - t1, history=hist,
               val_rmse_logk=float(np.sqrt(np.mean((yv[:, 0] - Yv[:, 0]) ** 2))),
               val_rmse_log2dk=float(np.sqrt(np.mean((yv[:, 1] - Yv[:, 1]) ** 2))),
               margin_k=mk, margin_d=md, target_mean=Y.mean(0).tolist(), target_std=Y.std(0).tolist(),
               dk_mult_hist=np.bincount(np.round(Y[:, 1]).astype(int), minlength=6).tolist())
    s.save(out)
    ctx.close()
    print(json.dumps(res), file=log)
    return s, res


def evaluate(weights, n_models=8, n_receivers=24, fp64=True, log=sys.stdout, use_stride=True):
    """Learned vs plain FP32 vs plain FP64 on held-out models."""
    s = Sampler.load(weights)
    ctx = Context()
    rows = []
    for seed in list(HELD_OUT_SEEDS)[:n_models]:
        rng = np.random.default_rng(seed)
        m = synth.crust(rng, 40, rng.uniform(1.0, 30.0))
        dists = np.sort(rng.uniform(1.0, 500.0, n_receivers))
        model = make_model(**m)
        plan = Plan(ctx, model, plain_opts(), dists)
        plan.execute()
        ms_plain = plan.report.ms_total
        tp, _ = plan.fetch(True, False)
        plan.close()
        tl, info = run_learned(s, m, dists, ctx=ctx, use_stride=use_stride)
        row = dict(seed=seed, hs=m["hs"], ms_plain=ms_plain, **{k: v for k, v in info.items() if k != "fallback"},
                   n_fallback=len(info["fallback"]))
        ref = tp
        if fp64:
            plan = Plan(ctx, model, plain_opts(precision=FP64), dists)
            plan.execute()
            ref, _ = plan.fetch(True, False)
            plan.close()
        def rel(a):
            e = np.sqrt(np.sum((a - ref) ** 2, axis=(1, 2)) / np.sum(ref ** 2, axis=(1, 2)))
            return float(e.max()), float(np.median(e)), float(np.mean(e <= 1e-3))
        row["learned_vs_ref"] = rel(tl)
        row["plain_vs_ref"] = rel(tp)
        rows.append(row)
        print(json.dumps(row), file=log, flush=True)
    ctx.close()
    return rows


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=WEIGHTS)
    ap.add_argument("--models", type=int, default=320)
    ap.add_argument("--tol", type=float, default=1e-4)
    ap.add_argument("--eval", action="store_true")
    ap.add_argument("--weights", default=WEIGHTS)
    ap.add_argument("--eval-models", type=int, default=8)
    ap.add_argument("--receivers", type=int, default=24)
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--dump", default=None, help="also write the sweep dataset (npz)")
    ap.add_argument("--no-stride", action="store_true", help="evaluate with unit k stride")
    ap.add_argument("--recalibrate", action="store_true",
                    help="keep the network of --weights, measure per-band k margins, write --out")
    ap.add_argument("--bands", type=int, default=8, help="recalibrate: bands of log w")
    ap.add_argument("--q-k", type=float, default=0.995,
                    help="recalibrate: quantile of the k_max under-prediction a band's margin covers")
    a = ap.parse_args()
    if a.recalibrate:
        recalibrate(a.weights, a.out, n_bands=a.bands, tol=a.tol, dump=a.dump, q_k=a.q_k)
    elif a.eval:
        evaluate(a.weights, a.eval_models, a.receivers, not a.no_fp64, use_stride=not a.no_stride)
    else:
        train(a.out, a.models, tol=a.tol, dump=a.dump)


if __name__ == "__main__":
    main()
