"""Green's-function throughput on one GB300 (and N independent replicas).

Workload (one step = one complete job): a seeded 20-layer crustal model over a
half-space (thickness U(0.5, 5) km, Vp 2.5 -> 8.0 km/s linear plus N(0, 0.15),
Vs = Vp / U(1.65, 1.85), Gardner density, Qs U(50, 300), Qp = 2 Qs),
moment-tensor (double-couple) source at 15 km, 200 receivers log-spaced
5-300 km, nt = 4096, dt = 0.05 s, fixed grid of 16384 wavenumbers,
sigma = pi / T.  A trace is one receiver with its 20 moment-tensor Green's
function columns over all nt samples.

  value  traces/s from the device time of the four kernels of a step (CUDA
         events on the library's stream); inputs resident in HBM.
  e2e    traces/s through the public call grt_run with host buffers: layer
         tables and receivers uploaded, traces downloaded, every step.
Accuracy: rel-L2 of the FP32 traces against the FP64 GPU path of the same
method is measured once per run and reported.

Launch: python bench.py [--gpus N --steps K --warmup W] [--impl reference]
(for N > 1 under torch.distributed.run: every rank runs its own seeded model,
no collective on the data path; the timing is the max over ranks).
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

F_LAYER = 1490.0   # algorithmic flops per (w,k,layer), counted on the method (cmul 6, cdiv 11, cexp/csqrt 20)
F_SRC_TENSOR = 710.0
F_SRC_SINGLE = 449.0


def config2_model(seed):
    rng = np.random.default_rng(seed)
    nl = 20
    h = rng.uniform(0.5, 5.0, nl)
    tops = np.concatenate([[0.0], np.cumsum(h)])            # 20 layers + half-space
    vp = np.linspace(2.5, 8.0, nl + 1) + rng.normal(0.0, 0.15, nl + 1)
    vs = vp / rng.uniform(1.65, 1.85, nl + 1)
    rho = 1.74 * vp ** 0.25
    qs = rng.uniform(50.0, 300.0, nl + 1)
    qp = 2.0 * qs
    hs = 15.0
    if np.min(np.abs(tops - hs)) < 1e-9:
        hs += 0.0005
    dists = np.logspace(np.log10(5.0), np.log10(300.0), 200)
    return dict(ztop=tops, vp=vp, vs=vs, rho=rho, qp=qp, qs=qs, hs=hs, hr=0.0, src_type=1), dists


WORKLOAD = dict(dt=0.05, log2n=12, t0=0.0, taper=0.3, sigma_factor=np.pi, nk=16384)


def config1_model(seed=0):
    """Tops 0/2/10/20/35 km, Vp 3.0/5.8/6.5/7.0/8.0, Vs = Vp/1.73, Gardner
    density, Qp 200, Qs 100; source at 10 km moved 0.5 m below the interface;
    10 receivers at 10-100 km."""
    vp = np.array([3.0, 5.8, 6.5, 7.0, 8.0])
    mk = dict(ztop=np.array([0.0, 2.0, 10.0, 20.0, 35.0]), vp=vp, vs=vp / 1.73, rho=1.74 * vp ** 0.25,
              qp=np.full(5, 200.0), qs=np.full(5, 100.0), hs=10.0005, hr=0.0, src_type=1)
    return mk, np.arange(10.0, 101.0, 10.0)


WORKLOAD1 = dict(dt=0.1, log2n=10, t0=0.0, taper=0.3, sigma_factor=np.pi, nk=4096)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as td
        td.init_process_group("gloo")
        return ws, rank, local, td
    return 1, 0, 0, None


def barrier(td):
    if td is not None:
        td.barrier()


def allmax(td, x):
    if td is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    td.all_reduce(t, op=td.ReduceOp.MAX)
    return float(t.item())


def device_sync():
    try:
        import torch
        if torch.cuda.is_available():
            torch.cuda.synchronize()
    except Exception:
        pass


def fp32_peak_tflops():
    """cuBLAS FP32 SGEMM (TF32 off) as the FP32-pipe denominator."""
    try:
        import torch
        torch.backends.cuda.matmul.allow_tf32 = False
        n = 8192
        a = torch.randn(n, n, device="cuda")
        b = torch.randn(n, n, device="cuda")
        for _ in range(2):
            torch.matmul(a, b)
        torch.cuda.synchronize()
        best = 0.0
        for _ in range(5):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            torch.matmul(a, b)
            e1.record()
            e1.synchronize()
            best = max(best, 2.0 * n ** 3 / (e0.elapsed_time(e1) * 1e-3) / 1e12)
        del a, b
        torch.cuda.empty_cache()
        return best
    except Exception:
        return None


def measured_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return {}


def cpu_baseline(mk, dists, kw, budget_s=12.0, impl_ref=False):
    """The oracle (the reference's algorithm restated in C, all host cores) on a
    bounded sample of the same job: a band of frequencies spread over the
    spectrum, scaled to the whole job."""
    from oracle import oracle as O
    O.build()
    job = O.model(mk["ztop"], mk["vp"], mk["vs"], mk["rho"], mk["qp"], mk["qs"], mk["hs"], mk["hr"], mk["src_type"])
    O.setup(job, kw["dt"], kw["log2n"], kw["t0"], kw["taper"], kw["sigma_factor"], O.K_FIXED, kw["nk"], fix=O.FIX_RLAYER)
    cores = os.cpu_count() or 1
    nw = job.nw
    # calibrate on one frequency, then size the sample to the budget
    t = time.time()
    O.run_band(job, dists, nw // 2, nw // 2 + 1, cores)
    t1 = time.time() - t
    nf = int(max(1, min(nw, budget_s / max(t1, 1e-3))))
    iw0 = (nw - nf) // 2
    t = time.time()
    O.run_band(job, dists, iw0, iw0 + nf, cores)
    el = time.time() - t
    full = el * nw / nf
    return {"value": len(dists) / full, "unit": "traces/s", "cores": cores,
            "kind": "port",
            "sample": f"{nf} of {nw} frequencies x {kw['nk']} wavenumbers x {len(dists)} receivers "
                      f"({el:.1f} s), scaled to the whole job ({full:.0f} s)"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    ap.add_argument("--case", default="config2", choices=["config2", "config1"],
                    help="config2: 20 layers, 200 receivers (the metric's workload); config1: 4 layers, 10 receivers")
    args = ap.parse_args()
    ws, rank, local, td = dist_setup()
    if args.case == "config1":
        kw = dict(WORKLOAD1)
        mk, dists = config1_model()
        config = {"workload": "GRT Green's functions: 4 layers over a half-space, double-couple source at 10 km, "
                              "10 receivers 10-100 km, nt 1024, dt 0.1 s, nk 4096, sigma=pi/T",
                  "traces_per_step": len(dists), "cols_per_trace": 20, "nt": 1024, "nk": kw["nk"], "layers": 6,
                  "receivers": len(dists), "l2": "inputs larger than L2 (per-(w,k) coefficients 134 MB per step)",
                  "parallelism": f"replicas x{ws}" if ws > 1 else "single GPU"}
    else:
        kw = dict(WORKLOAD)
        mk, dists = config2_model(1234 + rank)
        config = {"workload": "GRT Green's functions: seeded 20-layer crust over a half-space, double-couple "
                              "source at 15 km, 200 receivers 5-300 km, nt 4096, dt 0.05 s, nk 16384, sigma=pi/T",
                  "traces_per_step": len(dists), "cols_per_trace": 20, "nt": 4096, "nk": kw["nk"], "layers": 21,
                  "receivers": len(dists), "l2": "inputs larger than L2 (per-(w,k) coefficients 2.1 GB per step)",
                  "parallelism": f"replicas x{ws}" if ws > 1 else "single GPU"}
    metric = "Green's-fn traces/s at <=1e-3 rel-L2 vs FP64 (1 GB300)"

    if args.impl == "reference":
        if rank == 0:
            cb = cpu_baseline(mk, dists, kw, budget_s=20.0, impl_ref=True)
            steps = []
            for _ in range(max(1, min(args.steps, 3))):
                steps.append(cpu_baseline(mk, dists, kw, budget_s=8.0, impl_ref=True)["value"])
            v = float(np.median(steps))
            out = {"impl": "reference", "metric": metric, "value": v, "unit": "traces/s", "n_gpus": args.gpus,
                   "steps": len(steps), "warmup": 1, "ms_per_step": 1000.0 * len(dists) / v,
                   "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128",
                   "data": "synthetic (seeded)", "config": config,
                   "cpu_baseline": dict(cb, value=v),
                   "e2e": {"value": v, "unit": "traces/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
                   "note": "the reference has no CPU implementation of the GRT path; this times the FP64 C "
                           "restatement of its algorithm (oracle/) on all host cores"}
            print(json.dumps(out))
        barrier(td)
        return

    import grtm_cuda_gb300 as g
    g.lib()
    ctx = g.Context(local)
    m = g.make_model(**mk)
    o32 = g.make_opts(kw["dt"], kw["log2n"], kw["t0"], kw["taper"], kw["sigma_factor"], g.K_FIXED, kw["nk"],
                      precision=g.FP32, fix=g.FIX_RLAYER)
    plan = g.Plan(ctx, m, o32, dists)
    for _ in range(args.warmup):
        plan.execute()
    tr32, _ = plan.fetch(True, False)
    # accuracy against the FP64 GPU path of the same method (once, untimed)
    o64 = g.make_opts(kw["dt"], kw["log2n"], kw["t0"], kw["taper"], kw["sigma_factor"], g.K_FIXED, kw["nk"],
                      precision=g.FP64, fix=g.FIX_RLAYER)
    p64 = g.Plan(ctx, m, o64, dists)
    p64.execute()
    tr64, _ = p64.fetch(True, False)
    p64.close()
    per_rcv = np.linalg.norm(tr32 - tr64, axis=(1, 2)) / np.linalg.norm(tr64, axis=(1, 2))
    rel_all = float(np.linalg.norm(tr32 - tr64) / np.linalg.norm(tr64))

    clocks = ClockSampler(local)
    clocks.start()
    barrier(td)
    device_sync()
    reps = []
    t0 = time.time()
    for _ in range(args.steps):
        reps.append(plan.execute().as_dict())
    device_sync()
    wall = time.time() - t0
    barrier(td)
    dev_ms = float(np.sum([r["ms_total"] for r in reps]))
    dev_ms = allmax(td, dev_ms)
    rep = reps[-1]
    ms_step = dev_ms / args.steps
    value = ws * len(dists) / (ms_step * 1e-3)

    # e2e through the public call with host buffers
    e2e_t = []
    for i in range(max(2, min(args.steps, 4)) + 1):
        device_sync()
        t = time.time()
        tr, _, r = g.run(m, o32, dists, ctx)
        device_sync()
        if i > 0:
            e2e_t.append(time.time() - t)
    e2e_t = allmax(td, float(np.median(e2e_t)))
    clk = clocks.stop()
    plan.close()

    if rank != 0:
        barrier(td)
        return
    # roofline of the dominant kernel
    peaks = measured_peaks()
    fp32_peak = fp32_peak_tflops()
    L = rep["n_layer"]
    grt_flops = rep["n_wk"] * (L * F_LAYER + F_SRC_TENSOR)
    kernels = {"grt_point": rep["ms_grt"], "bessel_table": rep["ms_bessel"], "ksum": rep["ms_ksum"],
               "spectral": rep["ms_spectral"]}
    dom = max(kernels, key=kernels.get)
    ksum_flops = 2.0 * rep["n_wk"] * len(dists) * 25 * 2   # 25 complex x real pairs per (w,k,receiver)
    spec_bytes = len(dists) * 20 * (rep["nw"] * 8 + rep["n_samples"] * 4 + rep["n_samples"] * 8)
    rl = {
        "grt_point": {"bound": "fp32", "achieved": grt_flops / (rep["ms_grt"] * 1e-3) / 1e12,
                      "peak": fp32_peak, "unit": "TFLOP/s", "traffic": None,
                      "per_launch": f"{rep['n_wk']} (w,k) points x ({L} x {F_LAYER:.0f} + {F_SRC_TENSOR:.0f}) flops"},
        "ksum": {"bound": "fp32", "achieved": ksum_flops / (rep["ms_ksum"] * 1e-3) / 1e12,
                 "peak": fp32_peak, "unit": "TFLOP/s", "traffic": None},
        "spectral": {"bound": "hbm", "achieved": spec_bytes / (rep["ms_spectral"] * 1e-3) / 1e9,
                     "peak": peaks.get("hbm_gbs"), "unit": "GB/s", "traffic": None},
    }
    for v in rl.values():
        v["frac"] = (v["achieved"] / v["peak"]) if v.get("peak") else None
    roof = dict(rl[dom], kernel=dom)
    roof["peak_source"] = ("cuBLAS FP32 SGEMM (TF32 off) measured in this run" if roof["bound"] == "fp32"
                           else "MEASURED_PEAKS.json hbm_gbs")
    out = {
        "metric": metric, "value": value, "unit": "traces/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "c64 (FP32 complex; FP64 branch selection, Bessel and exp(sigma t))",
        "data": "synthetic (seeded model and receivers)", "config": config,
        "accuracy": {"rel_l2_vs_fp64": rel_all, "max_per_receiver": float(per_rcv.max()),
                     "median_per_receiver": float(np.median(per_rcv))},
        "kernel_ms": kernels, "wall_s_timed": wall,
        "gpu_launches": rep["kernel_launches"] * args.steps,
        "roofline": roof, "rooflines": rl,
        "e2e": {"value": ws * len(dists) / e2e_t, "unit": "traces/s",
                "h2d_bytes_per_step": rep["h2d_bytes"], "d2h_bytes_per_step": rep["d2h_bytes"]},
        "clocks": clk,
    }
    if not args.no_cpu:
        out["cpu_baseline"] = cpu_baseline(mk, dists, kw)
    print(json.dumps(out))
    barrier(td)


if __name__ == "__main__":
    main()
