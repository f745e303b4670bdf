"""Benchmark: NUTS (diag_e, adaptive) on the 1024-chain logistic GLM.

Workload (one step = one complete fit): Bayesian logistic regression,
N = 100000 rows, K = 100 predictors, X ~ N(0,1) with standardised columns
stored FP32, alpha, beta ~ N(0, 2.5) priors; 1024 chains in one device run,
500 warmup + 1000 sampling iterations, max tree depth 10, delta 0.8.
Synthetic seeded data (no public dataset is named for this path).

value       : whole-job gradient evaluations per second (sum over chains of
              leapfrog steps + step-size search trials + init evaluations,
              divided by the device time of the fits, CUDA events).
extra keys  : min bulk ESS/s of the fit (split rank-normalised bulk ESS over
              all parameters and lp__), ESS per gradient evaluation, the
              gradient kernel's roofline, the FP64 form's gradient rate,
              the CPU baseline.
e2e         : the same metric through the C ABI with host buffers (model
              creation with the H2D copy of X and y, the fit, and the D2H copy
              of every draw inside the timed region).

--impl reference runs the CPU restatement of the reference's sampler (the
reference itself cannot be built here) on all host cores.
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

# DRAM bytes (read + write) of one launch of the dominant gradient kernel,
# from an ncu capture of `python bench.py --case grad --workload W --precision P`
# (one launch, dram__bytes_read.sum + dram__bytes_write.sum).
TRAFFIC = {
    ("logistic_100k", "f16x3"): (5.70e7, "ncu --set full --clock-control none -k regex:glm_tct "
                                         "-s 1 -c 1 on python bench.py --case grad "
                                         "--workload logistic_100k --precision f16x3: "
                                         "53.8 MB read + 3.2 MB written, full-size launch"),
}

WORKLOADS = {
    "logistic_100k": dict(kind="logistic_100k", chains=1024, warmup=500, samples=1000),
    "logistic_1k": dict(kind="logistic", chains=4, warmup=1000, samples=1000),
    "hier_normal": dict(kind="hier_normal", chains=256, warmup=500, samples=1000),
    "poisson_262k": dict(kind="poisson", chains=512, warmup=500, samples=1000),
}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def select_device(ws, local):
    """One GPU per rank, chosen before the library initialises CUDA: the
    local-th entry of an existing CUDA_VISIBLE_DEVICES list (a launcher or
    scheduler may have set one), else GPU `local`.  Returns the device as
    nvidia-smi names it (index or UUID), for the clock sampler."""
    vis = os.environ.get("CUDA_VISIBLE_DEVICES")
    if ws <= 1:
        return (vis.split(",")[0].strip() if vis else "0")
    if vis:
        lst = [v.strip() for v in vis.split(",") if v.strip()]
        if local >= len(lst):
            raise RuntimeError(f"local rank {local} has no GPU in CUDA_VISIBLE_DEVICES={vis}")
        dev = lst[local]
    else:
        dev = str(local)
    os.environ["CUDA_VISIBLE_DEVICES"] = dev
    return dev


class ClockSampler:
    """Samples SM clocks and throttle reasons with nvidia-smi during a region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx = float(p[2])
            except ValueError:
                continue
            for n, v in zip(names, p[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def flush_l2(lib_module=None):
    """Writes a 256 MiB device buffer (twice the 129 MB L2) between timed fits."""
    import ctypes
    cudart = ctypes.CDLL("libcudart.so")
    p = ctypes.c_void_p()
    n = 256 << 20
    if cudart.cudaMalloc(ctypes.byref(p), ctypes.c_size_t(n)) == 0:
        cudart.cudaMemset(p, 1, ctypes.c_size_t(n))
        cudart.cudaDeviceSynchronize()
        cudart.cudaFree(p)


def fit_stats(res, ds):
    from stan_gb300 import analyze
    grads = int(res.n_grad.sum())
    secs = res.total_ms / 1e3
    draws = res.sampling_draws()  # (iters, chains, 7 + D)
    q = np.concatenate([draws[:, :, 0:1], draws[:, :, 7:]], axis=2)
    ess, which = analyze.min_bulk_ess(q, ["lp__"] + ds.param_names())
    return grads, secs, ess, which


def cpu_baseline(ds, wl, seconds_target=20.0, stepsize=None, inv_metric=None):
    """The oracle (plain FP64 sums, the reference's algorithm) on all host cores:
    one chain per core, non-adaptive NUTS at the GPU-adapted step size and
    metric, timed until ~seconds_target of work; gradient evaluations per
    second counts every evaluation (including the recompute at each
    transition start that the reference performs)."""
    import oracle
    cores = os.cpu_count() or 1
    om = oracle.OracleModel(ds.kind, ds.X, ds.y, group=ds.group, J=ds.J, hp=list(ds.hp),
                            intercept=ds.intercept, compensated=False)
    C = cores
    kw = dict(num_chains=C, adapt=False, num_warmup=0, max_depth=10, seed=99,
              stepsize=stepsize if stepsize else 0.05, init_radius=0.5, num_threads=cores)
    if inv_metric is not None:
        kw["inv_metrics"] = np.tile(inv_metric, (C, 1))
    # calibrate with a short run, then size the sample to ~seconds_target
    t0 = time.time()
    r = om.sample(num_samples=2, **kw)
    t1 = time.time()
    g = int(r["n_grad_total"].sum())
    rate = g / max(t1 - t0, 1e-9)
    per_transition = max(g / (2 * C), 1)
    n = int(max(2, min(2000, seconds_target * rate / (per_transition * C))))
    t0 = time.time()
    r = om.sample(num_samples=n, **kw)
    dt = time.time() - t0
    g = int(r["n_grad_total"].sum())
    return {"value": g / dt, "unit": "grad evals/s", "cores": cores, "kind": "port",
            "sample": f"{C} chains x {n} non-adaptive NUTS transitions of the same posterior "
                      f"(one chain per core, FP64, {g} gradient evaluations in {dt:.1f} s)"}


def run_ours(args, ws, rank, gpu):
    from stan_gb300 import Model, _lib, sampler, workloads
    wl = WORKLOADS[args.workload]
    ds = workloads.make_dataset(wl["kind"], seed=1 + rank)
    _lib.load(build_if_missing=False)
    model = Model.from_dataset(ds)
    C = wl["chains"]
    kw = dict(num_chains=C, num_warmup=wl["warmup"], num_samples=wl["samples"], adapt=True,
              max_depth=10, delta=0.8, precision=args.precision, init_radius=2.0)
    for i in range(args.warmup):
        sampler.run(model, random_seed=1000 + i, **kw)
    barrier(ws)
    grads_total, secs_total = 0, 0.0
    last = None
    grad_ms = []
    steps = 0
    launches = 0
    with ClockSampler(gpu) as clk:
        t_wall = time.time()
        for i in range(args.steps):
            flush_l2()
            res = sampler.run(model, random_seed=2000 + i, **kw)
            grads_total += int(res.n_grad.sum())
            secs_total += res.total_ms / 1e3
            grad_ms.append(res.grad_ms)
            steps += res.steps
            launches += res.kernel_launches
            last = res
        wall = time.time() - t_wall
    secs_total = max_over_ranks(secs_total, ws)
    grads_all = sum_over_ranks(grads_total, ws)
    value = grads_all / secs_total
    g, s, ess, which = fit_stats(last, ds)
    ess_per_s = ess / s
    samp_s = float(np.max(last.seconds[:, 1])) if last.seconds.size else s
    # roofline of the batched gradient kernel (dominant): 4 N K flops per chain
    # that requests a gradient; a launch serves the fit's active chains (all C
    # at first, fewer as chains finish: the launch shrinks with them), so the
    # per-launch work is taken at the fit's mean active chains per step
    N, K = ds.N, ds.K
    active_mean = grads_total / max(steps, 1)
    flops = 4.0 * N * K * active_mean
    mean_ms = float(np.mean(grad_ms))
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(ROOT, "MEASURED_PEAKS.json")) else {}
    # the gradient runs inside a seconds-long fit: the sustained bf16 peak applies
    peak = peaks.get("bf16_tflops_sustained", peaks.get("bf16_tflops", 1700.0))
    ach = flops / (mean_ms * 1e-3) / 1e12
    kpad = 16 * ((K + 1 + 15) // 16)
    tensor = args.precision in ("bf16x3", "f16x3")
    # three 16-bit products, two contractions, K padded (active chains)
    executed = 3 * 2 * 2.0 * N * active_mean * kpad
    traffic = TRAFFIC.get((args.workload, args.precision))
    roof = {"bound": "tensor", "achieved": ach, "peak": peak, "unit": "TFLOP/s",
            "frac": ach / peak,
            # dram__bytes_read.sum + dram__bytes_write.sum of one launch
            "traffic": traffic[0] if traffic else None,
            "traffic_source": traffic[1] if traffic else None,
            "peak_source": "MEASURED_PEAKS.json bf16_tflops_sustained (of measured)",
            "kernel": "glm_tct_kernel" if tensor else "loglik_partial_pool_kernel",
            "executed_tflops": executed / (mean_ms * 1e-3) / 1e12,
            "executed_frac": executed / (mean_ms * 1e-3) / 1e12 / peak,
            "mean_launch_ms": mean_ms,
            "flops_per_launch": flops,
            "active_chains_per_launch": active_mean}
    out = {"metric": "grad evals/s", "value": value, "unit": "grad evals/s", "n_gpus": ws,
           "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": secs_total * 1e3 / args.steps, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64" if args.precision == "fp64" else "f32+f64",
           "data": "synthetic (seeded; shapes and distributions of the workload)",
           "config": {"workload": f"{args.workload}: logistic GLM N={N} K={K} X fp32, {C} chains, "
                                  f"{wl['warmup']} warmup + {wl['samples']} draws, max_depth 10",
                      "precision": args.precision, "parallelism": f"replicas x{ws}",
                      "l2": "256 MiB buffer written between timed fits"},
           "min_bulk_ess_per_s": ess_per_s, "min_bulk_ess": ess, "min_ess_param": which,
           "min_bulk_ess_per_s_sampling": ess / samp_s if samp_s > 0 else None,
           "ess_per_grad": ess / g, "fit_seconds": s, "device_steps": steps,
           "roofline": roof, "gpu_launches": int(launches), "clocks": clk.summary(),
           "wall_seconds_timed": wall}
    if rank == 0 and not args.no_e2e:
        out["e2e"] = e2e(args, ds, kw)
    if rank == 0 and not args.no_fp64:
        out["fp64_form"] = fp64_rate(model, ds, C)
        # the FP64 form's ESS/s, estimated with the mixed run's ESS per gradient
        # (a full FP64 fit of this workload takes over an hour)
        out["fp64_form"]["min_bulk_ess_per_s_estimate"] = (
            out["fp64_form"]["grad_evals_per_s"] * ess / g)
        out["mixed_over_fp64_ess_per_s_estimate"] = ess_per_s / out["fp64_form"][
            "min_bulk_ess_per_s_estimate"]
        if args.precision != "fp64":
            out["precision_errors"] = precision_errors(model, last, args.precision)
    if rank == 0 and not args.no_csv:
        try:
            out["csv_output"] = csv_leg(model, last)
        except Exception as e:  # reported, not fatal to the headline line
            out["csv_output"] = {"error": repr(e)}
    if rank == 0 and not args.no_config_d:
        try:
            out["config_d"] = config_d_leg()
        except Exception as e:  # reported, not fatal to the headline line
            out["config_d"] = {"error": repr(e)}
    if rank == 0 and not args.no_config_c:
        try:
            out["config_c"] = config_c_leg()
        except Exception as e:  # reported, not fatal to the headline line
            out["config_c"] = {"error": repr(e)}
    if rank == 0 and not args.no_config_a:
        try:
            out["config_a"] = config_a_leg()
        except Exception as e:  # reported, not fatal to the headline line
            out["config_a"] = {"error": repr(e)}
    if rank == 0 and not args.no_serving:
        try:
            out["serving"] = serving_leg()
        except Exception as e:  # reported, not fatal to the headline line
            out["serving"] = {"error": repr(e)}
    if rank == 0 and not args.no_cpu:
        eps = float(np.median(last.stepsize))
        out["cpu_baseline"] = cpu_baseline(ds, wl, args.cpu_seconds, eps,
                                           np.median(last.inv_metric, axis=0))
    return out


def e2e(args, ds, kw):
    """Through the C ABI with host buffers: H2D of X and y (model creation),
    the fit, and the D2H copy of all draws, timed on the host."""
    from stan_gb300 import Model, sampler
    t0 = time.time()
    grads = 0
    d2h = 0
    for i in range(args.steps):
        m = Model.from_dataset(ds)
        res = sampler.run(m, random_seed=3000 + i, **kw)
        grads += int(res.n_grad.sum())
        d2h += res.draws.nbytes
        m.close()
    dt = time.time() - t0
    h2d = ds.N * ds.K * 4 + ds.N * 8
    return {"value": grads / dt, "unit": "grad evals/s", "h2d_bytes_per_step": h2d,
            "d2h_bytes_per_step": d2h // max(args.steps, 1)}


def precision_errors(model, res, precision, n_theta=64):
    """Mixed form against the FP64 form (itself pinned to the oracle at 1e-12)
    at the fit's final draws: max relative log p error and gradient error
    (2-norm) over n_theta seeded draws, and |H_mixed - H_fp64| per transition
    end state (equal to the log p difference: the kinetic term is shared)."""
    C, D = res.draws.shape[0], model.D
    last = np.stack([res.draws[c, max(int(res.n_rows[c]) - 1, 0), 7:] for c in range(C)])
    th = np.stack([model.unconstrain_array(last[c]) for c in range(C)])
    lp_m, g_m = model.log_prob_grad_batch(th, precision)
    lp_d, g_d = model.log_prob_grad_batch(th, "fp64")
    sel = np.random.default_rng(64).choice(C, size=min(n_theta, C), replace=False)
    lp_rel = np.abs(lp_m[sel] - lp_d[sel]) / np.abs(lp_d[sel])
    g_rel = np.linalg.norm(g_m[sel] - g_d[sel], axis=1) / np.linalg.norm(g_d[sel], axis=1)
    dh = np.abs(lp_m - lp_d)
    return {"vs": "fp64 GPU form", "n_theta": int(len(sel)),
            "lp_max_rel": float(lp_rel.max()), "grad_max_rel": float(g_rel.max()),
            "energy_abs_diff": {"n": int(C), "median": float(np.median(dh)),
                                "p99": float(np.percentile(dh, 99)), "max": float(dh.max())}}


def config_d_leg():
    """Poisson GLM, N = 262144, K = 512, X stored bf16, 512 chains: gradient
    time of each form inside a short fit (CUDA events), and the mixed forms'
    errors against the FP64 form at 64 seeded points."""
    from stan_gb300 import Model, sampler, workloads
    ds = workloads.make_dataset("poisson", seed=1)
    m = Model.from_dataset(ds)
    C = 512
    out = {"workload": "Poisson GLM N=262144 K=512, X bf16, 512 chains",
           "flops_per_grad": 4.0 * ds.N * ds.K * C}
    for prec in ("bf16x3", "bf16", "fp32"):
        sampler.run(m, num_chains=C, num_warmup=4, num_samples=0, precision=prec,
                    random_seed=1, init_radius=0.5)
        r = sampler.run(m, num_chains=C, num_warmup=10, num_samples=0, precision=prec,
                        random_seed=2, init_radius=0.5)
        out[prec] = {"grad_ms": r.grad_ms,
                     "tflops": out["flops_per_grad"] / (r.grad_ms * 1e-3) / 1e12}
    th = np.random.default_rng(3).normal(size=(64, m.D)) * 0.05
    lp64, g64 = m.log_prob_grad_batch(th, "fp64")
    for prec in ("bf16x3", "bf16", "fp32"):
        lp, g = m.log_prob_grad_batch(th, prec)
        out[prec]["lp_max_rel"] = float(np.max(np.abs(lp - lp64) / np.abs(lp64)))
        out[prec]["grad_max_rel"] = float(np.max(np.linalg.norm(g - g64, axis=1) /
                                                 np.linalg.norm(g64, axis=1)))
    m.close()
    return out


def csv_leg(model, res, chains=256):
    """Stan CSV output of the headline fit through the native writer
    (gbnuts_write_run with gbnuts_csv_open's callbacks: the service protocol,
    values at 6 significant digits) for its first `chains` chains, written to a
    temporary directory and removed: once with the chains formatted
    concurrently on the host cores and once on one thread."""
    import ctypes
    import shutil
    import tempfile
    from stan_gb300 import _lib
    from stan_gb300.callbacks import CsvFiles
    cfg, out = res._run
    sub = type(cfg).from_buffer_copy(cfg)
    sub.num_chains = min(chains, cfg.num_chains)
    rows = int(res.n_rows[:sub.num_chains].sum())
    report = {"chains": int(sub.num_chains), "rows": rows, "columns": int(out.n_cols),
              "host_threads": os.cpu_count()}
    for label, concurrent in (("concurrent", 1), ("one_thread", 0)):
        d = tempfile.mkdtemp(prefix="gbnuts_csv_")
        try:
            csv = CsvFiles(os.path.join(d, "out"))
            t0 = time.perf_counter()
            cb = csv.open(sub.num_chains, sub.init_chain_id)
            cb.chains_concurrent = concurrent
            rc = _lib.load().gbnuts_write_run(model.handle, ctypes.byref(sub), ctypes.byref(out),
                                              ctypes.byref(cb))
            csv.close()
            dt = time.perf_counter() - t0
            _lib.check(rc, "gbnuts_write_run")
            nbytes = sum(os.path.getsize(os.path.join(d, f)) for f in os.listdir(d))
        finally:
            shutil.rmtree(d, ignore_errors=True)
        report[label] = {"seconds": dt, "bytes": nbytes, "MB_per_s": nbytes / dt / 1e6,
                         "rows_per_s": rows / dt}
    # The service writing the same kind of files for a fresh `chains`-chain
    # fit: its rows are formatted while the device run goes on (the host
    # drain), so the call takes about the fit's own time; the array run of
    # the same fit, and writing its rows after it, for comparison.
    from stan_gb300 import sampler, services
    n_c = int(sub.num_chains)
    kw = dict(random_seed=31, init_chain_id=1, init_radius=2.0, num_warmup=int(sub.num_warmup),
              num_samples=int(sub.num_samples), num_thin=1, save_warmup=0, stepsize=1.0,
              stepsize_jitter=0.0, max_depth=10, delta=0.8, gamma=0.05, kappa=0.75, t0=10.0,
              init_buffer=75, term_buffer=50, window=25)
    prec = {v: k for k, v in _lib.PRECISIONS.items()}[int(sub.precision)]
    d = tempfile.mkdtemp(prefix="gbnuts_csv_")
    try:
        t0 = time.perf_counter()
        rc = services.hmc_nuts_diag_e_adapt(model, n_c, None, None, refresh=0, precision=prec,
                                            csv=CsvFiles(os.path.join(d, "svc")), **kw)
        t_svc = time.perf_counter() - t0
        _lib.check(rc, "gbnuts_hmc_nuts_diag_e_adapt")
        svc_bytes = sum(os.path.getsize(os.path.join(d, f)) for f in os.listdir(d))
    finally:
        shutil.rmtree(d, ignore_errors=True)
    t0 = time.perf_counter()
    r = sampler.run(model, num_chains=n_c, precision=prec, **kw)
    t_arr = time.perf_counter() - t0
    d = tempfile.mkdtemp(prefix="gbnuts_csv_")
    try:
        t0 = time.perf_counter()
        sampler.write_csv(model, r, CsvFiles(os.path.join(d, "arr")))
        t_write = time.perf_counter() - t0
    finally:
        shutil.rmtree(d, ignore_errors=True)
    report["service_drained"] = {
        "chains": n_c, "bytes": svc_bytes, "service_call_s": t_svc,
        "array_run_call_s": t_arr, "array_run_device_s": r.total_ms / 1e3,
        "write_after_run_s": t_write,
        "note": "service_call_s includes the run, formatting its rows while it goes on, and "
                "the rest after it; array_run_call_s + write_after_run_s is the same work "
                "done one after the other"}
    return report


def fp64_rate(model, ds, C):
    """The plain FP64 form on the same workload: gradient evaluations per
    second over a bounded prefix of the fit (its warmup), not a full fit."""
    from stan_gb300 import sampler
    res = sampler.run(model, num_chains=C, num_warmup=20, num_samples=0, adapt=True,
                      precision="fp64", random_seed=7, init_radius=2.0)
    return {"grad_evals_per_s": float(res.n_grad.sum()) / (res.total_ms / 1e3),
            "sample": f"{C} chains x 20 warmup iterations", "grad_kernel_ms": res.grad_ms}


# The default serving leg: 100 fits at 1 fit/s, about 70 % of the mixed form's
# measured capacity on this stream, so latency is service time, not a growing queue.
SERVING = dict(fits=100, rate=1.0, chains=4, warmup=300, samples=500, steps_per_call=32,
               forms=("fp32",))


def serving_leg(n_fits=None, rate=None, forms=None):
    """Continuous batching on the serving stream (N log-uniform in [200, 5e4],
    K in {8, ..., 128}, data at prior draws, 4 chains, 300 + 500): fits
    arrive as a Poisson process and run in one pool per form; p50 / p99
    latency (arrival to every draw and its on-device convergence summary (ESS,
    R-hat, MCSE) on the host) and
    fits/s, for the mixed
    (fp32 gradients, FP64 control) and the plain FP64 form."""
    from stan_gb300 import workloads
    from stan_gb300.serving import Pool, poisson_arrivals, serve
    S = SERVING
    forms = forms or S["forms"]
    n_fits = n_fits or S["fits"]
    rate = rate or S["rate"]
    dss = workloads.serving_stream(n_fits)
    kw = dict(num_chains=S["chains"], num_warmup=S["warmup"], num_samples=S["samples"],
              random_seed=1, max_depth=10, delta=0.8, report_summary=True)
    arrivals = poisson_arrivals(rate, len(dss), seed=1)
    out = {"workload": f"{n_fits} hierarchical logistic fits (N log-uniform 200-50000, K in "
                       f"8/16/32/64/128, J = N/50, y at prior draws), {S['chains']} chains, "
                       f"{S['warmup']} warmup + {S['samples']} draws",
           "arrival_rate_per_s": rate, "latency_unit": "s",
           "latency": "arrival to the fit's draws and convergence summary (ESS, R-hat, MCSE) "
                      "in host memory"}
    for form in forms:
        pool = Pool(precision=form, x_dtype="f32", max_fits=512, reserve_bytes=2 << 30)
        pool.submit(dss[0], **dict(kw, num_warmup=20, num_samples=0))  # warm-up fit
        pool.run_all()
        ess, rhat = {}, {}

        def done(i, r):
            ess[i] = float(np.nanmin(r.summary[:, 0]))
            rhat[i] = float(np.nanmax(r.summary[:, 2:4]))

        rep = serve(pool, dss, arrivals, steps_per_call=S["steps_per_call"], run_kwargs=kw,
                    on_done=done)
        pool.close()
        summ = rep.summary()
        # convergence report computed on the device as each fit retires
        summ["min_bulk_ess_median_over_fits"] = float(np.median(list(ess.values())))
        summ["max_rhat_median_over_fits"] = float(np.median(list(rhat.values())))
        summ["max_rhat_max_over_fits"] = float(np.max(list(rhat.values())))
        out["mixed" if form == "fp32" else "fp64"] = summ
    if "fp32" in forms:
        out["precision_errors"] = serving_precision(dss, kw)
    return out


def serving_precision(dss, kw, n=6):
    """The mixed serving form's errors against the FP64 form on a spread of
    the stream's fits (smallest to largest N): each fit runs alone in the
    fp32 form with the stream's schedule, then at its chains' final draws
    (and 64 points around them) log p and the gradient of both forms are
    compared; the largest over the fits."""
    from stan_gb300 import Model, sampler
    order = np.argsort([d.N for d in dss])
    pick = [int(order[int(round(i * (len(dss) - 1) / (n - 1)))]) for i in range(n)]
    lp_max, g_max, dh = 0.0, 0.0, []
    for i in pick:
        m = Model.from_dataset(dss[i])
        r = sampler.run(m, precision="fp32", **{k: v for k, v in kw.items() if k != "report_summary"})
        C = r.draws.shape[0]
        last = np.stack([r.draws[c, max(int(r.n_rows[c]) - 1, 0), 7:] for c in range(C)])
        th0 = np.stack([m.unconstrain_array(last[c]) for c in range(C)])
        th = th0[np.random.default_rng(i).integers(0, C, 64)] + \
            np.random.default_rng(i + 1).normal(size=(64, m.D)) * 0.01
        th = np.concatenate([th0, th])
        lp32, g32 = m.log_prob_grad_batch(th, "fp32")
        lp64, g64 = m.log_prob_grad_batch(th, "fp64")
        lp_max = max(lp_max, float(np.max(np.abs(lp32 - lp64) / np.abs(lp64))))
        g_max = max(g_max, float(np.max(np.linalg.norm(g32 - g64, axis=1) /
                                        np.linalg.norm(g64, axis=1))))
        dh.extend(np.abs(lp32[:C] - lp64[:C]).tolist())
        m.close()
    return {"vs": "fp64 GPU form", "fits": [int(dss[i].N) for i in pick],
            "n_theta_per_fit": 64 + int(kw["num_chains"]), "lp_max_rel": lp_max,
            "grad_max_rel": g_max,
            "energy_abs_diff": {"n": len(dh), "median": float(np.median(dh)),
                                "max": float(np.max(dh))}}


def _moment_z(d_a, d_b):
    """Largest |difference| / combined MCSE over parameters, of posterior means
    and of posterior sds (mcse.hpp:22-61 estimates on each run's draws)."""
    from stan_gb300 import analyze
    zm, zs = 0.0, 0.0
    for j in range(d_a.shape[2]):
        a, b = d_a[:, :, j], d_b[:, :, j]
        se_m = np.hypot(analyze.mcse_mean(a), analyze.mcse_mean(b))
        se_s = np.hypot(analyze.mcse_sd(a), analyze.mcse_sd(b))
        zm = max(zm, abs(a.mean() - b.mean()) / se_m)
        zs = max(zs, abs(a.std() - b.std()) / se_s)
    return zm, zs


def fp64_fit_leg(chains=128, mixed="f16x3"):
    """The plain FP64 form and the mixed form, each a complete fit of the
    benchmark's design (N = 1e5, K = 100, 500 warmup + 1000 draws) with
    `chains` chains: measured min bulk ESS/s (fit wall time on the device),
    gradient evaluations/s, their ratio, and the posterior moments of the two
    runs compared in MCSE units."""
    from stan_gb300 import Model, sampler, workloads
    ds = workloads.make_dataset("logistic_100k", seed=1)
    m = Model.from_dataset(ds)
    kw = dict(num_chains=chains, num_warmup=500, num_samples=1000, adapt=True, max_depth=10,
              delta=0.8, init_radius=2.0, random_seed=4242)
    out = {"workload": f"logistic GLM N={ds.N} K={ds.K} X fp32, {chains} chains, "
                       "500 warmup + 1000 draws"}
    draws = {}
    for form in ("fp64", mixed):
        res = sampler.run(m, precision=form, **kw)
        g, sec, ess, which = fit_stats(res, ds)
        out[form] = {"fit_seconds": sec, "grad_evals_per_s": g / sec, "min_bulk_ess": ess,
                     "min_bulk_ess_per_s": ess / sec, "min_ess_param": which,
                     "grad_kernel_ms": res.grad_ms, "status_ok": bool(np.all(res.status == 0))}
        draws[form] = res.sampling_draws()[:, :, 7:]
    out["mixed_over_fp64_min_bulk_ess_per_s"] = (out[mixed]["min_bulk_ess_per_s"] /
                                                 out["fp64"]["min_bulk_ess_per_s"])
    zm, zs = _moment_z(draws["fp64"], draws[mixed])
    out["moments_max_z"] = {"mean": zm, "sd": zs, "bound": 4.0}
    m.close()
    return out


def config_c_leg(precision="fp32"):
    """Config C: non-centred hierarchical normal, J = 2000 groups (~42k rows),
    K = 10, D = 2013, 256 chains, 500 warmup + 1000 draws, in the given form:
    fit time, gradient evaluations/s, min bulk ESS/s, the gradient launch
    time, and the form's errors against the FP64 GPU form at the chains'
    final draws (lp, gradient 2-norm, |delta H| per chain)."""
    from stan_gb300 import Model, sampler, workloads
    ds = workloads.make_dataset("hier_normal", seed=1)
    m = Model.from_dataset(ds)
    kw = dict(num_chains=256, num_warmup=500, num_samples=1000, adapt=True, max_depth=10,
              delta=0.8, init_radius=2.0)
    sampler.run(m, precision=precision, random_seed=1, **dict(kw, num_warmup=20, num_samples=0))
    res = sampler.run(m, precision=precision, random_seed=4321, **kw)
    g, sec, ess, which = fit_stats(res, ds)
    out = {"workload": f"hierarchical normal J={ds.J} (N={ds.N}) K={ds.K} D={m.D}, 256 chains, "
                       "500 warmup + 1000 draws",
           "precision": precision, "fit_seconds": sec, "grad_evals_per_s": g / sec,
           "min_bulk_ess": ess, "min_bulk_ess_per_s": ess / sec, "min_ess_param": which,
           "grad_kernel_ms": res.grad_ms, "ms_per_step": res.total_ms / max(res.steps, 1),
           "status_ok": bool(np.all(res.status == 0))}
    if precision != "fp64":
        out["precision_errors"] = precision_errors(m, res, precision)
    m.close()
    return out


def config_a_leg(reps=3):
    """The drop-in case: logistic N = 1000, K = 25 (X fp64), 4 chains, 1000
    warmup + 1000 draws, FP64, adaptive.  The GPU form through the array API
    (device time, CUDA events) against the CPU restatement of the reference
    sampler running the same 4 chains on 4 host threads (wall time); min bulk
    ESS/s and gradient evaluations/s on both sides, and the GPU's time per
    step (one step-kernel launch and one gradient launch; steps run in
    captured CUDA-graph chunks)."""
    import oracle
    from stan_gb300 import Model, analyze, sampler, workloads
    ds = workloads.make_dataset("logistic", seed=1)
    m = Model.from_dataset(ds)
    kw = dict(num_chains=4, num_warmup=1000, num_samples=1000, adapt=True, max_depth=10,
              delta=0.8, init_radius=2.0)
    sampler.run(m, precision="fp64", random_seed=1, **dict(kw, num_warmup=50, num_samples=10))
    gpu = []
    for i in range(reps):
        res = sampler.run(m, precision="fp64", random_seed=100 + i, **kw)
        g, sec, ess, _ = fit_stats(res, ds)
        gpu.append({"fit_seconds": sec, "grad_evals_per_s": g / sec, "min_bulk_ess_per_s": ess / sec,
                    "ms_per_step": res.total_ms / max(res.steps, 1), "steps": int(res.steps),
                    "grad_kernel_ms": res.grad_ms})
    om = oracle.OracleModel(ds.kind, ds.X, ds.y, hp=list(ds.hp), intercept=ds.intercept,
                            compensated=False)
    cpu = []
    for i in range(reps):
        t0 = time.perf_counter()
        r = om.sample(seed=100 + i, num_threads=4, **{k: v for k, v in kw.items()
                                                       if k != "num_chains"}, num_chains=4)
        dt = time.perf_counter() - t0
        rows = r["rows"][:, -1000:]
        q = np.concatenate([rows[:, :, 0:1], rows[:, :, 7:]], axis=2).transpose(1, 0, 2)
        ess, _ = analyze.min_bulk_ess(q)
        cpu.append({"fit_seconds": dt, "grad_evals_per_s": float(r["n_grad_total"].sum()) / dt,
                    "min_bulk_ess_per_s": ess / dt})
    med = lambda rs, k: float(np.median([x[k] for x in rs]))  # noqa: E731
    m.close()
    return {"workload": "logistic GLM N=1000 K=25 X fp64, 4 chains, 1000 warmup + 1000 draws, "
                        "FP64, adaptive",
            "gpu_fp64": {k: med(gpu, k) for k in gpu[0]},
            "cpu_reference_restatement": dict({k: med(cpu, k) for k in cpu[0]},
                                              threads=4, cores=os.cpu_count()),
            "reps": reps}


def run_reference(args, ws, rank):
    from stan_gb300 import workloads
    wl = WORKLOADS[args.workload]
    ds = workloads.make_dataset(wl["kind"], seed=1)
    for _ in range(args.warmup):
        cpu_baseline(ds, wl, 2.0, 0.02)
    vals, samples = [], None
    for _ in range(args.steps):
        r = cpu_baseline(ds, wl, args.cpu_seconds, 0.02)
        vals.append(r["value"])
        samples = r
    v = float(np.mean(vals))
    return {"impl": "reference", "metric": "grad evals/s", "value": v, "unit": "grad evals/s",
            "n_gpus": ws, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": args.workload,
                       "note": "the reference cannot be built here (Stan Math, Eigen, Boost absent); "
                               "its sampler is timed through the CPU restatement in oracle/"},
            "cpu_baseline": {"value": v, "unit": "grad evals/s", "cores": samples["cores"],
                             "kind": "port", "sample": samples["sample"]},
            "e2e": {"value": v, "unit": "grad evals/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}


def profile_case(args):
    """Small, self-terminating invocations of the workload's kernels, for ncu."""
    from stan_gb300 import Model, _lib, sampler, workloads
    wl = WORKLOADS[args.workload]
    ds = workloads.make_dataset(wl["kind"], seed=1)
    _lib.load(build_if_missing=False)
    model = Model.from_dataset(ds)
    C = wl["chains"]
    if args.case == "grad":
        th = np.random.default_rng(0).normal(size=(C, model.D)) * 0.05
        for _ in range(2):
            lp, _g = model.log_prob_grad_batch(th, args.precision)
        print(json.dumps({"case": "grad", "chains": C, "lp0": float(lp[0])}))
    else:
        r = sampler.run(model, num_chains=C, num_warmup=args.short_iters, num_samples=0,
                        precision=args.precision, random_seed=1)
        print(json.dumps({"case": "shortfit", "steps": int(r.steps), "ms": r.total_ms}))


_dist = None


def _init_dist(ws):
    global _dist
    if ws > 1 and _dist is None:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo")
        _dist = dist
    return _dist


def barrier(ws):
    d = _init_dist(ws)
    if d:
        d.barrier()


def max_over_ranks(x, ws):
    d = _init_dist(ws)
    if not d:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    d.all_reduce(t, op=d.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(x, ws):
    d = _init_dist(ws)
    if not d:
        return x
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64)
    d.all_reduce(t, op=d.ReduceOp.SUM)
    return float(t.item())


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="logistic_100k", choices=list(WORKLOADS))
    ap.add_argument("--precision", default="f16x3", choices=["fp64", "fp32", "bf16x3", "f16x3"])
    ap.add_argument("--cpu-seconds", type=float, default=20.0)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-serving", action="store_true")
    ap.add_argument("--no-config-d", action="store_true")
    ap.add_argument("--no-csv", action="store_true")
    ap.add_argument("--no-config-a", action="store_true")
    ap.add_argument("--no-config-c", action="store_true")
    ap.add_argument("--serving-fits", type=int, default=None)
    ap.add_argument("--serving-rate", type=float, default=None)
    ap.add_argument("--serving-forms", default="fp32",
                    help="comma list of the serving leg's gradient forms (fp32: mixed)")
    ap.add_argument("--fp64-fit-chains", type=int, default=128)
    ap.add_argument("--case", default="fit",
                    choices=["fit", "grad", "shortfit", "serving", "fp64fit", "config_a",
                             "config_c"],
                    help="fit: the benchmark; grad: two batched-gradient launches of the "
                         "workload (for kernel captures); shortfit: a fit of --short-iters "
                         "warmup iterations (for launch lists)")
    ap.add_argument("--short-iters", type=int, default=40)
    args = ap.parse_args()
    if args.case == "serving":
        print(json.dumps(serving_leg(args.serving_fits, args.serving_rate,
                                     tuple(args.serving_forms.split(",")))))
        return
    if args.case == "fp64fit":
        print(json.dumps(fp64_fit_leg(args.fp64_fit_chains)))
        return
    if args.case == "config_a":
        print(json.dumps(config_a_leg()))
        return
    if args.case == "config_c":
        print(json.dumps(config_c_leg(args.precision if args.precision != "f16x3" else "fp32")))
        return
    if args.case != "fit":
        profile_case(args)
        return
    ws, rank, local = dist_env()
    if args.impl == "reference":
        if rank != 0:
            return
        print(json.dumps(run_reference(args, ws, rank)))
        return
    gpu = select_device(ws, local)
    out = run_ours(args, ws, rank, gpu)
    if rank == 0:
        print(json.dumps(out))


if __name__ == "__main__":
    main()
