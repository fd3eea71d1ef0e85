"""Benchmark: chi^2 evaluations/s of the fitting hot path on one GB300 (config 2 by default).

Workload (config 2 of the benchmark set): a 2000-point, 3-filter light curve over 60 days with
INTERP ephemerides, TORQUE + P_PSI + ACC + NUDGE, TIME_STEP 5e-3, fitted by 65536 random-start
simplex chains of 20000 chi^2 evaluations each.  The full job (1.3e9 evaluations) takes far
longer than a benchmark may run, so a "step" is one resumable launch of the persistent simplex
kernel in which every chain slot performs a fixed number of evaluations at full per-evaluation
cost; `value` is the evaluations of the timed steps over their device time.

Keys beyond the driver's contract:
  fp64        the plain FP64 path on the same workload (evals/s) and mixed/fp64 speed-up
  accuracy    |dchi2|/chi2 of the mixed path against the FP64 path on sampled vectors
  roofline    algorithmic flops per evaluation x evals/s against the measured FMA peak
  cpu_baseline  the oracle port on the host cores (bounded sample)
  e2e         chi^2 evals/s through ast_eval_batch with host buffers (copies included)

--impl reference times the CPU implementation of the path (the oracle port of the reference's
chi2one; the reference's own host build is x86-only and does not run on the Arm host) on all
host cores, same metric and workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "chi2_evals_per_s"
UNIT = "evals/s"


# Executed work per evaluation on the config-2 workload, from ncu captures of the two fit
# kernels (sm__sass_thread_inst_executed_op_{ffma,fadd,fmul}_pred_on.sum and the d* FP64
# counterparts, dram__bytes_read.sum + dram__bytes_write.sum): FP32 flops of the mixed path
# (FFMA x 2 + FADD + FMUL, the double-float formulation's own arithmetic; counted on the scalar
# build of the step -- the packed FP32x2 build performs the same lane operations, bit for bit,
# in fewer instructions, and those counters see only its scalar part), FP64 flops of the plain
# path (DFMA x 2 + DADD + DMUL, including the FP64 transcendental functions), and DRAM bytes of
# one launch (the slot state in and out; independent of the evaluations per slot) over the
# kernels' resident slots: 58 368 for the mixed path (three CTAs of 128 per SM), 38 912 for
# FP64.  Other workloads scale the per-evaluation figures by their RK4 step count.
NCU_C2 = {"rk4_steps": 12568, "mixed_fp32_flops": 3.37e7, "fp64_flops": 7.75e6,
          "slots": 58368, "dram_bytes_mixed": 1.619e8, "dram_bytes_fp64": 5.71e6}


def rk4_steps(obs, time_step):
    return int(np.sum(np.floor(np.diff(obs.mjd) / time_step + 1)))


def algorithmic_flops(obs, model):
    """Per-evaluation flops counted from the reference source (add/mul/div/sqrt = 1, fma = 2):
    152 per RK4 step (4 right-hand sides of 18 + 80 for the stage combinations), 156 per
    observation for the LS brightness and the filter sums, 6 per filter, 50 per-evaluation set-up.
    Transcendental calls are not counted as flops (16 per RK4 step, 14 per observation)."""
    n_rk4 = rk4_steps(obs, model.time_step)
    return 152 * n_rk4 + 156 * obs.n_data + 6 * obs.n_filters + 50, 16 * n_rk4 + 14 * obs.n_data


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, gpu_index):
        self.samples = []
        self.proc = None
        self.gpu = gpu_index

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=clocks.sm,clocks.max.sm,power.draw,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL,
                text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 7:
                self.samples.append(parts)

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for s in self.samples for k in range(4) if s[3 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch
        import torch.distributed as dist

        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    return world, rank, local, dist


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(dist, v):
    if dist is None:
        return v
    import torch

    t = torch.tensor([float(v)], device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(dist, v):
    if dist is None:
        return v
    import torch

    t = torch.tensor([float(v)], device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def make_workload(args, tmp):
    from asteroid_gb300 import synth

    return synth.generate(args.config, tmp)


def sample_vectors(model, n, seed, reopt=0):
    from asteroid_gb300 import api

    rng = np.random.default_rng(seed)
    iL = api.param_names(model).index("L")
    out = []
    while len(out) < n:
        p = api.x2params(model, rng.uniform(0, 1, model.n_params), reopt=reopt)
        if p is not None and p[iL] * model.time_step <= 0.5:
            out.append(p)
    return np.array(out)


def workload_vectors(model, n, seed, params_true=None, radius=0.02):
    """Parameter vectors of the workload: from the fit's prior, or -- for NUDGE, which the
    reference runs as a re-optimisation -- jittered by up to `radius` in every dimensionless
    coordinate around the true model."""
    from asteroid_gb300 import api

    if params_true is None or not model.flags & api.NUDGE:
        return sample_vectors(model, n, seed)
    rng = np.random.default_rng(seed)
    x0 = api.params2x(model, params_true)
    out = []
    while len(out) < n:
        p = api.x2params(model, x0 + rng.uniform(-radius, radius, model.n_params), reopt=1)
        if p is not None:
            out.append(p)
    return np.array(out)


def cpu_baseline(model, obs, seconds=15.0, params_true=None):
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle as O

    from asteroid_gb300 import build

    build.build_oracle()
    threads = O.max_threads()
    P = workload_vectors(model, 8 * threads, 99, params_true)
    t0 = time.perf_counter()
    O.chi2_batch(model, obs, P[: threads], threads=threads)  # warm
    per = (time.perf_counter() - t0) / 1.0
    n = max(threads, int(seconds / max(per, 1e-6) * threads))
    P = workload_vectors(model, n, 100, params_true)
    t0 = time.perf_counter()
    O.chi2_batch(model, obs, P, threads=threads)
    dt = time.perf_counter() - t0
    return {"value": n / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{n} parameter vectors of the workload's object, oracle chi2one restatement, OpenMP"}


def run_fit_steps(eng, precision, n_chains, group, evals_cap, budget, warmup, steps, seed, stream_events,
                  reopt=False, params0=None, target_s=1.5):
    """Warm-up + timed resumable launches; returns (evals, ms, fits, launches, budget).  With
    budget 0 the first warm-up launch (2 evaluations per slot) calibrates the budget to about
    target_s of device time per step."""
    eng.fit_begin(n_chains=n_chains, group_size=group, seed=seed, precision=precision, evals_cap=evals_cap,
                  reopt=reopt, params0=params0)
    if budget <= 0:
        t0 = time.perf_counter()
        eng.fit_step(2)
        dt = time.perf_counter() - t0
        budget = max(1, int(round(2 * target_s / max(dt, 1e-3))))
        warmup = max(0, warmup - 1)
    for _ in range(warmup):
        eng.fit_step(budget)
    e0, f0 = eng.fit_counters()
    ms, launches = stream_events(lambda: [eng.fit_step(budget) for _ in range(steps)])
    e1, f1 = eng.fit_counters()
    eng.fit_end()
    return e1 - e0, ms, f1 - f0, steps, budget


def run_batch_steps(s, precision, n_chains, group, evals_cap, budget, warmup, steps, seed, stream_events, reopt,
                    params0):
    """Evaluations/s of bounded ast_batch_step launches with the workload as one batch object."""
    from asteroid_gb300 import api

    kw = dict(n_chains=n_chains, group_size=group, seed=seed, evals_cap=evals_cap)
    if reopt:
        kw.update(reopt=True, params0=params0)
    with api.Batch(precision=precision, acc=bool(s.model.flags & api.ACC)) as b:
        b.add(s.model, s.obs, **kw)
        for _ in range(warmup):
            b.step(budget)
        e0 = b.counters()["n_evals"]
        t = [0.0]

        def go():
            for _ in range(steps):
                t[0] += b.step(budget)[1]

        stream_events(go)
        e1 = b.counters()["n_evals"]
    return (e1 - e0) / (t[0] * 1e-3)


def measure_fits(device, chains=4096, evals=2000, seed=777, precisions=("mixed",), polish_evals=300):
    """Completed fits per second, measured: config 0 (300 points, LS + TORQUE + P_PSI, FP64
    simplex) run to completion -- `chains` random-start chains of `evals` chi^2 evaluations each
    (ast_fit, one stage, groups of 256) -- in each of `precisions`; device time of the simplex
    launches.  A fit is one chain, as in the reference (one chain per thread).  4096 chains fill
    a fraction of the GPU, so a chain's evaluations run at their latency: the FP64 run takes
    minutes (bench.py --mode fits), the mixed one seconds."""
    from asteroid_gb300 import api, synth

    with tempfile.TemporaryDirectory() as d:
        s = synth.generate("c0acc", d)
        out = {"workload": f"c0: {s.obs.n_data} points, {api.flag_names(s.model.flags)}, {chains} chains x "
                           f"{evals} evals, one stage, run to completion"}
        with api.Engine(s.model, s.obs, device=device) as eng:
            eng.fit(n_chains=256, group_size=256, seed=seed, evals_cap=20)  # warm-up
            res = {}
            for prec, name in ((api.PREC_MIXED, "mixed"), (api.PREC_FP64, "fp64")):
                if name not in precisions:
                    continue
                r = eng.fit(n_chains=chains, group_size=256, seed=seed, evals_cap=evals, precision=prec)
                res[name] = r
                sec = r.kernel_ms * 1e-3
                out[name] = {"fits_per_s": r.n_fits / sec, "evals_per_s": r.n_evals / sec, "seconds": sec,
                             "n_fits": r.n_fits, "n_evals": r.n_evals, "best_chi2": float(r.best_f.min())}
            # The mixed search's result against FP64: the chi^2 of its best parameters in FP64, and
            # the parameter error -- the same re-optimisation (-reopt from the mixed best, 256
            # chains, same seed, same start simplexes) run once in each precision; the distance
            # between the two optima, in the fit's dimensionless coordinates x, is where the mixed
            # arithmetic moves the answer.
            m = res["mixed"]
            p_mixed = m.best_params[int(np.argmin(m.best_f))]
            c64, _ = eng.eval(p_mixed[None, :], api.PREC_FP64)
            pol = {}
            for prec, name in ((api.PREC_MIXED, "mixed"), (api.PREC_FP64, "fp64")):
                pol[name] = eng.fit(n_chains=256, group_size=256, seed=seed + 1, evals_cap=polish_evals, reopt=True,
                                    params0=p_mixed, precision=prec, fp64_result=True)
            pm, p64 = pol["mixed"].best_params[0], pol["fp64"].best_params[0]
            dx = np.abs(api.params2x(s.model, pm) - api.params2x(s.model, p64))
            out["mixed_result_vs_fp64"] = {
                "chi2_mixed": float(m.best_f.min()), "chi2_fp64_at_mixed_params": float(c64[0]),
                "rel_chi2_error": float(abs(m.best_f.min() - c64[0]) / c64[0]),
                "reoptimised_chi2_fp64_of_mixed": float(pol["mixed"].best_f[0]),
                "reoptimised_chi2_fp64": float(pol["fp64"].best_f[0]),
                "max_abs_dx": float(dx.max()), "dx": dx.tolist(),
                "params_mixed": pm.tolist(), "params_fp64": p64.tolist(),
                "note": f"parameter error: one re-optimisation from the mixed best (-reopt, 256 chains x "
                        f"{polish_evals} evaluations, same seed and start simplexes) in each precision; "
                        f"|x_mixed - x_fp64| per parameter in the fit's x coordinates, chi^2 of both in FP64"}
    return out


def wrap(a):
    return (a + np.pi) % (2 * np.pi) - np.pi


def phase_drift(eng, model, obs, truth, vectors):
    """Largest |mixed - FP64| Euler angle (rad, modulo 2 pi) over the light curve, for the true
    model and a few workload vectors, and the total rotation phase the FP64 path accumulates."""
    from asteroid_gb300 import api

    out = {"max_rad": 0.0, "at_last_point_rad": 0.0, "total_phase_rad": 0.0,
           "span_days": float(obs.mjd[-1] - obs.mjd[0]), "vectors": 0}
    for p in np.vstack([truth, vectors]):
        a64 = eng.model_angles(p, api.PREC_FP64)
        a32 = eng.model_angles(p, api.PREC_MIXED)
        if not (np.all(np.isfinite(a64)) and np.all(np.isfinite(a32))):
            continue
        d = np.abs(wrap(a32 - a64))
        out["max_rad"] = max(out["max_rad"], float(d.max()))
        out["at_last_point_rad"] = max(out["at_last_point_rad"], float(d[-1].max()))
        out["total_phase_rad"] = max(out["total_phase_rad"], float(np.abs(a64[-1] - a64[0]).max()))
        out["vectors"] += 1
    return out


def bench_compare(args, tmp, rank, world):
    """Full fits of one configuration in both precisions at the same seed: the best-chi^2
    distributions over groups, the best parameters, and the mixed best re-evaluated in FP64
    (simplex trajectories legitimately diverge between precisions, so runs are compared by their
    distributions, not chain by chain)."""
    from asteroid_gb300 import api

    s = make_workload(args, tmp)
    reopt = bool(s.model.flags & api.NUDGE)
    kw = dict(n_chains=args.chains, group_size=256, n_stages=1, seed=4242, evals_cap=args.evals_cap)
    if reopt:
        kw.update(reopt=True, params0=s.params_true)
    out = {"mode": "compare", "config": args.config, "chains": args.chains, "evals_cap": args.evals_cap,
           "model": api.flag_names(s.model.flags), "n_data": s.obs.n_data}
    names = api.param_names(s.model)
    with api.Engine(s.model, s.obs) as eng:
        res = {}
        for prec, name in ((api.PREC_MIXED, "mixed"), (api.PREC_FP64, "fp64")):
            r = eng.fit(precision=prec, **kw)
            res[name] = r
            out[name] = {"best_chi2": float(r.best_f[r.best]), "kernel_s": r.kernel_ms * 1e-3, "evals": r.n_evals,
                         "evals_per_s": r.n_evals / (r.kernel_ms * 1e-3),
                         "group_chi2_quantiles": [float(q) for q in np.quantile(r.best_f, [0.1, 0.5, 0.9])]}
        m, d = res["mixed"], res["fp64"]
        c64, _ = eng.eval(m.best_params[m.best][None, :], api.PREC_FP64)
        out["mixed_best_reevaluated_fp64_rel"] = float(abs(m.best_f[m.best] - c64[0]) / abs(c64[0]))
        out["best_chi2_rel_diff"] = float(abs(m.best_f[m.best] - d.best_f[d.best]) / d.best_f[d.best])
        out["best_params"] = {n: [float(a), float(b)] for n, a, b in zip(names, m.best_params[m.best],
                                                                          d.best_params[d.best])}
    out["note"] = "both runs fill only n_chains slots; the rates are not the saturated throughput"
    print(json.dumps(out))


def bench_batch(args, tmp, rank, world):
    """Config 3: uneven objects (log-uniform 50-2000 points, 1-4 filters, 3-60 day spans, LS+TORQUE
    / BC / BW_BALL) with 1024 chains each, as one batch: the autotuner's choice over thread per
    model (refill 1), warp per object (refill 32) and warp per model with observation tiles (tile
    8/16/32), then bounded timed launches (evals/s) of the tuned geometry and of each mapping,
    FP64 beside it, and one graph-captured run to completion of the whole batch at
    --graph-evals evaluations per chain."""
    from asteroid_gb300 import api, synth

    objs = synth.generate_batch(args.objects, tmp)
    line = {"metric": METRIC, "unit": UNIT, "mode": "batch", "objects": len(objs), "chains_per_object": 1024,
            "data": "synthetic (config-3 generator)"}

    def timed_steps(prec, geometry=None):
        with api.Batch(precision=prec, acc=True) as b:
            for k, s in enumerate(objs):
                b.add(s.model, s.obs, n_chains=1024, group_size=256, seed=17 + k, evals_cap=5000)
            tune = b.tune(evals_per_slot=2) if geometry is None else None
            if geometry is not None:
                b.set_geometry(**geometry)
            budget = 4 if prec == api.PREC_MIXED else 2
            for _ in range(args.warmup):
                b.step(budget)
            e0 = b.counters()["n_evals"]
            ms = 0.0
            for _ in range(args.steps):
                ms += b.step(budget)[1]
            c = b.counters()
            geo = {k: c[k] for k in ("tpb", "refill", "tile", "ctas")}
            return {"value": (c["n_evals"] - e0) / (ms * 1e-3), "tuned": tune, "geometry": geo,
                    "timed_evals": c["n_evals"] - e0, "ms": ms}

    if args.profile:
        # Only the warp-tiled kernel on this batch (the command profiled under ncu).
        print(json.dumps({"profile": "batch_tile_kernel",
                          **timed_steps(api.PREC_MIXED, dict(tpb=64, refill=32, tile=16))}))
        return
    if not args.graph_only:
        line["mixed"] = timed_steps(api.PREC_MIXED)
        line["fp64"] = timed_steps(api.PREC_FP64)
        line["speedup_mixed_over_fp64"] = line["mixed"]["value"] / line["fp64"]["value"]
    # Each mapping of the mixed path, measured the same way.
    line["mappings"] = {} if args.graph_only else {
        "thread_per_model": timed_steps(api.PREC_MIXED, dict(tpb=128, refill=1, tile=0)),
        "warp_per_object": timed_steps(api.PREC_MIXED, dict(tpb=128, refill=32, tile=0)),
        "warp_per_model_tile8": timed_steps(api.PREC_MIXED, dict(tpb=64, refill=32, tile=8)),
        "warp_per_model_tile16": timed_steps(api.PREC_MIXED, dict(tpb=64, refill=32, tile=16)),
        "warp_per_model_tile32": timed_steps(api.PREC_MIXED, dict(tpb=64, refill=32, tile=32)),
    }
    # The whole batch in one graph-captured persistent launch to completion.
    with api.Batch(precision=api.PREC_MIXED, acc=True) as b:
        for k, s in enumerate(objs):
            b.add(s.model, s.obs, n_chains=1024, group_size=256, seed=17 + k, evals_cap=args.graph_evals)
        tune = b.tune(evals_per_slot=2)
        ms = b.run()
        c = b.counters()
        line["graph_run"] = {"evals_cap": args.graph_evals, "ms": ms, "evals": c["n_evals"], "fits": c["n_fits"],
                             "evals_per_s": c["n_evals"] / (ms * 1e-3), "fits_per_s": c["n_fits"] / (ms * 1e-3),
                             "tuned": tune, "geometry": c}
    print(json.dumps(line))


def periodogram_curve():
    """The periodogram workload: a 20000-point plot grid (NPLOT) over 60 days carrying a 0.21-day
    double wave with noise, 4809 minima, 1.16e7 intervals: 1.16e11 interval tests per call."""
    n, span = 20000, 60.0
    rng = np.random.default_rng(22)
    t = np.arange(n) * (span / (n - 1))
    return t, 0.3 * np.sin(2 * np.pi * t / 0.21) + 0.02 * rng.standard_normal(n)


# Lane instructions of one interval test in the count kernel's fast path: the product rounded to
# an integer (FFMA + FADD), the remainder (FFMA), its distance to the threshold (FADD), the sign
# bit added to the count (IADD) and the smallest distance kept (FMNMX).
PERIODOGRAM_OPS = 6


def bench_periodogram(args, tmp, rank, world):
    """The periodogram of model minima of -plot mode (minima(), misc.c:65-276): interval tests/s
    of the CUDA count, the same through ast_minima with host buffers, and the -plot sequence of
    the config-2 object (model curve on the 20000-point grid, then the periodogram)."""
    import torch

    from asteroid_gb300 import api, synth

    local = int(os.environ.get("LOCAL_RANK", "0"))
    t, vm = periodogram_curve()
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=f"cuda:{local}")
    for _ in range(max(args.warmup, 3)):
        r = api.minima(t, vm, device=local)
    kernel_ms, count_ms, call_s = [], [], []
    with Clocks(local) as clk:
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            r = api.minima(t, vm, device=local)
            call_s.append(time.perf_counter() - t0)
            kernel_ms.append(r.kernel_ms)
            count_ms.append(r.count_ms)
    tests = r.n_intervals * 10000          # the reference's interval tests
    value = tests / (statistics.mean(kernel_ms) * 1e-3)
    e2e = tests / statistics.mean(call_s)
    distinct_tests = r.n_distinct * 10000  # the tests the count kernel makes
    if args.profile:   # the periodogram calls only (for ncu)
        print(json.dumps({"mode": "periodogram", "value": value, "unit": "tests/s", "kernel_ms": kernel_ms}))
        return
    peak_ops = api.probe_peak("fp32", local) * 1e9 / 2   # FMA lane instructions/s: the issue rate
    achieved = distinct_tests / (statistics.mean(count_ms) * 1e-3) * PERIODOGRAM_OPS
    line = {"metric": "interval_tests_per_s", "value": value, "unit": "tests/s (the reference's NN x N(N-1)/2)",
            "n_gpus": 1, "steps": args.steps,
            "warmup": max(args.warmup, 3), "ms_per_step": statistics.mean(kernel_ms), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 (double-float) + f64 fallback",
            "data": "synthetic", "mode": "periodogram",
            "config": {"workload": "minima() periodogram of a 20000-point plot curve, 60 days, "
                                   f"{r.n_minima} minima, {r.n_intervals} intervals ({r.n_distinct} distinct) "
                                   "x 10000 frequencies",
                       "l2": "flushed (256 MB write) before each call; the count kernel is compute-bound"},
            "clocks": clk.summary(), "gpu_launches": 2 * args.steps,
            "e2e": {"value": e2e, "unit": "tests/s", "h2d_bytes_per_step": 16 * t.size,
                    "d2h_bytes_per_step": 4 * 10000},
            "stages_ms": {"total": statistics.mean(kernel_ms), "count": statistics.mean(count_ms),
                          "reduce_to_distinct": statistics.mean(kernel_ms) - statistics.mean(count_ms)},
            "roofline": {"bound": "instruction issue (FP32 + ALU pipes, CUDA cores)", "kernel": "interval_count_kernel",
                         "achieved": achieved / 1e12,
                         "peak": peak_ops / 1e12, "unit": "T lane-ops/s", "frac": achieved / peak_ops,
                         "traffic": None,
                         "note": f"{PERIODOGRAM_OPS} lane instructions per test of a distinct interval (the fast "
                                 "path), over the count kernel's own time; peak = one "
                                 "warp instruction per SM sub-partition per clock, taken as the FP32 FMA rate "
                                 "measured by ast_probe_peak in this run"},
            "result": {"cl_fr": list(r.cl_fr), "cl_H": list(r.cl_H)}}
    # CPU: the oracle port on all host threads, on the same curve (about 15 s on 16 cores).
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle as O

    threads = O.max_threads()
    t0 = time.perf_counter()
    fr, h, counts, n_min = O.minima(t, vm, threads=threads)
    cpu_s = time.perf_counter() - t0
    line["cpu_baseline"] = {"value": tests / cpu_s, "unit": "tests/s", "cores": threads, "kind": "port",
                            "sample": "the whole workload once (the reference's own minima() is single-threaded)"}
    line["parity"] = {"counts_equal_oracle": bool(np.array_equal(counts, r.counts)),
                      "clusters_equal_oracle": bool(np.array_equal(fr, r.cl_fr) and np.array_equal(h, r.cl_H))}
    # The -plot sequence on the config-2 object, through the public API.
    s = synth.generate("c2", tmp)
    with api.Engine(s.model, s.obs, device=local) as eng:
        tg, eg, sg = api.plot_grid(s.dir / "lc.dat", s.dir, 20000, interp=True)
        _, dv = eng.eval(np.asarray(s.params_true)[None, :])
        eng.model_curve_at(s.params_true, tg, eg, sg)
        t0 = time.perf_counter()
        curve = eng.model_curve_at(s.params_true, tg, eg, sg) + dv[0, 0]
        t1 = time.perf_counter()
        rp = api.minima(tg, curve, device=local)
        t2 = time.perf_counter()
    line["plot_c2"] = {"model_curve_ms": 1e3 * (t1 - t0), "minima_ms": 1e3 * (t2 - t1), "n_minima": rp.n_minima,
                       "cl_fr": list(rp.cl_fr)}
    print(json.dumps(line))


def reference_workload(name):
    """The config's object from tests/golden/workload_<name>.npz (tests/golden/make_workload.py)
    as (model, obs, true parameters), built without the engine library: the ast_model bytes and
    the converted observation arrays."""
    from asteroid_gb300 import api, capi

    z = np.load(ROOT / "tests" / "golden" / f"workload_{name}.npz")
    model = capi.Model.from_buffer_copy(z["model"].tobytes())
    obs = api.Obs(z["mjd"], z["v"], z["w"], z["filt"], z["e_unit"], z["s_unit"], z["eph_e"], z["eph_s"], z["eph_mjd0"],
                  z["t_min"], z["v_min"], float(z["hmjd0"][0]))
    return model, obs, z["params_true"]


def reference_vectors(O, model, n, seed, params_true, radius=0.02):
    """workload_vectors through the oracle's own x2params / params2x (the reference arm loads no
    engine code): the prior with resolved rotation, or for NUDGE a jitter around the truth."""
    from asteroid_gb300 import capi

    rng = np.random.default_rng(seed)
    out = []
    if model.flags & capi.NUDGE:
        x0 = O.params2x(model, params_true)
        while len(out) < n:
            p = O.x2params(model, x0 + rng.uniform(-radius, radius, model.n_params), reopt=1)
            if p is not None:
                out.append(p)
    else:
        iL = model.types[model.ids.L]
        while len(out) < n:
            p = O.x2params(model, rng.uniform(0, 1, model.n_params), reopt=0)
            if p is not None and p[iL] * model.time_step <= 0.5:
                out.append(p)
    return np.array(out)


def bench_reference(args):
    """The CPU implementation of the path on the host cores: the oracle port of the reference's
    chi2one (OpenMP, all threads) on the config's object, no engine code loaded."""
    from asteroid_gb300 import build

    build.build_oracle()
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle as O

    model, obs, p_true = reference_workload(args.config)
    threads = O.max_threads()
    P = reference_vectors(O, model, threads, 5, p_true)
    for _ in range(1 + args.warmup):
        O.chi2_batch(model, obs, P, threads=threads)
    t0 = time.perf_counter()
    O.chi2_batch(model, obs, P, threads=threads)
    n = max(threads, int(args.cpu_seconds * 2 / 3 / max(time.perf_counter() - t0, 1e-6) * threads))
    P = reference_vectors(O, model, n, 6, p_true)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        O.chi2_batch(model, obs, P, threads=threads)
        times.append(time.perf_counter() - t0)
    v = n * args.steps / sum(times)
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (tests/golden/workload_" + args.config + ".npz)",
            "config": {"workload": f"{args.config}: chi2one on {n} parameter vectors per step"},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"{n} vectors per step; the reference's host build is x86-only, so the "
                                       f"oracle port of its chi2one runs on this host"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "engine_library_loaded": engine_library_loaded()}
    print(json.dumps(line))


def engine_library_loaded() -> bool:
    """Whether this process has mapped libasteroid_gb300.so (Linux /proc/self/maps)."""
    try:
        return "libasteroid_gb300" in Path("/proc/self/maps").read_text()
    except OSError:
        return False


def bench_precisions(args, tmp, rank, world):
    """The three evaluation precisions on one configuration: chi^2 evaluations/s of the fit kernel
    (bounded resumable launches, the headline's timing) and the relative chi^2 error against FP64
    on the workload's vectors whose FP64 chi^2 is stable to a one-ulp move of the parameters,
    plus the Euler-angle drift of each mixed form over the light curve."""
    import torch

    from asteroid_gb300 import api

    s = make_workload(args, tmp)
    model, obs = s.model, s.obs
    reopt = bool(model.flags & api.NUDGE)
    p0 = s.params_true if reopt else None
    out = {"mode": "precisions", "config": args.config, "n_data": obs.n_data, "chains": args.chains,
           "model": api.flag_names(model.flags)}
    with api.Engine(model, obs) as eng:
        stream = torch.cuda.ExternalStream(eng.stream)

        def timed(fn):
            torch.cuda.synchronize()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            r = fn()
            b.record(stream)
            torch.cuda.synchronize()
            return a.elapsed_time(b), r

        P = np.vstack([workload_vectors(model, 2047, 11, s.params_true), s.params_true[None, :]])
        c64, _ = eng.eval(P, api.PREC_FP64)
        Q = P * (1 + np.random.default_rng(0).choice([-1.0, 1.0], size=P.shape) * 2.3e-16)
        q64, _ = eng.eval(Q, api.PREC_FP64)
        with np.errstate(invalid="ignore", divide="ignore"):
            cond = np.abs(q64 - c64) / np.abs(c64)
        good = np.isfinite(c64) & (c64 < 1e29) & (cond <= 1e-10)
        for prec, name in ((api.PREC_FP64, "fp64"), (api.PREC_MIXED, "mixed"), (api.PREC_MIXED_RHS32, "mixed_rhs32")):
            ev, ms, _, _, b = run_fit_steps(eng, prec, args.chains, 256, args.evals_cap, 0, 2, 3, 1234, timed, reopt, p0)
            row = {"evals_per_s": ev / (ms * 1e-3), "budget": b}
            if prec != api.PREC_FP64:
                c, _ = eng.eval(P, prec)
                ok = good & (c < 1e29)
                rel = np.abs(c[ok] - c64[ok]) / np.abs(c64[ok])
                drift = 0.0
                for p in P[-1:]:
                    a64, a = eng.model_angles(p, api.PREC_FP64), eng.model_angles(p, prec)
                    drift = max(drift, float(np.abs(wrap(a - a64)).max()))
                row.update({"vectors": int(ok.sum()), "median_rel": float(np.median(rel)),
                            "p99_rel": float(np.quantile(rel, 0.99)), "max_rel": float(rel.max()),
                            "frac_le_1e-6": float(np.mean(rel <= 1e-6)),
                            "true_model_rel": float(abs(c[-1] - c64[-1]) / abs(c64[-1])),
                            "true_model_angle_drift_rad": drift})
            out[name] = row
    print(json.dumps(out))


def bench_rmsd(args, tmp, rank, world):
    """RMSD confidence intervals (chi2_gpu_rms, cuda.c:2148-2389) of the config-2 object's true
    model (TORQUE + P_PSI + INTERP + ACC + NUDGE with RMSD), dx = 1e-4: RMSD models/s of the
    sampling kernel in both precisions, the same through ast_rmsd, and the oracle on the host."""
    import torch

    from asteroid_gb300 import api, capi, synth

    local = int(os.environ.get("LOCAL_RANK", "0"))
    s = synth.generate("c2", tmp)
    m = api.make_model(s.model.flags | capi.RMSD, s.model.time_step, ppsi_hours=s.cfg.ppsi_hours)
    streams = 116736  # a multiple of both kernels' resident threads (152 SMs x 3 x 128 mixed, x 256 FP64)
    line = {"metric": "rmsd_models_per_s", "unit": "models/s", "n_gpus": 1, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "data": "synthetic", "mode": "rmsd",
            "config": {"workload": f"c2 object, RMSD variant, dx 1e-4, {streams} streams", "l2": "observations in L1/L2"}}
    with api.Engine(m, s.obs, device=local) as eng:
        if args.profile:   # the sampling launches only (for ncu): one model per stream, mixed
            for k in range(args.warmup + args.steps):
                r = eng.rmsd(s.params_true, 1e-4, n_streams=streams, samples=1, seed=1, call=k,
                             precision=api.PREC_FP64 if args.precision == "fp64" else api.PREC_MIXED)
            print(json.dumps({"mode": "rmsd", "models": r["n_tot"], "kernel_ms": r["kernel_ms"]}))
            return
        for prec, name in ((api.PREC_MIXED, "mixed"), (api.PREC_FP64, "fp64")):
            r = eng.rmsd(s.params_true, 1e-4, n_streams=streams, samples=1, seed=1, precision=prec)
            per_model = r["kernel_ms"] / max(r["n_tot"], 1)
            samples = max(1, int(1500.0 / (per_model * streams)))
            for k in range(max(args.warmup, 3) - 1):
                eng.rmsd(s.params_true, 1e-4, n_streams=streams, samples=1, seed=2, call=k, precision=prec)
            ms, models, wall = 0.0, 0, 0.0
            with Clocks(local) as clk:
                for k in range(args.steps):
                    t0 = time.perf_counter()
                    r = eng.rmsd(s.params_true, 1e-4, n_streams=streams, samples=samples, seed=3, call=k,
                                 precision=prec)
                    wall += time.perf_counter() - t0
                    ms += r["kernel_ms"]
                    models += r["n_tot"]
            line[name] = {"value": models / (ms * 1e-3), "e2e": models / wall, "samples_per_stream": samples,
                          "models": models, "ms": ms, "bad_fraction": r["n_bad"] / max(r["n_tot"], 1),
                          "f0": r["f0"], "f1": r["f1"], "clocks": clk.summary()}
    line["value"] = line["mixed"]["value"]
    line["dtype"] = "mixed (double-float RK4 on the FP32 pipe); fp64 beside it"
    line["steps"], line["warmup"] = args.steps, max(args.warmup, 3)
    line["ms_per_step"] = line["mixed"]["ms"] / args.steps
    line["e2e"] = {"value": line["mixed"]["e2e"], "unit": "models/s", "h2d_bytes_per_step": 8 * m.n_params,
                   "d2h_bytes_per_step": 8 * (4 + 2 * 16)}
    line["speedup_mixed_over_fp64"] = line["mixed"]["value"] / line["fp64"]["value"]
    line["gpu_launches"] = 4 * args.steps
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle as O

    t0 = time.perf_counter()
    ro = O.rmsd(m, s.obs, s.params_true, seed=3, call=0, n_streams=2000, samples=1, dx=1e-4, reopt=1)
    cpu_s = time.perf_counter() - t0
    line["cpu_baseline"] = {"value": ro["n_tot"] / cpu_s, "unit": "models/s", "cores": 1, "kind": "port",
                            "sample": f"{ro['n_tot']} models on one host thread (the oracle's RMSD loop is serial)"}
    print(json.dumps(line))


def bench_animate(args, tmp, rank, world):
    """ANIMATE frames (compute_rgb, cuda.c:2394-2540): the config-0 object's true model on the
    ANIMATE plot grid (15 440 snapshots), 1080 x 1080 frames; frames/s of the render kernel, the
    same through ast_render_frames with the frames copied to host memory, and the oracle."""
    from asteroid_gb300 import api, synth

    local = int(os.environ.get("LOCAL_RANK", "0"))
    s = synth.generate("c0acc", tmp)
    n_plot, S, per_step = 15440, 1080, 256
    t, e, u = api.plot_grid(s.dir / "lc.dat", s.dir, n_plot)
    with api.Engine(s.model, s.obs, device=local) as eng:
        t0 = time.perf_counter()
        geo = eng.model_geometry(s.params_true, t, e, u)
        geo_s = time.perf_counter() - t0
    for k in range(max(args.warmup, 3)):
        api.render_frames(geo[:per_step], S, device=local)
    ms, wall, frames = 0.0, 0.0, 0
    with Clocks(local) as clk:
        for k in range(args.steps):
            f0 = (k * per_step) % (n_plot - per_step)
            t0 = time.perf_counter()
            rgb, m = api.render_frames(geo[f0:f0 + per_step], S, device=local)
            wall += time.perf_counter() - t0
            ms += m
            frames += per_step
    lit = float(np.mean(rgb[..., 0] > 0))
    line = {"metric": "frames_per_s", "value": frames / (ms * 1e-3), "unit": "frames/s", "n_gpus": 1,
            "steps": args.steps, "warmup": max(args.warmup, 3), "ms_per_step": ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "mode": "animate",
            "config": {"workload": f"config-0 object, {per_step} frames of {S}x{S} per step from the {n_plot}-snapshot "
                                   "ANIMATE grid", "l2": "output frames (896 MB per step) larger than L2"},
            "pixels_per_s": frames * S * S / (ms * 1e-3), "lit_fraction": lit, "geometry_s": geo_s,
            "clocks": clk.summary(), "gpu_launches": args.steps,
            "e2e": {"value": frames / wall, "unit": "frames/s", "h2d_bytes_per_step": 160 * per_step,
                    "d2h_bytes_per_step": 3 * S * S * per_step}}
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle as O

    t0 = time.perf_counter()
    O.render(geo[:2], S)
    cpu_s = time.perf_counter() - t0
    line["cpu_baseline"] = {"value": 2 / cpu_s, "unit": "frames/s", "cores": 1, "kind": "port",
                            "sample": "2 frames of 1080x1080 on one host thread"}
    print(json.dumps(line))


def bench_serve(args, tmp, rank, world):
    """Config 4: Poisson arrivals of config-3 objects (1024 chains x 5000 evaluations each) at 1, 4,
    16 and 64 requests/s into one server (150 GB HBM budget); p50/p99 latency from submission to
    retirement, fits/s, and each served best chi^2 against the FP64 path at its parameters.  The
    search is mixed precision; requests ask for FP64 results (fp64_result), so the reported chi^2
    of each group is the plain path's at the group's best parameters."""
    from asteroid_gb300 import api, synth

    pool = synth.generate_batch(32, tmp)
    rng = np.random.default_rng(2024)
    line = {"metric": "fit_latency", "unit": "s", "mode": "serve", "requests_per_rate": args.requests,
            "lanes_per_chain": args.lanes,
            "chains_per_request": 1024, "evals_per_chain": 5000, "hbm_budget_gb": 150, "rates": {}}
    checked = []
    engines = {}
    # The latency floor: one request alone on the GPU, for each of the first four pool objects.
    alone = []
    for k in range(args.alone):
        s = pool[k]
        with api.Server(precision=api.PREC_MIXED, acc=True, hbm_budget=150 << 30, lanes=args.lanes) as srv:
            r = srv.submit(s.model, s.obs, n_chains=1024, group_size=256, seed=100 + k, evals_cap=5000,
                                   fp64_result=True)
            while srv.poll(r) is None:
                srv.step(32)
            alone.append({"n_data": s.obs.n_data, "span_days": float(s.obs.mjd[-1] - s.obs.mjd[0]),
                          "model": api.flag_names(s.model.flags), "latency_s": srv.poll(r)[1]})
    line["alone"] = alone
    print(json.dumps({"mode": "serve", "alone": alone, "lanes_per_chain": args.lanes}), flush=True)
    for lam in [float(r) for r in args.rates.split(",")]:
        arrivals = np.cumsum(rng.exponential(1.0 / lam, size=args.requests))
        with api.Server(precision=api.PREC_MIXED, acc=True, hbm_budget=150 << 30, lanes=args.lanes) as srv:
            t0 = time.perf_counter()
            ids, objs, done, lat = [], [], {}, {}
            k = 0
            while len(done) < args.requests:
                now = time.perf_counter() - t0
                while k < args.requests and arrivals[k] <= now:
                    s = pool[(k * 7 + int(lam)) % len(pool)]
                    ids.append(srv.submit(s.model, s.obs, n_chains=1024, group_size=256, seed=100 + k, evals_cap=5000,
                                   fp64_result=True))
                    objs.append(s)
                    k += 1
                if not ids or len(done) == len(ids):
                    time.sleep(max(0.0, min(0.01, arrivals[k] - now)) if k < args.requests else 0.0)
                    continue
                srv.step(32)
                for j, r in enumerate(ids):
                    if r not in done:
                        got = srv.poll(r)
                        if got is not None:
                            done[r] = got[0]
                            lat[r] = got[1]
            wall = time.perf_counter() - t0
            st = srv.stats()
        L = np.array([lat[r] for r in ids])
        # Served results against FP64: the best group's parameters re-evaluated by the plain path,
        # with the FP64 chi^2's own conditioning (its change under a one-ulp move of every
        # parameter): a fit may end where the fixed-step RK4 is under-resolved and chaotic.
        for r, s in zip(ids, objs):
            res = done[r]
            g = res.best
            key = id(s)
            if key not in engines:
                engines[key] = api.Engine(s.model, s.obs)
            p = res.best_params[g]
            q = p * (1 + np.random.default_rng(r).choice([-1.0, 1.0], size=p.shape) * 2.3e-16)
            c64, _ = engines[key].eval(np.vstack([p, q]), api.PREC_FP64)
            if not (np.isfinite(c64[0]) and c64[0] < 1e29):
                continue
            checked.append((abs(res.best_f[g] - c64[0]) / abs(c64[0]), abs(c64[1] - c64[0]) / abs(c64[0])))
        line["rates"][f"{lam:g}/s"] = {"p50_s": float(np.percentile(L, 50)), "p99_s": float(np.percentile(L, 99)),
                                       "fits_per_s": len(ids) / wall, "wall_s": wall,
                                       "evals_per_s": st["n_evals"] / (st["kernel_ms"] * 1e-3)}
        # One line per rate as it completes (a long run keeps what it measured).
        print(json.dumps({"mode": "serve", "rate": f"{lam:g}/s", **line["rates"][f"{lam:g}/s"],
                          "requests": args.requests, "lanes_per_chain": args.lanes}), flush=True)
    for e in engines.values():
        e.close()
    good = [rel for rel, cond in checked if cond <= 1e-10]
    line["served_vs_fp64"] = {
        "requests": len(checked), "well_conditioned": len(good),
        "well_conditioned_within_1e-6": int(sum(r <= 1e-6 for r in good)),
        "max_rel_dchi2_well_conditioned": float(max(good)) if good else None,
        "ill_conditioned_max_rel_dchi2": float(max([r for r, c in checked if c > 1e-10], default=0.0)),
        "note": "best chi2 of each served request against the FP64 chi2 of its best parameters; "
                "well-conditioned = FP64 chi2 stable to 1e-10 under a one-ulp move of the parameters"}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="c2")
    ap.add_argument("--chains", type=int, default=65536)
    ap.add_argument("--evals-cap", type=int, default=20000)
    ap.add_argument("--budget-mixed", type=int, default=0, help="evaluations per slot per step (0 = auto)")
    ap.add_argument("--budget-fp64", type=int, default=0)
    ap.add_argument("--skip-fp64", action="store_true")
    ap.add_argument("--skip-batched", action="store_true")
    ap.add_argument("--skip-fits", action="store_true", help="skip the full-length config-0 fits")
    ap.add_argument("--mode", default="fit",
                    choices=["fit", "batch", "serve", "compare", "periodogram", "rmsd", "animate", "precisions", "fits"],
                    help="fit: the headline line; batch: config 3 (uneven objects, one launch); "
                         "serve: config 4 (Poisson arrivals, continuous batching); compare: full fits of "
                         "--config in both precisions at one seed; periodogram: minima() of plot mode; "
                         "rmsd: RMSD confidence intervals; animate: ANIMATE frames")
    ap.add_argument("--objects", type=int, default=512, help="batch mode: objects")
    ap.add_argument("--graph-only", action="store_true", help="batch mode: only the graph-captured run")
    ap.add_argument("--graph-evals", type=int, default=50,
                    help="batch mode: evaluations per chain of the graph-captured run to completion")
    ap.add_argument("--requests", type=int, default=8, help="serve mode: requests per arrival rate")
    ap.add_argument("--lanes", type=int, default=4, choices=[1, 4], help="serve mode: lanes per chain")
    ap.add_argument("--alone", type=int, default=4, help="serve mode: requests timed alone (the latency floor)")
    ap.add_argument("--rates", default="1,4,16,64", help="serve mode: arrival rates, requests/s")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--profile", action="store_true", help="only the fit launches (for ncu)")
    args = ap.parse_args()

    world, rank, local, dist = dist_setup()
    tmp = tempfile.mkdtemp(prefix="astbench_")

    if args.impl == "reference":
        if rank != 0:
            return
        return bench_reference(args)

    import torch

    from asteroid_gb300 import api, build

    build.build_engine()
    torch.cuda.set_device(local)
    if args.mode == "batch":
        return bench_batch(args, tmp, rank, world)
    if args.mode == "serve":
        return bench_serve(args, tmp, rank, world)
    if args.mode == "compare":
        return bench_compare(args, tmp, rank, world)
    if args.mode == "periodogram":
        return bench_periodogram(args, tmp, rank, world)
    if args.mode == "rmsd":
        return bench_rmsd(args, tmp, rank, world)
    if args.mode == "animate":
        return bench_animate(args, tmp, rank, world)
    if args.mode == "precisions":
        return bench_precisions(args, tmp, rank, world)
    if args.mode == "fits":
        print(json.dumps({"mode": "fits", **measure_fits(local, precisions=("mixed", "fp64"))}))
        return
    s = make_workload(args, tmp)
    model, obs = s.model, s.obs
    eng = api.Engine(model, obs, device=local)
    stream = torch.cuda.ExternalStream(eng.stream)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=f"cuda:{local}")

    def timed(fn):
        """Run fn between two events on the engine's stream, L2 flushed first; returns (ms, out)."""
        barrier(dist)
        torch.cuda.synchronize()
        with torch.cuda.stream(stream):
            flush.zero_()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        out = fn()
        b.record(stream)
        torch.cuda.synchronize()
        barrier(dist)
        return a.elapsed_time(b), out

    n_rk4 = rk4_steps(obs, model.time_step)
    flops, trans = algorithmic_flops(obs, model)
    from asteroid_gb300 import replicas

    seed = replicas.replica_seed(1234, rank)  # one replica per GPU, distinct seeds

    # NUDGE is the reference's Stage-Three option, run with -reopt from a good model
    # (README.md:88-103): chains start around the true model.  From random starts nearly every
    # evaluation would take the "more than M_MAX model minima" early exit (cuda.c:738-742).
    reopt = bool(model.flags & api.NUDGE)
    p0 = s.params_true if reopt else None
    main_prec = api.PREC_FP64 if args.precision == "fp64" else api.PREC_MIXED

    if args.profile:
        # Only the fit launches of one precision (the command profiled under ncu).
        ev, ms, _, launches, b = run_fit_steps(eng, main_prec, args.chains, 256, args.evals_cap, args.budget_mixed,
                                               args.warmup, args.steps, seed, timed, reopt, p0)
        print(json.dumps({"profile": args.precision, "evals": ev, "ms": ms, "evals_per_s": ev / (ms * 1e-3),
                          "budget": b, "slots": eng.fit_slots()}))
        eng.close()
        return

    with Clocks(local) as clk:
        ev_m, ms_m, fits_m, launches_m, b_mixed = run_fit_steps(
            eng, api.PREC_MIXED, args.chains, 256, args.evals_cap, args.budget_mixed, args.warmup, args.steps, seed,
            timed, reopt, p0)
    slots_m = eng.fit_slots() or NCU_C2["slots"]  # the mixed launch's resident slots
    ms_m = max_over_ranks(dist, ms_m)
    ev_m_all = sum_over_ranks(dist, ev_m)
    value = ev_m_all / (ms_m * 1e-3)

    # The same workload through the batch engine (ast_batch_step): one object of the batch path.
    batched = run_batch_steps(s, api.PREC_MIXED, args.chains, 256, args.evals_cap, b_mixed, args.warmup, args.steps,
                              seed, timed, reopt, p0) if not args.skip_batched else None

    fp64 = None
    if not args.skip_fp64:
        ev_d, ms_d, _, _, b_fp64 = run_fit_steps(eng, api.PREC_FP64, args.chains, 256, args.evals_cap,
                                                 args.budget_fp64, max(1, args.warmup // 2 + 1),
                                                 max(2, args.steps // 2), seed, timed, reopt, p0)
        ms_d = max_over_ranks(dist, ms_d)
        fp64 = sum_over_ranks(dist, ev_d) / (ms_d * 1e-3)

    # Accuracy of the mixed path against FP64 on sampled vectors and on the truth.
    P = np.vstack([workload_vectors(model, 2047, 11 + rank, s.params_true), s.params_true[None, :]])
    c64, _ = eng.eval(P, api.PREC_FP64)
    c32, _ = eng.eval(P, api.PREC_MIXED)
    # Conditioning on the FP64 path itself: chi^2 after a one-ulp move of every parameter.
    Q = P * (1 + np.random.default_rng(0).choice([-1.0, 1.0], size=P.shape) * 2.3e-16)
    q64, _ = eng.eval(Q, api.PREC_FP64)
    with np.errstate(invalid="ignore", divide="ignore"):
        cond = np.abs(q64 - c64) / np.abs(c64)
    ok = np.isfinite(c64) & (c64 < 1e29) & (cond <= 1e-10)
    flips = int(np.sum(ok & (c32 >= 1e29)))
    ok &= c32 < 1e29
    rel = np.abs(c32[ok] - c64[ok]) / np.abs(c64[ok])
    truth_rel = float(abs(c32[-1] - c64[-1]) / abs(c64[-1]))

    # Phase drift of the double-float integration against FP64 over the whole light curve.
    drift = phase_drift(eng, model, obs, P[-1:] if len(P) else P, P[:7])

    # End to end through the C ABI with host buffers: ast_eval_batch, copies included; four
    # vectors per resident thread of the evaluation kernel (the fit's slot count), so the launch
    # fills the GPU as the fit does.
    B = 4 * slots_m
    # Page-locked host buffers for the vectors in and the results out (numpy views of pinned
    # torch tensors), as a caller streaming batches through ast_eval_batch would keep them.
    Pe = torch.empty((B, model.n_params), dtype=torch.float64, pin_memory=True).numpy()
    Pe[:] = workload_vectors(model, B, 21 + rank, s.params_true)
    ce = torch.empty(B, dtype=torch.float64, pin_memory=True).numpy()
    de = torch.empty((B, obs.n_filters), dtype=torch.float64, pin_memory=True).numpy()
    eng.eval(Pe, api.PREC_MIXED, chi2_out=ce, dv_out=de)  # warm-up at full size: scratch allocated
    t0 = time.perf_counter()
    e2e_steps = 2
    for _ in range(e2e_steps):
        eng.eval(Pe, api.PREC_MIXED, chi2_out=ce, dv_out=de)
    e2e_dt = max_over_ranks(dist, time.perf_counter() - t0)
    e2e = sum_over_ranks(dist, B * e2e_steps) / e2e_dt

    peak32 = api.probe_peak("fp32", local)
    peak64 = api.probe_peak("fp64", local)
    scale = n_rk4 / NCU_C2["rk4_steps"]
    # Algorithmic work: the reference source's flop count per evaluation (flops) times the
    # evaluations per second; executed work: the FP32 (mixed) or FP64 flops ncu counts per
    # evaluation of these kernels.
    achieved = flops * value / 1e12 / max(world, 1)
    executed = NCU_C2["mixed_fp32_flops"] * scale * value / 1e12 / max(world, 1)
    achieved64 = flops * fp64 / 1e12 / max(world, 1) if fp64 else None
    executed64 = NCU_C2["fp64_flops"] * scale * fp64 / 1e12 / max(world, 1) if fp64 else None
    fits = measure_fits(local) if (rank == 0 and world == 1 and not args.skip_fits) else None
    cpu = cpu_baseline(model, obs, args.cpu_seconds, s.params_true) if (rank == 0 and world == 1) else None
    clocks = clk.summary()

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_m / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 (double-float state and RHS, f32 brightness; f64 set-up and chi2 sums)",
            "data": "synthetic",
            "config": {"workload": f"{args.config}: {obs.n_data} points, {obs.n_filters} filters, "
                                   f"{api.flag_names(model.flags)}, TIME_STEP {model.time_step}, "
                                   f"{args.chains} chains x {args.evals_cap} evals"
                                   f"{' re-optimised from the true model (Stage Three, -reopt)' if reopt else ''}; "
                                   f"timed slice of {b_mixed} evals/slot/step", "chains_per_gpu": args.chains,
                       "n_data": obs.n_data, "rk4_steps_per_eval": n_rk4, "parallelism": f"replicas x{world}",
                       "l2": "flushed before every timed region (256 MB write); simplex state ~100 MB, obs in smem"},
            "fits_per_s": fits["mixed"]["fits_per_s"] if fits else None,
            "fits": fits,
            "fp64": {"value": fp64, "unit": UNIT, "speedup_mixed_over_fp64": (value / fp64) if fp64 else None},
            "batched": None if batched is None else {
                "value": batched, "unit": UNIT, "speedup_over_fp64": (batched / fp64) if fp64 else None,
                "path": "ast_batch_step: the workload as one object of the multi-object batch engine"},
            "phase_drift": drift,
            "accuracy": {"vectors": int(ok.sum()), "of": int(len(P)), "median_rel_dchi2": float(np.median(rel)),
                         "p99_rel_dchi2": float(np.quantile(rel, 0.99)), "max_rel_dchi2": float(rel.max()),
                         "frac_le_1e-6": float(np.mean(rel <= 1e-6)), "true_model_rel_dchi2": truth_rel,
                         "nudge_flips": flips,
                         "note": "mixed vs FP64 on sampled vectors whose FP64 chi2 is stable to a one-ulp move of "
                                 "the parameters (cond <= 1e-10)"},
            "roofline": {"bound": "fp32 pipe (CUDA cores)", "achieved": achieved, "peak": peak32 / 1e3,
                         "unit": "TFLOP/s", "frac": achieved / (peak32 / 1e3),
                         "traffic": NCU_C2["dram_bytes_mixed"] * slots_m / NCU_C2["slots"],
                         "kernel": "fit_kernel<double, MIXED>",
                         "per_eval": {"flops": flops, "transcendentals": trans,
                                      "source": "the reference's chi2one counted from its source: 152 per RK4 "
                                                "step, 156 per observation, 6 per filter, 50 per evaluation "
                                                "(add/mul/div/sqrt 1, fma 2); transcendental calls not counted"},
                         "executed": {"achieved": executed, "frac": executed / (peak32 / 1e3),
                                      "fp32_flops_per_eval": NCU_C2["mixed_fp32_flops"] * scale,
                                      "source": "ncu FFMA x 2 + FADD + FMUL per evaluation of this kernel "
                                                "(the double-float formulation's own arithmetic)"},
                         "peak_source": "measured in this run by ast_probe_peak (FP32 FMA loop over every SM); "
                                        "MEASURED_PEAKS.json holds HBM and bf16 only",
                         "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum per launch of the "
                                           "config-2 capture, scaled by this launch's resident slots",
                         "fp64_path": {"kernel": "fit_kernel<double, FP64>", "bound": "fp64 pipe",
                                       "achieved": achieved64, "peak": peak64 / 1e3, "unit": "TFLOP/s",
                                       "frac": (achieved64 / (peak64 / 1e3)) if achieved64 else None,
                                       "executed": executed64,
                                       "executed_frac": (executed64 / (peak64 / 1e3)) if executed64 else None,
                                       "per_eval_fp64_flops_executed": NCU_C2["fp64_flops"] * scale}},
            "cpu_baseline": cpu,
            "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": B * model.n_params * 8,
                    "d2h_bytes_per_step": B * (1 + obs.n_filters) * 8,
                    "path": "ast_eval_batch, mixed, page-locked host buffers, copies inside the timed region"},
            "gpu_launches": launches_m,
            "clocks": clocks,
        }
        print(json.dumps(line))
    eng.close()
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
