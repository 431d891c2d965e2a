"""Benchmark of the nested-sampling inner loop on one GB300.

Default workload ("shells", the Gaussian-shells configuration): R = 1024 independent runs
(seeds PRNGKey(0..R-1)) of the D=10 two-shell likelihood in U[-6,6]^10 (radius 2, width 0.1,
centres +-3.5 e_0), 1000 live points, num_slices = 50, terminate at dlogZ < 1e-4, advanced
together by the batched engine (one sampler launch + one merge launch per iteration,
replayed from a captured CUDA graph).  One "step" = every run from its initial live points
to termination plus the device results pass (tree counts, FP64 evidence).

--workload config3: 4096 independent correlated-Gaussian runs, D ~ U{2..64}, n = 50 D,
num_slices = 5 D, Sigma = A A^T / D + 0.1 I, prior U[-10,10]^D, dlogZ < 1e-4.

All inputs are seeded synthetic data.  The sample stores exceed L2 (no flush needed).
Metric: NS runs/s of the whole batch, likelihood evaluations/s alongside.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gbns|reference] [--runs R]

--impl reference times the CPU restatement of the reference (oracle/, FP64 C) on the host's
cores: complete runs of the same workload (shells), or a bounded per-iteration sample scaled
to whole runs (config3).  Under torchrun each rank runs its own R runs (weak scaling, no
collective on the data path).
"""
from __future__ import annotations

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

METRIC = "NS runs/s & likelihood evals/s at |dlogZ|<0.1, batched/adjoint vs plain GPU"
SHELLS_D = 10


def workload(R: int, seed: int = 2024, name: str = "shells"):
    """Seeded problems: list of (D, kind, params, n, S, cap)."""
    out = []
    if name == "shells":
        c1 = np.zeros(SHELLS_D)
        c1[0] = 3.5
        for r in range(R):
            out.append((SHELLS_D, "shells", (c1, -c1, 2.0, 0.1), 1000, 50, 100000))
        return out
    rng = np.random.default_rng(seed)
    Ds = rng.integers(2, 65, size=R)
    for r, D in enumerate(Ds):
        D = int(D)
        g = np.random.default_rng([seed, r])
        mu = g.standard_normal(D)
        A = g.standard_normal((D, D))
        cov = A @ A.T / D + 0.1 * np.eye(D)
        n = 50 * D
        s = n // 2
        cap = int(np.ceil(50 * D * (2.5 * D + 15) / s)) * s
        out.append((D, "mvn", (mu, cov), n, 5 * D, cap))
    return out


def shells_log_Z(D=SHELLS_D, R=2.0, w=0.1, box=12.0):
    """FP64 quadrature of the radial integral (two non-overlapping shells inside the box)."""
    from scipy import integrate, special
    S = 2 * np.pi ** (D / 2) / special.gamma(D / 2)
    f = lambda r: r ** (D - 1) * np.exp(-0.5 * ((r - R) / w) ** 2) / np.sqrt(2 * np.pi * w * w)
    I, _ = integrate.quad(f, max(0.0, R - 12 * w), R + 12 * w, epsabs=0, epsrel=1e-12)
    return np.log(2 * S * I) - D * np.log(box)


def make_samplers(wl):
    import jaxns_gb300 as gb
    samplers = []
    cache = {}
    for D, kind, params, n, S, cap in wl:
        if kind == "shells":
            if "shells" not in cache:
                def prior_model(D=D):
                    x = yield gb.Prior(gb.Uniform(-6.0 * np.ones(D), 6.0 * np.ones(D)), name="x")
                    return x
                cache["shells"] = gb.Model(prior_model, gb.GaussianShellsLikelihood(*params))
            model = cache["shells"]
        else:
            def prior_model(D=D):
                x = yield gb.Prior(gb.Uniform(-10.0 * np.ones(D), 10.0 * np.ones(D)), name="x")
                return x
            model = gb.Model(prior_model, gb.MultivariateNormalLikelihood(*params))
        samplers.append(gb.NestedSampler(model, num_live_points=n, num_slices=S, max_samples=cap, store_U=False))
    return samplers


def oracle_models(wl, idx):
    from oracle import oracle
    models, cfgs = [], []
    for r in idx:
        D, kind, params, n, S, cap = wl[r]
        if kind == "shells":
            models.append(oracle.shells_model(-6, 6, params[0], params[1], params[2], params[3]))
        else:
            models.append(oracle.mvn_model(-10 * np.ones(D), 10 * np.ones(D), params[0], params[1]))
        cfgs.append(dict(num_live_points=n, num_slices=S, max_samples=cap))
    return models, cfgs


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.rows = []
        self.index = index
        self._stop = threading.Event()
        self._th = None

    def _loop(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                for line in out.stdout.strip().splitlines():
                    self.rows.append([x.strip() for x in line.split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._th = threading.Thread(target=self._loop, daemon=True)
        self._th.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        self._th.join(timeout=10)

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if len(r) > 5 + i and r[5 + i] == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


# ----------------------------------------------------------------- CPU side

def cpu_sample(wl, idx, iters: int, threads: int):
    """Oracle (FP64 C restatement, one host thread per run) on runs idx of the workload
    (iters > 0: at most that many NS iterations); per-run (seconds, evals, iterations)."""
    from oracle import oracle
    models, cfgs = oracle_models(wl, idx)
    keys = np.array([oracle.PRNGKey(r) for r in idx])
    tcs = [{"dlogZ": 1e-4}] * len(idx)
    return oracle.ns_run_batch_timed(models, cfgs, keys, tcs, threads, iters)


def iterations_model(D: int) -> float:
    """Expected NS iterations of one config3 run (N_s ~ n (2.1 D + 8), s = n/2)."""
    return 2.0 * (2.1 * D + 8.0) - 2.0


def cpu_runs_per_s(wl, name, threads):
    """Host runs/s of the oracle on this workload.  shells: `threads` complete runs on
    `threads` host threads.  config3: every (R/16)-th run for 2 NS iterations, scaled to whole
    runs by the expected iteration count."""
    if name == "shells":
        idx = list(range(min(threads, len(wl))))
        secs, evals, its = cpu_sample(wl, idx, 0, threads)
        t = float(np.max(secs))  # the threads ran concurrently
        return len(idx) / t, dict(runs=len(idx), seconds=float(np.sum(secs)),
                                  sample=f"{len(idx)} complete runs on {threads} host threads")
    stride = max(1, len(wl) // 16)
    idx = list(range(0, len(wl), stride))
    secs, evals, its = cpu_sample(wl, idx, 2, threads)
    t_est = sum(secs[k] / max(its[k], 1) * max(iterations_model(wl[r][0]), its[k]) for k, r in enumerate(idx))
    t_total = t_est * stride
    return len(wl) / (t_total / threads), dict(
        runs=len(idx), seconds=float(np.sum(secs)),
        sample=f"every {stride}th run ({len(idx)} runs), 2 NS iterations each on {threads} threads, scaled to whole "
               f"runs by the expected iteration count 2(2.1D+8)-2")


# ----------------------------------------------------------------- main

def flops_per_eval(D, kind):
    """Algorithmic FP32 flops of one likelihood evaluation: MVN D^2 + 8D (proposal, prior
    quantile, triangular solve, sum of squares); shells 10D + 22 (proposal, quantile, two
    norms, shell terms, logaddexp)."""
    return D * D + 8 * D if kind == "mvn" else 10 * D + 22


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gbns", choices=["gbns", "reference"])
    ap.add_argument("--workload", default="shells", choices=["shells", "config3"])
    ap.add_argument("--runs", type=int, default=None)
    ap.add_argument("--block", type=int, default=16)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--only-dim", type=int, default=None,
                    help="config3: keep only runs of this dimension (repeated to --runs); for kernel profiling")
    ap.add_argument("--iterations", type=int, default=None,
                    help="time init + this many NS iterations instead of whole runs (kernel profiling)")
    args = ap.parse_args()
    if args.runs is None:
        args.runs = 1024 if args.workload == "shells" else 4096

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    wl = workload(args.runs, seed=2024 + rank, name=args.workload)
    if args.only_dim is not None:
        pool = [w for w in workload(4096, seed=2024 + rank, name=args.workload) if w[0] == args.only_dim]
        if not pool:
            raise SystemExit(f"no run of dimension {args.only_dim} in the workload")
        wl = [pool[i % len(pool)] for i in range(args.runs)]
    threads = os.cpu_count() or 1
    if args.workload == "shells":
        wdesc = (f"configs[1] Gaussian shells D=10 (R=2, w=0.1, centres +-3.5 e0, U[-6,6]^10), 1000 live points, "
                 f"50 slices, dlogZ<1e-4; {args.runs} independent seeds per GPU in one batched launch")
    else:
        wdesc = (f"configs[2] batched correlated Gaussians: {args.runs} runs per GPU, D~U{{2..64}}, n=50D, S=5D, "
                 f"dlogZ<1e-4")

    if args.impl == "reference":
        if rank != 0:
            return
        from oracle import oracle
        oracle.build()
        vals = []
        for step in range(args.warmup + args.steps):
            v, info = cpu_runs_per_s(wl, args.workload, threads)
            if step >= args.warmup:
                vals.append(v)
        v = float(np.mean(vals))
        print(json.dumps({"metric": METRIC, "value": v, "unit": "runs/s", "impl": "reference", "n_gpus": args.gpus,
                          "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
                          "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
                          "config": {"workload": wdesc, "runs": args.runs},
                          "cpu_baseline": {"value": v, "unit": "runs/s", "cores": threads, "kind": "port",
                                           "sample": info["sample"]},
                          "e2e": {"value": v, "unit": "runs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}))
        return

    import torch
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    from jaxns_gb300.build import build_library
    build_library()
    from jaxns_gb300.batched import BatchedNestedSampler
    import jaxns_gb300 as gb

    samplers = make_samplers(wl)
    keys = np.array([gb.random.PRNGKey(r) for r in range(len(wl))])
    bns = BatchedNestedSampler(samplers, keys, [gb.TerminationCondition(dlogZ=1e-4)] * len(wl), block=args.block)
    b = bns.batch
    if args.iterations is not None:
        # kernel-profiling mode: init + a fixed number of eager iterations, no results pass
        b.init()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        b.iterate(args.iterations)
        e1.record()
        torch.cuda.synchronize()
        st = b.state()
        ev = int(st["num_likelihood_evaluations"].sum())
        fl = float(np.sum(st["num_likelihood_evaluations"] * np.array([flops_per_eval(w[0], w[1]) for w in wl])))
        ms = e0.elapsed_time(e1)
        print(json.dumps({"mode": "iterations", "iterations": args.iterations, "runs": len(wl), "ms": ms,
                          "likelihood_evals": ev, "algorithmic_tflops": fl / ms / 1e9}))
        return

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    def step(from_host=False):
        bns(from_host=from_host)
        if from_host:
            return bns.summary()  # device results pass + D2H of the [R, 8] summary
        b.results(with_U=False)
        return None

    b.timing = True  # graphs carry event pairs around the sampler launches
    for _ in range(args.warmup):
        step()
    barrier()

    # ---- device-resident timed region
    b.shell_ms, b.shell_launch_groups = 0.0, 0
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches0 = b.kernel_launches
    nevals = 0
    with ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) as clk:
        barrier()
        ev0.record()
        for _ in range(args.steps):
            step()
            nevals += int(b.state()["num_likelihood_evaluations"].sum())
        ev1.record()
        barrier()
    ms = ev0.elapsed_time(ev1)
    gpu_launches = b.kernel_launches - launches0
    st = b.state()
    if world > 1:
        t = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    runs_total = args.runs * args.steps * world
    value = runs_total / (ms / 1e3)
    evals_per_s = nevals * world / (ms / 1e3)

    # sampler-kernel roofline (FP32 CUDA-core bound): algorithmic flops / sampler device time
    Dr = np.array([w[0] for w in wl])
    fpe = np.array([flops_per_eval(w[0], w[1]) for w in wl], np.float64)
    flops = float(np.sum(st["num_likelihood_evaluations"] * fpe)) * args.steps
    shell_s = b.shell_ms / 1e3
    clocks = clk.summary()
    sm_mhz = clocks["sm_mhz"] or 1900.0
    fp32_peak = 152 * 128 * 2 * sm_mhz * 1e6 / 1e12
    achieved = flops / shell_s / 1e12 if shell_s > 0 else None
    roofline = {"bound": "fp32", "kernel": "k_slice_shell (fused slice sampler)", "achieved": achieved,
                "peak": fp32_peak, "unit": "TFLOP/s", "frac": (achieved / fp32_peak) if achieved else None,
                "traffic": None,
                "peak_source": "derived: 152 SMs x 128 FP32 lanes x 2 flop x median SM clock under load "
                               "(MEASURED_PEAKS.json has no FP32 CUDA-core figure)",
                "flops_per_eval": "MVN D^2+8D, shells 10D+22",
                "sampler_share_of_step": shell_s / (ms / 1e3) if ms else None,
                "sampler_launch_groups": b.shell_launch_groups}

    # ---- end-to-end through the public API: run table + keys from pinned host memory, the
    # [R, 8] summary (log Z, uncertainty, ESS, H, counts) back to the host
    h2d = int(b.t_state.numel())
    d2h = 8 * 8 * args.runs
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        sc = step(from_host=True)
    e1.record()
    barrier()
    e2e_ms = e0.elapsed_time(e1)
    e2e = {"value": runs_total / (e2e_ms / 1e3), "unit": "runs/s", "h2d_bytes_per_step": h2d,
           "d2h_bytes_per_step": d2h}

    truth = np.full(len(wl), shells_log_Z()) if args.workload == "shells" else -Dr * np.log(20.0)
    dz = sc[:, 0] - truth
    accuracy = {"truth": "FP64 radial quadrature" if args.workload == "shells" else "analytic -D log 20",
                "mean_log_Z": float(np.mean(sc[:, 0])), "truth_log_Z": float(np.mean(truth)),
                "mean_abs_dlogZ": float(np.mean(np.abs(dz))), "frac_abs_dlogZ_lt_0.1": float(np.mean(np.abs(dz) < 0.1)),
                "frac_within_3sigma": float(np.mean(np.abs(dz) < 3 * sc[:, 1])),
                "mean_log_Z_uncert": float(np.mean(sc[:, 1])), "ensemble_mean_error": float(np.mean(dz))}

    line = {"metric": METRIC, "value": value, "unit": "runs/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 (FP64 evidence)", "data": "synthetic (seeded)",
            "config": {"workload": wdesc, "runs_per_gpu": args.runs, "graph_block": args.block,
                       "l2": "per-step sample store > L2 (no flush needed)"},
            "likelihood_evals_per_s": evals_per_s, "gpu_launches": int(gpu_launches), "roofline": roofline,
            "e2e": e2e, "clocks": clocks, "accuracy": accuracy,
            "iterations": {"max": int(st["iterations"].max()), "mean": float(st["iterations"].mean())}}

    if rank == 0 and not args.no_plain:
        # plain single-run GPU kernel loop: runs one at a time, eager launches, no graph
        from jaxns_gb300.engine import NSBatch
        idx = list(range(0, args.runs, max(1, args.runs // 8)))
        tot = 0.0
        for r in idx:
            one = NSBatch([b.specs[r]])
            torch.cuda.synchronize()
            t0 = time.time()
            one.run(block=1, use_graph=False)
            one.results(with_U=False)
            torch.cuda.synchronize()
            tot += time.time() - t0
            del one
        plain = len(idx) / tot
        line["plain_single_run_loop"] = {"runs_per_s": plain, "sample": f"{len(idx)} runs one at a time, eager launches",
                                         "batched_speedup": value / world / plain}
    if rank == 0 and not args.no_cpu:
        from oracle import oracle
        oracle.build()
        v, info = cpu_runs_per_s(wl, args.workload, threads)
        line["cpu_baseline"] = {"value": v, "unit": "runs/s", "cores": threads, "kind": "port",
                                "sample": info["sample"]}
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
