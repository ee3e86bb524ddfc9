#!/usr/bin/env python
"""Benchmark: vectorized NUTS on covtype-shaped Bayesian logistic regression.

Workload (1 GPU): N=581,012 rows x D=55 (10 continuous + 44 binary + intercept),
1024 chains, prior N(0,1), synthetic seeded data; NUTS with Stan warmup
(500 iterations, untimed setup), then W warm-up steps and K timed steps.  A
"step" is one sampling block of ``--iters-per-step`` NUTS transitions for all
chains.  value = min over the 55 coefficients of bulk-ESS (rank-normalised
split-ESS) of the draws of the timed steps / timed seconds; grad evals/s is
reported beside it.  L2 is flushed (a 512 MB write) before every timed step.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
import argparse
import ctypes
import json
import os
import subprocess
import tempfile
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "min bulk-ESS/s & grad evals/s: fused vs plain NUTS on 1 GB300 at R-hat<1.01"
WORKLOAD = "logreg-covtype-shaped N=581012 D=55, 1024 chains, NUTS max_tree_depth=10, 500 warmup"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--engine", default="fused", choices=["fused", "plain"])
    p.add_argument("--precision", default=None, choices=["fp32", "bf16x3"])
    p.add_argument("--chains", type=int, default=1024)
    p.add_argument("--n", type=int, default=581012)
    p.add_argument("--num-warmup", type=int, default=500)
    p.add_argument("--iters-per-step", type=int, default=10)
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--cpu-samples", type=int, default=50, help="transitions per chain of the CPU baseline")
    p.add_argument("--plain-steps", type=int, default=3,
                   help="steps of the plain (lock-step FP32) engine from the same adapted state; 0 = skip")
    p.add_argument("--mode", default="nuts", choices=["nuts", "potential"],
                   help="potential: time only the dominant kernel (U and dU for every chain)")
    p.add_argument("--reps", type=int, default=20)
    p.add_argument("--workload", default="logreg",
                   choices=["logreg", "eight_schools", "uneven_hier", "horseshoe", "horseshoe_nc", "sv", "sv_nc"],
                   help="non-default workloads: a full warmup+sampling run of that model family")
    p.add_argument("--samples", type=int, default=None, help="sampling iterations of a --workload run")
    p.add_argument("--full-samples", type=int, default=1000,
                   help="sampling iterations of the full run (500 warmup + this) reported beside the timed steps")
    p.add_argument("--oracle-samples", type=int, default=200,
                   help="transitions per chain of the FP64 oracle leg of the posterior check; 0 = skip "
                        "(with 50 the oracle's short chains understate their own Monte Carlo error)")
    p.add_argument("--diagnose", action="store_true",
                   help="--workload uneven_hier / sv: also run numpyro's algorithm (FP64 C restatement) on "
                        "the same chains and report its R-hat beside the GPU's")
    p.add_argument("--no-workloads", action="store_true",
                   help="skip the other benchmark configurations (eight schools, uneven hierarchical, horseshoe, SV)")
    return p.parse_args()


def workload_run(w, precision=None, num_warmup=None, num_samples=None, diagnose=False):
    """Full NUTS run (warmup + sampling, both timed with CUDA events) of one of the other
    benchmark configurations at its shape; returns the figures of one JSON sub-object."""
    import torch

    from numpyro_gb300 import NUTS, datasets, models

    if w == "eight_schools":
        y, s = datasets.eight_schools(0)
        model, C, W, S = models.HierarchicalNormal(y, s), 4, 1000, 1000
        shape = "J=8, 4 chains"
    elif w == "uneven_hier":
        ds = datasets.uneven_hierarchical(seed=0)
        # the [16384, S, 258] draws stay on the device; the chains of a strided sample of 64 models
        # are gathered there before the copy
        model, C, W, S = models.HierarchicalNormal(datasets=ds), 4 * len(ds), 1000, 1000
        shape = "4096 datasets, J in [4,256], 16384 chains"
    elif w in ("horseshoe", "horseshoe_nc"):
        X, y, _ = datasets.horseshoe_data(seed=0)
        nc = w == "horseshoe_nc"
        model, C, W, S = models.HorseshoeRegression(X, y, noncentered=nc), 256, 500, 500
        shape = "N=2000, P=1000 (D=2002), 256 chains, %s beta" % ("non-centred" if nc else "centred")
    else:
        r, _ = datasets.sv_returns(seed=0)
        nc = w == "sv_nc"
        model, C, W, S = models.StochasticVolatility(r, noncentered=nc), 256, 1000, 1000
        shape = "T=4096 (D=4098), 256 chains, %s walk" % ("non-centred" if nc else "centred")
    if num_warmup is not None:
        W = num_warmup
    if num_samples:
        S = num_samples
    kw = {"precision": precision} if precision else {}
    k = NUTS(model, num_chains=C, **kw)
    if precision:
        shape += ", precision " + precision
    log("%s: %s, %d warmup + %d samples" % (w, shape, W, S))
    st = k.init(1, W)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    ev[0].record()
    k.run_device(st, W, collect_start=W, collect=())
    ev[1].record()
    t_ticks = k.stats()["ticks"]
    out = k.run_device(st, S, collect=("z", "num_steps", "diverging"))
    ev[2].record()
    torch.cuda.synchronize()
    warm_s, samp_s = ev[0].elapsed_time(ev[1]) / 1e3, ev[1].elapsed_time(ev[2]) / 1e3
    ticks = k.stats()["ticks"] - t_ticks
    ns = out["num_steps"].cpu().numpy()
    divergences = int(out["diverging"].sum().item())
    # bulk-ESS and split R-hat of every coordinate, computed where the draws are (device_diagnostics);
    # only the subsample the --diagnose comparison with the oracle needs comes to the host
    from numpyro_gb300 import device_diagnostics as DD

    zd = out["z"]
    z = None
    extra = {}
    if w in ("sv", "sv_nc"):
        T = zd.shape[-1] - 2
        zall = zd
        if w == "sv_nc":  # the derived walk h = s * cumsum(h_base) as well
            h = (torch.exp(zd[..., T + 1:].double()) * torch.cumsum(zd[..., :T].double(), dim=-1)).float()
            zall = torch.cat([zd, h], dim=2)
            del h
        ess = DD.bulk_effective_sample_size(zall, chunk=256)
        rhat = DD.split_gelman_rubin(zall, chunk=256)
        ess_min, rhat_max = float(torch.nan_to_num(ess, nan=float("inf")).min()), float(torch.nan_to_num(rhat).max())
        ess_note = "min over all %d latent coordinates%s, computed on the device" % (
            zall.shape[-1], " and the derived walk h" if w == "sv_nc" else "")
        del zall
        if diagnose:
            idx = torch.tensor(list(range(0, T, 16)) + [T, T + 1], device=zd.device)
            z = zd.index_select(2, idx).cpu().numpy()
    elif w == "uneven_hier":
        M, cpm = model.num_models, C // model.num_models
        ess_m, rhat_m = per_model_diagnostics(zd, M, cpm, [model.chain_latent_dim(cpm * m, cpm) for m in range(M)])
        ess_min, rhat_max = float(ess_m.min()), float(rhat_m.max())
        ess_note = "min over all %d models of the per-model min bulk-ESS (its %d chains), computed on the device" % (
            M, cpm)
        extra = {"median_model_min_bulk_ess": float(ess_m.median()),
                 "models_rhat_over_1.01": int((rhat_m > 1.01).sum()),
                 "models_rhat_over_1.05": int((rhat_m > 1.05).sum()),
                 "models": M}
        picked = list(range(0, M, 64))  # the strided sample the --diagnose comparison runs on the oracle
        worst = [int(m) for m in torch.argsort(rhat_m, descending=True)[:4].tolist()]  # and the GPU's worst
        if diagnose:
            rows = torch.tensor([cpm * m + i for m in picked + worst for i in range(cpm)], device=zd.device)
            z = zd.index_select(0, rows).cpu().numpy()
        rhat = worst
    else:
        ess = DD.bulk_effective_sample_size(zd)
        rhat = DD.split_gelman_rubin(zd)
        ess_min, rhat_max = float(ess.min()), float(rhat.max())
        ess_note = "min over latent coordinates, computed on the device"
        if diagnose:
            z = zd.cpu().numpy()
    del out, zd
    grad_evals = float(ns.sum())
    burst, _, hbm, peak_kind = measured_peaks()
    if w == "eight_schools":
        # 4 chains: a latency figure, the time of one leapfrog step of one chain
        roof = {"bound": "latency", "us_per_leapfrog_step": 1e6 * samp_s / (grad_evals / C)}
    elif w == "uneven_hier":
        # 24 D_c bytes of chain state (z, r, grad read and written) + 8 J_c bytes of data per evaluation
        J = np.array([model.chain_latent_dim(c, 4) - 2 for c in range(C)], np.float64)
        nbytes = float(np.sum(ns.sum(axis=1) * (24.0 * (J + 2) + 8.0 * J)))
        gbs = nbytes / samp_s / 1e9
        roof = {"bound": "hbm", "achieved": gbs, "peak": hbm, "unit": "GB/s", "frac": gbs / hbm,
                "bytes_per_grad_eval": "24 (J_c + 2) + 8 J_c", "peak_kind": peak_kind}
    elif w in ("sv", "sv_nc"):
        T = model.latent_dim - 2
        per = 24.0 * (T + 2) + 4.0 * T
        gbs = grad_evals * per / samp_s / 1e9
        roof = {"bound": "hbm", "achieved": gbs, "peak": hbm, "unit": "GB/s", "frac": gbs / hbm,
                "bytes_per_grad_eval": per, "peak_kind": peak_kind}
    else:
        N, P = 2000, 1000
        tf = grad_evals * 4.0 * N * P / samp_s / 1e12
        roof = {"bound": "tensor" if precision == "bf16x3" else "fp32", "achieved": tf, "peak": burst,
                "unit": "TFLOP/s", "frac": tf / burst, "flop_per_grad_eval": 4.0 * N * P,
                "peak_kind": peak_kind + " burst bf16"}
    diag = None
    if diagnose:
        diag = _oracle_diagnosis(w, model, z, picked if w == "uneven_hier" else None, W, S, rhat if w == "uneven_hier"
                                 else None)
    line = {"workload": w, "shape": shape, "chains": C, "num_warmup": W, "num_samples": S,
            "warmup_s": warm_s, "sampling_s": samp_s, "grad_evals_per_s_sampling": grad_evals / samp_s,
            "mean_num_steps": float(ns.mean()), "divergences": divergences,
            "min_bulk_ess": ess_min, "min_bulk_ess_per_s_sampling": ess_min / samp_s,
            "min_bulk_ess_per_s_total": ess_min / (warm_s + samp_s), "rhat_max": rhat_max,
            "ess_definition": ess_note, **extra, "ticks_sampling": ticks if ticks else None,
            "us_per_tick": 1e6 * samp_s / ticks if ticks else None,
            "engine": "tick engine + CUDA graphs" if ticks else "persistent (one launch)",
            "roofline": roof, "tuning": k.tuning()}
    if diag is not None:
        line["fp64_oracle_diagnosis"] = diag
    k.close()
    return line


def _oracle_diagnosis(w, model, z, picked, W, S, model_rhat):
    """Runs numpyro's algorithm (the FP64 C restatement, oracle/nuts_ref.c) on chains of the same
    workload with the same chain ids and random stream as the GPU run, and reports its split
    R-hat and divergences beside the GPU's on the same chains: whether the GPU's R-hat reflects
    the sampler on this posterior or the engine."""
    from oracle import build_oracle

    lib = build_oracle.load("f64")
    cores = len(os.sched_getaffinity(0))
    cm = build_oracle.model_from_registry(model, 4)
    out = {"oracle": "FP64 C restatement of numpyro's NUTS, same chain ids and Philox stream, %d warmup + "
                     "%d samples, %d host threads" % (W, S, cores)}
    if w == "uneven_hier":
        # every model of the strided sample, 4 chains each with the GPU's chain ids and stream: the
        # distribution of per-model R-hat and ESS under numpyro's algorithm beside the GPU's; then
        # the GPU's four worst models of all (model_rhat: their ids; their draws follow in z)
        worst_rows = []
        for i, m in enumerate(model_rhat or []):
            D = model.chain_latent_dim(4 * m, 4)
            res = build_oracle.run_model(lib, cm, model.latent_dim, 4, W, S, seed=1, first_chain=4 * m,
                                         threads=min(cores, 4))
            e_o, r_o = min_bulk_ess(res["samples"][:, :, :D])
            k = len(picked) + i
            e_g, r_g = min_bulk_ess(z[4 * k:4 * k + 4, :, :D])
            worst_rows.append({"model": int(m), "J": D - 2, "gpu_rhat": r_g, "oracle_rhat": r_o,
                               "gpu_min_bulk_ess": e_g,
                               "oracle_min_bulk_ess": e_o, "oracle_divergences": int(res["diverging"].sum()),
                               "gpu_chain_sds_of_log_tau": [float(np.std(z[4 * k + j, :, 1])) for j in range(4)],
                               "oracle_chain_sds_of_log_tau": [float(np.std(res["samples"][j, :, 1]))
                                                               for j in range(4)]})
        out["gpu_worst_models_of_all"] = worst_rows
        g_r, g_e, o_r, o_e, o_div, rows = [], [], [], [], 0, []
        for i, m in enumerate(picked):
            D = model.chain_latent_dim(4 * m, 4)
            res = build_oracle.run_model(lib, cm, model.latent_dim, 4, W, S, seed=1, first_chain=4 * m,
                                         threads=min(cores, 4))
            e_o, r_o = min_bulk_ess(res["samples"][:, :, :D])
            e_g, r_g = min_bulk_ess(z[4 * i:4 * i + 4, :, :D])
            g_r.append(r_g), g_e.append(e_g), o_r.append(r_o), o_e.append(e_o)
            o_div += int(res["diverging"].sum())
            rows.append({"model": int(m), "J": D - 2, "gpu_rhat": r_g, "oracle_rhat": r_o, "gpu_min_bulk_ess": e_g,
                         "oracle_min_bulk_ess": e_o, "oracle_divergences": int(res["diverging"].sum())})
        g_r, o_r, g_e, o_e = map(np.asarray, (g_r, o_r, g_e, o_e))
        out.update({"models": len(picked),
                    "gpu_models_rhat_over_1.01": int(np.sum(g_r > 1.01)),
                    "oracle_models_rhat_over_1.01": int(np.sum(o_r > 1.01)),
                    "gpu_models_rhat_over_1.05": int(np.sum(g_r > 1.05)),
                    "oracle_models_rhat_over_1.05": int(np.sum(o_r > 1.05)),
                    "gpu_rhat_max": float(g_r.max()), "oracle_rhat_max": float(o_r.max()),
                    "gpu_median_min_bulk_ess": float(np.median(g_e)), "oracle_median_min_bulk_ess": float(np.median(o_e)),
                    "oracle_divergences": o_div,
                    "worst_models": sorted(rows, key=lambda r: -max(r["gpu_rhat"], r["oracle_rhat"]))[:6]})
        return out
    if w in ("sv", "sv_nc"):
        nc = min(16, cores)
        T = model.latent_dim - 2
        res = build_oracle.run_model(lib, cm, model.latent_dim, nc, W, S, seed=1, threads=nc)
        idx = list(range(0, T, 16)) + [T, T + 1]
        zo = res["samples"][:, :, idx]
        e_o, r_o = min_bulk_ess(zo)
        e_g, r_g = min_bulk_ess(z[:nc, :, :len(idx)])
        out.update({"chains": nc, "gpu_rhat_same_chains": r_g, "oracle_rhat": r_o, "gpu_min_bulk_ess_same_chains": e_g,
                    "oracle_min_bulk_ess": e_o, "oracle_divergences": int(res["diverging"].sum()),
                    "oracle_s": [float(np.exp(zo[c, :, -1]).mean()) for c in range(nc)]})
        return out
    return None


def run_workload(args):
    """--workload: one JSON line for one of the other benchmark configurations."""
    print(json.dumps(workload_run(args.workload, args.precision,
                                  None if args.num_warmup == 500 else args.num_warmup, args.samples,
                                  diagnose=args.diagnose)))
    return 0


def run_potential_only(args):
    """Times the logistic potential + adjoint for all chains alone (profiling entry)."""
    import torch

    from numpyro_gb300 import NUTS, datasets, models

    precision = args.precision or ("bf16x3" if _tc_available() else "fp32")
    X, y, beta = datasets.covtype_like(seed=0, n=args.n)
    C = args.chains
    kernel = NUTS(models.LogisticRegression(X, y), num_chains=C, precision=precision)
    rng = np.random.default_rng(0)
    z = torch.as_tensor((beta[None, :] + 0.01 * rng.standard_normal((C, X.shape[1]))).astype(np.float32),
                        device="cuda")
    for _ in range(max(1, args.warmup)):
        kernel.potential_and_grad(z)
    torch.cuda.synchronize()
    ms = _time_potential(kernel, type("S", (), {"z": z})(), reps=args.reps)
    flop = 4.0 * X.shape[0] * X.shape[1] * C
    burst, _, _, kind = measured_peaks()
    print(json.dumps({"mode": "potential", "precision": precision, "n": X.shape[0], "d": X.shape[1], "chains": C,
                      "launch_ms": ms, "tflops": flop / ms / 1e9, "frac_bf16_peak": flop / ms / 1e9 / burst,
                      "peak_kind": kind}))
    kernel.close()
    return 0


_T0 = time.perf_counter()


def log(msg):
    """Phase progress on stderr (the JSON result line goes to stdout)."""
    sys.stderr.write("[bench %7.1fs] %s\n" % (time.perf_counter() - _T0, msg))
    sys.stderr.flush()


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        d = json.load(open(path))
        return d.get("bf16_tflops", 1900.0), d.get("bf16_tflops_sustained", 1700.0), d.get("hbm_gbs", 6800.0), \
            "measured"
    return 1900.0, 1700.0, 6800.0, "fallback"


class Clocks:
    """Samples nvidia-smi clocks/throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None
        # raw samples (summarised in the JSON line); GBN_CLOCKS_CSV keeps them somewhere else
        self.path = os.environ.get("GBN_CLOCKS_CSV", os.path.join(tempfile.gettempdir(), "gbn_clocks_bench.csv"))

    def start(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait()
        self.f.close()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        med = float(np.median(sm)) if sm else None
        return {"sm_mhz": med, "sm_max_mhz": smax, "reasons": sorted(reasons), "samples": len(sm)}


def per_model_diagnostics(zd, num_models, chains_per_model, dims, chunk=4096):
    """Per-model min bulk-ESS and max split R-hat of a batch of models' draws zd [models x chains,
    draws, padded dim] (model m's chains are rows m * chains_per_model ...), over each model's own
    dims[m] coordinates, on zd's device without copying the draws (a model-major view)."""
    import torch

    from numpyro_gb300 import device_diagnostics as DD

    M, cpm, Dmax = num_models, chains_per_model, zd.shape[-1]
    zm = zd.view(M, cpm, zd.shape[1], Dmax).permute(1, 2, 0, 3)  # [chains of a model, draws, model, coord]
    ess = DD.bulk_effective_sample_size(zm, chunk=chunk)
    rhat = DD.split_gelman_rubin(zm, chunk=chunk)
    d = torch.as_tensor(dims, device=zd.device)
    valid = torch.arange(Dmax, device=zd.device)[None, :] < d[:, None]  # padding excluded
    ess_m = torch.where(valid, torch.nan_to_num(ess, nan=float("inf")), torch.full_like(ess, float("inf")))
    rhat_m = torch.where(valid, torch.nan_to_num(rhat), torch.zeros_like(rhat))
    return ess_m.min(dim=1).values, rhat_m.max(dim=1).values


def min_bulk_ess(z):
    from numpyro_gb300.diagnostics import bulk_effective_sample_size, split_gelman_rubin

    if z.shape[1] < 4:  # split diagnostics need at least 4 draws per chain
        return float("nan"), float("nan")
    ess, rhat = [], []
    for d0 in range(0, z.shape[-1], 64):  # blocks of coordinates, vectorised over each block
        blk = np.asarray(z[..., d0:d0 + 64], np.float64)
        ess.append(np.atleast_1d(bulk_effective_sample_size(blk)))
        rhat.append(np.atleast_1d(split_gelman_rubin(blk)))
    ess, rhat = np.concatenate(ess), np.concatenate(rhat)
    return float(ess.min()), float(np.max(rhat))


def cpu_baseline(X, y, chains, num_samples, init=None, num_warmup=0, budget_s=0.0, prec="f32"):
    """Times the C oracle of numpyro's NUTS (OpenMP, one chain per thread) on a bounded
    sample of the workload: ``chains`` chains for ``num_samples`` transitions, started
    either from an adapted state (``init`` = (z, step, inverse mass)) or from
    init_to_uniform with a (time-bounded) Stan warmup of ``num_warmup`` iterations."""
    from oracle import build_oracle

    lib = build_oracle.load(prec)
    cores = len(os.sched_getaffinity(0))
    res = build_oracle.run_logreg(lib, X, y, chains=chains, num_warmup=num_warmup, num_samples=num_samples,
                                  seed=0, threads=min(cores, chains), init=init, warmup_budget_s=budget_s)
    ess, rhat = min_bulk_ess(res["samples"])
    start = "the GPU run's adapted state" if init is not None else \
        "init_to_uniform + %d-iteration Stan warmup (%.0f s budget)" % (num_warmup, budget_s)
    return {
        "value": ess / res["sampling_s"],
        "unit": "ESS/s",
        "cores": res["threads"],
        "kind": "port",
        "grad_evals_per_s": res["sampling_grad_evals"] / res["sampling_s"],
        "sampling_s": res["sampling_s"],
        "warmup_s": res["warmup_s"],
        "min_bulk_ess": ess,
        "sample": "%d chains x %d NUTS transitions (max_tree_depth 10) on the full N=%d x %d data from %s; "
                  "%s C oracle of numpyro's NUTS, one chain per host thread; ESS/s = min bulk-ESS of those "
                  "draws / sampling seconds" % (res["chains"], num_samples, X.shape[0], X.shape[1], start, prec),
    }


def oracle_moment_check(X, y, state, zgpu, chains, transitions):
    """The GPU posterior against the FP64 oracle's: the C oracle (FP64 build) runs ``chains``
    chains for ``transitions`` NUTS transitions from the GPU's adapted state, and each
    coefficient's posterior mean and sd are compared, in units of their Monte Carlo standard
    errors combined over both samples (diagnostics.mcse_mean, mcse_sd)."""
    from oracle import build_oracle
    from numpyro_gb300.diagnostics import bulk_effective_sample_size, mcse_mean, mcse_sd

    lib = build_oracle.load("f64")
    cores = len(os.sched_getaffinity(0))
    init = (state.z[:chains].cpu().numpy(), state.adapt_state.step_size[:chains].cpu().numpy(),
            state.adapt_state.inverse_mass_matrix[:chains].cpu().numpy())
    # the oracle chains start where the GPU chains stood; they continue from there on their own stream
    res = build_oracle.run_logreg(lib, X, y, chains=chains, num_warmup=0, num_samples=transitions, seed=7,
                                  threads=min(cores, chains), init=init, first_chain=0)
    zo = np.asarray(res["samples"], np.float64)
    zg = np.asarray(zgpu, np.float64)

    def moments(z):
        return (z.mean(axis=(0, 1)), z.std(axis=(0, 1), ddof=1), mcse_mean(z), mcse_sd(z),
                np.atleast_1d(bulk_effective_sample_size(z)))

    mg, sg, emg, esg, _ = moments(zg)
    mo, so, emo, eso, eo = moments(zo)
    zm = np.abs(mg - mo) / np.sqrt(emg ** 2 + emo ** 2)
    zs = np.abs(sg - so) / np.sqrt(esg ** 2 + eso ** 2)
    # what chance allows for n independent comparisons: n p3 + 3 sd + 1 beyond 3 MCSE, and all
    # within the Bonferroni bound at a 1 % family-wise rate
    from scipy.stats import norm

    n = zm.size + zs.size
    p3 = 2 * norm.sf(3.0)
    return {"oracle": "FP64 C restatement of numpyro's NUTS, %d chains x %d transitions from the GPU's "
                      "adapted state (%.0f s on %d host threads)" % (chains, transitions, res["sampling_s"],
                                                                    res["threads"]),
            "gpu_draws": "%d chains x %d draws" % zg.shape[:2],
            "max_abs_dmean_over_mcse": float(zm.max()), "max_abs_dsd_over_mcse": float(zs.max()),
            "coords_beyond_3_mcse": int(np.sum(zm > 3) + np.sum(zs > 3)), "coords": int(zg.shape[-1]),
            "chance_allows_beyond_3": int(np.floor(n * p3 + 3 * np.sqrt(n * p3 * (1 - p3)) + 1)),
            "bonferroni_bound": float(norm.isf(0.005 / n)),
            "oracle_min_bulk_ess": float(eo.min())}


def reference_leg(X, y, chains, num_warmup, num_samples, cores, budget_s=300.0):
    """The reference arm's timed CPU work: numpyro's NUTS as the FP32 C restatement (numpyro's
    default dtype) on the host cores, from init_to_uniform with the Stan warmup, ``chains``
    chains one after another, each evaluating its potential on all ``cores`` threads (rows
    split across the threads, as XLA's CPU backend splits one chain's matrix products)."""
    from oracle import build_oracle

    lib = build_oracle.load("f32")
    model = build_oracle.Model("logreg", X=X, y=y, row_threads=cores)
    res = build_oracle.run_model(lib, model, X.shape[1], chains, num_warmup, num_samples, seed=0, threads=cores,
                                 warmup_budget_s=budget_s)
    ess, rhat = min_bulk_ess(res["samples"])
    sample = ("%d of the 1024 chains: init_to_uniform, %d-iteration Stan warmup (%.0f s, %s), then %d sampling "
              "transitions each (max_tree_depth 10) on the full N=%d x %d data; FP32 C restatement of numpyro's "
              "NUTS with each chain's potential split across %d host threads; ESS/s = min bulk-ESS of the sampling "
              "draws / sampling seconds" % (chains, num_warmup, res["warmup_s"],
                                            "completed" if res["warmup_s"] < budget_s else "cut at the time budget",
                                            num_samples, X.shape[0], X.shape[1], cores))
    return {"value": ess / res["sampling_s"], "unit": "ESS/s", "cores": cores, "kind": "port", "sample": sample,
            "grad_evals_per_s": res["sampling_grad_evals"] / res["sampling_s"], "sampling_s": res["sampling_s"],
            "warmup_s": res["warmup_s"], "warmup_grad_evals": res["warmup_grad_evals"], "min_bulk_ess": ess,
            "rhat_max": rhat}


def run_reference(args):
    """--impl reference: numpyro itself cannot run here (no jax); its NUTS algorithm runs as the
    C restatement on the host cores, on the workload of our arm: the same 500-iteration Stan
    warmup, then --steps sampling steps of --iters-per-step transitions, on a bounded sample of
    4 of the 1024 chains (reference_leg)."""
    from numpyro_gb300 import datasets

    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    X, y, _ = datasets.covtype_like(seed=0, n=args.n)
    cores = len(os.sched_getaffinity(0))
    chains = 4
    B = getattr(args, "iters_per_step", 10)
    S = max(4, args.steps * B)
    num_warmup = getattr(args, "num_warmup", 500)
    cb = reference_leg(X, y, chains, num_warmup, S, cores)
    value = cb["value"]
    line = {"metric": METRIC, "value": value, "unit": "ESS/s", "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * cb["sampling_s"] / max(1, args.steps),
            "higher_is_better": True, "scaling": "weak", "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "chains_timed": chains, "iters_per_step": B, "num_warmup": num_warmup},
            "cpu_baseline": cb,
            "e2e": {"value": value, "unit": "ESS/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "grad_evals_per_s": cb["grad_evals_per_s"], "vs_baseline": None}
    print(json.dumps(line))
    return 0


def replica_chains(rank, chains):
    """Replicas: one seed for every rank, and rank r runs the global chains r C .. (r + 1) C - 1
    (first_chain): every draw is addressed by (seed, global chain id, ...) in the counter-based
    streams, so an N-GPU run is the single-GPU run of N C chains split by chain, chain for chain.
    Nothing is exchanged during sampling."""
    return 1000, rank * chains


def reduce_over_ranks(dist, total_ms, ess, grad_evals, device="cpu"):
    """Whole-job figures of a replica run: the slowest rank's time, and the ranks' ESS and
    gradient evaluations summed (each rank samples independent chains)."""
    import torch

    t = torch.tensor([total_ms, ess, float(grad_evals)], dtype=torch.float64, device=device)
    tmax = t.clone()
    dist.all_reduce(tmax, op=dist.ReduceOp.MAX)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(tmax[0]), float(t[1]), int(t[2])


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.mode == "potential":
        return run_potential_only(args)
    if args.workload != "logreg":
        return run_workload(args)
    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    from numpyro_gb300 import NUTS, datasets, models

    precision = args.precision or ("bf16x3" if _tc_available() else "fp32")
    X, y, _ = datasets.covtype_like(seed=0, n=args.n)
    model = models.LogisticRegression(X, y)
    C = args.chains
    seed, first_chain = replica_chains(rank, C)
    kernel = NUTS(model, num_chains=C, engine=args.engine, precision=precision, first_chain=first_chain)
    t0 = time.perf_counter()
    log("init %d chains, precision %s" % (C, precision))
    state = kernel.init(seed, args.num_warmup)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record()
    kernel.run_device(state, args.num_warmup, collect_start=args.num_warmup, collect=())
    ev1.record()
    torch.cuda.synchronize()
    warmup_ms = ev0.elapsed_time(ev1)
    B = args.iters_per_step
    flush = torch.empty(128 * 1024 * 1024, dtype=torch.float32, device="cuda")
    for _ in range(args.warmup):
        kernel.run_device(state, B, collect=())
    torch.cuda.synchronize()
    # ---------------- timed region (device-resident inputs)
    clocks = Clocks(local)
    log("warmup done (%.1f s); timed steps" % (warmup_ms / 1e3))
    clocks.start()
    ticks0 = kernel.stats()["ticks"]
    zs, nsteps, step_ms = [], [], []
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    for _ in range(args.steps):
        flush.fill_(1.0)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        out = kernel.run_device(state, B, collect=("z", "num_steps"))
        b.record()
        zs.append(out["z"])
        nsteps.append(out["num_steps"])
        b.synchronize()
        step_ms.append(a.elapsed_time(b))
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    ticks = kernel.stats()["ticks"] - ticks0
    clk = clocks.stop()
    total_ms = float(sum(step_ms))
    z = torch.cat(zs, dim=1).cpu().numpy()
    grad_evals = int(torch.cat(nsteps, dim=1).sum().item())
    ess, rhat = min_bulk_ess(z)
    if dist:
        total_ms, ess, grad_evals = reduce_over_ranks(dist, total_ms, ess, grad_evals, device="cuda")
    value = ess / (total_ms / 1e3)
    # ---------------- dominant kernel: the potential, timed alone on the same stream
    log("timed steps done: %.1f ms/step" % (total_ms / max(1, args.steps)))
    pot_ms = _time_tick_potential(kernel, reps=10)
    burst, sustained, hbm, peak_kind = measured_peaks()
    flop = 4.0 * X.shape[0] * X.shape[1] * C
    achieved = flop / (pot_ms / 1e3) / 1e12
    # DRAM bytes (read + write) of one launch of the dominant kernel, from the ncu capture summarised
    # in profiles/ for this kernel at 1024 chains
    traffic, traffic_src = profiled_traffic(
        "logreg_tc_kernel_covtype_1024chains" if precision == "bf16x3" else "logreg_simt_kernel_covtype_1024chains",
        X.shape[0])
    if C != 1024:
        traffic, traffic_src = None, None
    roofline = {"bound": "tensor", "achieved": achieved, "peak": burst, "unit": "TFLOP/s",
                "frac": achieved / burst, "traffic": traffic, "traffic_unit": "bytes per launch",
                "traffic_source": traffic_src,
                "peak_kind": peak_kind + " burst bf16",
                "kernel": ("logreg_tc_kernel (bf16x3; coefficient split and row-group finish fused into the "
                           "state-machine kernel)" if precision == "bf16x3" else
                           "logreg potential (fp32: logreg_simt_kernel + logreg_finish_kernel)"),
                "algorithmic_flop_per_launch": flop, "launch_ms": pot_ms}
    if precision == "bf16x3":
        # the special-function unit's share of the tensor-core potential (one ex2 per logit, tanh for
        # half the rows, one rcp and one lg2 per 8 rows), against its own measured peak on this GPU
        roofline["special_function_unit"] = _sfu_roofline(pot_ms, X.shape[0], C)
    # ---------------- end to end through the public API with host buffers
    e2e = None
    if not args.no_e2e:
        log("e2e")
        e2e = _e2e(kernel, state, args.steps, B)
    # ---------------- the configuration's full run: 500 warmup + 1000 sampling iterations
    full, zfull = None, None
    if args.full_samples > 0:
        log("full run: %d sampling iterations" % args.full_samples)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        out = kernel.run_device(state, args.full_samples, collect=("z", "num_steps"))
        b.record()
        b.synchronize()
        samp_ms = a.elapsed_time(b)
        full_evals = int(out["num_steps"].sum().item())
        zfull = out["z"].cpu().numpy()
        del out
        ess_f, rhat_f = min_bulk_ess(zfull)
        if dist:
            samp_ms, ess_f, full_evals = reduce_over_ranks(dist, samp_ms, ess_f, full_evals, device="cuda")
        full = {"num_warmup": args.num_warmup, "num_samples": args.full_samples, "warmup_s": warmup_ms / 1e3,
                "sampling_s": samp_ms / 1e3, "min_bulk_ess": ess_f,
                "min_bulk_ess_per_s_total": ess_f / ((warmup_ms + samp_ms) / 1e3),
                "min_bulk_ess_per_s_sampling": ess_f / (samp_ms / 1e3), "rhat_max": rhat_f,
                "grad_evals_per_s_sampling": full_evals / (samp_ms / 1e3),
                "definition": "min over the 55 coefficients of bulk-ESS of all post-warmup draws, divided by "
                              "warmup + sampling seconds (total) or sampling seconds"}
    plain = None
    if args.plain_steps > 0 and world == 1:
        log("plain engine comparison")
        plain = _plain_compare(model, state, C, seed, args.plain_steps, B, args.num_warmup, value,
                               grad_evals / (total_ms / 1e3))
    line = {
        "metric": METRIC, "value": value, "unit": "ESS/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / max(1, args.steps), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "bf16x3" if precision == "bf16x3" else "f32",
        "data": "synthetic", "impl": "ours",
        "config": {"workload": WORKLOAD, "chains": C, "n": X.shape[0], "d": X.shape[1], "engine": args.engine,
                   "precision": precision, "iters_per_step": B, "l2": "flushed (512 MB write) before each step",
                   "parallelism": "replicas, chains sharded by global chain id" if world > 1 else "single"},
        "grad_evals_per_s": grad_evals / (total_ms / 1e3),
        "min_bulk_ess": ess, "rhat_max": rhat, "warmup_s": warmup_ms / 1e3,
        "setup_s": time.perf_counter() - t0,
        "roofline": roofline, "clocks": clk, "gpu_launches": int(ticks * _launches_per_tick(precision)),
        "e2e": e2e, "plain_engine": plain, "full_run": full,
    }
    if rank == 0 and not args.no_cpu and world == 1:
        try:
            nc = min(16, len(os.sched_getaffinity(0)))
            init = (state.z[:nc].cpu().numpy(), state.adapt_state.step_size[:nc].cpu().numpy(),
                    state.adapt_state.inverse_mass_matrix[:nc].cpu().numpy())
            log("cpu baseline")
            line["cpu_baseline"] = cpu_baseline(X, y, chains=nc, num_samples=args.cpu_samples, init=init)
        except Exception as ex:  # the baseline is reported, never required for the GPU number
            line["cpu_baseline"] = {"value": None, "error": str(ex)[:200]}
        if args.oracle_samples > 0 and zfull is not None:
            try:
                log("FP64 oracle posterior check")
                line["posterior_vs_fp64_oracle"] = oracle_moment_check(X, y, state, zfull, nc, args.oracle_samples)
            except Exception as ex:
                line["posterior_vs_fp64_oracle"] = {"error": str(ex)[:200]}
    del zfull
    if rank == 0 and not args.no_workloads and world == 1:
        kernel.close()
        kernel = None
        line["workloads"] = {}
        for w, prec in (("eight_schools", None), ("uneven_hier", None),
                        ("horseshoe_nc", "bf16x3" if _tc_available() else None), ("sv", None)):
            try:
                line["workloads"][w] = workload_run(w, prec)
            except Exception as ex:
                line["workloads"][w] = {"error": str(ex)[:200]}
    if rank == 0:
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()
    if kernel is not None:
        kernel.close()
    return 0


def _tc_available():
    try:
        from numpyro_gb300 import _lib

        return bool(getattr(_lib.load(), "gbn_tc_available", lambda: 0)())
    except Exception:
        return False


# special-function operations per logit of the tensor-core logistic epilogue (logreg_tc.cu,
# epilogue_part): one ex2; tanh for half the rows; one rcp per 8 rows for the other half; one lg2
# per 8 rows
SFU_OPS_PER_LOGIT = 1.0 + 0.5 + 0.5 / 8 + 1.0 / 8


def _sfu_roofline(launch_ms, n, chains):
    """Special-function operations of one tensor-core potential launch (SFU_OPS_PER_LOGIT per
    logit) per second, against the unit's peak measured on this GPU for the same mix
    (gbn_measure_sfu)."""
    import torch

    from numpyro_gb300 import _lib

    peak = ctypes.c_double(0.0)
    rc = _lib.load().gbn_measure_sfu(ctypes.c_void_p(torch.cuda.current_stream().cuda_stream), 2,
                                     ctypes.byref(peak))
    ops = SFU_OPS_PER_LOGIT * n * chains
    achieved = ops / (launch_ms * 1e-3)
    if rc != 0 or peak.value <= 0:
        return {"bound": "sfu", "achieved": achieved / 1e12, "peak": None, "unit": "Tops/s", "frac": None}
    return {"bound": "sfu", "achieved": achieved / 1e12, "peak": peak.value / 1e12, "unit": "Tops/s",
            "frac": achieved / peak.value, "ops_per_launch": ops, "ops_per_logit": SFU_OPS_PER_LOGIT,
            "peak_kind": "measured in this run (gbn_measure_sfu: the epilogue's ex2/tanh/rcp/lg2 mix on every SM)"}


def _launches_per_tick(precision):
    # advance_kernel, then the potential: on the tensor cores the tcgen05 kernel alone (the
    # coefficient split and the row-group finish run inside advance_kernel; GBN_FUSE_TICK=0 launches
    # them separately, 4 per tick), on CUDA cores logreg_simt + logreg_finish
    if precision == "bf16x3":
        return 4 if os.environ.get("GBN_FUSE_TICK", "1") == "0" else 2
    return 3


def _time_potential(kernel, state, reps=10, batch=20):
    """Average duration of one potential launch (for the tensor-core path: coefficient split,
    tcgen05 kernel and row-group finish), from CUDA events on the kernel's stream around
    ``batch`` back-to-back launches, as the tick loop issues them; median over ``reps`` batches."""
    import torch

    z = state.z.clone()
    kernel.potential_and_grad(z)
    torch.cuda.synchronize()
    ts = []
    for _ in range(reps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(batch):
            kernel.potential_and_grad(z)
        b.record()
        b.synchronize()
        ts.append(a.elapsed_time(b) / batch)
    return float(np.median(ts))


def _time_tick_potential(kernel, reps=10, batch=20):
    """Duration of one potential launch as the tick engine issues it (for the tensor-core path the
    tcgen05 kernel alone; gbn_time_potential), from CUDA events around ``batch`` back-to-back
    launches on the current stream; median over ``reps`` batches."""
    import torch

    from numpyro_gb300 import _lib

    lib = _lib.load()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    ts = []
    for _ in range(reps):
        v = ctypes.c_float(0.0)
        _lib.check(lib.gbn_time_potential(kernel._handle, stream, batch, ctypes.byref(v)), kernel._handle)
        ts.append(v.value)
    return float(np.median(ts))


def profiled_traffic(kernel_name, n_rows):
    """DRAM bytes (read + write) of one launch of a profiled kernel, from the ncu summary in
    profiles/ (its ``traffic_bytes_per_launch`` line, captured at ``rows``); scaled to n_rows
    rows, since the launch streams the design matrix once."""
    import re

    path = os.path.join(ROOT, "profiles", kernel_name + ".md")
    try:
        text = open(path).read()
    except OSError:
        return None, None
    m = re.search(r"traffic_bytes_per_launch\s*=\s*([0-9.eE+]+)\s*\(rows\s*=\s*([0-9]+)", text)
    if not m:
        return None, None
    t, rows = float(m.group(1)), int(m.group(2))
    return t * n_rows / rows, "ncu capture (%s), %d rows%s" % (
        os.path.basename(path), rows, "" if rows == n_rows else ", scaled to %d rows" % n_rows)


def _state_leaves(st):
    a = st.adapt_state
    return [st.i, st.z, st.z_grad, st.potential_energy, st.energy, st.num_steps, st.accept_prob,
            st.mean_accept_prob, st.diverging, a.step_size, a.inverse_mass_matrix, a.mass_matrix_sqrt,
            a.mass_matrix_sqrt_inv, a.ss_state, a.mm_state[0], a.mm_state[1], a.mm_state[2], a.window_idx,
            st.rng_key]


def _plain_compare(model, state, C, seed, steps, B, num_warmup, fused_value, fused_gps):
    """The plain engine (lock-step trees as under numpyro's vmap, FP32 CUDA-core potential)
    resumed from the fused run's adapted state: same metric, same chains."""
    import torch

    from numpyro_gb300 import NUTS

    k = NUTS(model, num_chains=C, engine="plain", precision="fp32")
    st = k.init(seed, num_warmup)
    for d, s in zip(_state_leaves(st), _state_leaves(state)):
        d.copy_(s)
    k.run_device(st, 1, collect=())
    zs, ns, ms = [], [], 0.0
    for _ in range(steps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        out = k.run_device(st, B, collect=("z", "num_steps"))
        b.record()
        b.synchronize()
        ms += a.elapsed_time(b)
        zs.append(out["z"])
        ns.append(out["num_steps"])
    z = torch.cat(zs, dim=1).cpu().numpy()
    ess, rhat = min_bulk_ess(z)
    gps = float(torch.cat(ns, dim=1).sum().item()) / (ms / 1e3)
    k.close()
    return {"value": ess / (ms / 1e3), "unit": "ESS/s", "grad_evals_per_s": gps, "ms_per_step": ms / steps,
            "steps": steps, "min_bulk_ess": ess, "rhat_max": rhat,
            "fused_over_plain_ess_per_s": fused_value / (ess / (ms / 1e3)) if ess > 0 else None,
            "fused_over_plain_grad_evals_per_s": fused_gps / gps}


def _e2e(kernel, state, steps, B):
    """Same metric through the public API with host-resident state: every step
    copies the chain state host->device, runs B transitions, and copies the
    draws and state back."""
    import torch

    host = {}

    def leaves(st):
        a = st.adapt_state
        return [st.i, st.z, st.z_grad, st.potential_energy, st.energy, st.num_steps, st.accept_prob,
                st.mean_accept_prob, st.diverging, a.step_size, a.inverse_mass_matrix, a.mass_matrix_sqrt,
                a.mass_matrix_sqrt_inv, a.ss_state, a.mm_state[0], a.mm_state[1], a.mm_state[2], a.window_idx,
                st.rng_key]

    dev = leaves(state)
    host = [t.cpu().pin_memory() for t in dev]
    h2d = sum(t.numel() * t.element_size() for t in host)
    zs = []
    d2h = 0
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    a.record()
    for _ in range(steps):
        for d, h in zip(dev, host):
            d.copy_(h, non_blocking=True)
        out = kernel.run_device(state, B, collect=("z", "num_steps"))
        zh = torch.empty(out["z"].shape, dtype=out["z"].dtype, pin_memory=True)
        zh.copy_(out["z"], non_blocking=True)
        for d, h in zip(dev, host):
            h.copy_(d, non_blocking=True)
        zs.append(zh)
        d2h = zh.numel() * 4 + h2d
    b.record()
    torch.cuda.synchronize()
    ms = a.elapsed_time(b)
    z = torch.cat(zs, dim=1).numpy()
    ess, _ = min_bulk_ess(z)
    return {"value": ess / (ms / 1e3), "unit": "ESS/s", "h2d_bytes_per_step": int(h2d),
            "d2h_bytes_per_step": int(d2h), "ms_per_step": ms / steps}


if __name__ == "__main__":
    sys.exit(main())
