"""Throughput of the MCMC over SNP inclusion on one GB300.

Workload (default "scan"): n = 10,000 individuals, p = 500,000 SNPs of
synthetic genotypes in LD blocks of 50 (AR(1) latent Gaussian, rho 0.8,
thresholded to MAF ~ U(0.05, 0.5)), 30 causal SNPs, additive coding,
32 chains, the Rao-Blackwellised scan of all SNPs every iteration (n_rao = 1),
add/remove/swap moves with the adaptive proposal.

A step is one MCMC iteration of every chain: the moves of all chains, the
p-wide scan, the proposal update.  value = chain-iterations per second with the
genotypes resident on the device; e2e = the same metric through the C ABI from
host buffers (genotype upload, precompute, run, read-back of the traces and
posteriors inside the timed region).

--impl reference times the CPU restatement of the reference sampler
(oracle/port) on the host cores on a bounded sample of the same workload.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np

from bmagwa_gb300.workloads import WORKLOADS, make_data, options, scan_terms  # noqa: E402

# sizes of the inclusion-ESS leg per workload: burn-in iterations, then
# sampled iterations (thinned samples = sampled / thin)
ESS_LEG = {"scan": (1000, 2000), "batched": (10000, 20000), "plain": (10000, 20000)}

PEAKS = os.path.join(ROOT, "MEASURED_PEAKS.json")
FALLBACK_HBM = 6800.0
FALLBACK_BF16_SUSTAINED = 1700.0


def env_rank():
    from bmagwa_gb300 import replicas
    return replicas.rank_info()


def set_pheno(ctx, y):
    if isinstance(y, tuple):
        ctx.set_phenotypes(y[0], y[1])
    else:
        ctx.set_phenotypes(y)


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during a region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.stop = threading.Event()

    def _run(self):
        while not self.stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True,
                                     timeout=5).stdout.strip()
                if out:
                    self.rows.append([x.strip() for x in out.split(",")])
            except Exception:
                pass
            self.stop.wait(0.2)

    def __enter__(self):
        self.t = threading.Thread(target=self._run, daemon=True)
        self.t.start()
        return self

    def __exit__(self, *a):
        self.stop.set()
        self.t.join(timeout=10)

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in self.rows for k in range(4)
                          if len(r) > 5 + k and r[5 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.rows)}


def peak_hbm():
    try:
        with open(PEAKS) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM, "fallback"


def peak_bf16_sustained():
    """Dense bf16 TFLOP/s sustained over seconds (the scan runs inside a long step)."""
    try:
        with open(PEAKS) as f:
            return float(json.load(f)["bf16_tflops_sustained"]), "measured (sustained)"
    except Exception:
        return FALLBACK_BF16_SUSTAINED, "fallback (sustained)"


def scan_traffic_per_launch(workload):
    """DRAM bytes per scan launch from the committed ncu summary, if present."""
    path = os.path.join(ROOT, "profiles", "scan_%s_ncu.md" % workload)
    try:
        for line in open(path):
            if line.startswith("traffic_bytes_per_launch:"):
                return float(line.split(":")[1])
    except OSError:
        pass
    return None


# iterations of each chain in the CPU leg: the scan workload's FP64 scan of
# 500,000 SNPs takes seconds per iteration on a core, the move-bound
# workloads run >= 1,000 iterations including RB steps
CPU_ITERS = {"scan": 1, "batched": 1000, "plain": 3000}


def cpu_sample(wl, workload, packed, y, threads, seed0):
    """The oracle on the host cores: `threads` chains (one pthread each) of
    the same workload for CPU_ITERS[workload] iterations; returns
    (chain-iterations/s, seconds, iterations)."""
    import oracle.port as op
    iters = CPU_ITERS.get(workload, 1)
    o = options(wl, seed0, iters, chains=threads)
    o.max_model_size = 1024
    port = op.Port(o, packed, y)
    t0 = time.perf_counter()
    port.run(iters, threads=threads)
    dt = time.perf_counter() - t0
    return threads * iters / dt, dt, iters


def ess_leg_gpu(bg, wl, workload, packed, y, seed, scan_impl):
    """Inclusion-indicator ESS of the sampling phase after a burn-in, outside
    the timed value: ESS_LEG[workload] = (burn-in, sampled iterations), ESS
    (Geyer) over SNPs with 0.05 < PIP < 0.95 per chain, per second of device
    time of the sampled iterations."""
    import torch
    from bmagwa_gb300 import ess
    burn, samp = ESS_LEG[workload]
    o = options(wl, seed + 29, burn + samp)
    o.scan_impl = scan_impl
    o.n_rao_burnin = max(1, burn // wl["n_rao"])
    ctx = bg.Context(o)
    ctx.load_bed(packed)
    set_pheno(ctx, y)
    ctx.set_covariates(None)
    ctx.precompute()
    ctx.run(burn, collect=False)
    torch.cuda.synchronize()
    ctx.reset_timings()
    col = ctx.run(samp, collect=True)
    sec = ctx.timings()[3] / 1000.0
    tr = [col.chain(c) for c in range(wl["chains"])]
    ctx.close()
    out = ess.summarize([(t["modelsize"], t["loci"]) for t in tr], sec)
    out.update(burnin_iters=burn, sample_iters=samp, samples_per_chain=int(len(tr[0]["modelsize"])),
               seconds=sec, chains=wl["chains"])
    return out


def ess_leg_cpu(wl, workload, packed, y, seed, threads):
    """The same ESS leg on the oracle: min(chains, threads) chains, one
    pthread each, seconds = wall time of the sampled iterations."""
    import oracle.port as op
    from bmagwa_gb300 import ess
    burn, samp = ESS_LEG[workload]
    chains = max(1, min(wl["chains"], threads))
    o = options(wl, seed + 29, burn + samp, chains=chains)
    o.n_rao_burnin = max(1, burn // wl["n_rao"])
    o.max_model_size = 1024
    port = op.Port(o, packed, y)
    port.run(burn, threads=chains)
    t0 = time.perf_counter()
    col = port.run(samp, threads=chains)
    sec = time.perf_counter() - t0
    tr = [col.chain(c) for c in range(chains)]
    out = ess.summarize([(t["modelsize"], t["loci"]) for t in tr], sec)
    out.update(burnin_iters=burn, sample_iters=samp, samples_per_chain=int(len(tr[0]["modelsize"])),
               seconds=sec, chains=chains, cores=chains)
    return out


def run_gb300(args, wl):
    import torch
    import bmagwa_gb300 as bg
    rank, world, local = env_rank()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    bg.build()
    seed = 1 + 7919 * rank
    packed, y = make_data(wl, seed, "cuda")
    iters_total = args.warmup + args.steps
    o = options(wl, seed, iters_total)
    o.scan_impl = args.scan
    ctx = bg.Context(o)
    ctx.load_bed(packed)
    set_pheno(ctx, y)
    ctx.set_covariates(None)
    ctx.precompute()
    ctx.run(args.warmup, collect=False)
    # the scan's launch-shape tuner times its candidates on the first scans;
    # finish it before the timed region
    extra = 0
    while ctx.scan_shape()[0] < 0 and extra < 40:
        ctx.run(1, collect=False)
        extra += 1
    torch.cuda.synchronize()
    ctx.reset_timings()
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    clocks = Clocks(local)
    with clocks:
        t0 = time.perf_counter()
        ctx.run(args.steps, collect=False)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
    ms = ctx.timings()
    launches = ctx.launch_count()
    scan_shape = ctx.scan_shape()[1]
    scan_tuning = ctx.scan_tuning()
    n_scans = ctx.reset_timings()
    dev_s = ms[3] / 1000.0
    from bmagwa_gb300 import replicas
    if world > 1:
        dev_s = replicas.max_over_ranks(dev_s, device="cuda")
        dist.barrier()
    value = replicas.job_throughput(dev_s, args.steps, wl["chains"], world)
    # e2e: the whole job through the C ABI from host buffers
    ctx.close()
    e2e = None
    if args.e2e:
        o2 = options(wl, seed + 17, iters_total)
        o2.scan_impl = args.scan
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        marks = []
        ctx2 = bg.Context(o2)
        marks.append(("create", time.perf_counter()))
        ctx2.load_bed(packed)
        marks.append(("load_bed", time.perf_counter()))
        ctx2.set_phenotypes(y)
        ctx2.set_covariates(None)
        marks.append(("phenotypes", time.perf_counter()))
        ctx2.precompute()
        marks.append(("precompute", time.perf_counter()))
        col = ctx2.run(args.steps, collect=True)
        marks.append(("run", time.perf_counter()))
        rao = [ctx2.rao_all()[0]]
        torch.cuda.synchronize()
        e2e_s = time.perf_counter() - t0
        marks.append(("read_back", t0 + e2e_s))
        breakdown, prev = {}, t0
        for name, t in marks:
            breakdown[name] = round(t - prev, 4)
            prev = t
        d2h = sum(int(sum(a.nbytes for a in col.chain(c).values())) for c in range(wl["chains"]))
        d2h += sum(r.nbytes for r in rao)
        h2d = packed.nbytes + y.nbytes
        ctx2.close()
        e2e = {"value": args.steps * wl["chains"] * world / e2e_s, "unit": "iter/s",
               "h2d_bytes_per_step": h2d / args.steps, "d2h_bytes_per_step": d2h / args.steps,
               "seconds": breakdown}
    # roofline of the scan kernel
    p, n, C = wl["p"], wl["n"], wl["chains"]
    scan_ms = ms[1] / max(1, n_scans)
    # packed genotypes + per (SNP, chain) the p_r write and one running mean
    # read and written (p_proposal during burn-in, p_rao after) + the residual
    # limbs (L bf16 digits per individual and chain)
    L = int(o.scan_limbs) if o.scan_limbs else 6
    alg_bytes = p * ((n + 3) // 4) + p * C * (8 + 16) + C * n * 2 * L
    peak_h, peak_h_kind = peak_hbm()
    hbm_gbs = alg_bytes / (scan_ms / 1000.0) / 1e9 if scan_ms > 0 else None
    # the scan is an exact-integer GEMM on the tensor cores: 2 n_pad (p terms)
    # (C L) bf16 flops per launch (n_pad = individuals rounded up to 128)
    n_pad = ((n + 127) // 128) * 128
    flops = 2.0 * n_pad * p * scan_terms(wl["types"]) * C * L
    peak, peak_kind = peak_bf16_sustained()
    achieved = flops / (scan_ms / 1000.0) / 1e12 if scan_ms > 0 else None
    out = {
        "metric": "MCMC chain-iterations/s (RB scan of all SNPs every iteration)",
        "value": value,
        "unit": "iter/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": 1000.0 * dev_s / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64 (moves) / bf16-limb exact int (scan)" if args.scan == 0 else "f64 / int64",
        "data": "synthetic (seeded LD-block genotypes and phenotypes)",
        "config": {"workload": args.workload, "n": n, "p": p, "chains": C, "n_rao": wl["n_rao"],
                   "types": wl["types"], "max_move_size": wl.get("max_move_size", 20),
                   "parallelism": "replicas" if world > 1 else "single",
                   "l2": "inputs larger than L2 (%.2f GB packed genotypes)" % (packed.nbytes / 1e9),
                   "scan_impl": "tcgen05" if args.scan == 0 else "simt",
                   "scan_shape": scan_shape, "scan_tuning_ms": scan_tuning},
        "e2e": e2e,
        "gpu_launches": launches,
        "phase_ms": {"move": ms[0], "scan": ms[1], "rebuild": ms[2], "total": ms[3],
                     "scans": n_scans, "wall_s": dt},
        "roofline": {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": (achieved / peak) if achieved else None,
                     "traffic": scan_traffic_per_launch(args.workload),
                     "kernel": "scan", "peak_kind": peak_kind, "scan_ms": scan_ms,
                     "alg_flops_per_launch": flops, "alg_bytes_per_launch": alg_bytes,
                     "hbm": {"achieved": hbm_gbs, "peak": peak_h, "unit": "GB/s",
                             "frac": (hbm_gbs / peak_h) if hbm_gbs else None, "peak_kind": peak_h_kind}},
        "clocks": clocks.summary(),
    }
    if rank == 0 and args.ess and args.workload in ESS_LEG:
        out["inclusion_ess"] = ess_leg_gpu(bg, wl, args.workload, packed, y, seed, args.scan)
    if rank == 0 and args.cpu_baseline:
        threads = max(1, min(C, os.cpu_count() or 1))
        cv, cdt, citers = cpu_sample(wl, args.workload, packed, y, threads, seed)
        out["cpu_baseline"] = {"value": cv, "unit": "iter/s", "cores": threads, "kind": "port",
                               "sample": "%d chains x %d iterations of the same workload (%.1f s)"
                                         % (threads, citers, cdt)}
        if args.ess and args.workload in ("plain", "batched"):
            out["cpu_baseline"]["inclusion_ess"] = ess_leg_cpu(wl, args.workload, packed, y, seed, threads)
    if rank == 0:
        print(json.dumps(out))
    if world > 1:
        dist.destroy_process_group()


def run_learned_compare(args, wl):
    """Inclusion-indicator ESS per second of the sampling phase (after the
    same burn-in) with the plain adaptive add proposal and with the learned
    mixture; one JSON line with both."""
    import torch
    import bmagwa_gb300 as bg
    from bmagwa_gb300 import ess
    torch.cuda.set_device(0)
    bg.build()
    seed = 11
    packed, y = make_data(wl, seed, "cuda")
    burn, samp = wl["burnin"], wl["sample"]
    out = {}
    for name, mode in (("plain", 0), ("learned", 1)):
        o = options(wl, seed, burn + samp)
        o.n_rao_burnin = burn // wl["n_rao"]
        o.proposal = mode
        ctx = bg.Context(o)
        ctx.load_bed(packed)
        ctx.set_phenotypes(y)
        ctx.set_covariates(None)
        ctx.precompute()
        ctx.run(burn, collect=False)
        torch.cuda.synchronize()
        ctx.reset_timings()
        col = ctx.run(samp, collect=True)
        sec = ctx.timings()[3] / 1000.0
        chains = [col.chain(c) for c in range(wl["chains"])]
        e = ess.summarize([(t["modelsize"], t["loci"]) for t in chains], sec)
        acc = [ctx.state(c)[0].n_accepted / max(1, ctx.state(c)[0].n_iter) for c in range(wl["chains"])]
        mt = np.concatenate([np.asarray(t["move_type"]) for t in chains])
        jd = np.concatenate([np.asarray(t["jumpdistance"]) for t in chains])
        moves = {kind: [int(np.sum(mt == m)), int(np.sum((mt == m) & (jd > 0)))]
                 for m, kind in enumerate(("addrem", "swap", "statechange", "typeswitch"))}
        out[name] = dict(e, moves_proposed_accepted=moves, iter_per_s=samp * wl["chains"] / sec, seconds=sec,
                         mean_model_size=float(np.mean([len(t["loci"]) / max(1, len(t["modelsize"])) for t in chains])),
                         acceptance=float(np.mean(acc)))
        ctx.close()
    ratio = (out["learned"]["per_s"] / out["plain"]["per_s"]) if out["plain"]["per_s"] else None
    print(json.dumps({"metric": "inclusion-indicator ESS/s, learned vs plain adaptive add proposal",
                      "value": ratio, "unit": "ratio", "n_gpus": 1, "higher_is_better": True,
                      "data": "synthetic (seeded LD-block genotypes, 50 causal SNPs, 10 in dominance coding)",
                      "config": {"workload": "learned", "n": wl["n"], "p": wl["p"], "chains": wl["chains"],
                                 "types": wl["types"], "n_rao": wl["n_rao"], "burnin_iters": burn,
                                 "sample_iters": samp},
                      "plain": out["plain"], "learned": out["learned"]}))


def run_reference(args, wl):
    """The reference's CPU path (the oracle port, bit-identical to the
    compiled reference) on the host cores: one pthread per chain, as many
    chains as cores (at most the workload's), the same workload and options.
    Only oracle/ libraries are loaded here; the options come from the
    library-free mirror of the defaults."""
    rank, world, _ = env_rank()
    if rank != 0:
        return
    import oracle.port as op
    op.build()
    seed = 1
    packed, y = make_data(wl, seed, "cpu")
    threads = max(1, min(wl["chains"], os.cpu_count() or 1))
    per_step = CPU_ITERS.get(args.workload, 1)
    o = options(wl, seed, (args.warmup + args.steps) * per_step, chains=threads)
    o.max_model_size = 1024
    port = op.Port(o, packed, y)
    if args.warmup:
        port.run(per_step if per_step > 1 else 1, threads=threads)
    # each step is per_step iterations of `threads` chains; stop after about a minute
    done, dt = 0, 0.0
    while done < args.steps and (done == 0 or dt < 60.0):
        t0 = time.perf_counter()
        port.run(per_step, threads=threads)
        dt += time.perf_counter() - t0
        done += 1
    args.steps = done
    v = done * per_step * threads / dt
    print(json.dumps({
        "impl": "reference",
        "metric": "MCMC chain-iterations/s (RB scan of all SNPs every iteration)",
        "value": v, "unit": "iter/s", "n_gpus": 0, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * dt / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded LD-block genotypes and phenotypes)",
        "config": {"workload": args.workload, "n": wl["n"], "p": wl["p"], "chains": threads,
                   "n_rao": wl["n_rao"], "types": wl["types"]},
        "cpu_baseline": {"value": v, "unit": "iter/s", "cores": threads, "kind": "port",
                         "sample": "%d chains x %d iterations (one pthread per chain)"
                                   % (threads, args.steps * per_step)},
        "e2e": {"value": v, "unit": "iter/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="scan", choices=sorted(WORKLOADS))
    ap.add_argument("--scan", type=int, default=0, help="0 tcgen05, 1 SIMT")
    ap.add_argument("--no-cpu-baseline", dest="cpu_baseline", action="store_false")
    ap.add_argument("--p", type=int, default=None, help="override the SNP count (profiling)")
    ap.add_argument("--n", type=int, default=None, help="override the individuals (profiling)")
    ap.add_argument("--chains", type=int, default=None, help="override the chains (profiling)")
    ap.add_argument("--max-move-size", type=int, default=None,
                    help="override the largest multi-SNP move (profiling)")
    ap.add_argument("--no-e2e", dest="e2e", action="store_false")
    ap.add_argument("--no-ess", dest="ess", action="store_false",
                    help="skip the inclusion-ESS leg (burn-in + sampled iterations after the timed region)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    wl = dict(WORKLOADS[args.workload])
    for key in ("p", "n", "chains", "max_move_size"):
        if getattr(args, key):
            wl[key] = getattr(args, key)
    if "keep" in wl:
        # the reference has no missingness masks: its counterpart is one run
        # per phenotype on a subset .bed, which this bench does not time; the
        # end-to-end leg re-runs the single-phenotype path only
        args.e2e = False
        args.cpu_baseline = False
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the reference has no per-phenotype masks; "
                              "its counterpart is one process per phenotype on a subset .bed"}))
            return
    if args.impl == "reference":
        run_reference(args, wl)
    elif args.workload == "learned":
        run_learned_compare(args, wl)
    else:
        run_gb300(args, wl)


if __name__ == "__main__":
    main()
