"""Benchmark: SCF seconds per molecule and ERI quartets/s on one GB300.

Workload: (H2O)16 RHF/6-31G (208 basis functions, seeded geometry, EMSL
basis), mixed FP32/FP64 direct SCF (FP32 for quartets with Schwarz bound
below 1e-4, Schwarz cutoff 1e-12, incremental dD Fock builds, superposition-
of-atomic-densities guess, DIIS with 6 vectors, converged to dE < 1e-10 and
RMS dD < 1e-8).  One step
is one complete SCF of the molecule, including the screening setup, with the
basis already on the device; the plain FP64 GPU SCF is run once beside it and
both energies are reported.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gbhf|reference]

--impl reference times the CPU implementation (the FP64 oracle, a
restatement of the reference's numerics; the Haskell original cannot be
built here) on the same workload.  For N > 1 (torchrun), each rank runs its
own replica of the molecule (independent molecules, no data exchange) and
rank 0 prints the whole-job number.
"""
import argparse
import datetime
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "haskell-abinitio_gb300"))
sys.path.insert(0, str(ROOT / "oracle"))

METRIC = "SCF s/molecule & ERI quartets/s: mixed vs FP64 on one GB300 at |ΔE|≤1e-6 Eh"
WORKLOAD = "(H2O)16 RHF/6-31G, 208 basis functions, seeded water cluster (seed 0)"


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo", rank=rank, world_size=world)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(world, v):
    if world == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(v)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clocks/throttle reasons every 200 ms.  The sampler starts
    before the work it watches (its start-up queries the driver for about a
    tenth of a second, which stalled a timed SCF step when it fell inside the
    timed region); begin()/end() mark the timed region, and the summary keeps
    the samples stamped inside it (widened by one sampling period, so that a
    short region keeps its neighbouring samples)."""

    FIELDS = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    PERIOD_S = 0.2

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.t0 = self.t1 = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", str(int(1000 * self.PERIOD_S))],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def begin(self):
        self.t0 = datetime.datetime.now()

    def end(self):
        self.t1 = datetime.datetime.now()

    def __exit__(self, *a):
        self.lines = []
        if self.proc:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [l for l in out.splitlines() if l.strip()]

    def _in_region(self, stamp):
        if self.t0 is None:
            return True
        try:
            ts = datetime.datetime.strptime(stamp, "%Y/%m/%d %H:%M:%S.%f")
        except ValueError:
            return True
        pad = datetime.timedelta(seconds=self.PERIOD_S)
        t1 = self.t1 if self.t1 is not None else datetime.datetime.now()
        return self.t0 - pad <= ts <= t1 + pad

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for l in getattr(self, "lines", []):
            p = [x.strip() for x in l.split(",")]
            if len(p) < 10 or not self._in_region(p[0]):
                continue
            try:
                sm.append(float(p[2]))
                mx.append(float(p[3]))
            except ValueError:
                continue
            for nm, v in zip(names, p[6:10]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["clock sampling unavailable"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def load_measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    return json.loads(p.read_text()) if p.exists() else {}


def traffic_profile():
    p = ROOT / "profiles" / "traffic.json"
    return json.loads(p.read_text()) if p.exists() else {}


class OracleSCFSteps:
    """Complete FP64 oracle SCFs of one molecule, one SCF iteration per step.

    A step is one SCF iteration (direct Fock build, DIIS error and
    extrapolation, diagonalisation); the setup of an SCF (integrals,
    orthogonaliser, SAD start) is timed inside the first step of that SCF.
    When an SCF converges the next step starts a new one, so ``complete``
    collects the wall time of every SCF that ran from setup to convergence."""

    def __init__(self, fb):
        import oracle as O
        self.O, self.fb = O, fb
        self.gen, self.t_scf, self.iters = None, 0.0, 0
        self.complete = []          # (seconds, iterations, energy) of finished SCFs
        self.iteration_s = []       # step times without a setup

    def step(self):
        t0 = time.perf_counter()
        setup = self.gen is None
        if setup:
            self.gen = self.O.scf_steps(self.fb, self.O.SCFOptions.baseline(guess="sad"))
            next(self.gen)          # setup
        _, res = next(self.gen)
        dt = time.perf_counter() - t0
        self.t_scf += dt
        self.iters += 1
        if not setup:
            self.iteration_s.append(dt)
        if res is not None:
            self.complete.append((self.t_scf, self.iters, res.energy))
            self.gen, self.t_scf, self.iters = None, 0.0, 0
        return dt


def run_reference(args, world, rank):
    """The reference arm: the FP64 oracle (a restatement of the reference's
    numerics; the Haskell original cannot be built here) running complete SCFs
    of the workload on all host threads.  value = the mean wall time of the
    SCFs that ran from setup to convergence inside the timed steps; with fewer
    timed steps than one SCF needs, the setup plus the measured mean iteration
    times the oracle's own iteration count (and the line says so)."""
    if rank != 0:
        return
    import oracle as O
    from gbhf import basis as B, molecules as M
    fb = B.flatten(M.cluster_atoms("w16", "6-31g"))
    rec = json.loads((ROOT / "tests" / "golden" / "clusters.json").read_text()).get("w16_631g", {})
    n_iter = int(rec.get("iterations_sad", rec.get("iterations", 17)))
    warm = OracleSCFSteps(fb)
    for _ in range(args.warmup):
        warm.step()
    run = OracleSCFSteps(fb)
    t0 = time.perf_counter()
    times = [run.step() for _ in range(args.steps)]
    wall = time.perf_counter() - t0
    if run.complete:
        v = statistics.mean(c[0] for c in run.complete)
        how = (f"{len(run.complete)} complete SCF(s) ({run.complete[0][1]} iterations, E = {run.complete[0][2]:.10f}) "
               f"timed from setup to convergence within the {args.steps} timed steps")
    else:
        setup_s = times[0] - (statistics.mean(run.iteration_s) if run.iteration_s else 0.0)
        v = setup_s + n_iter * statistics.mean(run.iteration_s or times)
        how = (f"no SCF completed within {args.steps} steps: setup + {n_iter} x the mean measured iteration "
               f"({n_iter} = the oracle's own iteration count for this molecule)")
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "s/molecule", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * wall / args.steps,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": {"workload": WORKLOAD, "precision": "FP64 (CPU)",
                                            "parallelism": "OpenMP, all host threads"},
            "complete_scfs": [{"seconds": c[0], "iterations": c[1], "energy": c[2]} for c in run.complete],
            "iteration_s_mean": statistics.mean(run.iteration_s) if run.iteration_s else None,
            "cpu_baseline": {"value": v, "unit": "s/molecule", "cores": O.lib().orc_num_threads(),
                             "kind": "port",
                             "sample": "per step one iteration of a complete FP64 oracle SCF (direct Fock build "
                                       "with Schwarz and density screening, DIIS, diagonalisation; SAD start, "
                                       "dE < 1e-10, RMS dD < 1e-8), setup inside each SCF's first step; " + how},
            "e2e": {"value": v, "unit": "s/molecule", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def autotune_jk(ctx, fb, args):
    """With --autotune: tune the J/K task budgets on the workload's basis (SAD
    density, mixed precision) before the warm-up; returns a summary for the
    JSON line.  Off by default for this workload: the tuner times one full build
    on the start density, and budgets that win there (once (pp|pp) at 2
    primitive quartets per lane) slowed the incremental builds that follow
    (Fock phase 31.4 -> 36.3 ms per SCF on one box)."""
    from gbhf import _lib
    if not args.autotune:
        return {"enabled": False, "why": "default budgets: tuning on the first build's density can slow the "
                                         "incremental builds of the SCF"}
    ctx.set_basis(fb)
    t0 = time.perf_counter()
    ms0, ms1 = ctx.autotune(0, _lib.PREC_MIXED, 1e-12, 1e-4)
    dt = time.perf_counter() - t0
    tab = ctx.task_budgets(0)
    changed = {name: [int(x) for x in tab[k]] for k, name in enumerate(ctx.CLASSES) if ms1[k] < ms0[k]}
    return {"enabled": True, "tuning_s": dt, "jk_ms_default": float(ms0.sum()), "jk_ms_tuned": float(ms1.sum()),
            "changed_budgets": changed}


def run_gbhf(args, world, rank, local):
    import numpy as np
    from gbhf import _lib, basis as B, molecules as M
    from gbhf.flops_model import F_KERNEL
    ctx = _lib.Context(local)
    fb = B.flatten(M.cluster_atoms("w16", "6-31g"))
    # incremental builds without periodic full rebuilds (|dE| vs FP64 stays ~5e-10 Eh)
    mixed = _lib.baseline_opts(precision=_lib.PREC_MIXED, incremental=1, final_fp64=0, full_rebuild_every=0)
    fp64 = _lib.baseline_opts(precision=_lib.PREC_FP64, incremental=0, final_fp64=0)

    def step(opts, matrices=False):
        ctx.set_basis(fb)
        ctx.event_record(0)
        r = ctx.scf(opts, want_matrices=matrices)
        ctx.event_record(1)
        return r, ctx.event_elapsed(0, 1)

    tune = autotune_jk(ctx, fb, args)
    times = []
    with ClockSampler(local) as clk:   # started before the warm-up (see ClockSampler)
        for _ in range(max(args.warmup, 3)):
            step(mixed)
        # plain FP64 GPU SCF, once (reported beside the headline)
        r64, t64 = step(fp64)
        barrier(world)
        ctx.profile_reset(events=False)
        barrier(world)
        clk.begin()
        for _ in range(args.steps):
            ctx.flush_l2()
            r, ms = step(mixed)
            times.append(ms)
        barrier(world)
        clk.end()
    prof = ctx.profile_read()
    # per-class kernel times: one more SCF with an event around every J/K
    # launch (the class launches then run one after another on one stream)
    ctx.profile_reset(events=True)
    ctx.flush_l2()
    r_prof, ms_prof = step(mixed)
    cls = ctx.profile_classes()
    prof_cls = ctx.profile_read()
    total_ms = max_over_ranks(world, sum(times))
    value = total_ms / 1e3 / (args.steps * world)
    # end to end: host basis in, every result matrix back to host memory (the
    # production path again: class launches concurrent, no per-launch events)
    ctx.profile_reset(events=False)
    e2e_t = []
    h2d = sum(a.nbytes for a in (fb.xyz, fb.charge, fb.cgf_atom, fb.cgf_lxyz, fb.cgf_nprim, fb.prim_coef,
                                 fb.prim_exp))
    n = fb.n_cgf
    d2h = 8 * (2 * n * (n + 1) // 2 + n * n + n) + 8
    for _ in range(args.steps):
        t0 = time.perf_counter()
        ctx.set_basis(fb)
        ctx.scf(mixed, want_matrices=True)
        e2e_t.append(time.perf_counter() - t0)
    e2e_v = max_over_ranks(world, sum(e2e_t)) / (args.steps * world)
    # the same call on a new context each time (gbhf_create, basis, SCF with every
    # matrix back, gbhf_destroy): what a caller that keeps no context pays
    cold_t = []
    for _ in range(3):
        t0 = time.perf_counter()
        with _lib.Context(local) as c2:
            c2.set_basis(fb)
            c2.scf(mixed, want_matrices=True)
        cold_t.append(time.perf_counter() - t0)
    cold_v = max_over_ranks(world, statistics.median(cold_t))
    batch = None
    if not args.no_batch:
        batch = [batch_measure(args, world, rank, local, cut, gcut) for cut, gcut in ((1e-2, 1.0), (1e-4, 1e-4))]
    peaks_clk = measure_fma_peaks(ctx, local)
    if rank != 0:
        return
    # roofline of the dominant J/K kernel class (profiling SCF)
    dom = max(cls.items(), key=lambda kv: kv[1]["ms"])
    (cname, prec), st = dom
    flops = st["prim_quartets"] * F_KERNEL[cname]
    achieved = flops / (st["ms"] * 1e-3) / 1e12 if st["ms"] > 0 else 0.0
    peak64, peak32 = peaks_clk["fp64_tflops"], peaks_clk["fp32_tflops"]
    peak = peak64 if prec == "fp64" else peak32
    cls_tab = {}
    for (cn, pr), v in cls.items():
        if v["ms"] <= 0:
            continue
        a = v["prim_quartets"] * F_KERNEL[cn] / (v["ms"] * 1e-3) / 1e12
        cls_tab[f"{cn}_{pr}"] = {**v, "flops_per_prim_quartet": F_KERNEL[cn], "achieved_tflops": a,
                                 "frac": a / (peak64 if pr == "fp64" else peak32)}
    prof_tr = traffic_profile().get(f"{cname}_{prec}", {}).get("dram_bytes_per_launch")
    jk_ms = prof_cls["jk_ms_fp64"] + prof_cls["jk_ms_fp32"]
    fnq_step = prof["fn_quartets"] / args.steps
    line = {
        "metric": METRIC, "value": value, "unit": "s/molecule", "n_gpus": world, "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": total_ms / args.steps, "step_ms": [round(t, 3) for t in times],
        "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
        "data": "synthetic (seeded water cluster, EMSL 6-31G)",
        "config": {"workload": WORKLOAD, "n_basis": n, "precision": "mixed: FP32 ERIs below Schwarz bound 1e-4, "
                   "FP64 Fock accumulation, DIIS and eigen-solve", "schwarz_cutoff": 1e-12,
                   "incremental_fock": True, "full_rebuild_every": 0, "guess": "SAD",
                   "l2": "flushed (256 MiB write) before every timed step",
                   "parallelism": f"{world} independent replica(s), one per GPU"},
        "energy": r["energy"], "iterations": r["iterations"],
        "fp64": {"s_per_molecule": t64 / 1e3, "energy": r64["energy"], "iterations": r64["iterations"],
                 "delta_e_mixed_vs_fp64": r["energy"] - r64["energy"],
                 "speedup_mixed_vs_fp64": (t64 / 1e3) / value if value > 0 else None},
        "eri_quartets_per_s": fnq_step / (total_ms / args.steps / 1e3),
        "eri_quartets_per_step": fnq_step,
        "eri_quartets_unscreened": (n * (n + 1) // 2) ** 2,
        "eri_fp32_fraction": r["eri_fp32_fraction"],
        "jk_ms_serialized_profiling_scf": jk_ms, "profiling_scf_ms": ms_prof,
        "phases_ms_per_step": {k: prof[k] / args.steps for k in ("ms_setup", "ms_fock", "ms_diis", "ms_diag",
                                                                  "ms_other")},
        "jacobi_sweeps_per_call": prof["jacobi_sweeps"] / max(prof["jacobi_calls"], 1),
        "gpu_launches": int(prof["launches"]),
        "autotune": tune,
        "roofline": {"kernel": f"k_jk<{cname}, {prec}>", "bound": f"{prec} CUDA-core pipe", "achieved": achieved,
                     "timing": "CUDA events around each launch of this class in one profiling SCF run after "
                               "the timed steps (class launches serialised on one stream)",
                     "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak if peak else None,
                     "peak_source": f"FMA microbenchmark on this GPU (FP64 {peak64:.2f}, FP32 {peak32:.1f} TFLOP/s, "
                                    f"SM clock median {peaks_clk['sm_mhz']} MHz while it ran); "
                                    "MEASURED_PEAKS.json holds only HBM and bf16 tensor peaks",
                     "flop_model": "primitive quartets x F_KERNEL (gbhf/flops_model.py): F_alg, or for the "
                                   "deferred-ket classes the work per primitive quartet of that form",
                     "flops_per_launch": flops / max(r_prof["iterations"], 1), "traffic": prof_tr,
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of this class's launch "
                                       "in a full mixed Fock build (profiles/traffic.json); the ERI kernels "
                                       "are compute-bound, traffic far below their roofline"},
        "classes": cls_tab,
        "fma_peaks": peaks_clk,
        "clocks": clk.summary(),
        "e2e": {"value": e2e_v, "unit": "s/molecule", "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                "context": "one context kept across calls (Boys tables, SAD atoms, tuned budgets resident)"},
        "e2e_cold_context": {"value": cold_v, "unit": "s/molecule", "calls": len(cold_t),
                             "what": "median of gbhf_create + gbhf_set_basis + gbhf_scf (all matrices back) + "
                                     "gbhf_destroy, a new context per call (default task budgets); the host Boys "
                                     "tables and the SAD atom densities are computed once per process and shared "
                                     "by its contexts (the first context of a process pays for them)"},
    }
    if batch:
        line["batch256"] = batch
    tr_all = traffic_profile()
    red = sum(v.get("l2_red_sectors_per_launch", 0.0) for v in tr_all.values()) * 32
    line["fock_scatter"] = {"algorithmic_bytes_per_build": 24 * n * n,
                            "l2_reduction_bytes_per_full_build": red or None, "dram_write_bytes_per_full_build": 0,
                            "source": "ncu lts__t_sectors_srcunit_tex_op_red.sum x 32 B over the twelve class launches "
                                      "of one full mixed build (profiles/traffic.json, profiles/k_jk_w16_fock_full.md): "
                                      "every quartet adds its J/K terms with FP64 reductions in L2; none reach DRAM"}
    peaks = load_measured_peaks()
    if peaks:
        line["measured_peaks"] = {"hbm_gbs": peaks.get("hbm_gbs"), "bf16_tflops": peaks.get("bf16_tflops")}
    if world == 1 and not args.no_cpu_baseline:
        # one complete FP64 oracle SCF of the same molecule on all host threads
        import oracle as O
        steps = OracleSCFSteps(fb)
        while not steps.complete:
            steps.step()
        secs, iters, e_cpu = steps.complete[0]
        line["cpu_baseline"] = {"value": secs, "unit": "s/molecule", "cores": O.lib().orc_num_threads(), "kind": "port",
                                "sample": f"one complete FP64 oracle SCF of the workload ({iters} iterations, "
                                          f"E = {e_cpu:.10f}): setup, SAD start, direct Fock builds with Schwarz "
                                          "and density screening, DIIS, diagonalisations"}
    print(json.dumps(line), flush=True)


def measure_fma_peaks(ctx, local, seconds=1.0):
    """FP64 and FP32 FMA microbenchmark peaks (best of repeated runs over about
    a second each) with the SM clock sampled while they ran."""
    from gbhf import _lib
    out = {}
    with ClockSampler(local) as clk:
        for key, prec in (("fp64_tflops", _lib.PREC_FP64), ("fp32_tflops", _lib.PREC_MIXED)):
            best, t0 = 0.0, time.perf_counter()
            while time.perf_counter() - t0 < seconds:
                best = max(best, ctx.peak_flops(prec))
            out[key] = best
    out.update({"sm_mhz": clk.summary()["sm_mhz"], "clock_reasons": clk.summary()["reasons"]})
    return out


def batch_measure(args, world, rank, local, mixed_cutoff, grad_cutoff, quick=False):
    """256 seeded conformers (H2O)_n, n in [1, 12], STO-3G (even) / 6-31G (odd):
    mixed-precision SCF + analytic gradient for every molecule in one batched
    call, versus one-at-a-time plain FP64 SCF + gradient (timed on every 8th
    molecule and scaled).  Returns the record (rank 0) or None."""
    import numpy as np
    from gbhf import _lib, basis as B, molecules as M, replicas
    mols = M.batch_workload()
    flats = [B.flatten(a) for a in mols]
    mine = replicas.shard([f.n_cgf ** 4 for f in flats], world, rank)
    sub = [flats[i] for i in mine]
    mixed = _lib.baseline_opts(precision=_lib.PREC_MIXED, incremental=1, final_fp64=0, full_rebuild_every=0,
                               mixed_cutoff=mixed_cutoff, grad_mixed_cutoff=grad_cutoff)
    ctx = _lib.Context(local)                                 # its own context: budgets tuned for the batch
    ctx.scf_batch(sub[:16], mixed, gradients=True)          # warm-up (tables, SAD atoms)
    tune = {"enabled": not args.no_autotune}
    if not args.no_autotune:
        # tune the J/K and gradient budgets on the whole batch once (untimed)
        mixed.autotune = 1
        t0 = time.perf_counter()
        ctx.scf_batch(sub, mixed, gradients=True)
        tune["tuning_run_s"] = time.perf_counter() - t0
        mixed.autotune = 0
    barrier(world)
    ctx.profile_reset(events=False)
    t0 = time.perf_counter()
    e, it, cv, g = ctx.scf_batch(sub, mixed, gradients=True)
    wall = time.perf_counter() - t0
    prof = ctx.profile_read()
    wall = max_over_ranks(world, wall)
    fp64 = _lib.baseline_opts()
    sample = list(range(0, len(sub), 8)) if not quick else []
    t_single, de, dg = 0.0, [], []
    for k in sample:
        t1 = time.perf_counter()
        ctx.set_basis(sub[k])
        r = ctx.scf(fp64, want_matrices=False)
        g64 = ctx.gradient()
        t_single += time.perf_counter() - t1
        de.append(abs(r["energy"] - e[k]))
        dg.append(float(np.max(np.abs(g64 - g[k]))))
    single_est = t_single * len(sub) / max(len(sample), 1)
    ctx.close()
    if rank != 0:
        return None
    n_total = len(flats)
    return {"workload": "batch256", "metric": "molecules/s (mixed SCF + analytic gradient, batched)",
            "value": n_total / wall, "unit": "molecules/s", "n_gpus": world, "wall_s": wall,
            "converged": int(cv.sum()) * world, "molecules": n_total,
            "fp64_one_at_a_time_molecules_per_s": len(sub) / single_est if single_est > 0 else None,
            "speedup_vs_fp64_one_at_a_time": single_est / wall * world if wall > 0 else None,
            "max_abs_delta_e_mixed_vs_fp64_sample": float(max(de)) if de else None,
            "max_abs_grad_mixed_vs_fp64_sample": float(max(dg)) if dg else None,
            "meets_1e-6_eh_and_1e-5_eh_per_bohr": bool(de and max(de) <= 1e-6 and max(dg) <= 1e-5),
            "mixed_cutoff": mixed_cutoff, "grad_mixed_cutoff": grad_cutoff,
            "sample": f"FP64 one-at-a-time SCF + gradient timed on {len(sample)} of {len(sub)} molecules "
                      "(every 8th) and scaled; dE and gradient errors on the same sample",
            "batch_steps": int(prof["batch_steps"]), "gpu_launches": int(prof["launches"]), "autotune": tune,
            "phases_ms": {k: prof[k] for k in ("ms_pairs", "ms_setup", "ms_fock", "ms_diis", "ms_diag", "ms_other",
                                               "ms_grad")},
            "jk_prim_quartets": prof["prim_quartets_fp64"] + prof["prim_quartets_fp32"],
            "data": "synthetic (256 seeded water conformers)", "dtype": "f32+f64", "higher_is_better": True}


def run_batch(args, world, rank, local):
    rec = batch_measure(args, world, rank, local, args.mixed_cutoff, args.grad_mixed_cutoff, quick=args.quick)
    if rec is not None:
        print(json.dumps(rec), flush=True)


def run_gradient(args, world, rank, local):
    """(H2O)8 RHF/6-31G analytic gradient: FP64 and mixed, checked against
    central finite differences (1e-4 bohr) of the GPU SCF energy on all 72
    Cartesian coordinates."""
    import numpy as np
    from gbhf import _lib, basis as B, molecules as M
    ctx = _lib.Context(local)
    xyz = M.cluster_coords("w8")
    labels = M.water_labels(len(xyz) // 3)
    tight = dict(conv_energy=1e-12, conv_density=1e-10, max_iter=200)

    def setup(p):
        ctx.set_basis(B.flatten(B.make_atoms(labels, p, "6-31g")))

    setup(xyz)
    ctx.scf(_lib.baseline_opts(**tight), want_matrices=False)
    ctx.event_record(0)
    r64 = ctx.scf(_lib.baseline_opts(**tight), want_matrices=False)
    g64 = ctx.gradient()
    ctx.event_record(1)
    t64 = ctx.event_elapsed(0, 1)
    ctx.event_record(2)
    rmx = ctx.scf(_lib.baseline_opts(precision=_lib.PREC_MIXED, incremental=1, **tight), want_matrices=False)
    gmx = ctx.gradient(precision=_lib.PREC_MIXED)
    ctx.event_record(3)
    tmx = ctx.event_elapsed(2, 3)
    n_coords = len(xyz) * 3 if not args.quick else 6
    fd_err = 0.0
    h = 1e-4
    for idx in range(n_coords):
        a, x = divmod(idx, 3)
        e = []
        for s in (1, -1):
            p = xyz.copy()
            p[a, x] += s * h
            setup(p)
            e.append(ctx.scf(_lib.baseline_opts(**tight), want_matrices=False)["energy"])
        fd = (e[0] - e[1]) / (2 * h)
        fd_err = max(fd_err, abs(fd - g64[a, x]))
    if rank != 0:
        return
    line = {"workload": "grad8", "metric": "analytic RHF/6-31G gradient of (H2O)8", "n_basis": 104,
            "fp64_scf_plus_gradient_s": t64 / 1e3, "mixed_scf_plus_gradient_s": tmx / 1e3,
            "max_abs_grad_fd_error": fd_err, "fd_coordinates": n_coords, "fd_step_bohr": h,
            "max_abs_grad_mixed_vs_fp64": float(np.max(np.abs(gmx - g64))),
            "translational_invariance": float(np.max(np.abs(g64.sum(axis=0)))),
            "energy_fp64": r64["energy"], "energy_mixed": rmx["energy"], "unit": "hartree/bohr"}
    print(json.dumps(line), flush=True)


def run_large(args, world, rank, local, cluster="w64", basis="6-31g"):
    """A cluster SCF with its gradient: mixed direct SCF with incremental builds,
    then the analytic gradient; the plain FP64 GPU SCF beside it.  w64:
    (H2O)64 RHF/6-31G (832 functions); w16d: (H2O)16 RHF/6-31G* (304 functions,
    the d-shell classes)."""
    from gbhf import _lib, basis as B, molecules as M
    ctx = _lib.Context(local)
    fb = B.flatten(M.cluster_atoms(cluster, basis))
    ctx.set_basis(fb)
    if args.workload == "w16d":   # first launches of the d-class kernels load their code
        ctx.scf(_lib.baseline_opts(precision=_lib.PREC_MIXED, incremental=1), want_matrices=False)
        ctx.gradient(precision=_lib.PREC_MIXED)
        ctx.set_basis(fb)
    ctx.profile_reset(events=True)
    ctx.event_record(0)
    rmx = ctx.scf(_lib.baseline_opts(precision=_lib.PREC_MIXED, incremental=1), want_matrices=False)
    ctx.event_record(1)
    tmx = ctx.event_elapsed(0, 1)
    prof = ctx.profile_read()
    cls = ctx.profile_classes()
    gmx = ctx.gradient(precision=_lib.PREC_MIXED)
    ctx.event_record(2)
    tg = ctx.event_elapsed(1, 2)
    g64 = ctx.gradient()
    ctx.event_record(5)
    tg64 = ctx.event_elapsed(2, 5)
    out = {"workload": args.workload, "basis": basis, "n_basis": fb.n_cgf, "mixed_scf_s": tmx / 1e3, "gradient_mixed_s": tg / 1e3,
           "gradient_fp64_s": tg64 / 1e3, "max_abs_grad_mixed_vs_fp64": float(abs(gmx - g64).max()),
           "energy_mixed": rmx["energy"], "iterations": rmx["iterations"],
           "eri_quartets_per_s": prof["fn_quartets"] / (tmx / 1e3),
           "jk_ms": prof["jk_ms_fp64"] + prof["jk_ms_fp32"], "phases_ms": {k: prof[k] for k in (
               "ms_setup", "ms_fock", "ms_diis", "ms_diag", "ms_other")},
           "eri_quartets_unscreened": (fb.n_cgf * (fb.n_cgf + 1) // 2) ** 2,
           "fp32_fraction": rmx["eri_fp32_fraction"],
           "classes": {f"{k[0]}_{k[1]}": v for k, v in cls.items() if v["ms"] > 0}}
    if not args.quick:
        ctx.set_basis(fb)
        ctx.event_record(3)
        r64 = ctx.scf(_lib.baseline_opts(), want_matrices=False)
        ctx.event_record(4)
        out["fp64_scf_s"] = ctx.event_elapsed(3, 4) / 1e3
        out["energy_fp64"] = r64["energy"]
        out["delta_e_mixed_vs_fp64"] = rmx["energy"] - r64["energy"]
    if rank == 0:
        print(json.dumps(out), flush=True)


def run_fock_case(args, world, rank, local):
    """Profiling case: one mixed-precision full direct Fock build of (H2O)16/6-31G
    for a seeded symmetric density (every J/K class launched once per precision)."""
    import numpy as np
    from gbhf import _lib, basis as B, molecules as M
    ctx = _lib.Context(local)
    fb = B.flatten(M.cluster_atoms("w16", "6-31g"))
    ctx.set_basis(fb)
    n = fb.n_cgf
    h = ctx.hcore(_lib.MODE_EXACT)
    d = np.random.default_rng(2).standard_normal((n, n)) * 0.05
    d = (d + d.T)[np.triu_indices(n)]
    f = ctx.fock(h, d, _lib.MODE_EXACT, _lib.PREC_MIXED, 1e-12, 1e-4)
    if rank == 0:
        print(json.dumps({"workload": "fock", "n_basis": n, "checksum": float(np.abs(f).sum())}), flush=True)


def run_scf_case(args, world, rank, local):
    """Profiling case: one mixed-precision SCF of (H2O)16/6-31G with the J/K
    class launches timed one by one; prints each class's counted quartets
    (to divide ncu counters of the class launches by)."""
    from gbhf import _lib, basis as B, molecules as M
    ctx = _lib.Context(local)
    fb = B.flatten(M.cluster_atoms("w16", "6-31g"))
    mixed = _lib.baseline_opts(precision=_lib.PREC_MIXED, incremental=1, final_fp64=0, full_rebuild_every=0)
    ctx.set_basis(fb)
    ctx.profile_reset(events=True)
    r = ctx.scf(mixed, want_matrices=False)
    cls = {f"{k[0]}_{k[1]}": v for k, v in ctx.profile_classes().items() if v["ms"] > 0}
    if rank == 0:
        print(json.dumps({"workload": "scf1", "energy": r["energy"], "classes": cls}), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gbhf", choices=["gbhf", "reference"])
    ap.add_argument("--workload", default="w16", choices=["w16", "batch256", "grad8", "w64", "w16d", "fock", "scf1"])
    ap.add_argument("--quick", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-autotune", action="store_true", help="batch256: keep the default task budgets")
    ap.add_argument("--autotune", action="store_true", help="w16: tune the J/K task budgets first")
    ap.add_argument("--no-batch", action="store_true", help="w16: leave out the 256-conformer batch record")
    ap.add_argument("--mixed-cutoff", type=float, default=1e-2,
                    help="batch256: Schwarz-bound cutoff below which ERIs run in FP32 (the workload leaves "
                         "it free; 1e-2 keeps |dE| vs FP64 near 1e-8 Eh)")
    ap.add_argument("--grad-mixed-cutoff", type=float, default=1.0,
                    help="batch256: the same for derivative ERIs (1.0 keeps the gradient within ~1e-6 "
                         "Eh/bohr of FP64; 0: --mixed-cutoff)")
    args = ap.parse_args()
    world, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, world, rank)
    elif args.workload == "batch256":
        run_batch(args, world, rank, local)
    elif args.workload == "grad8":
        run_gradient(args, world, rank, local)
    elif args.workload == "w64":
        run_large(args, world, rank, local)
    elif args.workload == "w16d":
        run_large(args, world, rank, local, "w16", "6-31g*")
    elif args.workload == "fock":
        run_fock_case(args, world, rank, local)
    elif args.workload == "scf1":
        run_scf_case(args, world, rank, local)
    else:
        run_gbhf(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
