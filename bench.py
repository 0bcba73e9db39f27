#!/usr/bin/env python
"""LES grid-point RK3 steps/s on GB300 (one JSON line on stdout).

Default workload: the roofline-sizing channel, 8pi x 2 x 3pi, 256x96x192
cells, Re_tau 5200, equilibrium log-law wall model, dynamic Smagorinsky
(``--workload c3_smag`` for the static-Smagorinsky variant).  A step is one
iteration of the reference's solver loop: compute_dt + compute_time_step_RK3
(app_main.f90:114-117), replayed from one CUDA graph.

  value   grid points x steps / device seconds (CUDA events on the library's
          stream), fields resident in HBM; per-step working set >> L2.
  e2e     same metric through the C ABI with host buffers: every step uploads
          U, V, W from pinned host memory (chl_set_fields), steps, and reads
          U, V, W back (chl_download_async), timed on the host clock; the
          library's copy streams overlap each step's copies with the
          neighbouring steps, and the host synchronises once at the end.
  --impl reference
          the reference algorithm on all host cores: the oracle's C++/OpenMP
          restatement of the step (the Fortran reference cannot be built: no
          gfortran/MPI/FFTW here or on the GPU host), whole steps of the same
          workload until a time budget (--ref-budget) is spent.

Multi-GPU (torchrun): the channels are independent, so nothing is
exchanged.  A batched workload (c4, c5, rl_batch16) is sharded: rank r
takes instances q = r, r + N, ... (strong scaling, the analogue of the
reference's environments spread over worker processes, scripts/submit.sh:2).
A single-channel workload runs one replica per rank with the rank's own seed
(weak scaling).  value = all ranks' grid-point steps / max rank time.

  --measure-peaks
          compiles bench_peaks.cu and rewrites profiles/fp64_peak.json (FP64
          issue rates, the FP64 roofline's denominator) and
          profiles/c2c_bandwidth.json (host<->device copies, the e2e floor).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

import numpy as np

from channel_rl_gb300 import cases as C

METRIC = "LES grid-point RK3 steps/s"
UNIT = "grid-point-steps/s"

# Algorithmic HBM bytes per grid point per launch of each kernel (compulsory
# 8-byte streams; spectral arrays count their half-spectrum share).
KERNEL_BYTES = {
    "rhs_flux": 8 * 13.0,        # U, V, W, nu+nu_t in; 9 face fluxes out
    "rhs_update": 8 * 18.0,      # 9 fluxes + 3 base (+3 F1) in; 3 (+3 F1) out
    # 15 components in + out (the 3 centre velocities on the wall rows only)
    "filter_y": 8 * 30.0, "filter_x": 8 * 30.0, "filter_z": 8 * 30.0,
    "centre_strain": 8 * 19.0,   # U,V,W + 3 edge fields in, |S| + 12 filter inputs out
    "edges": 8 * 6.0,
    "dsm_LM_MM": 8 * 18.0,       # 12 filtered centre fields, 3 filtered faces, 3 edge fields
    "nut": 8 * 2.0,
    "div_fft_x": 8 * 4.0,        # U,V,W in, half spectrum out
    "fft_z": 8 * 2.0,
    "tridiag": 8 * 5.5,
    "ifft_x": 8 * 2.0,
    "project": 8 * 7.0,
    "massflow_shift": 8 * 2.0,
    "dt_minabs": 8 * 3.0,
    "z_solve": 8 * 3.5,          # half spectrum in and out (8 B per point each), tridiagonal factors (12 B)
    "amd": 8 * 4.0,              # U, V, W in, nu_t out
    "vreman": 8 * 4.0,           # U, V, W in, nu_t out
}
# Compulsory traffic of an ideally fused step (8-byte streams per point):
# 107 with the dynamic model, 101 with static Smagorinsky.
STEP_STREAMS = {"dsm": 107, "smag": 101}


def workload(name):
    from dataclasses import replace
    if name == "c3_dsm":
        return [C.c3_roofline(les=C.LES_DSM)]
    if name == "c3_smag":
        return [C.c3_roofline(les=C.LES_SMAG)]
    if name == "c3_amd":
        return [replace(C.c3_roofline(les=C.LES_DSM), LES_model=C.LES_AMD, name="c3_256x96x192_amd_eqwm")]
    if name == "c3_vreman":
        return [replace(C.c3_roofline(les=C.LES_DSM), LES_model=C.LES_VREMAN, name="c3_256x96x192_vreman_eqwm")]
    if name == "rl_case":
        return [C.rl_case()]
    if name == "rl_batch16":
        # 16 environments of the reference's RL size in one handle, one seed each
        return [replace(C.rl_case(seed=2000 + q), name=f"rl_env{q}") for q in range(16)]
    if name == "c3_dsm_small":
        return [C.smaller(C.c3_roofline(les=C.LES_DSM), 128, 96, 96)]
    if name == "c1":
        return [C.c1_small()]
    if name == "c2":
        return [C.c2_wm64()]
    if name == "c4":
        return C.c4_ensemble()
    if name == "c5":
        return C.c5_learned()
    raise SystemExit(f"unknown workload {name}")


BATCHED = ("c4", "c5", "rl_batch16")


def shard(cases_, workload_name, rank, world):
    """This rank's channels: a batched workload's instances q = rank, rank +
    world, ... (each instance exactly once over the ranks), or for a
    single-channel workload one replica with the rank's own seed."""
    if world <= 1:
        return list(cases_)
    if workload_name in BATCHED:
        return [c for q, c in enumerate(cases_) if q % world == rank]
    from dataclasses import replace
    return [replace(c, seed=c.seed + 7919 * rank, name=f"{c.name}_rank{rank}") for c in cases_]


def scaling_of(workload_name, world):
    return "strong" if (workload_name in BATCHED and world > 1) else "weak"


def load_json(path, default=None):
    try:
        with open(path) as f:
            return json.load(f)
    except Exception:
        return default


# ---------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled during the timed region."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.idx), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            time.sleep(0.3)
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 7:
                continue
            try:
                sm.append(float(p[0]))
                mx.append(float(p[1]))
            except ValueError:
                continue
            for n, v in zip(names, p[3:7]):
                if v.lower() in ("active", "1"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------- distributed plumbing
def dist_setup(n):
    if n <= 1 or "RANK" not in os.environ:
        return 0, 1, None
    import torch
    import torch.distributed as dist
    rank, world = int(os.environ["RANK"]), int(os.environ["WORLD_SIZE"])
    backend = "nccl" if torch.cuda.is_available() else "gloo"
    if backend == "nccl":
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
    dist.init_process_group(backend=backend)
    return rank, world, dist


def reduce_max_sum(dist, tmax, work):
    """Max of the per-rank time, sum of the per-rank work (grid-point steps)."""
    if dist is None:
        return tmax, work
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([tmax], dtype=torch.float64, device=dev)
    w = torch.tensor([work], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(w, op=dist.ReduceOp.SUM)
    return float(t.item()), float(w.item())


def barrier(dist):
    if dist is not None:
        dist.barrier()


# ---------------------------------------------------------------- host-core timing
def host_step_rate(cases_, budget_s, max_steps, warmup=1):
    """Grid-point steps/s of the oracle's multi-core C++ restatement of the
    reference step (OpenMP over all host cores) on the given workload: per
    instance `warmup` untimed steps, then whole steps until its share of
    budget_s is spent (at least one).  The learned wall model has no host
    restatement; its instances run the equilibrium model it corrects."""
    from dataclasses import replace
    from oracle.refcpu import RefCPU
    total_pts, total_t, nsteps = 0, 0.0, 0
    for case in cases_:
        c = replace(case, wall_model=min(case.wall_model, C.WM_EQLOG))
        r = RefCPU(c, threads=os.cpu_count())
        r.upload(*C.initial_fields(c))
        r.step(warmup)
        t0 = time.perf_counter()
        n = 0
        while n < max_steps:
            r.step(1)
            n += 1
            if time.perf_counter() - t0 > budget_s / len(cases_):
                break
        total_t += time.perf_counter() - t0
        total_pts += c.points * n
        nsteps += n
        r.close()
    return total_pts / total_t, nsteps, total_t, RefCPU.threads()


def host_single_thread_rate(case):
    """The same restatement on one host thread: one untimed and one timed
    whole step of the workload's first instance."""
    from dataclasses import replace
    from oracle.refcpu import RefCPU
    c = replace(case, wall_model=min(case.wall_model, C.WM_EQLOG))
    r = RefCPU(c)
    n0 = RefCPU.threads()
    RefCPU.set_threads(1)
    try:
        r.upload(*C.initial_fields(c))
        r.step(1)
        t0 = time.perf_counter()
        r.step(1)
        secs = time.perf_counter() - t0
    finally:
        RefCPU.set_threads(n0)
        r.close()
    return {"value": c.points / secs, "unit": UNIT, "cores": 1,
            "sample": f"1 whole RK3 step of {c.Nx}x{c.Ny}x{c.Nz}, {secs:.2f} s on 1 host thread"}


def describe(cases_):
    if len(cases_) == 1:
        c = cases_[0]
        return f"{c.Nx}x{c.Ny}x{c.Nz}"
    return f"{len(cases_)} instances, {sum(c.points for c in cases_)} cells"


def host_sample_text(nsteps, cases_, args, secs, cores):
    wm = " (learned wall model replaced by the equilibrium model)" if cases_[0].wall_model == C.WM_MLP else ""
    return (f"{nsteps} whole RK3 step(s) (compute_dt + compute_time_step_RK3) of {args.workload} "
            f"({describe(cases_)}){wm}, C++/OpenMP restatement of the reference step "
            f"(oracle/refcpu.cpp), {secs:.1f} s on {cores} host threads")


def run_reference(args):
    rank, world, dist = dist_setup(args.gpus)
    if rank != 0:
        return
    cases_ = workload(args.workload)
    rate, nsteps, secs, cores = host_step_rate(cases_, args.ref_budget, max(1, args.steps),
                                               warmup=max(args.warmup, 0))
    sample = host_sample_text(nsteps, cases_, args, secs, cores)
    line = {"impl": "reference", "metric": METRIC, "value": rate, "unit": UNIT, "n_gpus": args.gpus,
            "steps": nsteps, "warmup": max(args.warmup, 0), "ms_per_step": 1e3 * secs / nsteps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": config_of(args, cases_),
            "cpu_baseline": {"value": rate, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def config_of(args, cases_, world=1):
    c0 = cases_[0]
    les = {0: "none", 1: "static-smagorinsky", 2: "dynamic-smagorinsky", 3: "amd", 4: "vreman"}[c0.LES_model]
    wm = {0: "none", 1: "stress", 2: "equilibrium-loglaw", 3: "mlp"}[c0.wall_model]
    pts = sum(c.points for c in cases_)
    streams = STEP_STREAMS["dsm" if c0.LES_model == C.LES_DSM else "smag"]
    ws = pts * streams * 8
    l2 = (f"inputs larger than L2 (per-step compulsory traffic {ws / 1e9:.2f} GB vs 129 MB L2)" if ws > 129e6
          else f"working set {ws / 1e6:.0f} MB fits L2, no flush (small-instance line)")
    sharded = args.workload in BATCHED and world > 1
    return {"workload": args.workload, "instances": len(cases_),
            "grid": f"{c0.Nx}x{c0.Ny}x{c0.Nz}" if len(cases_) == 1 else "mixed",
            "points": pts, "Re_tau": c0.Retau, "sgs": les, "wall_model": wm,
            "parallelism": (f"instances sharded over {world} ranks" if sharded else f"replicas{world}"),
            "l2": l2}


def roofline_of(args, prof, points, step_ms, workload_name, rank=0, dev_index=0):
    """Roofline of the dominant kernel (largest share of the profiled step).

    Both ceilings are computed: HBM bytes (algorithmic bytes per point of the
    kernel, KERNEL_BYTES) against MEASURED_PEAKS.json's copy bandwidth, and
    FP64 issue (FP64-pipe instructions per point of the kernel from the
    committed ncu capture, profiles/kernel_traffic.json) against the best
    measured FP64 issue rate (profiles/fp64_peak.json, bench.py
    --measure-peaks).  The primary entry is the ceiling the kernel is
    nearer to; the other is kept under its own key."""
    dom = max(prof, key=lambda k: prof[k][0])
    dom_ms, dom_n = prof[dom]
    per_launch_s = dom_ms / dom_n * 1e-3
    peaks = load_json(os.path.join(HERE, "MEASURED_PEAKS.json"), {})
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    hbm_src = "measured (MEASURED_PEAKS.json hbm_gbs)" if "hbm_gbs" in peaks else "fallback 6.8 TB/s"
    # measured live by rank 0 (the rank that prints) on its own GPU
    fp64 = (live_fp64_peak(dev_index) if rank == 0 else None) or \
        load_json(os.path.join(HERE, "profiles", "fp64_peak.json"), {})
    traffic = load_json(os.path.join(HERE, "profiles", "kernel_traffic.json"), {})
    byt = KERNEL_BYTES.get(dom, 0.0) * points
    ach = byt / per_launch_s / 1e9
    hbm = {"bound": "hbm", "kernel": dom, "achieved": ach, "peak": hbm_peak, "unit": "GB/s",
           "frac": ach / hbm_peak, "peak_source": hbm_src,
           "traffic": (traffic.get(workload_name, {}).get(dom) if traffic else None),
           "algorithmic_bytes_per_launch": byt, "launch_ms": per_launch_s * 1e3}
    sgs = "dsm" if args.sgs == C.LES_DSM else "smag"
    hbm["step_hbm_gbs_vs_fused_minimum"] = 8 * STEP_STREAMS[sgs] * points / (step_ms * 1e-3) / 1e9
    fl = (traffic or {}).get("fp64_instr_per_point", {}).get(workload_name, {})
    peak_gops = fp64.get("fp64_peak_gops")
    peak_src = ("measured live on this GPU before the timed steps (bench_peaks.cu fp64: best FP64 issue rate, "
                "a DFMA loop on register operands)" if fp64.get("live") else
                "measured on a GB300 (profiles/fp64_peak.json from bench.py --measure-peaks: best FP64 "
                "issue rate, a DFMA loop on register operands)")
    if not (peak_gops and dom in fl):
        return hbm
    achf = fl[dom] * points / per_launch_s / 1e9
    step_instr = sum(fl.get(k, 0.0) * n for k, (_, n) in prof.items()) * points
    step_ach = step_instr / (step_ms * 1e-3) / 1e9
    f64 = {"bound": "fp64-issue", "kernel": dom, "achieved": achf, "peak": peak_gops, "unit": "G FP64 instr/s",
           "frac": achf / peak_gops, "traffic": hbm["traffic"], "launch_ms": hbm["launch_ms"],
           "fp64_instr_per_point": fl[dom],
           "step_achieved": step_ach, "step_frac": step_ach / peak_gops,
           "step_fp64_instr_per_point": step_instr / points,
           "peak_source": peak_src}
    if f64["frac"] >= hbm["frac"]:
        f64["hbm"] = hbm
        return f64
    hbm["fp64"] = f64
    return hbm


# ---------------------------------------------------------------- our arm
def run_ours(args):
    rank, world, dist = dist_setup(args.gpus)
    import torch
    from channel_rl_gb300.host import Channel, load
    torch.cuda.init()
    dev_index = int(os.environ.get("LOCAL_RANK", 0))
    cases_ = shard(workload(args.workload), args.workload, rank, world)
    args.sgs = cases_[0].LES_model
    ch = Channel(cases_)
    for q, case in enumerate(cases_):
        ch.upload(*C.initial_fields(case), inst=q)
    if cases_[0].wall_model == C.WM_MLP:
        ch.mlp_set_params(mlp_params()[0])
    # tile shapes picked by the library's tuner, or given (results are
    # bit-identical for every candidate; untimed)
    if args.tile_shapes:
        ch.set_tile_shapes(*(int(v) for v in args.tile_shapes.split(",")))
        tune_report = f"given: {args.tile_shapes}"
    else:
        tune_report = None if args.no_autotune else ch.autotune()
    points = sum(c.points for c in cases_)
    # warm-up (builds the graph on the first call)
    ch.step(max(args.warmup, 1))
    ch.synchronize()
    nker = ch.graph_kernel_count()
    # timed region: barrier + sync on both sides, device time by CUDA events
    # over exactly `steps` graph replays; then a sustained window of at least
    # --min-seconds (the same graph replayed back to back), whose clocks are
    # the ones reported
    barrier(dist)
    torch.cuda.synchronize()
    with ClockSampler(physical_gpu(dev_index)) as clk:
        t0 = time.perf_counter()
        ms = ch.time_steps(args.steps)
        wall = time.perf_counter() - t0
        torch.cuda.synchronize()
        barrier(dist)
        tmax_ms, work = reduce_max_sum(dist, ms, points * args.steps)
        sus = None
        if args.min_seconds > 0:
            n_sus = max(args.steps, int(args.steps * args.min_seconds * 1e3 / max(tmax_ms, 1e-3)) + 1)
            barrier(dist)
            torch.cuda.synchronize()
            ms_s = ch.time_steps(n_sus)
            torch.cuda.synchronize()
            barrier(dist)
            tmax_s, work_s = reduce_max_sum(dist, ms_s, points * n_sus)
            sus = {"value": work_s / (tmax_s * 1e-3), "steps": n_sus, "seconds": tmax_s * 1e-3,
                   "ms_per_step": tmax_s / n_sus}
    value = work / (tmax_ms * 1e-3)
    # per-kernel breakdown (event-bracketed, un-graphed steps)
    prof = ch.profile_step(reps=args.prof_reps)
    tot_prof = sum(v[0] for v in prof.values())
    roof = roofline_of(args, prof, points, tmax_ms / args.steps, args.workload, rank, dev_index)
    # e2e through the C ABI with pinned host buffers
    e2e = None
    if not args.no_e2e and len(cases_) == 1:
        e2e = e2e_rate(ch, cases_[0], args)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": tmax_ms / args.steps, "higher_is_better": True,
            "scaling": scaling_of(args.workload, world), "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": config_of(args, cases_ if world == 1 else workload(args.workload), world),
            "e2e": e2e, "roofline": roof,
            "gpu_launches": nker * args.steps, "clocks": clk.summary(), "sustained": sus,
            "tile_shapes": dict(ch.tile_shapes(), tuner=tune_report or "off (defaults)"),
            "host_wall_s": wall,
            "kernels_ms_per_step": {k: round(v[0], 4) for k, v in sorted(prof.items(), key=lambda kv: -kv[1][0])},
            "profiled_step_ms": tot_prof}
    if args.workload in ("c3_dsm", "c3_smag") and not args.no_batched and world == 1:
        line["batched_mlp"] = batched_mlp_rate(args)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        rate, nsteps, secs, cores = host_step_rate(cases_, args.cpu_budget, 50)
        line["cpu_baseline"] = {"value": rate, "unit": UNIT, "cores": cores, "kind": "port",
                                "sample": host_sample_text(nsteps, cases_, args, secs, cores),
                                "single_thread": host_single_thread_rate(cases_[0])}
    if rank == 0:
        print(json.dumps(line), flush=True)
    ch.close()


def mlp_params():
    """Trained wall-model parameters if a checkpoint ships with the package,
    else the seeded initial network."""
    from channel_rl_gb300 import rl
    path = os.path.join(HERE, "channel_rl_gb300", "data", "mlp_wm.npy")
    if os.path.exists(path):
        return np.load(path).astype(np.float32), "trained checkpoint"
    return rl.init_params(1234), "seeded Xavier initialisation"


def timed_rate(cases_, args, steps, setup=None):
    from channel_rl_gb300.host import Channel
    ch = Channel(cases_)
    for q, c in enumerate(cases_):
        ch.upload(*C.initial_fields(c), inst=q)
    if setup:
        setup(ch)
    if not args.no_autotune:
        ch.autotune()
    ch.step(max(args.warmup, 3))
    ch.synchronize()
    ms = ch.time_steps(steps)
    ch.close()
    return sum(c.points for c in cases_) * steps / (ms * 1e-3), ms / steps


def utau_gate(theta, steps=120, spinup=200):
    """The accuracy half of the batched line: u_tau error of each of the 16
    channels against its target, from the wall stress averaged over `steps`
    deterministic steps after a `spinup`, with the learned correction and
    with the equilibrium model it corrects (channel_rl_gb300.rl.Trainer)."""
    from channel_rl_gb300.rl import Trainer
    tr = Trainer(C.c5_learned(), spinup=spinup)
    try:
        _, ut_l = tr.evaluate(theta, steps=steps)
        _, ut_e = tr.evaluate(None, steps=steps)
    finally:
        tr.close()
    return {"gate": 0.02, "steps": steps, "spinup": spinup,
            "learned_max": float(max(ut_l)), "learned_mean": float(sum(ut_l) / len(ut_l)),
            "equilibrium_max": float(max(ut_e)), "equilibrium_mean": float(sum(ut_e) / len(ut_e)),
            "within_gate": bool(max(ut_l) <= 0.02)}


def batched_mlp_rate(args):
    """16 uneven channels with the learned wall model in one launch per
    kernel, against the same 16 channels run one at a time, each as a plain
    single instance (equilibrium wall model): sum of points / sum of times."""
    from dataclasses import replace
    batch = C.c5_learned()
    theta, src = mlp_params()
    rate_b, ms_b = timed_rate(batch, args, 20, setup=lambda ch: ch.mlp_set_params(theta))
    ms_seq, smallest = 0.0, None
    for c in batch:
        single = replace(c, wall_model=C.WM_EQLOG)
        r, ms = timed_rate([single], args, 20)
        ms_seq += ms
        if smallest is None or single.points < smallest[0]:
            smallest = (single.points, r, f"{single.Nx}x{single.Ny}x{single.Nz}")
    pts = sum(c.points for c in batch)
    rate_s = pts / (ms_seq * 1e-3)
    small = C.c1_small()
    rate_c1, _ = timed_rate([small], args, 40)
    return {"metric": METRIC, "value": rate_b, "unit": UNIT, "ms_per_step": ms_b, "instances": len(batch),
            "points": pts, "wall_model": f"mlp ({src})",
            "plain_single_instances_in_sequence": {"value": rate_s, "ms_per_step": ms_seq,
                                                   "wall_model": "equilibrium-loglaw"},
            "smallest_plain_single_instance": {"grid": smallest[2], "value": smallest[1]},
            "speedup_vs_plain_single": rate_b / rate_s,
            "plain_single_small_channel": {"grid": f"{small.Nx}x{small.Ny}x{small.Nz}", "value": rate_c1,
                                           "sgs": "dynamic-smagorinsky", "wall_model": "none"},
            "speedup_vs_plain_single_small_channel": rate_b / rate_c1,
            "u_tau_error": utau_gate(theta)}


def e2e_rate(ch, case, args):
    import torch
    U, V, W = C.initial_fields(case)
    pin = []
    for a in (U, V, W):
        t = torch.empty(a.size, dtype=torch.float64, pin_memory=True)
        v = t.numpy().reshape(a.shape, order="F")
        v[...] = a
        pin.append((t, v))
    out = []
    for a in (U, V, W):
        t = torch.empty(a.size, dtype=torch.float64, pin_memory=True)
        out.append((t, t.numpy().reshape(a.shape, order="F")))
    hb = sum(a.size * 8 for a in (U, V, W))
    for _ in range(2):
        ch.set_fields_ptr(pin[0][1], pin[1][1], pin[2][1])
        ch.step(1)
        ch.download_async(out[0][1], out[1][1], out[2][1])
    ch.synchronize()
    n = max(1, args.e2e_steps)
    # every step copies its inputs in and its result out; the library runs
    # the copies on its copy streams, so one step's upload and the previous
    # step's download overlap the step in between; the host waits for all of
    # it once, at the end of the timed region
    t0 = time.perf_counter()
    for _ in range(n):
        ch.set_fields_ptr(pin[0][1], pin[1][1], pin[2][1])
        ch.step(1)
        ch.download_async(out[0][1], out[1][1], out[2][1])
    ch.synchronize()
    secs = time.perf_counter() - t0
    out = {"value": case.points * n / secs, "unit": UNIT, "h2d_bytes_per_step": hb, "d2h_bytes_per_step": hb,
           "steps": n, "ms_per_step": 1e3 * secs / n,
           "path": "chl_set_fields + chl_rk3_step + chl_download_async per step, pinned host U,V,W; copies on the "
                   "library's copy streams overlap the neighbouring steps; one chl_synchronize at the end"}
    c2c = load_json(os.path.join(HERE, "profiles", "c2c_bandwidth.json"), {})
    if c2c.get("memcpy_h2d_gbs") and c2c.get("memcpy_d2h_gbs"):
        # the copies run beside the neighbouring steps; their time per step
        # (the two directions use separate copy engines) is the floor when it
        # exceeds the step's own
        out["transfer_ms_per_step"] = 1e3 * max(hb / (c2c["memcpy_h2d_gbs"] * 1e9), hb / (c2c["memcpy_d2h_gbs"] * 1e9))
        out["transfer_source"] = "profiles/c2c_bandwidth.json (measured pinned-copy bandwidth)"
    return out


# ---------------------------------------------------------------- peak probes
def _fp64_record(out):
    """bench_peaks fp64 output as the profiles/fp64_peak.json record."""
    import re
    res = {"raw": out.strip().splitlines()}
    m = re.search(r"^BEST dfma ([0-9.]+) dadd ([0-9.]+) mixed ([0-9.]+) ddiv ([0-9.]+) dsqrt ([0-9.]+) ffma ([0-9.]+)"
                  r" reg ([0-9.]+)", out, re.M)
    if m:
        for key, v in zip(("dfma", "dadd", "mixed", "ddiv", "dsqrt", "ffma", "reg_operands"), m.groups()):
            res[key + "_gops"] = float(v)
        res["fp64_peak_gops"] = max(res["dfma_gops"], res["dadd_gops"], res["mixed_gops"], res["reg_operands_gops"])
        res["dfma_gflops"] = 2.0 * res["fp64_peak_gops"]
    # DFMA reading three different registers each (no operand reuse), the
    # form of the stencil kernels' FMAs: the practical rate for such code
    distinct = [float(x) for x in re.findall(r"^DFMA 3 distinct regs x\d+ chains: [0-9.]+ ms, ([0-9.]+) Gop/s", out, re.M)]
    if distinct:
        res["dfma_distinct_operands_gops"] = max(distinct)
    res["how"] = ("bench_peaks.cu fp64: 8, 16 and 32 independent dependency chains per thread (loop unrolled 4x), "
                  "152x8 blocks x 256 threads, CUDA events, third repetition, best of the sweep; thread-instructions "
                  "per second; operands from the constant bank, and from registers in the reg_operands probes")
    return res


def _c2c_record(out):
    """bench_peaks c2c output as the profiles/c2c_bandwidth.json record."""
    import re
    res = {"raw": out.strip().splitlines()}
    for key, pat in (("memcpy_h2d_gbs", r"^memcpy H2D ([0-9.]+)"), ("memcpy_d2h_gbs", r"^memcpy D2H ([0-9.]+)"),
                     ("kernel_read_host_gbs", r"^kernel read host x8 ([0-9.]+)"),
                     ("kernel_write_host_gbs", r"^kernel write host x8 ([0-9.]+)")):
        m = re.search(pat, out, re.M)
        if m:
            res[key] = float(m.group(1))
    res["how"] = "bench_peaks.cu c2c: 118 MB pinned buffers (cudaMallocHost), CUDA events, third repetition"
    return res


def _barrier_record(out):
    """bench_peaks barrier output: microseconds per phase of each ordering."""
    import re
    res = {"raw": out.strip().splitlines()}
    per = [float(x) for x in re.findall(r"^persistent .*: ([0-9.]+) us per phase", out, re.M)]
    pdl = [float(x) for x in re.findall(r"^graph pdl .*: ([0-9.]+) us per phase", out, re.M)]
    if per and pdl:
        res["persistent_barrier_us_best"] = min(per)
        res["graph_pdl_boundary_us_best"] = min(pdl)
    res["how"] = ("bench_peaks.cu barrier: 49152-double update per phase; 2000 phases in one cooperative kernel "
                  "(grid barrier: arrival counter and generation word) vs 200 kernels in one CUDA graph, CUDA events")
    return res


_LIVE_FP64 = None


def physical_gpu(dev_index):
    """The GPU (index or UUID as nvidia-smi and CUDA_VISIBLE_DEVICES name it)
    behind visible device dev_index."""
    vis = [v.strip() for v in os.environ.get("CUDA_VISIBLE_DEVICES", "").split(",") if v.strip()]
    return vis[dev_index] if dev_index < len(vis) else str(dev_index)


def live_fp64_peak(dev_index=0):
    """The FP64 issue rates of this rank's GPU (dev_index among the visible
    ones) from bench_peaks.cu, run once per process (about a second of GPU
    time), or None where the probe binary was not built."""
    global _LIVE_FP64
    if _LIVE_FP64 is None:
        _LIVE_FP64 = {}
        try:
            from channel_rl_gb300 import build as b
            exe = b.PEAKS_BIN
            if os.path.exists(exe):
                env = dict(os.environ)
                env["CUDA_VISIBLE_DEVICES"] = physical_gpu(dev_index)
                out = subprocess.run([exe, "fp64"], check=True, capture_output=True, text=True, timeout=120,
                                     env=env).stdout
                rec = _fp64_record(out)
                if rec.get("fp64_peak_gops"):
                    rec["live"] = True
                    _LIVE_FP64 = rec
        except Exception:
            _LIVE_FP64 = {}
    return _LIVE_FP64 or None


def measure_peaks():
    """Compile bench_peaks.cu, run both probes, write their records."""
    import tempfile
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "bench_peaks")
        subprocess.run(["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-o", exe,
                        os.path.join(HERE, "bench_peaks.cu")], check=True)
        outs = {m: subprocess.run([exe, m], check=True, capture_output=True, text=True).stdout
                for m in ("fp64", "c2c", "barrier")}
    os.makedirs(os.path.join(HERE, "profiles"), exist_ok=True)
    for name, rec in (("fp64_peak.json", _fp64_record(outs["fp64"])), ("c2c_bandwidth.json", _c2c_record(outs["c2c"])),
                      ("phase_ordering.json", _barrier_record(outs["barrier"]))):
        with open(os.path.join(HERE, "profiles", name), "w") as f:
            json.dump(rec, f, indent=1)
    print(outs["fp64"] + outs["c2c"] + outs["barrier"])


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=60)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=("ours", "reference"), default="ours")
    ap.add_argument("--workload", default="c3_dsm")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default tile shapes")
    ap.add_argument("--tile-shapes", default="",
                    help="x_min_blocks,z_min_blocks,tri_mode,point_threads instead of tuning (e.g. to profile the "
                         "tuned shapes without the tuner's own launches)")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched learned-wall-model line")
    ap.add_argument("--e2e-steps", type=int, default=20)
    ap.add_argument("--prof-reps", type=int, default=3)
    ap.add_argument("--cpu-budget", type=float, default=20.0)
    ap.add_argument("--ref-budget", type=float, default=120.0)
    ap.add_argument("--min-seconds", type=float, default=2.0,
                    help="length of the sustained window after the timed steps (0: none)")
    ap.add_argument("--measure-peaks", action="store_true", help="run bench_peaks.cu and rewrite its records")
    args = ap.parse_args()
    if args.measure_peaks:
        measure_peaks()
        return
    if args.warmup < 3 and args.impl == "ours":
        print("warning: fewer than 3 warm-up steps", file=sys.stderr)
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
