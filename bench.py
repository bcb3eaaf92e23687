#!/usr/bin/env python3
"""Benchmark of the batched FWI gradient on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

A step is one full gradient of the shot batch of the workload (default: the
560 x 1700 grid, nt 4000, 64 shots, 1700 receivers): forward modelling with
strip saving, L2 misfit and residual, exact adjoint with source rebuild and
imaging, and the FP64 reduction over shots.  Prints one JSON line.

* ``value``: shot-gradients/s over the whole job with every input resident in
  HBM (CUDA events on the engine's stream, W warm-up steps, K timed steps).
* ``e2e``: the same metric through the C ABI with host buffers: every step
  uploads the model and the observed traces from pinned memory and reads back
  the misfit and the FP64 gradient (fwi_set_model, then fwi_gradient_obs, whose
  trace upload runs on a copy stream beside the forward phase).
* ``roofline``: the dominant kernel (the fused backward step) at its
  algorithmic 36 B per physical cell-step against the measured HBM copy peak.
* ``c3``: the 256-shot uneven batch (600 x 2000, records of 3000-6000 steps,
  off-end spreads of 200-1200 receivers) measured in the same run: throughput,
  backward roofline, plain per-shot ratio and the FP64 check of its shortest
  shot (single-GPU runs of the default workload; ``--skip c3`` leaves it out).
* ``aux``: sfbandpass and grad_precond_new5 through the C ABI against the
  reference's own compiled routines (bit-identical outputs, wall times).
* ``cpu_baseline``: the reference's CPU path on the machine's host cores on a
  bounded sample of the same workload (--cpu-shots shots, the first
  --cpu-steps time steps), scaled linearly; ``kind`` "reference" when the reference's own
  kernels are built (oracle/_ref: a_lap_opt_2d_pml, a_lap_opt_2d,
  time_integral, write_bdr, read_bdr under a restated gradient driver, since
  the reference's driver does not exist), else "port" (the restatement in
  oracle/).  The first shot of the sample checks the GPU gradient against the
  FP64 oracle.

``--impl reference`` times only that CPU path, with all host threads, on the
same workload and metric; it loads nothing but oracle/ libraries.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "fwi2dacoustic-mpi-lbfgs_gb300")
sys.path.insert(0, PKG)

METRIC = "shot-gradients/s & Gcell-steps/s, batched vs plain, at ≤1e-4 grad rel err"
UNIT = "shot-gradients/s"
BWD_BYTES = 36.0   # algorithmic bytes per physical cell-step of the fused backward step
FWD_BYTES = 16.0   # ... of the forward step


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="c2")
    ap.add_argument("--scale", type=float, default=1.0)
    ap.add_argument("--nshots", type=int, default=None)
    ap.add_argument("--nt", type=int, default=None)
    ap.add_argument("--plain-shots", type=int, default=4)
    ap.add_argument("--cpu-steps", type=int, default=4000, help="time steps of the cpu_baseline sample and accuracy check")
    ap.add_argument("--cpu-shots", type=int, default=2, help="shots of the CPU sample in the cpu_baseline leg")
    ap.add_argument("--ref-steps", type=int, default=500, help="time steps of each reference-arm sample")
    ap.add_argument("--no-graph", action="store_true")
    ap.add_argument("--store", default="auto", choices=["auto", "strips", "snapshots"],
                    help="forward-field storage of the backward half")
    ap.add_argument("--snapshots", type=int, default=0, help="segments of the checkpointed backward (0: sqrt(nt))")
    ap.add_argument("--snap-precision", default="f32", choices=["f32", "f16", "bf16"])
    ap.add_argument("--hbm-budget-mb", type=int, default=0, help="budget of --store auto (0: 90%% of free memory)")
    ap.add_argument("--fd-order", type=int, default=4, choices=[4, 8], help="4: the reference's; 8: the extension")
    ap.add_argument("--skip", default="", help="comma list of: e2e,plain,cpu,strips,tune,c3,aux")
    return ap.parse_args()


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class Clocks:
    """Samples nvidia-smi every 200 ms while the timed region runs."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                       "-lms", "200", "-i", str(device)], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        if self.p:
            self.p.terminate()
            try:
                self.p.wait(5)
            except Exception:
                self.p.kill()
        self.f.flush()
        self.f.seek(0)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.f.read().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for n, v in zip(names, parts[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        os.unlink(self.f.name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def traffic_per_cell_step(kernel):
    """DRAM bytes per physical cell-step of one launch of `kernel`, as measured
    by ncu (profiles/traffic.txt: lines of `kernel bytes`)."""
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.txt")) as f:
            for line in f:
                parts = line.split()
                if len(parts) == 2 and parts[0] == kernel:
                    return float(parts[1])
    except OSError:
        pass
    return None


def workload(args, world=1, rank=0):
    """The workload's shots; on world > 1 ranks, rank's cost-balanced share of
    world x nshots shots (shots_parallel.partition_shots)."""
    import workloads
    per_rank = args.nshots or workloads.CONFIGS[args.workload]["nshots"]
    cfgkw, vtrue, vstart, shots = workloads.build(args.workload, scale=args.scale, nshots=per_rank * world, nt=args.nt)
    if world > 1:
        import shots_parallel
        mine = shots_parallel.partition_shots([s.nt for s in shots], world, rank)
        shots = [shots[i] for i in mine]
    return cfgkw, vtrue, vstart, shots


STORE_NAMES = {0: "auto", 1: "strips", 2: "snapshots"}


def describe(args, cfgkw, shots, stats=None):
    nts = sorted({s.nt for s in shots})
    nrs = sorted({s.nr for s in shots})
    if stats is None or stats.get("store") in (None, 0, 1):
        ckpt = "boundary strips of every step in HBM"
    else:
        ckpt = (f"checkpoints: {stats['segments']} segments, {args.snap_precision} storage, forward recompute "
                f"per segment")
    return {"workload": f"{args.workload}: {cfgkw['nz']}x{cfgkw['nx']} grid, dx {cfgkw['dx']} m, "
                        f"dt {cfgkw['dt'] * 1e3:g} ms, CPML {cfgkw['npml']}, {len(shots)} shots",
            "nz": cfgkw["nz"], "nx": cfgkw["nx"], "npml": cfgkw["npml"], "shots": len(shots),
            "nt": nts[0] if len(nts) == 1 else [nts[0], nts[-1]],
            "receivers": nrs[0] if len(nrs) == 1 else [nrs[0], nrs[-1]],
            "fd_order": args.fd_order, "free_surface": True, "checkpointing": ckpt,
            "store_gb": None if stats is None else stats["store_bytes"] / 1e9,
            "l2": "working set larger than L2 (no flush)", "parallelism": f"shots batched per launch",
            "data": "synthetic seeded model and acquisition; observed traces modelled on the true model"}


def oracle_shots(O, o, shots, dx, dz, nt):
    """The shots in cell indices for the CPU paths (the cell rounding of
    fwi_2d.c:363-364, restated in the oracle), wavelets cut to nt steps."""
    import numpy as np
    out = []
    for shot in shots:
        isx, isz = o.cell_of(shot.src_x, shot.src_z, dx, dz)
        cells = [o.cell_of(float(x), float(z), dx, dz) for x, z in shot.rec_xz]
        irx = np.array([c[0] for c in cells], np.int32)
        irz = np.array([c[1] for c in cells], np.int32)
        out.append(O.Shot(isx, isz, irx, irz, shot.wavelet[:nt]))
    return out


def cpu_sample(args, cfgkw, vstart, vtrue, shots, nt_sample, kind, check_gpu=None, cache=None):
    """Times one CPU gradient of the given shots over the first nt_sample
    time steps of the first shot's record on all host cores: the reference's
    own kernels driven as the reference would (kind "reference", oracle/_ref)
    or the CPU restatement (kind "port", FP32 oracle).  Optionally checks a
    GPU gradient of the first shot against the FP64 oracle.  `cache` keeps
    the modelled observed traces between calls (setup, untimed)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import numpy as np
    import oracle as O
    O.build()
    cache = {} if cache is None else cache
    nt = min([nt_sample] + [s.nt for s in shots])
    nt = (nt - 1) // cfgkw["jump"] * cfgkw["jump"] + 1
    cores = os.cpu_count() or 1
    ocfg = O.make_config(nx=cfgkw["nx"], nz=cfgkw["nz"], npml=cfgkw["npml"], nt=nt, dx=cfgkw["dx"],
                         dz=cfgkw["dz"], dt=cfgkw["dt"], free_surface=1, jump=cfgkw["jump"], nthreads=cores)
    o32 = O.Oracle("f32")
    oshots = oracle_shots(O, o32, shots, cfgkw["dx"], cfgkw["dz"], nt)
    obss = []
    for shot, osh in zip(shots, oshots):
        key = (id(shot), nt)
        if key not in cache:
            cache[key] = o32.forward(ocfg, vtrue, osh).astype(np.float32)
        obss.append(cache[key])
    if kind == "reference":
        ref = O.RefKernels()
        t0 = time.perf_counter()
        ref.gradient(ocfg, vstart, oshots, obss)
        sec = time.perf_counter() - t0
    else:
        t0 = time.perf_counter()
        o32.gradient(ocfg, vstart, oshots, obss)
        sec = time.perf_counter() - t0
    out = {"sec": sec, "nt": nt, "shots": len(shots), "cores": cores, "kind": kind}
    if check_gpu is not None:
        o64 = O.Oracle("f64")
        J64, g64, _ = o64.gradient(ocfg, vstart, oshots[:1], obss[:1])
        J32, g32, _ = o32.gradient(ocfg, vstart, oshots[:1], obss[:1])
        g_gpu = check_gpu(nt, obss[0])
        out["grad_rel_err"] = float(np.linalg.norm(g_gpu - g64) / np.linalg.norm(g64))
        out["grad_rel_err_cpu_fp32"] = float(np.linalg.norm(g32 - g64) / np.linalg.norm(g64))
    return out


def cpu_kind():
    """"reference" when the reference's own kernels are built (oracle/_ref),
    else "port" (the oracle's restatement)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    O.build()
    return "reference" if O.RefKernels.available() else "port"


def run_reference(args):
    """The reference's CPU path on the workload: each timed step is one
    gradient of one shot over the first --ref-steps time steps (a bounded
    sample, 10-30 s of CPU work), and ms_per_step scales it linearly to the
    full gradient of every shot of the workload."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    cfgkw, vtrue, vstart, shots = workload(args)
    nshots = len(shots)
    kind = cpu_kind()
    times, cache = [], {}
    warm = max(3, args.warmup)
    for i in range(warm + args.steps):
        r = cpu_sample(args, cfgkw, vstart, vtrue, shots[:1], args.ref_steps, kind, cache=cache)
        if i >= warm:
            times.append(r["sec"])
    sample_s = statistics.median(times)
    factor = sum(s.nt for s in shots) / r["nt"]                 # linear in shot-steps
    ms_step = sample_s * factor * 1e3
    value = nshots / (ms_step / 1e3)
    what = ("the reference's own compiled kernels (a_lap_opt_2d_pml, a_lap_opt_2d, time_integral, write_bdr, "
            "read_bdr) under a restated gradient driver" if kind == "reference" else
            "the CPU restatement of the reference path (oracle/, FP32)")
    sample = (f"{what}; each step: 1 shot, {r['nt']} of {shots[0].nt} time steps (forward, L2 misfit, rebuild, "
              f"adjoint, imaging), {sample_s:.2f} s on {r['cores']} threads; ms_per_step = that time x {factor:.1f} "
              f"(all {nshots} shots, every step)")
    line = {"metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": warm, "ms_per_step": ms_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": describe(args, cfgkw, shots),
            "extrapolated": {"sample_ms_per_step": sample_s * 1e3, "factor": factor,
                             "timed_wall_s": sample_s * args.steps,
                             "note": "each timed step runs a sample of the full gradient, so ms_per_step x steps "
                                     "exceeds the run's wall time by the factor"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": r["cores"], "kind": kind, "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def aux_leg(local):
    """The routines around the gradient on data of the 560 x 1700, 64-shot
    workload's sizes, each through the C
    ABI (host buffers in and out, device buffers allocated per call) against
    the reference's own compiled routine on one host core (the reference runs
    them serially): sfbandpass on one shot record of 1700 traces x 4000
    samples, grad_precond_new5 on a 560 x 1700 gradient.  Outputs are compared
    bit for bit."""
    import numpy as np
    import fwigpu
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    O.build()
    ref = O.RefAux() if O.RefAux.available() else O.AuxOracle()
    kind = "reference" if O.RefAux.available() else "port"
    rng = np.random.default_rng(7)
    out = {}
    traces = rng.standard_normal((1700, 4000)).astype(np.float32)
    bp = (0.0008, 0, 6, 6, 10.0, 3.0)                       # dt, zero phase, orders, fhi, flo
    grad = (rng.standard_normal((560, 1700)) * 1e-3).astype(np.float32)
    bottom = rng.integers(0, 40, 1700).astype(np.int32)
    pc = (0.95, 20, 3, 15, 2, 1.0)                           # perc, rect1, repeat1, rect2, repeat2, alpha
    for name, gpu, cpu in (
            ("bandpass", lambda: fwigpu.bandpass(traces, *bp), lambda: ref.bandpass(traces, *bp)),
            ("grad_precond", lambda: fwigpu.grad_precond(grad, *pc, bottom),
             lambda: ref.grad_precond(grad, *pc, bottom))):
        gpu()                                                # first call: module load
        t0 = time.perf_counter()
        g_out = gpu()
        t_gpu = time.perf_counter() - t0
        t0 = time.perf_counter()
        c_out = cpu()
        t_cpu = time.perf_counter() - t0
        out[name] = {"gpu_ms": t_gpu * 1e3, "cpu_ms": t_cpu * 1e3, "cpu_kind": kind, "cpu_threads": 1,
                     "speedup": t_cpu / t_gpu, "bit_identical": bool(np.array_equal(g_out, c_out))}
    out["bandpass"]["data"] = "1700 traces x 4000 samples, zero phase, orders 6/6, 3-10 Hz"
    out["grad_precond"]["data"] = "560 x 1700, perc 0.95, triangle 20 x3 then 15 x2"
    out["note"] = ("wall time of one call each: the GPU's includes the host-device copies and the per-call device "
                   "allocations of the C ABI")
    return out


def extra_leg(name, args, local, stream):
    """A second workload measured in the same run (single GPU): its own
    throughput (CUDA events on the engine's stream, 3 warm-up gradients, one
    timed), backward roofline, plain per-shot ratio over 4 shots and the
    gradient of its shortest shot against the FP64 oracle (a bounded CPU
    check).  Reported as an extra key of the main line."""
    import numpy as np
    import torch
    import fwigpu
    import tuning
    import workloads
    cfgkw, vtrue, vstart, shots = workloads.build(name)
    cells = float(cfgkw["nx"] * cfgkw["nz"])
    step_cells = sum(s.nt for s in shots) * cells
    with fwigpu.Engine(fwigpu.make_config(**cfgkw, device=local, use_graph=1)) as eng:
        eng.set_stream(stream.cuda_stream)
        eng.set_shots(shots)
        tune = tuning.autotune(eng, shots, vstart)
        eng.set_model(vtrue)
        obs = eng.forward()
        eng.set_observed(obs)
        eng.set_model(vstart)
        for _ in range(3):
            eng.gradient(keep_on_device=True)
        torch.cuda.synchronize()
        clk = Clocks(local)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        eng.gradient(keep_on_device=True)
        e1.record(stream)
        torch.cuda.synchronize()
        clocks = clk.stop()
        ms = e0.elapsed_time(e1)
        st = eng.stats()
    nt_max = max(s.nt for s in shots)
    peak, peak_kind = peaks()
    bwd_launch_ms = st["ms_backward"] / nt_max
    achieved = BWD_BYTES * step_cells / nt_max / (bwd_launch_ms / 1e3) / 1e9
    out = {"workload": describe(argparse.Namespace(**dict(vars(args), workload=name)), cfgkw, shots)["workload"],
           "value": len(shots) / (ms / 1e3), "unit": UNIT,
           "ms_per_step": ms, "steps": 1, "warmup": 3, "gcell_steps_per_s": 3.0 * step_cells / (ms / 1e3) / 1e9,
           "nt": [min(s.nt for s in shots), nt_max], "receivers": [min(s.nr for s in shots), max(s.nr for s in shots)],
           "clocks": clocks, "tuning": tune["tuning"],
           "roofline": {"kernel": "k_backward", "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                        "frac": achieved / peak, "peak_kind": peak_kind, "avg_launch_ms": bwd_launch_ms}}
    # plain per-shot path on 4 shots of the batch
    k = 4
    with fwigpu.Engine(fwigpu.make_config(**dict(cfgkw, nt_max=max(s.nt for s in shots[:k])), device=local,
                                          plain_per_shot=1)) as pe:
        pe.set_stream(stream.cuda_stream)
        pe.set_shots(shots[:k])
        pe.set_model(vstart)
        pe.set_observed(obs[:pe.nsamples])
        pe.gradient(keep_on_device=True)
        e0.record(stream)
        pe.gradient(keep_on_device=True)
        e1.record(stream)
        torch.cuda.synchronize()
        plain = k / (e0.elapsed_time(e1) / 1e3)
    out["plain"] = {"shots": k, "value": plain, "batched_over_plain": out["value"] / plain}
    # accuracy: the shortest shot against the FP64 oracle
    if "cpu" not in set(filter(None, args.skip.split(","))):
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as O
        O.build()
        i = min(range(len(shots)), key=lambda q: shots[q].nt)
        s0 = shots[i]
        o64 = O.Oracle("f64")
        ocfg = O.make_config(nx=cfgkw["nx"], nz=cfgkw["nz"], npml=cfgkw["npml"], nt=s0.nt, dx=cfgkw["dx"],
                             dz=cfgkw["dz"], dt=cfgkw["dt"], free_surface=1, jump=cfgkw["jump"],
                             nthreads=os.cpu_count() or 1)
        osh = oracle_shots(O, o64, [s0], cfgkw["dx"], cfgkw["dz"], s0.nt)[0]
        ob = o64.forward(ocfg, vtrue, osh).astype(np.float32)
        _, g64, _ = o64.gradient(ocfg, vstart, [osh], [ob])
        with fwigpu.Engine(fwigpu.make_config(**dict(cfgkw, nt_max=s0.nt), device=local)) as e1_:
            e1_.set_shots([s0])
            e1_.set_model(vstart)
            e1_.set_observed(ob)
            g = e1_.gradient()[1]
        out["accuracy"] = {"grad_rel_err_vs_fp64": float(np.linalg.norm(g - g64) / np.linalg.norm(g64)),
                           "sample": f"the shortest shot ({s0.nt} steps, {s0.nr} receivers), workload grid"}
    return out


def run_ours(args):
    import numpy as np
    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    skip = set(filter(None, args.skip.split(",")))
    import build as engine_build
    if rank == 0:
        engine_build.build()
    if dist:
        dist.barrier()
    import fwigpu

    cfgkw, vtrue, vstart, shots = workload(args, world, rank)
    nshots = len(shots)
    store = {"auto": fwigpu.STORE_AUTO, "strips": fwigpu.STORE_STRIPS, "snapshots": fwigpu.STORE_SNAPSHOTS}[args.store]
    cfg = fwigpu.make_config(**cfgkw, device=local, use_graph=0 if args.no_graph else 1, store=store,
                             snapshots=args.snapshots, snap_precision=args.snap_precision,
                             hbm_budget_mb=args.hbm_budget_mb, fd_order=args.fd_order)
    eng = fwigpu.Engine(cfg)
    stream = torch.cuda.Stream()
    eng.set_stream(stream.cuda_stream)
    eng.set_shots(shots)
    tune = None
    if "tune" not in skip:
        # launch autotuner (tuning.py): a few timed steps per candidate, cached by grid and batch shape
        import tuning
        tune = tuning.autotune(eng, shots, vstart, cache=tuning.DEFAULT_CACHE if rank == 0 else None)
    eng.set_model(vtrue)
    obs = eng.forward()                      # observed traces from the true model (setup, untimed)
    eng.set_observed(obs)
    eng.set_model(vstart)
    cells = float(cfgkw["nx"] * cfgkw["nz"])
    step_cells = sum(s.nt for s in shots) * cells          # physical cell-steps of one propagation pass

    def barrier():
        torch.cuda.synchronize()
        if dist:
            dist.barrier()

    grad_t = mis_t = None
    if dist:
        # the gradient lives in the engine; the ranks sum their shot shares in FP64
        import shots_parallel
        grad_t = shots_parallel.device_tensor(eng.grad_device_ptr(), int(cells), f"cuda:{local}")
        mis_t = torch.zeros(2, dtype=torch.float64, device=f"cuda:{local}")

    def step():
        J, _ = eng.gradient(keep_on_device=True)
        if dist:
            with torch.cuda.stream(stream):
                mis_t.fill_(J)
                shots_parallel.allreduce_gradient(grad_t, mis_t)
        return J

    for _ in range(max(3, args.warmup)):
        step()
    barrier()
    clk = Clocks(local)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    fwd_ms = bwd_ms = 0.0
    launches = 0
    for _ in range(args.steps):
        step()
        st = eng.stats()
        fwd_ms += st["ms_forward"]
        bwd_ms += st["ms_backward"]
        launches += st["launches"]
    e1.record(stream)
    barrier()
    clocks = clk.stop()
    ms = e0.elapsed_time(e1) / args.steps
    if dist:
        t = torch.tensor([ms], device=f"cuda:{local}")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    value = world * nshots / (ms / 1e3)
    gcell = world * 3.0 * step_cells / (ms / 1e3) / 1e9

    # roofline of the dominant kernel (fused backward step), per launch
    nt_max = max(s.nt for s in shots)
    bwd_launch_ms = bwd_ms / args.steps / nt_max
    bwd_bytes_launch = BWD_BYTES * step_cells / nt_max                   # average over launches
    peak, peak_kind = peaks()
    achieved = bwd_bytes_launch / (bwd_launch_ms / 1e3) / 1e9
    tpc = traffic_per_cell_step("k_backward")
    roof = {"kernel": "k_backward", "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "peak_kind": peak_kind,
            "traffic": (tpc * step_cells / nt_max) if tpc else None,
            "algorithmic_bytes_per_launch": bwd_bytes_launch, "avg_launch_ms": bwd_launch_ms,
            "forward_avg_launch_ms": fwd_ms / args.steps / nt_max,
            "forward_achieved_gbs": FWD_BYTES * step_cells / nt_max / (fwd_ms / args.steps / nt_max / 1e3) / 1e9}

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": max(3, args.warmup), "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": describe(args, cfgkw, shots, eng.stats()),
            "gcell_steps_per_s": gcell,
            "tuning": None if tune is None else {
                "chosen": tune["tuning"], "ms_step": tune["ms_step"], "default_ms_step": tune["default_ms_step"],
                "trials": len(tune.get("trials", [])), "cached": tune["cached"],
                "note": "fwd + bwd ms per time step of fwi_time_steps, before the timed region"}, "gpu_launches": launches, "clocks": clocks, "roofline": roof}

    # end to end through the C ABI with pinned host buffers: every step uploads the
    # model and the observed traces and reads back the misfit and the (reduced) gradient;
    # fwi_gradient_obs uploads the traces on a copy stream beside the forward phase
    if "e2e" not in skip:
        v_h = torch.empty(vstart.shape, dtype=torch.float32, pin_memory=True).numpy()
        v_h[:] = vstart
        o_h = torch.empty(obs.shape, dtype=torch.float32, pin_memory=True).numpy()
        o_h[:] = obs
        g_pin = torch.empty(vstart.shape, dtype=torch.float64, pin_memory=True)
        g_h = g_pin.numpy()

        def e2e_step():
            eng.set_model(v_h)
            if not dist:
                return eng.gradient(out=g_h, observed=o_h)[0]
            J, _ = eng.gradient(keep_on_device=True, observed=o_h)
            with torch.cuda.stream(stream):
                mis_t.fill_(J)
                shots_parallel.allreduce_gradient(grad_t, mis_t)
                g_pin.view(-1).copy_(grad_t, non_blocking=True)
            return mis_t
        for _ in range(max(3, args.warmup)):
            e2e_step()
        barrier()
        clk2 = Clocks(local)
        t_wall = time.perf_counter()
        e0.record(stream)
        for _ in range(args.steps):
            e2e_step()
        e1.record(stream)
        barrier()
        wall2 = (time.perf_counter() - t_wall) * 1e3 / args.steps
        clocks2 = clk2.stop()
        ms2 = e0.elapsed_time(e1) / args.steps
        if dist:
            t = torch.tensor([ms2], device=f"cuda:{local}")
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            ms2 = float(t.item())
        line["e2e"] = {"value": world * nshots / (ms2 / 1e3), "unit": UNIT, "ms_per_step": ms2, "steps": args.steps,
                       "wall_ms_per_step": wall2, "clocks": clocks2, "calls": "fwi_set_model, fwi_gradient_obs",
                       "h2d_bytes_per_step": int(v_h.nbytes + o_h.nbytes), "d2h_bytes_per_step": int(g_h.nbytes + 16)}

    # plain per-shot path (one shot per launch, shots one after another)
    if "plain" not in skip and rank == 0:
        k = min(args.plain_shots, nshots)
        pcfg = fwigpu.make_config(**dict(cfgkw, nt_max=max(s.nt for s in shots[:k])), device=local,
                                  use_graph=0, plain_per_shot=1)
        with fwigpu.Engine(pcfg) as pe:
            pe.set_stream(stream.cuda_stream)
            pe.set_shots(shots[:k])
            pe.set_model(vstart)
            pe.set_observed(obs[:pe.nsamples])
            pe.gradient(keep_on_device=True)
            e0.record(stream)
            pe.gradient(keep_on_device=True)
            e1.record(stream)
            barrier()
            pms = e0.elapsed_time(e1)
        line["plain"] = {"shots": k, "value": k / (pms / 1e3), "unit": UNIT,
                         "batched_over_plain": value / world / (k / (pms / 1e3))}

    # checkpointed runs: the same gradient with the strip ring, at full size, on the GPU
    if eng.stats()["store"] == fwigpu.STORE_SNAPSHOTS and "strips" not in skip and rank == 0:
        import numpy as np
        J_c, g_c = eng.gradient()
        eng.close()
        with fwigpu.Engine(fwigpu.make_config(**cfgkw, device=local, use_graph=1, store=fwigpu.STORE_STRIPS,
                                              fd_order=args.fd_order)) as se:
            se.set_stream(stream.cuda_stream)
            se.set_shots(shots)
            se.set_model(vstart)
            se.set_observed(obs)
            J_s, g_s = se.gradient()
        line["vs_strips"] = {"grad_rel_diff": float(np.linalg.norm(g_c - g_s) / np.linalg.norm(g_s)),
                             "misfit_equal": bool(J_c == J_s),
                             "note": "the strip ring's gradient is within 5e-6 of the FP64 oracle on the "
                                     "560 x 1700 workload"}

    # CPU baseline (the reference's own kernels, or their restatement) and the accuracy check
    if "cpu" not in skip and rank == 0 and world == 1:
        def gpu_grad(nt, obs_sample):
            s0 = shots[0]
            sh = fwigpu.ShotSpec(s0.src_x, s0.src_z, s0.rec_xz, s0.wavelet[:nt])
            c1 = fwigpu.make_config(**dict(cfgkw, nt_max=nt), device=local)
            with fwigpu.Engine(c1) as e1_:
                e1_.set_shots([sh])
                e1_.set_model(vstart)
                e1_.set_observed(obs_sample)
                return e1_.gradient()[1]
        kind = cpu_kind()
        r = cpu_sample(args, cfgkw, vstart, vtrue, shots[:max(1, min(args.cpu_shots, nshots))], args.cpu_steps,
                       kind, check_gpu=gpu_grad)
        sec_shot = r["sec"] / r["shots"] * shots[0].nt / r["nt"]
        line["cpu_baseline"] = {"value": 1.0 / sec_shot, "unit": UNIT, "cores": r["cores"], "kind": kind,
                                "sample": f"{r['shots']} shot(s) in one gradient, {r['nt']} of {shots[0].nt} steps, "
                                          f"FP32, {r['sec']:.2f} s" +
                                          ("" if r["nt"] == shots[0].nt else ", scaled linearly in steps")}
        line["accuracy"] = {"grad_rel_err_vs_fp64": r["grad_rel_err"],
                            "cpu_fp32_grad_rel_err_vs_fp64": r["grad_rel_err_cpu_fp32"],
                            "sample": f"1 shot, {r['nt']} steps, workload grid"}
    if rank == 0 and world == 1 and "aux" not in skip:
        try:
            line["aux"] = aux_leg(local)
        except Exception as e:
            line["aux"] = {"error": f"{type(e).__name__}: {e}"}
    # the uneven-batch configuration beside the default one (single GPU only)
    if args.workload == "c2" and world == 1 and "c3" not in skip:
        eng.close()
        try:
            line["c3"] = extra_leg("c3", args, local, stream)
        except Exception as e:                                  # the main line stands on its own
            line["c3"] = {"error": f"{type(e).__name__}: {e}"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    eng.close()     # idempotent
    if dist:
        dist.destroy_process_group()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
