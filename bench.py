#!/usr/bin/env python
"""Benchmark of the two-fluid ghost-fluid Euler step on GB300.

Workload: the 1000x400 shock-bubble (light gas gamma=1.648, rho=0.182 bubble
of radius 0.025 at (0.175, 0.0445) in air; Mach 1.22 shock from x=0.225;
reflective top/bottom, transmissive ends), Riemann GFM with the HOUC5 level
set, MUSCL-Hancock + exact Riemann fluxes, CFL 0.6, FP64.  One step is one
iteration of the reference's time loop (sourcecode/sim_twofluid.cpp:64-88):
CFL dt, ghost fill, both flux updates, level set, BCs.  Metric: cell-updates
per second (real cells x steps / device time).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gfm|reference]

Timed region: W untimed steps from the initial condition, then K steps, each
timed with CUDA events on the library's stream, with a 512 MiB write between
steps to flush the 129 MB L2.  Multi-GPU: independent replicas per rank
(torchrun), barrier + max over ranks.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "phd-2d-gfm_gb300"))

# The configurations this metric is quoted on (the default is the headline one).
WORKLOADS = {
    "shock_bubble": {"workload": "shock_bubble_1000x400_riemannGFM_MUSCL_LS5", "sim": "twofluid",
                     "test_case": "shock_bubble", "Nx": 1000, "Ny": 400, "GFM": "riemannGFM", "FS": "MUSCL",
                     "ITM": "LS5", "CFL": 0.6, "reinit_every": 1, "run_steps": 2000},
    "underwater_explosion": {"workload": "underwater_explosion_800x800_realGFM_MUSCL_LS5", "sim": "twofluid",
                             "test_case": "underwater_explosion_sg", "Nx": 800, "Ny": 800, "GFM": "realGFM",
                             "FS": "MUSCL", "ITM": "LS5", "CFL": 0.5, "reinit_every": 5, "run_steps": 1500},
    # the same flow with the VOF tracker and GFM_VOF (a workload of the VOF
    # ghost-fluid methods, not the headline configuration)
    "shock_bubble_vof": {"workload": "shock_bubble_1000x400_VOFGFM_MUSCL_PYVOF", "sim": "twofluid",
                         "test_case": "shock_bubble", "Nx": 1000, "Ny": 400, "GFM": "VOFGFM", "FS": "MUSCL",
                         "ITM": "PYVOF", "CFL": 0.6, "reinit_every": 0, "run_steps": 2000},
    # CFL 0.4 as in the reference's settings files: at 0.8 the unsplit
    # MUSCL-Hancock update diverges at step 23 (oracle and GPU alike)
    "circular_explosion": {"workload": "circular_explosion_200x200_onefluid_MUSCL_CFL0.4", "sim": "onefluid",
                           "test_case": "circularexplosion", "Nx": 200, "Ny": 200, "GFM": None, "FS": "MUSCL",
                           "ITM": None, "CFL": 0.4, "reinit_every": 0, "run_steps": 132},
}
METRIC = "cell-updates/s/GB300 FP64: plain vs batched+learned p* guess at L1 err<=1e-10"
UNIT = "cell-updates/s"
FLUX_BYTES_PER_CELL = 128   # flux update, both fluids: 32 B read + 32 B write of U each
STEP_BYTES_PER_CELL = 144   # whole step: the flux update's 128 B plus phi read and write
NPHASES = 9
PHASE_NAMES = ["cfl", "ghost_fill", "flux_update", "commit_bcs_and_level_set_join", "end_step", "interface_loop",
               "far_partition",
               "near_extrapolation", "far_flux_update"]


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--workload", default="shock_bubble", choices=sorted(WORKLOADS) + ["batch64"])
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gfm", choices=["gfm", "reference"])
    ap.add_argument("--e2e-steps", type=int, default=-1,
                    help="steps of the end-to-end leg (default: the same steps as the timed region)")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--overlap", default="auto", choices=["auto", "on", "off"],
                    help="ghost-fill schedule (gfm_set_overlap); results are identical")
    ap.add_argument("--no-batched-learned", dest="batched_learned", action="store_false",
                    help="skip the batched / learned-proposal block of the default line")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(x, device):
    """The largest of the ranks' values (the slowest replica sets the job's time)."""
    import torch
    import torch.distributed as tdist
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    tdist.all_reduce(t, op=tdist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(cells, steps, world, step_ms_max):
    """Whole-job cell-updates/s of `world` independent replicas of the same
    workload, timed by the slowest one (weak scaling)."""
    return cells * steps * world / (step_ms_max * 1e-3)


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


def ncu_summary(workload):
    """Figures of the committed ncu summary of the flux update on `workload`
    (key=value lines): DRAM bytes per full-grid launch, FP64 flops per cell,
    FP64 pipe activity, the step the captured launch belongs to."""
    p = os.path.join(ROOT, "profiles", "flux_update_%s.txt" % workload)
    out = {}
    if not os.path.exists(p):
        return out
    for line in open(p):
        if "=" not in line or line.startswith("#"):
            continue
        k, v = line.split("=", 1)
        try:
            out[k.strip()] = float(v.split()[0])
        except (IndexError, ValueError):
            pass
    return out


def step_summary(workload):
    """key=value lines of the committed whole-step ncu summary on `workload`."""
    p = os.path.join(ROOT, "profiles", "step_fp64_%s.md" % workload)
    out = {}
    if not os.path.exists(p):
        return out
    for line in open(p):
        k, _, v = line.partition("=")
        if not v or not k.strip().isidentifier() or line.startswith((" ", "|")):
            continue
        try:
            out[k.strip()] = float(v.split()[0])
        except (IndexError, ValueError):
            pass
    return out


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.proc = None
        self.path = os.path.join("/tmp", "gfm_clocks_%d_%d.csv" % (os.getpid(), gpu_index))

    def __enter__(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if not self.proc or not os.path.exists(self.path):
            return None
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
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def tiles_from_report(tuning, descs):
    """The flux tile gfm_batch_autotune's report gives each grid: that of its
    grid-size class, the class with the smallest bound (max_padded_cells, -1:
    none) above the grid's padded cell count; None where no class fits."""
    classes = sorted((c["max_padded_cells"] if c["max_padded_cells"] > 0 else float("inf"), c["tile"])
                     for c in tuning.get("classes", []))
    out = []
    for d in descs:
        padded = (d.Nx + 2 * d.numGC) * (d.Ny + 2 * d.numGC)
        fits = [t for bound, t in classes if padded < bound]
        out.append(fits[0] if fits else None)
    return out


def setup(W):
    import gfm_gb300 as g
    desc, T = g.case_params(W["sim"], W["test_case"], W["Nx"], W["Ny"])
    U1, U2, phi = g.case_init(W["sim"], W["test_case"], desc)
    if W.get("ITM") == "PYVOF":   # the VOF tracker's field is the volume fraction
        phi = g.case_init_z(W["test_case"], desc)
    if W["sim"] == "twofluid":
        m = g.method(fs=W["FS"], gfm=W["GFM"], itm=W["ITM"], CFL=W["CFL"], T=T, reinit_every=W["reinit_every"])
    else:
        m = g.method(fs=W["FS"], CFL=W["CFL"], T=T)
    return desc, T, U1, U2, phi, m


def run_gfm(args):
    import ctypes
    import numpy as np
    import torch
    import gfm_gb300 as g

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as tdist
        tdist.init_process_group("nccl", device_id=torch.device("cuda", local))
    W = WORKLOADS[args.workload]
    two = W["sim"] == "twofluid"
    desc, T, U1, U2, phi, m = setup(W)
    # a run shorter than warm-up + steps (the circular explosion ends at T after
    # 132 steps) is timed over the steps it has
    args.steps = max(1, min(args.steps, W["run_steps"] - args.warmup))
    stream = torch.cuda.current_stream()
    ctx = g.Context(desc, two_fluid=two, stream=stream.cuda_stream)
    ctx.upload(U1, U2, phi)
    if two and not ctx.set_overlap(args.overlap):   # no SM partitions: one stream
        ctx.set_overlap("off")
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    ctx.step(m, args.warmup)
    torch.cuda.synchronize()
    ctx.clear_status()
    e2e_start = ctx.download() + ctx.time()[:2]
    cells = desc.Nx * desc.Ny
    phases = np.zeros(NPHASES)
    ph = np.zeros(NPHASES)
    L = g.lib()
    prof = ncu_summary(args.workload)
    prof_step = int(prof.get("profiled_step", -1))
    flux_ms_prof = None
    step_prof = step_summary(args.workload)
    step_ms_prof = None
    launches0 = L.gfm_launch_count()
    if world > 1:
        import torch.distributed as tdist
        tdist.barrier()
    torch.cuda.synchronize()
    t_wall = time.time()
    with ClockSampler(local) as clk:
        for s in range(args.steps):
            flush.zero_()
            ph[:] = 0.0
            rc = L.gfm_step_timed(ctx._p, ctypes.byref(m), 1, ph.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
            if rc != 0:
                raise RuntimeError("gfm_step_timed failed: %d" % rc)
            phases += ph
            if args.warmup + s == prof_step:   # the step of the profiled launch
                flux_ms_prof = ph[2] + ph[8]
            if args.warmup + s == int(step_prof.get("profiled_step", -1)):
                step_ms_prof = float(ph[:5].sum())
        torch.cuda.synchronize()
    wall = time.time() - t_wall
    launches = L.gfm_launch_count() - launches0
    step_ms = float(phases[:5].sum())   # phases 5-8 are sub-intervals of 1-2
    if world > 1:
        import torch.distributed as tdist
        step_ms = max_over_ranks(step_ms, "cuda")
        tdist.barrier()
    status = ctx.status()
    stats = ctx.stats()
    t_sim, nsteps_done, _ = ctx.time()
    value = replica_throughput(cells, args.steps, world, step_ms)

    # roofline of the dominant kernel, the flux update (both fluids per
    # launch; with the overlapped schedule two launches per step, far tiles
    # and near tiles, cover the grid once: their times are added)
    flux_ms = (phases[2] + phases[8]) / args.steps
    achieved = FLUX_BYTES_PER_CELL * cells / (flux_ms * 1e-3) / 1e9
    peak, peak_kind = peaks()
    fp64_peak = ctypes.c_double(0.0)
    L.gfm_fp64_peak(ctypes.byref(fp64_peak), ctypes.c_void_p(stream.cuda_stream))
    fp64 = {"kernel": "k_flux_update<MUSCL>", "peak_gflops": round(fp64_peak.value, 1),
            "peak_source": "measured now (gfm_fp64_peak: FMA loop on every SM)"}
    if "fp64_flops_per_cell" in prof and flux_ms_prof:
        # the flop count of the profiled launch over that same step's flux
        # time, measured here with CUDA events (the count varies along the run)
        fl = prof["fp64_flops_per_cell"] * cells
        fp64.update({"flops_per_cell": prof["fp64_flops_per_cell"], "step": prof_step,
                     "kernel_ms_at_step": round(flux_ms_prof, 5),
                     "achieved_gflops": round(fl / (flux_ms_prof * 1e-3) / 1e9, 1),
                     "frac": round(fl / (flux_ms_prof * 1e-3) / 1e9 / fp64_peak.value, 4),
                     "pipe_active_frac_ncu": prof.get("fp64_pipe_active_frac")})
        if "fp64_lane_instructions_per_cell" in prof:
            # an FP64 add or multiply holds the pipe as long as a fused
            # multiply-add: the pipe's share is the lane-instruction rate over
            # the peak's (the FMA loop's flop rate / 2)
            li = prof["fp64_lane_instructions_per_cell"] * cells / (flux_ms_prof * 1e-3) / 1e9
            fp64.update({"lane_instructions_per_cell": prof["fp64_lane_instructions_per_cell"],
                         "achieved_g_lane_inst": round(li, 1), "peak_g_lane_inst": round(fp64_peak.value / 2, 1),
                         "pipe_frac": round(li / (fp64_peak.value / 2), 4)})
    if "fp64_flops_per_cell_step" in step_prof and step_ms_prof:
        # the whole step's FP64 work (ncu, all kernels of one step) over that
        # step's time measured here
        fs_ = step_prof["fp64_flops_per_cell_step"] * cells / (step_ms_prof * 1e-3) / 1e9
        fp64["step"] = {"flops_per_cell": step_prof["fp64_flops_per_cell_step"],
                        "step": int(step_prof["profiled_step"]), "ms_at_step": round(step_ms_prof, 5),
                        "achieved_gflops": round(fs_, 1), "frac": round(fs_ / fp64_peak.value, 4)}
    roof = {"bound": "hbm", "achieved": round(achieved, 2), "peak": peak, "unit": "GB/s",
            "frac": round(achieved / peak, 5), "traffic": prof.get("traffic_bytes_per_launch_full_size"),
            "kernel": "k_flux_update<MUSCL>", "peak_source": peak_kind, "bytes_per_cell": FLUX_BYTES_PER_CELL,
            "kernel_ms_per_step": round(flux_ms, 5),
            "step_achieved_gbs": round(STEP_BYTES_PER_CELL * value / 1e9, 2),
            "fp64": fp64,
            "phase_ms_per_step": {n: round(v / args.steps, 5) for n, v in zip(PHASE_NAMES, phases)}}

    # end to end through the C ABI: pinned host state -> device -> step -> host
    e2e = None
    if args.e2e_steps != 0:
        # the same steps again from the pre-timing state (a one-fluid run that
        # reached T would do nothing more)
        shp = desc.shape
        hU1 = torch.empty((4,) + shp, dtype=torch.float64, pin_memory=True).numpy()
        hU2 = torch.empty((4,) + shp, dtype=torch.float64, pin_memory=True).numpy()
        hphi = torch.empty(shp, dtype=torch.float64, pin_memory=True).numpy()
        hU1[...] = e2e_start[0]
        if two:
            hU2[...] = e2e_start[1]
            hphi[...] = e2e_start[2]
        L.gfm_set_time(ctx._p, e2e_start[3], e2e_start[4])
        pd = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))  # noqa: E731
        n_e2e = args.steps if args.e2e_steps < 0 else min(args.e2e_steps, args.steps)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        up = (pd(hU1), pd(hU2), pd(hphi)) if two else (pd(hU1), None, None)
        for s in range(n_e2e):
            # the whole state in and out through the C ABI every step (the
            # upload is ordered before the step on the context's stream; the
            # download synchronises)
            L.gfm_upload_state_async(ctx._p, *up)
            L.gfm_step(ctx._p, ctypes.byref(m), 1)
            L.gfm_download_state(ctx._p, *up)
        torch.cuda.synchronize()
        e2e_s = time.perf_counter() - t0
        args.e2e_steps = n_e2e
        nbytes = hU1.nbytes + ((hU2.nbytes + hphi.nbytes) if two else 0)
        e2e = {"value": cells * args.e2e_steps * world / e2e_s, "unit": UNIT, "h2d_bytes_per_step": nbytes,
               "d2h_bytes_per_step": nbytes, "steps": args.e2e_steps}

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": step_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": W["workload"], "Nx": desc.Nx, "Ny": desc.Ny, "GFM": W["GFM"],
                       "FS": W["FS"], "ITM": W["ITM"], "CFL": W["CFL"], "parallelism": "replicas%d" % world,
                       "l2": "512 MiB flush between timed steps", "steps_from": args.warmup,
                       "schedule": "overlap " + args.overlap, "p_star_guess": "plain (PVRS / TSRS)"},
            "roofline": roof, "e2e": e2e, "gpu_launches": int(launches),
            "clocks": clk.summary(), "device_status": g.status_names(status),
            "stats_last_step": stats, "sim_time": t_sim, "wall_s": wall}
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(W, desc, m, e2e_start, args.cpu_seconds)
    ctx.close()
    if rank == 0 and world == 1 and args.batched_learned:
        line["batched_learned"] = batched_learned_block(args)
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        import torch.distributed as tdist
        tdist.destroy_process_group()


def _oracle_steps(desc_fields, m_fields, U1, U2, phi, nsteps, t, numsteps, seconds):
    """One oracle process: step until `seconds` elapse (at least one step)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle_binding as orc
    import gfm_gb300 as g
    desc = g.GridDesc(**desc_fields)
    m = g.MethodDesc(**m_fields)
    done = 0
    t0 = time.perf_counter()
    while done < nsteps:
        if U2 is None:   # one fluid
            U1, t, numsteps, taken = orc.onefluid_run(desc, m, U1, 1, t, numsteps)
            if taken == 0:   # reached T
                break
        else:
            r = orc.twofluid_run(desc, m, U1, U2, phi, 1, t, numsteps)
            U1, U2, phi, t, numsteps = r["U1"], r["U2"], r["phi"], r["t"], r["numsteps"]
        done += 1
        if time.perf_counter() - t0 > seconds:
            break
    return done, time.perf_counter() - t0


def _fields(s):
    return {k: getattr(s, k) for k, _ in s._fields_}


def cpu_baseline(W, desc, m, start, seconds):
    """The CPU oracle (single-threaded, like the reference) timed on this host on
    a bounded sample: oracle steps of the same workload from the GPU's state
    after the warm-up (the first timed step)."""
    U1, U2, phi, t, n = start
    done, el = _oracle_steps(_fields(desc), _fields(m), U1, U2, phi, 10 ** 6, t, n, seconds)
    cells = desc.Nx * desc.Ny
    return {"value": cells * done / el, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": "%d oracle steps of %s from the state after %d steps (%.1f s)"
                      % (done, W["workload"], n, el)}


def setup_oracle(W):
    """The workload's initial state from the oracle's own restatement of its
    initial conditions: the reference arm loads nothing of the library."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle_binding as orc
    import gfm_gb300 as g   # the C-ABI struct layouts and method table only: no library is loaded
    desc, T, U1, U2, phi = orc.case_setup(W["sim"], W["test_case"], W["Nx"], W["Ny"])
    if W["sim"] == "twofluid":
        m = g.method(fs=W["FS"], gfm=W["GFM"], itm=W["ITM"], CFL=W["CFL"], T=T, reinit_every=W["reinit_every"])
    else:
        m = g.method(fs=W["FS"], CFL=W["CFL"], T=T)
    return desc, T, U1, U2, phi, m


def run_reference(args):
    """--impl reference: the CPU oracle on this host's cores, one independent
    run per core, aggregate.  The oracle is pinned bit for bit to the
    reference's own code (tests/test_oracle_vs_reference.py), which cannot be
    built on this host (its external libraries are absent; the checker that
    compiles its sources against the oracle's stand-ins is x86 test
    infrastructure).  Nothing of the GPU library is loaded here."""
    rank, world, local = dist_env()
    if rank != 0:
        return
    import multiprocessing as mp
    if args.workload == "batch64":
        return run_reference_batch(args)
    W = WORKLOADS[args.workload]
    desc, T, U1, U2, phi, m = setup_oracle(W)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle_binding as orc
    if W["sim"] == "twofluid":
        r = orc.twofluid_run(desc, m, U1, U2, phi, args.warmup)
        start = (r["U1"], r["U2"], r["phi"], r["t"], r["numsteps"])
    else:
        U, t, n, _ = orc.onefluid_run(desc, m, U1, args.warmup)
        start = (U, None, None, t, n)
    cores = os.cpu_count() or 1
    budget = 60.0
    ctxm = mp.get_context("spawn")
    with ctxm.Pool(cores) as pool:
        t0 = time.perf_counter()
        res = pool.starmap(_oracle_steps, [(_fields(desc), _fields(m), start[0], start[1], start[2], args.steps,
                                            start[3], start[4], budget)] * cores)
        wall = time.perf_counter() - t0
    total_steps = sum(d for d, _ in res)
    cells = desc.Nx * desc.Ny
    # the processes step side by side: their aggregate rate is the cell-updates
    # over the longest process's own stepping time (the state's transfer to
    # the processes and their start are not the reference's work)
    value = cells * total_steps / max(max(el for _, el in res), 1e-9)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": wall * 1e3 / max(1, total_steps / cores),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "impl": "reference",
            "config": {"workload": W["workload"], "Nx": desc.Nx, "Ny": desc.Ny, "GFM": W["GFM"], "FS": W["FS"],
                       "ITM": W["ITM"], "CFL": W["CFL"], "parallelism": "%d independent CPU runs" % cores},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": "%d independent oracle runs x up to %d steps from step %d, %.0f s budget; "
                                       "rate over the longest run's own stepping time" % (cores, args.steps, args.warmup,
                                                                                          budget)},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def _oracle_member(spec, nsteps, seconds):
    """One oracle process on one batch member from its initial state (the
    oracle's own initial conditions; nothing of the GPU library)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle_binding as orc
    import gfm_gb300 as g   # struct layouts and method table only: no library is loaded
    d, T, U1, U2, phi = orc.bubble_setup(*spec)
    m = g.method(gfm="riemannGFM", CFL=0.6, T=1.0)
    done, el = _oracle_steps(_fields(d), _fields(m), U1, U2, phi, nsteps, 0.0, 0, seconds)
    return d.Nx * d.Ny * done, el


def run_reference_batch(args):
    """--impl reference for the batched workload: the oracle on every host
    core, each core stepping batch members (members spread over the cores)."""
    import multiprocessing as mp
    spec = batch_members()
    cores = os.cpu_count() or 1
    budget = 60.0
    per = max(1.0, budget * cores / len(spec))
    ctxm = mp.get_context("spawn")
    with ctxm.Pool(cores) as pool:
        t0 = time.perf_counter()
        res = pool.starmap(_oracle_member, [(sp, args.steps, per) for sp in spec])
        wall = time.perf_counter() - t0
    value = sum(c for c, _ in res) / wall
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": {"workload": "batch64_shock_bubble_riemannGFM", "instances": len(spec), "seed": BATCH_SEED,
                       "parallelism": "%d CPU processes over the members" % cores},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": "each of %d members stepped by the oracle for up to %.1f s from its initial "
                                       "state (at most %d steps), %d processes" % (len(spec), per, args.steps, cores)},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


BATCH_SEED = 0x6F4D


def batch_members(n=64, seed=BATCH_SEED):
    """The batched workload: n shock-bubble instances, sides 128..1024 in steps
    of 64, aspect ratio U[1,3] (Ny = max(128, Nx/aspect rounded to 64)), Mach
    U[1.1,3], bubble gamma U[1.09,1.67], density ratio log-U[0.1,10], radius
    U[0.1,0.3] of the height."""
    import numpy as np
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        nx = int(rng.integers(2, 17)) * 64
        aspect = rng.uniform(1.0, 3.0)
        ny = max(128, int(round(nx / aspect / 64.0)) * 64)
        out.append((nx, ny, rng.uniform(1.1, 3.0), rng.uniform(1.09, 1.67), float(np.exp(rng.uniform(np.log(0.1),
                    np.log(10.0)))), rng.uniform(0.1, 0.3)))
    return out


def batched_learned_block(args):
    """The metric's second half on the batched workload: the 64 instances of
    the seeded shock-bubble family stepped (1) one after another with the
    plain guess, (2) together through the recorded step graph with the plain
    guess, and (3) together with the learned star-pressure proposal (weights
    from phd-2d-gfm_gb300/data/pstar_mlp.f32, trained by train_pstar.py),
    each for the same steps from the same state after the warm-up; the
    Newton iterations per interface solve of (2) and (3) and the largest
    relative L1 difference of their end fields (real cells, per field)."""
    import numpy as np
    import torch
    import gfm_gb300 as g
    import train_pstar
    K = max(1, min(args.steps, 20))
    spec = batch_members()
    cases = [g.shock_bubble_case(*p) for p in spec]
    m = g.method(gfm="riemannGFM", CFL=0.6, T=1.0)
    mlp = train_pstar.load()
    weights = "phd-2d-gfm_gb300/data/pstar_mlp.f32 (train_pstar.py)"
    if mlp is None:   # no saved weights: a short training run here
        n = 1 << 20
        X = torch.empty((n, 10), dtype=torch.float32, device="cuda")
        Y = torch.empty(n, dtype=torch.float32, device="cuda")
        got = g.mlp_generate(21, n, X.data_ptr(), Y.data_ptr())
        mlp = g.MLP(seed=5)
        mlp.train(X.data_ptr(), Y.data_ptr(), got, epochs=10, batch=4096, lr=2e-3)
        weights = "trained in this run (%d synthetic problems, 10 epochs)" % got
    descs = [c[0] for c in cases]
    bp = g.Batch(descs, two_fluid=True)
    bl = g.Batch(descs, two_fluid=True)
    for ctx in bl.instances:
        ctx.set_mlp(mlp)
    for ctx, (d, T, U1, U2, phi) in zip(bp.instances, cases):
        ctx.upload(U1, U2, phi)
    bp.step(m, args.warmup, graph=True)
    bp.synchronize()
    start = [ctx.download() + ctx.time()[:2] for ctx in bp.instances]
    cells = sum(d.Nx * d.Ny for d in descs)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def timed(b, graph):
        if graph:
            # the graph (8 steps per replay) recorded outside the timed region
            for ctx, st in zip(b.instances, start):
                ctx.upload(st[0], st[1], st[2], t=st[3], numsteps=st[4])
            b.step(m, 8, graph=True)
            b.synchronize()
        for ctx, st in zip(b.instances, start):
            ctx.upload(st[0], st[1], st[2], t=st[3], numsteps=st[4])
        torch.cuda.synchronize()
        flush.zero_()
        stream = torch.cuda.current_stream()
        import ctypes
        g.lib().gfm_batch_set_stream(b._p, ctypes.c_void_p(stream.cuda_stream))
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        b.step(m, K, graph=graph)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        tot = [ctx.interface_totals() for ctx in b.instances]
        solves = sum(x["solves"] for x in tot)
        iters = sum(x["newton_iters"] for x in tot)
        return {"value": cells * K / (ms * 1e-3), "ms_per_step": ms / K, "interface_solves": solves,
                "newton_per_interface_solve": iters / max(1, solves),
                "from_proposal": sum(x["proposed"] for x in tot),
                "device_status_nonzero": int(sum(1 for ctx in b.instances if ctx.status()))}

    seq = timed(bp, False)
    plain = timed(bp, True)
    outp = [ctx.download() for ctx in bp.instances]
    learned = timed(bl, True)
    outl = [ctx.download() for ctx in bl.instances]
    # the project's autotuner: flux tile shape per grid-size class and the
    # schedule (per-instance streams, or one persistent flux launch over all
    # instances per step), timed on the batch's state; then the tuned run
    for ctx, st in zip(bp.instances, start):
        ctx.upload(st[0], st[1], st[2], t=st[3], numsteps=st[4])
    tuning = bp.autotune(m, steps=16)
    tuned = timed(bp, True)
    outt = [ctx.download() for ctx in bp.instances]
    # the learned batch with the tuner's tiles (each instance takes the tile
    # of its grid-size class: the class with the smallest bound above its
    # padded cell count)
    learned_tuned = None
    if tuning.get("tiles") == "per class":
        for ctx, tile in zip(bl.instances, tiles_from_report(tuning, descs)):
            if tile:
                ctx.set_flux_tile(tile)
        learned_tuned = timed(bl, True)
    tuned_identical = all(np.array_equal(a, b) for a3, b3 in zip(outt, outp) for a, b in zip(a3, b3))
    rel = 0.0
    identical = True
    for (d, *_), a3, b3 in zip(cases, outl, outp):
        gc = d.numGC
        for a, b in zip(a3, b3):
            ra, rb = a[..., gc:-gc, gc:-gc], b[..., gc:-gc, gc:-gc]
            rel = max(rel, float(np.abs(ra - rb).sum() / max(np.abs(rb).sum(), 1e-300)))
            identical = identical and np.array_equal(a, b)
    bp.close()
    bl.close()
    mlp.close()
    return {"workload": "batch64_shock_bubble_riemannGFM", "instances": len(spec), "cells": cells, "steps": K,
            "warmup": args.warmup, "seed": BATCH_SEED, "weights": weights,
            "plain_sequential": seq, "batched_plain": plain, "batched_learned": learned,
            "autotune": tuning, "batched_tuned": tuned, "tuned_bit_identical_to_plain": tuned_identical,
            "batched_learned_tuned": learned_tuned,
            "batched_learned_tuned_over_plain_sequential": (learned_tuned["value"] / seq["value"]
                                                            if learned_tuned else None),
            "batched_tuned_over_plain_sequential": tuned["value"] / seq["value"],
            "batched_learned_over_plain_sequential": learned["value"] / seq["value"],
            "batched_plain_over_plain_sequential": plain["value"] / seq["value"],
            "max_rel_l1_learned_vs_plain": rel, "learned_bit_identical_to_plain": identical,
            "l2": "inputs larger than L2 (%.1f GB of state); 512 MiB flush before each timed run"
                  % (cells * 9 * 8 / 1e9)}


def run_batch(args):
    """64 independent shock-bubble instances: K steps of all of them one
    instance after another (the unbatched path), through the recorded step
    graph with the default schedule, and -- the line's value -- through the
    graph after gfm_batch_autotune has chosen the schedule and the flux tile
    shape per grid-size class, each from the same state."""
    import ctypes
    import numpy as np
    import torch
    import gfm_gb300 as g
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    spec = batch_members()
    cases = [g.shock_bubble_case(*p) for p in spec]
    m = g.method(gfm="riemannGFM", CFL=0.6, T=1.0)
    b = g.Batch([c[0] for c in cases], two_fluid=True)
    for ctx, (d, T, U1, U2, phi) in zip(b.instances, cases):
        ctx.upload(U1, U2, phi)
    b.step(m, args.warmup, graph=True)
    b.synchronize()
    start = [ctx.download() + ctx.time()[:2] for ctx in b.instances]
    cells = sum(c[0].Nx * c[0].Ny for c in cases)
    L = g.lib()
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()
    L.gfm_batch_set_stream(b._p, ctypes.c_void_p(stream.cuda_stream))

    def timed(graph):
        if graph:
            # the graph (8 steps per replay) recorded outside the timed region
            for ctx, st in zip(b.instances, start):
                ctx.upload(st[0], st[1], st[2], t=st[3], numsteps=st[4])
            b.step(m, 8, graph=True)
            b.synchronize()
        for ctx, st in zip(b.instances, start):
            ctx.upload(st[0], st[1], st[2], t=st[3], numsteps=st[4])
        torch.cuda.synchronize()
        flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        l0 = L.gfm_launch_count()
        with ClockSampler(local) as clk:
            e0.record(stream)
            b.step(m, args.steps, graph=graph)
            e1.record(stream)
            torch.cuda.synchronize()
        return e0.elapsed_time(e1), L.gfm_launch_count() - l0, clk.summary()

    ms_seq, launches_seq, clk_seq = timed(False)
    ms_streams, launches_streams, clk_streams = timed(True)
    # the project's autotuner (tile shape per grid-size class, schedule),
    # timed on the state after the warm-up and restored; then the tuned run
    for ctx, st in zip(b.instances, start):
        ctx.upload(st[0], st[1], st[2], t=st[3], numsteps=st[4])
    tuning = b.autotune(m, steps=16)
    L.gfm_batch_set_stream(b._p, ctypes.c_void_p(stream.cuda_stream))
    ms_graph, launches, clk = timed(True)
    stats = [ctx.status() for ctx in b.instances]
    value = cells * args.steps / (ms_graph * 1e-3)
    plain = cells * args.steps / (ms_seq * 1e-3)
    # end to end: every step uploads all instances' state from pinned host
    # memory, steps the batch and downloads it again
    e2e = None
    if args.e2e_steps != 0:
        n_e2e = min(args.steps, 20) if args.e2e_steps < 0 else min(args.e2e_steps, args.steps)
        pinned = []
        for st in start:
            arrs = []
            for a in st[:3]:
                h = torch.empty(a.shape, dtype=torch.float64, pin_memory=True).numpy()
                h[...] = a
                arrs.append(h)
            pinned.append(arrs)
        for ctx, st in zip(b.instances, start):
            L.gfm_set_time(ctx._p, st[3], st[4])
        pd = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))  # noqa: E731
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(n_e2e):
            for ctx, (h1, h2, hp) in zip(b.instances, pinned):
                L.gfm_upload_state_async(ctx._p, pd(h1), pd(h2), pd(hp))
            b.step(m, 1, graph=True)
            for ctx, (h1, h2, hp) in zip(b.instances, pinned):
                L.gfm_download_state(ctx._p, pd(h1), pd(h2), pd(hp))
        torch.cuda.synchronize()
        el = time.perf_counter() - t0
        nbytes = sum(sum(a.nbytes for a in arrs) for arrs in pinned)
        e2e = {"value": cells * n_e2e / el, "unit": UNIT, "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes,
               "steps": n_e2e}
    b.close()
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms_graph / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic",
            "config": {"workload": "batch64_shock_bubble_riemannGFM", "instances": len(spec), "cells": cells,
                       "seed": BATCH_SEED, "sides": "128..1024 step 64, aspect U[1,3]", "CFL": 0.6,
                       "p_star_guess": "plain (PVRS / TSRS)",
                       "schedule": "recorded CUDA graph, 8 steps per replay; %s schedule and tile shapes per size "
                                   "class from gfm_batch_autotune" % tuning["schedule"],
                       "l2": "inputs larger than L2 (%.1f GB of state)" % (cells * 9 * 8 / 1e9)},
            "plain_sequential": {"value": plain, "ms_per_step": ms_seq / args.steps, "gpu_launches": launches_seq,
                                 "clocks": clk_seq},
            "batched_streams_untuned": {"value": cells * args.steps / (ms_streams * 1e-3),
                                        "ms_per_step": ms_streams / args.steps, "gpu_launches": launches_streams,
                                        "clocks": clk_streams},
            "autotune": tuning,
            "batched_over_plain": value / plain,
            "e2e": e2e, "gpu_launches": int(launches), "clocks": clk,
            "device_status_nonzero": int(sum(1 for x in stats if x))}
    print(json.dumps(line))


def relaunch_command(argv, gpus, port):
    """The command that runs this benchmark as `gpus` ranks, one per GPU, when
    --gpus N > 1 is asked outside a distributed launch (the same command line
    as a distributed launch of the benchmark)."""
    return [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", str(gpus),
            "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.abspath(__file__)] + list(argv)


def main():
    args = parse()
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        # one process per GPU: independent replicas with a barrier and the
        # max over ranks (rank 0 prints the line)
        port = 29500 + os.getpid() % 2000
        sys.exit(subprocess.call(relaunch_command(sys.argv[1:], args.gpus, port)))
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "batch64":
        run_batch(args)
    else:
        run_gfm(args)


if __name__ == "__main__":
    main()
