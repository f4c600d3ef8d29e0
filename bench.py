#!/usr/bin/env python
"""Benchmark of the MPAS-O-FleCSI RK4 tendency path on GB300.

Metric: RK4 cell-updates/s (one cell x one level advanced one full RK4 step),
whole job, plus the fraction of the HBM roofline of the dominant kernel.

Default workload (--config sw_l7): shallow water on the sphere, dual of a
level-7 icosahedral subdivision (163,842 cells, 491,520 edges, 327,680
vertices, a = 6.371e6 m), FP64, Coriolis 2 Omega sin(lat), one passive tracer
with FCT advection, del2 tracer and momentum diffusion (1e4 m^2/s), RK4
dt = 60 s; seeded synthetic state (degree-8 random fields: h = 8000 m +/- 100 m,
u peak 30 m/s, tracer in [0, 1]).  Other configs: ocean_l7 (60 levels,
3 tracers, FCT + del2 tracer only, dt = 300 s), sw_l6.

Arms:
  default           the CUDA path through the fused graph-captured RK4 step;
  --impl reference  the reference algorithm on the host CPU cores: the
                    reference's own task sources built through the oracle
                    shim where they were built here, else the oracle's C
                    restatement (bit-identical to them), one process per core.

Multi-GPU (torchrun): every rank advances its own replica of the workload
(no communication; the path has no exchange step), value = total
cell-updates/s, "scaling": "weak".
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "mpas-o-flecsi-2.0_gb300")
for _p in (PKG,):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "SW RK4 cell-updates/s on 1 GB300 & % HBM roofline; adjoint/forward time ratio"
CONFIGS = {
    "sw_l7": dict(workload="sphere-level7 shallow-water RK4 + FCT tracer + del2 (163842 cells, L=1, T=1)",
                  level=7, app="sw", L=1, T=1, dt=60.0, fct=True, hmix=True, kappa=1e4, nu=1e4),
    "sw_l6": dict(workload="sphere-level6 shallow-water RK4 + FCT tracer + del2 (40962 cells, L=1, T=1)",
                  level=6, app="sw", L=1, T=1, dt=90.0, fct=True, hmix=True, kappa=1e4, nu=1e4),
    "ocean_l7": dict(workload="sphere-level7 ocean tracers, 60 levels x 3 tracers, FCT + del2 (9.8M cell-levels)",
                     level=7, app="ocean", L=60, T=3, dt=300.0, fct=True, hmix=True, kappa=1e4, nu=0.0),
    "ocean_l6": dict(workload="sphere-level6 ocean tracers, 60 levels x 3 tracers, FCT + del2 (2.5M cell-levels)",
                     level=6, app="ocean", L=60, T=3, dt=450.0, fct=True, hmix=True, kappa=1e4, nu=0.0),
}
L2_BYTES = 129e6


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def build_workload(cfg, seed, fct=True):
    import mpaso
    from mpaso.initial import ocean_state, sw_state
    from mpaso.setup import fct_statics
    t0 = time.time()
    mesh = mpaso.Mesh.icosa(cfg["level"])
    fct = fct_statics(mesh, cfg["L"]) if fct else None
    if cfg["app"] == "sw":
        state = sw_state(mesh, seed, cfg["L"], cfg["T"])
    else:
        state = ocean_state(mesh, seed, cfg["L"], cfg["T"])
    log(f"workload built in {time.time() - t0:.1f}s: {mesh.nCells} cells")
    return mesh, fct, state


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap,utilization.gpu")

    def __init__(self, index):
        self.index = index
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={index}", f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "100"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        self.p.wait()
        self.f.seek(0)
        rows = [[x.strip() for x in r.split(",")] for r in self.f.read().strip().splitlines() if r.strip()]
        os.unlink(self.f.name)
        num = lambda x: x.replace(".", "", 1).isdigit()  # noqa: E731
        rows = [r for r in rows if len(r) >= 10 and num(r[1]) and num(r[2])]
        busy = [r for r in rows if num(r[9]) and float(r[9]) >= 50]
        under = busy or rows
        sm = [float(r[1]) for r in under]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(float(r[2]) for r in rows) if rows else None,
                "samples": len(rows), "samples_under_load": len(busy),
                "power_w_max": max((float(r[3]) for r in rows if num(r[3])), default=None),
                "reasons": reasons}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def workload_config(args, cfg, mesh, world):
    """The `config` object of the line: what the workload is (the reference
    arm repeats it verbatim)."""
    return {"workload": cfg["workload"], "config": args.config, "cells": mesh.nCells, "edges": mesh.nEdges,
            "vertices": mesh.nVertices, "levels": cfg["L"], "tracers": cfg["T"], "dt_s": cfg["dt"],
            "fct": cfg["fct"], "del2_tracer": cfg["kappa"], "del2_momentum": cfg["nu"],
            "parallelism": f"replicas x{world}"}


def timed_regions(fn, ext, barrier, min_ms, min_reps=3):
    """Runs fn() (the timed region) repeatedly, each time bracketed by a
    barrier and device synchronisation and timed with CUDA events on the
    state stream, until at least min_ms of regions and min_reps regions ran.
    The repeat count is fixed before the first timed region (from one
    untimed calibration region, max over ranks) so every rank runs the same
    number.  Returns the per-region times in ms."""
    import torch

    from mpaso.replicas import reduce_over_ranks
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def one():
        barrier()
        e0.record(ext)
        fn()
        e1.record(ext)
        e1.synchronize()
        barrier()
        return e0.elapsed_time(e1)
    cal = reduce_over_ranks(one(), "max", device="cuda")
    reps = max(min_reps, int(-(-min_ms // max(cal, 1e-3))))
    return [one() for _ in range(reps)]


def gpu_arm(args, cfg, extras=True):
    import numpy as np
    import torch

    import mpaso.gpu as G
    from mpaso.perfmodel import Dims, dataflow_bytes, ocean_kernels, per_step, sw_kernels
    from mpaso.replicas import reduce_over_ranks

    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    if world > 1 and not torch.distributed.is_initialized():
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    mesh, fct, state = build_workload(cfg, seed=1000 + rank)
    dm = G.DeviceMesh(mesh, fct=fct, device=local)
    app = G.APP_SW if cfg["app"] == "sw" else G.APP_OCEAN
    st = G.State(dm, app=app, nlev=cfg["L"], ntr=cfg["T"], fct=cfg["fct"], hmix=cfg["hmix"],
                 kappa=cfg["kappa"], nu=cfg["nu"])
    if app == G.APP_SW:
        h, u, tr = state
        fields = ((G.FIELD_H, h), (G.FIELD_U, u), (G.FIELD_TRACERS, tr))
    else:
        h, hE, u, tr = state
        fields = ((G.FIELD_H, h), (G.FIELD_U, u), (G.FIELD_TRACERS, tr), (G.FIELD_LAYER_THICKNESS_EDGE, hE))
    for f, a in fields:
        st.set(f, a)
    dt, K, W = cfg["dt"], args.steps, args.warmup
    ext = torch.cuda.ExternalStream(st.stream())
    # per-mesh launch autotuning at set-up (untimed; the state is restored after it)
    launch = st.autotune(dt, 3) if not args.no_autotune else st.launch_config()
    log(f"launch configuration: {launch}")
    st.step_graph(dt, W)
    st.sync()

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    # ---- timed region: K graph-replayed steps, repeated for >= min_timed_s
    sampler = ClockSampler(local)
    time.sleep(0.3)
    regions = timed_regions(lambda: st.step_graph(dt, K), ext, barrier, args.min_timed_s * 1e3)
    clocks = sampler.stop()
    ms = statistics.median(regions)
    ms_max = reduce_over_ranks(ms, "max", device="cuda")
    units_rank = mesh.nCells * cfg["L"]
    value = world * units_rank * K / (ms_max * 1e-3)
    ms_step = ms_max / K

    # ---- per-kernel device time: shares from the replayed step graph with an
    # event node after every kernel (the nodes cost the launches their overlap,
    # so those intervals add up to more than the plain step), applied to the
    # measured step time so the kernels add up to it
    prof_raw = st.profile(dt, min(max(K, 10), 50))
    prof_sum = sum(prof_raw.values())
    prof = {k: v / prof_sum * ms_step / 4 for k, v in prof_raw.items()}
    dims = Dims.of(mesh, cfg["L"], cfg["T"], fct)
    model = (sw_kernels(dims, cfg["fct"], cfg["hmix"], cfg["nu"] != 0.0) if app == G.APP_SW
             else ocean_kernels(dims, cfg["fct"], cfg["hmix"]))
    model_bytes, step_fp64 = per_step(model)
    prof_step = 4 * prof_sum
    peak, peak_kind = measured_peaks()
    # roofline of record: the whole step's minimal-dataflow bytes over the
    # step time; the step is the unit the bytes are defined on (each array
    # once per stage, summed over the fused kernels)
    step_bytes = dataflow_bytes(mesh, cfg["L"], cfg["T"], fct, cfg["fct"], cfg["hmix"])
    achieved = step_bytes / (ms_step * 1e-3) / 1e9
    traffic = None
    tkern = {}
    traffic_scaled = None
    for k in model:
        # the capture of this workload, else one of the same kernel on a smaller
        # mesh (same levels and tracers) scaled by the cells processed
        for name in (args.config, args.config.replace("_l7", "_l6")):
            tfile = os.path.join(ROOT, "profiles", f"{k}_{name}.txt")
            if not os.path.exists(tfile):
                continue
            vals = {}
            for line in open(tfile):
                if ":" in line and not line.startswith("#"):
                    key, _, v = line.partition(":")
                    vals[key.strip()] = v.split()[0] if v.split() else ""
            if "dram_bytes_per_launch" in vals:
                scale = mesh.nCells / float(vals.get("cells", mesh.nCells)) if name != args.config else 1.0
                tkern[k] = float(vals["dram_bytes_per_launch"]) * scale
                if name != args.config:
                    traffic_scaled = f"ncu capture of {name} scaled by cells ({scale:.2f}x)"
                break
    if len(tkern) == len(model):
        traffic = 4 * sum(tkern.values())
    top = max(prof, key=prof.get)
    roofline = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "traffic": traffic,
                "kernel": "rk4_step (the graph of 3 kernels x 4 RK stages)",
                "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured"
                else "fallback 6.8 TB/s",
                "byte_model": "minimal fused dataflow: each array read/written once per RK stage "
                              "(mpaso/perfmodel.py dataflow_bytes)",
                "algorithmic_bytes_per_step": int(step_bytes),
                "bytes_per_cell_update": round(step_bytes / units_rank, 1),
                "traffic_note": "sum over the step's 12 launches of ncu dram__bytes_read + write (profiles/)"
                                + (f"; {traffic_scaled}" if traffic_scaled else ""),
                "traffic_model": {"per_launch_bytes_per_step": int(model_bytes),
                                  "frac": round(model_bytes / (ms_step * 1e-3) / 1e9 / peak, 4),
                                  "note": "every array each launch touches, re-reads across the three "
                                          "kernels of a stage included (mpaso/perfmodel.py sw_kernels)"},
                "dominant_kernel": top, "dominant_kernel_time_share": round(prof[top] / sum(prof.values()), 3)}
    # FP64 pipe: 2 DFMA/DADD/DMUL per clock per SM (ncu's peak for the pipe),
    # at the median SM clock under load
    sms = torch.cuda.get_device_properties(local).multi_processor_count
    mhz = clocks.get("sm_mhz") or clocks.get("sm_max_mhz") or 2070.0
    pipe_peak = 2.0 * sms * mhz * 1e6
    fp64 = {"bound": "fp64", "peak_per_s": pipe_peak,
            "peak_note": f"2 FP64 instructions per clock per SM x {sms} SMs x {mhz:.0f} MHz (median under load)",
            "step_frac": round(step_fp64 / (ms_step * 1e-3) / pipe_peak, 4),
            "instructions_per_cell_update": round(step_fp64 / units_rank, 1),
            "per_kernel_frac": {k: round(model[k][1] / (prof[k] * 1e-3) / pipe_peak, 4) for k in model},
            "note": "FP64 thread instructions from mpaso/perfmodel.py (within 4% of ncu's counts, tests/test_perfmodel.py) over the "
                    "graph-replayed time; the FP64 pipe, not HBM, is the binding ceiling of this path"}
    kernels = {k: {"ms_per_launch": round(v, 5), "share": round(v / sum(prof.values()), 3),
                   "model_bytes": int(model[k][0]),
                   "model_gbs": round(model[k][0] / (v * 1e-3) / 1e9, 1),
                   "ncu_dram_bytes": tkern.get(k)} for k, v in prof.items()}

    # ---- end to end through the C ABI with host buffers (pinned)
    Ke = min(K, 200)
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory()  # noqa: E731
    if app == G.APP_SW:
        hp, up, tp = pin(h), pin(u), pin(tr)
        nbytes = (hp.numel() + up.numel() + tp.numel()) * 8
        st.step_host(dt, 1, hp, up, tp)  # warm the staging path
        torch.cuda.synchronize()

        def blocking():
            for _ in range(Ke):
                st.step_host(dt, 1, hp, up, tp)

        def queued():
            # each call still copies its inputs in from and its results out to
            # the page-locked buffers, in order, but the host does not wait in
            # between; one sync at the end
            for _ in range(Ke):
                st.step_host_async(dt, 1, hp, up, tp)
            st.sync()
        st.step_host_async(dt, 1, hp, up, tp)
        st.sync()
        blocking_ms = statistics.median(timed_regions(blocking, ext, barrier, args.min_timed_s * 5e2))
        e2e_ms = statistics.median(timed_regions(queued, ext, barrier, args.min_timed_s * 5e2))
    else:
        tp = pin(tr)
        nbytes = tp.numel() * 8

        def io_steps():
            for _ in range(Ke):
                st.set(G.FIELD_TRACERS, tp)
                st.step_graph(dt, 1)
                st.get(G.FIELD_TRACERS, tp.numpy())
        e2e_ms = statistics.median(timed_regions(io_steps, ext, barrier, args.min_timed_s * 5e2))
    e2e_max = reduce_over_ranks(e2e_ms, "max", device="cuda")
    e2e = {"value": world * units_rank * Ke / (e2e_max * 1e-3), "unit": "cell-updates/s",
           "h2d_bytes_per_step": int(nbytes), "d2h_bytes_per_step": int(nbytes),
           "path": "mpaso_rk4_step_host_async x steps, then mpaso_state_sync (C ABI, pinned host buffers: "
                   "copy in -> 1 step -> copy out every step)"
           if app == G.APP_SW else "mpaso_state_set/rk4_step_graph/state_get (C ABI, pinned host buffers)",
           "timing": f"median of repeated regions of {Ke} calls"}
    e2e["host_link"] = host_link_rates(local)
    if app == G.APP_SW:
        bl = reduce_over_ranks(blocking_ms, "max", device="cuda")
        e2e["blocking"] = {"value": world * units_rank * Ke / (bl * 1e-3),
                           "path": "mpaso_rk4_step_host, which returns after each step's copy out"}

    # ---- conservation and bounds over an untimed trajectory from the initial state
    Kd = min(K, 200)
    for f, a in fields:
        st.set(f, a)
    st.step_graph(dt, Kd)
    st.check_finite()
    area = mesh.fields["areaCell"][:, None]
    hN, trN = st.get(G.FIELD_H), st.get(G.FIELD_TRACERS)
    if app == G.APP_SW:  # thickness-weighted tracer content
        c0 = (area[..., None] * h[..., None] * tr).sum(axis=(0, 1))
        cN = (area[..., None] * hN[..., None] * trN).sum(axis=(0, 1))
    else:  # prescribed constant thickness: the tracer content per area
        c0 = (area[..., None] * tr).sum(axis=(0, 1))
        cN = (area[..., None] * trN).sum(axis=(0, 1))
    lo, hi = tr.min(axis=(0, 1)), tr.max(axis=(0, 1))
    tol = 1e-12 * (hi - lo)
    diagnostics = {
        "steps": Kd,
        "mass_rel_drift": float(abs((area * hN).sum() - (area * h).sum()) / (area * h).sum()),
        "tracer_content_rel_drift": [float(abs(x - y) / abs(y)) for x, y in zip(cN, c0)],
        "tracer_range_initial": [[float(x), float(y)] for x, y in zip(lo, hi)],
        "tracer_range_final": [[float(x), float(y)] for x, y in zip(trN.min(axis=(0, 1)), trN.max(axis=(0, 1)))],
        "cells_outside_initial_range": int(((trN < lo - tol) | (trN > hi + tol)).sum()),
        "finite": True,
    }

    out = None
    if rank == 0:
        cpu = (cpu_baseline(cfg, mesh, fct, state)
               if (world == 1 and not args.no_cpu_baseline and extras) else None)
        working_set = dm.device_bytes() + st.device_bytes()
        out = {
            "metric": METRIC, "value": value, "unit": "cell-updates/s", "n_gpus": world, "steps": K,
            "warmup": W, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded smooth fields on generated mesh)",
            "config": workload_config(args, cfg, mesh, world),
            "run": {"timing": f"CUDA events on the state stream; the {K}-step graph-replayed region repeated "
                              f"{len(regions)} times (>= {args.min_timed_s} s), median region reported",
                    "regions_ms": {"median": round(ms, 4), "min": round(min(regions), 4),
                                   "max": round(max(regions), 4), "count": len(regions)},
                    "l2": f"device working set {working_set / 1e6:.0f} MB > {L2_BYTES / 1e6:.0f} MB L2 "
                          "(inputs larger than L2, no flush)",
                    "launch": dict(launch, autotuned=not args.no_autotune),
                    "profiled_step_ms": round(prof_step, 5),
                    "kernel_times": "per-kernel shares from the step graph replayed with an event node after "
                                    "every kernel (that graph's step: profiled_step_ms), times the measured "
                                    "step; ncu launch-list shares in profiles/"},
            "roofline": roofline, "fp64": fp64,
            "kernels_ms_per_launch": {k: round(v, 5) for k, v in prof.items()}, "kernels": kernels,
            "e2e": e2e, "clocks": clocks, "cpu_baseline": cpu, "diagnostics": diagnostics,
            "gpu_launches": st.launches_per_step() * K,
            "gpu_launches_note": f"per timed region: {st.launches_per_step()} kernels per step x {K} steps "
                                 f"(the region ran {len(regions)} times)",
        }
    st.close()
    dm.close()
    return out


def host_link_rates(device, sizes_mb=(0.0625, 1, 6.5, 64, 256)):
    """Copy rates between page-locked host memory and the device by transfer
    size (one cudaMemcpyAsync each way, CUDA events, best of 5), and where the
    page-locked buffers sit: the NUMA node of the host CPUs this process runs
    on, next to the GPU's own node."""
    import torch
    out = {"unit": "GB/s", "h2d": {}, "d2h": {}}
    st = torch.cuda.Stream(device)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for mb in sizes_mb:
        n = int(mb * (1 << 20)) // 8
        hb = torch.empty(n, dtype=torch.float64).pin_memory()
        db = torch.empty(n, dtype=torch.float64, device=device)
        for key, dst, src in (("h2d", db, hb), ("d2h", hb, db)):
            best = 1e30
            with torch.cuda.stream(st):
                for _ in range(5):
                    e0.record(st)
                    dst.copy_(src, non_blocking=True)
                    e1.record(st)
                    e1.synchronize()
                    best = min(best, e0.elapsed_time(e1))
            out[key][f"{mb:g}MB"] = round(n * 8 / (best * 1e-3) / 1e9, 1)
    try:
        cpus = sorted(os.sched_getaffinity(0))
        nodes = set()
        for c in cpus:
            for d in os.listdir(f"/sys/devices/system/cpu/cpu{c}"):
                if d.startswith("node"):
                    nodes.add(int(d[4:]))
        out["host_cpu_numa_nodes"] = sorted(nodes)
        bus = torch.cuda.get_device_properties(device).pci_bus_id if hasattr(
            torch.cuda.get_device_properties(device), "pci_bus_id") else None
        out["gpu_pci_bus_id"] = bus
    except Exception as e:  # noqa: BLE001
        out["numa"] = repr(e)
    return out


def cpu_baseline(cfg, mesh, fct, state, budget_s=12.0):
    """The reference algorithm on one core, a bounded number of full RK4 steps
    on the same mesh and state: the reference's own task sources compiled
    through the oracle's shim where that library was built for the workload's
    levels and tracers (kind "reference"), else the oracle's C restatement,
    bit-identical to them (kind "port")."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    from oracle import Oracle
    kind = "port"
    if os.path.exists(os.path.join(ROOT, "oracle", "_ref", f"libref_L{cfg['L']}_T{cfg['T']}.so")):
        try:
            O = Oracle("ref", cfg["L"], cfg["T"])
            kind = "reference"
        except OSError:
            pass
    if kind == "port":
        O = Oracle("restatement")
    st = O.static(mesh, fct)
    c = O.config(cfg["L"], cfg["T"], fct=cfg["fct"], hmix=cfg["hmix"], kappa=cfg["kappa"], nu=cfg["nu"])
    om = O.mesh(mesh)
    run = ((lambda n: O.sw_run(om, st, c, cfg["dt"], n, *state)) if cfg["app"] == "sw"
           else (lambda n: O.ocean_run(om, st, c, cfg["dt"], n, state[0], state[1], state[2], state[3])))
    t0 = time.perf_counter()
    run(1)
    t1 = time.perf_counter() - t0
    n = max(1, min(50, int(budget_s / max(t1, 1e-3))))
    t0 = time.perf_counter()
    run(n)
    el = time.perf_counter() - t0
    what = ("the reference's task sources compiled through the oracle shim" if kind == "reference" else
            "oracle C restatement (bit-identical to the reference tasks)")
    return {"value": mesh.nCells * cfg["L"] * n / el, "unit": "cell-updates/s", "cores": 1, "kind": kind,
            "sample": f"{n} RK4 steps of the same {mesh.nCells}-cell workload, {what}, gcc -O3, one thread"}


# ---------------------------------------------------------------- adjoint (cfg3)
def adjoint_arm(args):
    """Gradient of J = 1/2 <area (h_N - h_target)^2> / sum(area) w.r.t. (h0, u0):
    level-6 sphere, 500 RK4 steps of dt = 90 s, checkpoints every 25 steps."""
    import numpy as np
    import torch

    import mpaso
    import mpaso.gpu as G
    from mpaso.initial import sw_state
    N, K, dt, level = args.adj_steps, args.adj_ckpt, 90.0, 6
    mesh = mpaso.Mesh.icosa(level)
    h0, u0, _ = sw_state(mesh, 1234, 1, 1)
    ht, _, _ = sw_state(mesh, 4321, 1, 1)
    area = mesh.fields["areaCell"][:, None]
    w = area / area.sum()
    dm = G.DeviceMesh(mesh)
    st = G.State(dm, nlev=1, ntr=0)
    ext = torch.cuda.ExternalStream(st.stream())

    def timed(fn):
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(ext)
        fn()
        e1.record(ext)
        e1.synchronize()
        return e0.elapsed_time(e1)

    def loss(h, u):
        st.set(G.FIELD_H, h)
        st.set(G.FIELD_U, u)
        st.step(dt, N)
        hN = st.get(G.FIELD_H)
        return 0.5 * float((w * (hN - ht) ** 2).sum()), hN

    # warm-up: builds the step graph and the captured reverse sweep for (N, K, dt)
    st.set(G.FIELD_H, h0), st.set(G.FIELD_U, u0)
    st.forward(dt, N, K)
    st.vjp(np.zeros_like(h0), np.zeros_like(u0))
    st.set(G.FIELD_H, h0), st.set(G.FIELD_U, u0)
    st.step_graph(dt, 2)
    st.set(G.FIELD_H, h0), st.set(G.FIELD_U, u0)
    t_plain = timed(lambda: st.step_graph(dt, N))
    st.set(G.FIELD_H, h0), st.set(G.FIELD_U, u0)
    t_fwd = timed(lambda: st.forward(dt, N, K))
    hN = st.get(G.FIELD_H)
    gh_N = w * (hN - ht)
    out = {}
    t_vjp = timed(lambda: out.update(g=st.vjp(gh_N, np.zeros_like(u0))))
    gh, gu = out["g"]
    # the same gradient with the whole window stored (ckpt_every = 0): no recompute
    st.set(G.FIELD_H, h0), st.set(G.FIELD_U, u0)
    st.forward(dt, N, 0)
    st.vjp(gh_N, np.zeros_like(u0))  # warm-up: captures the stored-mode graphs
    st.set(G.FIELD_H, h0), st.set(G.FIELD_U, u0)
    t_fwd_s = timed(lambda: st.forward(dt, N, 0))
    t_vjp_s = timed(lambda: out.update(gs=st.vjp(gh_N, np.zeros_like(u0))))
    stored = {"forward_ms": t_fwd_s, "vjp_ms": t_vjp_s, "vjp_over_plain_forward": t_vjp_s / t_plain,
              "gradient_over_plain_forward": (t_fwd_s + t_vjp_s) / t_plain,
              "max_rel_diff_vs_checkpointed": float(max(np.abs(a - b).max() / np.abs(b).max()
                                                        for a, b in zip(out["gs"], (gh, gu)))),
              "adjoint_device_bytes": int(st.adjoint_device_bytes())}
    rng = np.random.default_rng(7)
    errs = []
    for _ in range(args.adj_dirs):
        dh = rng.standard_normal(h0.shape) * 0.1
        du = rng.standard_normal(u0.shape) * 1e-3
        eps = 1.0
        jp, _ = loss(h0 + eps * dh, u0 + eps * du)
        jm, _ = loss(h0 - eps * dh, u0 - eps * du)
        fd = (jp - jm) / (2 * eps)
        ad = float((gh * dh).sum() + (gu * du).sum())
        errs.append(abs(fd - ad) / max(abs(ad), 1e-300))
    mem = dm.device_bytes() + st.device_bytes() + st.adjoint_device_bytes()
    tracers = adjoint_tracer_leg(args, mesh, N, K, dt)
    del st, dm
    ocean = ocean_adjoint_leg(args)
    return {"metric": "adjoint/forward time ratio (sw RK4, level-6 sphere)",
            "value": t_vjp / t_fwd, "unit": "ratio", "higher_is_better": False, "n_gpus": 1,
            "steps": N, "dtype": "f64", "data": "synthetic (seeded smooth fields)",
            "config": {"workload": f"sphere-level{level} sw RK4, {N} steps, dt={dt}s, checkpoint every {K}",
                       "cells": mesh.nCells, "edges": mesh.nEdges,
                       "loss": "0.5 * sum(area (h_N - h_target)^2) / sum(area)"},
            "forward_ms": t_fwd, "forward_plain_ms": t_plain, "vjp_ms": t_vjp,
            "vjp_over_plain_forward": t_vjp / t_plain,
            "fd_check": {"directions": args.adj_dirs, "max_rel_err": max(errs) if errs else None,
                         "median_rel_err": float(np.median(errs)) if errs else None},
            "peak_device_bytes": int(mem), "stored_window": stored, "tracers": tracers, "ocean_tracers": ocean}


def adjoint_tracer_leg(args, mesh, N, K, dt):
    """The same window with one FCT-advected, del2-mixed tracer (kappa 1e4
    m^2/s): J = 1/2 <area (tr_N - tr_target)^2> / sum(area), gradient w.r.t.
    (h0, u0, tr0) through mpaso_rk4_vjp_tracers (limiter differentiated on
    its active branch), timed against the forward of the same state."""
    import numpy as np
    import torch

    import mpaso.gpu as G
    from mpaso.initial import sw_state
    from mpaso.setup import fct_statics
    h0, u0, tr0 = sw_state(mesh, 1234, 1, 1)
    _, _, trt = sw_state(mesh, 4321, 1, 1)
    w = (mesh.fields["areaCell"] / mesh.fields["areaCell"].sum())[:, None, None]
    dm = G.DeviceMesh(mesh, fct=fct_statics(mesh, 1))
    st = G.State(dm, nlev=1, ntr=1, fct=True, hmix=True, kappa=1e4)
    ext = torch.cuda.ExternalStream(st.stream())

    def timed(fn):
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(ext)
        fn()
        e1.record(ext)
        e1.synchronize()
        return e0.elapsed_time(e1)

    def put(h, u, tr):
        st.set(G.FIELD_H, h), st.set(G.FIELD_U, u), st.set(G.FIELD_TRACERS, tr)

    def loss(h, u, tr):
        put(h, u, tr)
        st.step(dt, N)
        return 0.5 * float((w * (st.get(G.FIELD_TRACERS) - trt) ** 2).sum())

    zh, zu = np.zeros_like(h0), np.zeros_like(u0)
    put(h0, u0, tr0)
    st.forward(dt, N, K)
    st.vjp_tracers(zh, zu, np.zeros_like(tr0))
    put(h0, u0, tr0)
    st.step_graph(dt, 2)
    put(h0, u0, tr0)
    t_plain = timed(lambda: st.step_graph(dt, N))
    put(h0, u0, tr0)
    t_fwd = timed(lambda: st.forward(dt, N, K))
    gtr_N = w * (st.get(G.FIELD_TRACERS) - trt)
    out = {}
    t_vjp = timed(lambda: out.update(g=st.vjp_tracers(zh, zu, gtr_N)))
    gh, gu, gt = out["g"]
    put(h0, u0, tr0)
    st.forward(dt, N, 0)
    st.vjp_tracers(zh, zu, gtr_N)
    put(h0, u0, tr0)
    t_fwd_s = timed(lambda: st.forward(dt, N, 0))
    t_vjp_s = timed(lambda: out.update(gs=st.vjp_tracers(zh, zu, gtr_N)))
    stored = {"forward_ms": t_fwd_s, "vjp_ms": t_vjp_s, "vjp_over_plain_forward": t_vjp_s / t_plain,
              "gradient_over_plain_forward": (t_fwd_s + t_vjp_s) / t_plain,
              "bitwise_equal_to_checkpointed": bool(all(np.array_equal(a, b) for a, b in zip(out["gs"], (gh, gu, gt)))),
              "adjoint_device_bytes": int(st.adjoint_device_bytes())}
    rng = np.random.default_rng(8)
    errs = []
    for _ in range(min(args.adj_dirs, 4)):
        v = (rng.standard_normal(h0.shape) * 0.1, rng.standard_normal(u0.shape) * 1e-3,
             rng.standard_normal(tr0.shape) * 1e-4)
        eps = 1e-2
        fd = (loss(*[a + eps * b for a, b in zip((h0, u0, tr0), v)]) -
              loss(*[a - eps * b for a, b in zip((h0, u0, tr0), v)])) / (2 * eps)
        ad = float(sum((g * x).sum() for g, x in zip((gh, gu, gt), v)))
        errs.append(abs(fd - ad) / max(abs(ad), 1e-300))
    # the tracer part alone, over a short window, along directions away from the
    # tracer's extrema (where the limiter keeps its branch)
    fd_local = ocean_fd_away_from_extrema(st, mesh, tr0, trt, w, dt, min(args.adj_dirs, 8),
                                          reset=((G.FIELD_H, h0), (G.FIELD_U, u0)))
    return {"workload": "same window, 1 tracer (FCT + del2 kappa=1e4), loss on the final tracer",
            "forward_ms": t_fwd, "forward_plain_ms": t_plain, "vjp_ms": t_vjp, "ratio": t_vjp / t_fwd,
            "vjp_over_plain_forward": t_vjp / t_plain, "stored_window": stored,
            "fd_check": {"directions": len(errs), "max_rel_err": max(errs) if errs else None,
                         "note": f"h, u and the tracer perturbed together over the whole {N}-step window: "
                                 "the FCT limiter changes branch within the perturbation"},
            "fd_away_from_extrema": fd_local,
            "peak_device_bytes": int(dm.device_bytes() + st.device_bytes() + st.adjoint_device_bytes())}


def ocean_adjoint_leg(args, N=20, K=10):
    """The ocean app's tracers (level-6 sphere, 60 levels x 3 tracers, FCT +
    del2, dt = 450 s, unclipped temperature; thickness and velocity prescribed): J = 1/2 <area
    (tr_N - tr_target)^2> / sum(area), gradient w.r.t. tr0 through
    mpaso_rk4_vjp_tracers, checkpoints every K of N steps, timed against the
    forward of the same state."""
    import numpy as np
    import torch

    import mpaso
    import mpaso.gpu as G
    from mpaso.initial import ocean_state
    from mpaso.setup import fct_statics
    cfg = CONFIGS["ocean_l6"]
    mesh = mpaso.Mesh.icosa(cfg["level"])
    fct = fct_statics(mesh, cfg["L"])
    # temperature not clipped to [0, 30]: on clipped plateaus the limiter's
    # quotients divide rounding-level differences by its 1e-10 regulariser and
    # no difference quotient can check the branch derivative
    h, hE, u, tr0 = ocean_state(mesh, 1234, cfg["L"], cfg["T"], clip=False)
    trt = tr0[::-1].copy()
    w = (mesh.fields["areaCell"] / mesh.fields["areaCell"].sum())[:, None, None]
    dm = G.DeviceMesh(mesh, fct=fct)
    st = G.State(dm, app=G.APP_OCEAN, nlev=cfg["L"], ntr=cfg["T"], fct=True, hmix=True, kappa=cfg["kappa"])
    for f, a in ((G.FIELD_H, h), (G.FIELD_U, u), (G.FIELD_LAYER_THICKNESS_EDGE, hE)):
        st.set(f, a)
    ext = torch.cuda.ExternalStream(st.stream())
    dt = cfg["dt"]

    def timed(fn):
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(ext)
        fn()
        e1.record(ext)
        e1.synchronize()
        return e0.elapsed_time(e1)

    def final(tr):
        st.set(G.FIELD_TRACERS, tr)
        st.step(dt, N)
        return st.get(G.FIELD_TRACERS)

    zh, zu = np.zeros_like(h), np.zeros_like(u)
    st.set(G.FIELD_TRACERS, tr0)
    st.forward(dt, N, K)
    st.vjp_tracers(zh, zu, np.zeros_like(tr0))
    st.set(G.FIELD_TRACERS, tr0)
    st.step_graph(dt, 2)
    st.set(G.FIELD_TRACERS, tr0)
    t_plain = timed(lambda: st.step_graph(dt, N))
    st.set(G.FIELD_TRACERS, tr0)
    t_fwd = timed(lambda: st.forward(dt, N, K))
    g_N = w * (st.get(G.FIELD_TRACERS) - trt)
    out = {}
    t_vjp = timed(lambda: out.update(g=st.vjp_tracers(zh, zu, g_N)))
    gt = out["g"][2]
    # central differences along random directions at two perturbation sizes:
    # the FCT limiter's quotients (regularised by 1e-10) change branch under
    # larger perturbations, so the difference quotient approaches the branch
    # derivative only as the perturbation shrinks.  J(+) - J(-) is summed as
    # sum w (a+ - a-)(a+ + a- - 2 target) / 2, each cell's difference taken
    # before the sum (the sum of squares itself cancels to ~1e-11).
    rng = np.random.default_rng(8)
    fd_rows = []
    for _ in range(min(args.adj_dirs, 2)):
        v = rng.standard_normal(tr0.shape)
        ad = float((gt * v).sum())
        for d in (1e-6, 1e-8, 1e-10):
            ap, am = final(tr0 + d * v), final(tr0 - d * v)
            fd = float((w * (ap - am) * (ap + am - 2.0 * trt)).sum()) / (4 * d)
            fd_rows.append({"perturbation": d, "fd": fd, "ad": ad, "rel_err": abs(fd - ad) / max(abs(ad), 1e-300)})
    fd_local = ocean_fd_away_from_extrema(st, mesh, tr0, trt, w, dt, min(args.adj_dirs, 8))
    return {"workload": f"{cfg['workload']}, {N} steps, dt={dt}s, checkpoint every {K}, loss on the final tracers",
            "forward_ms": t_fwd, "forward_plain_ms": t_plain, "vjp_ms": t_vjp, "ratio": t_vjp / t_fwd,
            "vjp_over_plain_forward": t_vjp / t_plain,
            "fd_check": fd_rows, "fd_away_from_extrema": fd_local,
            "fd_note": "fd_check perturbs every cell over the whole window: near tracer extrema the perturbation "
                       "moves the FCT limiter across its branches (the loss is not differentiable there), so those "
                       "quotients need not converge to the adjoint; fd_away_from_extrema keeps the limiter on one "
                       "branch and is the check of record",
            "adjoint_device_bytes": int(st.adjoint_device_bytes()),
            "peak_device_bytes": int(dm.device_bytes() + st.device_bytes() + st.adjoint_device_bytes())}


def ocean_fd_away_from_extrema(st, mesh, tr0, trt, w, dt, ndirs, nsteps=2, rings=6, reset=()):
    """Central differences of the forward against the adjoint over a short
    window (nsteps), along directions each supported on one cell and its
    neighbours, at one level and tracer, at least `rings` cells from every
    local extremum of that tracer: there the FCT limiter keeps its branch
    under the perturbation (near an extremum with no antidiffusive inflow its
    quotient divides rounding-level numbers by the 1e-10 regulariser)."""
    import numpy as np

    import mpaso.gpu as G
    if ndirs <= 0:
        return None
    f = mesh.fields
    coc, nEoC = f["cellsOnCell"] - 1, f["nEdgesOnCell"]
    valid = np.arange(coc.shape[1])[None, :] < nEoC[:, None]
    nb = np.where(valid, coc, np.arange(mesh.nCells)[:, None])

    def extremum_distance(x):
        ext = np.all(x[:, None] >= x[nb], axis=1) | np.all(x[:, None] <= x[nb], axis=1)
        dist = np.full(mesh.nCells, -1, np.int64)
        front, d = np.flatnonzero(ext), 0
        dist[front] = 0
        while front.size:
            d += 1
            cand = np.unique(nb[front][valid[front]])
            cand = cand[dist[cand] < 0]
            dist[cand] = d
            front = cand
        return dist

    def put(x):  # the tracers, and the fields a step advances with them (sw: h, u)
        for fld, a in reset:
            st.set(fld, a)
        st.set(G.FIELD_TRACERS, x)

    def final(x):
        put(x)
        st.step(dt, nsteps)
        return st.get(G.FIELD_TRACERS)
    put(tr0)
    st.forward(dt, nsteps, 1)
    gN = w * (st.get(G.FIELD_TRACERS) - trt)
    gt = st.vjp_tracers(np.zeros((mesh.nCells, tr0.shape[1])), np.zeros((mesh.nEdges, tr0.shape[1])), gN)[2]
    rng = np.random.default_rng(12)
    L, T = tr0.shape[1], tr0.shape[2]
    rows = []
    for _ in range(500):
        if len(rows) == ndirs:
            break
        k, t = int(rng.integers(L)), int(rng.integers(T))
        centres = np.flatnonzero(extremum_distance(tr0[:, k, t]) >= rings)
        if centres.size == 0:
            continue
        c0 = int(rng.choice(centres))
        patch = np.concatenate([[c0], coc[c0, :nEoC[c0]]])
        v = np.zeros_like(tr0)
        v[patch, k, t] = rng.standard_normal(patch.size)
        d = 1e-6 * np.abs(tr0[:, k, t]).max()
        ap, am = final(tr0 + d * v), final(tr0 - d * v)
        fd = float((w * (ap - am) * (ap + am - 2.0 * trt)).sum()) / (4 * d)
        ad = float((gt * v).sum())
        rows.append(abs(fd - ad) / abs(ad))
    return {"directions": len(rows), "steps": nsteps, "min_rings_from_extrema": rings,
            "max_rel_err": max(rows) if rows else None, "rel_errs": rows}


# ---------------------------------------------------------------- ensemble (cfg4)
def ensemble_arm(args):
    """256 uneven members (192 periodic hex meshes, 64 spheres) advanced as one
    ensemble context (mpaso_mesh_create_ensemble), against the same members
    advanced one at a time.  Under torchrun the members are sharded across
    ranks by cell count (no communication but the timing reduction)."""
    import numpy as np
    import torch

    import mpaso
    import mpaso.gpu as G
    from mpaso.initial import sw_state
    from mpaso.replicas import reduce_over_ranks, shard
    from mpaso.setup import fct_statics
    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    rng = np.random.default_rng(2024)
    sides = [int(x) for x in args.ens_sides.split(",")]
    levels = [int(x) for x in args.ens_levels.split(",")]
    specs = [("hex", int(s)) for s in rng.choice(sides, args.ens_planar)]
    specs += [("icosa", int(l)) for l in rng.choice(levels, args.ens_sphere)] if args.ens_sphere else []
    cells = [s[1] * s[1] if s[0] == "hex" else 10 * 4 ** s[1] + 2 for s in specs]
    mine = shard(cells, world, rank)
    # set-up: meshes, FCT statics and initial states on a pool of host
    # threads (the C calls release the GIL).  The one-call GPU setup of every
    # member's statics is timed beside it: its kernels take milliseconds, but
    # the reference layout it returns ([nE][16] stencils, 8.7 GB here) makes
    # the copy back to host memory the larger cost on this many small meshes
    from concurrent.futures import ThreadPoolExecutor

    from mpaso.setup import fct_statics_many
    threads = os.cpu_count() or 1

    def make_mesh(s):
        return mpaso.Mesh.hex(s[1], s[1], 10e3, 1e-4) if s[0] == "hex" else mpaso.Mesh.icosa(s[1])

    t0 = time.time()
    with ThreadPoolExecutor(threads) as pool:
        members = list(pool.map(make_mesh, [specs[i] for i in mine]))
        t1 = time.time()
        mfct = list(pool.map(lambda m: fct_statics(m, 1), members))
        t2 = time.time()
        fct_statics_many(members, 1, device=local)
        t3 = time.time()
        states = list(pool.map(lambda a: sw_state(a[1], 5000 + a[0], 1, 1), zip(mine, members)))
    t4 = time.time()
    opts = dict(fct=True, hmix=True, kappa=1e3, nu=1e3)
    dt, K, W = 30.0, min(args.steps, 200), args.warmup  # the ensemble workload is 200 steps
    dm = G.DeviceMesh.ensemble(members, mfct, device=local)
    t5 = time.time()
    setup = {"host_threads": threads, "meshes_s": t1 - t0, "fct_statics_host_threads_s": t2 - t1,
             "fct_statics_gpu_one_call_s": t3 - t2, "initial_states_s": t4 - t3, "device_mesh_s": t5 - t4,
             "total_s": (t2 - t0) + (t5 - t3)}
    log(f"ensemble built in {setup['total_s']:.1f}s: {len(members)} members, {dm.nC} cells on rank {rank}")
    st = G.State(dm, nlev=1, ntr=1, **opts)
    for f, k in ((G.FIELD_H, 0), (G.FIELD_U, 1), (G.FIELD_TRACERS, 2)):
        st.set(f, np.concatenate([s[k] for s in states]))
    ext = torch.cuda.ExternalStream(st.stream())
    launch = st.autotune(dt, 3) if not args.no_autotune else st.launch_config()
    st.step_graph(dt, W)
    st.sync()
    if world > 1:
        torch.distributed.barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(ext)
    st.step_graph(dt, K)
    e1.record(ext)
    e1.synchronize()
    t_batch = reduce_over_ranks(e0.elapsed_time(e1) * 1e-3, "max", device="cuda")
    # the same batch as one persistent launch (grid barriers between phases)
    st.step_persistent(dt, W)
    e0.record(ext)
    st.step_persistent(dt, K)
    e1.record(ext)
    e1.synchronize()
    t_persist = reduce_over_ranks(e0.elapsed_time(e1) * 1e-3, "max", device="cuda")
    # one member at a time: its own context and graph (same launch shapes),
    # members advanced in turn
    singles = []
    for i, m in enumerate(members):
        d = G.DeviceMesh(m, fct=mfct[i], device=local)
        s = G.State(d, nlev=1, ntr=1, **opts)
        for f, k in ((G.FIELD_H, 0), (G.FIELD_U, 1), (G.FIELD_TRACERS, 2)):
            s.set(f, states[i][k])
        s.set_launch_config(launch["unroll"], launch["threads"], launch["capped"], 0, launch["overlap"],
                            launch["split"], launch["lanes"])
        s.step_graph(dt, W)
        singles.append((d, s))
    torch.cuda.synchronize()
    # (a) every member on its own stream, all launched before any wait (members may overlap)
    t1 = time.perf_counter()
    for d, s in singles:
        s.step_graph(dt, K)
    for d, s in singles:
        s.sync()
    t_single = reduce_over_ranks(time.perf_counter() - t1, "max", device="cuda")
    # (b) members strictly one after another (a per-member loop that waits for each member)
    t1 = time.perf_counter()
    for d, s in singles:
        s.step_graph(dt, K)
        s.sync()
    t_serial = reduce_over_ranks(time.perf_counter() - t1, "max", device="cuda")
    n, ncells = len(specs), sum(cells)
    # FP64 issue of the batch against the pipe's peak: the model's instructions
    # per step of every member (mpaso/perfmodel.py) over the batch's step time
    from mpaso.perfmodel import Dims, per_step, sw_kernels
    fp64_step = sum(per_step(sw_kernels(Dims.of(mm, 1, 1, ff), True, True, True))[1]
                    for mm, ff in zip(members, mfct))
    pipe_peak = 2.0 * torch.cuda.get_device_properties(local).multi_processor_count * 2070e6
    fp64_batch = {"instructions_per_step": int(fp64_step),
                  "frac_of_pipe_peak": fp64_step * K / t_batch / pipe_peak,
                  "ceiling_speedup_vs_serial": (t_serial / K) / (fp64_step / pipe_peak),
                  "note": "FP64 thread instructions of all members' steps (model) over the batch time, against "
                          "2 per clock per SM at 2070 MHz; ceiling = the serial time over the time the batch's "
                          "FP64 work takes at the pipe's peak"}
    out = None
    if rank == 0:
        out = {"metric": "ensemble members*steps/s (one graph-captured launch sequence vs one at a time)",
               "value": n * K / t_batch, "unit": "member-steps/s", "higher_is_better": True, "n_gpus": world,
               "steps": K, "warmup": W, "dtype": "f64", "data": "synthetic (seeded smooth fields)",
               "scaling": "strong",
               "config": {"workload": f"{args.ens_planar} periodic hex (sides {args.ens_sides}) + "
                                      f"{args.ens_sphere} sphere (levels {args.ens_levels}) members, sw + FCT "
                                      f"tracer + del2, dt={dt}s",
                          "cells": int(ncells), "members": n, "launch": launch,
                          "parallelism": f"members sharded x{world}"},
               "cell_updates_per_s": ncells * K / t_batch,
               "persistent": {"value": n * K / t_persist, "unit": "member-steps/s",
                              "cell_updates_per_s": ncells * K / t_persist,
                              "speedup_vs_serial": t_serial / t_persist,
                              "speedup_vs_one_at_a_time": t_single / t_persist,
                              "how": "mpaso_rk4_step_persistent: all steps in one cooperative launch, grid "
                                     "barriers between the phases of each stage"},
               "one_at_a_time": {"value": n * K / t_single, "unit": "member-steps/s",
                                 "cell_updates_per_s": ncells * K / t_single,
                                 "how": "one context, graph and stream per member; all members launched, then waited"},
               "speedup_vs_one_at_a_time": t_single / t_batch,
               "one_at_a_time_serial": {"value": n * K / t_serial, "unit": "member-steps/s",
                                        "how": "members advanced strictly in turn (wait after each member)"},
               "speedup_vs_serial": t_serial / t_batch,
               "fp64": fp64_batch,
               "setup": setup,
               "gpu_launches": st.launches_per_step() * K}
    for d, s in singles:
        s.close()
        d.close()
    st.close()
    dm.close()
    if world > 1:
        torch.distributed.barrier()
        torch.distributed.destroy_process_group()
    return out


# ---------------------------------------------------------------- reference arm
_REF_FIELDS = ("areaCell", "dvEdge", "dcEdge", "areaTriangle", "kiteAreasOnVertex", "fVertex", "weightsOnEdge")


def make_ref_inputs(cfg_name, seed, path):
    """Writes the reference arm's inputs -- the mesh's connectivity (as the
    reference's mesh holds it) and geometry, the FCT statics from the oracle
    and the seeded initial state -- to `path` (.npz).  Runs in its own
    process, so the processes that time the reference load nothing but the
    oracle."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import numpy as np

    from oracle import Oracle
    cfg = CONFIGS[cfg_name]
    mesh, _, state = build_workload(cfg, seed, fct=False)
    O = Oracle("restatement")
    fct = O.fct_statics(mesh, cfg["L"], cfg=O.config(cfg["L"], cfg["T"]))
    arrays = {f"f_{k}": mesh.fields[k] for k in _REF_FIELDS}
    arrays.update({f"fct_{k}": v for k, v in fct.items()})
    for name, (off, idx) in mesh.crs().items():
        arrays[f"off_{name}"], arrays[f"idx_{name}"] = off, idx
    arrays.update({f"state_{i}": a for i, a in enumerate(state)})
    arrays["sizes"] = np.array([mesh.nCells, mesh.nEdges, mesh.nVertices, len(state)], np.int64)
    np.savez(path, **arrays)


class MeshSizes:
    def __init__(self, nC, nE, nV):
        self.nCells, self.nEdges, self.nVertices = nC, nE, nV


class SavedMesh:
    """The mesh as the oracle reads it (sizes, fields, reference-ordered CRS),
    loaded from make_ref_inputs' file."""

    def __init__(self, z):
        self.nCells, self.nEdges, self.nVertices = (int(x) for x in z["sizes"][:3])
        self.fields = {k: z[f"f_{k}"] for k in _REF_FIELDS}
        self._crs = {k[4:]: (z[k], z["idx_" + k[4:]]) for k in z.files if k.startswith("off_")}

    def crs(self):
        return self._crs


def _ref_load(cfg_name, inputs, kind):
    """(units, run(n)) of the reference arm in this process, from the inputs file."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import numpy as np

    from oracle import Oracle
    cfg = CONFIGS[cfg_name]
    z = np.load(inputs)
    mesh = SavedMesh(z)
    fct = {k[4:]: z[k] for k in z.files if k.startswith("fct_")}
    state = [z[f"state_{i}"] for i in range(int(z["sizes"][3]))]
    O = Oracle("restatement") if kind == "port" else Oracle("ref", cfg["L"], cfg["T"])
    st, om = O.static(mesh, fct), O.mesh(mesh)
    c = O.config(cfg["L"], cfg["T"], fct=cfg["fct"], hmix=cfg["hmix"], kappa=cfg["kappa"], nu=cfg["nu"])

    def run(n):
        if cfg["app"] == "sw":
            return O.sw_run(om, st, c, cfg["dt"], n, *state)
        return O.ocean_run(om, st, c, cfg["dt"], n, *state)
    return mesh, run


def _ref_size(args):
    """Seconds of one step of the reference arm (one core)."""
    cfg_name, inputs, kind = args
    mesh, run = _ref_load(cfg_name, inputs, kind)
    t0 = time.perf_counter()
    run(1)
    return time.perf_counter() - t0, (mesh.nCells, mesh.nEdges, mesh.nVertices)


def _ref_timed(args):
    cfg_name, inputs, kind, steps, warm, barrier = args
    mesh, run = _ref_load(cfg_name, inputs, kind)
    if warm:
        run(warm)  # untimed warm-up in this process
    barrier.wait()  # every process built and warmed up; the parent starts its clock
    t0 = time.perf_counter()
    run(steps)
    return mesh.nCells * CONFIGS[cfg_name]["L"], time.perf_counter() - t0


def reference_arm(args, cfg):
    """The reference algorithm on the host cores: the shim-built reference
    task sources where they were built, else the oracle's C restatement
    (bit-identical to them), one process per core, each advancing its own copy
    of the workload.  Inputs are made once in a separate process; the timed
    processes load only the oracle library.  Steps per process: --steps when
    the CPU budget allows it, else as many as fit (the line says which)."""
    world, rank, _ = dist_setup()
    if rank != 0:
        return None
    import multiprocessing as mp
    kind = "port"
    ref_lib = os.path.join(ROOT, "oracle", "_ref", f"libref_L{cfg['L']}_T{cfg['T']}.so")
    if os.path.exists(ref_lib):
        try:
            import ctypes
            ctypes.CDLL(ref_lib)
            kind = "reference"
        except OSError:
            kind = "port"
    cores = args.ref_procs or (os.cpu_count() or 1)
    ctx = mp.get_context("spawn")
    with tempfile.TemporaryDirectory() as tmp:
        inputs = os.path.join(tmp, "inputs.npz")
        t0 = time.time()
        p = ctx.Process(target=make_ref_inputs, args=(args.config, 2000, inputs))
        p.start()
        p.join()
        if p.exitcode != 0:
            raise RuntimeError("reference arm: making the inputs failed")
        log(f"reference inputs made in {time.time() - t0:.1f}s")
        # one process sizes the sample: a step's CPU time against the budget
        with ctx.Pool(1) as pool:
            t1, sizes = pool.apply(_ref_size, ((args.config, inputs, kind),))
        warm = max(1, min(args.warmup, int(0.1 * args.ref_budget_s / t1)))
        steps = max(1, min(args.steps, int((args.ref_budget_s - warm * t1) / t1)))
        barrier = ctx.Manager().Barrier(cores + 1)
        with ctx.Pool(cores) as pool:
            res = pool.map_async(_ref_timed, [(args.config, inputs, kind, steps, warm, barrier)
                                              for _ in range(cores)])
            barrier.wait()
            t0 = time.perf_counter()
            out = res.get()
            wall = time.perf_counter() - t0
    units = [u for u, _ in out]
    times = [t for _, t in out]
    value = sum(units) * steps / max(max(times), 1e-9)
    desc = (f"{cores} processes x {steps} RK4 steps of the {cfg['workload']} workload (each process its own "
            f"copy), {'reference task sources via the oracle shim' if kind == 'reference' else 'oracle C restatement of the reference tasks'}, "
            "gcc -O3, one thread each; inputs (mesh, FCT statics, initial state) made beforehand in a "
            "separate process")
    line = {"metric": METRIC, "value": value, "unit": "cell-updates/s", "n_gpus": world, "steps": steps,
            "warmup": warm, "ms_per_step": max(times) / steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded smooth fields on generated mesh)", "impl": "reference",
            "config": workload_config(args, cfg, MeshSizes(*sizes), world),
            "run": {"wall_s": round(wall, 2), "first_step_s": round(t1, 3), "cpu_budget_s": args.ref_budget_s},
            "cpu_baseline": {"value": value, "unit": "cell-updates/s", "cores": cores, "kind": kind,
                             "sample": desc},
            "e2e": {"value": value, "unit": "cell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "gpu_launches": 0}
    if steps < args.steps:
        line["run"]["steps_note"] = (f"{steps} of the requested {args.steps} steps per process: a step takes "
                                     f"{t1:.2f} s of one core, and the sample is held to {args.ref_budget_s:.0f} s")
    if warm < args.warmup:
        line["run"]["warmup_note"] = f"{warm} untimed warm-up steps (of {args.warmup}) within the budget"
    return line


def extras_for_line(args):
    """The rest of the metric, measured in the same run: the adjoint (level-6
    sphere, 500 steps, checkpoints every 25), the 60-level ocean workload and
    the 256-member ensemble, each summarised.  A part that fails records its
    error instead of stopping the line."""
    out = {}
    t0 = time.time()
    try:
        a = adjoint_arm(args)
        tr, oc = a.get("tracers") or {}, a.get("ocean_tracers") or {}
        out["adjoint"] = {
            "workload": a["config"]["workload"], "vjp_over_forward": a["value"],
            "gradient_over_plain_forward": (a["forward_ms"] + a["vjp_ms"]) / a["forward_plain_ms"],
            "forward_ms": a["forward_ms"], "forward_plain_ms": a["forward_plain_ms"], "vjp_ms": a["vjp_ms"],
            "fd_check": a["fd_check"], "peak_device_bytes": a["peak_device_bytes"],
            "stored_window": a["stored_window"],
            "with_tracer": {k: tr.get(k) for k in ("workload", "ratio", "vjp_over_plain_forward", "fd_check",
                                                   "fd_away_from_extrema", "peak_device_bytes")},
            "ocean_tracers": {k: oc.get(k) for k in ("workload", "ratio", "vjp_over_plain_forward", "fd_check",
                                                     "fd_away_from_extrema", "fd_note", "peak_device_bytes")}}
    except Exception as e:  # noqa: BLE001
        out["adjoint"] = {"error": repr(e)}
    log(f"extras: adjoint done at {time.time() - t0:.0f}s")
    try:
        sub = argparse.Namespace(**vars(args))
        sub.config, sub.steps, sub.no_cpu_baseline = "ocean_l7", min(args.steps, 20), True
        o = gpu_arm(sub, CONFIGS["ocean_l7"], extras=False)
        out["cfg2"] = {"workload": o["config"]["workload"], "value": o["value"],
                       "unit": "cell-level-updates/s", "ms_per_step": o["ms_per_step"], "steps": o["steps"],
                       "roofline_frac": o["roofline"]["frac"], "roofline": o["roofline"],
                       "fp64_step_frac": o["fp64"]["step_frac"], "fp64": o["fp64"],
                       "kernels_ms_per_launch": o["kernels_ms_per_launch"], "e2e": o["e2e"],
                       "diagnostics": o["diagnostics"], "launch": o["run"]["launch"], "clocks": o["clocks"]}
    except Exception as e:  # noqa: BLE001
        out["cfg2"] = {"error": repr(e)}
    log(f"extras: cfg2 done at {time.time() - t0:.0f}s")
    try:
        e = ensemble_arm(args)
        out["ensemble"] = {k: e[k] for k in ("value", "unit", "steps", "cell_updates_per_s", "persistent",
                                             "fp64", "one_at_a_time",
                                             "speedup_vs_one_at_a_time", "one_at_a_time_serial",
                                             "speedup_vs_serial", "setup")}
        out["ensemble"]["workload"] = e["config"]["workload"]
        out["ensemble"]["launch"] = e["config"]["launch"]
    except Exception as e:  # noqa: BLE001
        out["ensemble"] = {"error": repr(e)}
    try:
        out["threads_per_edge"] = lanes_table(args)
    except Exception as e:  # noqa: BLE001
        out["threads_per_edge"] = {"error": repr(e)}
    out["extras_wall_s"] = round(time.time() - t0, 1)
    return out


def lanes_table(args, levels=(3, 4, 5, 7)):
    """Time per RK4 step (sw + FCT tracer + del2) with 1, 2 and 4 threads per
    edge-level in the TRiSK loop, the rest of the launch configuration as the
    autotuner chose it, on spheres from too small to fill the GPU to the
    benchmark's size; the autotuner's own lane choice per mesh; and the same
    steps as one persistent launch."""
    import torch

    import mpaso
    import mpaso.gpu as G
    from mpaso.initial import sw_state
    from mpaso.setup import fct_statics
    rows = []
    for level in levels:
        mesh = mpaso.Mesh.icosa(level)
        dm = G.DeviceMesh(mesh, fct=fct_statics(mesh, 1))
        st = G.State(dm, nlev=1, ntr=1, fct=True, hmix=True, kappa=1e4, nu=1e4)
        h, u, tr = sw_state(mesh, 77, 1, 1)
        for f, a in ((G.FIELD_H, h), (G.FIELD_U, u), (G.FIELD_TRACERS, tr)):
            st.set(f, a)
        dt = 60.0 * 2 ** (7 - level)
        cfg = st.autotune(dt, 3)
        ext = torch.cuda.ExternalStream(st.stream())
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ms = {}
        n = max(20, 2000 >> max(level - 3, 0))
        for lanes in (1, 2, 4):
            st.set_launch_config(cfg["unroll"], cfg["threads"], cfg["capped"], cfg["l2"], cfg["overlap"],
                                 cfg["split"], lanes)
            st.step_graph(dt, 3)
            st.sync()
            e0.record(ext)
            st.step_graph(dt, n)
            e1.record(ext)
            e1.synchronize()
            ms[lanes] = e0.elapsed_time(e1) / n
        # the same steps in one persistent launch (autotuned launch shapes do not apply)
        st.set_launch_config(cfg["unroll"], cfg["threads"], cfg["capped"], cfg["l2"], cfg["overlap"],
                             cfg["split"], cfg["lanes"])
        st.step_persistent(dt, 3)
        e0.record(ext)
        st.step_persistent(dt, n)
        e1.record(ext)
        e1.synchronize()
        rows.append({"level": level, "cells": mesh.nCells, "autotuned_lanes": cfg["lanes"],
                     "ms_per_step": {str(k): round(v, 5) for k, v in ms.items()},
                     "persistent_ms_per_step": round(e0.elapsed_time(e1) / n, 5)})
        st.close()
        dm.close()
    return rows


def main():
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)  # the workload's 1000 RK4 steps (0.4 s timed)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--config", default="sw_l7",
                    choices=sorted(CONFIGS) + ["adjoint_l6", "adjoint_ocean_l6", "ensemble"])
    ap.add_argument("--adj-steps", type=int, default=500)
    ap.add_argument("--adj-ckpt", type=int, default=25)
    ap.add_argument("--adj-dirs", type=int, default=32)
    ap.add_argument("--ens-planar", type=int, default=192)
    ap.add_argument("--ens-sphere", type=int, default=64)
    ap.add_argument("--ens-sides", default="32,48,64,96,128,192,256", help="hex member sides to draw from")
    ap.add_argument("--ens-levels", default="5,6", help="sphere member levels to draw from")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default launch configuration")
    ap.add_argument("--min-timed-s", type=float, default=1.5,
                    help="repeat the timed region until this many seconds of it ran (median reported)")
    ap.add_argument("--no-extras", action="store_true",
                    help="headline workload only (no adjoint, 60-level ocean and ensemble objects)")
    ap.add_argument("--ref-budget-s", type=float, default=90.0,
                    help="reference arm: CPU seconds per process for warm-up + timed steps")
    ap.add_argument("--ref-procs", type=int, default=0, help="reference arm: processes (0 = all cores)")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "gb300":
        log("note: fewer than 3 warm-up steps")
    if args.config == "adjoint_l6":
        out = adjoint_arm(args)
    elif args.config == "adjoint_ocean_l6":
        leg = ocean_adjoint_leg(args)
        out = {"metric": "adjoint/forward time ratio (ocean tracer RK4, level-6 sphere, 60 levels x 3 tracers)",
               "value": leg["ratio"], "unit": "ratio", "higher_is_better": False, "n_gpus": 1, "steps": 20,
               "dtype": "f64", "data": "synthetic (seeded smooth fields, temperature unclipped)",
               "config": {"workload": leg["workload"]}, **{k: v for k, v in leg.items() if k != "workload"}}
    elif args.config == "ensemble":
        out = ensemble_arm(args)
    else:
        cfg = CONFIGS[args.config]
        if args.impl == "reference":
            out = reference_arm(args, cfg)
        else:
            out = gpu_arm(args, cfg)
            world, rank, _ = dist_setup()
            if out is not None and world == 1 and args.config == "sw_l7" and not args.no_extras:
                out.update(extras_for_line(args))
            if world > 1:
                import torch
                torch.distributed.barrier()
                torch.distributed.destroy_process_group()
    if out is not None:
        print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
