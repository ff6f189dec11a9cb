#!/usr/bin/env python3
"""Benchmark of chiML's time-step loop on GB300: Gcell-updates/s and HBM roofline.

Workload: the 3-D dispersive configuration (256^3 cells, 12-cell CPML, 16
seeded uniaxial ellipsoids, a Drude + two-Lorentz metal sphere, an x-polarised TFSF
plane wave along +z, a 150-frequency DFT flux box), generated by chiml_gb300.configs.config2.
One step is one full time step (H half + E half + detectors + DFT).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload c2|c1|c3|c4|c5]

The other workloads: c1 (2-D TMz 400^2), c3 (3-D Maxwell-Liouville 192^3), c4 (batched
sweep of 96 2-D emitter sheets), c5 (3-D mixed scene 640x640x320 with a four-level emitter
sheet; its CPU legs run a 160x160x80 crop).

Every line carries `fp64_error`: the split form against the FP64 form on the workload's
scene run to its last step (c1 and the c4 members at full size, c2 at 128^3, c3 at 96^3,
c5 on the crop), the worst relative L2 of each data column group of the detector, flux and
emitter output files.

`value` is the split form (fields, CPML and polarisations in FP32; DFT sums and
emitter density matrices as float-float pairs; TFSF lines in FP64) with all state
resident in HBM; `fp64` is the same
workload in FP64 (the parity form). `e2e` times the public C ABI end to end:
chiml_create (JSON read, plan, upload), the K steps, chiml_finalize (flux integration
on the device, download and file writes). Under torchrun every rank runs its own replica (the
single-domain path does not shard); value sums cells x steps over ranks and
divides by the slowest rank's time.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_DEFAULT = 256

# DRAM bytes of one launch per physical cell, split form of this workload, measured with
# ncu (dram__bytes_read.sum + dram__bytes_write.sum, --cache-control none) at 256^3:
# H pass 736.8 MB; E pass 946.3 MB (oriented-dipole P kernel 97.4 MB + the pass with its
# inline dispersive cells 848.9 MB).
MEASURED_TRAFFIC_PER_CELL = {"h_pass": 736.8e6 / 16777216, "e_pass": 946.3e6 / 16777216}
TRAFFIC_CAPTURE = "256^3, split form"


NOMINAL_HBM_GBS = 7900.0  # GB300 HBM3e nominal bandwidth, reported beside the measured copy peak


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            parts = [p.strip() for p in l.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def _dist():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


# The workloads: the default is the 3-D anisotropic + dispersive scene the headline
# metric is quoted on; c1 (2-D TMz), c3 (3-D Maxwell-Liouville), c4 (batched sweep of
# 2-D emitter sheets) and c5 (large 3-D mixed scene) are the other configurations.
WORKLOADS = {
    "c2": ("Gcell-updates/s (FP32/FP64-split, 3-D dispersive 256^3)",
           "3-D anisotropic + dispersive: %s cells, 12-cell CPML, 16 uniaxial ellipsoids, Drude+2-Lorentz sphere, "
           "x-polarised TFSF plane wave at 550 nm, DFT flux box x 150 freqs", 256, "config2"),
    "c1": ("Gcell-updates/s (FP32/FP64-split, 2-D TMz 400^2)",
           "2-D TMz: %s cells, 20-cell CPML, dielectric disk, Ez point source, 8 point detectors, flux line x 100 freqs",
           400, "config1"),
    "c3": ("Gcell-updates/s (FP32 fields, float-float density matrices, 3-D Maxwell-Liouville 192^3)",
           "3-D Maxwell-Liouville: %s cells, 12-cell CPML, 20-cell slab of 3-level ladder emitters (9 ensemble members "
           "per cell from 20 meV Gaussian broadening), 1e26 m^-3, Ez plane source at 2.1 eV, flux plane x 50 freqs",
           192, "config3"),
    "c5": ("Gcell-updates/s (FP32 fields, float-float density matrices, 3-D mixed 640x640x320)",
           "3-D mixed: %s cells, dx=4 nm, 16-cell CPML, 16 uniaxial ellipsoids, Drude film, 10-cell sheet of 4-level "
           "emitters (1e26 m^-3), p-polarised TFSF pulse along (1,1,3) at 550 nm, 6 DFT flux planes x 200 freqs",
           640, "config5"),
}

# Config 5's CPU samples run on a 160 x 160 x 80 crop of the same scene (the full 131 M-cell
# grid needs minutes of host set-up per oracle run).
C5_CROP = dict(n=160, nz=80, pml=8, nell=4, film_cells=4, sheet_cells=4)
C5_CROP_STEPS = 1600  # the pulse has passed every flux plane of the crop by then

# The FP64-vs-split accuracy check of each workload: the same scene at a size both forms
# run to its last step in seconds, compared per data column of every output file.
# c1 and the c4 members run at their full size and step count.
ERROR_SCENES = {
    "c1": ("the full workload (400^2, 4000 steps)", "config1", {}),
    "c2": ("the scene at 128^3, 5000 steps", "config2", dict(n=128, steps=5000)),
    "c3": ("the scene at 96^3 (20-cell emitter slab), 8000 steps", "config3", dict(n=96, steps=8000)),
    "c5": ("the 160x160x80 crop of the scene, 1600 steps", "config5", dict(steps=C5_CROP_STEPS, **C5_CROP)),
}


def _dims(name, n):
    if name == "c1":
        return "%d^2" % n
    if name == "c5":
        return "%dx%dx%d" % (n, n, n // 2)
    return "%d^3" % n


def _metric(name, n):
    """The workload's metric name, with its grid size when --n changes it."""
    return WORKLOADS[name][0].replace(_dims(name, WORKLOADS[name][2]), _dims(name, n))


def _workload(n, steps, name="c2"):
    from chiml_gb300 import configs
    if name == "c5":
        return configs.config5(n=n, nz=n // 2, steps=steps)
    return getattr(configs, WORKLOADS[name][3])(n=n, steps=steps)


def _cpu_sample_config(args, work, cfg_path, steps):
    """(config path, description) of the input the CPU legs time: the workload itself, or
    for c5 the crop."""
    if args.workload != "c5":
        return cfg_path, "the full workload"
    from chiml_gb300 import configs
    path = configs.write_json(configs.config5(steps=steps, **C5_CROP), os.path.join(work, "crop.json"))
    return path, "the %dx%dx%d crop of the workload" % (C5_CROP["n"], C5_CROP["n"], C5_CROP["nz"])


def _run_both(paths, work, local, graph, tag):
    """Runs every input to its last step in FP64 and in the split form; returns the
    per-class worst relative L2 of the split outputs against the FP64 ones."""
    from chiml_gb300 import Simulation
    from chiml_gb300.outfiles import error_summary
    worst = {"fields": None, "flux": None, "populations": None}
    for i, path in enumerate(paths):
        dirs = {}
        for prec in ("fp64", "split"):
            dirs[prec] = os.path.join(work, "%s_%d_%s" % (tag, i, prec))
            sim = Simulation(path, precision=prec, device=local, steps_per_graph=graph, out_dir=dirs[prec])
            sim.step()
            sim.finalize()
            sim.close()
        for k, v in error_summary(dirs["fp64"], dirs["split"]).items():
            if v is not None:
                worst[k] = v if worst[k] is None else max(worst[k], v)
    return {k: (float("%.3g" % v) if v is not None else None) for k, v in worst.items()}


def fp64_error(workload, work, local, graph, members=4):
    """The split form's error against the FP64 form on the workload's scene (ERROR_SCENES;
    for c4, the first ``members`` members of the sweep at full size): worst relative L2 per
    data column group over the detector fields, the flux spectra and the emitter outputs."""
    from chiml_gb300 import configs
    t0 = time.perf_counter()
    if workload == "c4":
        what = "the first %d members of the sweep, full size, 6000 steps" % members
        paths = _c4_members(os.path.join(work, "err_c4"), members, 6000)
    else:
        what, fn, kw = ERROR_SCENES[workload]
        paths = [configs.write_json(getattr(configs, fn)(**kw), os.path.join(work, "err_%s.json" % workload))]
    out = _run_both(paths, work, local, graph, "err_" + workload)
    out["scene"] = what
    out["compared"] = "split vs FP64 outputs, relative L2 of each data column group (worst per class)"
    out["seconds"] = round(time.perf_counter() - t0, 1)
    return out


def _time_steps(sim, k, torch):
    stream = torch.cuda.ExternalStream(sim.stream)
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    sim.sync()
    torch.cuda.synchronize()
    a.record(stream)
    sim.step(k)
    b.record(stream)
    b.synchronize()
    sim.sync()
    return a.elapsed_time(b)


def run_ours(args):
    import torch
    from chiml_gb300 import Simulation, configs

    world, rank, local = _dist()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    n = args.n
    total_steps = args.warmup + args.steps + args.profile_steps + 2
    work = tempfile.mkdtemp(prefix="chiml_bench_")
    cfg_path = configs.write_json(_workload(n, total_steps, args.workload), os.path.join(work, "in.json"))
    peak, peak_kind = _peaks()
    results = {}
    for prec in ("split", "fp64"):
        out_dir = os.path.join(work, prec)
        t_create0 = time.perf_counter()
        sim = Simulation(cfg_path, precision=prec, device=local, steps_per_graph=args.graph, out_dir=out_dir)
        t_create = time.perf_counter() - t_create0
        st = sim.stats()
        sim.step(args.warmup)
        sim.sync()
        sampler = ClockSampler(local) if prec == "split" else None
        if sampler:
            sampler.start()
        if dist:
            dist.barrier()
        ms = _time_steps(sim, args.steps, torch)
        if dist:
            dist.barrier()
        clocks = sampler.stop() if sampler else None
        prof = sim.profile_steps(args.profile_steps)
        st = sim.stats()
        results[prec] = {"ms": ms, "stats": st, "prof": prof, "clocks": clocks, "create_s": t_create}
        sim.close()
    cells = results["split"]["stats"].cells_physical
    ms_max = results["split"]["ms"]
    if dist:
        t = torch.tensor([ms_max], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms_max = float(t.item())
    value = world * cells * args.steps / (ms_max * 1e-3) / 1e9

    # per-kernel roofline of the split form from the event-timed profile steps
    sp = results["split"]
    prof = sp["prof"]
    nprof = max(args.profile_steps, 1)
    per_launch = {k: v / nprof for k, v in prof.items()}
    kbytes = {"h_pass": sp["stats"].bytes_h_pass, "e_pass": sp["stats"].bytes_e_pass}
    dft_ms = sum(v for k, v in per_launch.items() if k.startswith("dft"))
    dom = max(("h_pass", "e_pass", "dft"), key=lambda k: dft_ms if k == "dft" else per_launch.get(k, 0.0))
    dom_ms = dft_ms if dom == "dft" else per_launch[dom]
    dom_bytes = sp["stats"].bytes_dft if dom == "dft" else kbytes[dom]
    achieved = dom_bytes / (dom_ms * 1e-3) / 1e9
    # DRAM traffic is known from an ncu capture of this workload's scene only (c2)
    traffic, traffic_src = None, "no ncu DRAM capture of this workload's pass kernels"
    if args.workload == "c2" and dom in MEASURED_TRAFFIC_PER_CELL:
        traffic = round(MEASURED_TRAFFIC_PER_CELL[dom] * cells, 0)
        traffic_src = "ncu dram bytes per cell of this scene (captured at %s), times this run's cells" % TRAFFIC_CAPTURE
    fp = results["fp64"]
    fp_value = cells * args.steps / (fp["ms"] * 1e-3) / 1e9
    fp_prof = {k: v / nprof for k, v in fp["prof"].items()}

    # end to end through the C ABI with host buffers: create + K steps + finalize
    e2e = None
    if rank == 0 and not args.no_e2e:
        out_dir = os.path.join(work, "e2e")
        t0 = time.perf_counter()
        sim = Simulation(cfg_path, precision="split", device=local, steps_per_graph=args.graph, out_dir=out_dir)
        sim.step(args.steps)
        sim.finalize()
        t1 = time.perf_counter()
        s = sim.stats()
        sim.close()
        e2e = {"value": cells * args.steps / (t1 - t0) / 1e9, "unit": "Gcell-updates/s",
               "h2d_bytes_per_step": s.h2d_bytes / args.steps, "d2h_bytes_per_step": s.d2h_bytes / args.steps,
               "seconds": t1 - t0, "includes": "JSON read, plan build, upload, steps, flux integration, download, file writes",
               "seconds_plan": round(s.seconds_plan, 3), "seconds_upload": round(s.seconds_upload, 3),
               "seconds_finalize": round(s.seconds_finalize, 3)}

    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu_path, what = _cpu_sample_config(args, work, cfg_path, total_steps)
        cpu = cpu_baseline(cpu_path, what, args.cpu_seconds)

    err = fp64_error(args.workload, work, local, args.graph) if (rank == 0 and not args.no_check) else None

    if rank == 0:
        launches = sp["stats"].kernels_per_step * args.steps
        line = {
            "metric": _metric(args.workload, n),
            "value": round(value, 3),
            "unit": "Gcell-updates/s",
            "n_gpus": world,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": round(ms_max / args.steps, 4),
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f32 fields; DFT sums and emitter density matrices as float-float (f32 pairs)",
            "data": "synthetic (seeded PCG64 geometry, chiml_gb300.configs.%s)" % WORKLOADS[args.workload][3],
            "config": {
                "workload": WORKLOADS[args.workload][1] % _dims(args.workload, n),
                "cells": cells,
                "precision": "split",
                "l2": "inputs larger than L2 (%.0f MB of field state vs 129 MB L2)" % (sp["stats"].device_bytes / 1e6),
                "graph_steps": args.graph,
                "dft_fold": ("staggered: the point tiles of each DFT table fold in K/4 groups, one group every 4 "
                             "samples (K = 256 samples per fold), so any window of steps carries its share of the "
                             "fold; %d steps carry %d group folds" % (args.steps, args.steps // 4)),
                "parallelism": "replicas" if world > 1 else "single GPU",
            },
            "fp64": {"value": round(fp_value, 3), "unit": "Gcell-updates/s", "ms_per_step": round(fp["ms"] / args.steps, 4),
                     "split_speedup": round(value / world / fp_value, 3),
                     "kernel_ms": {k: round(v, 4) for k, v in fp_prof.items()}},
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1), "peak": peak,
                         "unit": "GB/s", "frac": round(achieved / peak, 4), "peak_kind": peak_kind,
                         "frac_of_nominal": round(achieved / NOMINAL_HBM_GBS, 4),
                         "traffic": traffic,
                         "traffic_source": traffic_src,
                         "bytes_per_launch": dom_bytes,
                         "step_bytes_per_cell": round(sp["stats"].bytes_per_cell_update, 2),
                         "kernel_ms": {k: round(v, 4) for k, v in per_launch.items()}},
            "gpu_launches": launches,
            "clocks": sp["clocks"],
            "e2e": e2e,
            "cpu_baseline": cpu,
        }
        if err:
            line["fp64_error"] = err
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


def cpu_baseline(cfg_path, what, seconds):
    """The oracle (FP64 CPU port of the reference loop) on the machine's host cores, on a bounded
    sample: as many steps of cfg_path as fit in ``seconds``."""
    import oracle
    from chiml_gb300 import build
    build.build_oracle()
    sim = oracle.OracleSim(cfg_path)
    cells = sim.cells_physical()
    done = sim.step(1)
    t0 = time.perf_counter()
    n = 0
    while time.perf_counter() - t0 < seconds and done < sim.steps_total:
        done = sim.step(1)
        n += 1
    dt = time.perf_counter() - t0
    sim.close()
    v = cells * n / dt / 1e9
    return {"value": round(v, 5), "unit": "Gcell-updates/s", "cores": oracle.threads(), "kind": "port",
            "sample": "%d steps of %s (%d cells) in FP64 (setup excluded), %.1f s" % (n, what, cells, dt)}


def run_reference(args):
    world, rank, local = _dist()
    if rank != 0:
        return
    import oracle
    from chiml_gb300 import build, configs
    build.build_oracle()
    work = tempfile.mkdtemp(prefix="chiml_ref_")
    total = args.warmup + args.steps + 2
    cfg_path = configs.write_json(_workload(args.n, total, args.workload), os.path.join(work, "in.json"))
    cfg_path, what = _cpu_sample_config(args, work, cfg_path, total)
    sim = oracle.OracleSim(cfg_path)
    sim.step(args.warmup)
    cells = sim.cells_physical()
    per_step = []
    t_all = time.perf_counter()
    for _ in range(args.steps):
        t0 = time.perf_counter()
        sim.step(1)
        per_step.append(time.perf_counter() - t0)
    total_s = time.perf_counter() - t_all
    sim.close()
    v = cells * args.steps / total_s / 1e9
    line = {
        "metric": _metric(args.workload, args.n),
        "value": round(v, 5),
        "unit": "Gcell-updates/s",
        "impl": "reference",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(1e3 * total_s / args.steps, 3),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (seeded PCG64 geometry, chiml_gb300.configs.%s)" % WORKLOADS[args.workload][3],
        "config": {"workload": WORKLOADS[args.workload][1] % _dims(args.workload, args.n), "cells": cells},
        "cpu_baseline": {"value": round(v, 5), "unit": "Gcell-updates/s", "cores": oracle.threads(), "kind": "port",
                         "sample": "%d timed steps of %s after %d warm-up steps" % (args.steps, what, args.warmup)},
        "e2e": {"value": round(v, 5), "unit": "Gcell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def _c4_members(work, n_members, steps):
    from chiml_gb300 import configs
    paths = []
    for name, cfg in configs.config4(n=n_members, steps=steps):
        d = os.path.join(work, name)
        os.makedirs(d, exist_ok=True)
        paths.append(configs.write_json(cfg, os.path.join(d, "in.json")))
    return paths


C4_METRIC = "aggregate Gcell-updates/s (FP32 fields, float-float density matrices, batched sweep of 2-D emitter sheets)"
C4_WORKLOAD = ("batched sweep: %d 2-D TMz simulations, sides drawn from {192..768}, 16-cell CPML, 10-cell sheet of "
               "2-level emitters, detuning -100..+100 meV x density 1e25..1e26 m^-3, T2 = 30 fs")


def run_batch(args):
    """The sweep as one batch (packed launches per kind of work, graph-captured), against
    the same members run one after another through the single-simulation API."""
    world, rank, local = _dist()
    import torch
    from chiml_gb300 import Batch, Simulation
    torch.cuda.set_device(local)
    if rank != 0:
        return
    work = tempfile.mkdtemp(prefix="chiml_c4_")
    total = args.warmup + args.steps
    paths = _c4_members(work, args.members, total)
    t0 = time.perf_counter()
    b = Batch(paths, precision="split", device=local, steps_per_graph=args.graph)
    t_create = time.perf_counter() - t0
    sts = [b.member_stats(i) for i in range(len(paths))]
    cells = sum(st.cells_physical for st in sts)
    step_bytes = sum(st.bytes_per_cell_update * st.cells_physical for st in sts)
    b.step(args.warmup)
    sampler = ClockSampler(local)
    sampler.start()
    t0 = time.perf_counter()
    b.step(args.steps)
    t_batch = time.perf_counter() - t0
    clocks = sampler.stop()
    b.close()
    value = cells * args.steps / t_batch / 1e9
    peak, peak_kind = _peaks()
    achieved = step_bytes * args.steps / t_batch / 1e9
    # the members alone, one after another (each with its own graphs)
    t_seq = 0.0
    for p in paths:
        sim = Simulation(p, precision="split", device=local, steps_per_graph=args.graph, out_dir=os.path.join(work, "seq"))
        sim.step(args.warmup)
        sim.sync()
        t0 = time.perf_counter()
        sim.step(args.steps)
        sim.sync()
        t_seq += time.perf_counter() - t0
        sim.close()
    seq_value = cells * args.steps / t_seq / 1e9
    e2e = None
    if not args.no_e2e:
        t0 = time.perf_counter()
        b2 = Batch(paths, precision="split", device=local, steps_per_graph=args.graph, out_dir=os.path.join(work, "e2e"))
        b2.run()
        b2.finalize()
        t_e2e = time.perf_counter() - t0
        s2 = [b2.member_stats(i) for i in range(len(paths))]
        b2.close()
        e2e = {"value": cells * total / t_e2e / 1e9, "unit": "Gcell-updates/s",
               "h2d_bytes_per_step": sum(x.h2d_bytes for x in s2) / total,
               "d2h_bytes_per_step": sum(x.d2h_bytes for x in s2) / total, "seconds": t_e2e,
               "includes": "JSON reads, plans, uploads, %d steps of every member, downloads, file writes" % total}
    cpu = None
    if not args.no_cpu:
        cpu = batch_cpu_sample(paths, args.cpu_seconds)
    err = None if args.no_check else fp64_error("c4", work, local, args.graph)
    line = {
        "metric": C4_METRIC, "value": round(value, 3), "unit": "Gcell-updates/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * t_batch / args.steps, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 fields; DFT sums and emitter density matrices as float-float (f32 pairs)",
        "data": "synthetic (seeded PCG64 sizes and sweep values, chiml_gb300.configs.config4)",
        "config": {"workload": C4_WORKLOAD % len(paths), "members": len(paths), "cells": cells,
                   "graph_steps": args.graph, "create_s": round(t_create, 2),
                   "l2": "inputs larger than L2 (%d cells of field state)" % cells},
        "sequential": {"value": round(seq_value, 3), "unit": "Gcell-updates/s", "seconds": round(t_seq, 3),
                       "batch_speedup": round(value / seq_value, 2)},
        "roofline": {"bound": "hbm", "kernel": "whole packed step", "achieved": round(achieved, 1), "peak": peak,
                     "unit": "GB/s", "frac": round(achieved / peak, 4), "peak_kind": peak_kind,
                     "frac_of_nominal": round(achieved / NOMINAL_HBM_GBS, 4), "traffic": None,
                     "bytes_per_step": step_bytes},
        "gpu_launches": None, "clocks": clocks, "e2e": e2e, "cpu_baseline": cpu,
    }
    if err:
        line["fp64_error"] = err
    print(json.dumps(line))


def batch_cpu_sample(paths, seconds):
    """The oracle on the sweep's members in turn, a bounded number of steps each."""
    import oracle
    from chiml_gb300 import build
    build.build_oracle()
    cells_done, t_used, members = 0, 0.0, 0
    per = max(seconds / len(paths), 0.05)
    for p in paths:
        sim = oracle.OracleSim(p)
        done = sim.step(1)
        st = sim.cells_physical()
        t0 = time.perf_counter()
        n = 0
        while time.perf_counter() - t0 < per and done < sim.steps_total:
            done = sim.step(1)
            n += 1
        t_used += time.perf_counter() - t0
        cells_done += st * n
        members += 1
        sim.close()
    return {"value": round(cells_done / t_used / 1e9, 5), "unit": "Gcell-updates/s", "cores": oracle.threads(),
            "kind": "port", "sample": "every member of the sweep for %.2f s each (%d members)" % (per, members)}


def run_batch_reference(args):
    world, rank, local = _dist()
    if rank != 0:
        return
    import oracle
    from chiml_gb300 import build
    build.build_oracle()
    work = tempfile.mkdtemp(prefix="chiml_c4_ref_")
    paths = _c4_members(work, args.members, args.warmup + args.steps)
    cells, t_used = 0, 0.0
    for p in paths:
        sim = oracle.OracleSim(p)
        sim.step(args.warmup)
        t0 = time.perf_counter()
        sim.step(args.steps)
        t_used += time.perf_counter() - t0
        cells += sim.cells_physical() * args.steps
        sim.close()
    v = cells / t_used / 1e9
    print(json.dumps({
        "metric": C4_METRIC, "value": round(v, 5), "unit": "Gcell-updates/s", "impl": "reference", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * t_used / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded PCG64 sizes and sweep values, chiml_gb300.configs.config4)",
        "config": {"workload": C4_WORKLOAD % len(paths), "members": len(paths)},
        "cpu_baseline": {"value": round(v, 5), "unit": "Gcell-updates/s", "cores": oracle.threads(), "kind": "port",
                         "sample": "every member run alone for %d timed steps after %d warm-up steps" % (args.steps, args.warmup)},
        "e2e": {"value": round(v, 5), "unit": "Gcell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=512)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS) + ["c4"], default="c2",
                    help="c2 (default, the headline), c1, c3, or c4 (the batched sweep)")
    ap.add_argument("--n", type=int, default=None, help="cells per side (default: the workload's)")
    ap.add_argument("--members", type=int, default=96, help="c4: simulations in the sweep")
    ap.add_argument("--graph", type=int, default=20, help="steps per CUDA graph")
    ap.add_argument("--profile-steps", type=int, default=256)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-check", action="store_true", help="skip the FP64-vs-split accuracy check")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be at least 3")
    if args.n is None:
        args.n = WORKLOADS[args.workload][2] if args.workload in WORKLOADS else 0
    if args.workload == "c4":
        if args.impl == "reference":
            run_batch_reference(args)
        else:
            run_batch(args)
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
