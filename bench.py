#!/usr/bin/env python3
"""Benchmark of chiML's time-step loop on GB300: Gcell-updates/s and HBM roofline.

Workload: the 3-D dispersive configuration (256^3 cells, 12-cell CPML, 16
seeded ellipsoids, a Drude + two-Lorentz metal sphere, a plane Ex source, a
150-frequency DFT flux box), generated by chiml_gb300.configs.config2.
One step is one full time step (H half + E half + detectors + DFT).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

`value` is the FP32/FP64-split form (fields, CPML and polarisations in FP32,
DFT accumulators in FP64) with all state resident in HBM; `fp64` is the same
workload in FP64 (the parity form). `e2e` times the public C ABI end to end:
chiml_create (JSON read, plan, upload), the K steps, chiml_finalize (download
and file writes). Under torchrun every rank runs its own replica (the
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
# H pass 749.6 MB, E pass (main kernel 757.5 MB + dispersive-cell list 41.1 MB) 798.6 MB.
MEASURED_TRAFFIC_PER_CELL = {"h_pass": 749.6e6 / 16777216, "e_pass": 798.6e6 / 16777216}


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


def _workload(n, steps):
    from chiml_gb300 import configs
    return configs.config2(n=n, steps=steps)


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
    cfg_path = configs.write_json(_workload(n, total_steps), os.path.join(work, "in.json"))
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
               "seconds": t1 - t0, "includes": "JSON read, plan build, upload, steps, download, file writes"}

    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = cpu_baseline(cfg_path, cells, args.cpu_seconds)

    if rank == 0:
        launches = sp["stats"].kernels_per_step * args.steps
        line = {
            "metric": "Gcell-updates/s (FP32/FP64-split, 3-D dispersive 256^3)",
            "value": round(value, 3),
            "unit": "Gcell-updates/s",
            "n_gpus": world,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": round(ms_max / args.steps, 4),
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f32 fields, f64 DFT accumulators",
            "data": "synthetic (seeded PCG64 geometry, chiml_gb300.configs.config2)",
            "config": {
                "workload": "3-D dispersive: %d^3 cells, 12-cell CPML, 16 ellipsoids, Drude+2-Lorentz sphere, "
                            "plane Ex source, DFT flux box x 150 freqs" % n,
                "cells": cells,
                "precision": "split",
                "l2": "inputs larger than L2 (%.0f MB of field state vs 129 MB L2)" % (sp["stats"].device_bytes / 1e6),
                "graph_steps": args.graph,
                "parallelism": "replicas" if world > 1 else "single GPU",
            },
            "fp64": {"value": round(fp_value, 3), "unit": "Gcell-updates/s", "ms_per_step": round(fp["ms"] / args.steps, 4),
                     "split_speedup": round(value / world / fp_value, 3),
                     "kernel_ms": {k: round(v, 4) for k, v in fp_prof.items()}},
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1), "peak": peak,
                         "unit": "GB/s", "frac": round(achieved / peak, 4), "peak_kind": peak_kind,
                         "traffic": (round(MEASURED_TRAFFIC_PER_CELL[dom] * cells, 0)
                                     if dom in MEASURED_TRAFFIC_PER_CELL else None),
                         "traffic_source": "ncu dram bytes per cell at 256^3, scaled to this workload's cells",
                         "bytes_per_launch": dom_bytes,
                         "step_bytes_per_cell": round(sp["stats"].bytes_per_cell_update, 2),
                         "kernel_ms": {k: round(v, 4) for k, v in per_launch.items()}},
            "gpu_launches": launches,
            "clocks": sp["clocks"],
            "e2e": e2e,
            "cpu_baseline": cpu,
        }
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


def cpu_baseline(cfg_path, cells, seconds):
    """The oracle (FP64 CPU port of the reference loop) on the machine's host cores, on a bounded sample."""
    import oracle
    from chiml_gb300 import build
    build.build_oracle()
    sim = oracle.OracleSim(cfg_path)
    sim.step(1)
    t0 = time.perf_counter()
    n = 0
    while time.perf_counter() - t0 < seconds:
        sim.step(1)
        n += 1
    dt = time.perf_counter() - t0
    sim.close()
    v = cells * n / dt / 1e9
    return {"value": round(v, 5), "unit": "Gcell-updates/s", "cores": oracle.threads(), "kind": "port",
            "sample": "%d steps of the full %d-cell workload in FP64 (setup excluded), %.1f s" % (n, cells, dt)}


def run_reference(args):
    world, rank, local = _dist()
    if rank != 0:
        return
    import oracle
    from chiml_gb300 import build, configs
    build.build_oracle()
    work = tempfile.mkdtemp(prefix="chiml_ref_")
    total = args.warmup + args.steps + 2
    cfg_path = configs.write_json(_workload(args.n, total), os.path.join(work, "in.json"))
    sim = oracle.OracleSim(cfg_path)
    sim.step(args.warmup)
    cells = (args.n) ** 3
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
        "metric": "Gcell-updates/s (FP32/FP64-split, 3-D dispersive 256^3)",
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
        "data": "synthetic (seeded PCG64 geometry, chiml_gb300.configs.config2)",
        "config": {"workload": "3-D dispersive: %d^3 cells, same input as the GPU arm" % args.n, "cells": cells},
        "cpu_baseline": {"value": round(v, 5), "unit": "Gcell-updates/s", "cores": oracle.threads(), "kind": "port",
                         "sample": "%d timed steps of the full workload after %d warm-up steps" % (args.steps, args.warmup)},
        "e2e": {"value": round(v, 5), "unit": "Gcell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=512)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--n", type=int, default=N_DEFAULT, help="cells per side")
    ap.add_argument("--graph", type=int, default=20, help="steps per CUDA graph")
    ap.add_argument("--profile-steps", type=int, default=256)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be at least 3")
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
