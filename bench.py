#!/usr/bin/env python
"""Benchmark: collisions/s of the multigroup k-eigenvalue transport on one GB300.

Workload (default): config 1 -- 51x51 pin lattice, 200 cm tall in 10 axial
zones, 3 materials, 7 groups, delta tracking, 1,000,000 histories per
generation, 51x51x20 collision flux tally -- in the FP32-tracking/FP64-tally
mode.  One step = one power-iteration generation: transport of the whole bank
plus the fission-bank sort, weight normalisation, entropy and tally
statistics, all resident in HBM.

  value : collisions/s over K timed generations, device time (CUDA events on
          the engine's stream), inputs already in HBM.
  e2e   : the same metric through the reference-facing call (abx_transport,
          GpuDeltaTracker.transport) with the bank in pinned host memory:
          H2D of the bank and D2H of the fission bank inside the timed region.
  --impl reference : the CPU restatement of the reference (oracle, FP64) on all
          host cores; the reference itself cannot be built here.

Under torchrun with N>1 every rank runs an independent replica (its own seed);
the path has no exchange step, so there is no collective on the data path.
"""
import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# algorithmic bytes per unit of work (SoA state load + store), per precision
BYTES = {"fp64": {"flight": 112, "collision": 160, "site": 96},
         "mixed": {"flight": 76, "collision": 108, "site": 96}}
KERNELS_PER_GEN = 8  # step_begin, transport, 3 x scan, next_bank, tally_record, gen_end


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampling of SM clock and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.p = None
        return self

    def __exit__(self, *a):
        self.rows = []
        if self.p is None:
            return
        self.p.terminate()
        try:
            out, _ = self.p.communicate(timeout=5)
        except Exception:
            self.p.kill()
            out = ""
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) >= 9:
                self.rows.append(f)

    def summary(self):
        rows = getattr(self, "rows", [])
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({n for r in rows for n, v in zip(names, r[5:9]) if v.lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def dist_setup(n):
    if n <= 1 or "RANK" not in os.environ:
        return 0, 1, 0, None
    import torch
    import torch.distributed as dist
    rank, world = int(os.environ["RANK"]), int(os.environ["WORLD_SIZE"])
    local = int(os.environ.get("LOCAL_RANK", rank))
    torch.cuda.set_device(local)
    dist.init_process_group("nccl")
    return rank, world, local, dist


def cpu_baseline(config, nhist, precision_label="fp64"):
    """The oracle (CPU restatement of the reference, FP64) on all host cores, one
    bounded transport sample of the same workload."""
    import oracle
    from abeille_gb300 import decks
    built = decks.CONFIGS[config](nparticles=nhist).build(precision="fp64")
    o = oracle.Oracle(built, nthreads=oracle.cores())
    bank = o.sample_sources(0, nhist)
    t0 = time.perf_counter()
    _, sc = o.transport(bank, 1.0, True)
    dt = time.perf_counter() - t0
    return sc["collisions"] / dt, oracle.cores(), sc["collisions"], dt


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    vals, coll, secs = [], 0, 0.0
    cores = None
    for i in range(args.warmup + args.steps):
        v, cores, c, dt = cpu_baseline(args.config, args.ref_sample)
        if i >= args.warmup:
            vals.append(v)
            coll += c
            secs += dt
    value = coll / secs
    line = {
        "metric": "collisions/s", "value": value, "unit": "collisions/s", "impl": "reference",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * secs / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"config{args.config}", "histories_per_step": args.ref_sample,
                   "tracking": "delta", "precision": "fp64"},
        "cpu_baseline": {"value": value, "unit": "collisions/s", "cores": cores, "kind": "port",
                         "sample": f"{args.ref_sample} first-generation histories of config {args.config} per step"},
        "e2e": {"value": value, "unit": "collisions/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def e2e_measure(eng, bank_np, steps, warmup):
    """abx_transport with the bank and the site buffer in pinned host memory."""
    import numpy as np
    import torch
    from abeille_gb300 import SITE_DTYPE, abi
    n = bank_np.size
    cap = 3 * n + 4096
    pin_b = torch.empty(bank_np.nbytes, dtype=torch.uint8, pin_memory=True)
    pin_s = torch.empty(cap * SITE_DTYPE.itemsize, dtype=torch.uint8, pin_memory=True)
    bview = np.frombuffer(pin_b.numpy(), dtype=bank_np.dtype)
    bview[:] = bank_np
    lib = eng.lib
    ns = C.c_size_t()
    sc = abi.Scores()
    coll, secs, h2d, d2h = 0, 0.0, 0, 0
    for i in range(warmup + steps):
        t0 = time.perf_counter()
        rc = lib.abx_transport(eng.ctx, C.cast(pin_b.data_ptr(), C.POINTER(abi.Particle)), n, 1.0, 1,
                               C.cast(pin_s.data_ptr(), C.POINTER(abi.Site)), cap, C.byref(ns), C.byref(sc))
        dt = time.perf_counter() - t0
        abi.check(rc, lib)
        if i >= warmup:
            coll += sc.collisions
            secs += dt
            h2d = n * C.sizeof(abi.Particle)
            d2h = ns.value * C.sizeof(abi.Site) + 256
    return coll / secs, h2d, d2h


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", type=int, default=1)
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--particles", type=int, default=None)
    ap.add_argument("--ref-sample", type=int, default=100000)
    ap.add_argument("--cpu-sample", type=int, default=200000)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)

    import __graft_entry__
    __graft_entry__.build()
    from abeille_gb300 import Engine, decks

    rank, world, local, dist = dist_setup(args.gpus)
    npart = args.particles or {0: 10000, 1: 1000000, 2: 2000000}[args.config]
    builder = decks.CONFIGS[args.config](nparticles=npart)
    builder.seed = builder.seed + 7919 * rank  # independent replica per rank
    eng = Engine(builder.build(precision=args.precision), local)

    # L2 flush between generations, outside each generation's timed events
    from abeille_gb300 import abi as _abi
    _abi.check(eng.lib.abx_set_l2_flush(eng.ctx, L2_FLUSH_BYTES), eng.lib)
    # warm-up generations (untimed)
    eng.run_power_iteration(max(args.warmup, 1), 0)
    if dist:
        dist.barrier()
    with Clocks(local) as clk:
        t0 = time.perf_counter()
        stats, recs = eng.run_power_iteration_records(args.steps, 0)
        wall = time.perf_counter() - t0
    step_ms = sum(r["step_ms"] for r in recs)
    tr_ms = sum(r["transport_ms"] for r in recs)
    coll = sum(r["collisions"] for r in recs)
    flights = sum(r["flights"] for r in recs)
    sites = sum(r["sites"] for r in recs)
    if dist:
        import torch
        t = torch.tensor([step_ms / 1e3, float(coll)], dtype=torch.float64, device=f"cuda:{local}")
        tmax = t.clone()
        dist.all_reduce(tmax, op=dist.ReduceOp.MAX)
        dist.all_reduce(t, op=dist.ReduceOp.SUM)
        secs, coll_all = float(tmax[0]), float(t[1])
    else:
        secs, coll_all = step_ms / 1e3, float(coll)
    value = coll_all / secs

    e2e = None
    if not args.no_e2e:
        bank = eng.sample_sources(0, npart)
        v, h2d, d2h = e2e_measure(eng, bank, max(2, args.steps // 3), 1)
        e2e = {"value": v * world, "unit": "collisions/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h}

    if rank != 0:
        if dist:
            dist.barrier()
        return 0
    b = BYTES[args.precision]
    alg = flights * b["flight"] + coll * b["collision"] + sites * b["site"]
    achieved = alg / (tr_ms / 1e3) / 1e9
    peak, src = peaks()
    hist = sum(r["histories"] for r in recs) / max(len(recs), 1)
    tph = TRAFFIC_PER_HISTORY.get((args.config, args.precision))
    traffic = tph * hist if tph else None
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": traffic, "peak_source": src,
            "kernel": "transport_kernel", "algorithmic_bytes_per_launch": alg / max(len(recs), 1)}
    cpu = None
    if world == 1 and not args.no_cpu:
        v, cores, c, dt = cpu_baseline(args.config, args.cpu_sample)
        cpu = {"value": v, "unit": "collisions/s", "cores": cores, "kind": "port",
               "sample": f"{args.cpu_sample} first-generation histories of config {args.config}, FP64, one transport"}
    line = {
        "metric": "collisions/s", "value": value, "unit": "collisions/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": step_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32-track/f64-tally" if args.precision == "mixed" else "f64",
        "data": "synthetic",
        "config": {"workload": f"config{args.config}", "histories_per_generation": npart,
                   "tracking": "delta", "precision": args.precision,
                   "l2": f"flushed: {L2_FLUSH_BYTES >> 20} MiB written before each generation, outside its "
                   "timed events", "parallelism": f"replicas{world}"},
        "roofline": roof, "cpu_baseline": cpu, "e2e": e2e,
        "gpu_launches": KERNELS_PER_GEN * args.steps,
        "clocks": clk.summary(),
        "detail": {"flights": flights, "collisions": coll, "sites": sites, "transport_ms": tr_ms,
                   "wall_s": wall, "kcol_last": recs[-1]["kcol"], "lost": sum(r["lost"] for r in recs)},
    }
    print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
    return 0


# DRAM bytes (read + write) per history of a transport launch, from the ncu
# capture in profiles/transport_kernel_config1_mixed_300k.md (16.27 MB at
# 300,000 histories); the bank and site traffic grows with the histories.
TRAFFIC_PER_HISTORY = {(1, "mixed"): 16.27e6 / 3e5}
L2_FLUSH_BYTES = 256 << 20

if __name__ == "__main__":
    sys.exit(main())
