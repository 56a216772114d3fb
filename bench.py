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

# what each --config is (the synthetic decks of abeille_gb300.decks)
WORKLOADS = {
    0: "17x17 pin lattice, 2 materials, 7 groups, k-eigenvalue, 17x17x1 collision flux tally",
    1: "51x51 pins x 10 axial zones (200 cm), 3 materials, 7 groups, k-eigenvalue, 51x51x20 collision flux tally",
    2: "17x17 pins with fuel/gap/clad rings, 8 fuels, 70 groups with P1 scattering, k-eigenvalue, "
       "100x100x50 track-length flux tally",
    3: "4096 fixed-source slab boxes (1-4 slabs, G in 7/22/44), 10 batches each, 20x20x20 collision flux tallies",
    4: "request loop: fixed-source slab problems arriving as a Poisson stream",
}


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


def combine_replicas(dist, seconds, collisions, device):
    """Whole-job figures of N independent replicas: the slowest rank's device
    time and the collisions of all ranks (no data-path collective: only these
    two numbers cross ranks)."""
    if not dist:
        return seconds, float(collisions)
    import torch
    t = torch.tensor([seconds, float(collisions)], dtype=torch.float64, device=device)
    tmax = t.clone()
    dist.all_reduce(tmax, op=dist.ReduceOp.MAX)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(tmax[0]), float(t[1])


def host_cpu():
    """The host's CPU, for the baseline lines: architecture and, where
    /proc/cpuinfo names it, the model or the Arm part number."""
    import platform
    model = None
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                k, _, v = line.partition(":")
                if k.strip() in ("model name", "CPU part") and v.strip():
                    model = v.strip()
                    break
    except OSError:
        pass
    return f"{platform.machine()}" + (f" ({model})" if model else "")


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
        "config": {"workload": WORKLOADS[args.config], "deck": args.config, "histories_per_step": args.ref_sample,
                   "tracking": __import__("abeille_gb300.decks", fromlist=["CONFIGS"]).CONFIGS[args.config](
                       nparticles=1).tracking, "precision": "fp64"},
        "cpu_baseline": {"value": value, "unit": "collisions/s", "cores": cores, "kind": "port", "cpu": host_cpu(),
                         "sample": f"{args.ref_sample} first-generation histories of config {args.config} per step"},
        "e2e": {"value": value, "unit": "collisions/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def e2e_measure(eng, bank_np, kcol, steps, warmup):
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
        rc = lib.abx_transport(eng.ctx, C.cast(pin_b.data_ptr(), C.POINTER(abi.Particle)), n, kcol, 1,
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
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", type=int, default=1)
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--particles", type=int, default=None)
    ap.add_argument("--ref-sample", type=int, default=100000)
    ap.add_argument("--cpu-sample", type=int, default=200000)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64 comparison run of the mixed mode")
    ap.add_argument("--kernel", default="auto", choices=["auto", "history", "pool"],
                    help="configs 0-2: transport kernel (history: one lane per history; pool: event-sorted warps)")
    ap.add_argument("--tracking", default=None,
                    choices=["delta-tracking", "surface-tracking", "implicit-leakage-delta-tracking", "carter-tracking"])
    ap.add_argument("--problems", type=int, default=4096, help="config 3: problems in the batch")
    ap.add_argument("--per-problem-sample", type=int, default=128,
                    help="config 3/4: problems timed one launch per problem")
    ap.add_argument("--rates", default="200,1000,5000", help="config 4: Poisson arrival rates, requests/s")
    ap.add_argument("--duration", type=float, default=3.0, help="config 4: seconds of arrivals per rate")
    ap.add_argument("--warm", type=float, default=1.0,
                    help="config 4: seconds of arrivals at each rate before the measured ones (same server)")
    ap.add_argument("--budget-gb", type=float, default=150.0, help="config 4: HBM admission budget")
    ap.add_argument("--lanes", type=int, default=0, help="config 4: rounds on the GPU at once (0: the server's 3)")
    ap.add_argument("--quantum", type=int, default=0,
                    help="config 4: histories per warp before a block retires (0: the server's 256)")
    ap.add_argument("--autotune", type=int, default=-1,
                    help="configs 0-2: tune the transport launch shape on this many source histories first "
                         "(-1: one generation's histories; 0: off)")
    ap.add_argument("--zscore", type=int, default=0,
                    help="configs 0-2: compare mixed and FP64 over sets of this many replicas instead of timing")
    ap.add_argument("--zsets", type=int, default=1, help="with --zscore: replica sets per precision")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.zscore:
        return bench_zscore(args)
    if args.config == 3:
        return bench_batch(args)
    if args.config == 4:
        return bench_server(args)

    import __graft_entry__
    __graft_entry__.build()
    from abeille_gb300 import Engine, decks

    rank, world, local, dist = dist_setup(args.gpus)
    npart = args.particles or {0: 10000, 1: 1000000, 2: 2000000}[args.config]
    builder = decks.CONFIGS[args.config](nparticles=npart)
    if args.tracking:
        builder.tracking = args.tracking
    builder.seed = builder.seed + 7919 * rank  # independent replica per rank
    eng = Engine(builder.build(precision=args.precision), local)

    if args.kernel != "auto":
        eng.set_transport_kernel(args.kernel)
    shape = None
    if args.autotune:
        shape = eng.autotune(npart if args.autotune < 0 else args.autotune)
    kernel_used = eng.transport_kernel()
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
    secs, coll_all = combine_replicas(dist, step_ms / 1e3, coll, f"cuda:{local}")
    value = coll_all / secs

    e2e = None
    if not args.no_e2e:
        # the bank of the generation after the timed ones (the converged
        # source, the same workload as the timed generations)
        bank, kcol = eng.read_source_bank()
        v, h2d, d2h = e2e_measure(eng, bank, kcol, max(5, args.steps // 2), 2)
        e2e = {"value": v * world, "unit": "collisions/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h}

    fp64 = None
    if args.precision == "mixed" and not args.no_fp64 and world == 1:
        # the plain FP64 GPU path on the same deck and history count, device
        # time per generation as above: the mixed/FP64 ratio of the same run
        eng.close()
        fb = decks.CONFIGS[args.config](nparticles=npart)
        if args.tracking:
            fb.tracking = args.tracking
        eng64 = Engine(fb.build(precision="fp64"), local)
        _abi.check(eng64.lib.abx_set_l2_flush(eng64.ctx, L2_FLUSH_BYTES), eng64.lib)
        eng64.run_power_iteration(max(args.warmup, 1), 0)
        n64 = max(3, args.steps // 4)
        _, r64 = eng64.run_power_iteration_records(n64, 0)
        c64 = sum(r["collisions"] for r in r64)
        ms64 = sum(r["step_ms"] for r in r64)
        fp64 = {"value": c64 / (ms64 / 1e3), "unit": "collisions/s", "generations": n64,
                "ms_per_step": ms64 / n64}
        eng64.close()

    if rank != 0:
        if dist:
            dist.barrier()
        return 0
    b = BYTES[args.precision]
    alg = flights * b["flight"] + coll * b["collision"] + sites * b["site"]
    achieved = alg / (tr_ms / 1e3) / 1e9
    peak, src = peaks()
    hist = sum(r["histories"] for r in recs) / max(len(recs), 1)
    cnt = COUNTERS.get((args.config, args.precision, builder.tracking, kernel_used))
    traffic = cnt["dram_bytes_per_history"] * hist if cnt else None
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": traffic, "peak_source": src,
            "kernel": "transport_kernel", "algorithmic_bytes_per_launch": alg / max(len(recs), 1)}
    clocks = clk.summary()
    if cnt:
        # what binds this kernel: instruction issue, not HBM
        import torch
        sms = torch.cuda.get_device_properties(local).multi_processor_count
        mhz = clocks.get("sm_mhz") or 2070.0
        inst = cnt["warp_inst_per_collision"] * coll
        roof["issue"] = {"warp_inst_per_launch": inst / max(len(recs), 1),
                         "issue_frac": inst / (tr_ms / 1e3) / (sms * SCHEDULERS_PER_SM * mhz * 1e6),
                         "lanes_per_inst": cnt["thread_inst_per_collision"] / cnt["warp_inst_per_collision"],
                         "peak": f"{sms} SMs x {SCHEDULERS_PER_SM} schedulers x {mhz:.0f} MHz",
                         "counters": cnt["source"] + " (per collision and per history, scaled to this run)"}
    cpu = None
    if world == 1 and not args.no_cpu:
        v, cores, c, dt = cpu_baseline(args.config, args.cpu_sample)
        cpu = {"value": v, "unit": "collisions/s", "cores": cores, "kind": "port", "cpu": host_cpu(),
               "sample": f"{args.cpu_sample} first-generation histories of config {args.config}, FP64, one transport"}
    line = {
        "metric": "collisions/s", "value": value, "unit": "collisions/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": step_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32-track/f64-tally" if args.precision == "mixed" else "f64",
        "data": "synthetic",
        "config": {"workload": WORKLOADS[args.config], "deck": args.config, "histories_per_generation": npart,
                   "tracking": builder.tracking, "precision": args.precision,
                   "l2": f"flushed: {L2_FLUSH_BYTES >> 20} MiB written before each generation, outside its "
                   "timed events", "parallelism": f"replicas{world}",
                   "launch": {"autotuned": bool(shape), "block": shape[0] if shape else None,
                              "grid": shape[1] if shape else None, "kernel": kernel_used}},
        "roofline": roof, "cpu_baseline": cpu, "e2e": e2e,
        "gpu_launches": KERNELS_PER_GEN * args.steps,
        "clocks": clocks,
        "flights_per_s": flights / (step_ms / 1e3) * world,
        "detail": {"flights": flights, "collisions": coll, "sites": sites, "transport_ms": tr_ms,
                   "wall_s": wall, "kcol_last": recs[-1]["kcol"], "lost": sum(r["lost"] for r in recs),
                   "fp64": fp64, "mixed_over_fp64": (value / fp64["value"]) if fp64 else None},
    }
    print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
    return 0


def bench_batch(args):
    """Config 3: `--problems` independent fixed-source slab problems (10
    batches each) resident together.  One step = one run of every batch of
    every problem: source sampling, one transport launch over all of them, and
    the per-batch tally and leakage records.  Beside it, a sample of the same
    problems run one problem per launch (their own context and FixedSource
    loop each), in the same precision and in FP64."""
    import __graft_entry__
    __graft_entry__.build()
    import numpy as np
    from abeille_gb300 import BatchEngine, decks

    rank, world, local, dist = dist_setup(args.gpus)
    nb = 10
    builders = [decks.fixed_source_problem(i, seed=3 + rank, precision=args.precision, batches=nb)
                for i in range(args.problems)]
    if args.tracking:
        for b in builders:
            b.tracking = args.tracking
    builts = [b.build(precision=args.precision) for b in builders]
    hist_per_step = nb * sum(b.nparticles for b in builders)

    # the context, created once (its CUDA set-up is not part of a step)
    t0 = time.perf_counter()
    eng = BatchEngine(builts, local)
    t_first = time.perf_counter() - t0
    for _ in range(max(args.warmup, 1)):
        eng.run(nb)
    # end to end, every step: the problems' tables from host memory
    # (abx_batch_replace: host preparation + upload), the run, and the
    # average and variance of every tally bin read back
    t_load = t_run = t_read = 0.0
    e2e_coll = 0
    for _ in range(args.steps):
        t0 = time.perf_counter()
        eng.replace(builts)
        t1 = time.perf_counter()
        rows, st_e = eng.run(nb)
        t2 = time.perf_counter()
        avg, var = eng.tally_all()  # every problem's bins, problem after problem
        t3 = time.perf_counter()
        t_load += t1 - t0
        t_run += t2 - t1
        t_read += t3 - t2
        e2e_coll += st_e["collisions"]
    e2e_wall = t_load + t_run + t_read
    d2h = avg.nbytes + var.nbytes
    h2d = sum(sum(getattr(a, "nbytes", 0) for a in b._keep) for b in builts)
    if dist:
        dist.barrier()
    coll = flights = 0
    step_ms = tr_ms = 0.0
    with Clocks(local) as clk:
        for _ in range(args.steps):
            rows, st = eng.run(nb)
            coll += st["collisions"]
            flights += st["flights"]
            step_ms += st["total_ms"]
            tr_ms += st["transport_ms"]
    secs, coll_all = combine_replicas(dist, step_ms / 1e3, coll, f"cuda:{local}")
    eng.close()
    if rank != 0:
        if dist:
            dist.barrier()
        return 0

    # one problem per launch, on an evenly spaced sample of the same problems
    idx = np.linspace(0, args.problems - 1, min(args.per_problem_sample, args.problems)).astype(int)
    per = _per_problem_launch(idx, nb, sorted({args.precision, "fp64"}), local, args.tracking)
    b = BYTES[args.precision]
    alg = flights * b["flight"] + coll * b["collision"]
    peak, src = peaks()
    roof = {"bound": "hbm", "achieved": alg / (tr_ms / 1e3) / 1e9, "peak": peak, "unit": "GB/s",
            "frac": alg / (tr_ms / 1e3) / 1e9 / peak, "traffic": None, "peak_source": src,
            "kernel": "transport_kernel", "algorithmic_bytes_per_launch": alg / args.steps}
    cpu = None
    if world == 1 and not args.no_cpu:
        import oracle
        c_sum, secs_cpu, used = 0, 0.0, 0
        for i in idx:
            bo = decks.fixed_source_problem(int(i), seed=3, precision="fp64", batches=nb)
            o = oracle.Oracle(bo.build(precision="fp64"), nthreads=oracle.cores())
            ta = time.perf_counter()
            so = o.run_fixed_source(nb, bo.nparticles)
            secs_cpu += time.perf_counter() - ta
            c_sum += so["collisions"]
            used += 1
            if secs_cpu > 15.0:
                break
        cpu = {"value": c_sum / secs_cpu, "unit": "collisions/s", "cores": oracle.cores(), "kind": "port",
               "cpu": host_cpu(),
               "sample": f"{used} of the problems, {nb} batches each, FP64, one problem at a time"}
    line = {
        "metric": "collisions/s", "value": coll_all / secs, "unit": "collisions/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f32-track/f64-tally" if args.precision == "mixed" else "f64", "data": "synthetic",
        "config": {"workload": WORKLOADS[3], "deck": 3, "problems": args.problems, "histories_per_step": hist_per_step,
                   "batches": nb, "tracking": builders[0].tracking, "precision": args.precision,
                   "l2": "inputs larger than L2 (bank of all problems' batch, tallies of 4096x8000 bins)",
                   "parallelism": f"replicas{world}"},
        "roofline": roof, "cpu_baseline": cpu,
        "e2e": {"value": e2e_coll / e2e_wall, "unit": "collisions/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h,
                "what": "per step: abx_batch_replace (host tables + upload) + abx_run_fixed_source_batch + "
                        "abx_tally_read_all (average and variance of every bin), wall"},
        "per_problem_launch": per,
        # per step: zero the batch tallies, sample, step begin, transport,
        # batch tally record, problem record, generation end
        "gpu_launches": 7 * args.steps,
        "clocks": clk.summary(),
        "detail": {"collisions": coll, "flights": flights, "transport_ms": tr_ms, "first_create_s": t_first,
                   "e2e_load_s": t_load / args.steps, "e2e_run_s": t_run / args.steps,
                   "e2e_tally_read_s": t_read / args.steps,
                   "lost": int(sum(r["lost"] for r in rows))},
    }
    print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
    return 0


def _per_problem_launch(idx, nb, precisions, device, tracking=None):
    """Collisions/s of problems run one per context and launch (FixedSource
    loop each), wall time around the run."""
    from abeille_gb300 import Engine, decks
    per = {}
    for prec in precisions:
        c_sum, wall, dev = 0, 0.0, 0.0
        for i in idx:
            b = decks.fixed_source_problem(int(i), seed=3, precision=prec, batches=nb)
            if tracking:
                b.tracking = tracking
            e = Engine(b.build(precision=prec), device)
            ta = time.perf_counter()
            s1 = e.run_fixed_source(nb, b.nparticles)
            wall += time.perf_counter() - ta
            dev += s1["transport_ms"] / 1e3
            c_sum += s1["collisions"]
            e.close()
        per[prec] = {"value": c_sum / wall, "transport_only_value": c_sum / dev, "unit": "collisions/s",
                     "problems": len(idx), "precision": prec}
    return per


def bench_zscore(args):
    """Mixed against FP64 on `--config` (1 unless given; `--tracking` applies)
    over independent replicas: `--zsets` S
    sets of `--zscore` R replicas per precision (own seed each; `--particles`
    histories per generation, default 1e5, 10 inactive + 40 active
    generations).  Every pair of sets is compared: k difference in sigma and
    the fraction of flux bins with |z| < 2, sigma of each mean from the
    replica spread.  With R replicas per set the z of two identical
    distributions follows a Student t with about 2(R-1) degrees of freedom
    (the expected fraction is printed), and because all bins share one
    fission source the fraction moves by a percent or more from one pair of
    sets to another: FP64/FP64 pairs show that spread."""
    import itertools

    import __graft_entry__
    __graft_entry__.build()
    import numpy as np
    from scipy import stats as _st
    from abeille_gb300 import Engine, decks

    R, S = args.zscore, max(args.zsets, 1)
    npart = args.particles or 100000
    sets = {}
    t0 = time.perf_counter()
    for si in range(S):
        for prec in ("fp64", "mixed"):
            ks, avgs = [], []
            for rep in range(R):
                b = decks.CONFIGS[args.config](nparticles=npart)
                if args.tracking:
                    b.tracking = args.tracking
                b.seed = 20000 + 100000 * si + (50000 if prec == "mixed" else 0) + rep
                eng = Engine(b.build(precision=prec), 0)
                st, _, _ = eng.run_power_iteration(50, 10)
                ks.append(st["kcol_avg"])
                avgs.append(eng.tally(0)["avg"])
                eng.close()
            sets[f"{prec}{si + 1}"] = (np.array(ks), np.array(avgs))

    pairs = []
    for x, y in itertools.combinations(sorted(sets), 2):
        (kx, ax), (ky, ay) = sets[x], sets[y]
        dk = (kx.mean() - ky.mean()) / np.sqrt(kx.var(ddof=1) / R + ky.var(ddof=1) / R)
        keep = (ax.mean(0) > 0) & (ay.mean(0) > 0)
        z = ((ax.mean(0) - ay.mean(0)) / np.sqrt(ax.var(0, ddof=1) / R + ay.var(0, ddof=1) / R))[keep]
        kind = "mixed/fp64" if x[:2] != y[:2] else ("fp64/fp64" if x.startswith("fp64") else "mixed/mixed")
        pairs.append({"pair": f"{x} {y}", "kind": kind, "dk_sigma": round(float(dk), 3), "bins": int(keep.sum()),
                      "frac_abs_z_lt_2": round(float(np.mean(np.abs(z) < 2)), 4), "mean_z": round(float(z.mean()), 4)})
    dof = 2 * (R - 1)
    summ = {}
    for kind in ("fp64/fp64", "mixed/fp64", "mixed/mixed"):
        f = [p["frac_abs_z_lt_2"] for p in pairs if p["kind"] == kind]
        if f:
            summ[kind] = {"pairs": len(f), "frac_min": min(f), "frac_max": max(f), "frac_mean": round(float(np.mean(f)), 4)}
    line = {"metric": "mixed vs fp64 agreement", "workload": WORKLOADS[args.config], "deck": args.config,
            "tracking": b.tracking, "replicas_per_set": R, "sets_per_precision": S,
            "histories_per_generation": npart, "generations": "10 inactive + 40 active",
            "k_mixed": float(np.mean([sets[k][0].mean() for k in sets if k.startswith("mixed")])),
            "k_fp64": float(np.mean([sets[k][0].mean() for k in sets if k.startswith("fp64")])),
            "frac_expected_identical": round(float(_st.t.cdf(2, dof) - _st.t.cdf(-2, dof)), 4),
            "summary": summ, "pairs": pairs, "wall_s": round(time.perf_counter() - t0, 1)}
    print(json.dumps(line), flush=True)
    return 0


def bench_server(args):
    """Config 4: config-3 problems arriving as a Poisson stream at each rate of
    `--rates` for `--duration` s, served by the request loop (mixed
    precision); latency percentiles per rate, aggregate collisions/s, the
    one-problem-per-launch rates (mixed and FP64), and the leakage z-scores of the served
    results against FP64 runs of the same problems."""
    import gc
    import threading

    import __graft_entry__
    __graft_entry__.build()
    import numpy as np
    from abeille_gb300 import BatchEngine, Server, abi, decks

    rank, world, local, dist = dist_setup(args.gpus)
    nb = 10
    npool = min(args.problems, 4096)
    builders = [decks.fixed_source_problem(i, seed=3 + rank, precision=args.precision, batches=nb)
                for i in range(npool)]
    builts = [b.build(precision=args.precision) for b in builders]
    rates = [float(x) for x in args.rates.split(",") if x]
    rng = np.random.default_rng(11 + rank)

    def serve(rate, duration, record):
        """One server at one Poisson rate: `--warm` s of arrivals first (the
        server's lanes create their contexts and size their buffers), then
        `duration` s measured.  Percentiles and rates cover the requests
        submitted after the warm-up; the warm-up's own percentiles are kept
        under "cold"."""
        srv = Server(device=local, precision=args.precision, nbatches=nb,
                     hbm_budget_bytes=int(args.budget_gb * 1e9), keep_tallies=False, lanes=args.lanes,
                     history_quantum=args.quantum)
        done, lock = {}, threading.Lock()
        stop = threading.Event()

        def poller():
            while not (stop.is_set() and len(done) >= n_sub[0]):
                for r in srv.poll(512, 50):
                    with lock:
                        done[r["request_id"]] = (r, time.perf_counter())
        n_sub = [10 ** 9]
        th = threading.Thread(target=poller, daemon=True)
        th.start()
        # the arrival process must not pause: a cyclic-GC pass in this
        # thread would hold arrivals back and release them as one burst
        gc.collect()
        gc.disable()
        t0 = time.perf_counter()
        t_next, i, sub = t0, 0, {}
        st_w, t_w = None, None
        try:
            while True:
                t_next += rng.exponential(1.0 / rate)
                if t_next - t0 > args.warm + duration:
                    break
                while time.perf_counter() < t_next:
                    pass
                if st_w is None and t_next - t0 >= args.warm:
                    st_w, t_w = srv.stats(), time.perf_counter()
                sub[srv.submit(builts[i % npool], tag=i % npool)] = time.perf_counter() - t0
                i += 1
        finally:
            gc.enable()
        n_sub[0] = len(sub)
        stop.set()
        th.join(timeout=600)
        st1 = srv.stats()
        srv.close()
        if st_w is None:
            st_w, t_w = st1, time.perf_counter()
        meas = [k for k in sub if k in done and sub[k] >= args.warm]
        cold = np.array([done[k][0]["latency_ms"] for k in sub if k in done and sub[k] < args.warm])
        lat = np.array([done[k][0]["latency_ms"] for k in meas])
        t_end = max(done[k][1] for k in meas) if meas else time.perf_counter()
        coll = st1["collisions"] - st_w["collisions"]
        rows = [done[k][0] for k in meas]
        out = {"rate": rate, "requests": len([k for k in sub if sub[k] >= args.warm]), "completed": len(lat),
               "failed": int(sum(1 for r in rows if r["status"] != 0)),
               "p50_ms": float(np.percentile(lat, 50)), "p95_ms": float(np.percentile(lat, 95)),
               "p99_ms": float(np.percentile(lat, 99)), "p999_ms": float(np.percentile(lat, 99.9)),
               "max_ms": float(lat.max()), "collisions_per_s": coll / (t_end - t_w),
               "rounds": st1["rounds"] - st_w["rounds"], "busy_ms": st1["busy_ms"] - st_w["busy_ms"],
               "transport_ms": st1["transport_ms"] - st_w["transport_ms"], "collisions": coll,
               "round_ms": {k: st1[k + "_ms"] - st_w[k + "_ms"] for k in ("load", "run", "readback", "free")},
               "cold": {"warm_s": args.warm, "requests": int(cold.size),
                        "p50_ms": float(np.percentile(cold, 50)) if cold.size else None,
                        "p99_ms": float(np.percentile(cold, 99)) if cold.size else None}}
        if record is not None:
            record.extend(rows)
        return out

    serve(rates[0], 0.3, None)  # process warm-up (CUDA context and modules)
    if dist:
        dist.barrier()
    sweep, served = [], []
    with Clocks(local) as clk:
        for rate in rates:
            sweep.append(serve(rate, args.duration, served if rate == rates[-1] else None))
    head = sweep[-1]
    if rank != 0:
        if dist:
            dist.barrier()
        return 0
    # z-scores of the served (mixed) leakage against FP64 runs of the same problems
    uniq = {}
    for r in served:
        uniq.setdefault(r["tag"], r)
    tags = sorted(uniq)[:512]
    f64 = [decks.fixed_source_problem(t, seed=3 + rank, precision="fp64", batches=nb).build(precision="fp64")
           for t in tags]
    be = BatchEngine(f64, local)
    rows64, _ = be.run(nb)
    be.close()
    z = np.array([(uniq[t]["leak_avg"] - r64["leak_avg"]) / np.hypot(uniq[t]["leak_std"], r64["leak_std"])
                  for t, r64 in zip(tags, rows64) if np.hypot(uniq[t]["leak_std"], r64["leak_std"]) > 0])
    idx = np.linspace(0, npool - 1, min(args.per_problem_sample, npool)).astype(int)
    per = _per_problem_launch(idx, nb, sorted({args.precision, "fp64"}), local)
    line = {
        "metric": "collisions/s", "value": head["collisions_per_s"], "unit": "collisions/s", "n_gpus": world,
        "steps": len(rates), "warmup": 1, "ms_per_step": 1e3 * args.duration, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f32-track/f64-tally" if args.precision == "mixed" else "f64", "data": "synthetic",
        "config": {"workload": WORKLOADS[4], "deck": 4, "arrivals": "poisson", "rates": rates, "duration_s": args.duration,
                   "warm_s": args.warm, "measured": "requests submitted after warm_s of arrivals at the same rate "
                   "on the same server (steady state); the warm-up's own latencies under latency[].cold",
                   "problem_pool": npool, "batches": nb, "hbm_budget_gb": args.budget_gb,
                   "lanes": args.lanes or 3, "history_quantum": args.quantum or 256,
                   "precision": args.precision, "parallelism": f"replicas{world}",
                   "l2": "inputs larger than L2 at the high rates (rounds of thousands of problems)"},
        "latency": sweep,
        "per_problem_launch": per,
        # the served rate at the highest arrival rate over one problem per
        # launch, against the same precision and against FP64
        "served_over_per_problem_launch": {p: head["collisions_per_s"] / v["value"] for p, v in per.items()},
        "zscore_vs_fp64": {"problems": int(z.size), "frac_abs_z_lt_2": float(np.mean(np.abs(z) < 2)),
                           "mean_z": float(z.mean())},
        "e2e": {"value": head["collisions_per_s"], "unit": "collisions/s", "h2d_bytes_per_step": None,
                "d2h_bytes_per_step": None, "what": "abx_server_submit .. abx_server_poll wall, all requests"},
        "clocks": clk.summary(),
    }
    print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
    return 0


# Counters of the transport kernel per unit of work, from ncu captures of the
# same workloads at 300,000 histories per generation (one launch, the timed
# generation of `bench.py --steps 1 --warmup 1 --particles 300000 --no-e2e
# --no-cpu --no-fp64 --autotune 0`, metrics smsp__inst_executed.sum,
# smsp__thread_inst_executed.sum, dram__bytes_read.sum + dram__bytes_write.sum,
# divided by that launch's collisions and histories).  The bench line scales
# them by its own collisions and histories, and divides the instructions by its
# own device time and sampled SM clock for the fraction of the issue peak (one
# warp instruction per scheduler per cycle, 4 schedulers per SM).
COUNTERS = {
    (1, "mixed", "delta-tracking", "history"): {
        "warp_inst_per_collision": 3964713340 / 7371550, "thread_inst_per_collision": 21604900552 / 7371550,
        "dram_bytes_per_history": (18061824 + 104158208) / 3e5,
        "source": "profiles/transport_kernel_config1_mixed_300k.md"},
    (2, "mixed", "surface-tracking", "history"): {
        "warp_inst_per_collision": 2829894961 / 2417451, "thread_inst_per_collision": 28232959555 / 2417451,
        "dram_bytes_per_history": (22580224 + 15477760) / 3e5,
        "source": "profiles/transport_kernel_counters_300k.md"},
    (1, "fp64", "delta-tracking", "history"): {
        "warp_inst_per_collision": 7450495716 / 7371273, "thread_inst_per_collision": 44965331919 / 7371273,
        "dram_bytes_per_history": (361392384 + 3245730304) / 3e5,
        "source": "profiles/transport_kernel_counters_300k.md"},
}
SCHEDULERS_PER_SM = 4
L2_FLUSH_BYTES = 256 << 20

if __name__ == "__main__":
    sys.exit(main())
