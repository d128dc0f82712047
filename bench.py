"""Benchmark: LULESH Sedov FOM (zones*cycles/s, FP64) on the 150^3 problem.

A step is one LagrangeLeapFrog cycle (timeIncrement! + lagrangeLeapFrog) of
the 150^3 Sedov problem (3,375,000 elements, 11 regions, balance 1, cost 1,
the reference's own arithmetic). Inputs are generated by the problem setup;
the state (~2.6 GB) is larger than L2, so no flush is needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

The reference arm times the CPU restatement of the reference (the oracle,
OpenMP over all host cores): Julia, the reference's language, is not
available on these machines.
"""
import argparse
import ctypes
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (os.path.join(ROOT, "lulesh.jl_gb300"), os.path.join(ROOT, "oracle")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "FOM zones*cycles/s FP64 s=150"
UNIT = "zones*cycles/s"
NX = 150
# Algorithmic bytes (minimal HBM traffic of the method, FP64 fields, int32
# connectivity): 364 B per element + 152 B per node per cycle for the whole
# step. Per kernel, (bytes per element, bytes per node): the force pass reads
# nodelist, p, q, ss, v, volo, elemMass and x..zd; the kinematics pass reads
# nodelist, volo, v and x..zd and writes its nine outputs; the material pass
# reads those nine, e, p, q, v, volo, elemMass, elemBC and writes e, p, q, ss,
# v; the node pass reads x..zd and nodalMass and writes x..zd.
STEP_BYTES_PER_ELEM, STEP_BYTES_PER_NODE = 364, 152
KERNEL_BYTES = {"k_force": (80, 48), "k_kinematics": (120, 48), "k_material": (164, 0), "k_node": (0, 104)}
STATE_FIELDS = ["x", "y", "z", "xd", "yd", "zd", "e", "p", "q", "v", "ss"]
GEOMETRY_SPLIT = {0: "force geometry formed by k_kinematics and stored for k_force",
                  1: "force geometry formed inside k_force"}


def _measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            return json.load(f), "measured"
    return {"hbm_gbs": 6800.0}, "fallback"


def _profile_numbers():
    """Per-kernel ncu figures of the step kernels at 150^3 (per launch and per
    element), if the profile summary was committed."""
    path = os.path.join(ROOT, "profiles", "step_kernels_s150_ncu.json")
    if os.path.exists(path):
        with open(path) as f:
            return json.load(f)
    return {}


class ClockSampler:
    """nvidia-smi clock/throttle samples while the timed region runs."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.QUERY,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except (OSError, ValueError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sms, maxs, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sms.append(float(parts[1]))
                maxs.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sms:
            why = "nvidia-smi unavailable" if self.proc is None else "no sample during the timed region"
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [why], "samples": 0}
        sms.sort()
        return {"sm_mhz": sms[len(sms) // 2], "sm_max_mhz": max(maxs), "reasons": sorted(reasons),
                "samples": len(sms)}


def workload_config(nx, mode, world):
    """The `config` both arms print for the same problem (identical dicts)."""
    return {"workload": f"Sedov blast {nx}^3, 11 regions, balance 1, cost 1, FP64",
            "nx": nx, "elements": nx ** 3, "nodes": (nx + 1) ** 3, "mode": mode,
            "parallelism": "replicas" if world > 1 else "one problem",
            "l2": "state larger than L2 (no flush)"}


def _dist():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def max_over_ranks(value, world):
    """Max of a float over the torch.distributed ranks (identity at one rank)."""
    if world <= 1:
        return value
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([value], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def cpu_oracle_rate(nx, seconds, threads=0, min_cycles=2, warm=1, serial=False):
    """Oracle (reference restatement) zones*cycles/s over a time-bounded sample;
    `serial` times the single-threaded build (the reference is single-threaded)."""
    import oracle
    L = oracle.load(openmp=not serial)
    if threads and not serial:
        L.ora_set_threads(threads)
    used = 1 if serial else L.ora_max_threads()
    d = oracle.OracleDomain(nx, nr=11, openmp=not serial)
    for _ in range(warm):
        d.time_increment()
        d.lagrange_leapfrog()
    n, t0 = 0, time.perf_counter()
    while n < min_cycles or time.perf_counter() - t0 < seconds:
        d.time_increment()
        d.lagrange_leapfrog()
        n += 1
    dt = time.perf_counter() - t0
    d.close()
    return nx ** 3 * n / dt, used, n, dt


def run_reference(args):
    world, rank, _ = _dist()
    if rank != 0:
        return 0
    import oracle
    oracle.build()
    L = oracle.load(openmp=True)
    threads = L.ora_max_threads()
    d = oracle.OracleDomain(args.nx, nr=11, mode=args.mode)
    for _ in range(args.warmup):
        d.time_increment()
        d.lagrange_leapfrog()
    budget = 180.0  # seconds of timed CPU work at most
    n, t0 = 0, time.perf_counter()
    while n < args.steps and (n < 1 or time.perf_counter() - t0 < budget):
        d.time_increment()
        d.lagrange_leapfrog()
        n += 1
    dt = time.perf_counter() - t0
    value = args.nx ** 3 * n / dt
    sample = (f"{n} of {args.steps} cycles of the {args.nx}^3 problem after {args.warmup} warm-up cycles"
              + ("" if n == args.steps else f" (stopped at the {budget:.0f} s budget)"))
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": n, "warmup": args.warmup, "ms_per_step": 1e3 * dt / n, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload_config(args.nx, args.mode, world),
            "device": f"host CPU, {threads} threads",
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "Julia (the reference's language) is not installed; the reference arm is the "
                    "oracle, a C++ restatement of src/domain.jl + src/utils.jl, OpenMP over all cores"}
    print(json.dumps(line), flush=True)
    return 0


def ensemble_leg(L, torch, dev, n, cycles, world=1, rank=0):
    """Config C4: n seeded Sedov instances (nx in [16, 64], einit x U-log[0.5, 2],
    hgcoef in [2, 4], nr 1 or 11) advanced `cycles` cycles as one device-resident
    ensemble, against looping the single-problem GPU path over the same instances.
    With several ranks each advances its lulesh_ens_partition shard (no
    collective on the data path); times are the max over ranks."""
    all_inst = L.sedov_instances(0xC4, n, 16, 64)
    _, inst = L.shard(all_inst, world, rank) if world > 1 else (None, all_inst)
    ens = L.Ensemble(inst, mode=0, device=dev)
    tuning = ens.autotune(cycles=2)  # returns the ensemble to its initial state
    mine = len(inst)
    init_dt = [ens.scalars(i)["deltatime"] for i in range(mine)]
    stream = torch.cuda.ExternalStream(ens.stream(), device=dev)
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize(dev)
    barrier(world)
    t0 = time.perf_counter()
    a.record(stream)
    ens.run(cycles)  # one launch of a graph of the whole run (up to 512 cycles)
    b.record(stream)
    torch.cuda.synchronize(dev)
    host_s = time.perf_counter() - t0
    ens_s = max_over_ranks(a.elapsed_time(b) * 1e-3, world)
    done = sum(ens.scalars(i)["cycle"] == cycles for i in range(mine))
    total_elems = ens.total_elem
    ens.close()
    # the same instances, one single-problem handle after another (setup untimed)
    loop_s = 0.0
    per_instance = []
    for i, spec in enumerate(inst):
        g = L.Domain(L.LuleshProblem(nx=spec["nx"], nr=spec["nr"], device=dev))
        g.hgcoef = spec["hgcoef"]
        e = g.field("e")
        e[0] = spec["einit"]
        g.set_field("e", e)
        g.deltatime = init_dt[i]
        s = torch.cuda.ExternalStream(g.stream(), device=dev)
        torch.cuda.synchronize(dev)
        a.record(s)
        L.run(g, cycles)
        b.record(s)
        torch.cuda.synchronize(dev)
        t_i = a.elapsed_time(b) * 1e-3
        loop_s += t_i
        per_instance.append((spec["nx"], t_i))
        g.close()
    loop_s = max_over_ranks(loop_s, world)
    # where looping loses: per mesh-size bucket, the looped time against the
    # time the same zone-cycles take at the ensemble's rate
    ens_rate = total_elems * cycles / ens_s
    breakdown = []
    for lo, hi in ((16, 24), (25, 32), (33, 40), (41, 48), (49, 56), (57, 64)):
        sel = [(nx, t) for nx, t in per_instance if lo <= nx <= hi]
        if not sel:
            continue
        zc = sum(nx ** 3 for nx, _ in sel) * cycles
        t_loop = sum(t for _, t in sel)
        breakdown.append({"nx": f"{lo}-{hi}", "instances": len(sel), "looped_s": t_loop,
                          "looped_zones_cycles_per_s": zc / t_loop,
                          "us_per_cycle_per_instance": 1e6 * t_loop / (len(sel) * cycles),
                          "s_at_ensemble_rate": zc / ens_rate, "lost_s": t_loop - zc / ens_rate})
    return {"config": f"{n} Sedov instances, nx uniform in [16, 64] (seed 0xC4), {cycles} cycles each, FP64",
            "instances": n, "cycles": cycles, "total_elements_rank0": total_elems,
            "instances_rank0": mine, "instances_completed_rank0": int(done),
            "sharding": f"lulesh_ens_partition over {world} rank(s)" if world > 1 else "one GPU",
            "problems_per_s": n / ens_s, "seconds": ens_s,
            "graph_launches": -(-cycles // min(cycles, 512)), "host_wall_s_incl_graph_build": host_s,
            "looped_plain_problems_per_s": n / loop_s, "looped_plain_seconds": loop_s,
            "speedup_vs_looped_plain": loop_s / ens_s,
            "zones_cycles_per_s_rank0": total_elems * cycles / ens_s,
            "looped_breakdown_rank0": breakdown,
            "tuning": tuning, "geometry_split": GEOMETRY_SPLIT[tuning["geometry"]]}


def adjoint_leg(L, torch, dev, nx, cycles, every, dirs):
    """Config C5: gradient of the energy within r < 0.3 of the origin after
    `cycles` cycles of an nx^3 Sedov problem (origin energy the default, the
    others U[0, 1e-3] from seed 0xC5) w.r.t. the initial e field and hgcoef,
    with checkpoints every `every` cycles. Reports its cost against the
    forward run of the same cycles and its agreement with central finite
    differences of the GPU run on `dirs` directions (seed 0xF0, step 1e-6
    relative: d_i = N(0,1) * e0_i, and N(0,1) * hgcoef)."""
    g = L.Domain(L.LuleshProblem(nx=nx, nr=11, device=dev))
    rng = np.random.default_rng(0xC5)
    e0 = g.field("e")
    e0[1:] = rng.uniform(0.0, 1e-3, g.numElem - 1)
    g.set_field("e", e0)
    snap = ({f: g.field(f) for f in STATE_FIELDS},
            {s: getattr(g, s) for s in ("time", "deltatime", "dtcourant", "dthydro", "cycle", "hgcoef")})

    def restore(e=None, hg=None):
        for f, v in snap[0].items():
            g.set_field(f, v)
        for k, v in snap[1].items():
            setattr(g, k, v)
        if e is not None:
            g.set_field("e", e)
        if hg is not None:
            g.hgcoef = hg

    adj = L.Adjoint(g, radius=0.3, checkpoint_every=every)
    restore()
    L.run(g, cycles)  # warm-up (graph capture)
    fwd = []
    for _ in range(3):
        restore()
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        L.run(g, cycles)
        torch.cuda.synchronize(dev)
        fwd.append(time.perf_counter() - t0)
    fwd_s = min(fwd)
    restore()
    adj.gradient(cycles)  # warm-up (checkpoint buffers)
    times = []
    for _ in range(2):
        restore()
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        loss = adj.gradient(cycles)
        torch.cuda.synchronize(dev)
        times.append(time.perf_counter() - t0)
    adj_s = min(times)
    res = adj.result
    sweep = int(res.sweep)
    ge, ghg = adj.grad("e"), res.grad_hgcoef
    hg0 = snap[1]["hgcoef"]

    # the same gradient with the other reverse-sweep plans: each segment's
    # recompute and transpose in turn (mode 0), and overlapped on one tape
    # (mode 2, what runs where a second tape does not fit)
    def other_plan(mode):
        adj.set_overlap(mode)
        restore()
        adj.gradient(cycles)  # warm-up (graphs)
        ts = []
        for _ in range(2):
            restore()
            torch.cuda.synchronize(dev)
            t0 = time.perf_counter()
            adj.gradient(cycles)
            torch.cuda.synchronize(dev)
            ts.append(time.perf_counter() - t0)
        same = bool(np.array_equal(adj.grad("e"), ge)) and adj.result.grad_hgcoef == ghg
        return {"adjoint_s": min(ts), "adjoint_over_forward": min(ts) / fwd_s, "sweep": int(adj.result.sweep),
                "gradient_bitwise_equal": same}

    seq = other_plan(0)
    one_tape = other_plan(2)
    adj.set_overlap(1)

    def loss_at(e, hg):
        restore(e, hg)
        L.run(g, cycles)
        return adj.loss()

    drng = np.random.default_rng(0xF0)
    h = 1e-6
    errs = []
    for _ in range(dirs):
        de = drng.standard_normal(g.numElem) * e0
        dhg = drng.standard_normal() * hg0
        fd = (loss_at(e0 + h * de, hg0 + h * dhg) - loss_at(e0 - h * de, hg0 - h * dhg)) / (2 * h)
        an = float(np.dot(ge, de)) + ghg * dhg
        errs.append(abs(an - fd) / max(abs(fd), 1e-12 * abs(loss)))
    adj.close()
    # the same gradient with the whole run taped in HBM (no recompute): one
    # segment of `cycles` cycles, about 8 * (204 E + 6 N) bytes per cycle
    tape_gb = 8.0 * (204 * g.numElem + 6 * g.numNode) * cycles / 1e9
    full = None
    try:
        adj2 = L.Adjoint(g, radius=0.3, checkpoint_every=cycles)
    except L.LuleshError as exc:
        full = {"skipped": str(exc), "tape_gb": tape_gb}
    if full is None:
        restore()
        adj2.gradient(cycles)  # warm-up
        times2 = []
        for _ in range(2):
            restore()
            torch.cuda.synchronize(dev)
            t0 = time.perf_counter()
            adj2.gradient(cycles)
            torch.cuda.synchronize(dev)
            times2.append(time.perf_counter() - t0)
        same = bool(np.array_equal(adj2.grad("e"), ge)) and adj2.result.grad_hgcoef == ghg
        full = {"checkpoint_every": cycles, "tape_gb": tape_gb, "adjoint_s": min(times2),
                "adjoint_over_forward": min(times2) / fwd_s, "gradient_bitwise_equal": same}
        adj2.close()
    g.close()
    return {"config": f"Sedov {nx}^3, {cycles} cycles, energy within r < 0.3, d/d(e0, hgcoef), "
                      f"checkpoints every {every} cycles, FP64",
            "nx": nx, "cycles": int(res.cycles), "checkpoints": int(res.checkpoints),
            "forward_s": fwd_s, "adjoint_s": adj_s, "adjoint_over_forward": adj_s / fwd_s,
            "adjoint_sweep_ms": {"checkpointed_forward": res.forward_ms, "reverse": res.reverse_ms},
            "reverse_sweep": {0: "each segment recomputed, then transposed",
                              1: "recompute of each segment overlapped with the transpose of the next (two tapes)",
                              2: "recompute of each segment overlapped with the transpose of the next (one tape)"}[sweep],
            "sequential": seq, "one_tape": one_tape,
            "loss": loss, "grad_hgcoef": ghg, "grad_e_origin": float(ge[0]),
            "fd": {"directions": dirs, "step": h, "max_rel_err": max(errs),
                   "median_rel_err": float(np.median(errs))},
            "whole_run_taped": full}


def c3_leg(L, torch, dev, nx, cycles, warmup=2):
    """Config C3: the nx^3 Sedov problem with 11 unbalanced regions (balance 4,
    cost 2) and the region cost model on (each element's EOS evaluated its
    region's rep count times: 1, 3 or 30), timed over `cycles` cycles after
    `warmup`; the same problem without the extra EOS work (the reference's
    behaviour) is timed beside it. Results are identical (tested)."""
    out = {"config": f"Sedov {nx}^3, 11 regions, balance 4, cost 2, region reps on, FP64",
           "nx": nx, "cycles": cycles}
    for reps in (True, False):
        g = L.Domain(L.LuleshProblem(nx=nx, nr=11, balance=4, cost=2, region_reps=reps, device=dev))
        if reps:
            sizes, counts = g.field("regElemSize"), g.field("regReps")
            out["elements_by_reps"] = {str(int(r)): int(sizes[counts == r].sum()) for r in np.unique(counts)}
            out["mean_eos_evaluations"] = float((sizes * counts).sum() / sizes.sum())
        stream = torch.cuda.ExternalStream(g.stream(), device=dev)
        L.run(g, warmup)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        c0 = g.cycle
        torch.cuda.synchronize(dev)
        a.record(stream)
        sc = L.run(g, c0 + cycles)
        b.record(stream)
        torch.cuda.synchronize(dev)
        done = sc["cycle"] - c0
        ms = a.elapsed_time(b)
        key = "with_region_reps" if reps else "without_region_reps"
        out[key] = {"zones_cycles_per_s": g.numElem * done / (ms * 1e-3), "ms_per_cycle": ms / done,
                    "cycles": int(done), "origin_energy": float(g.field("e")[0])}
        g.close()
    out["reps_cost_factor"] = out["with_region_reps"]["ms_per_cycle"] / out["without_region_reps"]["ms_per_cycle"]
    return out


def c1_leg(L, torch, dev, cpu=True, cpu_seconds=3.0):
    """Config C1, the reference's CPU-runnable case: the 30^3 Sedov problem
    (11 regions) run to stoptime 1e-2 in the corrected mode (LULESH 2.0's
    method; 932 cycles) and, in the faithful mode, whose dt collapses before
    stoptime, for 1000 cycles. Each whole run is timed on the GPU through
    lulesh_run (after a run of another handle of the same problem), and the
    oracle on the host cores: the OpenMP build over the whole corrected run,
    the serial build over a bounded sample of it."""
    nx = 30
    out = {"config": f"Sedov {nx}^3, 11 regions, balance 1, cost 1, FP64, run to stoptime 1e-2", "nx": nx}
    for mode, iters, key in ((7, 10 ** 9, "corrected_to_stoptime"), (0, 1000, "faithful_1000_cycles")):
        w = L.Domain(L.LuleshProblem(nx=nx, mode=mode, device=dev))
        L.run(w, 20)
        w.close()
        g = L.Domain(L.LuleshProblem(nx=nx, mode=mode, device=dev))
        stream = torch.cuda.ExternalStream(g.stream(), device=dev)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        a.record(stream)
        sc = L.run(g, iters)
        b.record(stream)
        torch.cuda.synchronize(dev)
        wall = time.perf_counter() - t0
        ms = a.elapsed_time(b)
        out[key] = {"cycles": int(sc["cycle"]), "time": sc["time"], "origin_energy": float(g.field("e")[0]),
                    "gpu_s": ms * 1e-3, "host_wall_s": wall,
                    "zones_cycles_per_s": nx ** 3 * sc["cycle"] / (ms * 1e-3)}
        g.close()
    if cpu:
        import oracle
        d = oracle.OracleDomain(nx, nr=11, mode=7, openmp=True)
        used = oracle.load(True).ora_max_threads()
        t0 = time.perf_counter()
        while d.get("time") < d.get("stoptime"):
            d.time_increment()
            d.lagrange_leapfrog()
        dt = time.perf_counter() - t0
        n = d.get("cycle")
        d.close()
        rate1, _, n1, dt1 = cpu_oracle_rate(nx, cpu_seconds, serial=True)
        out["cpu_baseline"] = {
            "kind": "port", "openmp": {"cores": used, "cycles": n, "seconds": dt,
                                       "zones_cycles_per_s": nx ** 3 * n / dt,
                                       "sample": "the whole corrected run to stoptime (oracle, OpenMP)"},
            "serial": {"cores": 1, "zones_cycles_per_s": rate1, "projected_run_s": nx ** 3 * n / rate1,
                       "sample": f"{n1} cycles in {dt1:.1f} s (oracle, serial build, faithful mode)"}}
    return out


def blocks_leg(L, torch, dev, nx, tp, cycles, plain_ms, warmup=3):
    """The multi-rank decomposition on one GPU: the (tp*nx)^3 problem as tp^3
    blocks of nx^3 elements with halo copies across block faces (bitwise the
    single-block run, tested), timed over `cycles` cycles against the
    single-block step time of the same problem."""
    g = L.Domain(L.LuleshProblem(nx=nx, nr=11, blocks_per_edge=tp, device=dev))
    stream = torch.cuda.ExternalStream(g.stream(), device=dev)
    tuning = g.autotune(cycles=2)  # the state is kept
    L.run(g, warmup)
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    c0 = g.cycle
    torch.cuda.synchronize(dev)
    a.record(stream)
    L.run(g, c0 + cycles)
    b.record(stream)
    torch.cuda.synchronize(dev)
    ms = a.elapsed_time(b) / (g.cycle - c0)
    g.enable_timing(True)
    L.run(g, g.cycle + 5)
    kt = {k: v / 5 for k, v in g.kernel_times().items()}
    out = {"config": f"Sedov {nx * tp}^3 as {tp}^3 blocks of {nx}^3 (the reference's {tp ** 3}-rank "
                     "decomposition) with halo copies, FP64, one GPU",
           "blocks": tp ** 3, "block_nx": nx, "cycles": int(g.cycle - c0), "ms_per_cycle": ms,
           "zones_cycles_per_s": (nx * tp) ** 3 / (ms * 1e-3),
           "single_block_ms_per_cycle": plain_ms, "overhead_vs_single_block": ms / plain_ms - 1.0,
           "kernel_ms_per_cycle_with_halo": kt, "tuning": tuning,
           "nodes_packed": g.numNode, "nodes_whole_mesh": (nx * tp + 1) ** 3}
    g.close()
    return out


def run_ours(args):
    world, rank, local = _dist()
    import torch
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", init_method="env://")
    torch.cuda.set_device(local)
    import lulesh_gb300 as L

    dev = local
    prob = L.LuleshProblem(nx=args.nx, nr=11, balance=1, cost=1, mode=args.mode, device=dev)
    g = L.Domain(prob)
    E, N = g.numElem, g.numNode
    stream = torch.cuda.ExternalStream(g.stream(), device=dev)

    fma_s, add_s = ctypes.c_double(), ctypes.c_double()
    L.load_library().lulesh_measure_fp64_peak(dev, ctypes.byref(fma_s), ctypes.byref(add_s))

    # block sizes picked on this problem (the state is restored), then warm-up,
    # then the timed region: exactly K cycles, device-resident, with per-kernel
    # CUDA events on the library's stream
    tuning = g.autotune(cycles=2) if not args.no_tune else g.tuning()
    g.enable_timing(True)
    L.run(g, g.cycle + args.warmup)
    g.kernel_times()
    torch.cuda.synchronize(dev)
    barrier(world)
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    # The timed region (exactly K cycles) runs `repeats` times back to back,
    # through the problem's configured 200 cycles, so that the clock sampler
    # (one reading per 200 ms) sees several readings; the reported time is the
    # median region.
    repeats = max(1, args.config_cycles // args.steps)
    c0 = g.cycle
    region_ms = []
    with ClockSampler(dev) as clocks:
        for _ in range(repeats):
            torch.cuda.synchronize(dev)
            barrier(world)
            cr = g.cycle
            start.record(stream)
            s = L.run(g, cr + args.steps)
            end.record(stream)
            torch.cuda.synchronize(dev)
            if s["cycle"] - cr != args.steps:
                raise RuntimeError(f"a timed region ran {s['cycle'] - cr} of {args.steps} cycles")
            region_ms.append(start.elapsed_time(end))
    cycles = args.steps
    total_cycles = g.cycle - c0
    ms = sorted(region_ms)[len(region_ms) // 2]
    ms_max = max_over_ranks(ms, world)
    barrier(world)
    ktimes = {k: v * cycles / total_cycles for k, v in g.kernel_times().items()}
    value = world * E * cycles / (ms_max * 1e-3)

    # end to end through the reference-facing calls: the Domain state comes
    # from pinned host buffers, then K x (timeIncrement!, lagrangeLeapFrog),
    # each moving the step scalars, then the state goes back to the host
    g.enable_timing(False)
    host = {f: torch.empty(g.numElem if f in ("e", "p", "q", "v", "ss") else N, dtype=torch.float64,
                           pin_memory=True).numpy() for f in STATE_FIELDS}
    for f in STATE_FIELDS:
        host[f][:] = g.field(f)
    state_bytes = sum(a.nbytes for a in host.values())
    scalar_bytes = 72  # the device step state struct, each way, per step
    torch.cuda.synchronize(dev)
    barrier(world)
    t0 = time.perf_counter()
    for f in STATE_FIELDS:
        g.set_field(f, host[f])
    for _ in range(cycles):
        L.timeIncrement(g)
        L.lagrangeLeapFrog(g)
    for f in STATE_FIELDS:
        g.field(f, out=host[f])
    e2e_s = max_over_ranks(time.perf_counter() - t0, world)
    e2e = {"value": world * E * cycles / e2e_s, "unit": UNIT,
           "h2d_bytes_per_step": scalar_bytes + state_bytes / cycles,
           "d2h_bytes_per_step": scalar_bytes + state_bytes / cycles}

    # the ensemble leg runs on every rank (each advances its shard)
    ensemble = None
    if not args.no_ensemble:
        ensemble = ensemble_leg(L, torch, dev, args.ens_instances, args.ens_cycles, world, rank)

    if rank != 0:
        g.close()
        return 0

    peaks, peak_kind = _measured_peaks()
    hbm = float(peaks.get("hbm_gbs", 6800.0))
    # the roofline of the dominant step kernel (the one with the most time)
    dominant = max((k for k in ktimes if k in KERNEL_BYTES), key=ktimes.get)
    dom_ms = ktimes[dominant] / cycles
    be, bn = KERNEL_BYTES[dominant]
    dom_bytes = be * E + bn * N
    achieved = dom_bytes / (dom_ms * 1e-3) / 1e9
    prof = _profile_numbers().get(dominant, {})
    # the committed capture's per-launch figures are of the 150^3 problem
    # (3,375,000 elements); they grow with the elements of the run's problem
    prof_scale = E / 3375000.0
    traffic = prof["dram_bytes_per_launch"] * prof_scale if prof.get("dram_bytes_per_launch") else None
    roofline = {"bound": "hbm", "kernel": dominant, "achieved": achieved, "peak": hbm, "unit": "GB/s",
                "frac": achieved / hbm, "traffic": traffic,
                "traffic_source": _profile_numbers().get("source") if traffic else None,
                "peak_source": f"MEASURED_PEAKS.json hbm_gbs ({peak_kind})",
                "algorithmic_bytes_per_launch": dom_bytes}
    step_bytes = STEP_BYTES_PER_ELEM * E + STEP_BYTES_PER_NODE * N
    step_gbs = step_bytes * cycles / (ms * 1e-3) / 1e9
    fp64 = {"bound": "fp64", "peak_fma_per_s": fma_s.value, "peak_add_per_s": add_s.value,
            "peak_source": "lulesh_measure_fp64_peak (this run, this GPU)"}
    if prof.get("fp64_inst_per_element"):
        inst = prof["fp64_inst_per_element"] * E
        rate = inst / (dom_ms * 1e-3)
        fp64.update({"kernel": dominant, "achieved_inst_per_s": rate, "frac": rate / fma_s.value,
                     "fp64_inst_per_launch": inst, "fp64_inst_per_element": prof["fp64_inst_per_element"]})
    # the whole step: every step kernel's FP64 instructions per cycle over the
    # device-timed cycle
    allprof = _profile_numbers()
    if all(k in allprof for k in ("k_force", "k_node", "k_kinematics", "k_material")):
        step_inst = (sum(allprof[k]["fp64_inst_per_element"] for k in ("k_force", "k_kinematics", "k_material")) * E
                     + allprof["k_node"]["fp64_inst_per_node"] * N)
        step_rate = step_inst * cycles / (ms * 1e-3)
        fp64["step"] = {"fp64_inst_per_zone_cycle": step_inst / E, "achieved_inst_per_s": step_rate,
                        "frac": step_rate / fma_s.value}

    g.close()  # the remaining legs build their own problems
    blocks = None
    if not args.no_blocks and args.nx % 2 == 0:
        blocks = blocks_leg(L, torch, dev, args.nx // 2, 2, args.steps, ms / cycles)
    c3 = None
    if not args.no_c3:
        c3 = c3_leg(L, torch, dev, args.c3_nx, args.c3_cycles)
    c1 = None
    if not args.no_c1:
        c1 = c1_leg(L, torch, dev, cpu=world == 1 and not args.no_cpu)

    adjoint = None
    if not args.no_adjoint:
        adjoint = adjoint_leg(L, torch, dev, args.adj_nx, args.adj_cycles, args.adj_every, args.adj_dirs)

    cpu = None
    if world == 1 and not args.no_cpu:
        rate, used, n, dt = cpu_oracle_rate(args.nx, args.cpu_seconds)
        rate1, _, n1, dt1 = cpu_oracle_rate(args.nx, args.cpu_seconds / 2, serial=True)
        cpu = {"value": rate, "unit": UNIT, "cores": used, "kind": "port",
               "sample": f"{n} cycles of the {args.nx}^3 problem in {dt:.1f} s (oracle, OpenMP)",
               "single_thread": {"value": rate1, "cores": 1,
                                 "sample": f"{n1} cycles in {dt1:.1f} s (oracle, serial build)"}}

    clock_record = clocks.summary()
    if clock_record.get("sm_mhz"):
        clock_record["ms_per_step_x_sm_mhz"] = ms_max / cycles * clock_record["sm_mhz"]
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": cycles,
            "warmup": args.warmup, "ms_per_step": ms_max / cycles, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload_config(args.nx, args.mode, world),
            "device": "GB300",
            "roofline": roofline,
            "step_roofline": {"achieved": step_gbs, "peak": hbm, "unit": "GB/s", "frac": step_gbs / hbm,
                              "algorithmic_bytes_per_cycle": step_bytes},
            "fp64_roofline": fp64,
            "kernel_ms_per_cycle": {k: v / cycles for k, v in ktimes.items()},
            "dominant_kernel": dominant,
            "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": 5 * cycles,
            "clocks": clock_record, "timed_regions": {"repeats": repeats, "cycles_each": cycles,
                                                      "ms_each": region_ms, "reported": "median"},
            "tuning": tuning, "geometry_split": GEOMETRY_SPLIT[tuning["geometry"]], "ensemble": ensemble, "adjoint": adjoint,
            "c3_unbalanced_regions": c3, "c1_to_stoptime": c1, "blocks": blocks}
    print(json.dumps(line), flush=True)
    g.close()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--nx", type=int, default=NX)
    ap.add_argument("--mode", type=int, default=0)
    ap.add_argument("--config-cycles", type=int, default=200,
                    help="cycles of the configured problem the repeated timed regions span")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-tune", action="store_true", help="keep the default block sizes")
    ap.add_argument("--no-ensemble", action="store_true", help="skip the batched-ensemble leg")
    ap.add_argument("--ens-instances", type=int, default=256)
    ap.add_argument("--ens-cycles", type=int, default=300)
    ap.add_argument("--no-adjoint", action="store_true", help="skip the adjoint leg")
    ap.add_argument("--no-c3", action="store_true", help="skip the unbalanced-regions leg")
    ap.add_argument("--no-blocks", action="store_true", help="skip the multi-block (halo) leg")
    ap.add_argument("--no-c1", action="store_true", help="skip the 30^3 run-to-stoptime leg")
    ap.add_argument("--c3-nx", type=int, default=256)
    ap.add_argument("--c3-cycles", type=int, default=500)
    ap.add_argument("--adj-nx", type=int, default=48)
    ap.add_argument("--adj-cycles", type=int, default=200)
    ap.add_argument("--adj-every", type=int, default=20)
    ap.add_argument("--adj-dirs", type=int, default=16)
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be at least 3")
    return run_reference(args) if args.impl == "reference" else run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
