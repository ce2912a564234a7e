"""Analytic Marching throughput on GB300: analytic faces / second.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--form mixed|float32|float64]
                    [--workload large_skip|sphere|deep|polytope|batched]

Workload (default): the largest single-GPU configuration, the skip-connected
network 3 -> [512] x 8 -> 1 with the 3-D input added into layer 4 (geometric
init r = 0.6 + N(0, 0.01), seed 3, fp32 weights; 4096 constraint rows per
region, ~6.8 M regions), with 1024 dichotomy seed points (seed 1); synthetic,
seeded.  Chosen form: mixed precision.  One step = one complete Analytic
Marching of that network (every region visited, every face polygon built),
the window of the reference's am_time (backend/main.py:455-465): seed init
and mesh export are outside.  ``--workload sphere`` (3 -> [128] x 4 -> 1),
``deep`` (3 -> [256] x 6 -> 1 at level 0.35) and ``batched`` (the networks of
the batched configuration marched at once) select the other configurations.

``value``: faces / second with inputs resident in HBM, CUDA-event timed on
the launching stream, L2 flushed (256 MiB write) before every timed step.
``e2e``: the same through the C ABI with host buffers -- the weights, biases,
seed states and points wait in pinned host memory and are copied host ->
device inside the step, and the welded mesh is read back (am_combine_mesh +
am_get_mesh).

``--impl reference`` times the reference's own marching loop compiled for the
host cores (oracle/_ref, all host threads) on a bounded sample of the same
workload (its first regions: 4096 of the skip network, 16384 of the deep one,
65536 of the sphere).  Under torchrun every rank runs an independent replica
(the path does not shard); rank 0 prints one JSON line.

The line also carries the chosen result's error report against FP64
(``errors``: max |f(v)| and the largest vertex error over an evenly spaced
sample of its faces, am_error_report) and the plain FP32 form's outcome on the
same workload (``plain_fp32_value`` or ``plain_note``), its error report too.
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
sys.path.insert(0, ROOT)

# the reference arm's bounded sample (regions per step): about 10-30 s of the
# host cores per step
REF_SAMPLE = {"sphere": 65536, "deep": 16384, "large_skip": 4096, "polytope": 65536}
REF_SAMPLE_REGIONS = 65536
ERROR_SAMPLE = 4096  # regions of the error report
# DRAM bytes (read + write) per region of the two heavy kernels in the mixed
# form, from one ncu capture each (--set full, dram__bytes_read.sum +
# dram__bytes_write.sum): the sphere workload's wave of 12,672 regions, the
# deep workload's wave of ~40,150 regions and the skip network's wave of ~12,030
NCU_TRAFFIC_PER_REGION = {("sphere", "mixed"): {"compose": (1.214e6 + 45.631e6) / 12672,
                                                "polygon": (109.571e6 + 4.067e6) / 12672},
                          # a wave of ~12,030 regions of a bounded march (the full march is too
                          # large to capture): per region, scaled to the step's regions
                          ("large_skip", "mixed"): {"compose": (52.502e6 + 747.137e6) / 12030,
                                                    "polygon": (806.011e6 + 16.420e6) / 12030},
                          ("deep", "mixed"): {"compose": (27.491e6 + 957.757e6) / 40150,
                                              "polygon": (1018.464e6 + 20.326e6) / 40150}}
# the composition's tensor pipe (sm__pipe_tensor_cycles_active) in the same
# captures: the mixed form issues six bf16 products per algorithmic product,
# so `frac` (algorithmic FLOP/s over the bf16 peak) stays below 1/6 even with
# the pipe saturated; this is the pipe's own share of the kernel's time
NCU_TENSOR_ACTIVE = {("large_skip", "mixed"): 0.436, ("sphere", "mixed"): 0.152, ("deep", "mixed"): 0.257}


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--form", default="mixed", choices=["mixed", "float32", "float64"])
    p.add_argument("--workload", default="large_skip",
                   choices=["large_skip", "sphere", "deep", "polytope", "batched"])
    p.add_argument("--nets", type=int, default=64,
                   help="batched workload: the first NETS of the 64 networks (all 64: ~4.8 s per step on GB300)")
    p.add_argument("--seeds", type=int, default=1024)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--tune-sample", type=int, default=65536,
                   help="batched workload: regions per autotuner sample run")
    p.add_argument("--host-loop", action="store_true",
                   help="drive the wave loop from the host (one launch sequence per wave): for ncu launch lists, "
                        "which cannot see kernels inside conditional graphs")
    p.add_argument("--profile", action="store_true",
                   help="warm-up + timed steps only (for ncu launch lists): no e2e, phase, plain or CPU legs")
    p.add_argument("--max-regions", type=int, default=0,
                   help="with --profile: stop every marching after the wave that passes this many regions "
                        "(a bounded march small enough for a full ncu capture)")
    return p.parse_args()


def dist_init(args):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch
        import torch.distributed as dist

        if args.impl == "ours":
            torch.cuda.set_device(local)
            dist.init_process_group("nccl")
        else:
            dist.init_process_group("gloo")
    return ws, rank, local


def max_over_ranks(value, device="cpu"):
    """The largest ``value`` over all ranks (the slowest replica's time under
    torchrun); ``value`` itself in a single process.  ``device`` is where the
    process group's backend reduces (a CUDA device for NCCL, "cpu" for gloo)."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def composition_flops(nodes, arc_table, tms):
    """Algorithmic FLOPs of one region's composition: 4 columns x 2 flop per
    multiply-add over every layer product and every transformed connection
    (the input's included: 8 (sum n_l n_l+1 + sum n_dst n_src))."""
    macs = sum(nodes[i] * nodes[i + 1] for i in range(1, len(nodes) - 1))
    for row in arc_table:
        for c in range(int(row[0])):
            t = int(row[2 + 2 * c])
            if tms[t].size:
                macs += tms[t].shape[0] * tms[t].shape[1]
    return 8 * macs


def workload(name, nseeds):
    from analyticmesh_gb300 import workloads as wl

    model = {"sphere": wl.sphere, "deep": wl.deep, "large_skip": wl.large_skip, "polytope": wl.polytope}[name]()
    net = wl.net_arrays(model)
    iso = wl.DEEP_ISO if name == "deep" else 0.0
    states, points = wl.seeds_for(model, init_num=nseeds, seed=1, iso=iso)
    desc = {"sphere": "sphere MLP 3-[128]x4-1, seed 1", "deep": "perturbed MLP 3-[256]x6-1, seed 2",
            "large_skip": "skip MLP 3-[512]x8-1 (input into layer 4), seed 3",
            "polytope": "polytope MLP 3-14-1, seed 0"}[name]
    if iso:
        desc += ", level %g" % iso
    net.iso = iso
    return net, states, points, desc


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        try:
            rows = [r.split(",") for r in open(self.path).read().strip().splitlines() if r.strip()]
            os.unlink(self.path)
        except Exception:
            return out
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx = float(r[2])
                for nm, v in zip(names, r[5:9]):
                    if v.strip().lower() in ("active", "1"):
                        reasons.add(nm)
            except Exception:
                pass
        if sm:
            out.update(sm_mhz=statistics.median(sm), sm_max_mhz=mx, reasons=sorted(reasons), samples=len(sm))
        return out


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), float(p["bf16_tflops"]), "measured"
    except Exception:
        return 6800.0, 1900.0, "fallback"


def reference_workload(args):
    """The networks, seeds and per-network region budgets the reference arm
    marches: the bench's workload, or for ``batched`` the same NETS networks
    one after the other (the reference re-Inits per architecture,
    backend/main.py:437-446), the sample split evenly between them."""
    if args.workload != "batched":
        net, states, points, desc = workload(args.workload, args.seeds)
        return [(net, states, points, REF_SAMPLE[args.workload])], desc
    from analyticmesh_gb300 import workloads as wl

    items = []
    budget = max(1024, REF_SAMPLE_REGIONS // max(1, args.nets))
    for i, m in enumerate(wl.batched(args.nets, 100)):
        net = wl.net_arrays(m)
        net.iso = 0.0
        st, pt = wl.seeds_for(m, init_num=args.seeds, seed=100 + i)
        items.append((net, st, pt, budget))
    desc = "%d MLPs, seeds 100..%d, widths {32..512}, depths 2..8, one after the other" % (args.nets, 99 + args.nets)
    return items, desc


def reference_step(items, dtype, threads, kind):
    """One step of the reference arm: (faces, seconds) over every item,
    each marched up to its region budget inside the reference's am_time
    window (the oracle restatement's wall time when the reference build is
    unavailable)."""
    from oracle import oracle as O

    faces, secs = 0, 0.0
    for net, states, points, budget in items:
        if kind == "reference":
            tm = {}
            r = O.run_ref(net, states, points, iso=net.iso, dtype=dtype, threads=threads, region_budget=budget,
                          timing=tm)
            secs += tm["am_seconds"]
        else:
            t0 = time.perf_counter()
            r = O.run_oracle(net, states, points, iso=net.iso, dtype=dtype, region_budget=budget)
            secs += time.perf_counter() - t0
        faces += int((r.nverts >= 3).sum())
    return faces, secs


def reference_kind():
    """The cpu_baseline kind: ``reference`` when the reference's own loop is
    built for the host (or can be built), else ``port`` (the oracle
    restatement)."""
    from oracle import build_ref
    from oracle import oracle as O

    try:
        if not O.ref_available():
            build_ref.build_ref()
        return "reference" if O.ref_available() else "port"
    except Exception:
        return "port"


def run_reference(args, rank, ws):
    """--impl reference: the reference's own loop on the host cores.  Under
    torchrun rank 0 alone runs and prints; the other ranks return."""
    if rank != 0:
        return
    items, desc = reference_workload(args)
    threads = os.cpu_count() or 1
    kind = reference_kind()
    dtype = "float64" if args.form == "float64" else "float32"
    rates = []
    faces = 0
    for i in range(args.warmup + args.steps):
        faces, secs = reference_step(items, dtype, threads, kind)
        if i >= args.warmup:
            rates.append(faces / secs)
    value = statistics.mean(rates)
    sample = "first %d regions of %s per step" % (
        items[0][3], "the workload" if len(items) == 1 else "each network")
    line = {
        "impl": "reference", "metric": "analytic_faces_per_sec", "value": value, "unit": "faces/s",
        "n_gpus": args.gpus, "steps": len(rates), "warmup": args.warmup, "ms_per_step": 1e3 * faces / value,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32" if dtype == "float32" else "f64",
        "data": "synthetic (seeded network and dichotomy seeds)",
        "config": {"workload": desc, "seeds": args.seeds, "sample": sample},
        "cpu_baseline": {"value": value, "unit": "faces/s", "cores": threads, "kind": kind,
                         "sample": "%s, %s (OpenMP, %d threads)" % (
                             sample, "reference loop built for the host" if kind == "reference"
                             else "oracle restatement", threads)},
        "e2e": {"value": value, "unit": "faces/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def cpu_baseline(net, states, points, dtype, budget):
    """The cpu_baseline object of the bench line: the reference's loop built
    for the host (all threads) on the first ``budget`` regions of the
    workload, or the oracle restatement on the same sample."""
    threads = os.cpu_count() or 1
    kind = reference_kind()
    try:
        faces, secs = reference_step([(net, states, points, budget)], dtype, threads, kind)
    except Exception:  # a reference build that loads but cannot run: the restatement instead
        kind = "port"
        faces, secs = reference_step([(net, states, points, budget)], dtype, threads, kind)
    return {"value": faces / secs, "unit": "faces/s", "cores": threads, "kind": kind,
            "sample": "first %d regions of the workload, %s (OpenMP, %d threads)" % (
                budget, "reference loop built for the host" if kind == "reference"
                else "oracle restatement", threads)}


def bench_batched(args, ws, rank, local):
    """--workload batched: the 64-network workload (seeds 100..163, widths
    from {32, 64, 128, 256, 512}, depths 2..8, geometric init + N(0, 0.01)),
    every network with its own dichotomy seeds.  Chosen form: mixed
    precision, all networks marched at once (am_run_batch).  Plain form: FP32,
    one network after the other (am_analytic_marching each), as a user of the
    reference marches them (it re-Inits per architecture)."""
    import numpy as np
    import torch

    from analyticmesh_gb300 import engine, workloads as wl

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    models = wl.batched(args.nets, 100)
    nets, sts, pts = [], [], []
    for i, m in enumerate(models):
        nets.append(wl.net_arrays(m))
        st, pt = wl.seeds_for(m, init_num=args.seeds, seed=100 + i, device=dev)
        sts.append(torch.tensor(st, device=dev))
        pts.append(torch.tensor(pt, device=dev))

    def dev_net(n, dt):
        d = dict(W=[torch.tensor(w, dtype=dt, device=dev) for w in n.W], b=[torch.tensor(b, dtype=dt, device=dev) for b in n.b],
                 tms=[torch.tensor(t, dtype=dt, device=dev) for t in n.tms], w_extra=n.w_extra, b_extra=n.b_extra)
        return type("DevNet", (), d)

    dnets = [dev_net(n, torch.float32) for n in nets]
    pts = [p.float() for p in pts]
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    chosen = [engine.Engine("mixed", n.nodes, n.arc_table, n.num_extra) for n in nets]
    # autotuner (untimed setup): composition tile and warps per face per architecture
    tuned = [engine.autotune(e, n, s_, p_, sample_regions=args.tune_sample)
             for e, n, s_, p_ in zip(chosen, dnets, sts, pts)]
    for _ in range(args.warmup):
        engine.run_batch(chosen, dnets, sts, pts)
    torch.cuda.synchronize()
    if ws > 1:
        torch.distributed.barrier()
    times, faces = [], 0
    with Clocks(local) as clk:
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            wall = engine.run_batch(chosen, dnets, sts, pts)
            times.append(wall / 1e3)
            faces = sum(e.stats()["num_faces"] for e in chosen)
    step_s = max_over_ranks(sum(times) / len(times), dev)
    value = ws * faces / step_s
    clocks = clk.summary()
    regions = [e.stats()["num_regions"] for e in chosen]

    # end to end: inputs in pinned host memory (prepared outside the timed
    # region) copied in by the engines, every mesh welded and read back
    pin = lambda a: torch.tensor(np.asarray(a), dtype=torch.float32).pin_memory()
    hnets = [type("HostNet", (), dict(W=[pin(w) for w in n.W], b=[pin(b) for b in n.b], tms=[pin(t) for t in n.tms],
                                      w_extra=n.w_extra, b_extra=n.b_extra)) for n in nets]
    hsts = [s.cpu().pin_memory() for s in sts]
    hpts = [p.cpu().pin_memory() for p in pts]
    t0 = time.perf_counter()
    engine.run_batch(chosen, hnets, hsts, hpts)
    meshes = [e.combine() for e in chosen]
    e2e = ws * faces / (time.perf_counter() - t0)
    h2d = sum(t.numel() * t.element_size() for n in hnets for t in n.W + n.b + n.tms) + \
        sum(t.numel() * t.element_size() for t in hsts + hpts)
    d2h = sum(m.verts.nbytes + m.face_sizes.nbytes + m.face_indices.nbytes for m in meshes)

    # the chosen results go back before the plain form runs (tens of GB)
    for e in chosen:
        e.close()
    del chosen
    torch.cuda.empty_cache()

    # plain form: FP32, one network at a time (each engine closed before the
    # next; a run that passes twice the chosen form's regions for its network
    # is stopped there and counted as not converging)
    from analyticmesh_gb300 import _lib

    plain_ms, plain_faces, diverged = 0.0, 0, []
    for i, (na, n, s_, p_) in enumerate(zip(nets, dnets, sts, pts)):
        e = engine.Engine("float32", na.nodes, na.arc_table, na.num_extra)
        e.set_option(_lib.AM_OPT_MAX_REGIONS, 2 * int(regions[i]))
        try:
            e.run(n.W, n.b, s_, p_, n.tms)
            ms = []
            for _ in range(max(1, args.steps // 2)):
                flush.zero_()
                ev0 = torch.cuda.Event(enable_timing=True)
                ev1 = torch.cuda.Event(enable_timing=True)
                ev0.record()
                f = e.run(n.W, n.b, s_, p_, n.tms)["num_faces"]
                ev1.record()
                ev1.synchronize()
                ms.append(ev0.elapsed_time(ev1))
            plain_ms += statistics.mean(ms)
            plain_faces += f
        except _lib.AmError as exc:
            if exc.status != _lib.AM_ERR_CAPACITY:
                raise
            diverged.append(i)
        e.close()
        torch.cuda.empty_cache()
    plain = ws * plain_faces / (plain_ms / 1e3) if plain_ms > 0 and not diverged else None
    plain_note = ("plain FP32 does not converge on networks %s (stopped at twice the chosen form's regions)"
                  % diverged) if diverged else "float32, networks one after the other"
    if rank != 0:
        return
    line = {
        "metric": "analytic_faces_per_sec", "value": value, "unit": "faces/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * step_s, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 (bf16x3 composition, f64 solves)",
        "data": "synthetic (seeded networks and dichotomy seed points)",
        "config": {"workload": "%d MLPs, seeds 100..%d, widths {32..512}, depths 2..8, all marched at once"
                               % (args.nets, 99 + args.nets), "seeds": args.seeds, "form": "mixed, batched",
                   "faces_per_step": faces, "regions_per_step": int(sum(regions)),
                   "largest_network_regions": int(max(regions)), "l2": "256 MiB flush before every timed step",
                   "autotune": {"sample_regions": args.tune_sample,
                                "tile_and_face_warps": ["%d/%d" % t for t in tuned]},
                   "parallelism": "replicas" if ws > 1 else "single GPU"},
        "e2e": {"value": e2e, "unit": "faces/s", "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
        "plain_fp32_value": plain, "plain_note": plain_note,
        "chosen_vs_plain": (value / plain) if plain else None, "clocks": clocks,
    }
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    ws, rank, local = dist_init(args)
    if args.impl == "reference":
        run_reference(args, rank, ws)
        return
    if args.workload == "batched":
        bench_batched(args, ws, rank, local)
        return
    import numpy as np
    import torch

    from analyticmesh_gb300 import _lib, engine

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    net, states, points, desc = workload(args.workload, args.seeds)
    form = args.form
    tt = torch.float64 if form == "float64" else torch.float32
    # inputs resident in HBM
    W = [torch.tensor(w, dtype=tt, device=dev) for w in net.W]
    B = [torch.tensor(b, dtype=tt, device=dev) for b in net.b]
    TM = [torch.tensor(t, dtype=tt, device=dev) for t in net.tms]
    S = torch.tensor(states, dtype=torch.uint8, device=dev)
    P = torch.tensor(points, dtype=tt, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)

    eng = engine.Engine(form, net.nodes, net.arc_table, net.num_extra)
    if args.host_loop:
        eng.set_option(_lib.AM_OPT_GRAPH, 0)

    if args.profile and args.max_regions > 0:
        eng.set_option(_lib.AM_OPT_MAX_REGIONS, args.max_regions)

    def step():
        try:
            return eng.run(W, B, S, P, TM, None, None, net.iso, False, stream=stream)
        except _lib.AmError as exc:  # the bounded march of --max-regions
            if not (args.max_regions > 0 and exc.status == _lib.AM_ERR_CAPACITY):
                raise
            return eng.stats()

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    if ws > 1:
        torch.distributed.barrier()
    times, faces, launches = [], [], 0
    with Clocks(local) as clk:
        for _ in range(args.steps):
            flush.zero_()
            ev0 = torch.cuda.Event(enable_timing=True)
            ev1 = torch.cuda.Event(enable_timing=True)
            ev0.record(stream)
            s = step()
            ev1.record(stream)
            ev1.synchronize()
            times.append(ev0.elapsed_time(ev1) / 1e3)
            faces.append(s["num_faces"])
            launches += s["kernel_launches"] + 1
    torch.cuda.synchronize()
    if args.profile:
        if rank == 0:
            print(json.dumps({"metric": "analytic_faces_per_sec", "value": sum(faces) / sum(times), "unit": "faces/s",
                              "profile": True, "steps": args.steps, "launches": launches}), flush=True)
        eng.close()
        return
    total = max_over_ranks(sum(times), dev)
    if ws > 1:
        torch.distributed.barrier()
    value = ws * sum(faces) / total
    clocks = clk.summary()

    # end to end through the C ABI with host buffers: the step's inputs sit in
    # pinned host memory (prepared once, outside the timed region); the engine
    # copies them to the device inside every step, and the welded mesh comes back
    pin = lambda a, dt_: torch.tensor(np.asarray(a), dtype=dt_).pin_memory()
    hW = [pin(w, tt) for w in net.W]
    hB = [pin(b, tt) for b in net.b]
    hT = [pin(t, tt) for t in net.tms]
    hS = pin(states, torch.uint8)
    hP = pin(points, tt)
    h2d = sum(t.numel() * t.element_size() for t in hW + hB + hT + [hS, hP])
    e2e_faces, e2e_secs, d2h = 0, 0.0, 0
    for i in range(max(5, args.steps) + 1):  # the first call is untimed
        t0 = time.perf_counter()
        s = eng.run(hW, hB, hS, hP, hT, None, None, net.iso, False)
        mesh = eng.combine()
        dt = time.perf_counter() - t0
        if i > 0:
            e2e_faces += s["num_faces"]
            e2e_secs += dt
        d2h = mesh.verts.nbytes + mesh.face_sizes.nbytes + mesh.face_indices.nbytes
    e2e = ws * e2e_faces / max_over_ranks(e2e_secs, dev)

    # per-phase breakdown and the dominant kernel's roofline (separate, untimed run)
    eng.set_option(_lib.AM_OPT_PHASE_TIMING, 1)
    sp = step()
    eng.set_option(_lib.AM_OPT_PHASE_TIMING, 0)
    phases = {"compose_ms": sp["compose_ms"], "polygon_ms": sp["polygon_ms"], "frontier_ms": sp["frontier_ms"]}
    hbm, tflops, peak_kind = measured_peaks()
    regions = sp["num_regions"]
    ALL = int(sum(net.nodes[1:-1])) + net.num_extra
    flops = composition_flops(net.nodes, net.arc_table, net.tms) * regions
    elem = 8 if form == "float64" else 4
    poly_bytes = regions * (ALL * 4 * elem + 4 * elem + 12 * 6)
    per_region = NCU_TRAFFIC_PER_REGION.get((args.workload, form), {})
    if phases["compose_ms"] >= phases["polygon_ms"]:
        ach = flops / (phases["compose_ms"] / 1e3) / 1e12
        tr = per_region.get("compose")
        roof = {"kernel": "compose", "bound": "tensor", "achieved": ach, "peak": tflops, "unit": "TFLOP/s",
                "frac": ach / tflops, "traffic": tr * regions if tr else None, "peak_kind": peak_kind,
                "algorithmic": "%d FLOP/region x %d regions" % (flops // max(regions, 1), regions),
                "products_per_flop": 6, "tensor_pipe_active_ncu": NCU_TENSOR_ACTIVE.get((args.workload, form))}
    else:
        ach = poly_bytes / (phases["polygon_ms"] / 1e3) / 1e9
        tr = per_region.get("polygon")
        roof = {"kernel": "polygon", "bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s",
                "frac": ach / hbm, "traffic": tr * regions if tr else None, "peak_kind": peak_kind,
                "algorithmic": "%d B/region x %d regions" % (poly_bytes // max(regions, 1), regions)}
    if roof["traffic"] is not None:
        roof["traffic_note"] = "ncu dram bytes per region of one captured wave x regions per step"

    # the chosen result's error report against FP64 (an evenly spaced sample
    # of the faces of the phase-timed run above; outside every timed region)
    errors = eng.error_report(ERROR_SAMPLE)
    errors["sample_regions"] = ERROR_SAMPLE

    # the chosen engine's stores go back before the plain form's are built
    # (large networks hold tens of GB of regions)
    eng.close()
    torch.cuda.empty_cache()
    plain = None
    plain_note = None
    plain_errors = None
    if form != "float32":
        ep = engine.Engine("float32", net.nodes, net.arc_table, net.num_extra)
        # a plain run that passes twice the chosen form's regions is stopped
        # there (AM_ERR_CAPACITY) and reported as not converging
        ep.set_option(_lib.AM_OPT_MAX_REGIONS, 2 * regions)
        try:
            W32 = [w.float() for w in W]
            B32 = [b.float() for b in B]
            T32 = [t.float() for t in TM]
            P32 = P.float()
            for _ in range(2):
                ep.run(W32, B32, S, P32, T32, None, None, net.iso, False, stream=stream)
            pt = []
            for _ in range(max(3, args.steps // 2)):
                flush.zero_()
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                s2 = ep.run(W32, B32, S, P32, T32, None, None, net.iso, False, stream=stream)
                e1.record(stream)
                e1.synchronize()
                pt.append(s2["num_faces"] / (e0.elapsed_time(e1) / 1e3))
            plain = statistics.mean(pt) * ws
            plain_errors = ep.error_report(ERROR_SAMPLE)
            plain_note = "plain FP32: %d regions, %d faces per step" % (s2["num_regions"], s2["num_faces"])
        except _lib.AmError as exc:  # e.g. the FP32 form's store outgrowing the GPU
            if exc.status == _lib.AM_ERR_CAPACITY:
                st2 = ep.stats()
                plain_note = ("plain FP32 run does not converge: stopped after %d regions (the chosen form's "
                              "march has %d); %s" % (st2["num_regions"], regions, str(exc)[:120]))
                try:
                    plain_errors = ep.error_report(ERROR_SAMPLE)
                except _lib.AmError:
                    plain_errors = None
            else:
                plain_note = "plain FP32 run failed: %s" % str(exc)[:160]
        finally:
            ep.close()

    if rank != 0:
        return
    cpu = None
    if ws == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(net, states, points, "float64" if form == "float64" else "float32",
                           REF_SAMPLE.get(args.workload, REF_SAMPLE_REGIONS))
    line = {
        "metric": "analytic_faces_per_sec", "value": value, "unit": "faces/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": {"float32": "f32", "float64": "f64", "mixed": "f32 (bf16x3 composition, f64 solves)"}[form],
        "data": "synthetic (seeded network weights and dichotomy seed points)",
        "config": {"workload": desc, "seeds": args.seeds, "form": form, "faces_per_step": faces[-1],
                   "regions_per_step": regions, "l2": "256 MiB flush before every timed step",
                   "parallelism": "replicas" if ws > 1 else "single GPU"},
        "e2e": {"value": e2e, "unit": "faces/s", "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
        "roofline": roof, "phases_ms": phases, "errors": errors, "plain_fp32_value": plain,
        "plain_note": plain_note, "plain_errors": plain_errors,
        "chosen_vs_plain": (value / plain) if plain else None, "cpu_baseline": cpu, "clocks": clocks,
        "gpu_launches": launches,
    }
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
