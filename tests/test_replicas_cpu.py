"""The N > 1 path of bench.py on CPU (gloo, world size 2) and the bounded
samples its CPU legs time.

The marching path does not shard (every region query needs the global visited
set), so ``bench.py --gpus N`` runs N independent replicas: a barrier before
the timed steps, the slowest rank's time (max over ranks) after them, and
rank 0 alone prints.  The reference arm runs on rank 0 only.
"""
import json
import os
import socket
import subprocess
import sys

import numpy as np
import pytest
import torch.multiprocessing as mp

from analyticmesh_gb300 import workloads as wl
from oracle import compare as CM
from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _max_worker(rank, world, port, values, out):
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    import bench

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        got = bench.max_over_ranks(values[rank], "cpu")
        dist.barrier()
        out.put((rank, got))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_gloo_two_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    values = [0.25, 1.75]
    procs = [ctx.Process(target=_max_worker, args=(r, 2, port, values, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    assert all(p.exitcode == 0 for p in procs)
    got = dict(q.get(timeout=5) for _ in range(2))
    assert got == {0: 1.75, 1: 1.75}


def test_max_over_ranks_single_process():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.max_over_ranks(3.5) == 3.5


@pytest.mark.skipif(not O.ref_available(), reason="reference CPU build unavailable")
def test_reference_arm_under_torchrun_prints_once():
    """``torchrun --nproc-per-node 2 bench.py --impl reference``: rank 0 prints
    one JSON line, rank 1 exits 0 without work."""
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--workload", "polytope", "--gpus", "2", "--steps", "1", "--warmup", "1"]
    env = dict(os.environ, OMP_NUM_THREADS="2")
    r = subprocess.run(cmd, cwd=ROOT, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True, timeout=300, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [json.loads(x) for x in r.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1
    line = lines[0]
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "reference"
    assert line["e2e"] == {"value": line["value"], "unit": "faces/s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}


@pytest.mark.skipif(not O.ref_available(), reason="reference CPU build unavailable")
def test_region_budget_stops_oracle_and_reference_at_the_same_batch():
    """A timed sample (region budget) ends both loops after the same batch
    with the same records."""
    m = wl.geometric([48, 48], 5)
    net = wl.net_arrays(m)
    st, pt = wl.seeds_for(m, init_num=64, seed=3)
    full = O.run_oracle(net, st, pt)
    ro = O.run_oracle(net, st, pt, region_budget=1500)
    rr = O.run_ref(net, st, pt, region_budget=1500, threads=1)
    assert full.num > ro.num >= 1500
    assert ro.num == rr.num
    assert CM.exact_records(ro, rr) == []
    # the budget is per call: the next unbudgeted run is complete again
    again = O.run_oracle(net, st, pt)
    assert again.num == full.num and np.array_equal(again.bits, full.bits)


def test_composition_flop_counts_of_the_bench_workloads():
    """8 (sum n_l n_l+1 + sum n_dst n_src) FLOP per region: 4 columns x 2 per
    multiply-add over every layer product and transformed connection."""
    sys.path.insert(0, ROOT)
    import bench

    for factory, want in ((wl.sphere, 8 * (3 * 128 ** 2 + 128)), (wl.deep, 8 * (5 * 256 ** 2 + 256)),
                          (wl.large_skip, 8 * (7 * 512 ** 2 + 512 + 512 * 3))):
        net = wl.net_arrays(factory())
        assert bench.composition_flops(net.nodes, net.arc_table, net.tms) == want
