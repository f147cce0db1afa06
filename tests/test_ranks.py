"""The multi-GPU form of the benchmark is weak scaling with no exchange: every
rank builds the full grid with its own permutation seeds, and rank 0 reports
the chunks of all ranks over the slowest rank's time.  This checks that host
logic with two gloo ranks on the CPU (the oracle stands in for the GPU build)."""
import os
import sys
from pathlib import Path

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parent.parent


def _rank_main(rank, world, port, q):
    sys.path.insert(0, str(ROOT))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch
    import bench
    from oracle import oracle as O
    from underwaterworld_gb300 import abi
    dist.init_process_group("gloo", rank=rank, world_size=world)
    seeds = bench.rank_seeds(rank)
    p, d = bench.workload(seeds[0])
    sub = d[:32]
    from underwaterworld_gb300.chunk import make_descs
    b = O.build_chunks(p, make_descs(sub["pos"], sub["cells"]), precision=O.F32)
    counts = torch.tensor([len(sub), int(b.totals[0])], dtype=torch.float64)
    t = torch.tensor([0.5 + rank], dtype=torch.float64)          # this rank's time
    dist.all_reduce(counts, op=dist.ReduceOp.SUM)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    q.put((rank, seeds, counts.tolist(), float(t.item()), int(b.totals[0])))
    dist.destroy_process_group()


def test_two_gloo_ranks_weak_scaling(built_lib, oracle):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for pr in procs:
        pr.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for pr in procs:
        pr.join(timeout=60)
        assert pr.exitcode == 0
    (r0, s0, c0, t0, v0), (r1, s1, c1, t1, v1) = res
    assert not set(s0) & set(s1), "ranks must use distinct seeds"
    assert c0 == c1 == [64.0, float(v0 + v1)]   # chunks and vertices of both ranks
    assert t0 == t1 == 1.5                      # the slowest rank's time


def test_reference_arm_runs_on_rank_zero_only(built_lib, oracle, monkeypatch, capsys):
    """`bench.py --impl reference` under a 2-rank launch: rank 1 exits without
    work or output; rank 0 times exactly --steps bounded steps on the host
    cores and prints one JSON line for the launch's world size."""
    import argparse
    import json
    sys.path.insert(0, str(ROOT))
    import bench
    monkeypatch.setattr(bench, "REF_BUDGET_S", 0.5)
    monkeypatch.setattr(bench, "REF_ONE_THREAD_S", 0.2)
    args = argparse.Namespace(steps=7, warmup=3)
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")
    bench.run_reference(args)
    assert capsys.readouterr().out == ""
    monkeypatch.setenv("RANK", "0")
    bench.run_reference(args)
    lines = [l for l in capsys.readouterr().out.splitlines() if l.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["steps"] == 7 and d["warmup"] == 3 and d["n_gpus"] == 2
    assert d["value"] > 0 and d["unit"] == bench.UNIT and d["metric"] == bench.METRIC
    assert d["cpu_baseline"]["value"] == d["value"] and d["e2e"]["h2d_bytes_per_step"] == 0
    assert 32 <= d["chunks_per_timed_step"] <= 4096
    assert d["threads"] >= 1 and d["single_thread"]["cores"] == 1 and d["single_thread"]["value"] > 0
    assert d["config"]["chunks_per_step"] == 4096


def _reference_arm_maps(q):
    """In a fresh process: run the reference arm briefly, then report which
    shared objects of this repository the process has mapped."""
    import argparse
    import io
    from contextlib import redirect_stdout
    sys.path.insert(0, str(ROOT))
    os.environ.update(RANK="0", WORLD_SIZE="1")
    import bench
    bench.REF_BUDGET_S, bench.REF_ONE_THREAD_S = 0.3, 0.1
    with redirect_stdout(io.StringIO()):
        bench.run_reference(argparse.Namespace(steps=2, warmup=1))
    maps = Path("/proc/self/maps").read_text()
    q.put(sorted({line.split()[-1] for line in maps.splitlines() if line.endswith(".so") and str(ROOT) in line}))


def test_reference_arm_does_not_load_the_gpu_library(built_lib, oracle):
    """The reference arm runs the oracle only: libuww_gb300.so is never mapped
    into its process (its parameters and struct layouts come from
    underwaterworld_gb300.layout)."""
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    pr = ctx.Process(target=_reference_arm_maps, args=(q,))
    pr.start()
    mapped = q.get(timeout=300)
    pr.join(timeout=60)
    assert pr.exitcode == 0
    assert any(m.endswith("liboracle.so") for m in mapped), mapped
    assert not any("libuww" in Path(m).name for m in mapped), mapped
