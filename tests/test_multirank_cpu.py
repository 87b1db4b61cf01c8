"""Multi-rank host logic of bench.py on CPU (gloo, world size 2).

The plates of a batch are independent, so ranks shard them with no data-path
collective: each rank builds its own seeded shard, and torch.distributed is
used only for the barrier around the timed region and the max of the timers.
These tests run that logic as two gloo processes, and the reference arm as a
two-rank torchrun job (rank 0 measures and prints, rank 1 exits 0 without
work).
"""
import json
import os
import socket
import subprocess
import sys
import types

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, ws, port, out):
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(ws), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import numpy as np
    import torch.distributed as dist

    import __graft_entry__ as g
    import bench
    W = g.package().workloads
    r, n, _ = bench.dist_init(types.SimpleNamespace(impl="reference"))
    assert (r, n) == (rank, ws)
    scs, run = bench.rank_batch(W, 2, rank)
    sig = [float(np.asarray(s.mesh["coords"]).sum()) + float(np.sum(s.force_val)) for s in scs]
    allsig = [None] * ws
    dist.all_gather_object(allsig, (sig, run.dt, run.nft, W.dof_count(scs)))
    bench.barrier_sync(ws)
    t = bench.max_over_ranks(1.5 + rank, ws)
    bench.barrier_sync(ws)
    if rank == 0:
        with open(out, "w") as f:
            json.dump({"sigs": allsig, "t": t}, f)
    dist.destroy_process_group()


def test_two_rank_shards_and_timer_max(tmp_path):
    import torch.multiprocessing as mp
    out = str(tmp_path / "r.json")
    mp.start_processes(_rank_main, args=(2, _free_port(), out), nprocs=2, join=True, start_method="spawn")
    res = json.load(open(out))
    (s0, dt0, nft0, n0), (s1, dt1, nft1, n1) = res["sigs"]
    # same run (time step, length) on every rank, different plates per rank
    assert dt0 == dt1 and nft0 == nft1
    assert s0 != s1 and n0 > 0 and n1 > 0
    # timed region = max over ranks
    assert res["t"] == 2.5


@pytest.mark.timeout(300)
def test_reference_arm_under_torchrun(tmp_path):
    from oracle import oracle
    oracle.build()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), os.path.join(ROOT, "bench.py"),
           "--gpus", "2", "--impl", "reference", "--plates", "2", "--steps", "5", "--warmup", "3"]
    env = dict(os.environ, OMP_NUM_THREADS="2")
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=280, cwd=str(tmp_path), env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port" and d["e2e"]["h2d_bytes_per_step"] == 0
