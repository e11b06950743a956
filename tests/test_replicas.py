"""The N>1 benchmark path on the CPU: one process per GPU, each running an independent replica of
the factorisation ("replicas only": one matrix's tiled factorisation runs on one GPU), joined by a
barrier and a max over ranks of the step time. Checked here with world size 2 over gloo:
  * bench.dist_setup / barrier / max_over_ranks agree across two spawned ranks;
  * the reference arm under torch.distributed.run: rank 0 alone prints one JSON line, the other
    rank exits 0 without work.
"""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, ws, port, out_dir):
    os.environ.update({"RANK": str(rank), "LOCAL_RANK": str(rank), "WORLD_SIZE": str(ws),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, ROOT)
    import bench
    got_ws, got_rank, _ = bench.dist_setup(None)
    bench.barrier(got_ws)
    m = bench.max_over_ranks(got_ws, 10.0 * (got_rank + 1))
    bench.barrier(got_ws)
    import torch.distributed as dist
    dist.destroy_process_group()
    with open(os.path.join(out_dir, "rank%d.json" % rank), "w") as f:
        json.dump({"ws": got_ws, "rank": got_rank, "max": m}, f)


def test_barrier_and_max_over_two_gloo_ranks(tmp_path):
    pytest.importorskip("torch.distributed")
    import torch.multiprocessing as mp
    ws, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    procs = [ctx.Process(target=_rank_main, args=(r, ws, port, str(tmp_path))) for r in range(ws)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    for r in range(ws):
        d = json.load(open(tmp_path / ("rank%d.json" % r)))
        assert d == {"ws": ws, "rank": r, "max": 20.0}


def test_reference_arm_under_torchrun_prints_once(gbx):
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py", "--impl", "reference",
           "--gpus", "2", "--steps", "1", "--warmup", "1", "--N", "512", "--NB", "128"]
    env = dict(os.environ, OMP_NUM_THREADS="1")
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=300, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port" and d["e2e"]["h2d_bytes_per_step"] == 0
    # the reference arm times the same workload as the GPU arm
    assert d["config"] == bench_config(512, 128, 1, 2)


def bench_config(N, NB, nrhs, ws):
    sys.path.insert(0, ROOT)
    import argparse
    import bench
    return bench.main_config(argparse.Namespace(N=N, NB=NB, nrhs=nrhs), ws)
