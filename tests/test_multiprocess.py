"""The N > 1 host logic of the benchmark on CPU (gloo, world size 2): the
path runs as independent replicas, one per rank, joined only by a barrier
and the max-over-ranks timing; the reference arm runs on rank 0 alone and
the other ranks exit without work."""
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


def _worker(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    assert bench.dist_env() == (rank, world, rank)
    d = bench.init_dist(world, "gloo")
    d.barrier()
    # each replica reports its own time; the job time is the slowest rank's
    out[rank] = bench.max_over_ranks(d, 10.0 + 5.0 * rank)
    d.barrier()
    d.destroy_process_group()


def test_max_over_ranks_with_gloo():
    import torch.multiprocessing as mp
    port = _free_port()
    out = mp.get_context("spawn").Manager().dict()
    mp.start_processes(_worker, args=(2, port, out), nprocs=2, join=True, start_method="spawn")
    assert dict(out) == {0: 15.0, 1: 15.0}


@pytest.mark.timeout(600)
def test_reference_arm_under_torchrun_prints_once():
    """`torchrun --nproc-per-node 2 bench.py --impl reference`: rank 0 prints
    one JSON line, rank 1 exits 0 without output."""
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port),
           os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2",
           "--steps", "1", "--warmup", "3", "--luni", "1"]
    env = dict(os.environ, OMP_NUM_THREADS="2")
    res = subprocess.run(cmd, capture_output=True, text=True, env=env, cwd=ROOT, timeout=600)
    assert res.returncode == 0, res.stderr[-2000:]
    lines = [ln for ln in res.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0


def test_reference_arm_loads_no_product_code():
    """The reference arm runs the oracle on the oracle's own mesh: neither
    the product package nor its library is loaded, and its config is the
    GPU arm's config."""
    code = (
        "import sys, json, io, contextlib; sys.path.insert(0, %r); import bench\n"
        "a = type('A', (), dict(n=5, luni=1, steps=1, warmup=3))()\n"
        "buf = io.StringIO()\n"
        "with contextlib.redirect_stdout(buf): bench.run_reference(a, 0, 1)\n"
        "maps = open('/proc/self/maps').read()\n"
        "d = json.loads(buf.getvalue())\n"
        "print(json.dumps(dict(pkg='nmesh_gb300' in sys.modules, so='libnmg' in maps, "
        "cfg=d['config'] == bench.workload_config(5, 1), v=d['value'] > 0)))\n" % ROOT)
    env = dict(os.environ, OMP_NUM_THREADS="2")
    res = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env,
                         cwd=ROOT, timeout=300)
    assert res.returncode == 0, res.stderr[-2000:]
    assert json.loads(res.stdout.splitlines()[-1]) == dict(pkg=False, so=False, cfg=True, v=True)
