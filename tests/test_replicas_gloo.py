"""The N > 1 path of bench.py (independent replicas, max-over-ranks timing,
barrier) on two CPU processes over gloo."""
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import os, sys
sys.path.insert(0, {root!r})
import torch.distributed as dist
import bench
dist.init_process_group("gloo")
rank, world = dist.get_rank(), dist.get_world_size()
bench.barrier(world)
m = bench.max_over_ranks(10.0 + rank, world)
assert m == 10.0 + world - 1, m
bench.barrier(world)
print("ok", rank, m, flush=True)
dist.destroy_process_group()
"""


def free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def test_two_replicas_over_gloo():
    port = free_port()
    procs = []
    for rank in range(2):
        env = dict(os.environ, MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE="2",
                   LOCAL_RANK=str(rank))
        procs.append(subprocess.Popen([sys.executable, "-c", CHILD.format(root=ROOT)], env=env,
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    outs = [p.communicate(timeout=120) for p in procs]
    for p, (o, e) in zip(procs, outs):
        assert p.returncode == 0, e
        assert o.startswith("ok"), o + e


def test_reference_arm_rank_nonzero_does_no_work():
    """Under torchrun the reference arm runs on rank 0 only; other ranks exit
    without work and without output."""
    port = free_port()
    env = dict(os.environ, MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK="1", WORLD_SIZE="2",
               LOCAL_RANK="1")
    code = ("import sys; sys.path.insert(0, {root!r}); import bench, argparse; "
            "a = argparse.Namespace(impl='reference', workload='spgemm14', scale=0, steps=1, warmup=0); "
            "bench.run_reference(a, 2, 1); print('done')").format(root=ROOT)
    r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == "done", r.stdout + r.stderr


def test_reference_arm_line_matches_our_config():
    """Rank 0 of the reference arm times the oracle on the same workload and
    prints the same metric and config as the GPU arm (tiny scale-10 graph)."""
    code = ("import sys, json, io, contextlib; sys.path.insert(0, {root!r}); import bench, argparse; "
            "a = argparse.Namespace(impl='reference', workload='spgemm14', scale=10, steps=1, warmup=0, "
            "phase_nnz=3 << 30, bcols=0); buf = io.StringIO()\n"
            "with contextlib.redirect_stdout(buf): bench.run_reference(a, 1, 0)\n"
            "line = json.loads(buf.getvalue().strip().splitlines()[-1])\n"
            "assert line['impl'] == 'reference' and line['value'] > 0, line\n"
            "assert line['config'] == bench.workload_config(a, 10, 8, 1), line['config']\n"
            "assert line['metric'] == bench.metric_name('spgemm14', 10, 8)\n"
            "assert line['e2e']['h2d_bytes_per_step'] == 0 and line['cpu_baseline']['value'] == line['value']\n"
            "print('ok')").format(root=ROOT)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.strip().endswith("ok"), r.stdout + r.stderr
