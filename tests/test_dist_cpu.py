"""The multi-process (replica) path of bench.py on CPU: two ranks over gloo.

Every workload shards into independent replicas with no exchange on the data path; what
the N > 1 launch adds is the host-side plumbing: process-group setup from the torchrun
environment, the barrier around the timed region, the max over ranks of the elapsed time,
and rank 0 alone printing (and alone running the reference arm). This checks that
plumbing with world_size 2 on the gloo backend (no GPU).
"""
import json
import os
import socket
import subprocess
import sys
import textwrap

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def torchrun(args, timeout=240):
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr=127.0.0.1", "--master-port=%d" % free_port()] + args
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="", OMP_NUM_THREADS="1")
    return subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=timeout)


def test_barrier_and_max_over_ranks(tmp_path):
    pytest.importorskip("torch")
    script = tmp_path / "worker.py"
    script.write_text(textwrap.dedent("""
        import os, sys
        sys.path.insert(0, %r)
        import bench
        dist, rank, world = bench.dist_init(2)
        assert world == 2 and dist is not None
        bench.barrier(dist)
        m = bench.allmax(dist, float(rank + 1))
        print("rank %%d max %%.1f" %% (rank, m))
        dist.destroy_process_group()
    """ % ROOT))
    r = torchrun([str(script)])
    assert r.returncode == 0, r.stderr[-2000:]
    assert "rank 0 max 2.0" in r.stdout and "rank 1 max 2.0" in r.stdout


def test_reference_arm_rank0_only():
    pytest.importorskip("torch")
    r = torchrun(["bench.py", "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "1",
                  "--cpu-elems", "16"])
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["value"] > 0 and d["cpu_baseline"]["kind"] == "port"
    assert d["e2e"]["h2d_bytes_per_step"] == 0
