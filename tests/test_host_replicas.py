"""The bench's multi-process path on CPU: world_size 2 over gloo (127.0.0.1).

The smartpca path does not shard (one PCA per panel): `bench.py --gpus N` runs N independent
replicas and only needs a barrier and the max over ranks of the step time.  This checks those
host pieces with two gloo ranks, and that the reference arm's non-zero ranks exit without
work.
"""
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

WORKER = r"""
import os, sys
sys.path.insert(0, os.environ["REPO_ROOT"])
import bench
world, rank, local, dist = bench.dist_setup()
assert world == 2 and dist is not None
bench.barrier(dist)
t = bench.max_over_ranks(dist, 10.0 + rank)          # rank 1 is slower
assert t == 11.0, t
value = world * 100.0 / t                            # the bench's whole-job formula
print("rank", rank, "max", t, "value", value)
dist.destroy_process_group()
"""


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _run_two(code, extra_env=None, timeout=240):
    port = _free_port()
    procs = []
    for rank in range(2):
        env = dict(os.environ, REPO_ROOT=ROOT, RANK=str(rank), LOCAL_RANK=str(rank),
                   WORLD_SIZE="2", MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
        env.update(extra_env or {})
        procs.append(subprocess.Popen([sys.executable, "-c", code], env=env, cwd=ROOT,
                                      stdout=subprocess.PIPE, stderr=subprocess.STDOUT,
                                      text=True))
    outs = []
    for p in procs:
        try:
            out, _ = p.communicate(timeout=timeout)
        except subprocess.TimeoutExpired:
            p.kill()
            out, _ = p.communicate()
        outs.append((p.returncode, out))
    return outs


def test_replicas_barrier_and_max_over_ranks_gloo():
    pytest.importorskip("torch.distributed")
    outs = _run_two(WORKER)
    for rc, out in outs:
        assert rc == 0, out
        assert "max 11.0" in out and "value" in out


def test_reference_arm_non_zero_rank_exits_without_work():
    """under torchrun only rank 0 of the reference arm runs and prints"""
    env = dict(os.environ, RANK="1", LOCAL_RANK="1", WORLD_SIZE="2", MASTER_ADDR="127.0.0.1",
               MASTER_PORT=str(_free_port()))
    code = ("import sys; sys.path.insert(0, %r); sys.argv = ['bench.py', '--impl', 'reference']; "
            "import bench; bench.dist_setup = lambda: (2, 1, 1, None); bench.main()" % ROOT)
    r = subprocess.run([sys.executable, "-c", code], env=env, cwd=ROOT, capture_output=True,
                       text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""


def test_tridiag_roofline_figures():
    """the dominant-kernel roofline: dsytd2's algorithmic bytes 8 (n-1) n (n+1) / 3, achieved
    GB/s from the CUDA-event time, and the DRAM bytes of the committed ncu summary for the
    order it was captured at (none for other orders)"""
    sys.path.insert(0, ROOT)
    import bench

    res = {"tridiag_n": 5000, "tridiag_ms": 150.0}
    roof = bench.tridiag_roofline(res, {"hbm_gbs": 6000.0}, "measured")
    alg = 8.0 * 4999 * 5000 * 5001 / 3.0
    assert roof["bound"] == "hbm" and roof["unit"] == "GB/s"
    assert abs(roof["algorithmic_bytes"] - alg) < 1.0
    assert abs(roof["achieved"] - alg / 0.150 / 1e9) < 1e-6
    assert abs(roof["frac"] - roof["achieved"] / 6000.0) < 1e-12
    assert roof["traffic"] == bench.tridiag_traffic(5000) and roof["traffic"] > alg
    assert bench.tridiag_traffic(4000) is None
    assert bench.tridiag_roofline({"tridiag_n": 5000, "tridiag_ms": 0.0}, {}, "x") is None
