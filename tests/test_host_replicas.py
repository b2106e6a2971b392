"""The bench's launch handling on CPU: one GPU only.

The smartpca path runs one PCA per panel on one GPU and its split Gram multicasts TMA loads
within that GPU's memory, so `bench.py` has no multi-GPU mode: `--gpus N > 1`, or a torchrun
launch with WORLD_SIZE > 1, prints one JSON line with an "unavailable" reason on rank 0 and
exits 0 on every rank without touching a GPU.  The reference arm (CPU) runs on rank 0 only.
"""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench(args, rank=None, world=None):
    env = dict(os.environ)
    if world is not None:
        env.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(world),
                   MASTER_ADDR="127.0.0.1", MASTER_PORT="29533")
    # no GPU is visible to these runs: a refusal must come before any CUDA call
    env["CUDA_VISIBLE_DEVICES"] = ""
    return subprocess.run([sys.executable, os.path.join(ROOT, "bench.py")] + args, env=env,
                          cwd=ROOT, capture_output=True, text=True, timeout=120)


def test_gpu_arm_refuses_more_than_one_gpu():
    r = _bench(["--gpus", "2", "--steps", "1", "--warmup", "0"])
    assert r.returncode == 0, r.stderr
    lines = [ln for ln in r.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["n_gpus"] == 2 and "one GPU only" in d["unavailable"]


def test_gpu_arm_under_torchrun_world_two():
    """rank 0 prints the refusal, rank 1 prints nothing; neither initialises a process group"""
    r0 = _bench(["--steps", "1", "--warmup", "0"], rank=0, world=2)
    r1 = _bench(["--steps", "1", "--warmup", "0"], rank=1, world=2)
    assert r0.returncode == 0 and r1.returncode == 0, (r0.stderr, r1.stderr)
    assert "unavailable" in json.loads(r0.stdout.strip())
    assert r1.stdout.strip() == ""


def test_reference_arm_non_zero_rank_exits_without_work():
    """under torchrun only rank 0 of the reference arm runs and prints"""
    r = _bench(["--impl", "reference"], rank=1, world=2)
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
    # the tiled kernel's lower triangle mostly stays in L2: DRAM traffic below the algorithmic
    # bytes (the committed ncu summary's figure, 130 GB against 333 GB)
    assert roof["traffic"] == bench.tridiag_traffic(5000) and 0 < roof["traffic"] < alg
    assert bench.tridiag_traffic(4000) is None
    assert bench.tridiag_roofline({"tridiag_n": 5000, "tridiag_ms": 0.0}, {}, "x") is None
