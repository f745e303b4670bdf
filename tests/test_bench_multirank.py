"""bench.py's multi-rank path on the CPU (gloo, world size 2): the timing
reductions the GPU arm uses (barrier, max and sum over ranks; replicas only, no
data-path collective) and the reference arm launched through torchrun, where
rank 0 alone runs and prints the JSON line and the other rank exits 0."""
import json
import multiprocessing as mp
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


def _rank_main(rank, ws, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(ws), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    w, r, local = bench.dist_env()
    bench.barrier(w)
    mx = bench.max_over_ranks(1.5 + r, w)
    sm = bench.sum_over_ranks(10 * (r + 1), w)
    bench.barrier(w)
    q.put((r, w, local, mx, sm))


def test_timing_reductions_over_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert out == [(0, 2, 0, 2.5, 30.0), (1, 2, 1, 2.5, 30.0)]


def _select_main(rank, preset, q):
    os.environ.pop("CUDA_VISIBLE_DEVICES", None)
    if preset is not None:
        os.environ["CUDA_VISIBLE_DEVICES"] = preset
    sys.path.insert(0, ROOT)
    import bench
    dev = bench.select_device(2, rank)
    q.put((rank, dev, os.environ["CUDA_VISIBLE_DEVICES"]))


@pytest.mark.parametrize("preset,expect", [(None, ["0", "1"]), ("4,5,6,7", ["4", "5"]),
                                           ("GPU-a, GPU-b", ["GPU-a", "GPU-b"])])
def test_each_rank_narrows_the_visible_devices_to_its_own(preset, expect):
    """Two ranks: each ends with exactly one visible GPU, its local rank's
    entry of a list the launcher already exported (or its local rank)."""
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    ps = [ctx.Process(target=_select_main, args=(r, preset, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert out == [(0, expect[0], expect[0]), (1, expect[1], expect[1])]


def test_single_rank_reductions_are_identities():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.25, 1) == 3.25
    assert bench.sum_over_ranks(7, 1) == 7


@pytest.mark.timeout(300)
def test_reference_arm_under_torchrun_prints_once():
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py", "--impl",
           "reference", "--gpus", "2", "--steps", "1", "--warmup", "0", "--cpu-seconds", "0.5"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=280)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port"
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
