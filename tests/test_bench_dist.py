"""bench.py's multi-process contract on the CPU: two ranks launched by
torch.distributed.run (gloo), the reference arm runs on rank 0 only and prints
exactly one JSON line; the other rank exits 0 without work.  The timing
reduction of bench.py's own arm (maximum over ranks) runs with two gloo ranks."""
import json
import os
import socket
import subprocess
import sys

from conftest import ROOT


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def test_reference_arm_two_ranks_gloo():
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()),
           os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2", "--steps", "1",
           "--warmup", "0", "--side", "6"]
    env = {**os.environ, "OMP_NUM_THREADS": "1"}
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300, env=env, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    out = json.loads(lines[0])
    assert out["impl"] == "reference" and out["n_gpus"] == 2 and out["value"] > 0
    assert out["cpu_baseline"]["kind"] == "port"
    assert out["e2e"]["h2d_bytes_per_step"] == 0


def _rank_max(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=world)
    try:
        # rank r reports times that are largest on different ranks per slot
        vals = [float(rank + 1), float(10 - rank), 3.0]
        dist.barrier()
        got = bench.max_over_ranks(vals, world, "cpu")
        with open(os.path.join(out, f"r{rank}.json"), "w") as f:
            json.dump(got, f)
    finally:
        dist.destroy_process_group()


def test_ours_arm_rank_reduction_gloo(tmp_path):
    """The timing reduction of bench.py's own arm (max over ranks, all_reduce)
    with two ranks: every rank holds the maximum of each slot."""
    import torch.multiprocessing as mp
    mp.spawn(_rank_max, args=(2, _free_port(), str(tmp_path)), nprocs=2, join=True)
    for r in range(2):
        with open(os.path.join(tmp_path, f"r{r}.json")) as f:
            assert json.load(f) == [2.0, 10.0, 3.0]
