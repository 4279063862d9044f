"""The multi-process (replica) path of bench.py, on the host with gloo at world size 2.

The frame does not shard: every rank renders its own replica of the workload,
and the only cross-rank steps are the barrier around the timed region, the
max over ranks of the step time and the sum of the work done.  These tests
run those steps in real gloo process groups and run the reference arm under
torch.distributed.run with two ranks (rank 0 alone measures and prints).
"""
import json
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _reduce_worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    if ROOT not in sys.path:
        sys.path.insert(0, ROOT)
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    step_s = bench.over_ranks(0.5 + rank)            # rank 1 is the slow one
    frames = bench.over_ranks(100 * (rank + 1), "sum")
    bench.barrier()
    q.put((rank, step_s, frames))
    dist.destroy_process_group()


def _run_ranks(target, world=2):
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=target, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    return sorted(out)


def test_over_ranks_without_group():
    import bench
    assert bench.over_ranks(3.25) == 3.25
    assert bench.over_ranks(7, "sum") == 7
    bench.barrier()  # no process group: a no-op


def test_over_ranks_gloo_world2():
    out = _run_ranks(_reduce_worker)
    assert [r for r, _, _ in out] == [0, 1]
    for _, step_s, frames in out:
        assert step_s == 1.5       # every rank sees the slowest rank's time
        assert frames == 300.0     # and the work of all ranks


def test_reference_arm_torchrun_world2():
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()),
           os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2", "--steps", "1",
           "--warmup", "0", "--workload", "circles", "--cpu-budget", "2"]
    env = dict(os.environ, OMP_NUM_THREADS="1")
    r = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout   # rank 0 alone prints
    line = json.loads(lines[0])
    assert line["impl"] == "reference"
    assert line["n_gpus"] == 2
    assert line["metric"] == line["unit"] == "Msegments/s"
    assert line["value"] > 0 and line["ms_per_step"] > 0
    assert line["cpu_baseline"]["value"] == line["value"]
    assert line["e2e"] == {"value": line["value"], "unit": "Msegments/s",
                           "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert line["config"]["workload"] == "circles"
