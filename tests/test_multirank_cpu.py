"""Multi-rank host logic of the benchmark on CPU (gloo, world size 2): the
max-over-ranks timing reduction, a reference arm that prints from rank 0
only under torchrun, and the whole-trajectory extrapolation of the CPU legs.
The partition of one batch across ranks is covered by
tests/test_multigpu_cpu.py."""
import json
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    got = bench.max_over_ranks(1.0 + 2.5 * rank, world)
    q.put((rank, got))
    dist.destroy_process_group()


def test_max_over_ranks_with_gloo():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    res.sort()
    assert [r[1] for r in res] == [3.5, 3.5]          # both ranks see the slowest


def test_reference_arm_under_torchrun_prints_once():
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()),
           os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2",
           "--instances", "2", "--steps", "1", "--warmup", "3", "--ref-budget", "2"]
    env = dict(os.environ, OMP_NUM_THREADS="1")
    out = subprocess.run(cmd, capture_output=True, text=True, timeout=600, env=env, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["value"] > 0 and line["n_gpus"] == 2
    assert line["cpu_baseline"]["kind"] in ("reference", "port")
    assert line["e2e"]["h2d_bytes_per_step"] == 0


def test_trajectory_extrapolation_on_a_known_cost_law():
    """Per-step cost that grows with the memory window and is stationary
    once it is full: the estimate from a prefix equals the whole sum."""
    sys.path.insert(0, ROOT)
    import bench
    for dk in (25, 180, 290):
        true = [2e-3 * min(t, dk + 1) ** 1.3 for t in range(1, bench.NSTEPS_TRAJ + 1)]
        for tm in (15, 90, 260):
            est = bench.extrapolate_trajectory(true[:tm], dk)
            assert abs(est / sum(true) - 1) < 0.02, (dk, tm, est / sum(true))
