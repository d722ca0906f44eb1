"""Multi-GPU host logic on CPU (gloo, world size 2): one batch partitioned
across ranks by predicted cost, the states gathered to rank 0 equal a
single-rank solve; the process-tensor sweep split by system, gathered the
same way.  The per-rank solver here is the CPU oracle (the partition and the
gather do not depend on which engine solves a part)."""
import os
import socket
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
NSTEPS = 6


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _insts():
    sys.path.insert(0, ROOT)
    import bench
    return bench.make_instances(6, 4242)


def _solve(insts):
    from oracle import tempo_oracle as to
    out = []
    for x in insts:
        infl = x["influences"]
        st, _ = to.tempo_dynamics(np.asarray(x["rho0"]).reshape(-1),
                                  lambda dk: infl[dk] if 0 <= dk < len(infl) else None,
                                  x["unitary"], lambda s: (x["prop1"], x["prop2"]),
                                  x["dkmax"], x["epsrel"], NSTEPS)
        out.append(st)
    return np.array(out)


def _pt_and_systems():
    from oracle import tempo_oracle as to
    from tests import golden_cases as gc
    g = gc.load("nondiag_coupling")
    mpos, caps, _ = to.pt_tempo_build(g["d"], gc.pt_influence(g), g["nsteps"], g["dkmax"], g["epsrel"])
    rng = np.random.default_rng(7)
    from oqupy_gb300 import bath
    sx = np.array([[0, 1], [1, 0]], dtype=complex)
    sz = np.diag([1.0, -1.0]).astype(complex)
    props = [bath.half_step_propagators(a * sx + b * sz, g["dt"]) for a, b in rng.uniform(-2, 2, (5, 2))]
    return mpos, caps, props


def _sweep(mpos, caps, props):
    from oracle import tempo_oracle as to
    rho0 = np.array([1, 0, 0, 0], dtype=complex)
    return np.array([to.compute_dynamics_pt(rho0, lambda s, p=p: p, mpos, caps) for p in props])


def _worker(rank, world, port, q):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from oqupy_gb300 import multigpu as mg
    insts = _insts()
    costs = mg.predicted_costs([x["dkmax"] for x in insts], [4, 9, 2, 7, 5, 3])
    states, parts = mg.run_partitioned(insts, costs, _solve, rank, world)
    mpos, caps, props = _pt_and_systems()
    chunks = mg.split_range(len(props), world)
    local = _sweep(mpos, caps, [props[i] for i in chunks[rank]])
    swept = mg.gather_rows(local, [list(c) for c in chunks], len(props), rank, world)
    q.put((rank, states, parts, swept))
    dist.destroy_process_group()


def test_lpt_partition_balances_and_is_deterministic():
    from oqupy_gb300 import multigpu as mg
    rng = np.random.default_rng(0)
    costs = rng.pareto(1.5, size=512) + 1.0
    for world in (2, 4, 8):
        parts = mg.lpt_partition(costs, world)
        assert sorted(i for p in parts for i in p) == list(range(512))
        loads = np.array([costs[p].sum() for p in parts])
        # LPT bound: makespan <= mean load + the largest single cost
        assert loads.max() <= loads.mean() + costs.max() + 1e-9
        assert parts == mg.lpt_partition(costs, world)
    assert [list(r) for r in mg.split_range(5, 2)] == [[0, 1, 2], [3, 4]]


def test_partitioned_batch_and_split_sweep_equal_single_rank_with_gloo():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted([q.get(timeout=600) for _ in procs], key=lambda r: r[0])
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (_, states, parts, swept), (_, none1, parts1, none2) = res
    assert none1 is None and none2 is None and parts == parts1
    assert all(len(p) > 0 for p in parts)
    np.testing.assert_array_equal(states, _solve(_insts()))
    mpos, caps, props = _pt_and_systems()
    np.testing.assert_array_equal(swept, _sweep(mpos, caps, props))
