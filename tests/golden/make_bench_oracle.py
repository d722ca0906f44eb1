"""Whole-trajectory oracle states for a stratified subsample of the benchmark
batch (used by ``bench.py`` to state the mixed form's error against the FP64
oracle per instance).

Run from the repository root (CPU only; hours on 8 cores -- the
longest-memory instances take tens of minutes per 500-step run):

    python tests/golden/make_bench_oracle.py

The batch is ``bench.make_instances(512, bench.BATCH_SEED)``; the subsample
is ``bench.stratified_sample`` (one instance per 32-instance stratum of the
batch sorted by dkmax, 16 instances).  For each: the oracle's states over
all 500 steps, and its spread under influence perturbations of 1e-15 and
1e-14 relative (one seed each), the rounding envelope the error is read
against.
"""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def _run(args):
    idx, rel, seed = args
    import bench
    from oracle import tempo_oracle as to
    inst = bench.make_instances(512, bench.BATCH_SEED)[idx]
    infl = np.asarray(inst["influences"])
    if rel > 0:
        rng = np.random.default_rng(seed)
        infl = infl * (1.0 + rel * rng.normal(size=infl.shape))
    st, _ = to.tempo_dynamics(np.asarray(inst["rho0"]).reshape(-1),
                              lambda dk: infl[dk] if 0 <= dk < len(infl) else None,
                              inst["unitary"], lambda s: (inst["prop1"], inst["prop2"]),
                              inst["dkmax"], inst["epsrel"], bench.NSTEPS_TRAJ)
    return idx, rel, st


def main():
    import multiprocessing as mp
    import bench
    from oracle import tempo_oracle as to
    insts = bench.make_instances(512, bench.BATCH_SEED)
    idx = bench.stratified_sample(insts)
    jobs = [(i, rel, 1000 + k) for k, i in enumerate(idx) for rel in (0.0, 1e-15, 1e-14)]
    # the longest memories first, so the pool's tail is short
    jobs.sort(key=lambda j: -insts[j[0]]["dkmax"])
    os.environ["OPENBLAS_NUM_THREADS"] = "1"
    with mp.get_context("spawn").Pool(os.cpu_count() or 1) as pool:
        res = pool.map(_run, jobs, chunksize=1)
    got = {(i, rel): st for i, rel, st in res}
    states = np.array([got[(i, 0.0)] for i in idx])
    env = np.array([[max(to.trace_distance(a, b), to.trace_distance(a, c))
                     for a, b, c in zip(got[(i, 0.0)], got[(i, 1e-15)], got[(i, 1e-14)])]
                    for i in idx])
    path = os.path.join(HERE, "bench_oracle.npz")
    np.savez_compressed(path, index=np.array(idx), dkmax=np.array([insts[i]["dkmax"] for i in idx]),
                        seed=bench.BATCH_SEED, states=states, envelope=env)
    print(path, states.shape)


if __name__ == "__main__":
    main()
