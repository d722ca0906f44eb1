"""Generate the oracle fixtures for seeded draws from the batched TEMPO
configurations (used by ``tests/test_batched_parity_gpu.py``).

Run from the repository root (CPU only, a few minutes on 8 cores):

    python tests/golden/make_draws.py

Draws: ``bench.make_instances(16, 777)`` (spin-boson: alpha ~ U[0.01, 0.5],
wc ~ U[1, 10], T ~ U[0, 5], Omega ~ U[0.5, 2], dkmax ~ U{20..300}, dt 0.05,
epsrel 1e-6) and ``bench.make_qutrit_instances(16, 778)`` (d = 3,
super-ohmic, dkmax 100, epsrel 1e-7).  For every draw the fixture stores

* the exact inputs the engine consumes (influences for the dk the first
  NSTEPS steps use, propagators, coupling eigenbasis, initial state), so the
  GPU runs on bit-identical inputs on any host;
* the oracle's states and its MPS bond profile after every step;
* the oracle's cut fragility per step: over all bond splits of the step, the
  smallest relative distance of a tail norm at the cut from the threshold
  (``min |sqrt(sum_{j>=i} s_j^2) - epsrel s_0| / (epsrel s_0)`` for i at the
  cut, the rank decision's margin) and the smallest relative singular-value
  gap at the cut (``(s_{chi-1} - s_chi) / s_{chi-1}``);
* rounding envelopes: the per-step trace distance between the oracle and
  itself rerun with its influence matrices perturbed by 1e-15 relative
  (8 seeds), by 1e-14 relative (4 seeds; the backward error of a
  backward-stable SVD of the n-column matrices here is O(n eps) ~ 1e-14
  relative), with LAPACK's gesvd driver in place of gesdd, and by 1e-9
  relative (2 seeds; the scale of the mixed form's QR cut).
"""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

NSTEPS = {"spin_boson": 80, "qutrit": 30}
SEEDS = {"spin_boson": 777, "qutrit": 778}


def draws(kind):
    import bench
    if kind == "spin_boson":
        return bench.make_instances(16, SEEDS[kind])
    return bench.make_qutrit_instances(16, SEEDS[kind])


def _perturbed(infl, seed, rel):
    rng = np.random.default_rng(seed)
    return [m * (1.0 + rel * rng.normal(size=m.shape)) for m in infl]


def _run(inst, infl, nsteps, svd_driver=None, record=False):
    """Oracle run; returns (states, per-step bond profiles, margins, gaps)."""
    import scipy.linalg
    from oracle import tempo_oracle as to
    plain = to.truncated_svd
    steps_margin, steps_gap = [], []
    cur = {"m": np.inf, "g": np.inf}

    def recorder(mat, epsrel):
        if svd_driver is None:
            u, s, vh = np.linalg.svd(mat, full_matrices=False)
        else:
            u, s, vh = scipy.linalg.svd(mat, full_matrices=False, lapack_driver=svd_driver)
        k = to.truncation_rank(s, epsrel)
        if record and s.size and s[0] > 0:
            thr = epsrel * s[0]
            tail = np.sqrt(np.cumsum(np.square(s[::-1])))[::-1]   # tail[i] = |s[i:]|
            cand = [tail[k - 1]] + ([tail[k]] if k < s.size else [])
            cur["m"] = min(cur["m"], min(abs(t - thr) / thr for t in cand))
            if k < s.size:
                cur["g"] = min(cur["g"], (s[k - 1] - s[k]) / s[k - 1])
        return u[:, :k], s[:k], vh[:k, :], s[k:]

    to.truncated_svd = recorder
    try:
        o = to.TempoOracle(np.asarray(inst["rho0"]).reshape(-1),
                           lambda dk: infl[dk] if 0 <= dk < len(infl) else None,
                           inst["unitary"], lambda s: (inst["prop1"], inst["prop2"]),
                           np.ones(inst["hs_dim"] ** 2), np.ones(inst["hs_dim"] ** 2),
                           inst["dkmax"], inst["epsrel"])
        states = [o.initialize()[1]]
        bonds = []
        for _ in range(nsteps):
            cur["m"], cur["g"] = np.inf, np.inf
            states.append(o.compute_step()[1])
            bonds.append(list(o.bond_dimensions()))
            steps_margin.append(cur["m"])
            steps_gap.append(cur["g"])
    finally:
        to.truncated_svd = plain
    return np.array(states), bonds, np.array(steps_margin), np.array(steps_gap)


def one_draw(args):
    """All oracle runs of one draw (runs in a worker process)."""
    kind, idx = args
    from oracle import tempo_oracle as to
    inst = draws(kind)[idx]
    n = NSTEPS[kind]
    infl = list(np.asarray(inst["influences"]))
    ref, bonds, margin, gap = _run(inst, infl, n, record=True)

    def env_of(runs):
        return np.max([[to.trace_distance(a, b) for a, b in zip(v, ref)] for v in runs], axis=0)

    e15 = env_of([_run(inst, _perturbed(infl, 100 + s, 1e-15), n)[0] for s in range(8)]
                 + [_run(inst, infl, n, svd_driver="gesvd")[0]])
    e14 = env_of([_run(inst, _perturbed(infl, 200 + s, 1e-14), n)[0] for s in range(4)])
    e9 = env_of([_run(inst, _perturbed(infl, 300 + s, 1e-9), n)[0] for s in range(2)])
    return idx, ref, bonds, margin, gap, e15, e14, e9


def _pad(infl, n):
    """Influences dk = 0..n-1: the draw's own, then NaN (dk > dkmax is never
    read; NaN makes a read of it visible)."""
    out = np.full((n,) + infl.shape[1:], np.nan, dtype=np.complex128)
    out[: len(infl)] = infl
    return out


def make(kind, procs):
    import multiprocessing as mp
    insts = draws(kind)
    n = NSTEPS[kind]
    os.environ["OPENBLAS_NUM_THREADS"] = "1"
    with mp.get_context("spawn").Pool(procs) as pool:
        res = sorted(pool.map(one_draw, [(kind, i) for i in range(len(insts))]), key=lambda r: r[0])
    D = insts[0]["hs_dim"] ** 2
    nin = n + 1                                   # influences dk = 0..n used in n steps
    L = max(len(b) for r in res for b in r[2])
    bonds = np.zeros((len(insts), n, L), dtype=np.int32)
    for i, r in enumerate(res):
        for s, b in enumerate(r[2]):
            bonds[i, s, :len(b)] = b
    out = dict(
        kind=kind, seed=SEEDS[kind], nsteps=n, hs_dim=insts[0]["hs_dim"],
        epsrel=np.array([x["epsrel"] for x in insts]),
        dkmax=np.array([x["dkmax"] for x in insts]),
        influences=np.array([_pad(np.asarray(x["influences"])[:nin], nin) for x in insts]),
        prop1=np.array([x["prop1"] for x in insts]), prop2=np.array([x["prop2"] for x in insts]),
        unitary=np.array([x["unitary"] for x in insts]),
        rho0=np.array([np.asarray(x["rho0"]) for x in insts]),
        states=np.array([r[1] for r in res]), bonds=bonds,
        margin=np.array([r[3] for r in res]), gap=np.array([r[4] for r in res]),
        env15=np.array([r[5] for r in res]), env14=np.array([r[6] for r in res]),
        env9=np.array([r[7] for r in res]))
    path = os.path.join(HERE, f"draws_{kind}.npz")
    np.savez_compressed(path, **out)
    print(path, {k: np.asarray(v).shape for k, v in out.items()})


if __name__ == "__main__":
    kinds = sys.argv[1:] or ["spin_boson", "qutrit"]
    for k in kinds:
        make(k, os.cpu_count() or 1)
