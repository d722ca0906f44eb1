"""Loader for the golden fixtures written by ``tests/golden/make_golden.py``."""

import glob
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")


def names():
    return sorted(os.path.splitext(os.path.basename(p))[0]
                  for p in glob.glob(os.path.join(GOLDEN, "*.npz")))


def load(name):
    with np.load(os.path.join(GOLDEN, name + ".npz")) as z:
        g = {k: z[k] for k in z.files}
    g["name"] = name
    g["dkmax"] = int(g["dkmax"])
    g["dkmax"] = None if g["dkmax"] < 0 else g["dkmax"]
    g["add_corr"] = float(g["add_corr"])
    g["add_corr"] = None if g["add_corr"] < 0 else g["add_corr"]
    g["nsteps"] = int(g["nsteps"])
    g["epsrel"] = float(g["epsrel"])
    g["dt"] = float(g["dt"])
    g["d"] = g["rho0"].shape[0]
    return g


def tempo_influence(g):
    """``influence(dk)`` callable replaying the recorded TEMPO influences."""
    infl = g["tempo_infl"]
    neg = g.get("tempo_infl_neg")

    def f(dk):
        if dk >= 0:
            return infl[dk]
        if neg is None:
            return None
        return neg[-dk - 1]
    return f


def pt_influence(g):
    infl = g["pt_infl"]
    neg = g.get("pt_infl_neg")

    def f(dk):
        if dk >= 0:
            return infl[dk]
        if neg is None:
            return None
        return neg[-dk - 2]
    return f


def propagators(g, which=0):
    p1, p2 = g["prop1"][which], g["prop2"][which]
    return lambda step: (p1, p2)


PARITY_ABS = 1e-10     # trace distance on rounding-insensitive steps
ENVELOPE_FACTOR = 10.0  # allowance over the reference's own rounding spread


MIXED_ABS = 1e-6       # the mixed-precision form's trace-distance bar


def parity_violations(errors, envelope, abs_tol=PARITY_ABS):
    """Steps where ``errors`` (per-step trace distance to the reference)
    exceeds ``max(PARITY_ABS, ENVELOPE_FACTOR * envelope)``.

    ``envelope`` is the per-step spread of the unmodified reference under
    1e-15 relative input perturbations (recorded in the fixtures): where the
    reference's own result moves by more than 1e-10 for rounding-level
    changes (an epsrel cut falling inside a cluster of degenerate singular
    values), no other FP64 implementation can be held to 1e-10."""
    errors = np.asarray(errors)
    env = np.asarray(envelope)
    # A rounding-level tie persists once it has happened, and two perturbed
    # runs sample its amplitude only roughly, so every step from the first
    # sensitive one on is held to the run's largest spread.
    tol = np.full(env.shape, abs_tol)
    sensitive = env > PARITY_ABS
    if sensitive.any():
        first = int(np.argmax(sensitive))
        tol[first:] = max(abs_tol, ENVELOPE_FACTOR * float(env.max()))
    return [(i, float(e), float(t)) for i, (e, t) in
            enumerate(zip(errors, tol)) if e > t]
