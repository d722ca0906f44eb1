"""GPU parity of the TEMPO engine against the reference fixtures.

Every call goes through the C ABI (liboqupy_gb300.so)."""

import json

import numpy as np
import pytest

from oracle import tempo_oracle as to
from tests import golden_cases as gc

pytestmark = pytest.mark.gpu

TEMPO_CASES = ["config1_spin_boson", "ref_spin_boson_A", "ref_qutrit_C",
               "nondiag_coupling", "add_corr_time", "batched_like_hot",
               "qutrit_superohmic"]


# complex128 Jacobi on GB300's FP64 pipe is slow for D=9 bond splits of
# several hundred columns: the qutrit fixtures are compared on their first
# steps only (bond dimension grows with the step).
STEP_CAP = {"ref_qutrit_C": 6, "qutrit_superohmic": 6}


def _run_backend(g, precision="complex128", nsteps=None):
    from oqupy_gb300 import GpuTempoBackend
    D = g["d"] ** 2
    be = GpuTempoBackend(g["rho0"].reshape(-1), gc.tempo_influence(g),
                         g["unitary"], gc.propagators(g), np.ones(D),
                         np.ones(D), g["dkmax"], g["epsrel"],
                         config={"backend": "gb300", "precision": precision})
    out = [be.initialize()[1]]
    for _ in range(g["nsteps"] if nsteps is None else nsteps):
        out.append(be.compute_step()[1])
    return np.array(out), be


@pytest.mark.parametrize("name", TEMPO_CASES)
def test_gpu_tempo_complex128_matches_reference(name):
    g = gc.load(name)
    n = STEP_CAP.get(name, g["nsteps"])
    states, be = _run_backend(g, nsteps=n)
    errs = [to.trace_distance(a, b) for a, b in zip(states, g["tempo_states"])]
    bad = gc.parity_violations(errs, g["tempo_envelope"][: n + 1])
    assert not bad, bad[:5]
    env = g["tempo_envelope"]
    if not (env > 1e-10).any() and n == g["nsteps"]:
        assert max(errs) < 1e-10
        assert be.bond_dimensions() == list(g["tempo_final_bonds"])


def test_gpu_tempo_batch_mixed_memory_lengths():
    """Instances with different dkmax / D in one launch give the same
    per-instance results as the reference."""
    from oqupy_gb300 import TempoBatch
    names = ["config1_spin_boson", "nondiag_coupling", "add_corr_time",
             "batched_like_hot"]
    gs = [gc.load(n) for n in names]
    insts = []
    for g in gs:
        insts.append(dict(hs_dim=g["d"], dkmax=g["dkmax"], epsrel=g["epsrel"],
                          influences=g["tempo_infl"][: g["dkmax"] + 1],
                          prop1=g["prop1"][0], prop2=g["prop2"][0],
                          rho0=g["rho0"], unitary=g["unitary"]))
    # add_correlation_time needs per-step first-site influences: drop it
    # from the batch comparison window by stopping before dkmax is reached
    nsteps = min(g["nsteps"] for g in gs)
    b = TempoBatch(insts, out_cap=nsteps + 1)
    b.advance(nsteps)
    b.check_status()
    st = b.states(0, nsteps + 1)
    for g, s in zip(gs, st):
        n = nsteps + 1
        if g["add_corr"] is not None:
            n = g["dkmax"] + 1
        errs = [to.trace_distance(a, c) for a, c in zip(s[:n], g["tempo_states"][:n])]
        assert not gc.parity_violations(errs, g["tempo_envelope"][:n]), g["name"]


@pytest.mark.parametrize("name", ["config1_spin_boson", "nondiag_coupling",
                                  "add_corr_time", "batched_like_hot"])
def test_gpu_tempo_mixed_precision_matches_reference(name):
    """The mixed form (double-float Jacobi on the FP32 pipe, FP64 rank
    decisions): trace distance <= 1e-6 against the reference, or within
    ENVELOPE_FACTOR x the reference's own rounding envelope once that
    exceeds 1e-10."""
    g = gc.load(name)
    states, _ = _run_backend(g, "mixed")
    errs = [to.trace_distance(a, b) for a, b in zip(states, g["tempo_states"])]
    print(f"{name}: mixed-precision max trace distance {max(errs):.2e}")
    bad = gc.parity_violations(errs, g["tempo_envelope"], gc.MIXED_ABS)
    assert not bad, bad[:5]


def test_set_all_propagators_equals_per_instance_setter():
    """One batched upload of every instance's propagators (strided copy)
    gives bit-identical states to per-instance uploads, with the
    eigenbasis folding applied, for time-dependent propagators."""
    from oqupy_gb300 import TempoBatch
    names = ["config1_spin_boson", "nondiag_coupling", "batched_like_hot"]
    gs = [gc.load(n) for n in names]
    insts = [dict(hs_dim=g["d"], dkmax=g["dkmax"], epsrel=g["epsrel"],
                  influences=g["tempo_infl"][: g["dkmax"] + 1], prop1=g["prop1"][0],
                  prop2=g["prop2"][0], rho0=g["rho0"], unitary=g["unitary"]) for g in gs]
    nsteps = 8
    a = TempoBatch(insts, out_cap=nsteps + 1)
    b = TempoBatch(insts, out_cap=nsteps + 1)
    rng = np.random.default_rng(4)
    for step in range(nsteps):
        # a different (non-unitary but well-scaled) propagator pair every step
        p1s = [i["prop1"] @ (np.eye(4) + 0.01 * rng.normal(size=(4, 4))) for i in insts]
        p2s = [i["prop2"] @ (np.eye(4) + 0.01 * rng.normal(size=(4, 4))) for i in insts]
        for k, inst in enumerate(insts):
            a.set_propagators(k, p1s[k], p2s[k], inst["unitary"])
        b.set_all_propagators(p1s, p2s, [i["unitary"] for i in insts])
        a.advance(1)
        b.advance(1)
    a.check_status()
    b.check_status()
    np.testing.assert_array_equal(a.states(0, nsteps + 1), b.states(0, nsteps + 1))


def test_autotune_picks_a_timed_candidate_and_caches(tmp_path):
    """The launch-shape autotuner times each candidate on the batch, returns
    the fastest, caches it per (precision, D, dkmax bucket), and the chosen
    shape reproduces the reference within the mixed-form parity bar."""
    from oqupy_gb300 import TempoBatch, autotune
    g = gc.load("config1_spin_boson")
    insts = [dict(hs_dim=g["d"], dkmax=g["dkmax"], epsrel=g["epsrel"],
                  influences=g["tempo_infl"][: g["dkmax"] + 1], prop1=g["prop1"][0],
                  prop2=g["prop2"][0], rho0=g["rho0"], unitary=g["unitary"])] * 8
    cache = str(tmp_path / "tune.json")
    cands = [(256, 2, 88), (128, 4, 36)]
    res = autotune.tune(insts, precision="mixed", steps=4, candidates=cands, cache=cache)
    assert [tuple(c) for c, _ in res["timings"]] == cands
    assert (res["block"], res["ctas_per_sm"], res["smem_kb"]) in cands
    again = autotune.tune(insts, precision="mixed", steps=4, candidates=cands, cache=cache)
    assert again == json.loads(json.dumps(res))          # served from the cache
    a = TempoBatch(insts, precision="mixed", out_cap=11, block=res["block"], smem_kb=res["smem_kb"])
    a.advance(10)
    a.check_status()
    for st in a.states(0, 11):
        errs = [to.trace_distance(x, y) for x, y in zip(st, g["tempo_states"][:11])]
        assert not gc.parity_violations(errs, g["tempo_envelope"][:11], gc.MIXED_ABS)
