"""Pin the CPU oracle against fixtures produced by the unmodified reference."""

import os

import numpy as np
import pytest

from oracle import tempo_oracle as to
from oracle import bath_oracle as bo
from tests import golden_cases as gc

TEMPO_CASES = [n for n in gc.names() if "tempo_states" in np.load(
    gc.GOLDEN + "/" + n + ".npz").files]
PT_CASES = [n for n in gc.names() if "pt_states" in np.load(
    gc.GOLDEN + "/" + n + ".npz").files]


@pytest.mark.parametrize("name", TEMPO_CASES)
def test_oracle_tempo_matches_reference(name):
    g = gc.load(name)
    if name == "qutrit_superohmic" and not os.environ.get("OQUPY_GB300_SLOW"):
        pytest.skip("slow (D=9 dense oracle); set OQUPY_GB300_SLOW=1")
    states, o = to.tempo_dynamics(g["rho0"], gc.tempo_influence(g),
                                  g["unitary"], gc.propagators(g), g["dkmax"],
                                  g["epsrel"], g["nsteps"])
    ref = g["tempo_states"]
    assert states.shape == ref.shape
    errs = [to.trace_distance(a, b) for a, b in zip(states, ref)]
    assert not gc.parity_violations(errs, g["tempo_envelope"])
    # before the first rounding-sensitive step the match is at 1e-10
    env = g["tempo_envelope"]
    clean = len(env) if not (env > 1e-10).any() else int(np.argmax(env > 1e-10))
    assert max(errs[:clean]) < 1e-10
    if clean == len(env):
        assert np.array_equal(np.array(o.bond_history), g["tempo_max_bond"])


@pytest.mark.parametrize("name", PT_CASES)
def test_oracle_pt_matches_reference(name):
    g = gc.load(name)
    d = g["d"]
    dkmax = g["dkmax"] if g["dkmax"] is not None else g["nsteps"]
    mpos, caps, o = to.pt_tempo_build(d, gc.pt_influence(g), g["nsteps"],
                                      dkmax, g["epsrel"])
    bonds = [T.shape[0] for T in mpos] + [mpos[-1].shape[1]]
    assert bonds == list(g["pt_bonds"])
    tin = g.get("pt_transform_in")
    tout = g.get("pt_transform_out")
    for i in range(g["pt_states"].shape[0]):
        states = to.compute_dynamics_pt(
            g["rho0"], gc.propagators(g, i), mpos, caps,
            transform_in=tin, transform_out=tout)
        errs = [to.trace_distance(a, b)
                for a, b in zip(states, g["pt_states"][i])]
        assert not gc.parity_violations(errs, g["pt_envelope"][i]), i


def test_oracle_reproduces_reference_physics_goldens():
    """The reference's own stored results (decimal=4):
    tests/physics/tempo_spin_boson_test.py:45-46 and
    tests/physics/tempo_qutrit_test.py:59-62."""
    rho_A = np.array([[0.7809559 + 0.j, -0.09456333 + 0.16671419j],
                      [-0.09456333 - 0.16671419j, 0.2190441 + 0.j]])
    g = gc.load("ref_spin_boson_A")
    states, _ = to.tempo_dynamics(g["rho0"], gc.tempo_influence(g),
                                  g["unitary"], gc.propagators(g), g["dkmax"],
                                  g["epsrel"], g["nsteps"])
    np.testing.assert_almost_equal(states[-1].reshape(2, 2), rho_A, decimal=4)
    rho_C = np.array(
        [[0.12576653 + 0.j, -0.11739956 - 0.14312036j, 0.12211454 - 0.05963583j],
         [-0.11739956 + 0.14312036j, 0.61315893 + 0.j, -0.06636825 + 0.26917271j],
         [0.12211454 + 0.05963583j, -0.06636825 - 0.26917271j, 0.26107455 + 0.j]])
    g = gc.load("ref_qutrit_C")
    states, _ = to.tempo_dynamics(g["rho0"], gc.tempo_influence(g),
                                  g["unitary"], gc.propagators(g), g["dkmax"],
                                  g["epsrel"], g["nsteps"])
    np.testing.assert_almost_equal(states[-1].reshape(3, 3), rho_C, decimal=4)


@pytest.mark.parametrize("name", ["config1_spin_boson", "add_corr_time",
                                  "nondiag_coupling"])
def test_bath_oracle_influences_match_reference(name):
    g = gc.load(name)
    bath = bo.PowerLawBath(float(g["alpha"]), float(g["zeta"]),
                           float(g["wc"]), str(g["cutoff_type"]),
                           float(g["T"]))
    comm, acomm, _ = bo.coupling_diagonals(g["coupling"])
    for dk in range(g["tempo_infl"].shape[0]):
        got = bo.influence_matrix(dk, g["dt"], g["dkmax"], bath, comm, acomm,
                                  g["add_corr"], g["epsrel"])
        np.testing.assert_allclose(got, g["tempo_infl"][dk], rtol=0,
                                   atol=1e-13)


def test_oracle_reproduces_the_batched_draw_fixtures():
    """The draws fixtures (tests/golden/make_draws.py) are the oracle's own
    states on their stored inputs: two spin-boson and one qutrit draw,
    rerun for their first steps, agree to rounding."""
    import os
    d = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    for kind, idx, steps in (("spin_boson", [0, 7], 25), ("qutrit", [3], 6)):
        g = np.load(os.path.join(d, f"draws_{kind}.npz"))
        for i in idx:
            infl = g["influences"][i]
            nan = np.full_like(infl[0], np.nan)     # dk past the stored window: never used

            def influence(dk, infl=infl, nan=nan):
                return None if dk < 0 else (infl[dk] if dk < len(infl) else nan)
            st, _ = to.tempo_dynamics(g["rho0"][i].reshape(-1), influence,
                                      g["unitary"][i], lambda s: (g["prop1"][i], g["prop2"][i]),
                                      int(g["dkmax"][i]), float(g["epsrel"][i]), steps)
            err = max(to.trace_distance(a, b) for a, b in zip(st, g["states"][i][: steps + 1]))
            assert err <= 1e-12 + 10 * g["env14"][i][: steps + 1].max(), (kind, i, err)
