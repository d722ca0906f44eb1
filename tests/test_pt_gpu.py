"""GPU parity of PT-TEMPO builds and the process-tensor sweep against the
reference fixtures (every call through the C ABI)."""

import numpy as np
import pytest

from oracle import tempo_oracle as to
from tests import golden_cases as gc

pytestmark = pytest.mark.gpu

# D=4 fixtures; the big-bond and qutrit builds have their own tests below.
PT_CASES = ["ref_spin_boson_A", "nondiag_coupling", "add_corr_time"]


def _inst(g):
    dkmax = g["dkmax"] if g["dkmax"] is not None else g["nsteps"]
    inst = dict(hs_dim=g["d"], num_steps=g["nsteps"], dkmax=dkmax,
                epsrel=g["epsrel"], influences=g["pt_infl"])
    if "pt_infl_neg" in g:
        D = g["d"] ** 2
        neg = np.zeros((g["nsteps"] + 1, D, D), dtype=complex)
        neg[2:2 + len(g["pt_infl_neg"])] = g["pt_infl_neg"][: g["nsteps"] - 1]
        inst["neg_influences"] = neg
    return inst


def _check(batch, idx, g, abs_tol):
    states = batch.dynamics(idx, g["prop1"], g["prop2"],
                            np.repeat(g["rho0"].reshape(1, -1), len(g["prop1"]), 0),
                            transform_in=g.get("pt_transform_in"),
                            transform_out=g.get("pt_transform_out"))
    for h in range(states.shape[1]):
        errs = [to.trace_distance(a, b) for a, b in zip(states[:, h], g["pt_states"][h])]
        bad = gc.parity_violations(errs, g["pt_envelope"][h], abs_tol)
        assert not bad, (g["name"], h, bad[:3])
    return states


@pytest.mark.parametrize("name", PT_CASES)
@pytest.mark.parametrize("precision", ["complex128", "mixed"])
def test_gpu_pt_build_and_dynamics(name, precision):
    from oqupy_gb300 import PtBatch
    g = gc.load(name)
    b = PtBatch([_inst(g)], precision=precision)
    b.build()
    if float(g["pt_envelope"].max()) < 1e-10:
        assert list(b.bond_dimensions(0)) == list(g["pt_bonds"])
    _check(b, 0, g, gc.PARITY_ABS if precision == "complex128" else gc.MIXED_ABS)


def test_gpu_pt_batched_builds():
    """Several process tensors (different lengths, memory, transforms) built
    in one launch per call match the reference individually."""
    from oqupy_gb300 import PtBatch
    gs = [gc.load(n) for n in PT_CASES]
    b = PtBatch([_inst(g) for g in gs])
    b.build()
    for i, g in enumerate(gs):
        _check(b, i, g, gc.PARITY_ABS)


def test_gpu_pt_backend_dropin_matches_reference():
    """The drop-in backend driven like PtTempo.compute/get_process_tensor
    (pt_tempo.py:258-306), host tensors + caps as in the reference."""
    from oqupy_gb300 import GpuPtTempoBackend
    g = gc.load("nondiag_coupling")
    D = g["d"] ** 2

    class HostPT:
        transform_in = g["pt_transform_in"]
        transform_out = g["pt_transform_out"]

        def __init__(self):
            self.t = {}

        def set_mpo_tensor(self, step, t):
            self.t[step] = t

        def compute_caps(self):
            self.caps = to.compute_caps([self.t[k] for k in sorted(self.t)], g["d"])

    pt = HostPT()
    be = GpuPtTempoBackend(g["d"], gc.pt_influence(g), pt, np.ones(D), np.ones(D),
                           g["nsteps"], g["dkmax"], g["epsrel"], {"backend": "gb300"})
    be.initialize()
    while be.compute_step():
        pass
    be.update_process_tensor()
    mpos = [pt.t[k] for k in range(g["nsteps"])]
    assert [m.shape[0] for m in mpos] + [mpos[-1].shape[1]] == list(g["pt_bonds"])
    host = to.compute_dynamics_pt(g["rho0"], gc.propagators(g), mpos, pt.caps,
                                  transform_in=pt.transform_in,
                                  transform_out=pt.transform_out)
    dev = be._batch.dynamics(0, g["prop1"][:1], g["prop2"][:1], g["rho0"].reshape(1, -1),
                             transform_in=pt.transform_in, transform_out=pt.transform_out)[:, 0]
    for ref_states in (host, dev):
        errs = [to.trace_distance(a, b) for a, b in zip(ref_states, g["pt_states"][0])]
        assert not gc.parity_violations(errs, g["pt_envelope"][0])


@pytest.mark.parametrize("precision", ["complex128", "mixed"])
def test_gpu_pt_build_big_bonds(precision):
    """The process-tensor model of the big PT configuration (alpha 0.3,
    wc 5, T 1, dt 0.02, epsrel 1e-7) at dkmax 20 and 50 steps: bonds reach
    168, so the zip-up splits have up to 672 columns.  Bond profile and the
    dynamics of three Hamiltonians against the reference."""
    import time
    from oqupy_gb300 import PtBatch
    g = gc.load("pt_config2_small")
    t0 = time.perf_counter()
    b = PtBatch([_inst(g)], precision=precision, chi_cap=192)
    b.build()
    dt = time.perf_counter() - t0
    bonds = list(b.bond_dimensions(0))
    print(f"pt_config2_small {precision}: build {dt:.1f} s, max bond {max(bonds)}")
    if precision == "complex128" and float(g["pt_envelope"].max()) < 1e-10:
        assert bonds == list(g["pt_bonds"])
    _check(b, 0, g, gc.PARITY_ABS if precision == "complex128" else gc.MIXED_ABS)


def test_gpu_pt_build_qutrit():
    """A D = 9 process tensor (mixed form; bonds reach 105, splits of up to
    945 columns) and its dynamics.  (The qutrit_superohmic fixture's process
    tensor reaches bond 320, 2880-column splits, past the 1152-column limit
    of a split on one CTA.)"""
    from oqupy_gb300 import PtBatch
    g = gc.load("ref_qutrit_C")
    b = PtBatch([_inst(g)], precision="mixed", chi_cap=128)
    b.build()
    _check(b, 0, g, gc.MIXED_ABS)


def test_gpu_dynamics_is_bit_reproducible():
    """The sweep's read-out is summed in a fixed order: two runs of the same
    sweep (64 systems, bonds up to 168, several bond chunks per step) agree
    bit for bit."""
    from oqupy_gb300 import PtBatch, bath
    g = gc.load("pt_config2_small")
    b = PtBatch([_inst(g)], precision="mixed", chi_cap=192)
    b.build()
    rng = np.random.default_rng(11)
    sx = np.array([[0, 1], [1, 0]], dtype=complex)
    sz = np.diag([1.0, -1.0]).astype(complex)
    props = [bath.half_step_propagators(a * sx + c * sz, g["dt"]) for a, c in rng.uniform(-2, 2, (64, 2))]
    p1 = np.array([p[0] for p in props])
    p2 = np.array([p[1] for p in props])
    rho0 = np.repeat(g["rho0"].reshape(1, -1), 64, 0)
    a = b.dynamics(0, p1, p2, rho0)
    c = b.dynamics(0, p1, p2, rho0)
    assert max(b.bond_dimensions(0)) > 32
    np.testing.assert_array_equal(a, c)
