"""compute_dynamics routing of the install hook (no GPU: the device sweep is
replaced by the oracle to check the plumbing)."""

import numpy as np

from oracle import tempo_oracle as to
from tests import golden_cases as gc
from tests.reference_import import import_reference


def test_compute_dynamics_routes_device_process_tensors(monkeypatch):
    oqupy = import_reference()
    import oqupy_gb300
    from oqupy_gb300 import pt as ptmod
    g = gc.load("pt_config2_small")
    dkmax = g["dkmax"]
    mpos, caps, _ = to.pt_tempo_build(g["d"], gc.pt_influence(g), g["nsteps"],
                                      dkmax, g["epsrel"])
    pt = oqupy.SimpleProcessTensor(g["d"], g["dt"])
    for k, m in enumerate(mpos):
        pt.set_mpo_tensor(k, m)
    pt.compute_caps()
    calls = []

    def fake(process_tensor, pairs, rho0s, num_steps=None):
        calls.append(len(pairs))
        p1, p2 = pairs[0]
        st = to.compute_dynamics_pt(rho0s[0], lambda s: (p1, p2), mpos, caps,
                                    num_steps=num_steps)
        return st[:, None, :]

    monkeypatch.setattr(ptmod, "device_compute_dynamics", fake)
    h = g["prop1"]
    system = oqupy.System(np.array([[0.3, 0.5], [0.5, -0.3]]))
    rho0 = np.array([[1.0, 0], [0, 0]], dtype=complex)
    oqupy_gb300.install(oqupy)
    try:
        ref = oqupy.compute_dynamics(system=system, process_tensor=pt,
                                     initial_state=rho0)
        assert calls == []                      # no device twin: reference path
        pt._gb300 = ("batch", 0)
        dev = oqupy.compute_dynamics(system=system, process_tensor=pt,
                                     initial_state=rho0)
        assert calls == [1]
        np.testing.assert_allclose(np.array(dev.states), np.array(ref.states),
                                   atol=1e-12)
        np.testing.assert_allclose(np.array(dev.times), np.array(ref.times))
    finally:
        oqupy_gb300.uninstall(oqupy)
