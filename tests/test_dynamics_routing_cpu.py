"""compute_dynamics routing of the install hook and the DeviceProcessTensor
interface (no GPU: the device batch is a host stand-in holding the oracle's
tensors, and the device sweep is replaced by the oracle to check the
plumbing)."""

import numpy as np
import pytest

from oracle import tempo_oracle as to
from tests import golden_cases as gc
from tests.reference_import import import_reference


class HostBatch:
    """Stand-in for ``PtBatch`` with the accessors DeviceProcessTensor uses."""

    def __init__(self, mpos, caps):
        self.mpos, self.caps = mpos, caps
        self.meta = [dict(num_steps=len(mpos))]

    def mpo_tensor(self, i, step):
        return np.array(self.mpos[step])

    def cap(self, i, step):
        return np.array(self.caps[step])

    def bond_dimensions(self, i):
        return np.array([m.shape[0] for m in self.mpos] + [self.mpos[-1].shape[1]])

    def check_status(self):
        pass


def _build():
    g = gc.load("nondiag_coupling")
    mpos, caps, _ = to.pt_tempo_build(g["d"], gc.pt_influence(g), g["nsteps"],
                                      g["dkmax"], g["epsrel"])
    return g, mpos, caps


def test_device_process_tensor_matches_simple_process_tensor():
    oqupy = import_reference()
    from oqupy_gb300.device_pt import device_process_tensor_class
    g, mpos, caps = _build()
    rng = np.random.default_rng(3)
    tin = rng.normal(size=(4, 4)) + 1j * rng.normal(size=(4, 4))
    tout = rng.normal(size=(4, 4)) + 1j * rng.normal(size=(4, 4))
    simple = oqupy.SimpleProcessTensor(g["d"], g["dt"], tin, tout)
    for k, m in enumerate(mpos):
        simple.set_mpo_tensor(k, m)
    simple.compute_caps()
    cls = device_process_tensor_class(oqupy.process_tensor.BaseProcessTensor)
    dev = cls(HostBatch(mpos, [simple.get_cap_tensor(k) for k in range(len(mpos) + 1)]), 0,
              g["d"], g["dt"], tin, tout)
    assert isinstance(dev, oqupy.process_tensor.BaseProcessTensor)
    assert len(dev) == len(simple)
    assert dev.dt == simple.dt and dev.hilbert_space_dimension == simple.hilbert_space_dimension
    assert dev.get_initial_tensor() is None
    np.testing.assert_array_equal(dev.get_bond_dimensions(), simple.get_bond_dimensions())
    for k in (0, len(mpos) // 2, len(mpos) - 1):
        for tr in (True, False):
            np.testing.assert_allclose(dev.get_mpo_tensor(k, tr), simple.get_mpo_tensor(k, tr),
                                       rtol=1e-13, atol=1e-15)
    for k in (0, len(mpos)):
        np.testing.assert_allclose(dev.get_cap_tensor(k), simple.get_cap_tensor(k))
    assert dev.get_cap_tensor(len(mpos) + 1) is None
    with pytest.raises(IndexError):
        dev.get_mpo_tensor(len(mpos))
    host = dev.to_host(oqupy.SimpleProcessTensor)
    for k in range(len(mpos) + 1):
        np.testing.assert_allclose(host.get_cap_tensor(k), simple.get_cap_tensor(k), rtol=1e-12)


def test_compute_dynamics_routes_device_process_tensors(monkeypatch):
    oqupy = import_reference()
    import oqupy_gb300
    from oqupy_gb300.device_pt import device_process_tensor_class
    g, mpos, caps = _build()
    pt = oqupy.SimpleProcessTensor(g["d"], g["dt"])
    for k, m in enumerate(mpos):
        pt.set_mpo_tensor(k, m)
    pt.compute_caps()
    calls = []

    def fake(process_tensor, propagators, rho0s, num_steps, controls=None):
        calls.append(len(propagators))
        assert controls == [None]
        st = to.compute_dynamics_pt(rho0s[0], propagators[0], mpos, caps,
                                    num_steps=num_steps)
        return st[:, None, :]

    from oqupy_gb300 import correlations
    monkeypatch.setattr(correlations, "device_dynamics", fake)
    system = oqupy.System(np.array([[0.3, 0.5], [0.5, -0.3]]))
    rho0 = np.array([[1.0, 0], [0, 0]], dtype=complex)
    oqupy_gb300.install(oqupy)
    try:
        ref = oqupy.compute_dynamics(system=system, process_tensor=pt,
                                     initial_state=rho0)
        assert calls == []                      # host process tensor: reference path
        cls = device_process_tensor_class(oqupy.process_tensor.BaseProcessTensor)
        dev_pt = cls(HostBatch(mpos, [pt.get_cap_tensor(k) for k in range(len(mpos) + 1)]), 0,
                     g["d"], g["dt"])
        dev = oqupy.compute_dynamics(system=system, process_tensor=dev_pt,
                                     initial_state=rho0)
        assert calls == [1]
        np.testing.assert_allclose(np.array(dev.states), np.array(ref.states),
                                   atol=1e-12)
        np.testing.assert_allclose(np.array(dev.times), np.array(ref.times))
        # record_all=False is not routed: the reference runs on a host copy
        last = oqupy.compute_dynamics(system=system, process_tensor=dev_pt,
                                      initial_state=rho0, record_all=False)
        assert calls == [1]
        np.testing.assert_allclose(np.array(last.states)[-1], np.array(ref.states)[-1], atol=1e-12)
    finally:
        oqupy_gb300.uninstall(oqupy)
