"""n-time correlations and controlled / time-dependent process-tensor
dynamics on the CPU: the oracle reproduces the unmodified reference's
outputs (``tests/golden/correlations.npz``), and the GPU path's host logic
(``oqupy_gb300.correlations``: the propagator table, the folding of control
operations into it, the correlation slots) gives the same numbers when the
device sweep is replaced by a host stand-in that walks the table over the
oracle's process tensor.  Where the reference is importable, the install
hook routes ``compute_correlations`` / ``compute_dynamics`` on a device
process tensor to the GPU functions."""

import numpy as np
import pytest

from oracle import tempo_oracle as to
from tests import correlation_cases as cc


def oracle_pt(g, name):
    d = int(g[f"{name}/d"])
    mpos, caps, _ = to.pt_tempo_build(d, cc.influence(g, name), int(g[f"{name}/nsteps"]),
                                      int(g[f"{name}/dkmax"]), float(g[f"{name}/epsrel"]))
    return mpos, caps, cc.get(g, name, "transform_in"), cc.get(g, name, "transform_out")


def oracle_functions(g, name):
    mpos, caps, tin, tout = oracle_pt(g, name)

    def sweep(props, rho0, n, ctl):
        f = None
        if ctl is not None:
            def f(step):
                return ctl["pre"].get(step), ctl["post"].get(step)
        return to.compute_dynamics_pt(rho0, props, mpos, caps, n, tin, tout, controls=f)

    def corr(props, rho0, ops, steps, order):
        return to.correlations_nt_pt(rho0, props, mpos, caps, ops, steps, order, tin, tout)
    return sweep, corr


@pytest.mark.parametrize("name", cc.CASES)
def test_oracle_reproduces_reference_correlations(name):
    g = cc.load()
    out = cc.run(g, name, *oracle_functions(g, name))
    bad, worst = cc.check(g, name, out)
    print(name, worst)
    assert not bad, bad


class TableSweepBatch:
    """Stand-in for ``PtBatch.dynamics_steps``: walks the propagator table
    the GPU path builds over the oracle's process tensor (transforms and
    controls already folded into the table, as on the device)."""

    def __init__(self, mpos, caps):
        self.mpos, self.caps = mpos, caps

    def dynamics_steps(self, i, props, prop_index, rho0, num_steps, stream=None):
        props = np.asarray(props)
        rho0 = np.asarray(rho0)
        H, D = rho0.shape
        out = np.zeros((num_steps + 1, H, D), dtype=np.complex128)
        for h in range(H):
            v = rho0[h].reshape(1, D)
            out[0, h] = np.einsum("ba,b->a", v, self.caps[0])
            for k in range(num_steps):
                p1, p2 = props[prop_index[h][k]]
                v = v @ p1.T
                v = np.einsum("la,lrab->rb", v, to.pt_mpo_rank4(self.mpos[k]))
                v = v @ p2.T
                out[k + 1, h] = np.einsum("ba,b->a", v, self.caps[k + 1])
        return out


class FakeDevicePt:
    def __init__(self, batch, tin, tout):
        self.device = (batch, 0)
        self.transform_in, self.transform_out = tin, tout


@pytest.mark.parametrize("name", cc.CASES)
def test_gpu_host_logic_on_table_stand_in(name):
    from oqupy_gb300 import correlations as corr
    g = cc.load()
    mpos, caps, tin, tout = oracle_pt(g, name)
    pt = FakeDevicePt(TableSweepBatch(mpos, caps), tin, tout)

    def sweep(props, rho0, n, ctl):
        return corr.device_dynamics(pt, [props], [rho0], n, [ctl])[:, 0]

    def correl(props, rho0, ops, steps, order):
        return corr.device_correlations_nt(pt, props, rho0, ops, steps, order)
    out = cc.run(g, name, sweep, correl)
    bad, worst = cc.check(g, name, out)
    print(name, worst)
    assert not bad, bad


def test_propagator_table_deduplicates_and_folds():
    from oqupy_gb300 import correlations as corr
    g = cc.load()
    name = "corr_nondiag"
    mpos, caps, tin, tout = oracle_pt(g, name)
    seen = {}

    class Capture(TableSweepBatch):
        def dynamics_steps(self, i, props, prop_index, rho0, num_steps, stream=None):
            seen["props"], seen["index"] = np.asarray(props), np.asarray(prop_index)
            return super().dynamics_steps(i, props, prop_index, rho0, num_steps)
    pt = FakeDevicePt(Capture(mpos, caps), tin, tout)
    p1, p2 = g[f"{name}/prop1"], g[f"{name}/prop2"]

    def props(step):
        return p1, p2
    ctl = cc.controls(g, name)
    rho0 = g[f"{name}/rho0"]
    corr.device_dynamics(pt, [props, props], [rho0, rho0], 10, [None, ctl])
    # one base pair for the shared time-independent propagators, one per
    # step that carries a control (pre at 3 -> step 2's P2; post at 5)
    assert len(seen["props"]) == 3
    assert (seen["index"][0] == 0).all()
    assert set(np.flatnonzero(seen["index"][1])) == {2, 5}
    base1 = tin.T @ p1 if tin is not None else p1
    np.testing.assert_allclose(seen["props"][seen["index"][1][5]][0],
                               base1 @ ctl["post"][5], rtol=1e-14)


def test_install_routes_correlations_and_controlled_dynamics(monkeypatch):
    from tests.reference_import import import_reference
    from tests.reference_compat import patch_vectorize_checks
    oqupy = import_reference()
    patch_vectorize_checks(oqupy)
    import oqupy_gb300
    from oqupy_gb300 import correlations as corr
    from oqupy_gb300.device_pt import device_process_tensor_class
    g = cc.load()
    name = "corr_nondiag"
    mpos, caps, tin, tout = oracle_pt(g, name)
    batch = TableSweepBatch(mpos, caps)
    batch.meta = [dict(num_steps=len(mpos))]
    batch.mpo_tensor = lambda i, k: np.array(mpos[k])
    batch.cap = lambda i, k: np.array(caps[k])
    batch.bond_dimensions = lambda i: np.array([m.shape[0] for m in mpos] + [mpos[-1].shape[1]])
    batch.check_status = lambda: None
    calls = []
    real = corr.device_dynamics

    def spy(*a, **k):
        calls.append(len(a[2]))
        return real(*a, **k)
    monkeypatch.setattr(corr, "device_dynamics", spy)
    oqupy_gb300.install(oqupy)
    try:
        cls = device_process_tensor_class(oqupy.process_tensor.BaseProcessTensor)
        dev = cls(batch, 0, int(g[f"{name}/d"]), 0.1, tin, tout)
        sx, sz = oqupy.operators.sigma("x"), oqupy.operators.sigma("z")
        sm, sp = oqupy.operators.sigma("-"), oqupy.operators.sigma("+")
        system = oqupy.System(0.5 * sz + 0.3 * sx)
        t, c = oqupy.compute_correlations(system, dev, sm, sp, slice(0, 10, 3), slice(0, None),
                                          initial_state=g[f"{name}/rho0"].reshape(2, 2),
                                          progress_type="silent")
        np.testing.assert_allclose(c, g[f"{name}/ordered"], rtol=0, atol=1e-10)
        assert calls == [4]      # one batched sweep, one slot per time of operator A
        ctrl = oqupy.Control(2)
        for step, op, post in zip(g[f"{name}/control_steps"], g[f"{name}/control_ops"],
                                  g[f"{name}/control_post"]):
            ctrl.add_single(int(step), op, post=bool(post))
        dyn = oqupy.compute_dynamics(system, process_tensor=dev, control=ctrl,
                                     initial_state=g[f"{name}/rho0"].reshape(2, 2),
                                     progress_type="silent")
        st = np.array(dyn.states).reshape(len(dyn.states), -1)
        assert max(to.trace_distance(a, b) for a, b in zip(st, g[f"{name}/control_states"])) < 1e-10
        assert calls[-1] == 1
    finally:
        oqupy_gb300.uninstall(oqupy)
