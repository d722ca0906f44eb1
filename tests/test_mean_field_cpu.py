"""Mean-field TEMPO on the CPU: the oracle's restatement of
``MeanFieldTempoBackend`` (tempo_backend.py:629-773), driven by the
restated field-dependent propagators and Runge-Kutta field update of
``tests/mean_field_cases.py``, reproduces the unmodified reference's
``MeanFieldTempo`` run stored in ``tests/golden/mean_field.npz``; where the
reference is importable, the restated propagators equal its own, and
``oqupy_gb300.install()`` routes ``MeanFieldTempo`` to the GPU backend
(construction only: no device call)."""

import os

import numpy as np
import pytest

from oracle import tempo_oracle as to
from tests import golden_cases as gc
from tests import mean_field_cases as mfc

FIXTURE = os.path.join(gc.GOLDEN, "mean_field.npz")


def load():
    return np.load(FIXTURE)


def compare(name, states, fields, g, abs_tol=gc.PARITY_ABS):
    """Per-system trace distances and field errors against the fixture, at
    ``max(abs_tol, 10 x the reference's own spread)`` from the first
    rounding-sensitive step on (``golden_cases.parity_violations``)."""
    ref = g[f"{name}/states"]
    env = g[f"{name}/envelope"]
    bad, worst = [], 0.0
    for i in range(ref.shape[0]):
        err = [to.trace_distance(a, b) for a, b in zip(states[i], ref[i])]
        worst = max(worst, max(err))
        bad += [("system", i) + v for v in gc.parity_violations(err, env[i], abs_tol)]
    ferr = np.abs(np.asarray(fields) - g[f"{name}/fields"])
    # the field is computed from every system's state: it is as sensitive as
    # the most sensitive of them
    fenv = np.maximum(g[f"{name}/field_envelope"], env.max(axis=0))
    bad += [("field",) + v for v in gc.parity_violations(ferr, fenv, abs_tol)]
    return bad, worst, float(ferr.max())


def run_backend(be, nsteps):
    _, st0, f0 = be.initialize()
    states = [[s] for s in st0]
    fields = [f0]
    for _ in range(nsteps):
        _, st, f = be.compute_step()
        for i, s in enumerate(st):
            states[i].append(s)
        fields.append(f)
    return [np.array(s) for s in states], np.array(fields)


@pytest.mark.parametrize("name", sorted(mfc.CASES))
def test_oracle_reproduces_reference_mean_field(name):
    g = load()
    args = mfc.backend_args(name, g)
    o = to.MeanFieldOracle(**args)
    states, fields = run_backend(o, mfc.CASES[name]["nsteps"])
    bad, worst, fworst = compare(name, states, fields, g)
    print(f"{name}: max trace distance {worst:.2e}, max field error {fworst:.2e}")
    assert not bad, bad[:5]


def _reference():
    from tests.reference_import import import_reference
    oqupy = import_reference()
    mfc.patch_field_hamiltonian_check(oqupy)
    return oqupy


def test_restated_propagators_equal_reference():
    oqupy = _reference()
    for name, case in mfc.CASES.items():
        for s in case["systems"]:
            gam = [(lambda t, g=g: g) for g in s["gammas"]]
            lops = [(lambda t, a=a: a) for a in s["lops"]]
            sysf = oqupy.TimeDependentSystemWithField(s["h"], gammas=gam, lindblad_operators=lops)
            ref = sysf.get_propagators(case["dt"], 0.0, None, 1e-7)
            mine = mfc.propagators(s, case["dt"])
            for step, field, deriv in [(0, 1.0, 0.0), (3, 0.2 - 0.4j, -0.3 + 0.7j), (17, -0.05j, 1.1)]:
                for a, b in zip(ref(step, field, deriv), mine(step, field, deriv)):
                    np.testing.assert_allclose(b, a, rtol=0, atol=1e-14)


def test_install_routes_mean_field_tempo():
    oqupy = _reference()
    import oqupy_gb300
    from oqupy_gb300.mean_field import GpuMeanFieldTempoBackend
    case = mfc.CASES["dicke_G"]
    s = case["systems"][0]
    oqupy_gb300.install(oqupy)
    try:
        sysf = oqupy.TimeDependentSystemWithField(s["h"])
        mfs = oqupy.MeanFieldSystem([sysf], field_eom=case["field_eom"])
        corr = oqupy.PowerLawSD(alpha=s["alpha"], zeta=s["zeta"], cutoff=s["wc"],
                                cutoff_type=s["cutoff_type"], temperature=s["T"])
        bath = oqupy.Bath(s["coupling"], corr)
        params = oqupy.TempoParameters(dt=case["dt"], tcut=case["tcut"], epsrel=case["epsrel"])
        mft = oqupy.MeanFieldTempo(mfs, [bath], params, [s["rho0"]], case["field0"],
                                   backend_config={"backend": "gb300", "precision": "mixed"})
        assert isinstance(mft._backend_instance, GpuMeanFieldTempoBackend)
        # degeneracy maps stay on the reference backend
        mft2 = oqupy.MeanFieldTempo(mfs, [bath], params, [s["rho0"]], case["field0"],
                                    backend_config={"backend": "gb300"}, unique=True)
        assert not isinstance(mft2._backend_instance, GpuMeanFieldTempoBackend)
    finally:
        oqupy_gb300.uninstall(oqupy)
    mft3 = oqupy.MeanFieldTempo(mfs, [bath], params, [s["rho0"]], case["field0"])
    assert not isinstance(mft3._backend_instance, GpuMeanFieldTempoBackend)


class OracleBatch:
    """Stand-in for ``TempoBatch`` on the CPU: each instance is a
    ``TempoOracle`` fed through the same per-step calls the GPU backend makes
    (propagators of all systems, influences of a growing window, the
    first-site influence past dkmax), with the engine's bond-capacity
    overflow status.  Exercises the backend's host logic without a GPU."""

    def __init__(self, instances, precision="complex128", chi_cap=64, out_cap=4,
                 max_sites=0, block=0, smem_kb=0, qr_cut=0.0):
        from oqupy_gb300 import _native as nat
        self._overflow = nat.OTB_ERR_CHI_OVERFLOW
        self.n = len(instances)
        self.D = [int(inst["hs_dim"]) ** 2 for inst in instances]
        self.cap = chi_cap
        self._infl = [dict(enumerate(inst["influences"])) for inst in instances]
        self._neg = [None] * self.n
        self._status = [0] * self.n
        self._hist = [dict() for _ in range(self.n)]
        self._step = 0
        self._pending = [None] * self.n
        self._oracles = []
        for i, inst in enumerate(instances):
            ones = np.ones(self.D[i])
            o = to.TempoOracle(inst["rho0"], (lambda dk, i=i: self._influence(i, dk)),
                               inst["unitary"], None, ones, ones, inst["dkmax"], inst["epsrel"])
            self._hist[i][0] = o.initialize()[1]
            self._oracles.append(o)

    def _influence(self, i, dk):
        if dk < 0:
            return self._neg[i]
        if dk not in self._infl[i]:
            # full memory: the oracle fetches the influence of step s + 1's
            # new window site during step s (tempo_backend.py:487-497), the
            # engine reads it at step s + 1; a placeholder now, the matrix
            # the host set by then at the next advance
            self._pending[i] = dk
            return np.full((self.D[i], self.D[i]), np.nan, dtype=np.complex128)
        return self._infl[i][dk]

    def set_all_propagators(self, p1s, p2s, unitaries=None, stream=None):
        self._props = (list(p1s), list(p2s))   # the oracle applies the unitary itself

    def set_influence(self, i, dk, mat):
        self._infl[i][dk] = np.asarray(mat)

    def set_first_influence(self, i, mat=None):
        self._neg[i] = None if mat is None else np.asarray(mat)

    def reserve_sites(self, nslots):
        pass

    def advance(self, nsteps=1, stream=None):
        for _ in range(nsteps):
            self._step += 1
            for i, o in enumerate(self._oracles):
                if self._status[i] != 0:
                    continue
                if self._pending[i] is not None:
                    o._mpo[0] = to.delta_1001(self._infl[i][self._pending[i]])
                    self._pending[i] = None
                self._hist[i][self._step] = o.compute_system_step(
                    self._step, np.asarray(self._props[0][i]), np.asarray(self._props[1][i]))
                if max(o.bond_dimensions() or [1]) > self.cap:
                    self._status[i] = self._overflow

    def info(self, i):
        return {"status": self._status[i], "nsites": len(self._oracles[i]._mps)}

    def states(self, first, count):
        return [np.array([self._hist[i][first + k] for k in range(count)]) for i in range(self.n)]

    def bond_dims(self, i):
        return self._oracles[i].bond_dimensions()

    def close(self):
        pass


@pytest.mark.parametrize("name", sorted(mfc.CASES))
def test_mean_field_backend_host_logic(name, monkeypatch):
    """The GPU backend's per-step host logic on the oracle stand-in, started
    with a bond capacity of 4 so that it regrows and replays: the same
    numbers as the oracle's own mean-field loop."""
    from oqupy_gb300 import mean_field
    monkeypatch.setattr(mean_field, "TempoBatch", OracleBatch)
    g = load()
    args = mfc.backend_args(name, g)
    n = len(args["initial_state_list"])
    ones = [np.ones(np.asarray(s).size) for s in args["initial_state_list"]]
    be = mean_field.GpuMeanFieldTempoBackend(
        args["initial_state_list"], args["initial_field"], args["influence_list"],
        args["unitary_transform_list"], args["propagators_list"], args["compute_field"],
        args["compute_field_derivative"], ones, ones, args["dkmax"], args["epsrel"],
        config={"chi_cap": 4}, degeneracy_maps_list=[None] * n)
    nsteps = mfc.CASES[name]["nsteps"]
    states, fields = run_backend(be, nsteps)
    assert be.chi_cap > 4
    ref_states, ref_fields = run_backend(to.MeanFieldOracle(**args), nsteps)
    for a, b in zip(states, ref_states):
        np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(fields, ref_fields)


# -- mean-field dynamics on process tensors (compute_dynamics_with_field) --

def pt_inputs(g, name, i):
    """(influence callable, dkmax, transforms) of system i's process tensor."""
    infl = g[f"{name}/pt_influences{i}"]
    dk = int(g[f"{name}/pt_dkmax{i}"])
    dkmax = len(infl) - 1 if dk < 0 else dk       # full memory: every influence of the run
    tin = g[f"{name}/pt_transform_in{i}"] if f"{name}/pt_transform_in{i}" in g.files else None
    tout = g[f"{name}/pt_transform_out{i}"] if f"{name}/pt_transform_out{i}" in g.files else None
    return (lambda k: infl[k] if k >= 0 else None), dkmax, tin, tout


def oracle_pts(g, name):
    case = mfc.CASES[name]
    out = []
    for i, s in enumerate(case["systems"]):
        f, dkmax, tin, tout = pt_inputs(g, name, i)
        d = int(round(np.sqrt(np.asarray(s["rho0"]).size)))
        mpos, caps, _ = to.pt_tempo_build(d, f, case["nsteps"], dkmax, case["epsrel"])
        out.append((mpos, caps, tin, tout))
    return out


def compare_pt(name, states, fields, g, abs_tol=1e-10):
    ref = g[f"{name}/pt_states"]
    env = g[f"{name}/pt_envelope"]
    bad, worst = [], 0.0
    for i in range(ref.shape[0]):
        err = [to.trace_distance(np.asarray(a).reshape(-1), b) for a, b in zip([s[i] for s in states], ref[i])]
        worst = max(worst, max(err))
        bad += [("system", i) + v for v in gc.parity_violations(err, env[i], abs_tol)]
    ferr = np.abs(np.asarray(fields) - g[f"{name}/pt_fields"])
    fenv = np.maximum(g[f"{name}/pt_field_envelope"], env.max(axis=0))
    bad += [("field",) + v for v in gc.parity_violations(ferr, fenv, abs_tol)]
    return bad, worst, float(ferr.max())


@pytest.mark.parametrize("name", sorted(mfc.CASES))
def test_oracle_reproduces_reference_dynamics_with_field(name):
    g = load()
    case = mfc.CASES[name]
    props = [mfc.propagators(s, case["dt"]) for s in case["systems"]]
    states, fields = to.dynamics_with_field_pt([s["rho0"] for s in case["systems"]], props,
                                               case["field_eom"], case["field0"], oracle_pts(g, name),
                                               case["nsteps"], case["dt"])
    bad, worst, fworst = compare_pt(name, states, fields, g)
    print(name, f"{worst:.1e} {fworst:.1e}")
    assert not bad, bad[:5]


class SessionModelBatch:
    """Stand-in for ``PtBatch.session``: the step of ``dyn_step_kernel``
    (site storage ``[l][m][r]``, ``T = d * site``, one pair per system)
    over the oracle's process tensor."""

    def __init__(self, mpos, caps, d):
        self.d = d
        self.sites = [np.transpose(T, (0, 2, 1)) / d for T in mpos]
        self.caps = caps

    def session(self, i, rho0):
        batch = self

        class Session:
            def __init__(self):
                self.v = [np.asarray(r).reshape(1, -1) for r in np.asarray(rho0)]
                self.k = 0

            def state(self, step):
                assert step == 0
                return np.array([np.einsum("ra,r->a", v, batch.caps[0]) for v in self.v])

            def step(self, props):
                out = []
                for h, (P1, P2) in enumerate(np.asarray(props)):
                    u = np.einsum("ab,lb->la", P1, self.v[h])
                    w = batch.d * np.einsum("la,lar->ra", u, batch.sites[self.k])
                    self.v[h] = np.einsum("ab,rb->ra", P2, w)
                    out.append(np.einsum("ra,r->a", self.v[h], batch.caps[self.k + 1]))
                self.k += 1
                return np.array(out)

            def close(self):
                pass
        return Session()


class FakeDevPt:
    def __init__(self, batch, tin, tout):
        self.device = (batch, 0)
        self.transform_in, self.transform_out = tin, tout


@pytest.mark.parametrize("name", sorted(mfc.CASES))
def test_dynamics_with_field_host_logic_on_session_model(name):
    from oqupy_gb300.mean_field import device_dynamics_with_field
    g = load()
    case = mfc.CASES[name]
    pts = []
    for (mpos, caps, tin, tout), s in zip(oracle_pts(g, name), case["systems"]):
        d = int(round(np.sqrt(np.asarray(s["rho0"]).size)))
        pts.append(FakeDevPt(SessionModelBatch(mpos, caps, d), tin, tout))
    props = [mfc.propagators(s, case["dt"]) for s in case["systems"]]
    times, states, fields = device_dynamics_with_field(
        props, case["field_eom"], case["field0"], pts, [s["rho0"] for s in case["systems"]],
        case["nsteps"], case["dt"])
    assert len(times) == case["nsteps"] + 1
    bad, worst, fworst = compare_pt(name, states, fields, g)
    print(name, f"{worst:.1e} {fworst:.1e}")
    assert not bad, bad[:5]


def test_install_routes_dynamics_with_field(monkeypatch):
    """``oqupy.compute_dynamics_with_field`` on a device process tensor goes
    to ``mean_field.device_dynamics_with_field`` (here over the session
    model) and returns the reference's numbers."""
    from tests.reference_import import import_reference
    oqupy = import_reference()
    mfc.patch_field_hamiltonian_check(oqupy)
    import oqupy_gb300
    from oqupy_gb300 import mean_field
    from oqupy_gb300.device_pt import device_process_tensor_class
    g = load()
    name = "dicke_G"
    case = mfc.CASES[name]
    s = case["systems"][0]
    (mpos, caps, tin, tout), = oracle_pts(g, name)
    batch = SessionModelBatch(mpos, caps, 2)
    batch.meta = [dict(num_steps=len(mpos))]
    batch.mpo_tensor = lambda i, k: np.array(mpos[k])
    batch.cap = lambda i, k: np.array(caps[k])
    batch.bond_dimensions = lambda i: np.array([m.shape[0] for m in mpos] + [mpos[-1].shape[1]])
    batch.check_status = lambda: None
    calls = []
    real = mean_field.device_dynamics_with_field

    def spy(*a, **k):
        calls.append(1)
        return real(*a, **k)
    monkeypatch.setattr(mean_field, "device_dynamics_with_field", spy)
    sysf = oqupy.TimeDependentSystemWithField(s["h"])
    mfs = oqupy.MeanFieldSystem([sysf], field_eom=case["field_eom"])
    oqupy_gb300.install(oqupy)
    try:
        cls = device_process_tensor_class(oqupy.process_tensor.BaseProcessTensor)
        dev = cls(batch, 0, 2, case["dt"], tin, tout)
        dyn = oqupy.compute_dynamics_with_field(mfs, initial_field=case["field0"],
                                                process_tensor_list=[dev],
                                                initial_state_list=[s["rho0"]], subdiv_limit=None,
                                                progress_type="silent")
    finally:
        oqupy_gb300.uninstall(oqupy)
    assert calls == [1]
    states = [[np.asarray(m).reshape(-1)] for m in dyn.system_dynamics[0].states]
    bad, worst, fworst = compare_pt(name, states, dyn.fields, g)
    assert not bad, bad[:5]
