"""Gradients on the process-tensor sweep (``compute_gradient_and_dynamics``,
oqupy/gradient.py:169-437) on the CPU: the oracle's restatement reproduces
the unmodified reference's derivative tensors and states stored in
``tests/golden/gradient.npz`` (made by ``tests/golden/make_gradient.py``),
with and without control operations, at 1e-10 (10x the reference's own
spread where that is larger)."""

import os

import numpy as np
import pytest

from oracle import tempo_oracle as to
from tests import golden_cases as gc

FIXTURE = os.path.join(gc.GOLDEN, "gradient.npz")
CASES = ("grad_nondiag", "grad_diag")


def load():
    return np.load(FIXTURE)


def get(g, name, key):
    k = f"{name}/{key}"
    return g[k] if k in g.files else None


def controls(g, name):
    out = {"pre": {}, "post": {}}
    for step, op, post in zip(g[f"{name}/control_steps"], g[f"{name}/control_ops"],
                              g[f"{name}/control_post"]):
        side = out["post" if post else "pre"]
        side[int(step)] = op if int(step) not in side else op @ side[int(step)]
    return out


def propagators(g, name):
    p1, p2 = g[f"{name}/prop1"], g[f"{name}/prop2"]
    return lambda step: (p1[step], p2[step])


def oracle_pt(g, name):
    infl = g[f"{name}/influences"]
    d = int(g[f"{name}/d"])
    mpos, caps, _ = to.pt_tempo_build(d, lambda dk: infl[dk] if dk >= 0 else None,
                                      int(g[f"{name}/nsteps"]), int(g[f"{name}/dkmax"]),
                                      float(g[f"{name}/epsrel"]))
    return mpos, caps


def check(g, name, tag, derivs, states, abs_tol=gc.PARITY_ABS):
    ref_d, ref_s = g[f"{name}/{tag}_derivs"], g[f"{name}/{tag}_states"]
    env_d, env_s = g[f"{name}/{tag}_derivs_envelope"], g[f"{name}/{tag}_states_envelope"]
    err_d = np.abs(np.asarray(derivs) - ref_d).reshape(len(ref_d), -1).max(axis=1)
    err_s = np.abs(np.asarray(states) - ref_s).max(axis=1)
    bad = []
    if (err_d > np.maximum(abs_tol, gc.ENVELOPE_FACTOR * env_d)).any():
        bad.append(("derivs", float(err_d.max())))
    if (err_s > np.maximum(abs_tol, gc.ENVELOPE_FACTOR * env_s)).any():
        bad.append(("states", float(err_s.max())))
    return bad, float(err_d.max()), float(err_s.max())


@pytest.mark.parametrize("tag", ["plain", "control"])
@pytest.mark.parametrize("name", CASES)
def test_oracle_reproduces_reference_gradient(name, tag):
    g = load()
    mpos, caps = oracle_pt(g, name)
    ctl = controls(g, name) if tag == "control" else None
    f = None if ctl is None else (lambda s: (ctl["pre"].get(s), ctl["post"].get(s)))
    derivs, states = to.gradient_pt(g[f"{name}/rho0"], propagators(g, name), mpos, caps,
                                    int(g[f"{name}/nsteps"]), g[f"{name}/target"],
                                    get(g, name, "transform_in"), get(g, name, "transform_out"), f)
    bad, ed, es = check(g, name, tag, derivs, states)
    print(name, tag, f"derivs {ed:.1e}, states {es:.1e}")
    assert not bad, bad


class KernelModelBatch:
    """Stand-in for ``PtBatch.gradient_cores``: the three kernels of
    ``otb_dyn_gradient`` (forward step with recording, adjoint step,
    derivative cores) written out with their index conventions -- site
    storage ``[l][m][r]`` with ``T[l][r][m] = d * site[l][m][r]``, propagator
    pairs from the table -- over the oracle's process tensor.  Checks the
    host side (table, folding, leg maps) and the kernels' algebra on the
    CPU."""

    def __init__(self, mpos, caps, d):
        self.d = d
        self.sites = [np.transpose(T, (0, 2, 1)) / d for T in mpos]   # [l][m][r]
        self.caps = caps

    def gradient_cores(self, i, props, prop_index, rho0, target, num_steps, stream=None):
        props = np.asarray(props)
        H, D = np.asarray(rho0).shape
        n = int(num_steps)
        states = np.zeros((n + 1, H, D), dtype=np.complex128)
        cores = np.zeros((H, n, D, D, D), dtype=np.complex128)
        for h in range(H):
            v = np.asarray(rho0)[h].reshape(1, D)
            states[0, h] = v[0] * self.caps[0][0]
            fwd = []
            for k in range(n):
                fwd.append(v.copy())
                P1, P2 = props[prop_index[h][k]]
                site = self.sites[k]
                u = np.einsum("ab,lb->la", P1, v)                        # u[l][a] = sum_b P1[a][b] v[l][b]
                w = self.d * np.einsum("la,lar->ra", u, site)            # w[r][a]
                v = np.einsum("ab,rb->ra", P2, w)
                states[k + 1, h] = np.einsum("ra,r->a", v, self.caps[k + 1])
            Y = [None] * (n + 1)
            Y[n] = np.asarray(target)[h].reshape(1, D)
            for k in range(n - 1, 0, -1):
                P1, P2 = props[prop_index[h][k]]
                site = self.sites[k]
                u = np.einsum("ec,re->rc", P2, Y[k + 1])                 # u[r][c] = sum_e P2[e][c] Y[r][e]
                w = self.d * np.einsum("lbr,rb->lb", site, u)            # w[l][b]
                Y[k] = np.einsum("ba,lb->la", P1, w)                     # Y_k[l][a] = sum_b P1[b][a] w[l][b]
            for k in range(n):
                X = self.d * np.einsum("la,lmr->ram", fwd[k], self.sites[k])   # X[r][a][m]
                cores[h, k] = np.einsum("ram,re->ame", X, Y[k + 1])
        return states, cores


class FakePt:
    def __init__(self, batch, tin, tout):
        self.device = (batch, 0)
        self.transform_in, self.transform_out = tin, tout


@pytest.mark.parametrize("tag", ["plain", "control"])
@pytest.mark.parametrize("name", CASES)
def test_gpu_gradient_host_logic_on_kernel_model(name, tag):
    from oqupy_gb300 import correlations as corr
    g = load()
    mpos, caps = oracle_pt(g, name)
    pt = FakePt(KernelModelBatch(mpos, caps, int(g[f"{name}/d"])), get(g, name, "transform_in"),
                get(g, name, "transform_out"))
    ctl = controls(g, name) if tag == "control" else None
    derivs, states = corr.device_gradient(pt, propagators(g, name), g[f"{name}/rho0"],
                                          g[f"{name}/target"], int(g[f"{name}/nsteps"]), ctl)
    bad, ed, es = check(g, name, tag, derivs, states)
    print(name, tag, f"derivs {ed:.1e}, states {es:.1e}")
    assert not bad, bad


def test_install_routes_gradient_to_device_sweeps(monkeypatch):
    """``oqupy.gradient.compute_gradient_and_dynamics`` on a device process
    tensor goes to ``correlations.device_gradient`` (here over the kernel
    model) and returns the reference's numbers; ``state_gradient`` reaches it
    through the module global."""
    from tests.reference_import import import_reference
    from tests.reference_compat import patch_vectorize_checks
    oqupy = import_reference()
    patch_vectorize_checks(oqupy)
    import oqupy.gradient  # noqa: F401
    import oqupy_gb300
    from oqupy_gb300 import correlations as corr
    from oqupy_gb300.device_pt import device_process_tensor_class
    g = load()
    name = "grad_nondiag"
    mpos, caps = oracle_pt(g, name)
    d = int(g[f"{name}/d"])
    batch = KernelModelBatch(mpos, caps, d)
    batch.meta = [dict(num_steps=len(mpos))]
    batch.mpo_tensor = lambda i, k: np.array(mpos[k])
    batch.cap = lambda i, k: np.array(caps[k])
    batch.bond_dimensions = lambda i: np.array([m.shape[0] for m in mpos] + [mpos[-1].shape[1]])
    batch.check_status = lambda: None
    calls = []
    real = corr.device_gradient

    def spy(*a, **k):
        calls.append(1)
        return real(*a, **k)
    monkeypatch.setattr(corr, "device_gradient", spy)
    sx, sz, sm = oqupy.operators.sigma("x"), oqupy.operators.sigma("z"), oqupy.operators.sigma("-")
    h = lambda hx, hz: hx * sx + hz * sz   # noqa: E731
    ps = oqupy.ParameterizedSystem(h, gammas=[lambda hx, hz: 0.1], lindblad_operators=[lambda hx, hz: sm])
    ps._hamiltonian = h
    params = np.random.default_rng(42).uniform(-1.0, 1.0, size=(2 * len(mpos), 2))
    oqupy_gb300.install(oqupy)
    try:
        cls = device_process_tensor_class(oqupy.process_tensor.BaseProcessTensor)
        dev = cls(batch, 0, d, 0.1, get(g, name, "transform_in"), get(g, name, "transform_out"))
        derivs, dyn = oqupy.gradient.compute_gradient_and_dynamics(
            system=ps, initial_state=g[f"{name}/rho0"].reshape(2, 2),
            target_derivative=g[f"{name}/target"].reshape(2, 2), process_tensors=[dev],
            parameters=params, dt=0.1, num_steps=len(mpos), progress_type="silent")
    finally:
        oqupy_gb300.uninstall(oqupy)
    assert calls == [1]
    states = np.array(dyn.states).reshape(len(dyn.states), -1)
    bad, ed, es = check(g, name, "plain", np.array(derivs), states)
    assert not bad, bad
