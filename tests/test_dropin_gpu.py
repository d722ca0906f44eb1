"""The drop-in path end to end: the unmodified OQuPy reference (installed
under ``baseline/_ref``, its ``tensornetwork`` import served by
``oracle/tnshim``) with ``oqupy_gb300.install()`` selects the GPU backends
through ``backend_config={"backend": "gb300", ...}``:

* ``oqupy.Tempo(...).compute`` and the ``oqupy.tempo_compute`` shortcut
  (oqupy/tempo.py:444-486, 1142-1209), resumed over several ``compute``
  calls as the reference allows (tempo.py:469-484);
* ``oqupy.PtTempo(...).get_process_tensor`` returning a
  ``DeviceProcessTensor`` (oqupy/pt_tempo.py:280-306), the
  ``oqupy.pt_tempo_compute`` shortcut, and ``oqupy.compute_dynamics`` on it
  (oqupy/system_dynamics.py:41-182) routed to the GPU sweep.

The reference builds the system, bath and influences with its own code
(the same construction as ``tests/golden/make_golden.py``), and the results
are compared with the reference's own recorded outputs at the parity bar.
"""

import numpy as np
import pytest

from oracle import tempo_oracle as to
from tests import golden_cases as gc
from tests.reference_import import import_reference

pytestmark = pytest.mark.gpu


def _case(oqupy, name):
    import importlib.util
    import os
    spec = importlib.util.spec_from_file_location(
        "make_golden", os.path.join(gc.GOLDEN, "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    c = dict(mg.cases(oqupy))[name]
    corr = oqupy.PowerLawSD(alpha=c["alpha"], zeta=c["zeta"], cutoff=c["wc"],
                            cutoff_type=c["cutoff_type"], temperature=c["T"])
    bath = oqupy.Bath(c["coupling"], corr)
    params = oqupy.TempoParameters(dt=c["dt"], dkmax=c["dkmax"], epsrel=c["epsrel"],
                                   add_correlation_time=c["add_corr"])
    systems = [c["h"]] + list(c.get("h_list", [])[1:])
    sys_objs = [oqupy.System(h, gammas=c["gammas"], lindblad_operators=c["lops"])
                for h in systems]
    return c, bath, params, sys_objs


@pytest.fixture(scope="module")
def oqupy():
    ref = import_reference()
    import oqupy_gb300
    oqupy_gb300.install(ref)
    yield ref
    oqupy_gb300.uninstall(ref)


@pytest.mark.parametrize("precision", ["complex128", "mixed"])
@pytest.mark.parametrize("name", ["config1_spin_boson", "nondiag_coupling"])
def test_tempo_compute_through_the_reference_driver(oqupy, name, precision):
    from oqupy_gb300 import GpuTempoBackend
    g = gc.load(name)
    c, bath, params, sys_objs = _case(oqupy, name)
    cfg = {"backend": "gb300", "precision": precision}
    end = c["nsteps"] * c["dt"]
    t = oqupy.Tempo(sys_objs[0], bath, params, c["rho0"], 0.0, backend_config=cfg)
    assert isinstance(t._backend_instance, GpuTempoBackend)
    # resumed: two compute calls, as tests/coverage/tempo_test.py:43-45 does
    t.compute(end / 2, progress_type="silent")
    dyn = t.compute(end, progress_type="silent")
    st = np.array(dyn.states).reshape(len(dyn.states), -1)
    assert len(dyn.times) == c["nsteps"] + 1
    np.testing.assert_allclose(dyn.times, g["tempo_times"], atol=1e-12)
    errs = [to.trace_distance(a, b) for a, b in zip(st, g["tempo_states"])]
    tol = gc.PARITY_ABS if precision == "complex128" else gc.MIXED_ABS
    assert not gc.parity_violations(errs, g["tempo_envelope"], tol), max(errs)
    # the shortcut
    dyn2 = oqupy.tempo_compute(sys_objs[0], bath, c["rho0"], 0.0, end, parameters=params,
                               backend_config=cfg, progress_type="silent")
    st2 = np.array(dyn2.states).reshape(len(dyn2.states), -1)
    assert max(to.trace_distance(a, b) for a, b in zip(st2, st)) <= gc.PARITY_ABS
    print(f"{name} {precision}: max trace distance to the reference {max(errs):.2e}")


@pytest.mark.parametrize("name", ["ref_spin_boson_A", "nondiag_coupling"])
def test_pt_tempo_and_compute_dynamics_through_the_reference_driver(oqupy, name):
    g = gc.load(name)
    c, bath, params, sys_objs = _case(oqupy, name)
    end = c["nsteps"] * c["dt"]
    cfg = {"backend": "gb300", "precision": "complex128"}
    ptt = oqupy.PtTempo(bath, 0.0, end, params, backend_config=cfg)
    pt = ptt.get_process_tensor(progress_type="silent")
    assert isinstance(pt, oqupy.process_tensor.BaseProcessTensor)
    assert type(pt).__name__ == "DeviceProcessTensor"
    assert len(pt) == c["nsteps"]
    if float(g["pt_envelope"].max()) < 1e-10:
        assert list(pt.get_bond_dimensions()) == list(g["pt_bonds"])
    for i, s in enumerate(sys_objs):
        dyn = oqupy.compute_dynamics(system=s, process_tensor=pt, initial_state=c["rho0"],
                                     progress_type="silent")
        st = np.array(dyn.states).reshape(len(dyn.states), -1)
        errs = [to.trace_distance(a, b) for a, b in zip(st, g["pt_states"][i])]
        assert not gc.parity_violations(errs, g["pt_envelope"][i]), max(errs)
    # the shortcut returns the device process tensor too
    pt2 = oqupy.pt_tempo_compute(bath, 0.0, end, parameters=params, backend_config=cfg,
                                 progress_type="silent")
    assert type(pt2).__name__ == "DeviceProcessTensor"
    np.testing.assert_array_equal(pt2.get_bond_dimensions(), pt.get_bond_dimensions())


def test_bond_capacity_grows_instead_of_failing(oqupy):
    """A chi_cap far below the run's bonds: the backend regrows the device
    handle and replays, the results equal a run with room to spare."""
    from oqupy_gb300 import GpuTempoBackend
    g = gc.load("batched_like_hot")
    c, bath, params, sys_objs = _case(oqupy, "batched_like_hot")
    end = c["nsteps"] * c["dt"]
    small = oqupy.Tempo(sys_objs[0], bath, params, c["rho0"], 0.0,
                        backend_config={"backend": "gb300", "chi_cap": 4})
    dyn = small.compute(end, progress_type="silent")
    be = small._backend_instance
    assert isinstance(be, GpuTempoBackend) and be.chi_cap > 4
    st = np.array(dyn.states).reshape(len(dyn.states), -1)
    big = oqupy.Tempo(sys_objs[0], bath, params, c["rho0"], 0.0,
                      backend_config={"backend": "gb300", "chi_cap": 64})
    st_big = np.array(big.compute(end, progress_type="silent").states).reshape(len(st), -1)
    assert max(to.trace_distance(a, b) for a, b in zip(st, st_big)) <= gc.PARITY_ABS
    errs = [to.trace_distance(a, b) for a, b in zip(st, g["tempo_states"])]
    assert not gc.parity_violations(errs, g["tempo_envelope"])
