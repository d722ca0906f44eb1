"""Mean-field TEMPO on the GPU (``oqupy_gb300.mean_field``, the drop-in for
``MeanFieldTempoBackend``, tempo_backend.py:629-773) against the unmodified
reference's ``MeanFieldTempo`` runs stored in ``tests/golden/mean_field.npz``
(made by ``tests/golden/make_mean_field.py``): every system's state and the
field after every step, both precision forms, at the parity bar of
``golden_cases.parity_violations`` (complex128: 1e-10 trace distance until
the reference's own 1e-15-perturbation spread exceeds 1e-10, 10x that
spread from there; mixed: 1e-6 in place of 1e-10).  Also: a run that
starts with a bond capacity too small for the model regrows and replays
without changing a number, and, where the reference is importable,
``oqupy.MeanFieldTempo(..., backend_config={"backend": "gb300"})`` end to
end reproduces the known answer of the reference's
tests/physics/mean_field_tempo_test.py."""

import numpy as np
import pytest

from tests import golden_cases as gc
from tests import mean_field_cases as mfc
from tests.test_mean_field_cpu import compare, load, run_backend

pytestmark = pytest.mark.gpu


def gpu_backend(name, g, **config):
    from oqupy_gb300.mean_field import GpuMeanFieldTempoBackend
    args = mfc.backend_args(name, g)
    n = len(args["initial_state_list"])
    ones = [np.ones(np.asarray(s).size) for s in args["initial_state_list"]]
    return GpuMeanFieldTempoBackend(
        args["initial_state_list"], args["initial_field"], args["influence_list"],
        args["unitary_transform_list"], args["propagators_list"], args["compute_field"],
        args["compute_field_derivative"], ones, ones, args["dkmax"], args["epsrel"],
        config=config, degeneracy_maps_list=[None] * n, dim_list=None)


@pytest.mark.parametrize("precision", ["complex128", "mixed"])
@pytest.mark.parametrize("name", sorted(mfc.CASES))
def test_gpu_mean_field_matches_reference(name, precision):
    g = load()
    be = gpu_backend(name, g, precision=precision)
    states, fields = run_backend(be, mfc.CASES[name]["nsteps"])
    be.close()
    tol = gc.PARITY_ABS if precision == "complex128" else gc.MIXED_ABS
    bad, worst, fworst = compare(name, states, fields, g, tol)
    print(f"\n{name} {precision}: max trace distance {worst:.2e}, max field error {fworst:.2e}, "
          f"reference spread {g[name + '/envelope'].max():.1e}")
    assert not bad, bad[:5]


def test_gpu_mean_field_regrows_bond_capacity():
    g = load()
    name = "pair_finite_memory"
    n = mfc.CASES[name]["nsteps"]
    big = gpu_backend(name, g, chi_cap=64)
    s_big, f_big = run_backend(big, n)
    big.close()
    small = gpu_backend(name, g, chi_cap=4)
    s_small, f_small = run_backend(small, n)
    grown = small.chi_cap
    small.close()
    assert grown > 4
    for a, b in zip(s_big, s_small):
        np.testing.assert_allclose(b, a, rtol=0, atol=1e-13)
    np.testing.assert_allclose(f_small, f_big, rtol=0, atol=1e-13)


def test_mean_field_tempo_end_to_end():
    from tests.reference_import import import_reference
    oqupy = import_reference()
    mfc.patch_field_hamiltonian_check(oqupy)
    import oqupy_gb300
    case = mfc.CASES["dicke_G"]
    s = case["systems"][0]
    sysf = oqupy.TimeDependentSystemWithField(s["h"])
    mfs = oqupy.MeanFieldSystem([sysf], field_eom=case["field_eom"])
    corr = oqupy.PowerLawSD(alpha=s["alpha"], zeta=s["zeta"], cutoff=s["wc"],
                            cutoff_type=s["cutoff_type"], temperature=s["T"])
    bath = oqupy.Bath(s["coupling"], corr)
    params = oqupy.TempoParameters(dt=case["dt"], tcut=case["tcut"], epsrel=case["epsrel"])
    oqupy_gb300.install(oqupy)
    try:
        mft = oqupy.MeanFieldTempo(mfs, [bath], params, [s["rho0"]], case["field0"],
                                   backend_config={"backend": "gb300"})
        dyn = mft.compute(end_time=1.0, progress_type="silent")
    finally:
        oqupy_gb300.uninstall(oqupy)
    # tests/physics/mean_field_tempo_test.py, case G (4 decimals there)
    rho_g = np.array([[0.6245009 + 3.19373236e-15j, 0.14243496 - 2.19523032e-01j],
                      [0.14243496 + 2.19523032e-01j, 0.3754991 - 2.26692588e-15j]])
    field_g = 0.10602369935009 - 0.46986388684474406j
    assert len(dyn.fields) == 21
    np.testing.assert_almost_equal(dyn.fields[-1], field_g, decimal=4)
    np.testing.assert_almost_equal(dyn.system_dynamics[0].states[-1], rho_g, decimal=4)


@pytest.mark.parametrize("precision", ["complex128", "mixed"])
@pytest.mark.parametrize("name", sorted(mfc.CASES))
def test_gpu_dynamics_with_field_matches_reference(name, precision):
    """compute_dynamics_with_field (system_dynamics.py:184-476) on process
    tensors built on the device from the reference's influences."""
    from oqupy_gb300.mean_field import device_dynamics_with_field
    from oqupy_gb300.pt import PtBatch
    from tests.test_mean_field_cpu import compare_pt, pt_inputs
    g = load()
    case = mfc.CASES[name]
    pts, batches = [], []
    for i, s in enumerate(case["systems"]):
        f, dkmax, tin, tout = pt_inputs(g, name, i)
        d = int(round(np.sqrt(np.asarray(s["rho0"]).size)))
        b = PtBatch([dict(hs_dim=d, num_steps=case["nsteps"], dkmax=dkmax, epsrel=case["epsrel"],
                          influences=g[f"{name}/pt_influences{i}"])],
                    precision=precision, chi_cap=1152 // (d * d))
        b.build()
        batches.append(b)

        class Pt:
            device = (b, 0)
            transform_in = tin
            transform_out = tout
        pts.append(Pt())
    props = [mfc.propagators(s, case["dt"]) for s in case["systems"]]
    times, states, fields = device_dynamics_with_field(
        props, case["field_eom"], case["field0"], pts, [s["rho0"] for s in case["systems"]],
        case["nsteps"], case["dt"])
    for b in batches:
        b.close()
    tol = gc.PARITY_ABS if precision == "complex128" else gc.MIXED_ABS
    bad, worst, fworst = compare_pt(name, states, fields, g, tol)
    print(f"\n{name} {precision} on process tensors: max trace distance {worst:.2e}, "
          f"max field error {fworst:.2e}")
    assert not bad, bad[:5]


def test_dynamics_with_field_end_to_end():
    """The reference's tests/physics/mean_field_tempo_test.py case G on a
    process tensor: pt_tempo_compute with the GPU backend, then
    compute_dynamics_with_field routed to the device sweep."""
    from tests.reference_import import import_reference
    oqupy = import_reference()
    mfc.patch_field_hamiltonian_check(oqupy)
    import oqupy_gb300
    case = mfc.CASES["dicke_G"]
    s = case["systems"][0]
    sysf = oqupy.TimeDependentSystemWithField(s["h"])
    mfs = oqupy.MeanFieldSystem([sysf], field_eom=case["field_eom"])
    corr = oqupy.PowerLawSD(alpha=s["alpha"], zeta=s["zeta"], cutoff=s["wc"],
                            cutoff_type=s["cutoff_type"], temperature=s["T"])
    bath = oqupy.Bath(s["coupling"], corr)
    params = oqupy.TempoParameters(dt=case["dt"], tcut=case["tcut"], epsrel=case["epsrel"])
    oqupy_gb300.install(oqupy)
    try:
        pt = oqupy.pt_tempo_compute(bath, start_time=0.0, end_time=1.0, parameters=params,
                                    backend_config={"backend": "gb300"}, progress_type="silent")
        dyn = oqupy.compute_dynamics_with_field(mfs, initial_field=case["field0"],
                                                process_tensor_list=[pt],
                                                initial_state_list=[s["rho0"]], progress_type="silent")
    finally:
        oqupy_gb300.uninstall(oqupy)
    rho_g = np.array([[0.6245009 + 3.19373236e-15j, 0.14243496 - 2.19523032e-01j],
                      [0.14243496 + 2.19523032e-01j, 0.3754991 - 2.26692588e-15j]])
    field_g = 0.10602369935009 - 0.46986388684474406j
    np.testing.assert_almost_equal(dyn.fields[-1], field_g, decimal=4)
    np.testing.assert_almost_equal(dyn.system_dynamics[0].states[-1], rho_g, decimal=4)
