"""CPU checks of the drop-in boundary: the C-ABI library builds, loads and
exports every symbol the header declares; host-side folding is exact."""

import ctypes
import os
import re

import numpy as np
import pytest

from oracle import tempo_oracle as to
from tests import golden_cases as gc

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _header_symbols():
    txt = open(os.path.join(ROOT, "include", "oqupy_gb300.h")).read()
    decl = r"^(?:otb_status|void|const char\s*\*|int32_t)\s+(otb_[a-z0-9_]+)\s*\("
    return sorted(set(re.findall(decl, txt, flags=re.M)))


@pytest.fixture(scope="module")
def lib_path():
    from oqupy_gb300 import build
    return build.build()


def test_library_exports_every_declared_symbol(lib_path):
    lib = ctypes.CDLL(lib_path)
    missing = [s for s in _header_symbols() if not hasattr(lib, s)]
    assert not missing, missing
    assert lib.otb_version() >= 1


def test_binding_covers_header(lib_path):
    from oqupy_gb300 import _native
    declared = set(_header_symbols())
    bound = set(_native.exported_symbols())
    assert bound <= declared
    lib = _native.lib()
    for s in bound:
        assert hasattr(lib, s)


def test_folded_propagators_equal_reference_transform():
    """Folding the dk=0 eigenbasis rotation into the propagators (the GPU
    engine's input convention) reproduces the reference's transformed MPO
    (tempo_backend.py:419-424) on a non-diagonal coupling."""
    from oqupy_gb300.tempo import fold_propagators
    g = gc.load("nondiag_coupling")
    ref, _ = to.tempo_dynamics(g["rho0"], gc.tempo_influence(g), g["unitary"],
                               gc.propagators(g), g["dkmax"], g["epsrel"],
                               g["nsteps"])
    p1, p2 = fold_propagators(g["prop1"][0], g["prop2"][0], g["unitary"])
    D = g["d"] ** 2
    folded, _ = to.tempo_dynamics(g["rho0"], gc.tempo_influence(g),
                                  np.identity(g["d"]), lambda s: (p1, p2),
                                  g["dkmax"], g["epsrel"], g["nsteps"])
    assert to.max_trace_distance(ref, folded) < 1e-12


def test_create_rejects_bad_arguments(lib_path):
    """Argument validation happens on the host before any device work."""
    from oqupy_gb300 import _native as nat
    L = nat.lib()
    cfg = nat.TempoConfig(7, 64, 4, 0)      # bad precision
    arr = (nat.TempoInstance * 1)()
    h = ctypes.c_void_p()
    assert L.otb_tempo_create(ctypes.byref(cfg), 1, arr, ctypes.byref(h)) == nat.OTB_ERR_INVALID_ARG
    assert b"precision" in L.otb_last_error()
    cfg = nat.TempoConfig(0, 500, 4, 0)     # chi_cap too large
    assert L.otb_tempo_create(ctypes.byref(cfg), 1, arr, ctypes.byref(h)) == nat.OTB_ERR_INVALID_ARG
    assert L.otb_tempo_advance(None, 1, None) == nat.OTB_ERR_INVALID_ARG


def test_identity_mask_matches_fold_semantics():
    """The batched identity test used by set_all_propagators agrees with the
    per-instance np.allclose test of fold_propagators, so both setters fold
    exactly the same instances."""
    from oqupy_gb300.tempo import identity_mask
    rng = np.random.default_rng(5)
    us = [None, np.identity(2), np.identity(2) + 5e-9, np.identity(2) + 2e-5,
          np.array([[0, 1], [1, 0]], dtype=complex)]
    for _ in range(10):
        q, _ = np.linalg.qr(rng.normal(size=(2, 2)) + 1j * rng.normal(size=(2, 2)))
        us.append(q)
    want = [u is None or np.allclose(u, np.identity(2)) for u in us]
    assert identity_mask(us, 2).tolist() == want
