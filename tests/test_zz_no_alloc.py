"""The allocation-free TEMPO entry point (otb_tempo_advance_static).

Callers that cannot allocate device memory through this library — a host
framework that owns every device allocation through its own memory pool, or
code running where cudaMalloc is not allowed — allocate the input, MPS and
output buffers themselves and call otb_tempo_advance_static, which takes its
working memory from a fixed 1 MiB device array inside the library
(chi_cap * D <= 128).  This test allocates those buffers with torch, calls
the entry point twice in a row through the C ABI, and checks the states
against the handle-based entry point (otb_tempo_create / otb_tempo_advance)
at the complex128 parity bar.  It lives in its own file that pytest collects
last so that a run stopping at the first failure has run every other test.
"""

import ctypes

import numpy as np
import pytest

from oracle import tempo_oracle as to
from tests import golden_cases as gc

pytestmark = pytest.mark.gpu


class StaticIO(ctypes.Structure):
    _fields_ = [("hs_dim", ctypes.c_int32), ("dkmax", ctypes.c_int32),
                ("epsrel", ctypes.c_double), ("chi_cap", ctypes.c_int32),
                ("precision", ctypes.c_int32),
                ("influences", ctypes.c_void_p), ("props", ctypes.c_void_p),
                ("rho0", ctypes.c_void_p), ("mps", ctypes.c_void_p),
                ("mps_bytes", ctypes.c_int64), ("states_out", ctypes.c_void_p)]


def _mps_bytes(d, dkmax, chi_cap):
    """OTB_TEMPO_STATIC_MPS_BYTES of include/oqupy_gb300.h."""
    D = d * d
    nslots = dkmax + 2
    return 256 + ((nslots * 8 + 255) // 256) * 256 + nslots * chi_cap * D * chi_cap * 16


@pytest.mark.parametrize("precision", [0, 1])
def test_static_entry_point_matches_handle_entry_point(precision):
    torch = pytest.importorskip("torch")
    from oqupy_gb300 import TempoBatch, _native as nat
    from oqupy_gb300.tempo import fold_propagators
    g = gc.load("config1_spin_boson")
    d, D, dkmax, chi = g["d"], g["d"] ** 2, g["dkmax"], 32
    n1, n2 = 12, 9
    p1, p2 = fold_propagators(g["prop1"][0], g["prop2"][0], g["unitary"])
    dev = torch.device("cuda:0")

    def to_dev(a):
        a = np.ascontiguousarray(np.asarray(a, dtype=np.complex128))
        return torch.from_numpy(a.view(np.float64).copy()).to(dev)

    infl = to_dev(g["tempo_infl"][: dkmax + 1])
    props = to_dev(np.stack([p1, p2]))
    rho0 = to_dev(g["rho0"].reshape(-1))
    nbytes = _mps_bytes(d, dkmax, chi)
    mps = torch.zeros(nbytes, dtype=torch.uint8, device=dev)
    out1 = torch.zeros(n1 * D * 2, dtype=torch.float64, device=dev)
    out2 = torch.zeros(n2 * D * 2, dtype=torch.float64, device=dev)
    lib = nat.lib()
    f = lib.otb_tempo_advance_static
    f.restype = ctypes.c_int32
    f.argtypes = [ctypes.POINTER(StaticIO), ctypes.c_int32, ctypes.c_void_p]
    io = StaticIO(d, dkmax, g["epsrel"], chi, precision, infl.data_ptr(),
                  props.data_ptr(), rho0.data_ptr(), mps.data_ptr(), nbytes,
                  out1.data_ptr())
    stream = torch.cuda.current_stream().cuda_stream
    nat.check(f(ctypes.byref(io), n1, ctypes.c_void_p(stream)))
    io.states_out = out2.data_ptr()
    nat.check(f(ctypes.byref(io), n2, ctypes.c_void_p(stream)))
    torch.cuda.synchronize()
    got = np.concatenate([out1.cpu().numpy().view(np.complex128).reshape(n1, D),
                          out2.cpu().numpy().view(np.complex128).reshape(n2, D)])
    b = TempoBatch([dict(hs_dim=d, dkmax=dkmax, epsrel=g["epsrel"],
                         influences=g["tempo_infl"][: dkmax + 1],
                         prop1=g["prop1"][0], prop2=g["prop2"][0],
                         rho0=g["rho0"], unitary=g["unitary"])],
                   precision="complex128" if precision == 0 else "mixed",
                   chi_cap=chi, out_cap=n1 + n2 + 1)
    b.advance(n1 + n2)
    b.check_status()
    ref = b.states(0, n1 + n2 + 1)[0, 1:]
    err = max(to.trace_distance(a, c) for a, c in zip(got, ref))
    assert err <= gc.PARITY_ABS, err
    # the reference's own result, for scale
    errs = [to.trace_distance(a, c) for a, c in zip(got, g["tempo_states"][1:])]
    assert not gc.parity_violations([0.0] + errs, g["tempo_envelope"][: n1 + n2 + 1],
                                    gc.PARITY_ABS if precision == 0 else gc.MIXED_ABS)


def test_static_entry_point_rejects_oversized_bonds():
    from oqupy_gb300 import _native as nat
    lib = nat.lib()
    f = lib.otb_tempo_advance_static
    f.restype = ctypes.c_int32
    f.argtypes = [ctypes.POINTER(StaticIO), ctypes.c_int32, ctypes.c_void_p]
    io = StaticIO(2, 10, 1e-6, 64, 0, 1, 1, 1, 1, 1 << 30, 1)   # chi_cap * D = 256
    assert f(ctypes.byref(io), 1, None) == nat.OTB_ERR_INVALID_ARG
    assert b"static scratch" in lib.otb_last_error()
