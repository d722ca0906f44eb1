"""The allocation-free TEMPO entry point (otb_tempo_advance_static).

Callers that cannot allocate device memory through this library — a host
framework that owns every device allocation through its own memory pool, or
code running where cudaMalloc is not allowed — allocate the input, MPS,
output and status buffers themselves and call otb_tempo_advance_static,
which takes its working memory from a fixed 1 MiB device array inside the
library (chi_cap * D <= 128).  This test allocates those buffers with torch,
calls the entry point twice in a row through the C ABI, and checks the
states against the handle-based entry point (otb_tempo_create /
otb_tempo_advance) at the complex128 parity bar; that the calls leave the
device's free memory unchanged; the status the entry point reports (steps
completed, bond dimension, and a bond overflow that stops the instance);
and a qutrit case that fills the scratch array's limit.  It lives in its own
file that pytest collects last so that a run stopping at the first failure
has run every other test.
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
                ("mps_bytes", ctypes.c_int64), ("states_out", ctypes.c_void_p),
                ("status_out", ctypes.c_void_p)]


def _mps_bytes(d, dkmax, chi_cap):
    """OTB_TEMPO_STATIC_MPS_BYTES of include/oqupy_gb300.h."""
    D = d * d
    nslots = dkmax + 2
    return 256 + ((nslots * 8 + 255) // 256) * 256 + nslots * chi_cap * D * chi_cap * 16


def _entry():
    from oqupy_gb300 import _native as nat
    f = nat.lib().otb_tempo_advance_static
    f.restype = ctypes.c_int32
    f.argtypes = [ctypes.POINTER(StaticIO), ctypes.c_int32, ctypes.c_void_p]
    return f


def _to_dev(torch, a):
    a = np.ascontiguousarray(np.asarray(a, dtype=np.complex128))
    return torch.from_numpy(a.view(np.float64).copy()).to(torch.device("cuda:0"))


def _run_static(torch, inst, precision, chi, calls):
    """Calls of the entry point with ``calls[k]`` steps each; returns the
    states of all calls, the status after each call, and the device's free
    memory before and after the calls (after one warm-up call on a separate
    zeroed MPS buffer that loads the module)."""
    from oqupy_gb300 import _native as nat
    from oqupy_gb300.tempo import fold_propagators
    d, dkmax = inst["hs_dim"], inst["dkmax"]
    D = d * d
    p1, p2 = fold_propagators(inst["prop1"], inst["prop2"], inst.get("unitary"))
    dev = torch.device("cuda:0")
    infl = _to_dev(torch, np.asarray(inst["influences"])[: dkmax + 1])
    props = _to_dev(torch, np.stack([p1, p2]))
    rho0 = _to_dev(torch, np.asarray(inst["rho0"]).reshape(-1))
    nbytes = _mps_bytes(d, dkmax, chi)
    f = _entry()
    stream = torch.cuda.current_stream().cuda_stream
    outs = [torch.zeros(n * D * 2, dtype=torch.float64, device=dev) for n in calls]
    status = torch.zeros(4, dtype=torch.int32, device=dev)
    warm = torch.zeros(nbytes, dtype=torch.uint8, device=dev)
    mps = torch.zeros(nbytes, dtype=torch.uint8, device=dev)
    io = StaticIO(d, dkmax, inst["epsrel"], chi, precision, infl.data_ptr(), props.data_ptr(),
                  rho0.data_ptr(), warm.data_ptr(), nbytes, outs[0].data_ptr(), status.data_ptr())
    nat.check(f(ctypes.byref(io), 1, ctypes.c_void_p(stream)))
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    io.mps = mps.data_ptr()
    stats = []
    for n, out in zip(calls, outs):
        io.states_out = out.data_ptr()
        nat.check(f(ctypes.byref(io), n, ctypes.c_void_p(stream)))
        torch.cuda.synchronize()
        stats.append(status.cpu().numpy().tolist())
    free1 = torch.cuda.mem_get_info()[0]
    got = [o.cpu().numpy().view(np.complex128).reshape(n, D) for o, n in zip(outs, calls)]
    return got, stats, free0, free1


def _handle_states(inst, precision, chi, n):
    from oqupy_gb300 import TempoBatch
    b = TempoBatch([inst], precision="complex128" if precision == 0 else "mixed",
                   chi_cap=chi, out_cap=n + 1)
    b.advance(n)
    b.check_status()
    return b.states(0, n + 1)[0, 1:]


@pytest.mark.parametrize("precision", [0, 1])
def test_static_entry_point_matches_handle_entry_point(precision):
    torch = pytest.importorskip("torch")
    g = gc.load("config1_spin_boson")
    d, dkmax, chi = g["d"], g["dkmax"], 32
    inst = dict(hs_dim=d, dkmax=dkmax, epsrel=g["epsrel"], influences=g["tempo_infl"][: dkmax + 1],
                prop1=g["prop1"][0], prop2=g["prop2"][0], rho0=g["rho0"], unitary=g["unitary"])
    n1, n2 = 12, 9
    got, stats, free0, free1 = _run_static(torch, inst, precision, chi, [n1, n2])
    got = np.concatenate(got)
    # no device memory taken by the calls themselves
    assert free1 == free0, (free0, free1)
    assert stats[0][:3] == [0, n1, n1] and stats[1][:3] == [0, n2, n1 + n2], stats
    ref = _handle_states(inst, precision, chi, n1 + n2)
    err = max(to.trace_distance(a, c) for a, c in zip(got, ref))
    assert err <= gc.PARITY_ABS, err
    # the reference's own result, for scale
    errs = [to.trace_distance(a, c) for a, c in zip(got, g["tempo_states"][1:])]
    assert not gc.parity_violations([0.0] + errs, g["tempo_envelope"][: n1 + n2 + 1],
                                    gc.PARITY_ABS if precision == 0 else gc.MIXED_ABS)


@pytest.mark.parametrize("precision", [0, 1])
def test_static_entry_point_qutrit_at_the_scratch_limit(precision):
    """d = 3 with chi_cap * D = 126, next to the 128 limit: two steps whose
    bonds fit (parity with the handle path), then a third step whose splits
    fill the scratch array (126 columns) and keep more than 14 singular
    values: reported as a bond overflow, the earlier rows intact."""
    torch = pytest.importorskip("torch")
    from oqupy_gb300 import _native as nat
    g = gc.load("ref_qutrit_C")
    d, dkmax, chi = g["d"], g["dkmax"], 14
    inst = dict(hs_dim=d, dkmax=dkmax, epsrel=g["epsrel"], influences=g["tempo_infl"][: dkmax + 1],
                prop1=g["prop1"][0], prop2=g["prop2"][0], rho0=g["rho0"], unitary=g["unitary"])
    got, stats, free0, free1 = _run_static(torch, inst, precision, chi, [1, 1, 1])
    assert free1 == free0, (free0, free1)
    assert stats[0][:3] == [0, 1, 1] and stats[1][:3] == [0, 1, 2], stats
    assert stats[2][:3] == [nat.OTB_ERR_CHI_OVERFLOW, 0, 2], stats
    ref = _handle_states(inst, precision, 32, 2)
    err = max(to.trace_distance(a, c) for a, c in zip(np.concatenate(got[:2]), ref))
    assert err <= gc.PARITY_ABS, err


def test_static_entry_point_reports_bond_overflow():
    """A bond beyond chi_cap stops the instance: the status says so, the
    completed steps' states are written, and later calls complete nothing."""
    torch = pytest.importorskip("torch")
    from oqupy_gb300 import _native as nat
    g = gc.load("config1_spin_boson")
    d, dkmax, chi = g["d"], g["dkmax"], 4
    inst = dict(hs_dim=d, dkmax=dkmax, epsrel=1e-13, influences=g["tempo_infl"][: dkmax + 1],
                prop1=g["prop1"][0], prop2=g["prop2"][0], rho0=g["rho0"], unitary=g["unitary"])
    got, stats, _, _ = _run_static(torch, inst, 0, chi, [30, 5])
    st, done = stats[0][0], stats[0][1]
    assert st == nat.OTB_ERR_CHI_OVERFLOW, stats
    assert 0 < done < 30
    assert stats[1][:3] == [nat.OTB_ERR_CHI_OVERFLOW, 0, done], stats
    # the rows written before the overflow are the steps' states (the handle
    # path with room for the bonds)
    ref = _handle_states(inst, 0, 32, done)
    err = max(to.trace_distance(a, c) for a, c in zip(got[0][:done], ref))
    assert err <= gc.PARITY_ABS, err


def test_static_entry_point_rejects_oversized_bonds():
    from oqupy_gb300 import _native as nat
    lib = nat.lib()
    f = lib.otb_tempo_advance_static
    f.restype = ctypes.c_int32
    f.argtypes = [ctypes.POINTER(StaticIO), ctypes.c_int32, ctypes.c_void_p]
    io = StaticIO(2, 10, 1e-6, 64, 0, 1, 1, 1, 1, 1 << 30, 1, 1)   # chi_cap * D = 256
    assert f(ctypes.byref(io), 1, None) == nat.OTB_ERR_INVALID_ARG
    assert b"static scratch" in lib.otb_last_error()
