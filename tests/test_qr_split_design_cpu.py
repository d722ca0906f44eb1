"""The QR-preconditioned bond split of both precision forms, restated in
numpy (exact SVD in place of the one-sided Jacobi) and checked against the
plain truncated SVD: pivoted Householder QR without column exchanges,
stopped once the remaining block falls below delta |R_00| (mixed form:
min(1e-3 epsrel, 1e-9); complex128 form: 1e-14), the SVD of the k rows of
R, the dropped block's squared norm added to the tail sums.  The kept rank
must be the full SVD's and the reconstruction error its truncation error."""
import numpy as np

from oracle import tempo_oracle as to


def qr_truncated_split(A, epsrel, delta=None):
    """A (R x N, R >= N) -> (U, S V^H, kept, k) as the kernel forms them
    (oqupy_gb300/csrc/qr.cuh): pivoted Householder QR without column
    exchanges (colstep[j] = step at which column j was chosen, N = never),
    partial norms double-buffered by step parity, the diagonal stored one
    step late, Z[q, i] = conj(R[i, q]) for colstep[q] >= i, then the SVD of
    Z (exact here, one-sided Jacobi on the GPU); U = A W / s^2 with
    W = A^H U S."""
    X = np.array(A, dtype=np.complex128)
    R, N = X.shape
    if delta is None:
        delta = min(1e-3 * epsrel, 1e-9)
    colstep = np.full(N, N)
    cn = [np.sum(np.abs(X) ** 2, axis=0), np.zeros(N)]
    k, tail2, r00 = N, 0.0, None
    pend = None
    for i in range(N):
        cur, nxt = cn[i & 1], cn[(i + 1) & 1]
        avail = np.flatnonzero(colstep >= i)
        p = int(avail[np.argmax(cur[avail])])          # lowest index on ties
        tot = float(cur[avail].sum())
        if i == 0:
            r00 = float(cur[p])
        elif tot < delta * delta * r00:
            k, tail2 = i, tot
            break
        colstep[p] = i
        if pend is not None:                            # previous diagonal
            X[i - 1, pend[0]] = pend[1]
        x = X[i:, p]
        nrm = np.linalg.norm(x)
        a0 = abs(x[0])
        e = x[0] / a0 if a0 > 0 else 1.0
        v = x.copy()
        v[0] = e * (a0 + nrm)
        beta = 1.0 / (nrm * (nrm + a0)) if nrm > 0 else 0.0
        pend = (p, -e * nrm)
        for j in range(N):
            if j == p or colstep[j] < i:
                continue
            w = np.vdot(v, X[i:, j])
            X[i:, j] -= beta * v * w
            nxt[j] = np.sum(np.abs(X[i + 1:, j]) ** 2)
    if pend is not None:
        X[k - 1, pend[0]] = pend[1]
    Z = np.zeros((N, k), dtype=np.complex128)
    for i in range(k):
        for q in range(N):
            if colstep[q] >= i:
                Z[q, i] = np.conj(X[i, q])
    _last_Z["Z"], _last_Z["tail2"] = Z.copy(), tail2
    u, s, vh = np.linalg.svd(Z, full_matrices=False)
    W = u * s                                        # Z V: orthogonal columns
    cum = tail2 + np.cumsum((s ** 2)[::-1])[::-1]
    kept = max(1, int(np.sum(np.sqrt(cum) > epsrel * s[0])))
    U = A @ W[:, :kept] / s[:kept] ** 2
    return U, W[:, :kept].conj().T, kept, k


def householder_unit(Z):
    """Unpivoted Householder QR of Z (M x K, M >= K) as the kernel stores it:
    R in the upper triangle, below the diagonal the reflector w_i scaled to
    w_i[i] = 1, tau_i real with H_i = I - tau_i w_i w_i^H (the kernel writes
    the scaled column one step late, which changes no number)."""
    Z = np.array(Z, dtype=np.complex128)
    M, K = Z.shape
    tau = np.zeros(K)
    for i in range(K):
        x = Z[i:, i].copy()
        nrm = np.linalg.norm(x)
        a0 = abs(x[0])
        e = x[0] / a0 if a0 > 0 else 1.0
        v0 = e * (a0 + nrm)
        beta = 1.0 / (nrm * (nrm + a0)) if nrm > 0 else 0.0
        v = x.copy()
        v[0] = v0
        for j in range(i + 1, K):
            w = np.vdot(v, Z[i:, j])
            Z[i:, j] -= beta * v * w
        tau[i] = beta * abs(v0) ** 2
        Z[i + 1:, i] = x[1:] / v0 if nrm > 0 else 0.0
        Z[i, i] = -e * nrm
    return Z, tau


def apply_q(Zf, tau, Y):
    """Q Y with Q = H_0 H_1 ... H_{K-1} (reflectors applied last-first)."""
    M, K = Zf.shape
    Y = np.array(Y, dtype=np.complex128)
    for i in reversed(range(K)):
        w = np.concatenate([[1.0], Zf[i + 1:, i]])
        s = w.conj() @ Y[i:, :]
        Y[i:, :] -= tau[i] * np.outer(w, s)
    return Y


def lq_reduced_split(A, epsrel, delta=None):
    """The kernel's branch for k <= N / 2: Z = Q2 [R2; 0] by a second
    (unpivoted) Householder QR, the SVD of the k x k R2 (exact here, one-sided
    Jacobi on the GPU), the rank decision from R2's singular values, and
    W = Q2 [W2; 0] formed for the kept columns only."""
    U, C, kept, k = qr_truncated_split(A, epsrel, delta)      # the QR and Z
    N = A.shape[1]
    Zfull, tail2 = _last_Z["Z"], _last_Z["tail2"]
    Zf, tau = householder_unit(Zfull)
    R2 = np.triu(Zf[:k, :k])
    u, s, vh = np.linalg.svd(R2)
    W2 = u * s                                          # R2 V: orthogonal columns
    cum = tail2 + np.cumsum((s ** 2)[::-1])[::-1]
    kk = max(1, int(np.sum(np.sqrt(cum) > epsrel * s[0])))
    Y = np.zeros((N, kk), dtype=np.complex128)
    Y[:k] = W2[:, :kk]
    W = apply_q(Zf, tau, Y)                             # = Z V[:, :kk] = A^H U S
    Uk = A @ W / s[:kk] ** 2
    return Uk, W.conj().T, kk, k


_last_Z = {}


def _check(theta, epsrel=1e-6, delta=None):
    A = theta.conj().T if theta.shape[1] > theta.shape[0] else theta
    U, C, kept, k = qr_truncated_split(A, epsrel, delta)
    s = np.linalg.svd(A, compute_uv=False)
    assert kept == to.truncation_rank(s, epsrel)
    err = np.linalg.norm(U @ C - A) / np.linalg.norm(A)
    trunc = np.sqrt(np.sum(s[kept:] ** 2)) / np.linalg.norm(A)
    assert err <= 1.01 * trunc + 1e-12
    return k, A.shape[1]


def test_random_graded_matrices():
    rng = np.random.default_rng(0)
    for _ in range(30):
        m, n = rng.integers(8, 60, size=2)
        r = min(m, n)
        sv = np.sort(10.0 ** (-rng.uniform(0, 14, size=r)))[::-1]
        U = np.linalg.qr(rng.normal(size=(m, r)) + 1j * rng.normal(size=(m, r)))[0]
        V = np.linalg.qr(rng.normal(size=(n, r)) + 1j * rng.normal(size=(n, r)))[0]
        _check((U * sv) @ V.conj().T)
        _check((U * sv) @ V.conj().T, delta=1e-14)


def test_rank_deficient_and_tied_columns():
    """Exactly repeated columns, zero columns and ties in the pivot search
    (the lowest index wins) leave the kept rank and the reconstruction as
    the full SVD's."""
    rng = np.random.default_rng(1)
    base = rng.normal(size=(24, 6)) + 1j * rng.normal(size=(24, 6))
    A = np.concatenate([base, base, np.zeros((24, 3))], axis=1)
    for delta in (None, 1e-14):
        _check(A, delta=delta)


def test_captured_tempo_bond_splits():
    """Every zip-up and sweep split of 40 TEMPO steps of a strongly coupled
    spin-boson instance (matrices captured from the oracle)."""
    from oqupy_gb300 import bath
    sx = np.array([[0, 1], [1, 0]], dtype=complex)
    sz = np.diag([1.0, -1.0]).astype(complex)
    infl, U = bath.influences(0.4, 1.0, 8.0, "exponential", 3.0, 0.05, 20, 0.5 * sz)
    p1, p2 = bath.half_step_propagators(0.75 * sx, 0.05)
    captured = []
    orig = to.np.linalg.svd

    def rec(a, *args, **kw):
        if min(a.shape) >= 8:
            captured.append(np.array(a))
        return orig(a, *args, **kw)

    to.np.linalg.svd = rec
    try:
        o = to.TempoOracle(np.array([1, 0, 0, 0], dtype=complex), lambda dk: infl[dk] if dk >= 0 else None,
                           U, lambda s: (p1, p2), np.ones(4), np.ones(4), 20, 1e-6)
        o.initialize()
        for _ in range(40):
            o.compute_step()
    finally:
        to.np.linalg.svd = orig
    assert len(captured) > 100
    ks = [_check(th) for th in captured[::5]]
    # the rank-revealing cut shrinks the Jacobi problem on these matrices
    assert np.mean([k / n for k, n in ks]) < 0.95


def test_second_qr_reduction_of_the_jacobi_operand():
    """k <= N / 2: the Jacobi runs on the k x k R2 of Z = Q2 [R2; 0]; kept
    rank and reconstruction equal the full SVD's."""
    rng = np.random.default_rng(5)
    n_lq = 0
    for _ in range(20):
        m, n = rng.integers(24, 90, size=2)
        r = min(m, n)
        # fast geometric decay (TEMPO bond spectra): about half the values
        # above the mixed form's QR cut
        sv = 10.0 ** (-np.linspace(0, rng.uniform(18, 30), r))
        U = np.linalg.qr(rng.normal(size=(m, r)) + 1j * rng.normal(size=(m, r)))[0]
        V = np.linalg.qr(rng.normal(size=(n, r)) + 1j * rng.normal(size=(n, r)))[0]
        theta = (U * sv) @ V.conj().T
        A = theta.conj().T if theta.shape[1] > theta.shape[0] else theta
        for delta in (None, 1e-14):
            Uk, C, kept, k = lq_reduced_split(A, 1e-6, delta)
            if 2 * k > A.shape[1]:
                continue
            n_lq += 1
            s = np.linalg.svd(A, compute_uv=False)
            assert kept == to.truncation_rank(s, 1e-6)
            err = np.linalg.norm(Uk @ C - A) / np.linalg.norm(A)
            trunc = np.sqrt(np.sum(s[kept:] ** 2)) / np.linalg.norm(A)
            assert err <= 1.01 * trunc + 1e-12
    assert n_lq > 10
