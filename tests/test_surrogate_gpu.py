"""MLP surrogate on the GPU: tensor-core forward / backward against the CPU
oracle, training on the GPU, and screening with TEMPO fallback."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _mlp(sizes, seed=0):
    from oqupy_gb300.surrogate import Mlp
    return Mlp(sizes, seed=seed)


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


@pytest.mark.parametrize("sizes,batch", [([5, 64, 48, 30], 37), ([5, 512, 512, 1500], 256),
                                         ([5, 160, 130, 129, 200], 131)])
def test_gradients_match_oracle(sizes, batch):
    import torch
    from oracle import mlp_oracle as mo
    net = _mlp(sizes, seed=len(sizes))
    rng = np.random.default_rng(batch)
    for b in net.b:                                  # non-zero biases
        b.copy_(torch.tensor(0.1 * rng.normal(size=b.shape[0]), dtype=torch.float32))
    X = rng.uniform(-1, 1, size=(batch, sizes[0])).astype(np.float32)
    T = rng.normal(size=(batch, sizes[-1])).astype(np.float32)
    Xd = torch.tensor(X, device=net.dev)
    Td = torch.tensor(T, device=net.dev)
    loss, gW, gb = net.loss_and_grads(Xd, Td)
    net.check_errors()
    Ws = [w.cpu().double().numpy() for w in net.W]
    bs = [b.cpu().double().numpy() for b in net.b]
    rW, rb, rloss = mo.backward(Ws, bs, X.astype(np.float64), T.astype(np.float64))
    assert abs(loss.item() / T.size - rloss) <= 1e-3 * rloss
    for l in range(len(Ws)):
        # bf16 storage of activations: an occasional rounding flip between
        # the GPU's and numpy's GELU moves an element by one bf16 ulp
        assert _rel(gW[l].cpu().double().numpy(), rW[l]) < 1e-2, l
        assert _rel(gb[l].cpu().double().numpy(), rb[l]) < 1e-2, l
    Y = net.forward(Xd).cpu().double().numpy()
    rY, _, _ = mo.forward(Ws, bs, X.astype(np.float64))
    assert _rel(Y, rY) < 1e-2


def test_training_lowers_loss_on_smooth_targets():
    import torch
    net = _mlp([5, 256, 256, 96], seed=3)
    rng = np.random.default_rng(0)
    X = rng.uniform(-1, 1, size=(1024, 5)).astype(np.float32)
    t = np.linspace(0, 4, 32)
    T = np.concatenate([np.cos((1 + X[:, :1]) * t) * np.exp(-(X[:, 1:2] + 1.2) * t / 4),
                        np.sin((1.5 + X[:, 2:3]) * t), X[:, 3:4] * X[:, 4:5] + 0 * t], axis=1)
    Xd, Td = torch.tensor(X, device=net.dev), torch.tensor(T.astype(np.float32), device=net.dev)
    losses = []
    for it in range(300):
        idx = torch.tensor(rng.integers(0, 1024, size=128), device=net.dev)
        loss, gW, gb = net.loss_and_grads(Xd[idx], Td[idx])
        net.step(gW, gb, lr=2e-3)
        if it % 50 == 0 or it == 299:
            losses.append(loss.item() / (128 * 96))
    net.check_errors()
    assert losses[-1] < 0.05 * losses[0], losses


def test_screening_falls_back_outside_budget_and_box():
    """Small TEMPO-generated training set: out-of-box points and regions whose
    validation error exceeds the budget are answered by TEMPO (identical to a
    direct solve); the rest by the network, within the calibrated error."""
    from oqupy_gb300.surrogate import Surrogate, sample_params, tempo_bloch
    nsteps = 60
    sur = Surrogate(nsteps=nsteps, hidden=(256, 256, 256), dkmax=5, bins=2, seed=1)
    Ptr = sample_params(768, 10)
    Ytr, _ = tempo_bloch(Ptr, nsteps, dkmax=5)
    Pva = sample_params(256, 11)
    Yva, _ = tempo_bloch(Pva, nsteps, dkmax=5)
    losses = sur.fit(Ptr, Ytr, epochs=60, batch=128, lr=2e-3)
    assert losses[-1] < 0.2 * losses[0]
    err = sur.calibrate(Pva, Yva)
    budget = float(np.sort(sur.err_map)[1])          # at least two trusted regions
    Pte = sample_params(200, 12)
    Pte[:5, 0] = 0.9                                  # alpha outside the box
    out, fb, tim = sur.screen(Pte, budget=budget)
    assert fb[:5].all()
    assert (~fb).sum() > 0
    ref, _ = tempo_bloch(Pte, nsteps, dkmax=5)
    np.testing.assert_allclose(out[fb], ref[fb], atol=1e-12)
    trusted_err = np.abs(out[~fb] - ref[~fb]).max(axis=(1, 2))
    # calibrated on held-out points of the same regions: allow a margin
    assert np.quantile(trusted_err, 0.9) <= 2.0 * budget
    assert tim["points_per_s"] > 0


def test_device_baseline_matches_host_precession():
    """otb_mlp_bloch_free_add against the float64 host baseline (float32
    phases up to ~55 rad: tolerance 2e-5)."""
    import torch
    from oqupy_gb300 import _native as nat
    from oqupy_gb300.surrogate import free_bloch, sample_params
    P = sample_params(300, 21)
    nsteps, dt = 500, 0.05
    y = torch.zeros((len(P), 3 * nsteps), dtype=torch.float32, device="cuda")
    oe = torch.tensor(P[:, 3:5], dtype=torch.float32, device="cuda")
    nat.check(nat.lib().otb_mlp_bloch_free_add(y.data_ptr(), oe.data_ptr(), len(P), nsteps, dt, None))
    got = y.cpu().numpy().reshape(len(P), 3, nsteps)
    np.testing.assert_allclose(got, free_bloch(P, nsteps, dt), atol=2e-5)


def test_screening_gain_over_tempo_only():
    """What the trained network gains over TEMPO-only screening of the same
    points: at a budget met by part of the box (the calibrated error of the
    two best of four alpha x T regions), the points answered by the network
    skip their TEMPO solve.  Points/s of screening with fallback against
    TEMPO alone, and the error after fallback against the direct solve."""
    import time
    from oqupy_gb300.surrogate import Surrogate, sample_params, tempo_bloch
    nsteps = 60
    sur = Surrogate(nsteps=nsteps, hidden=(256, 256, 256), dkmax=5, bins=2, seed=1)
    Ptr = sample_params(768, 10)
    Ytr, _ = tempo_bloch(Ptr, nsteps, dkmax=5)
    Pva = sample_params(256, 11)
    Yva, _ = tempo_bloch(Pva, nsteps, dkmax=5)
    sur.fit(Ptr, Ytr, epochs=60, batch=128, lr=2e-3)
    sur.calibrate(Pva, Yva)
    budget = float(np.sort(sur.err_map)[1])
    Pte = sample_params(512, 13)
    tempo_bloch(Pte[:8], nsteps, dkmax=5)                 # warm-up
    t0 = time.perf_counter()
    ref, _ = tempo_bloch(Pte, nsteps, dkmax=5)
    t_tempo = time.perf_counter() - t0
    sur.screen(Pte[:8], budget=budget)                    # warm-up
    out, fb, tim = sur.screen(Pte, budget=budget)
    gain = tim["points_per_s"] / (len(Pte) / t_tempo)
    err = np.abs(out - ref).max(axis=(1, 2))
    print(f"budget {budget:.2e}: network answers {(~fb).mean():.0%} of the points, "
          f"{tim['points_per_s']:.0f} vs {len(Pte) / t_tempo:.0f} points/s TEMPO-only "
          f"(gain {gain:.2f}x); error after fallback p90 {np.quantile(err, 0.9):.2e}, "
          f"max {err.max():.2e}")
    assert (~fb).mean() > 0.2
    assert gain > 1.0
    assert np.quantile(err, 0.9) <= 2.0 * budget
