"""The MLP oracle's backward pass against central finite differences (exact
float64 arithmetic), and its bfloat16 rounding against torch's."""
import numpy as np
import pytest

from oracle import mlp_oracle as mo


def _net(sizes, seed):
    rng = np.random.default_rng(seed)
    Ws = [rng.normal(size=(o, i)) / np.sqrt(i) for i, o in zip(sizes[:-1], sizes[1:])]
    bs = [0.1 * rng.normal(size=o) for o in sizes[1:]]
    return Ws, bs


def test_oracle_gradients_match_finite_differences():
    sizes = [5, 7, 6, 4]
    Ws, bs = _net(sizes, 0)
    rng = np.random.default_rng(1)
    X = rng.uniform(-1, 1, size=(9, 5))
    T = rng.normal(size=(9, 4))
    gW, gb, _ = mo.backward(Ws, bs, X, T, rounding=False)

    def loss():
        Y, _, _ = mo.forward(Ws, bs, X, rounding=False)
        return np.mean((Y - T) ** 2)

    h = 1e-6
    for l in range(len(Ws)):
        for idx in [(0, 0), (1, 2), (Ws[l].shape[0] - 1, Ws[l].shape[1] - 1)]:
            old = Ws[l][idx]
            Ws[l][idx] = old + h
            lp = loss()
            Ws[l][idx] = old - h
            lm = loss()
            Ws[l][idx] = old
            assert abs((lp - lm) / (2 * h) - gW[l][idx]) < 1e-7
        for j in [0, bs[l].size - 1]:
            old = bs[l][j]
            bs[l][j] = old + h
            lp = loss()
            bs[l][j] = old - h
            lm = loss()
            bs[l][j] = old
            assert abs((lp - lm) / (2 * h) - gb[l][j]) < 1e-7


def test_bf16_rounding_matches_torch():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(3)
    x = np.concatenate([rng.normal(size=4000) * 10.0 ** rng.integers(-6, 6, size=4000),
                        [0.0, -0.0, 1.0, 65504.0, 1e-40]]).astype(np.float32)
    ref = torch.tensor(x).to(torch.bfloat16).to(torch.float64).numpy()
    np.testing.assert_array_equal(mo.bf16(x), ref)
