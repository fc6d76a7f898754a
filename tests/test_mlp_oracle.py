"""The NumPy oracle of the acoustic-cycle surrogate, checked on the CPU:
BF16 rounding against hand-computed values, the backward pass against
central finite differences (FP64, no rounding; relative error <= 1e-6), and
the feature layout against direct indexing."""
import numpy as np

from oracle import mlp_oracle as mo


def test_bf16_rounding_known_values():
    x = np.array([1.0, 1 + 2.0 ** -8, 1 + 3 * 2.0 ** -8, -2.5, 3.0e-3, 65504.0, 1 + 2.0 ** -7 + 2.0 ** -9],
                 np.float32)
    want = np.array([1.0, 1.0, 1 + 2.0 ** -6, -2.5, 0.0030059814453125, 65536.0, 1 + 2.0 ** -7], np.float32)
    assert np.array_equal(mo.bf16(x), want)


def _params(rng, sizes):
    return [(rng.normal(0, 0.5, (o, i)), rng.normal(0, 0.1, o)) for i, o in zip(sizes[:-1], sizes[1:])]


def test_backward_matches_finite_differences():
    rng = np.random.default_rng(0)
    sizes = (7, 5, 6, 4, 3)
    P = _params(rng, sizes)
    X = rng.normal(size=(9, 7))
    T = rng.normal(size=(9, 3))
    m = 2  # the last output is padding and carries no loss
    _, grads = mo.backward(P, X, T, m, rnd=False)

    def mse(PP):
        Y, _, _ = mo.forward(PP, X, rnd=False)
        return np.sum((Y[:, :m] - T[:, :m]) ** 2) / (X.shape[0] * m)

    eps = 1e-6
    for l in range(4):
        for which in (0, 1):
            a = P[l][which]
            num = np.zeros_like(a)
            for idx in np.ndindex(a.shape):
                old = a[idx]
                a[idx] = old + eps
                fp = mse(P)
                a[idx] = old - eps
                fm = mse(P)
                a[idx] = old
                num[idx] = (fp - fm) / (2 * eps)
            g = grads[l][which]
            assert np.linalg.norm(g - num) <= 1e-6 * max(np.linalg.norm(num), 1e-12), (l, which)


def test_feature_layout():
    rng = np.random.default_rng(1)
    kz, ni, nj = 3, 4, 5
    st = {f: rng.normal(size=(kz, ni, nj)) for f in ("u", "v", "pai", "tetav")}
    st["w"] = rng.normal(size=(kz + 1, ni, nj))
    X = mo.features(st)
    assert X.shape == (ni * nj, 45 * kz)
    flds = (st["u"], st["v"], st["w"][1:], st["pai"], st["tetav"])
    for (i, j) in ((0, 0), (3, 4), (2, 1)):
        c = j + nj * i
        for nb in range(9):
            di, dj = nb // 3 - 1, nb % 3 - 1
            for f in range(5):
                for k in range(kz):
                    assert X[c, (f * kz + k) * 9 + nb] == flds[f][k, (i + di) % ni, (j + dj) % nj]
