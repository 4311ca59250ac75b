"""The float64 restatement of the seed network (used to check the GPU
kernels) against central finite differences, on the CPU."""
import numpy as np

import mlp_ref


def test_restatement_backward_matches_finite_differences():
    rng = np.random.default_rng(3)
    layers = [(rng.standard_normal((6, 9)) * 0.4, rng.standard_normal(9) * 0.1),
              (rng.standard_normal((9, 9)) * 0.4, rng.standard_normal(9) * 0.1),
              (rng.standard_normal((9, 9)) * 0.4, rng.standard_normal(9) * 0.1),
              (rng.standard_normal((9, 4)) * 0.4, np.zeros(4))]
    X = rng.standard_normal((13, 6))
    T = rng.standard_normal((13, 4))
    _, g = mlp_ref.loss_and_grads(layers, X, T)
    h = 1e-6
    for li in range(4):
        for which in (0, 1):
            arr = layers[li][which]
            for _ in range(3):
                idx = tuple(rng.integers(0, n) for n in arr.shape)
                old = arr[idx]
                arr[idx] = old + h
                lp, _ = mlp_ref.loss_and_grads(layers, X, T)
                arr[idx] = old - h
                lm, _ = mlp_ref.loss_and_grads(layers, X, T)
                arr[idx] = old
                assert abs((lp - lm) / (2 * h) - g[li][which][idx]) < 1e-7


def test_tf32_reduction():
    x = np.array([1.0 + 2.0 ** -12, 1.0 + 2.0 ** -10, -3.0 - 2.0 ** -11, 1.0 + 2.0 ** -11 + 2.0 ** -20], np.float32)
    assert list(mlp_ref.to_tf32(x, "trunc")) == [1.0, 1.0 + 2.0 ** -10, -3.0, 1.0]
    assert list(mlp_ref.to_tf32(x, "rn")) == [1.0, 1.0 + 2.0 ** -10, -3.0, 1.0 + 2.0 ** -10]
    # ties: 1 + 2^-11 is halfway between 1 and 1 + 2^-10
    t = np.array([1.0 + 2.0 ** -11, -(1.0 + 3 * 2.0 ** -11)], np.float32)
    assert list(mlp_ref.to_tf32(t, "rn")) == [1.0, -(1.0 + 2 * 2.0 ** -10)]
    assert list(mlp_ref.to_tf32(t, "rna")) == [1.0 + 2.0 ** -10, -(1.0 + 2 * 2.0 ** -10)]
