"""NumPy float64 restatement of the seed network (test infrastructure):
forward and manual backward of input -> 3 x (Linear, GELU) -> Linear with the
mean-squared-error loss, used to check the GPU's FP32 kernels."""
import numpy as np

K = np.sqrt(2.0 / np.pi)
A = 0.044715


def gelu(z):
    return 0.5 * z * (1.0 + np.tanh(K * (z + A * z ** 3)))


def gelu_grad(z):
    t = np.tanh(K * (z + A * z ** 3))
    return 0.5 * (1.0 + t) + 0.5 * z * (1.0 - t * t) * K * (1.0 + 3.0 * A * z * z)


def forward(layers, X):
    acts, zs = [X], []
    a = X
    for i, (W, b) in enumerate(layers):
        z = a @ W + b
        zs.append(z)
        a = gelu(z) if i < len(layers) - 1 else z
        acts.append(a)
    return a, acts, zs


def loss_and_grads(layers, X, T):
    Y, acts, zs = forward(layers, X)
    n = Y.size
    loss = float(np.sum((Y - T) ** 2) / n)
    d = 2.0 * (Y - T) / n
    grads = [None] * len(layers)
    for i in range(len(layers) - 1, -1, -1):
        W, b = layers[i]
        grads[i] = (acts[i].T @ d, d.sum(axis=0))
        if i > 0:
            d = (d @ W.T) * gelu_grad(zs[i - 1])
    return loss, grads


def flatten(grads):
    return np.concatenate([np.concatenate([g[0].ravel(), g[1].ravel()]) for g in grads])
