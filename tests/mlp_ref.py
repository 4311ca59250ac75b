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


def to_tf32(x, rounding):
    """float32 values reduced to TF32 (10 explicit mantissa bits): rounding
    'trunc' drops the low 13 bits, 'rn' rounds to nearest even, 'rna' to
    nearest with ties away from zero."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    if rounding == "rn":
        u = u + 0x0FFF + ((u >> 13) & 1)
    elif rounding == "rna":
        u = u + 0x1000
    return (u & 0xFFFFE000).astype(np.uint32).view(np.float32).astype(np.float64)


def forward_tf32(layers, X, rounding):
    """forward() with every matrix product taking TF32 operands (activations
    and weights reduced from float32) and accumulating exactly."""
    a = X
    for i, (W, b) in enumerate(layers):
        z = to_tf32(a, rounding) @ to_tf32(W, rounding) + b
        a = gelu(z) if i < len(layers) - 1 else z
    return a


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
