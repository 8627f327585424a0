"""FP64 restatement of the surrogate network, its gradients and Adam (oracle only).

Test infrastructure: the GPU training kernels are checked against this module.
There is no counterpart in the reference (the surrogate is new); the maths
follows the standard definitions: dense layers y = x Wᵀ + b, GELU(x) =
x Φ(x) with Φ the standard normal CDF, mean-squared-error loss, and Adam
(Kingma & Ba, 2015) with bias correction.
"""
import math

import numpy as np
from scipy.special import erf


def gelu(x):
    return 0.5 * x * (1.0 + erf(x / math.sqrt(2.0)))


def gelu_grad(x):
    return 0.5 * (1.0 + erf(x / math.sqrt(2.0))) + x * np.exp(-0.5 * x * x) / math.sqrt(2.0 * math.pi)


def init(sizes, seed=0):
    """He-style initialisation: W ~ N(0, 2/fan_in), b = 0."""
    rng = np.random.default_rng(seed)
    params = []
    for fi, fo in zip(sizes[:-1], sizes[1:]):
        params.append((rng.normal(0.0, math.sqrt(2.0 / fi), (fo, fi)), np.zeros(fo)))
    return params


def forward(params, x):
    """Returns the output and the cache of pre-activations and inputs."""
    cache = []
    h = x
    for i, (W, b) in enumerate(params):
        z = h @ W.T + b
        cache.append((h, z))
        h = gelu(z) if i < len(params) - 1 else z
    return h, cache


def loss(params, x, y):
    out, _ = forward(params, x)
    return 0.5 * np.mean(np.sum((out - y) ** 2, axis=1))


def backward(params, x, y):
    """Gradients of loss() with respect to every W and b."""
    out, cache = forward(params, x)
    g = (out - y) / x.shape[0]
    grads = [None] * len(params)
    for i in range(len(params) - 1, -1, -1):
        h, z = cache[i]
        if i < len(params) - 1:
            g = g * gelu_grad(z)
        W, _ = params[i]
        grads[i] = (g.T @ h, g.sum(0))
        g = g @ W
    return grads


def adam_step(params, grads, state, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
    t = state.get("t", 0) + 1
    state["t"] = t
    new = []
    for k, ((W, b), (gW, gb)) in enumerate(zip(params, grads)):
        out = []
        for j, (p, g) in enumerate(((W, gW), (b, gb))):
            m, v = state.get((k, j, "m"), np.zeros_like(p)), state.get((k, j, "v"), np.zeros_like(p))
            m = b1 * m + (1 - b1) * g
            v = b2 * v + (1 - b2) * g * g
            state[(k, j, "m")], state[(k, j, "v")] = m, v
            mh = m / (1 - b1 ** t)
            vh = v / (1 - b2 ** t)
            out.append(p - lr * mh / (np.sqrt(vh) + eps))
        new.append(tuple(out))
    return new
