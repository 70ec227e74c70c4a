"""CPU oracle of the learned sampler's network -- TEST INFRASTRUCTURE ONLY.

Only tests/, the smoke check and the benchmark's CPU leg may import this
module; the product path never does.  The reference has no learned part, so
there is nothing to cite: this is a plain FP64 numpy restatement of the
network the CUDA kernels train (n_in -> 64 -> 64 -> 64 -> n_out, SiLU hidden
activations, linear output, mean squared error over samples and outputs),
with hand-derived backpropagation.  Its gradient is itself checked against
central finite differences in the CPU tests.

Parameter layout (one flat float vector): W1[64][n_in], b1[64], W2[64][64],
b2[64], W3[64][64], b3[64], W4[n_out][64], b4[n_out].
"""
import numpy as np

H = 64


def layout(n_in, n_out):
    sizes = [("W1", (H, n_in)), ("b1", (H,)), ("W2", (H, H)), ("b2", (H,)), ("W3", (H, H)), ("b3", (H,)),
             ("W4", (n_out, H)), ("b4", (n_out,))]
    out, off = {}, 0
    for name, shp in sizes:
        n = int(np.prod(shp))
        out[name] = (off, shp)
        off += n
    return out, off


def unpack(p, n_in, n_out):
    lay, n = layout(n_in, n_out)
    p = np.asarray(p, dtype=np.float64)
    assert p.size == n
    return {k: p[o:o + int(np.prod(s))].reshape(s) for k, (o, s) in lay.items()}


def _sig(z):
    return 1.0 / (1.0 + np.exp(-z))


def forward(p, x, n_in, n_out):
    """Returns the outputs [n, n_out] and the pre-activations (z1, z2, z3)."""
    w = unpack(p, n_in, n_out)
    x = np.asarray(x, dtype=np.float64)
    z1 = x @ w["W1"].T + w["b1"]
    h1 = z1 * _sig(z1)
    z2 = h1 @ w["W2"].T + w["b2"]
    h2 = z2 * _sig(z2)
    z3 = h2 @ w["W3"].T + w["b3"]
    h3 = z3 * _sig(z3)
    y = h3 @ w["W4"].T + w["b4"]
    return y, (z1, z2, z3)


def loss(p, x, t, n_in, n_out):
    y, _ = forward(p, x, n_in, n_out)
    return float(np.mean((y - np.asarray(t, dtype=np.float64)) ** 2))


def loss_grad(p, x, t, n_in, n_out):
    """Mean squared error and its gradient (flat, in the parameter layout)."""
    w = unpack(p, n_in, n_out)
    x = np.asarray(x, dtype=np.float64)
    t = np.asarray(t, dtype=np.float64)
    y, (z1, z2, z3) = forward(p, x, n_in, n_out)
    n = x.shape[0]
    d4 = 2.0 * (y - t) / (n * n_out)

    def dsilu(z):
        s = _sig(z)
        return s * (1.0 + z * (1.0 - s))

    h1, h2, h3 = z1 * _sig(z1), z2 * _sig(z2), z3 * _sig(z3)
    g = {"W4": d4.T @ h3, "b4": d4.sum(0)}
    d3 = (d4 @ w["W4"]) * dsilu(z3)
    g["W3"], g["b3"] = d3.T @ h2, d3.sum(0)
    d2 = (d3 @ w["W3"]) * dsilu(z2)
    g["W2"], g["b2"] = d2.T @ h1, d2.sum(0)
    d1 = (d2 @ w["W2"]) * dsilu(z1)
    g["W1"], g["b1"] = d1.T @ x, d1.sum(0)
    lay, nparam = layout(n_in, n_out)
    flat = np.empty(nparam)
    for k, (o, s) in lay.items():
        flat[o:o + int(np.prod(s))] = g[k].ravel()
    return float(np.mean((y - t) ** 2)), flat


def adam(p, g, m, v, step, lr, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam update (step counts from 1); returns new (p, m, v)."""
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    mh = m / (1 - b1 ** step)
    vh = v / (1 - b2 ** step)
    return p - lr * mh / (np.sqrt(vh) + eps), m, v
