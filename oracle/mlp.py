"""CPU oracle of the learned warm start (spinterps_gb300/csrc/spi_mlp.cu).

TEST INFRASTRUCTURE ONLY: numpy (FP64) restatements of the features, the
network's forward pass, its loss and its analytic gradient, against which
the GPU kernels are checked. The warm start has no counterpart in the
reference; the layout and loss are this project's own (documented in
spi_mlp.cu): in -> h1 (tanh) -> h2 (tanh) -> out, parameters packed as
W1[in][h1], b1, W2[h1][h2], b2, W3[h2][out], b3; loss = mean over the batch
of softmax cross-entropy on the first n_class outputs plus wp/2 * sum of
masked squared errors on the rest.
"""
import numpy as np


def offsets(nin, h1, h2, out):
    o = {}
    k = 0
    for name, size in (("W1", nin * h1), ("b1", h1), ("W2", h1 * h2), ("b2", h2),
                       ("W3", h2 * out), ("b3", out)):
        o[name] = (k, k + size)
        k += size
    o["n"] = k
    return o


def unpack(params, nin, h1, h2, out):
    o = offsets(nin, h1, h2, out)
    p = np.asarray(params, dtype=np.float64)
    return (p[o["W1"][0]:o["W1"][1]].reshape(nin, h1), p[o["b1"][0]:o["b1"][1]],
            p[o["W2"][0]:o["W2"][1]].reshape(h1, h2), p[o["b2"][0]:o["b2"][1]],
            p[o["W3"][0]:o["W3"][1]].reshape(h2, out), p[o["b3"][0]:o["b3"][1]])


def forward(params, X, dims):
    W1, b1, W2, b2, W3, b3 = unpack(params, *dims)
    H1 = np.tanh(X @ W1 + b1)
    H2 = np.tanh(H1 @ W2 + b2)
    return H1, H2, H2 @ W3 + b3


def loss_grad(params, X, cls, yp, mask, wp, dims, n_class):
    X = np.asarray(X, dtype=np.float64)
    B = X.shape[0]
    W1, b1, W2, b2, W3, b3 = unpack(params, *dims)
    H1, H2, O = forward(params, X, dims)
    logit = O[:, :n_class]
    mx = logit.max(1, keepdims=True)
    e = np.exp(logit - mx)
    se = e.sum(1, keepdims=True)
    prob = e / se
    loss = (np.log(se[:, 0]) + mx[:, 0] - logit[np.arange(B), cls])
    r = O[:, n_class:] - yp
    loss = loss + wp * 0.5 * (mask * r * r).sum(1)
    dO = np.zeros_like(O)
    dO[:, :n_class] = prob
    dO[np.arange(B), cls] -= 1
    dO[:, n_class:] = wp * mask * r
    dO /= B
    gW3 = H2.T @ dO
    gb3 = dO.sum(0)
    dH2 = (dO @ W3.T) * (1 - H2 ** 2)
    gW2 = H1.T @ dH2
    gb2 = dH2.sum(0)
    dH1 = (dH2 @ W2.T) * (1 - H1 ** 2)
    gW1 = X.T @ dH1
    gb1 = dH1.sum(0)
    grad = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3.ravel(), gb3])
    return loss.mean(), grad


def features(x, y, z, nb=20):
    """Semivariance in nb equal-width lag bins up to half the bounding-box
    diagonal, divided by the variance (0 for empty bins)."""
    x, y, z = (np.asarray(a, dtype=np.float64) for a in (x, y, z))
    i, j = np.tril_indices(z.size, -1)
    h = np.sqrt((x[i] - x[j]) ** 2 + (y[i] - y[j]) ** 2)
    hmax = 0.5 * np.hypot(np.ptp(x), np.ptp(y))
    keep = h < hmax
    b = np.minimum((h[keep] / hmax * nb).astype(int), nb - 1)
    dz2 = (z[i] - z[j])[keep] ** 2
    s = np.bincount(b, weights=dz2, minlength=nb)
    c = np.bincount(b, minlength=nb).astype(float)
    var = z.var()
    out = np.zeros(nb)
    ok = (c > 0) & (var > 0)
    out[ok] = s[ok] / (2 * c[ok]) / var
    return out
