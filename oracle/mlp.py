"""Test infrastructure: FP64 numpy restatement of the slip-rate warm-start network (5 -> 64 -> 64 -> 1,
tanh) and of the gradient of its mean-squared training loss, the checker of the GPU training kernels.

The network has no counterpart in the reference: its rate-and-state solve starts every Newton
sequence from the previous slip rate (src/DynamicRupture/FrictionLaws/CpuImpl/RateAndState.h:339-417, first guess :354-356).
Parameter order W1 [64][5], b1 [64], W2 [64][64], b2 [64], W3 [64], b3; samples [n][6] = (normal
stress sn, |shear traction| tau, state variable psi, a, b, log10 slip rate).  The network sees the
fixed features (tau / (|sn| a), psi / a, ln(|sn| a), a, b) (|sn| a floored at 1 Pa) and predicts
r = ln(2 V0) + tau / (|sn| a) - psi / a - ln V - softplus(tau / (|sn| a) - psi / a - ln(|sn| a));
norm [16] = feature shifts [5], feature scales [5],
output shift, output scale, ln(2 V0), three zeros.
"""
import numpy as np

H = 64
NUM_PARAMS = H * 5 + H + H * H + H + H + 1


def unpack(p):
    p = np.asarray(p, np.float64)
    o = 0
    W1 = p[o:o + H * 5].reshape(H, 5); o += H * 5
    b1 = p[o:o + H]; o += H
    W2 = p[o:o + H * H].reshape(H, H); o += H * H
    b2 = p[o:o + H]; o += H
    W3 = p[o:o + H]; o += H
    return W1, b1, W2, b2, W3, p[o]


LN10 = np.log(10.0)


def features(samples):
    s = np.asarray(samples, np.float64)
    sn, tau, psi, a, b = (s[:, i] for i in range(5))
    an = np.maximum(np.abs(sn) * a, 1.0)
    return np.stack([tau / an, psi / a, np.log(an), a, b], axis=1)


def baseline(f):
    """softplus(z), z = tau / (|sn| a) - psi / a - ln(|sn| a): the fixed part of the output."""
    z = f[:, 0] - f[:, 1] - f[:, 2]
    return np.where(z > 30.0, z, np.log1p(np.exp(np.minimum(z, 30.0))))


def target(samples, ln2v0):
    f = features(samples)
    return ln2v0 + f[:, 0] - f[:, 1] - LN10 * np.asarray(samples, np.float64)[:, 5] - baseline(f)


def usable(samples):
    """Samples the network applies to: |sn| a > 1 Pa and tau < 500 |sn| a."""
    s = np.asarray(samples, np.float64)
    an = np.abs(s[:, 0]) * s[:, 3]
    return (an > 1.0) & (s[:, 1] < 500.0 * an)


def _inputs(norm, samples):
    norm = np.asarray(norm, np.float64)
    return (features(samples) - norm[:5]) * norm[5:10]


def forward(params, norm, samples):
    """Normalised output y and hidden activations for samples [n][6]."""
    W1, b1, W2, b2, W3, b3 = unpack(params)
    x = _inputs(norm, samples)
    h1 = np.tanh(x @ W1.T + b1)
    h2 = np.tanh(h1 @ W2.T + b2)
    return h2 @ W3 + b3, x, h1, h2


def predict(params, norm, samples):
    """log10 slip rate predicted for each sample."""
    norm = np.asarray(norm, np.float64)
    f = features(samples)
    t = forward(params, norm, samples)[0] * norm[11] + norm[10]
    return (norm[12] + f[:, 0] - f[:, 1] - baseline(f) - t) / LN10


def loss_and_grad(params, norm, samples):
    """Mean-squared loss of y against the normalised target and its gradient (packed like params)."""
    norm = np.asarray(norm, np.float64)
    W1, b1, W2, b2, W3, b3 = unpack(params)
    y, x, h1, h2 = forward(params, norm, samples)
    t = (target(samples, norm[12]) - norm[10]) / norm[11]
    n = len(y)
    e = y - t
    dy = 2.0 * e / n
    d2 = dy[:, None] * W3[None, :] * (1.0 - h2 * h2)
    d1 = (d2 @ W2) * (1.0 - h1 * h1)
    g = np.concatenate([(d1.T @ x).ravel(), d1.sum(0), (d2.T @ h1).ravel(), d2.sum(0), dy @ h2, [dy.sum()]])
    return float(np.mean(e * e)), g


def glorot(seed=0):
    """Seeded parameters for tests (uniform Glorot limits, small random biases)."""
    rng = np.random.default_rng(seed)
    parts = [rng.uniform(-1, 1, H * 5) * np.sqrt(6 / (5 + H)), rng.uniform(-0.1, 0.1, H),
             rng.uniform(-1, 1, H * H) * np.sqrt(6 / (2 * H)), rng.uniform(-0.1, 0.1, H),
             rng.uniform(-1, 1, H) * np.sqrt(6 / (H + 1)), rng.uniform(-0.1, 0.1, 1)]
    return np.concatenate(parts).astype(np.float32)


def normalisation(samples, v0):
    """Feature shifts / scales, output shift / scale (mean, standard deviation) and ln(2 V0)."""
    ln2v0 = np.log(2.0 * v0)
    cols = np.concatenate([features(samples), target(samples, ln2v0)[:, None]], axis=1)
    m = cols.mean(0)
    var = (cols * cols).mean(0) - m * m
    sd = np.where(var > 1e-12 * (1 + m * m), np.sqrt(np.maximum(var, 0)), 0.0)
    scale = np.where(sd > 0, 1.0 / np.where(sd > 0, sd, 1.0), 1.0)
    out = np.zeros(16)
    out[:5] = m[:5]
    out[5:10] = scale[:5]
    out[10] = m[5]
    out[11] = sd[5] if sd[5] > 0 else 1.0
    out[12] = ln2v0
    return out.astype(np.float32)


def train_adam(samples, v0, steps=500, lr=3e-3, seed=1):
    """Full-batch Adam on the mean-squared loss with a cosine-decayed rate (floor 5 %): the
    training schedule of the GPU trainer, restated in FP64 for small CPU checks."""
    samples = np.asarray(samples)[usable(samples)]
    norm = normalisation(samples, v0)
    p = glorot(seed).astype(np.float64)
    m = np.zeros_like(p)
    v = np.zeros_like(p)
    losses = []
    for st in range(steps):
        lrt = lr * (0.05 + 0.95 * 0.5 * (1 + np.cos(np.pi * st / steps)))
        loss, g = loss_and_grad(p, norm, samples)
        losses.append(loss)
        m = 0.9 * m + 0.1 * g
        v = 0.999 * v + 0.001 * g * g
        p -= lrt * (m / (1 - 0.9 ** (st + 1))) / (np.sqrt(v / (1 - 0.999 ** (st + 1))) + 1e-8)
    return p.astype(np.float32), norm, losses
