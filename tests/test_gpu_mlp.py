"""The surrogate MLP's tcgen05 layers against a NumPy reference of the same
network (float64 arithmetic on the BF16-rounded weights and activations the
tensor cores see).  Tolerance: 2e-3 of the output scale (BF16 inputs, FP32
accumulation over 256 terms)."""
import numpy as np
import pytest

import pimc_gb300 as G

pytestmark = pytest.mark.gpu


def bf16(a):
    a = np.ascontiguousarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16          # round to nearest even
    return r.astype(np.uint32).view(np.float32)


def silu(z):
    return z / (1.0 + np.exp(-z))


def reference(x, w1, b1, w2, b2, w3, b3, w4, b4):
    h1 = bf16(silu(x.astype(np.float64) @ w1 + b1)).astype(np.float64)
    z2 = h1 @ bf16(w2).astype(np.float64) + b2
    h2 = bf16(silu(z2)).astype(np.float64)
    z3 = h2 @ bf16(w3).astype(np.float64) + b3
    return silu(z3) @ w4 + b4


def weights(rng):
    w1 = rng.normal(0, 1 / np.sqrt(6), (6, 256)).astype(np.float32)
    b1 = rng.normal(0, 0.1, 256).astype(np.float32)
    w2 = rng.normal(0, 1 / 16, (256, 256)).astype(np.float32)
    b2 = rng.normal(0, 0.1, 256).astype(np.float32)
    w3 = rng.normal(0, 1 / 16, (256, 256)).astype(np.float32)
    b3 = rng.normal(0, 0.1, 256).astype(np.float32)
    w4 = rng.normal(0, 1 / 16, 256).astype(np.float32)
    return w1, b1, w2, b2, w3, b3, w4, np.float32(0.25)


@pytest.mark.parametrize("n", [1, 128, 300, 4096])
def test_mlp_forward_matches_reference(n):
    rng = np.random.default_rng(n)
    W = weights(rng)
    x = rng.normal(0, 1, (n, 6)).astype(np.float32)
    m = G.Mlp()
    m.set_weights(*W)
    y = m.forward(x)
    ref = reference(x, *W)
    scale = max(1.0, float(np.max(np.abs(ref))))
    assert np.max(np.abs(y - ref)) <= 2e-3 * scale, (np.max(np.abs(y - ref)), y[:4], ref[:4])
    m.close()


def test_mlp_forward_uses_every_weight():
    """Changing one entry of each 256 x 256 weight matrix changes the output
    (every K step and every column block reaches the accumulator)."""
    rng = np.random.default_rng(7)
    W = list(weights(rng))
    x = rng.normal(0, 1, (256, 6)).astype(np.float32)
    m = G.Mlp()
    m.set_weights(*W)
    y0 = m.forward(x)
    for wi, (k, j) in ((2, (255, 3)), (2, (3, 255)), (4, (128, 200)), (4, (200, 17))):
        W2 = [a.copy() if isinstance(a, np.ndarray) else a for a in W]
        W2[wi][k, j] += 4.0
        m.set_weights(*W2)
        y1 = m.forward(x)
        ref = reference(x, *W2)
        assert np.max(np.abs(y1 - y0)) > 1e-3
        assert np.max(np.abs(y1 - ref)) <= 2e-3 * max(1.0, float(np.max(np.abs(ref))))
    m.close()


def reference_grads(x, e, w1, b1, w2, b2, w3, b3, w4, b4):
    """d mean((y-e)^2) / d params in float64 with the BF16 roundings of the
    tensor-core operands (activations, the back-propagated dz, W2, W3)."""
    x = x.astype(np.float64)
    n = len(x)
    W2, W3 = bf16(w2).astype(np.float64), bf16(w3).astype(np.float64)
    ds = lambda z: (1 / (1 + np.exp(-z))) * (1 + z * (1 - 1 / (1 + np.exp(-z))))
    z1 = x @ w1 + b1
    h1 = bf16(silu(z1)).astype(np.float64)
    z2 = h1 @ W2 + b2
    h2 = bf16(silu(z2)).astype(np.float64)
    z3 = h2 @ W3 + b3
    h3 = silu(z3)
    y = h3 @ w4 + b4
    dy = 2.0 / n * (y - e)
    gw4, gb4 = h3.T @ dy, dy.sum()
    dz3 = dy[:, None] * w4[None, :] * ds(z3)
    gb3 = dz3.sum(0)
    dz3b = bf16(dz3).astype(np.float64)
    gw3 = h2.T @ dz3b
    dz2 = (dz3b @ W3.T) * ds(z2)
    gb2 = dz2.sum(0)
    dz2b = bf16(dz2).astype(np.float64)
    gw2 = h1.T @ dz2b
    dz1 = (dz2b @ W2.T) * ds(z1)
    gb1 = dz1.sum(0)
    gw1 = x.T @ dz1
    loss = np.mean((y - e) ** 2)
    return [gw1.ravel(), gb1, gw2.ravel(), gb2, gw3.ravel(), gb3, gw4, np.array([gb4])], loss


@pytest.mark.parametrize("n", [128, 384, 1000])
def test_mlp_gradients_match_reference(n):
    """The training kernels' gradients (forward saving its operands, dW3 =
    h2^T dz3, dh2 = dz3 W3^T, dW2 = h1^T dz2, dh1 = dz2 W2^T on tcgen05)
    against the float64 reference, block by block within 1e-2 of the
    block's largest entry."""
    rng = np.random.default_rng(100 + n)
    W = weights(rng)
    x = rng.normal(0, 1, (n, 6)).astype(np.float32)
    e = rng.normal(0, 1, n).astype(np.float32)
    m = G.Mlp()
    m.set_weights(*W)
    g, loss = m.gradients(x, e)
    ref, rloss = reference_grads(x, e, *W)
    assert abs(loss - rloss) <= 1e-3 * max(1.0, rloss)
    sizes = [6 * 256, 256, 256 * 256, 256, 256 * 256, 256, 256, 1]
    off = 0
    for k, (sz, r) in enumerate(zip(sizes, ref)):
        got = g[off:off + sz]
        scale = max(float(np.max(np.abs(r))), 1e-6)
        assert np.max(np.abs(got - r)) <= 1e-2 * scale, (k, np.max(np.abs(got - r)) / scale)
        off += sz
    m.close()


def test_mlp_training_reduces_loss():
    """Adam on the GPU fits a smooth function of the six inputs."""
    rng = np.random.default_rng(3)
    W = weights(rng)
    x = rng.uniform(-1, 1, (16384, 6)).astype(np.float32)
    e = (np.sin(2 * x[:, 0]) + 0.5 * x[:, 1] ** 2 - 0.3 * x[:, 2] * x[:, 3]).astype(np.float32)
    m = G.Mlp()
    m.set_weights(*W)
    losses = m.train(x, e, epochs=20, batch=1024, lr=1e-3, seed=5)
    assert losses[-1] < 0.1 * losses[0], losses
    y = m.forward(x[:2048])
    assert np.mean((y - e[:2048]) ** 2) < 0.1 * np.var(e)
    m.close()
