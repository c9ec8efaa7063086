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
