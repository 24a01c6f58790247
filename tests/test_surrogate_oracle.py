"""The CPU restatement of the surrogate network (oracle/mlp_oracle.cpp) is
itself checked here: its gradient agrees with a plain float64 numpy
back-propagation (no BF16 rounding) to the BF16 storage precision, and that
numpy reference agrees with central finite differences.  The GPU kernels
are then held to the oracle (tests/test_gpu_surrogate.py)."""
import numpy as np
import pytest

from geliosphere_gb300 import surrogate as sg


def init_params(seed=3, scale=1.0):
    rng = np.random.default_rng(seed)
    p = np.zeros(199681, np.float32)
    for k, (off, shape) in sg.OFFSETS.items():
        n = int(np.prod(shape))
        fan_in = shape[1] if len(shape) == 2 else 256
        if k.startswith("b"):
            p[off:off + n] = rng.normal(0, 0.05, n)
        else:
            p[off:off + n] = rng.uniform(-1, 1, n) * np.sqrt(3.0 / fan_in) * scale
    return p


def np_forward_backward(p, x, t):
    w = sg.unflatten(p.astype(np.float64))
    silu = lambda z: z / (1 + np.exp(-z))  # noqa: E731

    def dsilu(z):
        s = 1 / (1 + np.exp(-z))
        return s * (1 + z * (1 - s))
    xs, zs = [x.astype(np.float64)], []
    for l in range(1, 5):
        z = xs[-1] @ w[f"W{l}"].T + w[f"b{l}"]
        zs.append(z)
        xs.append(silu(z))
    y = xs[-1] @ w["w5"] + w["b5"][0]
    e = y - t
    loss = np.mean(e * e)
    dy = 2 * e / len(t)
    g = {"w5": xs[-1].T @ dy, "b5": np.array([dy.sum()])}
    dh = np.outer(dy, w["w5"]) * dsilu(zs[3])
    for l in range(4, 0, -1):
        g[f"W{l}"] = dh.T @ xs[l - 1]
        g[f"b{l}"] = dh.sum(0)
        if l > 1:
            dh = (dh @ w[f"W{l}"]) * dsilu(zs[l - 2])
    flat = np.zeros(199681)
    for k, (off, shape) in sg.OFFSETS.items():
        flat[off:off + int(np.prod(shape))] = g[k].ravel()
    return loss, flat, y


def data(n=64, seed=5):
    rng = np.random.default_rng(seed)
    x = rng.uniform(-1.2, 1.2, (n, 7)).astype(np.float32)
    t = (0.5 * np.sin(2 * x[:, 0]) + 0.3 * x[:, 1] * x[:, 6] - 0.2 * x[:, 2] ** 2).astype(np.float32)
    return x, t


def test_numpy_reference_matches_finite_differences():
    p = init_params()
    x, t = data(16)
    _, g, _ = np_forward_backward(p, x, t)
    rng = np.random.default_rng(0)
    for k in ["W1", "b1", "W2", "W4", "b4", "w5", "b5"]:
        off, shape = sg.OFFSETS[k]
        for idx in rng.integers(0, int(np.prod(shape)), 3):
            q = p.astype(np.float64).copy()
            h = 1e-3
            q[off + idx] += h
            lp = np_forward_backward(q, x, t)[0]
            q[off + idx] -= 2 * h
            lm = np_forward_backward(q, x, t)[0]
            fd = (lp - lm) / (2 * h)
            assert abs(fd - g[off + idx]) <= 1e-5 + 1e-3 * abs(fd), (k, idx, fd, g[off + idx])


def test_oracle_matches_numpy_to_bf16_precision(oracle):
    p = init_params()
    x, t = data(256)
    loss_np, g_np, y_np = np_forward_backward(p, x, t)
    y_or = oracle.mlp_forward(p, x)
    np.testing.assert_allclose(y_or, y_np, atol=2e-2 * np.abs(y_np).max())
    loss_or, g_or = oracle.mlp_grad(p, x, t)
    assert abs(loss_or - loss_np) <= 2e-2 * loss_np
    for k, (off, shape) in sg.OFFSETS.items():
        n = int(np.prod(shape))
        a, b = g_or[off:off + n], g_np[off:off + n]
        rel = np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)
        assert rel < 3e-2, (k, rel)


def test_feature_normalisation():
    """gelio_surrogate_features (host function, no GPU) maps the batch
    parameter ranges onto [-1, 1]."""
    from geliosphere_gb300 import abi, make_sim
    from geliosphere_gb300.surrogate import Surrogate
    lo = make_sim(abi.GELIO_MODEL_2D_GELIOSPHERE, 1, K0_cm2s=1e22, V_kms=350, tilt_deg=5, polarity=-1,
                  r_injection=1.0, theta_deg=10)
    hi = make_sim(abi.GELIO_MODEL_2D_GELIOSPHERE, 1, K0_cm2s=1e23, V_kms=750, tilt_deg=75, polarity=1,
                  r_injection=80.0, theta_deg=170)
    np.testing.assert_allclose(Surrogate.features(lo, 0.01), [-1] * 7, atol=2e-6)
    np.testing.assert_allclose(Surrogate.features(hi, 100.0), [1] * 7, atol=2e-6)
