"""The warm-start network's numpy oracle (oracle/mlp.py) checked against
finite differences, and its bf16 rounding against torch's; CPU only."""

import numpy as np
import pytest
import torch

from oracle import mlp as OM


def test_bf16_rounding_matches_torch():
    rng = np.random.default_rng(0)
    x = (rng.standard_normal(10000) * 10.0 ** rng.integers(-5, 5, 10000)).astype(np.float32)
    ours = OM.bf16(x)
    ref = torch.as_tensor(x).to(torch.bfloat16).float().numpy()
    assert np.array_equal(ours, ref)


def test_loss_is_phase_invariant_and_zero_at_target():
    rng = np.random.default_rng(1)
    u = rng.standard_normal((5, 32))
    w = np.ones(5)
    ph = np.exp(1j * rng.uniform(0, 2 * np.pi, 5))
    uc = (u[:, 0::2] + 1j * u[:, 1::2]) * ph[:, None]
    y = np.empty_like(u)
    y[:, 0::2], y[:, 1::2] = uc.real, uc.imag
    loss, dy = OM.loss_and_grad(y, u, w)
    assert np.allclose(loss, 0, atol=1e-10)
    assert np.allclose(dy, 0, atol=1e-10)


def test_backward_matches_finite_differences(monkeypatch):
    monkeypatch.setattr(OM, "bf16", lambda a: np.asarray(a, dtype=np.float64))
    rng = np.random.default_rng(2)
    dims = (6, 5, 4, 32)
    params = [(w.astype(np.float64), rng.standard_normal(len(b)) * 0.1) for w, b in OM.init_params(dims, 3)]
    x = rng.standard_normal((7, dims[0]))
    u = rng.standard_normal((7, 32)) * 0.5
    w = rng.uniform(0.5, 1.5, 7)

    def total(ps):
        y, _ = OM.forward(ps, x)
        loss, _ = OM.loss_and_grad(y, u, w)
        return loss.sum() / w.sum()

    y, cache = OM.forward(params, x)
    _, dy = OM.loss_and_grad(y, u, w)
    grads = OM.backward(params, cache, dy)
    eps = 1e-6
    for j in range(len(params)):
        for which in (0, 1):
            arr = params[j][which]
            for idx in [tuple(rng.integers(0, s) for s in arr.shape) for _ in range(4)]:
                plus = [(a.copy(), b.copy()) for a, b in params]
                minus = [(a.copy(), b.copy()) for a, b in params]
                plus[j][which][idx] += eps
                minus[j][which][idx] -= eps
                fd = (total(plus) - total(minus)) / (2 * eps)
                an = grads[j][which][idx]
                assert abs(fd - an) < 1e-5 * max(1.0, abs(fd)), (j, which, idx, fd, an)


@pytest.mark.parametrize("z", [-3.0, -0.5, 0.0, 0.7, 2.5])
def test_gelu_grad(z):
    eps = 1e-6
    fd = (OM.gelu(z + eps) - OM.gelu(z - eps)) / (2 * eps)
    assert abs(fd - OM.gelu_grad(z)) < 1e-8


@pytest.mark.parametrize("m", [2, 4])
def test_overlap_grad_matches_finite_differences(m):
    """The circuit-overlap loss row: fid = |sum U*E|^2 tinv, and dY is the
    derivative of -gscale fid(polar(Y)) at a unitary Y = U (finite
    differences along random complex directions, both signs of the step)."""
    rng = np.random.default_rng(5 + m)
    z = rng.standard_normal((m, m)) + 1j * rng.standard_normal((m, m))
    u = OM.polar_factor(z)
    e = 0.4 * (rng.standard_normal((m, m)) + 1j * rng.standard_normal((m, m)))
    tinv, gscale = 0.8, 0.25
    env = np.zeros((1, 16), complex)
    gates = np.zeros((1, 16), complex)
    env[0, : m * m] = e.reshape(-1)
    gates[0, : m * m] = u.reshape(-1)
    kind = np.array([1 if m == 2 else 2])
    fid, dy = OM.overlap_grad(env, gates, kind, np.array([tinv]), gscale)
    assert np.isclose(fid[0], abs(np.sum(u * e)) ** 2 * tinv)
    assert np.all(dy[0, 2 * m * m:] == 0)
    g = dy[0, : 2 * m * m : 2] + 1j * dy[0, 1 : 2 * m * m : 2]

    def loss(y):
        return -gscale * tinv * abs(np.sum(OM.polar_factor(y) * e)) ** 2

    h = 1e-6
    for _ in range(6):
        d = rng.standard_normal((m, m)) + 1j * rng.standard_normal((m, m))
        num = (loss(u + h * d) - loss(u - h * d)) / (2 * h)
        ana = float(np.real(np.sum(np.conj(g) * d.reshape(-1))))
        assert abs(num - ana) < 1e-6 * max(1.0, abs(ana)), (num, ana)
    # a Hermitian stretch U (I + H) leaves the polar factor, so the gradient
    # has no component along it
    hm = rng.standard_normal((m, m)) + 1j * rng.standard_normal((m, m))
    d = u @ (hm + hm.conj().T)
    assert abs(np.real(np.sum(np.conj(g) * d.reshape(-1)))) < 1e-12
