"""Seeded synthetic statevector families used by the benchmark and examples.

* ``uniform_complex(n, seed)``   re, im i.i.d. U[0,1), L2-normalised (the
  reference tests' random states, ``test_sequential_encoding.py:29-44``).
* ``gaussian_mixture(n, seed)``  3 Gaussian components on 2^n grid points,
  means U[0,1), sigma U[0.02,0.2], equal weights, phases exp(2 pi i u).
* ``random_mps(n, bond, seed)``  i.i.d. complex Gaussian site tensors of the
  given bond dimension, left-canonicalised, contracted, normalised.
"""

from __future__ import annotations

import numpy as np


def uniform_complex(n: int, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    v = rng.random(2 ** n) + 1j * rng.random(2 ** n)
    return v / np.linalg.norm(v)


def gaussian_mixture(n: int, seed: int, components: int = 3) -> np.ndarray:
    rng = np.random.default_rng(seed)
    mu = rng.random(components)
    sigma = 0.02 + 0.18 * rng.random(components)
    x = np.arange(2 ** n, dtype=np.float64) / 2 ** n
    amp = np.zeros(2 ** n)
    for m, s in zip(mu, sigma):
        amp += np.exp(-0.5 * ((x - m) / s) ** 2) / s
    v = amp * np.exp(2j * np.pi * rng.random(2 ** n))
    return v / np.linalg.norm(v)


def random_mps(n: int, bond: int, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    dims = [1] + [min(bond, 2 ** min(i, n - i)) for i in range(1, n)] + [1]
    tensors = []
    for i in range(n):
        shape = (dims[i], 2, dims[i + 1])
        tensors.append((rng.standard_normal(shape) + 1j * rng.standard_normal(shape)) / np.sqrt(2.0))
    for i in range(n - 1):
        l, p, r = tensors[i].shape
        q, rr = np.linalg.qr(tensors[i].reshape(l * p, r))
        tensors[i] = q.reshape(l, p, q.shape[1])
        nl, np_, nr = tensors[i + 1].shape
        tensors[i + 1] = (rr @ tensors[i + 1].reshape(nl, np_ * nr)).reshape(q.shape[1], np_, nr)
    v = tensors[0].reshape(2, -1)
    for a in tensors[1:]:
        l, p, r = a.shape
        v = (v @ a.reshape(l, p * r)).reshape(-1, r)
    v = v.reshape(-1)
    return v / np.linalg.norm(v)
