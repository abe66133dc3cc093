"""Seeded synthetic input families (test infrastructure and bench inputs).

The reference ships no benchmark data; its tests and notebook draw unseeded
random states (``tests/synthesis/mps_encoding/test_sequential_encoding.py:29-44``,
notebook cell 27).  These generators reproduce those distributions with
explicit seeds, plus the structured families used by the workloads:

* ``uniform_complex``   re, im i.i.d. U[0,1), L2-normalised (reference tests).
* ``gaussian_mixture``  3-component 1-D Gaussian mixture on 2^N grid points,
                        means U[0,1), sigma U[0.02,0.2], equal weights, random
                        phases exp(2 pi i u), L2-normalised.
* ``random_mps``        i.i.d. complex Gaussian site tensors of a given bond
                        dimension, left-canonicalised, contracted, normalised.

The same generators live in ``qmprs_gb300.states`` for the product side, so
that nothing on the product path imports this package; tests check that both
produce identical arrays.
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
    phase = np.exp(2j * np.pi * rng.random(2 ** n))
    v = amp * phase
    return v / np.linalg.norm(v)


def random_mps(n: int, bond: int, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    dims = [1] + [min(bond, 2 ** min(i, n - i)) for i in range(1, n)] + [1]
    tensors = []
    for i in range(n):
        shape = (dims[i], 2, dims[i + 1])
        a = (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)) / np.sqrt(2.0)
        tensors.append(a)
    for i in range(n - 1):                       # left-canonicalise
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


def random_mps_batch(ns, bonds, seed: int, indices) -> list:
    """Statevectors ``indices`` of the batch drawn by the product's batched
    random-MPS generator (``qmprs_gb300.engine.Engine.random_mps_states``):
    one generator seeded with ``seed`` draws every state's site tensors in
    batch order (real then imaginary part per tensor), so the states are
    replayed here in the same order, then left-canonicalised and contracted
    in FP64 and normalised."""
    rng = np.random.default_rng(seed)
    want = set(int(i) for i in indices)
    out = {}
    for b, (n, bd) in enumerate(zip(ns, bonds)):
        dims = [1] + [min(int(bd), 2 ** min(i, n - i)) for i in range(1, n)] + [1]
        ts = []
        for i in range(n):
            shape = (dims[i], 2, dims[i + 1])
            ts.append((rng.standard_normal(shape) + 1j * rng.standard_normal(shape)) / np.sqrt(2.0))
        if b not in want:
            continue
        for i in range(n - 1):
            l, p, r = ts[i].shape
            q, rr = np.linalg.qr(ts[i].reshape(l * p, r))
            ts[i] = q.reshape(l, p, q.shape[1])
            nl, np_, nr = ts[i + 1].shape
            ts[i + 1] = (rr @ ts[i + 1].reshape(nl, np_ * nr)).reshape(q.shape[1], np_, nr)
        v = ts[0].reshape(2, -1)
        for a in ts[1:]:
            l, p, r = a.shape
            v = (v @ a.reshape(l, p * r)).reshape(-1, r)
        v = v.reshape(-1)
        out[b] = v / np.linalg.norm(v)
    return [out[int(i)] for i in indices]
