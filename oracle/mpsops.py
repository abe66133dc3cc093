"""MPS-based restatement of the encoding path (test infrastructure).

This module follows the reference call by call on an explicit MPS (a list of
site tensors in (left, phys, right) order, the ``permute("lpr")`` layout of
``qmprs/primitives/mps.py:538-563``) and restates the quimb 1.10.0
operations those calls reach:

* ``MatrixProductState.from_dense`` (``mps.py:242``): exact SVD chain,
  quimb's default 1e-10 ``rsum2`` cutoff.
* ``tensor_network_1d_compress(max_bond=chi)`` (``mps.py:247,445``): for an
  MPS input the default density-matrix method truncates from the right and
  returns a right-canonical MPS; restated as ``left_canonize`` followed by
  ``right_compress``.
* ``compress(form="right", max_bond=...)`` (``mps.py:453``): quimb's
  ``left_canonize`` then ``right_compress`` (each bond: QR/LQ reduction, SVD
  of ``R1 @ L2``, truncation, singular values absorbed to the left).
* ``left_canonize`` / ``right_canonize(normalize=...)`` (``mps.py:396,398``):
  sweeps of QR/LQ with a real non-negative diagonal (quimb's stabilised QR).
* ``gate_`` (``mps.py:913,953``) and ``gate_split_`` (``mps.py:928,968``):
  single-site contraction; two-site contraction plus SVD split with the
  default cutoff and the singular values shared between both sides.
* ``to_dense`` (``mps.py:270,1037``).

``conv="literal"`` keeps LAPACK's phases and ``scipy.linalg.null_space``
(what the reference computes); ``conv="canonical"`` applies the rules of
``oracle.conventions`` and must then agree with ``oracle.dense``.  The
literal pipeline, being the reference's own algorithm including the MPS SVD
chain per layer, is also the timed CPU proxy of the reference.
"""

from __future__ import annotations

import copy

import numpy as np

from . import conventions as cv
from . import dense as D

Mps = list  # list[np.ndarray] of shape (l, p, r)


def _qr_stab(a: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    q, r = np.linalg.qr(a)
    d = np.diag(r).copy()
    s = np.ones_like(d)
    nz = np.abs(d) > 0
    s[nz] = d[nz] / np.abs(d[nz])
    return q * s[None, :], r * np.conj(s)[:, None]


def _lq_stab(a: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    q, r = _qr_stab(a.conj().T)
    return r.conj().T, q.conj().T


def from_dense(psi: np.ndarray, n: int) -> Mps:
    """quimb ``MatrixProductState.from_dense`` (exact up to the 1e-10 cutoff)."""
    tensors: Mps = []
    m = psi.reshape(1, -1)
    l = 1
    for i in range(n - 1):
        m = m.reshape(l * 2, -1)
        u, s, vh = np.linalg.svd(m, full_matrices=False)
        k = cv.rank_by_cutoff(s)
        tensors.append(u[:, :k].reshape(l, 2, k))
        m = s[:k, None] * vh[:k]
        l = k
    tensors.append(m.reshape(l, 2, 1))
    return tensors


def to_dense(t: Mps) -> np.ndarray:
    return D.mps_to_dense(t)


def norm(t: Mps) -> float:
    return float(np.linalg.norm(to_dense(t)))


def left_canonize(t: Mps) -> None:
    for i in range(len(t) - 1):
        l, p, r = t[i].shape
        q, rr = _qr_stab(t[i].reshape(l * p, r))
        k = q.shape[1]
        t[i] = q.reshape(l, p, k)
        nl, np_, nr = t[i + 1].shape
        t[i + 1] = (rr @ t[i + 1].reshape(nl, np_ * nr)).reshape(k, np_, nr)


def right_canonize(t: Mps, normalize: bool = False) -> None:
    for i in range(len(t) - 1, 0, -1):
        l, p, r = t[i].shape
        lm, q = _lq_stab(t[i].reshape(l, p * r))
        k = q.shape[0]
        t[i] = q.reshape(k, p, r)
        pl, pp, pr = t[i - 1].shape
        t[i - 1] = (t[i - 1].reshape(pl * pp, pr) @ lm).reshape(pl, pp, k)
    if normalize:
        t[0] = t[0] / np.linalg.norm(t[0])


def right_compress(t: Mps, max_bond: int | None = None, cutoff: float = cv.CUTOFF,
                   conv: str = "literal") -> None:
    """quimb ``right_compress``: bonds from the right, singular values to the left."""
    for i in range(len(t) - 1, 0, -1):
        l1, p1, r1 = t[i - 1].shape
        l2, p2, r2 = t[i].shape
        q1, rr1 = _qr_stab(t[i - 1].reshape(l1 * p1, r1))
        ll2, q2 = _lq_stab(t[i].reshape(l2, p2 * r2))
        u, s, vh = np.linalg.svd(rr1 @ ll2, full_matrices=False)
        k = cv.rank_by_cutoff(s, cutoff, max_bond)
        total = float(np.sum(s * s))
        u, s, vh = u[:, :k], s[:k], vh[:k]
        if total > 0:                                   # quimb renorm for rsum2
            s = s * np.sqrt(total / float(np.sum(s * s)))
        right = vh @ q2
        if conv == "canonical":
            fixed = cv.phase_fix_rows(right)
            ph = np.array([np.vdot(right[a], fixed[a]) for a in range(k)])
            right = fixed
            u = u * np.conj(ph)[None, :]
        t[i] = right.reshape(k, p2, r2)
        t[i - 1] = (q1 @ (u * s[None, :])).reshape(l1, p1, k)


def compress(t: Mps, max_bond: int | None = None, conv: str = "literal") -> None:
    """``MPS.compress(mode="right", max_bond_dimension=...)`` (mps.py:402-459)."""
    left_canonize(t)
    right_compress(t, max_bond, conv=conv)


def gate_single(t: Mps, g: np.ndarray, i: int) -> None:
    t[i] = np.einsum("pq,lqr->lpr", g, t[i])


def gate_split(t: Mps, g: np.ndarray, i: int, cutoff: float = cv.CUTOFF) -> None:
    a, b = t[i], t[i + 1]
    l, _, _ = a.shape
    _, _, r = b.shape
    theta = np.einsum("lqr,rsm->lqsm", a, b).reshape(l, 4, r)
    theta = np.einsum("pq,lqm->lpm", g, theta).reshape(l * 2, 2 * r)
    u, s, vh = np.linalg.svd(theta, full_matrices=False)
    k = cv.rank_by_cutoff(s, cutoff)
    sq = np.sqrt(s[:k])
    t[i] = (u[:, :k] * sq[None, :]).reshape(l, 2, k)
    t[i + 1] = (sq[:, None] * vh[:k]).reshape(k, 2, r)


def from_statevector(sv: np.ndarray, chi: int, conv: str = "literal") -> Mps:
    """``MPS.from_statevector`` (mps.py:219-249)."""
    n = D.num_qubits(sv)
    t = from_dense(sv, n)
    compress(t, chi, conv=conv)
    return t


def generate_bond_d_layer(t: Mps, conv: str) -> D.Layer:
    """``MPS.generate_bond_D_unitary_layer`` (mps.py:849-891)."""
    c = copy.deepcopy(t)
    compress(c, 2, conv=conv)
    right_canonize(c, normalize=True)
    n = len(c)
    bonds = [c[i].shape[0] for i in range(1, n)]
    layer: D.Layer = []
    for start, end in D.submps_indices(bonds):
        gates = []
        for idx in range(start, end + 1):
            data = c[idx]
            if idx == end:
                gates.append(D.last_site_unitary(data, start, end, conv))
            elif idx == start:
                gates.append(D.first_site_unitary(data, conv))
            else:
                gates.append(D.two_site_unitary(data, conv))
        for g in gates:
            if not D.is_unitary(g):
                raise ValueError("All the generated unitaries must be unitary.")
        layer.append((start, end, gates))
    return layer


def apply_inverse_layer(t: Mps, layer: D.Layer) -> None:
    """``MPS._apply_inverse_unitary_layer`` (mps.py:933-971)."""
    for start, end, gates in layer:
        for idx in range(end, start - 1, -1):
            g = gates[idx - start].conj().T
            if idx == end:
                gate_single(t, g, idx)
            else:
                gate_split(t, g, idx)


def get_unitary_layers(mps: Mps, num_layers: int, threshold: float = 1 - 1e-6,
                       conv: str = "literal") -> tuple[list[D.Layer], list[complex]]:
    """``Sequential._get_unitary_layers`` (sequential.py:330-398)."""
    work = copy.deepcopy(mps)
    nrm = norm(work)
    if not np.isclose(nrm, 1.0):                         # MPS.normalize (mps.py:302-310)
        work[0] = work[0] / nrm
    compress(work, None, conv=conv)                       # compress(mode="right")
    right_canonize(work, normalize=True)                  # canonicalize("right", normalize=True)
    layers: list[D.Layer] = []
    fids: list[complex] = []
    for _ in range(num_layers):
        layer = generate_bond_d_layer(work, conv)
        apply_inverse_layer(work, layer)
        layers.append(layer)
        f = complex(np.conj(to_dense(work)[0]))            # fidelity_with_zero_state
        fids.append(f)
        if D.early_exit(f, threshold):
            break
    layers.reverse()
    return layers, fids


def prepare_state(statevector, bond_dimension: int, num_layers: int = 1, num_sweeps: int = 0,
                  threshold: float = 1 - 1e-6, conv: str = "literal",
                  stop_fidelity: float = 0.0) -> D.EncodeResult:
    """The reference path end to end on an explicit MPS (CPU proxy of the reference).

    ``stop_fidelity > 0`` ends the sweeps once a sweep's fidelity with the
    target reaches it (the per-state stop of the batched GPU path; the
    reference itself always runs ``num_sweeps``)."""
    sv = D.ket(statevector)
    n = D.num_qubits(sv)
    if n < 2:
        raise ValueError("The statevector must have at least 2 qubits.")
    mps = from_statevector(sv, bond_dimension, conv=conv)
    target = to_dense(mps)
    layers, lf = get_unitary_layers(mps, num_layers, threshold, conv)
    sf = []
    for _ in range(num_sweeps):
        layers, f = D.sweep(target, n, layers, conv)
        sf.append(f)
        if stop_fidelity > 0.0 and f >= stop_fidelity:
            break
    psi = D.circuit_state(layers, n)
    fid = float(abs(np.vdot(psi, sv)))
    return D.EncodeResult(layers=layers, layer_fidelities=lf, sweep_fidelities=sf, target=target, fidelity=fid)
