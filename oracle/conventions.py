"""Numerical conventions shared by the oracle restatements (test infrastructure).

The reference's tensor values depend on conventions that live inside LAPACK
and quimb (the phase of each singular vector, the basis LAPACK returns for a
null space).  The reference never fixes them, so its MPS tensors and layer
unitaries are only defined up to those gauges.  This module names two sets
of conventions:

``literal``    the routines the reference itself calls, as they fall:
               ``numpy.linalg.svd`` phases and ``scipy.linalg.null_space``
               (``qmprs/primitives/mps.py:597,657,730``).
``canonical``  deterministic rules that make every quantity a function of the
               state alone (for non-degenerate spectra).  The GPU kernels
               implement exactly these rules, so the GPU is compared with the
               oracle in this mode.

Rules of ``canonical`` mode
---------------------------
* Singular-vector phase: every right singular vector (a row of ``Vh``) is
  multiplied by a unit phase that makes its pivot entry real and positive.
  The pivot is the LOWEST index whose magnitude is at least
  ``(1 - PIVOT_TOL)`` times the largest magnitude of that vector.
* Completion to a unitary: given k orthonormal kets (rows of ``X``), the
  complement is built from a pivoted Householder product
  ``Q = H_1 H_2 ... H_k``.  ``H_a`` maps ``conj(phi_a) x_a'`` to
  ``-e_{j_a}`` where ``x_a' = H_{a-1} ... H_1 x_a``, ``j_a`` is the pivot of
  ``x_a'`` among the indices not yet used and ``phi_a`` the phase of that
  entry.  The complement columns are ``Q e_j`` for the unused ``j`` in
  increasing order.
* Middle-site phase fix (``mps.py:661-662``): the reference divides each
  null-space column by the phase of its row-0 entry; an entry with
  magnitude below ``ZERO_TOL`` counts as zero (phase 1, as ``np.angle(0)``).
* Truncation: quimb's default ``cutoff=1e-10`` with ``cutoff_mode="rsum2"``:
  the longest tail of singular values whose squared sum is at most
  ``cutoff * sum(s**2)`` is discarded, then at most ``max_bond`` are kept.
"""

from __future__ import annotations

import numpy as np
import scipy.linalg

CUTOFF = 1e-10
PIVOT_TOL = 1e-6
ZERO_TOL = 1e-12


def rank_by_cutoff(s: np.ndarray, cutoff: float = CUTOFF, max_bond: int | None = None) -> int:
    """Number of singular values kept by quimb's ``rsum2`` rule (then capped).

    Follows the truncation quimb 1.10 applies in ``tensor_split`` for MPS
    methods (``cutoff_mode="rsum2"``), the mode behind ``from_dense``,
    ``compress`` and ``tensor_network_1d_compress`` called at
    ``qmprs/primitives/mps.py:242,247,445,453``.
    """
    s = np.asarray(s, dtype=np.float64)
    if s.size == 0:
        return 0
    sq = s * s
    total = float(sq.sum())
    if total <= 0.0:
        keep = 1
    else:
        tail = np.cumsum(sq[::-1])[::-1]          # tail[j] = sum_{k>=j} s_k^2
        keep = int(np.sum(tail > cutoff * total))
        keep = max(keep, 1)
    if max_bond is not None:
        keep = min(keep, int(max_bond))
    return keep


def pivot_index(v: np.ndarray, allowed: np.ndarray | None = None) -> int:
    """Lowest index whose magnitude is within ``PIVOT_TOL`` of the maximum."""
    mag = np.abs(v)
    if allowed is not None:
        mag = np.where(allowed, mag, -1.0)
    m = mag.max()
    return int(np.nonzero(mag >= (1.0 - PIVOT_TOL) * m)[0][0])


def phase_fix_rows(vh: np.ndarray) -> np.ndarray:
    """Canonical phase of right singular vectors: pivot entry real positive."""
    out = np.array(vh, dtype=np.complex128, copy=True)
    for a in range(out.shape[0]):
        j = pivot_index(out[a])
        z = out[a, j]
        if abs(z) > 0:
            out[a] *= np.conj(z) / abs(z)
    return out


def householder_complement(x: np.ndarray) -> np.ndarray:
    """Canonical orthonormal complement of the kets in the rows of ``x``.

    ``x`` has shape (k, n) with orthonormal rows.  Returns an (n, n-k) array
    whose columns are orthonormal and orthogonal to every row of ``x``: the
    same object ``scipy.linalg.null_space(x.conj())`` returns, with a
    deterministic basis (module docstring).
    """
    x = np.atleast_2d(np.asarray(x, dtype=np.complex128))
    k, n = x.shape
    ws: list[np.ndarray] = []
    used = np.zeros(n, dtype=bool)
    for a in range(k):
        v = x[a].copy()
        for w in ws:                                   # v <- H_{a-1}...H_1 x_a
            v = v - w * (2.0 * np.vdot(w, v) / np.vdot(w, w).real)
        v[used] = 0.0
        j = pivot_index(v, ~used)
        phase = v[j] / abs(v[j])
        y = np.conj(phase) * v
        w = y.copy()
        w[j] += 1.0
        ws.append(w)
        used[j] = True
    cols = []
    for j in range(n):
        if used[j]:
            continue
        v = np.zeros(n, dtype=np.complex128)
        v[j] = 1.0
        for w in reversed(ws):                         # Q e_j = H_1 ... H_k e_j
            v = v - w * (2.0 * np.vdot(w, v) / np.vdot(w, w).real)
        cols.append(v)
    return np.stack(cols, axis=1)


def null_space_literal(x: np.ndarray) -> np.ndarray:
    """The reference's own completion: ``scipy.linalg.null_space(x.conj())``."""
    return scipy.linalg.null_space(np.atleast_2d(x).conj())


def complement(x: np.ndarray, mode: str) -> np.ndarray:
    if mode == "canonical":
        return householder_complement(x)
    if mode == "literal":
        return null_space_literal(x)
    raise ValueError(f"unknown convention mode {mode!r}")


def row0_phase(basis: np.ndarray) -> np.ndarray:
    """Phase per column used by the middle-site fix (``mps.py:661-662``)."""
    z = basis[0]
    out = np.ones_like(z)
    nz = np.abs(z) > ZERO_TOL
    out[nz] = z[nz] / np.abs(z[nz])
    return out


def schmidt_first_gate(m4: np.ndarray) -> np.ndarray:
    """First-site gate of a block in canonical mode: ``G|00> = m4`` with one CX.

    With ``M[p, r] = m4[2p + r] = sum_i s_i a_i b_i^T`` (``v_i`` the
    canonical-phase eigenvectors of ``M^H M``, ``b_i = conj(v_i)``,
    ``a_i = M v_i / |M v_i|``), ``G = (A (x) B) CX (Ry (x) I)`` with
    ``Ry = [[s0, -s1], [s1, s0]]`` and CX controlled by the first qubit.
    """
    m = np.asarray(m4, dtype=np.complex128).reshape(2, 2)
    lam, v = np.linalg.eigh(m.conj().T @ m)
    lam, v = lam[::-1], v[:, ::-1]
    v = phase_fix_rows(v.T).T
    s = np.sqrt(np.maximum(lam, 0.0))
    s = s / np.linalg.norm(s)
    a = np.zeros((2, 2), dtype=np.complex128)
    c0 = m @ v[:, 0]
    a[:, 0] = c0 / np.linalg.norm(c0)
    if s[1] > 1e-8 * s[0]:
        c1 = m @ v[:, 1]
        a[:, 1] = c1 / np.linalg.norm(c1)
    else:
        a[:, 1] = householder_complement(a[:, 0][None, :])[:, 0]
    b = v.conj()
    ry = np.array([[s[0], -s[1]], [s[1], s[0]]])
    cx = np.eye(4)[[0, 1, 3, 2]]
    return np.kron(a, b) @ cx @ np.kron(ry, np.eye(2))


def polar_unitary(env: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """Unitary polar factor ``u @ vh`` of an environment and its singular values.

    Restates ``qmprs/synthesis/mps_encoding/sequential.py:473-478``.
    """
    u, s, vh = np.linalg.svd(env)
    return u @ vh, s


POLAR_NULL_TOL = 1e-6


def _polar_isometry(x: np.ndarray, fixed: np.ndarray) -> np.ndarray:
    """Isometry nearest to ``x`` (m x c); rank-deficient columns are completed
    by Gram-Schmidt on e_0, e_1, ... against ``fixed`` and the others."""
    u, s, vh = np.linalg.svd(x, full_matrices=False)
    keep = s > 1e-8
    cols = [u[:, i] for i in range(u.shape[1]) if keep[i]]
    basis = [fixed[:, i] for i in range(fixed.shape[1])] + cols
    out_u = list(u.T)
    for i in range(u.shape[1]):
        if keep[i]:
            continue
        for k in range(x.shape[0]):
            v = np.zeros(x.shape[0], complex)
            v[k] = 1.0
            for _ in range(2):
                for b in basis:
                    v = v - b * np.vdot(b, v)
            if np.linalg.norm(v) > 0.5:
                v = v / np.linalg.norm(v)
                out_u[i] = v
                basis.append(v)
                break
    return np.stack(out_u, axis=1) @ vh


def polar_unitary_canonical(env: np.ndarray, w_prev: np.ndarray | None) -> tuple[np.ndarray, np.ndarray]:
    """Canonical-mode polar factor: maximiser of Re Tr(W^H E) nearest ``w_prev``
    on E's null space (singular values <= POLAR_NULL_TOL * max count as zero).

    For a non-singular environment this is ``u @ vh``; for a rank-deficient
    one every completion on the null space is a maximiser and the reference's
    choice is whatever LAPACK returns, so this mode fixes it to the
    orthogonal-Procrustes fit ``polar((I - U_s U_s^H) w_prev V_N)``.
    """
    u, s, vh = np.linalg.svd(env)
    sig = s > POLAR_NULL_TOL * s.max()
    if sig.all():
        return u @ vh, s
    us, vs = u[:, sig], vh[sig].conj().T
    vn = vh[~sig].conj().T
    w = us @ vs.conj().T
    x = w_prev @ vn if w_prev is not None else np.zeros((env.shape[0], vn.shape[1]), complex)
    x = x - us @ (us.conj().T @ x)
    q = _polar_isometry(x, us)
    return w + q @ vn.conj().T, s
