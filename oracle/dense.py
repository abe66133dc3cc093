"""Dense-state restatement of the encoding path (test infrastructure: the checker).

The reference keeps the working state as a quimb MPS but densifies it to
2^N amplitudes at every layer (``MPS.fidelity_with_zero_state``,
``qmprs/primitives/mps.py:1033-1039``) and in every sweep
(``qmprs/synthesis/mps_encoding/sequential.py:443-447,460,463,496``).  This
module keeps the working state dense throughout and expresses every MPS
operation on it as the equivalent dense operation:

* ``MPS.from_statevector`` (``mps.py:219-249``): right-to-left sequential
  truncated SVD of the amplitude vector (quimb ``from_dense`` followed by
  ``tensor_network_1d_compress``, whose default density-matrix method
  truncates from the right and returns a right-canonical MPS).
* ``MPS.generate_bond_D_unitary_layer`` (``mps.py:849-891``): the copy is
  compressed with ``form="right", max_bond=2`` and right-canonised; on a
  dense state this is the right-to-left truncated SVD with at most two
  singular values per cut, each right tensor being the (phase-fixed) right
  singular vectors, and site 0 the normalised remainder.
* ``MPS._apply_inverse_unitary_layer`` (``mps.py:933-971``): the gates'
  adjoints are applied to the amplitudes in the same order (``gate_`` on the
  block's last site, then ``gate_split_`` from the end of the block to its
  start).  ``gate_split_`` only drops singular values below quimb's 1e-10
  cutoff, so the dense state equals the reference's MPS state to that level.
* ``Sequential._sweep_unitary_layers`` (``sequential.py:400-507``): dense
  already in the reference after the first contraction.

Qubit order is the reference's MSB convention (``sequential.py:253``):
qubit 0 is the most significant bit of the amplitude index.
"""

from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import conventions as cv

# ---------------------------------------------------------------------------
# quick-core Ket behaviour (base.py:96-97, mps.py:170-171): pad + normalise
# ---------------------------------------------------------------------------


def ket(data) -> np.ndarray:
    """Statevector as quick's ``Ket`` holds it: complex128, padded, normalised."""
    v = np.asarray(data, dtype=np.complex128).reshape(-1)
    n = max(1, int(np.ceil(np.log2(max(v.size, 2)))))
    if v.size < 2 ** n:
        v = np.concatenate([v, np.zeros(2 ** n - v.size, dtype=np.complex128)])
    nrm = np.linalg.norm(v)
    if nrm == 0:
        raise ValueError("statevector has zero norm")
    return v / nrm


def num_qubits(v: np.ndarray) -> int:
    return int(round(np.log2(v.size)))


# ---------------------------------------------------------------------------
# dense primitives
# ---------------------------------------------------------------------------


def apply_gate(psi: np.ndarray, n: int, g: np.ndarray, q: int) -> np.ndarray:
    """Apply a 2x2 (on qubit q) or 4x4 (on qubits q, q+1) matrix, MSB order."""
    k = 1 if g.shape[0] == 2 else 2
    p = psi.reshape(2 ** q, 2 ** k, 2 ** (n - q - k))
    return np.einsum("ab,ibj->iaj", g, p).reshape(-1)


def environment(t: np.ndarray, psi: np.ndarray, n: int, q: int, k: int) -> np.ndarray:
    """E[a, b] = sum_rest conj(t[a, rest]) psi[b, rest] over the gate's qubits.

    The dense form of ``target_mps_adjoint @ circuit_mps`` with the gate's
    output legs as rows and input legs as columns (``sequential.py:463-477``).
    """
    tt = t.reshape(2 ** q, 2 ** k, 2 ** (n - q - k))
    pp = psi.reshape(2 ** q, 2 ** k, 2 ** (n - q - k))
    return np.einsum("iaj,ibj->ab", tt.conj(), pp)


def mps_to_dense(tensors: list[np.ndarray]) -> np.ndarray:
    """Contract site tensors of shape (l, p, r) to the amplitude vector."""
    v = tensors[0].reshape(2, -1)
    for a in tensors[1:]:
        l, p, r = a.shape
        v = (v @ a.reshape(l, p * r)).reshape(-1, r)
    return v.reshape(-1)


def tt_svd_right(psi: np.ndarray, n: int, max_bond: int, cutoff: float = cv.CUTOFF,
                 phase: str = "canonical") -> list[np.ndarray]:
    """Right-to-left sequential truncated SVD; site tensors in (l, p, r) order.

    Sites 1..n-1 are right isometries (rows of the truncated ``Vh``); site 0
    is the remainder ``U S``, rescaled so that the MPS keeps the norm of
    ``psi`` (quimb renormalises the kept singular values under ``rsum2``).
    """
    tensors: list[np.ndarray] = [None] * n  # type: ignore[list-item]
    r = 1
    m = psi.reshape(-1, 1)
    for c in range(n - 1, 0, -1):
        m = m.reshape(2 ** c, 2 * r)
        _, s, vh = np.linalg.svd(m, full_matrices=False)
        keep = cv.rank_by_cutoff(s, cutoff, max_bond)
        vh = vh[:keep]
        if phase == "canonical":
            vh = cv.phase_fix_rows(vh)
        tensors[c] = vh.reshape(keep, 2, r)
        m = m @ vh.conj().T
        r = keep
    nrm_in = np.linalg.norm(psi)
    nrm_out = np.linalg.norm(m)
    if nrm_out > 0:
        m = m * (nrm_in / nrm_out)
    tensors[0] = m.reshape(1, 2, r)
    return tensors


# ---------------------------------------------------------------------------
# (b) Ran's unitary completion (mps.py:565-744), restated step by step
# ---------------------------------------------------------------------------


def first_site_unitary(data: np.ndarray, mode: str) -> np.ndarray:
    """``MPS._generate_first_site_unitary`` (mps.py:565-623).

    Column 0 is the site tensor (mps.py:602) in both modes.  ``literal``
    completes it with ``scipy.linalg.null_space`` as the reference does;
    ``canonical`` uses the Schmidt form ``(A (x) B) CX (Ry (x) I)`` of the
    two-qubit state, which needs one CX (``conventions.schmidt_first_gate``).
    """
    if mode == "canonical":
        return cv.schmidt_first_gate(data.reshape(-1))
    m = data.reshape(1, -1)
    basis = cv.complement(m, mode)                       # (4, 3)
    u = np.zeros((2, 2, 2, 2), dtype=np.complex128)
    u[0, 0] = m.reshape(2, 2)
    u[0, 1] = basis[:, 0].reshape(2, 2)
    u[1, 0] = basis[:, 1].reshape(2, 2)
    u[1, 1] = basis[:, 2].reshape(2, 2)
    u = u.transpose(1, 0, 2, 3)
    return u.reshape(4, 4).T


def two_site_unitary(data: np.ndarray, mode: str) -> np.ndarray:
    """``MPS._generate_two_site_unitary`` (mps.py:625-687)."""
    m = data.reshape(2, -1)
    basis = cv.complement(m, mode)                       # (4, 2)
    basis = basis / cv.row0_phase(basis)
    u = np.zeros((2, 2, 2, 2), dtype=np.complex128)
    u[0] = data.reshape(2, 2, 2)
    u[1] = basis.reshape(2, 2, 2, 1).transpose(3, 2, 0, 1)[0]
    u = u.transpose(1, 0, 2, 3)
    return u.reshape(4, 4).T


def last_site_unitary(data: np.ndarray, start: int, end: int, mode: str) -> np.ndarray:
    """``MPS._generate_last_site_unitary`` (mps.py:689-744)."""
    if end == start:
        v = data.reshape(1, -1)
        u = np.zeros((2, 2), dtype=np.complex128)
        u[0] = v
        u[1] = cv.complement(v, mode).reshape(1, -1)
    else:
        u = data.reshape(2, 2)
    return u.T


def submps_indices(bonds: list[int]) -> list[tuple[int, int]]:
    """quick-core ``_get_submps_indices`` as described at ``mps.py:794-801``.

    ``bonds[c-1]`` is the dimension of the bond between sites c-1 and c.
    Blocks are maximal runs of sites joined by bonds larger than one.
    """
    n = len(bonds) + 1
    blocks = []
    start = 0
    for c in range(1, n):
        if bonds[c - 1] == 1:
            blocks.append((start, c - 1))
            start = c
    blocks.append((start, n - 1))
    return blocks


def is_unitary(u: np.ndarray) -> bool:
    """quick-core ``is_unitary_matrix`` restated as an ``np.allclose`` test."""
    return bool(np.allclose(u @ u.conj().T, np.eye(u.shape[0]), rtol=1e-5, atol=1e-8))


Layer = list  # list[tuple[int, int, list[np.ndarray]]]


def generate_layer(psi: np.ndarray, n: int, mode: str = "canonical") -> tuple[Layer, list[np.ndarray]]:
    """``MPS.generate_bond_D_unitary_layer`` + ``generate_unitary_layer`` (mps.py:746-891)."""
    tensors = tt_svd_right(psi, n, max_bond=2, phase=mode)
    tensors[0] = tensors[0] / np.linalg.norm(tensors[0])      # right_canonize(normalize=True)
    bonds = [tensors[c].shape[0] for c in range(1, n)]
    layer: Layer = []
    for start, end in submps_indices(bonds):
        gates = []
        for idx in range(start, end + 1):
            data = tensors[idx]
            if idx == end:
                gates.append(last_site_unitary(data, start, end, mode))
            elif idx == start:
                gates.append(first_site_unitary(data, mode))
            else:
                gates.append(two_site_unitary(data, mode))
        for g in gates:
            if not is_unitary(g):
                raise ValueError("All the generated unitaries must be unitary.")
        layer.append((start, end, gates))
    return layer, tensors


def apply_inverse_layer(psi: np.ndarray, n: int, layer: Layer) -> np.ndarray:
    """``MPS._apply_inverse_unitary_layer`` on a dense state (mps.py:933-971)."""
    for start, end, gates in layer:
        for idx in range(end, start - 1, -1):
            g = gates[idx - start].conj().T
            psi = apply_gate(psi, n, g, idx)
    return psi


def apply_layer(psi: np.ndarray, n: int, layer: Layer) -> np.ndarray:
    """``MPS._apply_unitary_layer`` on a dense state (mps.py:893-931)."""
    for start, end, gates in layer:
        for idx in range(start, end + 1):
            psi = apply_gate(psi, n, gates[idx - start], idx)
    return psi


def early_exit(fid0: complex, threshold: float) -> bool:
    """``np.isclose(fid, 1+0j, atol=1-threshold)`` with numpy's default rtol."""
    return bool(np.isclose(fid0, 1 + 0j, atol=1 - threshold))


def get_unitary_layers(target: np.ndarray, n: int, num_layers: int, threshold: float = 1 - 1e-6,
                       mode: str = "canonical") -> tuple[list[Layer], list[complex]]:
    """``Sequential._get_unitary_layers`` (sequential.py:330-398).

    Returns the layers in circuit order (reversed generation order) and the
    zero-state overlap ``conj(psi[0])`` measured after each generated layer.
    """
    psi = target / np.linalg.norm(target)
    layers: list[Layer] = []
    fids: list[complex] = []
    for _ in range(num_layers):
        layer, _ = generate_layer(psi, n, mode)
        psi = apply_inverse_layer(psi, n, layer)
        layers.append(layer)
        f = np.conj(psi[0])
        fids.append(complex(f))
        if early_exit(f, threshold):
            break
    layers.reverse()
    return layers, fids


# ---------------------------------------------------------------------------
# (d) sweeps (sequential.py:216-292, 400-541)
# ---------------------------------------------------------------------------


def circuit_gates(layers: list[Layer]) -> list[tuple[int, int, int, int, np.ndarray]]:
    """Gates in application order with their tags (layer, block, tensor, qubit).

    Same order as ``Sequential._tensor_network_from_unitary_layers``
    (sequential.py:247-270).
    """
    out = []
    for li, layer in enumerate(layers):
        for bi, (start, end, gates) in enumerate(layer):
            for idx in range(start, end + 1):
                out.append((li, bi, idx - start, idx, gates[idx - start]))
    return out


def circuit_state(layers: list[Layer], n: int) -> np.ndarray:
    psi = np.zeros(2 ** n, dtype=np.complex128)
    psi[0] = 1.0
    for _, _, _, q, g in circuit_gates(layers):
        psi = apply_gate(psi, n, g, q)
    return psi


def sweep(target: np.ndarray, n: int, layers: list[Layer], mode: str = "canonical") -> tuple[list[Layer], float]:
    """One ``Sequential._sweep_unitary_layers`` pass (sequential.py:400-507).

    Updates the layers in place and returns them with the overlap
    ``|<target|C_new|0>| / ||target||`` reached at the end of the sweep (the
    nuclear norm of the first gate's environment).  ``mode="literal"`` takes
    ``u @ vh`` as numpy returns it; ``"canonical"`` resolves rank-deficient
    environments towards the current gate (``conventions.polar_unitary_canonical``).
    """
    gates = circuit_gates(layers)
    psi = circuit_state(layers, n)
    t = target.astype(np.complex128, copy=True)
    nuc = 0.0
    for li, bi, ti, q, g in reversed(gates):
        k = 1 if g.shape[0] == 2 else 2
        psi = apply_gate(psi, n, g.conj().T, q)             # circuit_mps @ gate.conj()
        env = environment(t, psi, n, q, k)                  # target_mps_adjoint @ circuit_mps
        if mode == "canonical":
            w, s = cv.polar_unitary_canonical(env, g.conj())
        else:
            w, s = cv.polar_unitary(env)
        new = w.conj()                                      # stored as u_new.conj()
        t = apply_gate(t, n, new.conj().T, q)               # target_mps_adjoint @ new_tensor
        layers[li][bi][2][ti] = new
        nuc = float(s.sum())
    return layers, nuc / float(np.linalg.norm(target))


def environments(target: np.ndarray, n: int, layers: list[Layer]) -> list[np.ndarray]:
    """Every gate's environment at the fixed circuit, in circuit order.

    The backward pass of ``sweep`` (sequential.py:452-505) with the update
    left out: the circuit state peeled gate by gate and the target carried
    back through the same gates, so <target|C|0> = sum(G * E) for each
    gate G and its environment E.
    """
    gates = circuit_gates(layers)
    psi = circuit_state(layers, n)
    t = target.astype(np.complex128, copy=True)
    out = []
    for _, _, _, q, g in reversed(gates):
        k = 1 if g.shape[0] == 2 else 2
        psi = apply_gate(psi, n, g.conj().T, q)
        out.append(environment(t, psi, n, q, k))
        t = apply_gate(t, n, g.conj().T, q)
    return out[::-1]


def iter_dioall(target: np.ndarray, n: int, num_layers: int, sweeps_per_layer: int,
                mode: str = "canonical") -> tuple[list[Layer], list[list[float]]]:
    """Iter-DiOall schedule (arXiv:2209.00595; the reference documents it as
    the intended use of its sweep, sequential.py:410-433, without
    implementing it): k = 1..num_layers, disentangle one more layer from the
    residual C^H |target> (the newest layer is applied first in the
    circuit), then sweep all layers ``sweeps_per_layer`` times.  No early
    exit.  Returns the layers (circuit order) and the per-step lists of sweep
    fidelities."""
    t = target / np.linalg.norm(target)
    layers: list[Layer] = []            # circuit order
    fids: list[list[float]] = []
    residual = t.copy()
    for _ in range(num_layers):
        layer, _ = generate_layer(residual, n, mode)
        layers = [layer] + layers
        step = []
        for _ in range(sweeps_per_layer):
            layers, f = sweep(t, n, layers, mode)
            step.append(f)
        fids.append(step)
        residual = t.copy()
        for lay in reversed(layers):    # C^H t: the last-applied layer's inverse first
            residual = apply_inverse_layer(residual, n, lay)
    return layers, fids


def iter_dioi(target: np.ndarray, n: int, num_layers: int, sweeps_per_layer: int,
              mode: str = "canonical") -> tuple[list[Layer], list[list[float]]]:
    """Iter-DiOi schedule (arXiv:2209.00595; documented by the reference at
    sequential.py:410-433 next to Iter-DiOall, not implemented there): k =
    1..num_layers, disentangle one more layer from the residual r = C^H
    |target>, sweep only that layer against r ``sweeps_per_layer`` times (the
    older layers stay fixed; |<r|U|0>| is the whole circuit's fidelity), then
    r <- U^H r.  Returns the layers (circuit order) and the per-step lists of
    sweep fidelities."""
    t = target / np.linalg.norm(target)
    layers: list[Layer] = []            # circuit order
    fids: list[list[float]] = []
    residual = t.copy()
    for _ in range(num_layers):
        layer, _ = generate_layer(residual, n, mode)
        newest = [layer]
        step = []
        for _ in range(sweeps_per_layer):
            newest, f = sweep(residual, n, newest, mode)
            step.append(f)
        fids.append(step)
        layers = newest + layers
        residual = apply_inverse_layer(residual, n, newest[0])
    return layers, fids


@dataclass
class EncodeResult:
    layers: list
    layer_fidelities: list = field(default_factory=list)
    sweep_fidelities: list = field(default_factory=list)
    target: np.ndarray | None = None
    fidelity: float = 0.0


def prepare_state(statevector, bond_dimension: int, num_layers: int = 1, num_sweeps: int = 0,
                  threshold: float = 1 - 1e-6, mode: str = "canonical") -> EncodeResult:
    """``MPSEncoder.prepare_state`` -> ``Sequential.prepare_mps`` end to end.

    Returns the layers (circuit order), the per-layer zero-state overlaps,
    the per-sweep overlaps with the truncated target and the final fidelity
    ``|<sv|C|0>|`` with the normalised input (the reference tests' measure,
    ``test_sequential_encoding.py:67``).
    """
    sv = ket(statevector)
    n = num_qubits(sv)
    if n < 2:
        raise ValueError("The statevector must have at least 2 qubits.")
    tensors = tt_svd_right(sv, n, bond_dimension, phase=mode)
    target = mps_to_dense(tensors)
    layers, lf = get_unitary_layers(target, n, num_layers, threshold, mode)
    sf = []
    for _ in range(num_sweeps):
        layers, f = sweep(target, n, layers, mode)
        sf.append(f)
    psi = circuit_state(layers, n)
    fid = float(abs(np.vdot(psi, sv)))
    return EncodeResult(layers=layers, layer_fidelities=lf, sweep_fidelities=sf, target=target, fidelity=fid)
