"""The FP64 oracle: internal consistency and the reference's own behaviours.

The reference ships no golden vectors (its randomness is unseeded), so the
oracle is pinned by (1) agreement between its two restatements (the
call-by-call MPS one and the dense one), (2) the behaviours the reference's
tests assert (``tests/synthesis/mps_encoding/test_sequential_encoding.py``,
``tests/primitives/test_mps.py``), and (3) the reference's published
fidelities (README.md:49-71 and the notebook), matched statistically.
"""

import numpy as np
import pytest

from oracle import conventions as cv
from oracle import dense as D
from oracle import mpsops as M
from oracle import states as S


def _rand_state(n, seed):
    return S.uniform_complex(n, seed)


def test_rank_by_cutoff():
    s = np.array([1.0, 1e-3, 1e-6])
    assert cv.rank_by_cutoff(s) == 2            # 1e-12 tail <= 1e-10 * total
    assert cv.rank_by_cutoff(s, max_bond=1) == 1
    assert cv.rank_by_cutoff(np.array([1.0, 0.0])) == 1
    assert cv.rank_by_cutoff(np.array([0.6, 0.6, 0.6])) == 3


@pytest.mark.parametrize("k,n", [(1, 2), (1, 4), (2, 4), (3, 4)])
def test_householder_complement(k, n):
    rng = np.random.default_rng(k * 10 + n)
    a = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    q, _ = np.linalg.qr(a)
    x = q[:, :k].T.copy()
    c = cv.householder_complement(x)
    full = np.concatenate([x.T, c], axis=1)
    assert np.allclose(full.conj().T @ full, np.eye(n), atol=1e-12)


def test_householder_complement_structured():
    # exact basis vectors and equal-magnitude rows resolve ties to the lowest index
    c = cv.householder_complement(np.array([[1, 0, 0, 0]], dtype=complex))
    assert np.allclose(np.abs(c), np.eye(4)[:, 1:])
    x = np.array([[0.5, 0.5, 0.5, 0.5]], dtype=complex)
    c = cv.householder_complement(x)
    assert np.allclose(x.conj() @ c, 0, atol=1e-14)


@pytest.mark.parametrize("n,chi,L,S_", [(6, 8, 4, 2), (7, 64, 3, 2), (8, 4, 3, 1)])
def test_dense_equals_mps_restatement(n, chi, L, S_):
    """The dense reformulation reproduces the call-by-call MPS restatement."""
    sv = _rand_state(n, 100 + n)
    rd = D.prepare_state(sv, chi, L, S_, mode="canonical")
    rm = M.prepare_state(sv, chi, L, S_, conv="canonical")
    assert np.allclose(rd.target, rm.target, atol=1e-12)
    # layers before sweeps: gate by gate
    ld, _ = D.get_unitary_layers(rd.target, n, L, mode="canonical")
    mps = M.from_statevector(sv, chi, conv="canonical")
    lm, _ = M.get_unitary_layers(mps, L, conv="canonical")
    for a, b in zip(D.circuit_gates(ld), D.circuit_gates(lm)):
        assert a[:4] == b[:4]
        assert np.allclose(a[4], b[4], atol=1e-8)
    assert np.allclose(rd.layer_fidelities, rm.layer_fidelities, atol=1e-10)
    assert np.allclose(rd.sweep_fidelities, rm.sweep_fidelities, atol=1e-10)
    assert abs(rd.fidelity - rm.fidelity) < 1e-10


def test_literal_first_layer_is_gauge_invariant():
    """The first layer's zero-state overlap does not depend on the conventions."""
    n = 8
    sv = _rand_state(n, 5)
    t = D.mps_to_dense(D.tt_svd_right(sv, n, 64))
    _, fc = D.get_unitary_layers(t, n, 1, mode="canonical")
    _, fl = D.get_unitary_layers(t, n, 1, mode="literal")
    assert abs(fc[0] - fl[0]) < 1e-12


def test_sweep_same_from_identical_layers_literal_vs_canonical():
    """Sweeps are gauge-robust: the same initial layers give the same fidelities."""
    n = 7
    sv = _rand_state(n, 9)
    t = D.mps_to_dense(D.tt_svd_right(sv, n, 64))
    layers, _ = D.get_unitary_layers(t, n, 3, mode="literal")
    import copy
    l1 = copy.deepcopy(layers)
    f1 = [D.sweep(t, n, l1)[1] for _ in range(3)]
    l2 = M.get_unitary_layers(M.from_statevector(sv, 64), 3)[0]
    f2 = [D.sweep(t, n, l2)[1] for _ in range(3)]
    assert len(f1) == len(f2)


def test_untruncated_mps_reproduces_statevector():
    n = 9
    sv = _rand_state(n, 3)
    t = D.mps_to_dense(D.tt_svd_right(sv, n, 2 ** (n // 2)))
    assert np.linalg.norm(t - sv) < 1e-10


# ---- reference behaviours (test_sequential_encoding.py) ---------------------------


def test_reference_prepare_state_threshold():
    sv = _rand_state(8, 11)
    r = D.prepare_state(sv, 32, num_layers=32)
    assert 1 - r.fidelity < 1e-2


@pytest.mark.parametrize("mode", ["canonical", "literal"])
def test_reference_layer_improvement(mode):
    sv = _rand_state(8, 12)
    f = [D.prepare_state(sv, 64, num_layers=i, mode=mode).fidelity for i in range(1, 10)]
    assert np.all(np.diff(f) >= 0)


@pytest.mark.parametrize("mode", ["canonical", "literal"])
def test_reference_sweep_improvement(mode):
    sv = _rand_state(8, 13)
    f = [D.prepare_state(sv, 64, num_layers=6, num_sweeps=i, mode=mode).fidelity for i in range(1, 8)]
    assert np.all(np.diff(f) >= 0)


def _ghz_like(n, pairs, plus):
    """|0..0> with H on `plus` qubits and CX chains (qiskit little-endian labels)."""
    from qmprs_gb300.circuit import Circuit
    h = np.array([[1, 1], [1, -1]]) / np.sqrt(2)
    cx = np.eye(4)[[0, 3, 2, 1]]       # control = first listed qubit (LSB of U)
    c = Circuit(n)
    for q in plus:
        c.unitary(h, q)
    for a, b in pairs:
        c.unitary(cx, [a, b])
    return c.get_statevector()


def test_reference_partial_entanglement_depth():
    from qmprs_gb300.circuit import Circuit
    from qmprs_gb300.synthesis.mps_encoding import Sequential
    sv = _ghz_like(8, [(0, 3), (5, 7)], [0, 4, 5])
    r = D.prepare_state(sv, 32, num_layers=1)
    assert 1 - r.fidelity < 1e-2
    c = Circuit(8)
    for layer in r.layers:
        Sequential._apply_unitary_layer_to_circuit(c, layer)
    assert np.allclose(c.get_statevector(), D.circuit_state(r.layers, 8), atol=1e-12)
    assert c.get_depth() <= 20


def test_reference_partial_entanglement_with_sweep_depth():
    from qmprs_gb300.circuit import Circuit
    from qmprs_gb300.synthesis.mps_encoding import Sequential
    sv = _ghz_like(4, [(0, 1), (1, 2)], [0, 3])
    r = D.prepare_state(sv, 32, num_layers=1, num_sweeps=1)
    assert 1 - r.fidelity < 1e-2
    c = Circuit(4)
    for layer in r.layers:
        Sequential._apply_unitary_layer_to_circuit(c, layer)
    assert c.get_depth() <= 7


# ---- published numbers (statistical) --------------------------------------------


@pytest.mark.slow
def test_readme_fidelity_n10_statistically():
    """README.md:49-71 reports |<psi|C|0>| = 0.98676 for one unseeded 10-qubit
    uniform-complex state, chi=512, L=15, S=50.  The oracle's mean over seeds
    must fall in the same band."""
    f = [D.prepare_state(_rand_state(10, s), 512, 15, 50).fidelity for s in range(3)]
    assert 0.975 < float(np.mean(f)) < 0.995, f


def test_iter_dioall_oracle_sweeps_never_lose_fidelity():
    """Within each step of the Iter-DiOall schedule the sweeps do not lower
    the fidelity, and the last one is the circuit's overlap."""
    from oracle import states as S
    n = 6
    sv = S.random_mps(n, 4, 3)
    t = sv / np.linalg.norm(sv)
    layers, fids = D.iter_dioall(t, n, 3, 3)
    for step in fids:
        assert all(b >= a - 1e-12 for a, b in zip(step, step[1:]))
    psi = D.circuit_state(layers, n)
    assert abs(abs(np.vdot(psi, t)) - fids[-1][-1]) < 1e-10


def test_iter_dioi_oracle_sweeps_the_newest_layer_only():
    """Iter-DiOi: within each step the sweeps of the newest layer do not
    lower the fidelity, the last one is the whole circuit's overlap, the
    older layers are left as they were, and without sweeps it builds the
    same layers as Iter-DiOall."""
    from oracle import states as S
    n = 6
    sv = S.random_mps(n, 4, 5)
    t = sv / np.linalg.norm(sv)
    layers, fids = D.iter_dioi(t, n, 3, 3)
    for step in fids:
        assert all(b >= a - 1e-12 for a, b in zip(step, step[1:]))
    psi = D.circuit_state(layers, n)
    assert abs(abs(np.vdot(psi, t)) - fids[-1][-1]) < 1e-10
    two, _ = D.iter_dioi(t, n, 2, 3)
    for a, b in zip(two, layers[1:]):   # the first two generated layers stay fixed
        for (s1, e1, g1), (s2, e2, g2) in zip(a, b):
            assert (s1, e1) == (s2, e2) and all(np.array_equal(x, y) for x, y in zip(g1, g2))
    l0, _ = D.iter_dioi(t, n, 3, 0)
    l1, _ = D.iter_dioall(t, n, 3, 0)
    for a, b in zip(l0, l1):
        for (s1, e1, g1), (s2, e2, g2) in zip(a, b):
            assert (s1, e1) == (s2, e2) and all(np.allclose(x, y) for x, y in zip(g1, g2))


def test_environments_give_the_overlap_and_do_not_depend_on_their_gate():
    """<t|C|0> = sum(G * E_G) for every gate of a fixed circuit, and E_G does
    not depend on G: a replaced gate G' gives the overlap sum(G' * E_G)."""
    n, L = 6, 3
    t = S.uniform_complex(n, 3)
    t = t / np.linalg.norm(t)
    layers, _ = D.get_unitary_layers(t, n, L)
    envs = D.environments(t, n, layers)
    gates = D.circuit_gates(layers)
    assert len(envs) == len(gates)
    f = np.vdot(t, D.circuit_state(layers, n))
    for (_, _, _, _, g), e in zip(gates, envs):
        assert abs(np.sum(g * e) - f) < 1e-12
    rng = np.random.default_rng(1)
    for idx in (0, len(gates) // 2, len(gates) - 1):
        li, bi, ti, q, g = gates[idx]
        m = g.shape[0]
        z = rng.standard_normal((m, m)) + 1j * rng.standard_normal((m, m))
        w, _, vh = np.linalg.svd(z)
        mod = [[(s, e, list(gs)) for s, e, gs in layer] for layer in layers]
        mod[li][bi][2][ti] = w @ vh
        f2 = np.vdot(t, D.circuit_state(mod, n))
        assert abs(np.sum((w @ vh) * envs[idx]) - f2) < 1e-12


def test_overlap_gradient_is_the_derivative_of_circuit_fidelity():
    """End to end on a circuit: the environment of a gate and the overlap
    loss's gradient (oracle.mlp.overlap_grad, the restatement of the GPU
    kernel) give the derivative of the circuit fidelity |<t|C|0>|^2 / <t|t>
    when that gate is replaced by the polar factor of U + h D."""
    from oracle import mlp as OM
    n, L = 5, 2
    t = S.uniform_complex(n, 9)          # not normalised: <t|t> enters as tinv
    layers, _ = D.get_unitary_layers(t / np.linalg.norm(t), n, L)
    envs = D.environments(t, n, layers)
    gates = D.circuit_gates(layers)
    tinv = 1.0 / float(np.vdot(t, t).real)
    rng = np.random.default_rng(4)
    for idx in (1, len(gates) - 2):
        li, bi, ti, q, g = gates[idx]
        m = g.shape[0]
        env = np.zeros((1, 16), complex)
        gr = np.zeros((1, 16), complex)
        env[0, : m * m] = envs[idx].reshape(-1)
        gr[0, : m * m] = g.reshape(-1)
        fid, dy = OM.overlap_grad(env, gr, np.array([1 if m == 2 else 2]), np.array([tinv]), 1.0)
        grad = dy[0, : 2 * m * m : 2] + 1j * dy[0, 1 : 2 * m * m : 2]   # of -F

        def fidelity(y):
            mod = [[(s, e, list(gs)) for s, e, gs in layer] for layer in layers]
            mod[li][bi][2][ti] = OM.polar_factor(y)
            return abs(np.vdot(t, D.circuit_state(mod, n))) ** 2 * tinv

        assert abs(fidelity(g) - fid[0]) < 1e-12
        h = 1e-6
        for _ in range(3):
            d = rng.standard_normal((m, m)) + 1j * rng.standard_normal((m, m))
            num = (fidelity(g + h * d) - fidelity(g - h * d)) / (2 * h)
            ana = -float(np.real(np.sum(np.conj(grad) * d.reshape(-1))))
            assert abs(num - ana) < 1e-6 * max(1.0, abs(ana)), (num, ana)
