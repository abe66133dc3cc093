"""The FP64 small linear algebra compiled into the kernels, run on the CPU.

``qmprs_gb300/csrc/small_linalg.h`` is compiled both into the CUDA library
and into ``libqmprs_hostcheck.so``; these tests hold the host build to the
oracle's canonical conventions and to numpy's decompositions.
"""

import ctypes

import numpy as np
import pytest

from oracle import conventions as cv
from oracle import dense as D
from qmprs_gb300 import build as qb


@pytest.fixture(scope="module")
def hc():
    lib = ctypes.CDLL(str(qb.build_hostcheck()))
    dp = ctypes.POINTER(ctypes.c_double)
    lib.hc_herm_eig.argtypes = [dp, ctypes.c_int, dp, dp]
    lib.hc_polar.argtypes = [dp, ctypes.c_int, dp, dp]
    lib.hc_polar.restype = ctypes.c_double
    lib.hc_polar_pre.argtypes = [dp, ctypes.c_int, dp, dp]
    lib.hc_polar_pre.restype = ctypes.c_double
    lib.hc_polar_sweep.argtypes = [dp, ctypes.c_int, dp, dp]
    lib.hc_polar_sweep.restype = ctypes.c_double
    lib.hc_complement.argtypes = [dp, ctypes.c_int, ctypes.c_int, dp]
    lib.hc_rank_by_cutoff.argtypes = [dp, ctypes.c_int, ctypes.c_double, ctypes.c_int]
    lib.hc_rank_by_cutoff.restype = ctypes.c_int
    lib.hc_rank_from_tails.argtypes = [dp, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                       ctypes.c_double, ctypes.c_int]
    lib.hc_rank_from_tails.restype = ctypes.c_int
    ip = ctypes.POINTER(ctypes.c_int)
    lib.hc_round_robin_pair.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ip, ip]
    lib.hc_phase_fix_column.argtypes = [dp, ctypes.c_int, ctypes.c_int, ctypes.c_int]
    lib.hc_ran_gate.argtypes = [ctypes.c_int, dp, dp]
    return lib


def _p(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _c(a):
    return np.ascontiguousarray(a, dtype=np.complex128)


@pytest.mark.parametrize("n", [2, 3, 4, 8])
def test_herm_eig(hc, n):
    rng = np.random.default_rng(n)
    a = rng.standard_normal((n, 2 * n)) + 1j * rng.standard_normal((n, 2 * n))
    g = _c(a @ a.conj().T)
    v = np.zeros((n, n), np.complex128)
    lam = np.zeros(n)
    hc.hc_herm_eig(_p(g), n, _p(v), _p(lam))
    ref = np.linalg.eigvalsh(g)[::-1]
    assert np.allclose(lam, ref, rtol=1e-12, atol=1e-12)
    assert np.allclose(g @ v, v * lam[None, :], atol=1e-10)
    assert np.allclose(v.conj().T @ v, np.eye(n), atol=1e-12)


def test_herm_eig_rank_deficient_tail(hc):
    """Tiny eigenvalues of a PSD Gram matrix keep their relative accuracy."""
    rng = np.random.default_rng(0)
    q, _ = np.linalg.qr(rng.standard_normal((4, 4)) + 1j * rng.standard_normal((4, 4)))
    lam_true = np.array([1.0, 0.3, 1e-9, 1e-13])
    g = _c(q @ np.diag(lam_true) @ q.conj().T)
    v = np.zeros((4, 4), np.complex128)
    lam = np.zeros(4)
    hc.hc_herm_eig(_p(g), 4, _p(v), _p(lam))
    assert abs(lam[2] - 1e-9) < 1e-15
    sq = _c(lam).real.copy()
    assert hc.hc_rank_by_cutoff(sq.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), 4, 1e-10, 4) == \
        cv.rank_by_cutoff(np.sqrt(np.maximum(lam_true, 0)))


@pytest.mark.parametrize("m", [2, 4])
@pytest.mark.parametrize("seed", range(5))
def test_polar_matches_numpy(hc, m, seed):
    rng = np.random.default_rng(seed)
    e = _c(rng.standard_normal((m, m)) + 1j * rng.standard_normal((m, m)))
    w = np.zeros((m, m), np.complex128)
    nuc = hc.hc_polar(_p(e), m, _p(w), None)
    wref, s = cv.polar_unitary(e)
    assert np.allclose(w, wref, atol=1e-12)
    assert abs(nuc - s.sum()) < 1e-12


def test_polar_rank_one(hc):
    """Rank-deficient environments still give a unitary with the right column."""
    e = np.zeros((4, 4), np.complex128)
    e[:, 0] = [0.3, 0.1j, -0.2, 0.5]
    w = np.zeros((4, 4), np.complex128)
    nuc = hc.hc_polar(_p(_c(e)), 4, _p(w), None)
    assert np.allclose(w.conj().T @ w, np.eye(4), atol=1e-12)
    assert np.allclose(w[:, 0], e[:, 0] / np.linalg.norm(e[:, 0]), atol=1e-12)
    assert abs(nuc - np.linalg.norm(e[:, 0])) < 1e-12


@pytest.mark.parametrize("rank", [0, 1, 2, 3])
@pytest.mark.parametrize("seed", range(3))
def test_polar_null_space_follows_previous(hc, rank, seed):
    """Rank-deficient environments: the completion nearest to the previous
    unitary, identical to the oracle's canonical rule."""
    rng = np.random.default_rng(seed)
    a = rng.standard_normal((4, rank)) + 1j * rng.standard_normal((4, rank))
    b = rng.standard_normal((rank, 4)) + 1j * rng.standard_normal((rank, 4))
    e = _c(a @ b)
    e = e + 1e-9 * (rng.standard_normal((4, 4)))          # below the null threshold
    prev, _ = np.linalg.qr(rng.standard_normal((4, 4)) + 1j * rng.standard_normal((4, 4)))
    prev = _c(prev)
    w = np.zeros((4, 4), np.complex128)
    hc.hc_polar(_p(_c(e)), 4, _p(w), _p(prev))
    ref, _ = cv.polar_unitary_canonical(e, prev)
    assert np.allclose(w.conj().T @ w, np.eye(4), atol=1e-10)
    assert np.allclose(w, ref, atol=1e-7)


@pytest.mark.parametrize("m", [2, 4])
@pytest.mark.parametrize("seed", range(8))
@pytest.mark.parametrize("cond", [1.0, 1e-3, 1e-5])
def test_sweep_polar_fp32_sweeps(hc, m, seed, cond):
    """The sweep kernel's polar (FP32 Jacobi, FP64 orthonormalisation and
    trace): W is unitary to FP64 rounding, within FP32 accuracy of the exact
    polar factor, and its trace Re Tr(W^H E) -- the fidelity the sweep
    reports -- matches the nuclear norm to second order."""
    rng = np.random.default_rng(100 + seed)
    q1, _ = np.linalg.qr(rng.standard_normal((m, m)) + 1j * rng.standard_normal((m, m)))
    q2, _ = np.linalg.qr(rng.standard_normal((m, m)) + 1j * rng.standard_normal((m, m)))
    sv = np.geomspace(1.0, cond, m) * 0.37
    e = _c(q1 @ np.diag(sv) @ q2)
    w = np.zeros((m, m), np.complex128)
    nuc = hc.hc_polar_sweep(_p(e), m, _p(w), None)
    wref, s = cv.polar_unitary(e)
    assert np.allclose(w.conj().T @ w, np.eye(m), atol=1e-14)
    assert np.allclose(w, wref, atol=2e-5 / max(cond, 1e-2))
    # error ~ s_min * (eps32 / cond)^2: 1e-11 relative at cond 1e-5
    assert abs(nuc - s.sum()) <= 1e-10 * s.sum()


@pytest.mark.parametrize("rank", [0, 1, 2, 3])
@pytest.mark.parametrize("seed", range(3))
def test_sweep_polar_null_space(hc, rank, seed):
    """Rank-deficient environments in the sweep kernel's polar: same
    completion as the oracle's canonical rule, to FP32 accuracy."""
    rng = np.random.default_rng(seed)
    a = rng.standard_normal((4, rank)) + 1j * rng.standard_normal((4, rank))
    b = rng.standard_normal((rank, 4)) + 1j * rng.standard_normal((rank, 4))
    e = _c(a @ b)
    e = e + 1e-9 * (rng.standard_normal((4, 4)))
    prev, _ = np.linalg.qr(rng.standard_normal((4, 4)) + 1j * rng.standard_normal((4, 4)))
    prev = _c(prev)
    w = np.zeros((4, 4), np.complex128)
    nuc = hc.hc_polar_sweep(_p(_c(e)), 4, _p(w), _p(prev))
    ref, s = cv.polar_unitary_canonical(e, prev)
    assert np.allclose(w.conj().T @ w, np.eye(4), atol=1e-14)
    assert np.allclose(w, ref, atol=1e-4)
    sv = np.linalg.svd(e, compute_uv=False)
    # the null directions (below 1e-6 s_max) are filled towards prev, so they
    # contribute anything in [-s_null, s_null] to the trace
    assert abs(nuc - sv[:rank].sum()) <= sv[rank:].sum() + 1e-10 * max(1.0, sv[0])


@pytest.mark.parametrize("k,n", [(1, 2), (1, 4), (2, 4)])
@pytest.mark.parametrize("seed", range(4))
def test_complement_matches_oracle(hc, k, n, seed):
    rng = np.random.default_rng(seed)
    q, _ = np.linalg.qr(rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)))
    x = _c(q[:, :k].T)
    c = np.zeros((n - k, n), np.complex128)
    hc.hc_complement(_p(x), k, n, _p(c))
    ref = cv.householder_complement(x)
    assert np.allclose(c.T, ref, atol=1e-13)


def test_phase_fix_matches_oracle(hc):
    rng = np.random.default_rng(3)
    v = _c(rng.standard_normal((4, 3)) + 1j * rng.standard_normal((4, 3)))
    ref = cv.phase_fix_rows(v.T).T
    for col in range(3):
        hc.hc_phase_fix_column(_p(v), 4, 3, col)
    assert np.allclose(v, ref, atol=1e-14)


@pytest.mark.parametrize("seed", range(4))
def test_ran_gates_match_oracle(hc, seed):
    n = 6
    sv = np.random.default_rng(seed).standard_normal(2 ** n) + 0j
    sv = sv / np.linalg.norm(sv)
    tensors = D.tt_svd_right(sv, n, 2)
    tensors[0] = tensors[0] / np.linalg.norm(tensors[0])
    out = np.zeros((4, 4), np.complex128)
    hc.hc_ran_gate(0, _p(_c(tensors[0].reshape(-1))), _p(out))
    assert np.allclose(out, D.first_site_unitary(tensors[0], "canonical"), atol=1e-13)
    hc.hc_ran_gate(1, _p(_c(tensors[2].reshape(-1))), _p(out))
    assert np.allclose(out, D.two_site_unitary(tensors[2], "canonical"), atol=1e-13)
    o2 = np.zeros((2, 2), np.complex128)
    hc.hc_ran_gate(2, _p(_c(tensors[n - 1].reshape(-1))), _p(o2))
    assert np.allclose(o2, D.last_site_unitary(tensors[n - 1], 0, n - 1, "canonical"), atol=1e-13)
    v = _c([0.6, 0.8j])
    hc.hc_ran_gate(3, _p(v), _p(o2))
    assert np.allclose(o2, D.last_site_unitary(v.reshape(1, 2, 1), 3, 3, "canonical"), atol=1e-13)


# ---- tile layout of the pass kernels (qmprs_gb300/csrc/tile_layout.h) -------------

def _layout(hc):
    for f in (hc.hc_swz, hc.hc_rest_offset, hc.hc_apply_pos_offset):
        f.restype = ctypes.c_int
    return hc


def _masks(T, u=4):
    from itertools import combinations
    for bits in combinations(range(T), u):
        yield sum(1 << b for b in bits)


def test_swizzle_is_a_linear_bijection(hc):
    hc = _layout(hc)
    vals = [hc.hc_swz(i) for i in range(1 << 12)]
    assert sorted(vals) == list(range(1 << 12))
    rng = np.random.default_rng(0)
    for _ in range(200):
        a, b = (int(x) for x in rng.integers(0, 1 << 12, 2))
        assert hc.hc_swz(a ^ b) == vals[a] ^ vals[b]


@pytest.mark.parametrize("T", [8, 9, 10, 11])
def test_rest_and_position_orders_are_bijections(hc, T):
    """Every 4-qubit window placement in a 2^T tile: the rest index and the
    window position map one to one onto the tile bits outside the window
    (a non-bijective order would drop rests from the cross matrix)."""
    hc = _layout(hc)
    full = (1 << T) - 1
    for wmask in _masks(T):
        rmask = full & ~wmask
        subsets = set()
        for r in range(1 << (T - 4)):
            o = hc.hc_rest_offset(r, wmask, rmask)
            assert o & ~rmask == 0
            subsets.add(o)
        assert len(subsets) == 1 << (T - 4)
        pos = {hc.hc_apply_pos_offset(p, wmask, rmask) for p in range(1 << (T - 4))}
        assert len(pos) == 1 << (T - 4) and all(o & ~rmask == 0 for o in pos)


def _banks(addrs):
    return len({hc_addr & 15 for hc_addr in addrs})


def test_fragment_loads_hit_distinct_banks(hc):
    """The cross matrix's fragment loads: a half-warp (window entries g = 0..3
    times rest indices 2t, t = 0..3) reads 16 float2 slots; with the window
    on four consecutive tile bits (the common case) they fall on 16 distinct
    128-byte-row slots, and for every placement on at least 8."""
    hc = _layout(hc)
    T = 11
    full = (1 << T) - 1
    worst = 16
    for wmask in _masks(T):
        rmask = full & ~wmask
        from_w = lambda a: hc.hc_swz(_deposit(a, wmask))
        for e in (0, 1, 8, 9):
            addrs = [from_w(g) ^ hc.hc_swz(hc.hc_rest_offset(2 * t + e, wmask, rmask)) for g in range(4)
                     for t in range(4)]
            worst = min(worst, _banks(addrs))
            if wmask in (0b1111 << s for s in range(T - 3)):
                assert _banks(addrs) == 16, (bin(wmask), e)
    assert worst >= 8


def _deposit(v, mask):
    r, bit = 0, 0
    while mask:
        low = mask & -mask
        if (v >> bit) & 1:
            r |= low
        bit += 1
        mask ^= low
    return r


def test_gate_application_loads_and_stores_hit_distinct_banks(hc):
    """The window-gate products: a half-warp loads entries 2t + e (t = 0..3)
    at positions g (g = 0..3) and stores entries g at positions 2t + e; with
    the window on four consecutive tile bits both are conflict-free, and for
    every placement at most two-way."""
    hc = _layout(hc)
    T = 11
    full = (1 << T) - 1
    worst = 16
    for wmask in _masks(T):
        rmask = full & ~wmask
        ent = lambda a: hc.hc_swz(_deposit(a, wmask))
        pos = lambda p: hc.hc_swz(hc.hc_apply_pos_offset(p, wmask, rmask))
        consecutive = wmask in (0b1111 << s for s in range(T - 3))
        for e in (0, 1, 8, 9):
            loads = [ent(2 * t + e) ^ pos(g) for g in range(4) for t in range(4)]
            stores = [ent(g + (e & 8)) ^ pos(2 * t + (e & 1)) for g in range(4) for t in range(4)]
            for addrs in (loads, stores):
                worst = min(worst, _banks(addrs))
                if consecutive:
                    assert _banks(addrs) == 16, (bin(wmask), e)
    assert worst >= 8


def test_tensor_core_scale_keeps_fp16_in_range(hc):
    """vec_scale: |v s| <= 2^15 for every amplitude of a vector of norm nrm
    (|v| <= nrm), any size and norm, and the typical amplitude nrm 2^-n/2
    lands in [2^2, 2^5] where it fits (n/2 + 4 <= 15)."""
    hc.hc_vec_scale.restype = ctypes.c_float
    hc.hc_vec_scale.argtypes = [ctypes.c_int, ctypes.c_double]
    for n in range(2, 31):
        for nrm in (1e-3, 0.37, 0.999999, 1.0, 1.000001, 3.0, 1e3):
            s = hc.hc_vec_scale(n, nrm)
            assert s > 0 and np.log2(s) == int(np.log2(s))   # a power of two
            assert nrm * s <= 2.0 ** 15
            if n // 2 + 4 <= 15:
                assert 4.0 <= nrm * 2.0 ** (-n / 2) * s <= 32.0


@pytest.mark.parametrize("m", [2, 4])
@pytest.mark.parametrize("seed", range(8))
@pytest.mark.parametrize("cond", [1.0, 1e-3, 1e-5])
def test_preconditioned_polar_is_the_fp64_polar(hc, m, seed, cond):
    """The exact mode's polar (FP32 Hestenes sweeps, then the FP64 sweeps of
    polar_jacobi from there) gives the FP64 polar factor and nuclear norm,
    also for ill-conditioned environments."""
    rng = np.random.default_rng(300 + seed)
    u, _ = np.linalg.qr(rng.standard_normal((m, m)) + 1j * rng.standard_normal((m, m)))
    v, _ = np.linalg.qr(rng.standard_normal((m, m)) + 1j * rng.standard_normal((m, m)))
    s = np.geomspace(1.0, cond, m)
    e = _c((u * s) @ v.conj().T * 0.37)
    w = np.zeros((m, m), np.complex128)
    nuc = hc.hc_polar_pre(_p(e), m, _p(w), None)
    wref, sref = cv.polar_unitary(e)
    assert np.allclose(w, wref, atol=1e-11 / cond)
    assert abs(nuc - sref.sum()) < 1e-12
    w64 = np.zeros((m, m), np.complex128)
    hc.hc_polar(_p(e), m, _p(w64), None)
    assert np.allclose(w, w64, atol=1e-11 / cond)


@pytest.mark.parametrize("rank", [0, 1, 2, 3])
@pytest.mark.parametrize("seed", range(3))
def test_preconditioned_polar_null_space_follows_previous(hc, rank, seed):
    rng = np.random.default_rng(seed)
    a = rng.standard_normal((4, rank)) + 1j * rng.standard_normal((4, rank))
    b = rng.standard_normal((rank, 4)) + 1j * rng.standard_normal((rank, 4))
    e = _c(a @ b)
    e = e + 1e-9 * (rng.standard_normal((4, 4)))
    prev, _ = np.linalg.qr(rng.standard_normal((4, 4)) + 1j * rng.standard_normal((4, 4)))
    prev = _c(prev)
    w = np.zeros((4, 4), np.complex128)
    hc.hc_polar_pre(_p(_c(e)), 4, _p(w), _p(prev))
    ref, _ = cv.polar_unitary_canonical(e, prev)
    assert np.allclose(w.conj().T @ w, np.eye(4), atol=1e-10)
    assert np.allclose(w, ref, atol=1e-7)
    w64 = np.zeros((4, 4), np.complex128)
    hc.hc_polar(_p(_c(e)), 4, _p(w64), _p(prev))
    assert np.allclose(w, w64, atol=1e-9)


@pytest.mark.parametrize("seed", range(6))
def test_rank_from_tails_matches_rsum2(hc, seed):
    """The blocked eigensolver's rule (only the largest Kr eigenvalues known,
    the rest as one weight) keeps what quimb's rsum2 rule keeps on the full
    spectrum: decaying spectra that cross the 1e-10 cutoff, rank-deficient
    ones, and caps that bind."""
    rng = np.random.default_rng(seed)
    n = 200
    lam = np.sort(10.0 ** rng.uniform(-16, 0, n))[::-1]
    lam[rng.integers(40, n):] = 0.0                      # a null tail
    total = float(lam.sum())
    for K in (20, 60, 120, n):
        for Kr in sorted({K, min(n, K + 7), n}):
            rest = float(lam[Kr:].sum())
            ref = min(cv.rank_by_cutoff(np.sqrt(lam)), K)
            got = hc.hc_rank_from_tails(_p(np.ascontiguousarray(lam[:Kr])), Kr, K, rest, total, 1e-10, 0)
            assert got == ref, (K, Kr, got, ref)


@pytest.mark.parametrize("n", [2, 4, 32, 128, 2048 // 16])
def test_round_robin_rounds_are_matchings_meeting_every_pair_once(hc, n):
    """The tournament of the blocked Jacobi (blocks of a round, indices of a
    32 x 32 subproblem's inner rounds): each round pairs every index once,
    and a sweep of n - 1 rounds meets every pair exactly once."""
    seen = set()
    p, q = ctypes.c_int(), ctypes.c_int()
    for k in range(n - 1):
        used = set()
        for i in range(n // 2):
            hc.hc_round_robin_pair(n, k, i, ctypes.byref(p), ctypes.byref(q))
            assert 0 <= p.value < q.value < n
            assert p.value not in used and q.value not in used
            used |= {p.value, q.value}
            seen.add((p.value, q.value))
        assert len(used) == n
    assert len(seen) == n * (n - 1) // 2
