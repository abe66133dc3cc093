"""Stage (a) for bonds above 64: the blocked FP32 Jacobi with FP64
refinement of the kept columns (csrc/ttsvd_wide.cu), against the FP64
oracle's truncated SVD (oracle/dense.py tt_svd_right, which follows
qmprs/primitives/mps.py:242,247)."""

import numpy as np
import pytest

from oracle import dense as D
from oracle import states as S

pytestmark = pytest.mark.gpu

GATE_TOL = 2e-4


@pytest.fixture(scope="module")
def eng(cuda_lib):
    from qmprs_gb300 import engine
    return engine.engine()


def _fid(a, b):
    return abs(np.vdot(a, b)) / (np.linalg.norm(a) * np.linalg.norm(b))


@pytest.mark.parametrize("n,bond,chi", [(16, 96, 128), (15, 70, 100)])
def test_wide_rank_deficient_cuts(eng, n, bond, chi):
    """A random MPS of bond 96 (70) under bond dimension 128 (100): the
    wide Grams (up to 192 and 140 columns) have exact rank 96 (70), so the
    1e-10 cutoff, not the bond dimension, decides every bond."""
    sv = S.random_mps(n, bond, 3)
    p, svd = eng.upload([sv], 1, chi)
    tensors, bonds, target = eng.stage_mps(p, svd, chi)
    sv64 = sv.astype(np.complex64).astype(np.complex128)
    ts = D.tt_svd_right(sv64 / np.linalg.norm(sv64), n, chi)
    got = [int(x) for x in bonds.cpu().numpy()[1:n]]
    assert got == [t.shape[2] for t in ts[:-1]], got
    assert max(got) == bond
    st = eng.wide_stats(p)
    assert st["grams"] > 0, st
    t = target.cpu().numpy().view(np.complex64).astype(np.complex128)
    assert _fid(t, D.mps_to_dense(ts)) > 1 - 1e-6


@pytest.mark.parametrize("n,chi", [(16, 128), (17, 200)])
def test_wide_refinement_converges(eng, n, chi):
    """Full-rank uniform states: the FP32 sweeps and the refinement converge
    within a few steps per Gram, and the tensors match the oracle's."""
    sv = S.uniform_complex(n, 21 + n)
    res = eng.encode([sv], chi, num_layers=1, num_sweeps=0, keep_tensors=True)
    sv64 = sv.astype(np.complex64).astype(np.complex128)
    ref = D.tt_svd_right(sv64 / np.linalg.norm(sv64), n, chi)
    got = res.mps_tensors(0)
    assert [t.shape for t in got] == [t.shape for t in ref]
    for s_, (g, r) in enumerate(zip(got, ref)):
        assert np.max(np.abs(g - r)) < GATE_TOL, (s_, np.max(np.abs(g - r)))
    p, svd = eng.upload([sv], 1, chi)
    before = eng.wide_stats(p)       # the plan may be shared with earlier calls
    eng.stage_mps(p, svd, chi)
    st = {k: eng.wide_stats(p)[k] - before[k] for k in ("grams", "sweeps", "refine_steps")}
    assert st["grams"] > 0
    assert st["refine_steps"] <= 3 * st["grams"], st
    assert st["sweeps"] <= 12 * st["grams"], st


def test_wide_exact_mode_tolerance(eng):
    """The exact mode refines to its own tolerance (correction below 1e-7,
    so the eigenvectors carry FP64-level errors) and matches the oracle's
    truncated state on the complex128 input."""
    n, chi = 16, 128
    sv = S.uniform_complex(n, 9)
    p, svd = eng.upload([sv], 1, chi, "exact")
    before = eng.wide_stats(p)["grams"]
    _, bonds, target = eng.stage_mps(p, svd, chi)
    st = eng.wide_stats(p)
    assert st["grams"] > before and st["last_correction"] <= 1e-7, st
    ts = D.tt_svd_right(sv / np.linalg.norm(sv), n, chi)
    got = target.cpu().numpy().view(np.complex128)
    assert np.max(np.abs(got - D.mps_to_dense(ts))) < 1e-9


@pytest.mark.parametrize("seed", [3, 11])
def test_wide_decaying_spectra_keep_isometric_tensors(eng, seed):
    """Gaussian-mixture states with random phases (20 qubits, bond 256):
    decaying spectra send cuts through the deflated subproblem and the row
    Gram.  Every site tensor stays right-isometric (A A^H = I) and the
    truncated target keeps the input's norm, as the rsum2 renormalisation
    does."""
    import torch
    n, chi = 20, 256
    sv = S.gaussian_mixture(n, seed)
    p, svd = eng.upload([sv], 1, chi)
    tensors, bonds, target = eng.stage_mps(p, svd, chi)
    tn = eng.overlap(p, target, target).cpu().numpy()[0]
    assert abs(tn - 1.0) < 1e-6, tn
    torch.cuda.synchronize()
    bd = [int(x) for x in bonds.cpu().numpy()[: n + 1]]
    ce = min(chi, 2 ** (n // 2))
    t = tensors.cpu().numpy().view(np.complex128)
    base = int(p.tensor_off[0])
    for c in range(1, n):
        keep, w = bd[c], 2 * bd[c + 1]
        a = t[base + c * 2 * ce * ce: base + c * 2 * ce * ce + keep * w].reshape(keep, w)
        err = np.max(np.abs(a @ a.conj().T - np.eye(keep)))
        assert err < 1e-5, (c, keep, w, err)
