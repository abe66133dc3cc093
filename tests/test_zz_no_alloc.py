"""qmprs_overlap_noalloc: the overlap entry point that allocates nothing.

It exists for callers that cannot call cudaMalloc (their GPU memory is held
by another allocator, or they cannot afford the device synchronisation that
cudaMalloc/cudaFree imply).  The test calls it through the C ABI twice in a
row, on two different batches, and compares each result with the planned
entry point qmprs_overlap within the fidelity tolerance the GPU tests use.
This file is collected last so that a run stopping at the first failure has
already run every other test.
"""

import ctypes

import numpy as np
import pytest

from oracle import states as S

pytestmark = pytest.mark.gpu

TOL = 1e-6


def _batch(ns, seed):
    a = [S.uniform_complex(n, seed + i) for i, n in enumerate(ns)]
    b = [S.random_mps(n, 4, seed + 100 + i) for i, n in enumerate(ns)]
    pack = lambda vs: np.concatenate([v.astype(np.complex64) for v in vs])
    return pack(a), pack(b)


def test_overlap_noalloc_matches_planned_overlap(cuda_lib):
    import torch

    from qmprs_gb300 import engine

    eng = engine.engine()
    lib = cuda_lib
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for ns, seed in (([6, 13, 9, 16], 1), ([12, 5, 20], 7)):
        a, b = _batch(ns, seed)
        da = torch.from_numpy(a.view(np.float32)).cuda()
        db = torch.from_numpy(b.view(np.float32)).cuda()
        out = torch.zeros(2 * len(ns), dtype=torch.float64, device="cuda")
        nq = (ctypes.c_int * len(ns))(*ns)
        rc = lib.qmprs_overlap_noalloc(ctypes.c_void_p(da.data_ptr()), ctypes.c_void_p(db.data_ptr()), len(ns), nq,
                                       ctypes.c_void_p(out.data_ptr()), stream)
        assert rc == 0
        p = eng.plan(ns, 1, 2)
        ref = eng.overlap(p, da, db)
        torch.cuda.synchronize()
        got = out.cpu().numpy().view(np.complex128)
        want = ref.cpu().numpy().view(np.complex128)
        assert np.allclose(got, want, rtol=0, atol=TOL)
        exact = np.array([np.vdot(a[o:o + 2 ** n].astype(np.complex128), b[o:o + 2 ** n].astype(np.complex128))
                          for o, n in zip(np.cumsum([0] + [2 ** n for n in ns])[:-1], ns)])
        assert np.allclose(got, exact, rtol=0, atol=TOL)


def _noalloc(lib, da, db, ns):
    import torch
    out = torch.zeros(2 * len(ns), dtype=torch.float64, device="cuda")
    nq = (ctypes.c_int * len(ns))(*ns)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = lib.qmprs_overlap_noalloc(ctypes.c_void_p(da.data_ptr()), ctypes.c_void_p(db.data_ptr()), len(ns), nq,
                                   ctypes.c_void_p(out.data_ptr()), stream)
    assert rc == 0
    return out


@pytest.mark.parametrize("ns", [[25], [12] * 63 + [4]])
def test_overlap_noalloc_at_its_limits(cuda_lib, ns):
    """Requests that fill the static scratch exactly: one 25-qubit state
    (8192 tiles of 4096 amplitudes) and a 64-state batch."""
    import torch

    from qmprs_gb300 import engine

    a, b = _batch(ns, 31)
    da = torch.from_numpy(a.view(np.float32)).cuda()
    db = torch.from_numpy(b.view(np.float32)).cuda()
    out = _noalloc(cuda_lib, da, db, ns)
    p = engine.engine().plan(ns, 1, 2)
    ref = engine.engine().overlap(p, da, db)
    torch.cuda.synchronize()
    got = out.cpu().numpy().view(np.complex128)
    assert np.allclose(got, ref.cpu().numpy().view(np.complex128), rtol=0, atol=TOL)
    offs = np.cumsum([0] + [2 ** n for n in ns])[:-1]
    exact = np.array([np.vdot(a[o:o + 2 ** n].astype(np.complex128), b[o:o + 2 ** n].astype(np.complex128))
                      for o, n in zip(offs, ns)])
    assert np.allclose(got, exact, rtol=0, atol=TOL)


def test_overlap_noalloc_rejects_oversized_requests(cuda_lib):
    nq = (ctypes.c_int * 1)(26)                     # 2^14 tiles > the 8192-tile limit
    rc = cuda_lib.qmprs_overlap_noalloc(ctypes.c_void_p(1), ctypes.c_void_p(1), 1, nq, ctypes.c_void_p(1), None)
    assert rc == 2                                  # QMPRS_ERR_UNSUPPORTED, nothing launched
    nq = (ctypes.c_int * 65)(*([4] * 65))
    rc = cuda_lib.qmprs_overlap_noalloc(ctypes.c_void_p(1), ctypes.c_void_p(1), 65, nq, ctypes.c_void_p(1), None)
    assert rc == 2
