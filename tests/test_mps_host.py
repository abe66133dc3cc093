"""Host-side conversion of quimb MatrixProductState objects (the reference's
``MPS(mps=...)`` input type, qmprs/primitives/mps.py:183-197) into the
package's (l, p, r) site tensors.  quimb is not installed here: the stand-in
objects carry what the conversion uses of a quimb MPS, ``arrays`` and
``permute_arrays`` / ``copy`` (quimb's own reordering of every site's
indices), or an index-order string ``shape``; a real quimb MPS is tested
where quimb is importable."""

import numpy as np
import pytest

from qmprs_gb300.primitives.mps import MatrixProductState, _from_quimb, _quimb_like


class _QuimbLike:
    def __init__(self, arrays, shape):
        self.arrays = arrays
        self.shape = shape


class _QuimbPermutable:
    """Stores its arrays in some index order it does not expose; reorders
    them on ``permute_arrays`` like quimb's MatrixProductState."""

    def __init__(self, ts, order):
        self._ts = [t.copy() for t in ts]
        self._order = order
        self.arrays = tuple(_as_quimb(self._ts, order))

    def copy(self):
        return _QuimbPermutable(self._ts, self._order)

    def permute_arrays(self, shape="lrp"):
        self._order = shape
        self.arrays = tuple(_as_quimb(self._ts, shape))


def _random_lpr(L, seed):
    rng = np.random.default_rng(seed)
    dims = [1] + [min(4, 2 ** min(i, L - i)) for i in range(1, L)] + [1]
    return [rng.standard_normal((dims[i], 2, dims[i + 1])) + 1j * rng.standard_normal((dims[i], 2, dims[i + 1]))
            for i in range(L)]


def _as_quimb(ts, shape):
    """Open-boundary arrays in quimb's convention for index order `shape`."""
    L = len(ts)
    out = []
    for i, t in enumerate(ts):
        have, a = "lpr", t
        if i == 0:
            a, have = a[0], "pr"
        if i == L - 1:
            a, have = a[..., 0], have.replace("r", "")
        letters = "".join(c for c in shape if c in have)
        out.append(np.transpose(a, [have.index(c) for c in letters]))
    return out


@pytest.mark.parametrize("shape", ["lrp", "lpr", "rlp", "prl", "plr", "rpl"])
def test_quimb_arrays_in_any_index_order(shape):
    ts = _random_lpr(6, 3)
    q = _QuimbLike(_as_quimb(ts, shape), shape)
    assert _quimb_like(q)
    m = _from_quimb(q)
    assert isinstance(m, MatrixProductState)
    assert all(np.array_equal(a, b) for a, b in zip(m.tensors3d(), ts))


def test_non_mps_inputs_are_not_taken_for_quimb():
    assert not _quimb_like("not an MPS")
    assert not _quimb_like(_QuimbLike([], "lrx"))
    with pytest.raises(ValueError):
        _from_quimb(_QuimbLike([np.zeros((2, 2, 2, 2))] * 3, "lrp"))


@pytest.mark.parametrize("order", ["lrp", "rlp", "prl"])
def test_quimb_objects_are_reordered_with_their_own_permute_arrays(order):
    ts = _random_lpr(5, 8)
    q = _QuimbPermutable(ts, order)
    assert _quimb_like(q)
    m = _from_quimb(q)
    assert all(np.array_equal(a, b) for a, b in zip(m.tensors3d(), ts))
    assert q._order == order          # the caller's object is left as it was


def test_real_quimb_mps():
    qtn = pytest.importorskip("quimb.tensor")
    psi = qtn.MPS_rand_state(7, bond_dim=4, seed=3)
    m = _from_quimb(psi)
    dense = m.tensors3d()[0].reshape(2, -1)
    for t in m.tensors3d()[1:]:
        dense = (dense @ t.reshape(t.shape[0], -1)).reshape(-1, t.shape[2])
    assert np.allclose(dense.reshape(-1), psi.to_dense().reshape(-1))
