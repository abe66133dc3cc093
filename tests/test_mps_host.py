"""Host-side conversion of quimb MatrixProductState objects (the reference's
``MPS(mps=...)`` input type, qmprs/primitives/mps.py:183-197) into the
package's (l, p, r) site tensors.  quimb is not installed here: the test
objects carry what the conversion reads from a quimb MPS, ``arrays`` and the
index order ``shape``."""

import numpy as np
import pytest

from qmprs_gb300.primitives.mps import MatrixProductState, _from_quimb, _quimb_like


class _QuimbLike:
    def __init__(self, arrays, shape):
        self.arrays = arrays
        self.shape = shape


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
