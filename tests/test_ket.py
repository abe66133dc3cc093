"""The statevector wrapper's options on the encoding path
(``MPSEncoder.prepare_state``, reference
qmprs/synthesis/mps_encoding/base.py:96-102): index_type "row" / "snake"
and compression_percentage, as restated in qmprs_gb300/ket.py (quick-core,
which implements them for the reference, is not installed and is
unpinned)."""

import numpy as np
import pytest

from qmprs_gb300.ket import Ket


def test_padding_and_normalisation():
    k = Ket([3.0, 4.0, 0.0])
    assert k.num_qubits == 2
    assert np.allclose(k.data, [0.6, 0.8, 0.0, 0.0])
    with pytest.raises(ValueError):
        Ket([0.0, 0.0])
    with pytest.raises(ValueError):
        Ket([1.0, np.nan])


def test_row_indexing_keeps_the_order():
    v = np.arange(1, 17, dtype=float)
    k = Ket(v)
    before = k.data.copy()
    k.change_indexing("row")
    assert np.array_equal(k.data, before)


def test_snake_reverses_every_odd_row_of_a_square_image():
    img = np.arange(1, 17, dtype=float).reshape(4, 4)
    k = Ket(img)
    k.change_indexing("snake")
    want = np.array([1, 2, 3, 4, 8, 7, 6, 5, 9, 10, 11, 12, 16, 15, 14, 13], dtype=float)
    assert np.allclose(k.data, want / np.linalg.norm(want))


def test_snake_uses_the_rows_of_a_non_square_image():
    img = np.arange(1, 33, dtype=float).reshape(2, 16)       # 2 rows of 16
    k = Ket(img)
    k.change_indexing("snake")
    want = np.concatenate([np.arange(1, 17), np.arange(32, 16, -1)]).astype(float)
    assert np.allclose(k.data, want / np.linalg.norm(want))


def test_snake_of_a_flat_vector_uses_the_default_view():
    v = np.arange(1, 33, dtype=float)                          # 5 qubits: 8 x 4 view
    k = Ket(v)
    k.change_indexing("snake")
    img = v.reshape(8, 4).copy()
    img[1::2] = img[1::2, ::-1]
    assert np.allclose(k.data, img.reshape(-1) / np.linalg.norm(v))


def test_snake_is_an_involution():
    rng = np.random.default_rng(0)
    v = rng.standard_normal(64) + 1j * rng.standard_normal(64)
    k = Ket(v)
    k.change_indexing("snake")
    k.change_indexing("snake")
    assert np.allclose(k.data, v / np.linalg.norm(v))


def test_unknown_index_type_is_rejected():
    with pytest.raises(ValueError, match="index_type"):
        Ket(np.ones(4)).change_indexing("column")


def test_compression_zeroes_the_smallest_amplitudes_and_renormalises():
    v = np.array([0.1, -3.0, 0.2, 2.0, -0.05, 1.0, 0.3, 4.0])
    k = Ket(v)
    k.compress(50.0)                                           # 4 of 8 amplitudes
    want = np.array([0.0, -3.0, 0.0, 2.0, 0.0, 1.0, 0.0, 4.0])
    assert np.allclose(k.data, want / np.linalg.norm(want))
    assert np.isclose(np.linalg.norm(k.data), 1.0)


def test_compression_rounds_the_count_down_and_zero_is_the_identity():
    v = np.arange(1, 9, dtype=float)
    k = Ket(v)
    k.compress(0.0)
    assert np.allclose(k.data, v / np.linalg.norm(v))
    k.compress(20.0)                                           # floor(8 * 0.2) = 1
    assert np.count_nonzero(k.data) == 7 and k.data[0] == 0.0


def test_compression_percentage_out_of_range():
    with pytest.raises(ValueError):
        Ket(np.ones(8)).compress(120.0)
    with pytest.raises(ValueError):
        Ket(np.ones(8)).compress(-1.0)
