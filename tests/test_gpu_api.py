"""The reference's API on the GPU: the behaviours its own tests assert
(tests/primitives/test_mps.py, tests/synthesis/mps_encoding/test_sequential_encoding.py)."""

import numpy as np
import pytest

from oracle import dense as D
from oracle import states as S

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def api(cuda_lib):
    from qmprs_gb300.circuit import Circuit
    from qmprs_gb300.primitives import MPS
    from qmprs_gb300.synthesis.mps_encoding import Sequential
    return MPS, Sequential, Circuit


def _fid(circuit, sv):
    return abs(np.dot(circuit.get_statevector().conj(), sv))


def test_prepare_state(api):
    MPS, Sequential, Circuit = api
    sv = S.uniform_complex(8, 1)
    c = Sequential(Circuit).prepare_state(statevector=sv, bond_dimension=32, num_layers=32)
    assert 1 - _fid(c, sv) < 1e-2


def test_prepare_mps(api):
    MPS, Sequential, Circuit = api
    sv = S.uniform_complex(8, 2)
    mps = MPS(statevector=sv, bond_dimension=32)
    c = Sequential(Circuit).prepare_mps(mps=mps, num_layers=32)
    assert 1 - _fid(c, sv) < 1e-2


def test_partial_entanglement(api):
    MPS, Sequential, Circuit = api
    from tests.test_oracle import _ghz_like
    sv = _ghz_like(8, [(0, 3), (5, 7)], [0, 4, 5])
    c = Sequential(Circuit).prepare_state(statevector=sv, bond_dimension=32, num_layers=1)
    assert 1 - _fid(c, sv) < 1e-2
    assert c.get_depth() <= 20
    sv = _ghz_like(4, [(0, 1), (1, 2)], [0, 3])
    c = Sequential(Circuit).prepare_state(statevector=sv, bond_dimension=32, num_layers=1, num_sweeps=1)
    assert 1 - _fid(c, sv) < 1e-2
    assert c.get_depth() <= 7


def test_layer_and_sweep_improvement(api):
    MPS, Sequential, Circuit = api
    sv = S.uniform_complex(8, 3)
    enc = Sequential(Circuit)
    f = [_fid(enc.prepare_state(statevector=sv, bond_dimension=64, num_layers=i), sv) for i in range(1, 10)]
    assert np.all(np.diff(f) >= -1e-6)
    f = [_fid(enc.prepare_state(statevector=sv, bond_dimension=64, num_layers=6, num_sweeps=i), sv)
         for i in range(1, 8)]
    assert np.all(np.diff(f) >= -1e-6)


def test_circuit_matches_oracle(api):
    MPS, Sequential, Circuit = api
    sv = S.uniform_complex(7, 4)
    enc = Sequential(Circuit)
    c = enc.prepare_state(statevector=sv, bond_dimension=64, num_layers=3, num_sweeps=2)
    ref = D.prepare_state(sv.astype(np.complex64).astype(complex), 64, 3, 2)
    assert abs(_fid(c, sv) - ref.fidelity) < 1e-6


def test_mps_validation(api):
    MPS, _, _ = api
    with pytest.raises(ValueError):
        MPS([1, 2, 3], bond_dimension=-1)
    with pytest.raises(ValueError):
        MPS([1, 2, 3], bond_dimension=1.2)
    with pytest.raises(ValueError):
        MPS(statevector=np.array([1, 0]), bond_dimension=64)
    with pytest.raises(TypeError):
        MPS(mps="not an MPS", bond_dimension=64)


@pytest.mark.parametrize("n", [2, 4, 8])
def test_from_to_statevector(api, n):
    MPS, _, _ = api
    from qmprs_gb300.ket import Ket
    sv = S.uniform_complex(n, n)
    m = MPS.from_statevector(Ket(sv), 64)
    back = MPS.to_statevector(m)
    assert np.allclose(back.data, sv, atol=1e-6)


@pytest.mark.parametrize("L", [8, 10])
def test_normalize(api, L):
    MPS, _, _ = api
    from qmprs_gb300.primitives import MatrixProductState
    rng = np.random.default_rng(L)
    ts = []
    dims = [1] + [min(8, 2 ** min(i, L - i)) for i in range(1, L)] + [1]
    for i in range(L):
        ts.append(rng.standard_normal((dims[i], 2, dims[i + 1])) + 1j * rng.standard_normal((dims[i], 2, dims[i + 1])))
    m = MPS(mps=MatrixProductState.from_3d(ts), bond_dimension=64)
    assert not m.is_normalized
    m.normalize()
    assert m.is_normalized
    assert m.norm == pytest.approx(1.0, abs=1e-6)


@pytest.mark.parametrize("mode", ["left", "right"])
def test_canonicalize(api, mode):
    MPS, _, _ = api
    m = MPS(statevector=S.uniform_complex(8, 9), bond_dimension=16)
    m.canonicalize(mode=mode, normalize=True)
    assert m.is_normalized
    assert m.canonical_form == mode


@pytest.mark.parametrize("n,max_bond,mode", [(2, 32, "left"), (4, 16, "right"), (8, 8, "left")])
def test_compress_mode(api, n, max_bond, mode):
    MPS, _, _ = api
    m = MPS(statevector=S.uniform_complex(n, 1), bond_dimension=64)
    assert m.bond_dimension == 64
    m.compress(max_bond_dimension=max_bond, mode=mode)
    assert m.bond_dimension == max_bond
    assert m.canonical_form == mode


def test_layer_methods(api):
    MPS, _, _ = api
    n = 6
    sv = S.uniform_complex(n, 5)
    m = MPS(statevector=sv, bond_dimension=64)
    layer = m.generate_bond_D_unitary_layer()
    ref, _ = D.generate_layer(sv.astype(np.complex64).astype(complex), n)
    for (s1, e1, g1), (s2, e2, g2) in zip(layer, ref):
        assert (s1, e1) == (s2, e2)
        for a, b in zip(g1, g2):
            assert np.allclose(a, b, atol=2e-4)
    f_before = m.fidelity_with_zero_state()
    m.apply_unitary_layer(layer, inverse=True)
    f_after = m.fidelity_with_zero_state()
    assert abs(f_after) > abs(f_before)
    psi = D.apply_inverse_layer(sv, n, ref)
    assert abs(f_after - np.conj(psi[0])) < 1e-5


def test_packed_host_input_matches_device(api):
    """Packed complex64 batch from pinned host memory (qmprs_plan_upload into
    the plan's input buffer, reused by the second call) gives bit-identical
    results to the same batch resident on the device; a wrong size is
    rejected."""
    import torch
    _, Sequential, Circuit = api
    ns = [6, 9, 7]
    svs = [S.uniform_complex(n, 40 + n).astype(np.complex64) for n in ns]
    packed = np.concatenate([v.view(np.float32) for v in svs])
    host = torch.from_numpy(packed).pin_memory()
    dev = host.to("cuda")
    cfg = dict(bond_dimension=16, num_layers=2, num_sweeps=2)
    _, rd = Sequential(Circuit).prepare_states(dev, nqubits=ns, emit=False, **cfg)
    for _ in range(2):
        _, rh = Sequential(Circuit).prepare_states(host, nqubits=ns, emit=False, **cfg)
        assert np.array_equal(rh.gates, rd.gates)
        assert np.array_equal(rh.sweep_fidelities, rd.sweep_fidelities)
        assert np.array_equal(rh.fidelity, rd.fidelity)
    with pytest.raises(ValueError):
        Sequential(Circuit).prepare_states(host[:-2], nqubits=ns, emit=False, **cfg)


@pytest.mark.parametrize("n", [12, 14])
def test_compress_without_max_bond_truncates_only_at_the_cutoff(api, n):
    """compress() with no max_bond truncates only at quimb's cutoff
    (reference qmprs/primitives/mps.py:441-453): a random state keeps its
    full bonds (128 at 14 qubits) and the site tensors match the oracle's
    right-canonical ones."""
    MPS, _, _ = api
    sv = S.uniform_complex(n, 4)
    m = MPS(statevector=sv, bond_dimension=512)
    m.compress()
    got = m.mps.tensors3d()
    sv64 = sv.astype(np.complex64).astype(np.complex128)
    ref = D.tt_svd_right(sv64 / np.linalg.norm(sv64), n, 2 ** (n // 2))
    assert max(t.shape[2] for t in got[:-1]) == 2 ** (n // 2)
    for s in range(n):
        assert got[s].shape == ref[s].shape, s
        assert np.max(np.abs(got[s] - ref[s])) < 2e-4, s


def test_prepare_state_applies_snake_indexing_and_compression(api):
    """prepare_state(index_type="snake", compression_percentage=p)
    (reference qmprs/synthesis/mps_encoding/base.py:96-102) encodes the
    re-indexed, compressed state: the same circuit as encoding that state
    directly, and a better fit to it than to the raw input."""
    from qmprs_gb300.ket import Ket
    _, Sequential, Circuit = api
    img = S.uniform_complex(8, 21).reshape(16, 16)
    enc = Sequential(Circuit)
    c1 = enc.prepare_state(img, 64, compression_percentage=30.0, index_type="snake", num_layers=3, num_sweeps=2)
    k = Ket(img)
    k.change_indexing("snake")
    k.compress(30.0)
    c2 = enc.prepare_state(k.data, 64, num_layers=3, num_sweeps=2)
    assert np.allclose(c1.get_statevector(), c2.get_statevector(), atol=1e-6)
    raw = img.reshape(-1) / np.linalg.norm(img)
    assert _fid(c1, k.data) > _fid(c1, raw)


def test_packed_input_with_non_finite_amplitudes_is_rejected(api):
    """The packed batch path skips the statevector wrapper's validation;
    stage (a) checks every state's norm on the device instead."""
    import torch
    _, Sequential, Circuit = api
    good = S.uniform_complex(6, 3).astype(np.complex64)
    bad = S.uniform_complex(7, 4).astype(np.complex64)
    bad[5] = np.nan
    packed = torch.from_numpy(np.concatenate([good, bad]).view(np.float32).copy())
    with pytest.raises(ValueError, match="finite"):
        Sequential(Circuit).prepare_states(packed, 16, num_layers=1, nqubits=[6, 7])
    zero = torch.zeros(2 * 2 ** 6, dtype=torch.float32)
    with pytest.raises(ValueError, match="finite"):
        Sequential(Circuit).prepare_states(zero, 16, num_layers=1, nqubits=[6])
