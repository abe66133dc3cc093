"""GPU parity of the exact precision mode against the FP64 oracle.

The exact mode (``precision="exact"``, ``QMPRS_PRECISION_EXACT``) keeps the
working states in double-float, so the GPU follows an FP64 run of the
reference's algorithm through deep layer stacks, whose bond-2 truncations
amplify rounding by a few times per layer.  The bar is the per-layer and
per-sweep fidelity tolerance FID_TOL = 1e-6; the observed differences are
1e-10 for layers and 1e-8 for sweeps.  Inputs are complex128 on both sides.

The 20- and 24-qubit references and the sample of the benchmark batch take
minutes to an hour in the dense FP64 oracle, so their per-layer and
per-sweep fidelities are committed fixtures (tests/golden/make_large_golden.py)
and the inputs are regenerated from their seeds.
"""

import os

import numpy as np
import pytest

from oracle import dense as D
from oracle import states as S

pytestmark = pytest.mark.gpu

FID_TOL = 1e-6
TENSOR_TOL = 1e-9
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def eng(cuda_lib):
    from qmprs_gb300 import engine
    return engine.engine()


def _oracle(sv, chi, L, S_):
    n = D.num_qubits(sv)
    ts = D.tt_svd_right(sv / np.linalg.norm(sv), n, chi)
    t = D.mps_to_dense(ts)
    layers, lf = D.get_unitary_layers(t, n, L)
    sf = []
    for _ in range(S_):
        layers, f = D.sweep(t, n, layers)
        sf.append(f)
    fid = abs(np.vdot(D.circuit_state(layers, n), sv)) / np.linalg.norm(sv)
    return ts, np.array(lf), np.array(sf), fid


def _max_diffs(res, b, lf, sf):
    L = len(lf)
    assert int(res.num_layers[b]) == L, (b, int(res.num_layers[b]), L)
    dl = np.max(np.abs(res.layer_fidelities[b, :L] - lf)) if L else 0.0
    ds = np.max(np.abs(res.sweep_fidelities[b, : len(sf)] - sf)) if len(sf) else 0.0
    return dl, ds


@pytest.mark.parametrize("ns,chi", [([6], 64), ([9], 4), ([12], 16), ([7, 11, 9], 8)])
def test_exact_sv_to_mps(eng, ns, chi):
    svs = [S.uniform_complex(n, 40 + i) for i, n in enumerate(ns)]
    res = eng.encode(svs, chi, num_layers=1, keep_tensors=True, precision="exact")
    for b, sv in enumerate(svs):
        ref = D.tt_svd_right(sv / np.linalg.norm(sv), ns[b], chi)
        got = res.mps_tensors(b)
        for s in range(ns[b]):
            assert got[s].shape == ref[s].shape, (b, s)
            assert np.max(np.abs(got[s] - ref[s])) < TENSOR_TOL, (b, s, np.max(np.abs(got[s] - ref[s])))


@pytest.mark.parametrize("n,chi", [(16, 128), (18, 256)])
def test_exact_sv_to_mps_wide_bonds(eng, n, chi):
    """Bonds above 64 take the device-wide eigensolver; the projection and
    the target contraction stay in double-float."""
    from qmprs_gb300 import engine as E
    sv = S.uniform_complex(n, 7)
    p, svd = eng.upload([sv], 1, chi, "exact")
    tensors, bonds, target = eng.stage_mps(p, svd, chi)
    ts = D.tt_svd_right(sv / np.linalg.norm(sv), n, chi)
    tref = D.mps_to_dense(ts)
    got = target.cpu().numpy().view(np.complex128)
    assert [int(x) for x in bonds.cpu().numpy()[1:n]] == [t.shape[2] for t in ts[:-1]]
    assert np.max(np.abs(got - tref)) < TENSOR_TOL, np.max(np.abs(got - tref))
    assert isinstance(p, E.Plan) and p.precision == "exact"


def test_exact_small_batch_matches_oracle(eng):
    ns = [5, 8, 11]
    svs = [S.uniform_complex(n, 60 + i) for i, n in enumerate(ns)]
    res = eng.encode(svs, 16, num_layers=4, num_sweeps=5, precision="exact")
    for b, sv in enumerate(svs):
        _, lf, sf, fid = _oracle(sv, 16, 4, 5)
        dl, ds = _max_diffs(res, b, lf, sf)
        assert dl < 1e-7 and ds < 1e-7, (b, dl, ds)
        assert abs(res.fidelity[b] - fid) < 1e-7


def test_exact_readme_configuration_n10(eng):
    """The reference's headline configuration (README: 10 qubits, uniform
    complex state, bond 512, 15 layers, 50 sweeps): every per-layer and
    per-sweep fidelity within 1e-6 of the FP64 oracle."""
    sv = S.uniform_complex(10, 11)
    res = eng.encode([sv], 512, num_layers=15, num_sweeps=50, precision="exact")
    _, lf, sf, fid = _oracle(sv, 512, 15, 50)
    dl, ds = _max_diffs(res, 0, lf, sf)
    print(f"10 qubits, L15 S50: max layer diff {dl:.2e}, max sweep diff {ds:.2e}, final {sf[-1]:.9f}")
    assert dl < FID_TOL and ds < FID_TOL, (dl, ds)
    assert abs(res.fidelity[0] - fid) < FID_TOL


def test_exact_deterministic(eng):
    svs = [S.uniform_complex(n, 70 + i) for i, n in enumerate([9, 13])]
    a = eng.encode(svs, 32, num_layers=3, num_sweeps=3, precision="exact")
    b = eng.encode(svs, 32, num_layers=3, num_sweeps=3, precision="exact")
    assert np.array_equal(a.sweep_fidelities, b.sweep_fidelities)
    assert np.array_equal(a.gates, b.gates)


def test_exact_partial_entanglement_blocks(eng):
    """Block detection and early exit in the exact mode: the golden
    partially entangled 8-qubit state (product of small blocks)."""
    g = np.load(os.path.join(GOLDEN, "partial_entanglement_n8.npz"))
    sv = g["sv"].astype(np.complex128)
    res = eng.encode([sv], 64, num_layers=3, num_sweeps=1, precision="exact")
    _, lf, sf, _ = _oracle(sv, 64, 3, 1)
    dl, ds = _max_diffs(res, 0, lf, sf)
    assert dl < 1e-7 and ds < 1e-7, (dl, ds)


def _need(name):
    path = os.path.join(GOLDEN, name)
    if not os.path.exists(path):
        pytest.fail(f"missing fixture {name}: run tests/golden/make_large_golden.py")
    return np.load(path)


def test_exact_n20_configuration(eng):
    """20 qubits, uniform complex, bond 256, 10 layers, 20 sweeps against
    the committed FP64 oracle run."""
    g = _need("c2_n20.npz")
    sv = S.uniform_complex(int(g["n"]), int(g["seed"]))
    res = eng.encode([sv], int(g["chi"]), num_layers=int(g["L"]), num_sweeps=int(g["S"]), precision="exact")
    dl, ds = _max_diffs(res, 0, g["layer_fid"], g["sweep_fid"])
    print(f"20 qubits, bond 256, L10 S20: max layer diff {dl:.2e}, max sweep diff {ds:.2e}")
    assert dl < FID_TOL and ds < FID_TOL, (dl, ds)
    assert abs(res.fidelity[0] - float(g["fidelity"])) < FID_TOL


def _c4_sample():
    import bench
    g = _need("c4_sample.npz")
    ns, bonds, _, _ = bench.workload_spec("batched", 512, int(g["seed"]))
    idx = [int(i) for i in g["indices"]]
    assert [ns[i] for i in idx] == [int(x) for x in g["nqubits"]]
    return g, S.random_mps_batch(ns, bonds, int(g["seed"]), idx)


def test_exact_benchmark_batch_sample(eng):
    """Eight states of the benchmark batch (12 to 22 qubits), encoded as one
    batch at bond 64, 6 layers, 10 sweeps."""
    g, svs = _c4_sample()
    res = eng.encode(svs, int(g["chi"]), num_layers=int(g["L"]), num_sweeps=int(g["S"]), precision="exact")
    worst = 0.0
    for k in range(len(svs)):
        L = int(g["num_layers"][k])
        dl, ds = _max_diffs(res, k, g["layer_fid"][k, :L], g["sweep_fid"][k])
        worst = max(worst, dl, ds)
        assert dl < FID_TOL and ds < FID_TOL, (k, int(g["nqubits"][k]), dl, ds)
        assert abs(res.fidelity[k] - float(g["fidelity"][k])) < FID_TOL
    print(f"benchmark sample (8 states, 12-22 qubits): max difference {worst:.2e}")


def test_fast_mode_error_on_benchmark_sample(eng):
    """The fast mode (complex64 states, split-FP16 tensor-core products) on
    the same eight states: its per-layer and per-sweep fidelities stay within
    1e-4 of the FP64 run (4.1e-5 measured; the input rounded to complex64
    included)."""
    g, svs = _c4_sample()
    res = eng.encode(svs, int(g["chi"]), num_layers=int(g["L"]), num_sweeps=int(g["S"]))
    worst = 0.0
    for k in range(len(svs)):
        L = int(g["num_layers"][k])
        if int(res.num_layers[k]) != L:
            continue
        dl, ds = _max_diffs(res, k, g["layer_fid"][k, :L], g["sweep_fid"][k])
        worst = max(worst, dl, ds)
    print(f"fast mode on the benchmark sample: max difference {worst:.2e}")
    assert worst < 1e-4


def test_prepare_state_exact_precision_through_the_reference_api(cuda_lib):
    """``Sequential.prepare_state(..., precision="exact")``: the reference's
    entry point (qmprs/synthesis/mps_encoding/base.py:58-106) with the
    double-float mode; per-layer and per-sweep fidelities (``last_run``) and
    the emitted circuit's state against the FP64 oracle."""
    from qmprs_gb300.circuit import Circuit
    from qmprs_gb300.synthesis.mps_encoding import Sequential
    sv = S.uniform_complex(9, 5)
    enc = Sequential(Circuit)
    c = enc.prepare_state(sv, 32, num_layers=8, num_sweeps=6, precision="exact")
    _, lf, sf, fid = _oracle(sv, 32, 8, 6)
    assert len(enc.last_run["layer_fidelities"]) == len(lf)
    assert np.max(np.abs(enc.last_run["layer_fidelities"] - lf)) < FID_TOL
    assert np.max(np.abs(enc.last_run["sweep_fidelities"] - sf)) < FID_TOL
    assert abs(abs(np.vdot(c.get_statevector(), sv)) - fid) < 1e-5
