"""Golden fixtures (tests/golden/*.npz, made by tests/golden/make_golden.py).

CPU: the oracle reproduces every fixture (guards the checker against drift).
GPU: the CUDA path reproduces them, through the C ABI (engine) and the
reference-facing API.
"""

import os

import numpy as np
import pytest

from oracle import dense as D

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    with np.load(os.path.join(GOLD, name + ".npz")) as z:
        return {k: z[k] for k in z.files}


def up(v):
    v = v.astype(np.complex128)
    return v / np.linalg.norm(v)


# ---- CPU: oracle vs fixtures -------------------------------------------------------


def test_oracle_sv_to_mps_fixtures():
    for name in ["sv_to_mps_n8_chi4", "sv_to_mps_n9_chi64"]:
        g = load(name)
        n = int(round(np.log2(g["sv"].size)))
        ts = D.tt_svd_right(up(g["sv"]), n, int(g["chi"]))
        assert np.array_equal(np.array([t.shape for t in ts]), g["shapes"])
        assert np.allclose(np.concatenate([t.reshape(-1) for t in ts]), g["tensors"], atol=1e-12)
        assert np.allclose(D.mps_to_dense(ts), g["target"], atol=1e-12)


def test_oracle_layer_and_sweep_fixtures():
    g = load("layers_n7_L3")
    t = D.mps_to_dense(D.tt_svd_right(up(g["sv"]), 7, 64))
    layers, fids = D.get_unitary_layers(t, 7, 3)
    assert np.allclose(fids, g["layer_fid"], atol=1e-12)
    s = load("sweeps_n7_L3_S4")
    fs = []
    for _ in range(4):
        layers, f = D.sweep(t, 7, layers)
        fs.append(f)
    assert np.allclose(fs, s["sweep_fid"], atol=1e-12)


def test_oracle_encode_fixtures():
    g = load("encode_n8_chi16_L4_S3")
    r = D.prepare_state(up(g["sv"]), 16, 4, 3)
    assert np.allclose(r.sweep_fidelities, g["sweep_fid"], atol=1e-12)
    assert abs(r.fidelity - float(g["fidelity"])) < 1e-12
    g = load("partial_entanglement_n8")
    r = D.prepare_state(up(g["sv"]), 32, 1, 0)
    assert np.array_equal(np.array([(s, e) for s, e, _ in r.layers[0]]), g["blocks"])


# ---- GPU: CUDA path vs fixtures ----------------------------------------------------


@pytest.mark.gpu
def test_gpu_sv_to_mps_fixtures(cuda_lib):
    from qmprs_gb300 import engine
    for name in ["sv_to_mps_n8_chi4", "sv_to_mps_n9_chi64"]:
        g = load(name)
        res = engine.engine().encode([g["sv"]], int(g["chi"]), num_layers=1, keep_tensors=True)
        got = res.mps_tensors(0)
        assert np.array_equal(np.array([t.shape for t in got]), g["shapes"])
        assert np.allclose(np.concatenate([t.reshape(-1) for t in got]), g["tensors"], atol=2e-5)


@pytest.mark.gpu
def test_gpu_layer_and_sweep_fixtures(cuda_lib):
    from qmprs_gb300 import engine
    g = load("layers_n7_L3")
    s = load("sweeps_n7_L3_S4")
    res = engine.engine().encode([g["sv"]], 64, num_layers=3, num_sweeps=4)
    assert np.allclose(res.layer_fidelities[0], g["layer_fid"], atol=1e-6)
    assert np.allclose(res.sweep_fidelities[0], s["sweep_fid"], atol=1e-6)


@pytest.mark.gpu
def test_gpu_encode_fixtures(cuda_lib):
    from qmprs_gb300.circuit import Circuit
    from qmprs_gb300.synthesis.mps_encoding import Sequential
    g = load("encode_n8_chi16_L4_S3")
    enc = Sequential(Circuit)
    c = enc.prepare_state(statevector=g["sv"], bond_dimension=16, num_layers=4, num_sweeps=3)
    assert np.allclose(enc.last_run["sweep_fidelities"], g["sweep_fid"], atol=1e-6)
    sv = up(g["sv"])
    assert abs(abs(np.vdot(c.get_statevector(), sv)) - float(g["fidelity"])) < 1e-6
    g = load("partial_entanglement_n8")
    c = enc.prepare_state(statevector=g["sv"], bond_dimension=32, num_layers=1)
    from qmprs_gb300 import engine
    res = engine.engine().encode([g["sv"]], 32, num_layers=1)
    blocks = [(s, e) for s, e, _ in res.layers(0)[0]]
    assert np.array_equal(np.array(blocks), g["blocks"])
    assert abs(res.fidelity[0] - float(g["fidelity"])) < 1e-6


@pytest.mark.gpu
def test_gpu_batch_uneven_fixture(cuda_lib):
    from qmprs_gb300 import engine
    g = load("batch_uneven")
    ns = [int(x) for x in g["ns"]]
    offs = np.cumsum([0] + [2 ** n for n in ns])
    svs = [g["sv"][offs[i]: offs[i + 1]] for i in range(len(ns))]
    res = engine.engine().encode(svs, 16, num_layers=3, num_sweeps=2)
    assert np.allclose(res.fidelity, g["fidelity"], atol=1e-6)
    assert np.allclose(res.sweep_fidelities, g["sweep_fid"], atol=1e-6)
