"""CUDA-graph replay of the layer and sweep stages (qmprs_plan_set_graphs)
against the launch-by-launch path: bit-identical gates and fidelities.

The batch mixes states that leave the layer stage early (a two-block
product state disentangles in one layer) or stop sweeping at the stop
fidelity with states that run every layer and sweep, so the replayed graph,
which enqueues every layer and sweep and leaves finished states to the
kernels' active flags, is compared with the path that stops at the first
layer or sweep after which no state is left."""

import numpy as np
import pytest

from oracle import states as S

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eng(cuda_lib):
    from qmprs_gb300 import engine
    return engine.engine()


def _batch():
    from tests.test_oracle import _ghz_like
    return [S.random_mps(9, 2, 3), S.uniform_complex(11, 4), _ghz_like(8, [(0, 2), (5, 7)], [0, 5]),
            S.random_mps(12, 4, 5)]


def _fields(r):
    return [r.gates, r.arity, r.num_layers, r.layer_fidelities, r.sweep_fidelities, r.sweeps_done, r.fidelity]


@pytest.mark.parametrize("precision", ["fast", "exact"])
@pytest.mark.parametrize("stop", [0.0, 0.9])
def test_graph_replay_is_bit_identical(eng, precision, stop):
    svs = _batch()
    kw = dict(num_layers=5, num_sweeps=6, stop_fidelity=stop, precision=precision)
    ns = [int(np.log2(len(v))) for v in svs]
    p = eng.plan(ns, 5, 16, precision)
    eng.set_graphs(p, False)
    ref = eng.encode(svs, 16, **kw)
    eng.set_graphs(p, True)
    _, before = eng.graph_stats(p)
    runs = [eng.encode(svs, 16, **kw) for _ in range(4)]      # direct, capture, replay, replay
    cached, after = eng.graph_stats(p)
    assert cached >= 2 and after - before >= 6, (cached, before, after)
    for r in runs:
        for a, b in zip(_fields(r), _fields(ref)):
            assert np.array_equal(a, b)
    assert int(ref.num_layers[2]) < 5                         # the product state left the layer stage early
