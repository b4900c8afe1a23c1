"""Batched ensembles of independent R^3 realisations: one force evaluation +
fixed-dt KDK steps in one persistent work-list kernel per phase, captured in
a CUDA graph, against the plain per-realisation path and against the oracle
(StePS/src/step.cc:100-312 restated) run realisation by realisation."""
import math

import numpy as np
import pyoracle as O
import pytest

import steps_gb300 as S
from helpers import err_stats, port_params
from steps_gb300 import workloads as W

pytestmark = pytest.mark.gpu

SIZES = [4096, 300, 1500, 777, 2048, 128]
DT = 1e-3


def ensemble():
    return [W.r3_compactified(n, 200.0 + 100.0 * k, seed=40 + k, displace=True) for k, n in enumerate(SIZES)]


def oracle_run(port, ps, nsteps):
    s = port.system(0, ps.m, ps.eps, port_params(O))
    F0 = port.forces(s, ps.x)
    rho_part = ps.m.min() / (4.0 * math.pi * 0.05 ** 3 / 3.0)
    x, v, F, _ = port.kdk(s, nsteps, DT, ps.x, np.zeros_like(ps.x), F0, rho_part=rho_part)
    return x, v, F


@pytest.mark.parametrize("mode", [1, 2])
def test_batch_graph_and_plain_match_oracle(engine, port, mode):
    """mode 1: the whole run in one persistent kernel under a CUDA graph;
    mode 2: a CUDA graph of per-phase kernels."""
    sets = ensemble()
    p = S.params(S.R3)
    engine.set_variant(1)
    try:
        engine.batch_set([s.x for s in sets], [s.m for s in sets], [s.eps for s in sets])
        engine.batch_run(p, S.MIXED, 2, DT, graph=mode)
        graph = [engine.batch_get(k) for k in range(len(sets))]
        engine.batch_run(p, S.MIXED, 2, DT, graph=mode)  # replays the captured graph: 4 steps in all
        graph4 = [engine.batch_get(k) for k in range(len(sets))]
        engine.batch_set([s.x for s in sets], [s.m for s in sets], [s.eps for s in sets])
        engine.batch_run(p, S.MIXED, 2, DT, graph=0)
        plain = [engine.batch_get(k) for k in range(len(sets))]
        # same sizes registered again: new data, the tuned plan and graph are reused
        engine.batch_set([s.x for s in sets], [s.m for s in sets], [s.eps for s in sets])
        engine.batch_run(p, S.MIXED, 2, DT, graph=mode)
        again = [engine.batch_get(k) for k in range(len(sets))]
    finally:
        engine.set_variant(0)
    for k, ps in enumerate(sets):
        xo, vo, Fo = oracle_run(port, ps, 2)
        for name, (x, v, F) in (("graph", graph[k]), ("plain", plain[k])):
            assert np.abs(x - xo).max() < 1e-9 * (1 + np.abs(xo).max()), (k, name)
            assert err_stats(F, Fo)["p99"] < 1e-5, (k, name)
            assert err_stats(v, vo)["p99"] < 1e-5, (k, name)
        # Two tilings of the same realisation round independently, each within
        # the p99 bar of the oracle; their difference is held to that bar too.
        d = err_stats(graph[k][2], plain[k][2])
        assert d["p99"] < 1e-5 and d["max"] < 5e-5, (k, d)
        for a, b in zip(again[k], graph[k]):
            assert np.array_equal(a, b), k  # deterministic reduction order
        xo4, vo4, Fo4 = oracle_run(port, ps, 4)
        assert err_stats(graph4[k][2], Fo4)["p99"] < 1e-5, k
        assert np.abs(graph4[k][0] - xo4).max() < 1e-9 * (1 + np.abs(xo4).max()), k


def test_batch_errors(engine):
    with pytest.raises(S.StepsError) as e:
        engine.batch_set([], [], [])
    assert e.value.code == S.STEPS_E_ARG
    sets = ensemble()[:2]
    engine.batch_set([s.x for s in sets], [s.m for s in sets], [s.eps for s in sets])
    with pytest.raises(S.StepsError) as e:
        engine.batch_run(S.params(S.T3, is_periodic=2, L=100.0), S.MIXED, 1, DT)
    assert e.value.code == S.STEPS_E_ARG
