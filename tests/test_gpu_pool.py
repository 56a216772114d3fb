"""The pooled transport kernel (event-sorted warps over pools of histories)
against the oracle and against the history kernel, through the C-ABI.

FP64 mode: per-event traces (kind, group, cell, rng state bit-exact;
positions and directions within 1e-12 relative), fission banks, scores and
tallies, power iterations -- the same bars as the history kernel's parity
tests.  FP32-tracking mode: the pooled kernel runs each history through the
same operations as the history kernel, so the fission bank and the counts
match it bit for bit; the scores, whose per-history terms are summed in FP32,
agree within 1e-7 relative.
"""
import numpy as np
import pytest

import oracle
from abeille_gb300 import Engine, decks
from abeille_gb300.abi import AbxError

from test_gpu_parity import RTOL, close, compare_traces

pytestmark = pytest.mark.gpu


def pooled(builder, precision="fp64"):
    eng = Engine(builder.build(precision=precision), 0)
    eng.set_transport_kernel("pool")
    assert eng.transport_kernel() == "pool"
    return eng


@pytest.mark.parametrize("deck,tracking", [("config0", "delta-tracking"), ("config0", "surface-tracking"),
                                           ("config2", "delta-tracking"), ("config2", "surface-tracking"),
                                           ("quadrics", "delta-tracking"), ("quadrics", "surface-tracking")])
def test_pool_traces_match_per_history(deck, tracking):
    b = getattr(decks, deck)(nparticles=256, tracking=tracking)
    eng = pooled(b)
    ora = oracle.Oracle(b.build(precision="fp64"), nthreads=1)
    bank = ora.sample_sources(0, 256)
    eng.set_trace(96, 1 << 21)
    ora.set_trace(96, 1 << 21)
    eng.transport(bank, 1.0, True)
    ora.transport(bank, 1.0, True)
    compare_traces(eng.get_trace(), ora.get_trace())
    eng.close()


@pytest.mark.parametrize("cfg,tracking", [(0, "delta-tracking"), (1, "delta-tracking"), (2, "surface-tracking"),
                                          (2, "delta-tracking")])
def test_pool_transport_step_matches(cfg, tracking):
    n = 4096 if cfg != 2 else 1024
    b = decks.CONFIGS[cfg](nparticles=n, tracking=tracking)
    eng = pooled(b)
    ora = oracle.Oracle(b.build(precision="fp64"), nthreads=oracle.cores())
    bank = ora.sample_sources(0, n)
    sg, cg = eng.transport(bank, 1.1, True)
    sc, cc = ora.transport(bank, 1.1, True)
    assert len(sg) == len(sc)
    assert np.array_equal(sg["parent_history_id"], sc["parent_history_id"])
    assert np.array_equal(sg["parent_daughter_id"], sc["parent_daughter_id"])
    assert np.array_equal(sg["wgt"], sc["wgt"]) and np.array_equal(sg["E"], sc["E"])
    assert close(sg["r"], sc["r"], atol=1e-9) and close(sg["u"], sc["u"], atol=1e-9)
    for k in ("collisions", "flights", "lost"):
        assert cg[k] == cc[k], k
    for k in ("k_col", "k_abs", "k_trk", "leakage", "mig_area"):
        assert abs(cg[k] - cc[k]) <= RTOL * abs(cc[k]) + 1e-300, (k, cg[k], cc[k])
    tg, tc = eng.tally(0)["gen"], ora.tally(0)["gen"]
    assert np.array_equal(tg != 0, tc != 0)
    assert close(tg, tc, rtol=1e-9 if cfg == 2 else RTOL, atol=0.0)
    eng.close()


@pytest.mark.parametrize("graphs", [False, True])
def test_pool_power_iteration_matches(graphs):
    b = decks.config0(nparticles=2000)
    eng = pooled(b)
    eng.set_graphs(graphs)
    ora = oracle.Oracle(b.build(precision="fp64"), nthreads=oracle.cores())
    sg, kg, hg = eng.run_power_iteration(6, 2)
    sc, kc, hc = ora.run_power_iteration(6, 2)
    assert np.allclose(kg, kc, rtol=1e-11, atol=0) and np.allclose(hg, hc, rtol=1e-11, atol=0)
    assert sg["collisions"] == sc["collisions"] and sg["histories"] == sc["histories"]
    assert np.allclose(eng.tally(0)["avg"], ora.tally(0)["avg"], rtol=1e-10, atol=0)
    eng.close()


@pytest.mark.parametrize("cfg,tracking", [(0, "delta-tracking"), (1, "delta-tracking"), (2, "surface-tracking")])
def test_pool_matches_history_kernel_in_mixed_mode(cfg, tracking):
    n = 20000
    b = decks.CONFIGS[cfg](nparticles=n, tracking=tracking)
    out = {}
    for kind in ("history", "pool"):
        eng = Engine(b.build(precision="mixed"), 0)
        eng.set_transport_kernel(kind)
        bank = eng.sample_sources(0, n)
        out[kind] = eng.transport(bank, 1.1, True) + (eng.tally(0)["gen"],)
        eng.close()
    (sh, ch, th), (sp, cp, tp) = out["history"], out["pool"]
    assert len(sh) == len(sp)
    assert np.array_equal(sh["parent_history_id"], sp["parent_history_id"])
    assert np.array_equal(sh["parent_daughter_id"], sp["parent_daughter_id"])
    assert np.array_equal(sh["r"], sp["r"]) and np.array_equal(sh["u"], sp["u"])
    for k in ("collisions", "flights", "lost"):
        assert ch[k] == cp[k], k
    # per-history score terms are summed in FP32 in this mode; the compiler
    # may contract their products into FMAs differently in the two kernels
    for k in ("k_col", "k_abs", "k_trk", "leakage", "mig_area"):
        assert abs(ch[k] - cp[k]) <= 1e-7 * abs(ch[k]) + 1e-300, (k, ch[k], cp[k])
    assert close(th, tp, rtol=1e-7, atol=0.0)


def test_pool_refuses_what_it_does_not_serve():
    b = decks.fixed_source_problem(3, precision="fp64", nparticles=512, tracking="carter-tracking")
    eng = Engine(b.build(precision="fp64"), 0)
    with pytest.raises(AbxError) as e:
        eng.set_transport_kernel("pool")
    assert e.value.code == 9
    assert eng.transport_kernel() == "history"
    eng.close()
