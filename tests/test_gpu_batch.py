"""Batches of fixed-source problems (abx_create_batch / abx_run_fixed_source_batch).

Each problem of a batch must give the results FixedSource::run gives for it
alone (src/fixed_source.cpp:81-173): the oracle run of that single problem,
and the GPU run of that single problem.  Integer results (collisions,
flights, histories) are compared bit-exactly; leakage and tally bins within
1e-12 relative in FP64 (FP64 atomic additions in a different order) and, for
the mixed mode, the same integers bit-exactly and the scores within 1e-6
(FP32 tracking arithmetic is identical alone and in the mix; the FP64 sums
only change order).
"""
import numpy as np
import pytest

import oracle
from abeille_gb300 import BatchEngine, Engine, decks
from abeille_gb300.abi import AbxError

pytestmark = pytest.mark.gpu

NPROB = 8
NBATCH = 3


def _problems(precision, n=NPROB, nparticles=None):
    return [decks.fixed_source_problem(i, precision=precision, nparticles=nparticles, batches=NBATCH)
            for i in range(n)]


def _cap(b, hmax=400):
    b.nparticles = min(b.nparticles, hmax)
    return b


def test_batch_matches_oracle_per_problem():
    builders = [_cap(b) for b in _problems("fp64")]
    builts = [b.build(precision="fp64") for b in builders]
    assert len({b.G for b in builders}) > 1  # the batch mixes group structures
    eng = BatchEngine(builts, 0)
    rows, tot = eng.run(NBATCH)
    assert tot["histories"] == NBATCH * sum(b.nparticles for b in builders)
    for p, (b, built) in enumerate(zip(builders, builts)):
        o = oracle.Oracle(built, nthreads=oracle.cores())
        sc = o.run_fixed_source(NBATCH, b.nparticles)
        r = rows[p]
        assert r["histories"] == NBATCH * b.nparticles
        assert r["collisions"] == sc["collisions"], (p, r["collisions"], sc["collisions"])
        assert r["flights"] == sc["flights"], p
        assert abs(r["leak_avg"] - sc["leak_avg"]) <= 1e-12 * abs(sc["leak_avg"]), p
        assert abs(r["leak_std"] - sc["leak_std"]) <= 1e-9 * abs(sc["leak_std"]) + 1e-15, p
        tg, tc = eng.tally(r["tally_first"]), o.tally(0)
        assert tg["generations"] == tc["generations"] == NBATCH
        assert np.allclose(tg["avg"], tc["avg"], rtol=1e-10, atol=0), p
    # one read of every bin: the problems' tallies one after the other
    avg_all, var_all = eng.tally_all()
    per = [eng.tally(r["tally_first"]) for r in rows]
    assert np.array_equal(avg_all, np.concatenate([t["avg"] for t in per]))
    assert np.array_equal(var_all, np.concatenate([t["var"] for t in per]))
    eng.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_each_result_is_the_same_alone_and_in_the_mix(precision):
    builders = [_cap(b, 2000) for b in _problems(precision)]
    builts = [b.build(precision=precision) for b in builders]
    eng = BatchEngine(builts, 0)
    rows, _ = eng.run(NBATCH)
    tol = 1e-12 if precision == "fp64" else 1e-6
    for p, (b, built) in enumerate(zip(builders, builts)):
        alone = Engine(built, 0)
        st = alone.run_fixed_source(NBATCH, b.nparticles)
        r = rows[p]
        assert r["collisions"] == st["collisions"] and r["flights"] == st["flights"], p
        assert r["histories"] == st["histories"], p
        assert abs(r["leak_avg"] - st["leak_avg"]) <= tol * abs(st["leak_avg"]), p
        ta, tb = alone.tally(0)["avg"], eng.tally(r["tally_first"])["avg"]
        assert np.allclose(tb, ta, rtol=tol, atol=0), p
        alone.close()
    eng.close()


def test_batch_rejects_mixed_modes():
    a = decks.fixed_source_problem(0, precision="fp64", nparticles=100).build(precision="fp64")
    k = decks.config0(nparticles=100).build(precision="fp64")
    with pytest.raises(AbxError) as e:
        BatchEngine([a, k], 0)
    assert e.value.code == 9
    m = decks.fixed_source_problem(1, precision="mixed", nparticles=100).build(precision="mixed")
    with pytest.raises(AbxError) as e:
        BatchEngine([a, m], 0)
    assert e.value.code == 9


def test_replace_gives_the_results_of_a_fresh_context():
    first = [b.build(precision="fp64") for b in (_cap(b) for b in _problems("fp64", 5))]
    second_b = [_cap(decks.fixed_source_problem(100 + i, precision="fp64", batches=NBATCH)) for i in range(7)]
    second = [b.build(precision="fp64") for b in second_b]
    eng = BatchEngine(first, 0)
    eng.run(NBATCH)
    eng.replace(second)
    rows, _ = eng.run(NBATCH)
    fresh = BatchEngine(second, 0)
    rows_f, _ = fresh.run(NBATCH)
    for p, (r, f) in enumerate(zip(rows, rows_f)):
        assert r["collisions"] == f["collisions"] and r["flights"] == f["flights"], p
        assert abs(r["leak_avg"] - f["leak_avg"]) <= 1e-12 * abs(f["leak_avg"]), p
        assert np.allclose(eng.tally(r["tally_first"])["avg"], fresh.tally(f["tally_first"])["avg"],
                           rtol=1e-12, atol=0), p
    eng.close()
    fresh.close()
