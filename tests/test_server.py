"""The request loop (abx_server_*): admission, rounds, and each result equal to
its problem run alone.

CPU tests cover submission checks and the failure path (without a GPU every
round fails with ABX_ERR_CUDA and each request reports it).  GPU tests submit
problems at random times so that rounds hold different mixes, and compare
every request with the same problem run alone: collisions, flights and
histories bit-exactly, leakage and tally bins within 1e-12 relative (FP64).
"""
import time

import numpy as np
import pytest

from abeille_gb300 import BatchEngine, Engine, Server, decks
from abeille_gb300.abi import AbxError


def _problem(i, precision="fp64", hmax=600, nb=3):
    b = decks.fixed_source_problem(i, precision=precision, batches=nb)
    b.nparticles = min(b.nparticles, hmax)
    return b


def _collect(srv, n, timeout_s=120):
    got, t0 = {}, time.time()
    while len(got) < n and time.time() - t0 < timeout_s:
        for r in srv.poll(64, 200):
            got[r["request_id"]] = r
    assert len(got) == n, (len(got), n)
    return got


def test_submit_checks_without_device_work():
    srv = Server(precision="fp64", nbatches=3)
    k = decks.config0(nparticles=100).build(precision="fp64")
    with pytest.raises(AbxError) as e:
        srv.submit(k)
    assert e.value.code == 9
    m = _problem(0, "mixed").build(precision="mixed")
    with pytest.raises(AbxError) as e:
        srv.submit(m)
    assert e.value.code == 9
    srv.close()
    tiny = Server(precision="fp64", nbatches=3, hbm_budget_bytes=1 << 16)
    with pytest.raises(AbxError) as e:
        tiny.submit(_problem(1).build(precision="fp64"))
    assert e.value.code == 11
    tiny.close()


def test_round_failure_is_reported_per_request():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("needs a machine without a GPU")
    srv = Server(precision="fp64", nbatches=2)
    ids = [srv.submit(_problem(i).build(precision="fp64"), tag=100 + i) for i in range(3)]
    got = _collect(srv, 3, 60)
    for i, rid in enumerate(ids):
        assert got[rid]["status"] == 6 and got[rid]["tag"] == 100 + i
    st = srv.stats()
    assert st["submitted"] == 3 and st["completed"] == 3 and st["failed"] == 3
    srv.close()


@pytest.mark.gpu
@pytest.mark.parametrize("budget,max_round", [(0, 0), (3 << 20, 0), (0, 1)])
def test_each_request_equals_its_problem_alone(budget, max_round):
    nb = 3
    builders = [_problem(i, nb=nb) for i in range(10)]
    builts = [b.build(precision="fp64") for b in builders]
    srv = Server(precision="fp64", nbatches=nb, hbm_budget_bytes=budget, max_round_problems=max_round)
    rng = np.random.default_rng(5)
    ids = []
    for i, bt in enumerate(builts):
        ids.append(srv.submit(bt, tag=i))
        time.sleep(float(rng.exponential(0.002)))
    got = _collect(srv, len(ids))
    st = srv.stats()
    if max_round == 1:
        assert st["rounds"] == len(ids)
    for i, rid in enumerate(ids):
        r = got[rid]
        assert r["status"] == 0 and r["tag"] == i
        alone = Engine(builts[i], 0)
        sa = alone.run_fixed_source(nb, builders[i].nparticles)
        assert r["collisions"] == sa["collisions"] and r["flights"] == sa["flights"], i
        assert r["histories"] == sa["histories"] == nb * builders[i].nparticles
        assert abs(r["leak_avg"] - sa["leak_avg"]) <= 1e-12 * abs(sa["leak_avg"]), i
        avg, var = srv.tally(rid, r["n_tally_bins"])
        ta = alone.tally(0)
        assert np.allclose(avg, ta["avg"], rtol=1e-12, atol=0), i
        assert np.allclose(var, ta["var"], rtol=1e-9, atol=1e-300), i
        srv.release(rid)
        alone.close()
    assert st["completed"] == len(ids) and st["failed"] == 0
    srv.close()


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_request_admitted_while_another_runs(precision):
    """Continuous batching: a long request goes on the device, then short
    ones arrive.  Each short one is admitted at once into its own round on
    another lane, runs while the long one is still on the device (its
    launch takes SM slots as the long launch's blocks retire) and finishes
    first; every result equals its problem run alone in a batch context of
    its own (the same kernels): counts bit-exact, leakage and tally bins
    within 1e-12 relative."""
    nb = 4
    big = _problem(0, precision, hmax=400000 if precision == "mixed" else 100000, nb=nb)
    small = [_problem(i, precision, hmax=800, nb=nb) for i in range(1, 4)]
    builts = [b.build(precision=precision) for b in [big] + small]
    srv = Server(precision=precision, nbatches=nb, lanes=3)
    ids = [srv.submit(builts[0], tag=0)]
    time.sleep(0.02)
    for i, bt in enumerate(builts[1:], 1):
        ids.append(srv.submit(bt, tag=i))
        time.sleep(0.001)
    got = _collect(srv, len(ids))
    rb = got[ids[0]]
    assert rb["status"] == 0
    for rid in ids[1:]:
        r = got[rid]
        assert r["status"] == 0 and r["round"] != rb["round"], (r, rb)
        assert r["latency_ms"] < rb["latency_ms"], (r["latency_ms"], rb["latency_ms"])
    for i, rid in enumerate(ids):
        r = got[rid]
        alone = BatchEngine([builts[i]], 0)
        (sa,), _ = alone.run(nb)
        assert r["collisions"] == sa["collisions"] and r["flights"] == sa["flights"], i
        assert r["histories"] == sa["histories"] == nb * ([big] + small)[i].nparticles
        assert abs(r["leak_avg"] - sa["leak_avg"]) <= 1e-12 * abs(sa["leak_avg"]), i
        avg, _ = srv.tally(rid, r["n_tally_bins"])
        assert np.allclose(avg, alone.tally_all()[0], rtol=1e-12, atol=0), i
        alone.close()
    srv.close()
