"""Edge cases of the transport step through the C-ABI, against the oracle:
an empty bank, bank sizes that are not multiples of a warp or a block, a
fission-site buffer of exactly the size needed (and one site short), and a
history that starts outside the geometry (the reference warns and kills it,
src/delta_tracker.cpp:92-98; both sides count it in `lost`)."""
import numpy as np
import pytest

import oracle
from abeille_gb300 import PARTICLE_DTYPE, Engine, decks
from abeille_gb300.abi import AbxError

pytestmark = pytest.mark.gpu


def _same(eng, ora, bank, kcol=1.0):
    sg, cg = eng.transport(bank, kcol, True)
    sc, cc = ora.transport(bank, kcol, True)
    assert len(sg) == len(sc)
    assert np.array_equal(sg["parent_history_id"], sc["parent_history_id"])
    assert np.array_equal(sg["parent_daughter_id"], sc["parent_daughter_id"])
    assert np.allclose(sg["r"], sc["r"], rtol=1e-12, atol=1e-9)
    for k in ("collisions", "flights", "lost"):
        assert cg[k] == cc[k], k
    return sg, cg


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_empty_bank(precision):
    eng = Engine(decks.config0(nparticles=16).build(precision=precision), 0)
    sites, sc = eng.transport(np.zeros(0, PARTICLE_DTYPE), 1.0, True)
    assert len(sites) == 0
    assert sc["collisions"] == 0 and sc["flights"] == 0 and sc["lost"] == 0
    assert not np.any(eng.tally(0)["gen"])
    # the context still transports a real bank afterwards
    bank = eng.sample_sources(0, 64)
    sites, sc = eng.transport(bank, 1.0, True)
    assert sc["collisions"] > 0
    eng.close()


@pytest.mark.parametrize("n", [1, 31, 33, 257, 1000])
def test_ragged_bank_sizes_match(n):
    b = decks.config0(nparticles=n)
    built = b.build(precision="fp64")
    eng, ora = Engine(built, 0), oracle.Oracle(built, nthreads=1)
    bank = ora.sample_sources(11, n)
    _same(eng, ora, bank)
    tg, tc = eng.tally(0)["gen"], ora.tally(0)["gen"]
    assert np.allclose(tg, tc, rtol=1e-12, atol=0.0)
    eng.close()


def test_site_buffer_of_exactly_the_needed_size():
    b = decks.config0(nparticles=500)
    built = b.build(precision="fp64")
    eng = Engine(built, 0)
    bank = eng.sample_sources(0, 500)
    sites, _ = eng.transport(bank, 1.0, True)
    need = len(sites)
    assert need > 0
    exact, _ = eng.transport(bank, 1.0, True, site_capacity=need)
    assert np.array_equal(exact["parent_daughter_id"], sites["parent_daughter_id"])
    with pytest.raises(AbxError) as e:
        eng.transport(bank, 1.0, True, site_capacity=need - 1)
    assert e.value.code == 7  # ABX_ERR_CAPACITY
    again, _ = eng.transport(bank, 1.0, True)
    assert np.array_equal(again["parent_daughter_id"], sites["parent_daughter_id"])
    eng.close()


@pytest.mark.parametrize("tracking", ["delta-tracking", "surface-tracking"])
def test_history_born_outside_the_geometry_is_lost(tracking):
    b = decks.config0(nparticles=128, tracking=tracking)
    built = b.build(precision="fp64")
    eng, ora = Engine(built, 0), oracle.Oracle(built, nthreads=1)
    bank = ora.sample_sources(0, 128)
    bank["r"][17] = (500.0, 0.0, 0.0)  # far outside the reflective box
    _, cg = _same(eng, ora, bank)
    assert cg["lost"] == 1
    eng.close()
