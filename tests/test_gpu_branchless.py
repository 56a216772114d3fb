"""Branchless collisions (the branchless k-eigenvalue simulation) on the GPU
against the oracle: per-history event traces and transport steps in FP64,
the device power iteration generation by generation, and the analytic k of
the reference's critical slab and infinite-medium decks in both precisions.
Tolerances as in the other parity tests: integers bit-exact, floating values
within 1e-12 relative (CUDA's log/sin/cos against glibc's)."""
import json
import os

import numpy as np
import pytest

import oracle
from abeille_gb300 import Engine, decks

pytestmark = pytest.mark.gpu

DECKS = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_decks.json")))
FLAVOURS = [(True, False), (False, False), (True, True), (False, True)]  # (per material, splitting)


def _config0(n, tracking, material, splitting, combing=False):
    b = decks.config0(nparticles=n, tracking=tracking)
    b.mode = "branchless-k-eigenvalue"
    b.branchless_material, b.branchless_splitting, b.branchless_combing = material, splitting, combing
    return b


@pytest.mark.parametrize("tracking", ["delta-tracking", "surface-tracking"])
@pytest.mark.parametrize("material,splitting", FLAVOURS)
def test_branchless_traces_and_step_match(tracking, material, splitting):
    b = _config0(512, tracking, material, splitting)
    built = b.build(precision="fp64")
    assert built.struct.settings.branchless != 0
    eng, ora = Engine(built, 0), oracle.Oracle(built, nthreads=1)
    bank = ora.sample_sources(0, 512)
    bank["wgt"] *= 2.7  # weights well above wgt-split, so splitting happens
    eng.set_trace(64, 1 << 20)
    ora.set_trace(64, 1 << 20)
    sg, cg = eng.transport(bank, 1.2, True)
    sc, cc = ora.transport(bank, 1.2, True)
    tg, tc = eng.get_trace(), ora.get_trace()
    assert len(tg) == len(tc)
    for f in ("hist", "kind", "group", "cell", "rng_state"):
        assert np.array_equal(tg[f], tc[f]), f
    assert np.allclose(tg["wgt"], tc["wgt"], rtol=1e-12, atol=0)
    assert len(sg) == len(sc)
    assert np.array_equal(sg["parent_history_id"], sc["parent_history_id"])
    assert np.array_equal(sg["parent_daughter_id"], sc["parent_daughter_id"])
    assert np.allclose(sg["wgt"], sc["wgt"], rtol=1e-12, atol=0)
    assert np.allclose(sg["r"], sc["r"], rtol=1e-12, atol=1e-9)
    for k in ("collisions", "flights", "lost"):
        assert cg[k] == cc[k], k
    for k in ("k_col", "k_abs"):
        assert abs(cg[k] - cc[k]) <= 1e-12 * abs(cc[k]), k
    if splitting:
        assert np.any(tc["kind"] == 6)  # resurrected copies
    eng.close()


@pytest.mark.parametrize("material,splitting,combing", [(True, False, False), (False, True, False),
                                                       (True, False, True), (False, True, True)])
def test_branchless_power_iteration_matches(material, splitting, combing):
    """Generation by generation against the oracle; with combing the bank is
    normalised, combed (std::shuffle over the global stream, against the
    oracle's restatement pinned to libstdc++) and re-numbered on the host."""
    b = _config0(2000, "delta-tracking", material, splitting, combing)
    built = b.build(precision="fp64")
    eng, ora = Engine(built, 0), oracle.Oracle(built, nthreads=oracle.cores())
    sg, kg, hg = eng.run_power_iteration(6, 2)
    sc, kc, hc = ora.run_power_iteration(6, 2)
    assert np.allclose(kg, kc, rtol=1e-11, atol=0)
    assert np.allclose(hg, hc, rtol=1e-11, atol=0)
    assert sg["collisions"] == sc["collisions"] and sg["histories"] == sc["histories"]
    bank, _ = eng.read_source_bank()
    assert abs(bank["wgt"].sum() - 2000.0) <= 1e-9 * 2000.0  # normalised to N
    eng.close()


@pytest.mark.parametrize("name,precision,material,splitting,tracking", [
    ("PUa-1-0-IN", "fp64", True, False, "delta-tracking"), ("PUa-1-0-IN", "mixed", False, True, "delta-tracking"),
    ("PUb-1-0-SL", "mixed", True, True, "surface-tracking"), ("PUb-1-0-IN", "fp64", False, False, "surface-tracking"),
    ("PUa-1-0-SL", "mixed", True, None, "delta-tracking"), ("PUb-1-0-SL", "fp64", False, None, "surface-tracking")])
def test_branchless_analytic_k_on_gpu(name, precision, material, splitting, tracking):
    """Without combing a history ends in at most one fission site unless it
    splits, so a leaking system (the slabs) needs splitting to keep its
    population; the infinite media keep theirs without.  splitting None: the
    reference's default, combing on and no splitting."""
    deck = json.loads(json.dumps(DECKS[name]))
    deck["settings"].update({"simulation": "branchless-k-eigenvalue", "branchless-material": material})
    if splitting is not None:
        deck["settings"].update({"branchless-combing": False, "branchless-splitting": splitting})
    b = decks.from_reference_deck(deck, nparticles=100000, tracking=tracking)
    eng = Engine(b.build(precision=precision), 0)
    st, _, _ = eng.run_power_iteration(40, 10)
    assert abs(st["kcol_avg"] - DECKS[name]["_expected_k"]) < 4 * st["kcol_std"] + 2e-4, st
    eng.close()
