"""The bench workload at its own size through the C-ABI: config 1 (51x51 pins
x 10 axial zones, 7 groups) with 1,000,000 histories in one abx_transport
call, the bank, fission-site and scan sizes of the timed generations.

The oracle cannot transport a million histories in a test, but histories are
independent (each carries its own pcg32 state), so the oracle transports a
sample of them and each sampled history's fission sites must be, bit for
bit in the integers and weights, the ones the full-size GPU launch banked for
it (FP64 mode).  The whole bank is checked through properties that hold at
any size: sites sorted by (parent history, daughter), daughters numbered
0..m-1 without gaps, every parent a history of the bank.  The mixed mode runs
the same bank: the same properties, and per-history collisions, flights and
sites within 1 % of the FP64 run (both sample one distribution; at a million
histories 1 % is many standard deviations).
"""
import numpy as np
import pytest

import oracle
from abeille_gb300 import Engine, decks

pytestmark = pytest.mark.gpu

N = 1_000_000
KCOL = 1.3


def _bank_structure(sites, bank):
    ph = sites["parent_history_id"].astype(np.int64)
    pd = sites["parent_daughter_id"].astype(np.int64)
    key = ph * (1 << 20) + pd
    assert np.all(np.diff(key) > 0), "sites not in (parent, daughter) order"
    # daughters of each parent numbered 0..m-1
    first = np.r_[True, ph[1:] != ph[:-1]]
    start = np.maximum.accumulate(np.where(first, np.arange(ph.size), 0))
    assert np.array_equal(pd, np.arange(ph.size) - start)
    assert np.all(np.isin(np.unique(ph), bank["history_id"]))
    assert np.all(np.isfinite(sites["r"])) and np.all(sites["wgt"] > 0)


@pytest.fixture(scope="module")
def full_fp64():
    built = decks.config1(nparticles=N).build(precision="fp64")
    eng = Engine(built, 0)
    bank = eng.sample_sources(0, N)
    sites, sc = eng.transport(bank, KCOL, True)
    eng.close()
    return built, bank, sites, sc


def test_fp64_full_bank_structure(full_fp64):
    _, bank, sites, sc = full_fp64
    assert sc["lost"] == 0
    assert 0.5 * N < len(sites) < 2 * N
    _bank_structure(sites, bank)


def test_fp64_sampled_histories_match_the_oracle(full_fp64):
    built, bank, sites, _ = full_fp64
    rng = np.random.default_rng(5)
    pick = np.sort(rng.choice(N, 1500, replace=False))
    pick = np.r_[0, pick[(pick != 0) & (pick != N - 1)], N - 1]  # the first and last histories too
    ora = oracle.Oracle(built, nthreads=oracle.cores())
    so, _ = ora.transport(bank[pick], KCOL, True)
    mine = sites[np.isin(sites["parent_history_id"], bank["history_id"][pick])]
    assert len(mine) == len(so) and len(so) > 500
    for f in ("parent_history_id", "parent_daughter_id", "family_id"):
        assert np.array_equal(mine[f], so[f]), f
    assert np.array_equal(mine["wgt"], so["wgt"]) and np.array_equal(mine["E"], so["E"])
    assert np.allclose(mine["r"], so["r"], rtol=1e-12, atol=1e-9)
    assert np.allclose(mine["u"], so["u"], rtol=1e-12, atol=1e-9)


def test_mixed_full_bank_against_fp64(full_fp64):
    _, bank, s64, sc64 = full_fp64
    eng = Engine(decks.config1(nparticles=N).build(precision="mixed"), 0)
    sites, sc = eng.transport(bank, KCOL, True)
    eng.close()
    _bank_structure(sites, bank)
    assert sc["lost"] <= 1e-5 * N
    for k in ("collisions", "flights"):
        assert abs(sc[k] - sc64[k]) <= 0.01 * sc64[k], (k, sc[k], sc64[k])
    assert abs(len(sites) - len(s64)) <= 0.01 * len(s64)
    assert abs(sc["k_col"] - sc64["k_col"]) <= 0.01 * sc64["k_col"]
