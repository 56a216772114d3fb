"""Parity of the CUDA engine with the oracle, through the C-ABI.

FP64 mode: integers (rng states, event kinds, groups, cells, history and
daughter ids, collision counts) are compared bit-exactly; floating values
within 1e-12 relative (the engine calls CUDA's log/sin/cos where the
reference calls glibc's, which differ in the last bit on some inputs).
Tallies and scores are compared within 1e-12 relative, which absorbs the
order of atomic additions.
"""
import json
import os

import numpy as np
import pytest

import oracle
from abeille_gb300 import Engine, decks
from abeille_gb300.abi import AbxError

pytestmark = pytest.mark.gpu

RTOL = 1e-12
DECKS = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_decks.json")))


def pair(builder, precision="fp64", nthreads=1):
    built = builder.build(precision=precision)
    return Engine(built, 0), oracle.Oracle(built, nthreads=nthreads), built


def close(a, b, rtol=RTOL, atol=1e-10):
    return np.allclose(a, b, rtol=rtol, atol=atol)


def compare_traces(tg, tc):
    assert len(tg) == len(tc), (len(tg), len(tc))
    for f in ("hist", "kind", "group", "cell", "rng_state"):
        assert np.array_equal(tg[f], tc[f]), f
    assert close(tg["r"], tc["r"], atol=1e-9)
    assert close(tg["u"], tc["u"], atol=1e-9)
    assert close(tg["wgt"], tc["wgt"])
    exact = np.mean(np.all(tg["r"] == tc["r"], axis=1) & np.all(tg["u"] == tc["u"], axis=1))
    print(f"trace records: {len(tg)}, bit-identical position+direction: {exact:.4f}")


@pytest.mark.parametrize("cfg", [0, 2])
def test_source_sampling_matches(cfg):
    b = decks.CONFIGS[cfg](nparticles=4096)
    eng, ora, _ = pair(b)
    g = eng.sample_sources(123, 4096)
    c = ora.sample_sources(123, 4096)
    assert np.array_equal(g["rng_state"], c["rng_state"])
    assert np.array_equal(g["history_id"], c["history_id"])
    assert close(g["r"], c["r"]) and close(g["u"], c["u"])
    assert np.array_equal(g["E"], c["E"])


@pytest.mark.parametrize("cfg,tracking", [(0, "delta-tracking"), (0, "surface-tracking"),
                                          (2, "delta-tracking"), (2, "surface-tracking")])
def test_event_traces_match_per_history(cfg, tracking):
    b = decks.CONFIGS[cfg](nparticles=256, tracking=tracking)
    eng, ora, _ = pair(b)
    bank = ora.sample_sources(0, 256)
    eng.set_trace(64, 1 << 20)
    ora.set_trace(64, 1 << 20)
    eng.transport(bank, 1.0, True)
    ora.transport(bank, 1.0, True)
    compare_traces(eng.get_trace(), ora.get_trace())


def test_c5g7_transport_step_matches():
    """The reference's C5G7 core (input_files/c5g7.yaml: 2x2 assemblies of
    17x17 pins, seven materials, delta tracking, track-length tally): fission
    bank, scores and tally of one transport step against the oracle."""
    b = decks.from_reference_deck(reference_deck("c5g7"), nparticles=4096)
    eng, ora, _ = pair(b, nthreads=oracle.cores())
    bank = ora.sample_sources(0, 4096)
    sg, cg = eng.transport(bank, 1.1, True)
    sc, cc = ora.transport(bank, 1.1, True)
    assert len(sg) == len(sc) > 0
    assert np.array_equal(sg["parent_history_id"], sc["parent_history_id"])
    assert np.array_equal(sg["parent_daughter_id"], sc["parent_daughter_id"])
    assert close(sg["r"], sc["r"], atol=1e-9) and close(sg["u"], sc["u"], atol=1e-9)
    for k in ("collisions", "flights", "lost"):
        assert cg[k] == cc[k], k
    for k in ("k_col", "k_abs", "leakage", "mig_area"):
        assert abs(cg[k] - cc[k]) <= RTOL * abs(cc[k]) + 1e-300, (k, cg[k], cc[k])
    tg, tc = eng.tally(0)["gen"], ora.tally(0)["gen"]
    assert np.array_equal(tg != 0, tc != 0) and abs(tg.sum() - tc.sum()) <= RTOL * tc.sum()
    assert close(tg, tc, rtol=1e-9, atol=0.0)
    eng.close()


@pytest.mark.parametrize("cfg,tracking", [(0, "delta-tracking"), (1, "delta-tracking"), (2, "surface-tracking"),
                                          (2, "delta-tracking"), (1, "implicit-leakage-delta-tracking"),
                                          (2, "implicit-leakage-delta-tracking")])
def test_transport_step_matches(cfg, tracking):
    n = 4096 if cfg != 2 else 1024
    b = decks.CONFIGS[cfg](nparticles=n, tracking=tracking)
    eng, ora, _ = pair(b, nthreads=oracle.cores())
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
    assert abs(tg.sum() - tc.sum()) <= RTOL * tc.sum()
    if cfg == 2:
        # Track-length segments are differences of positions: a 1-ulp position
        # difference (CUDA vs glibc log/sin/cos) is ~1e-15 cm absolute, which
        # is up to ~1e-11 relative on the shortest segments of a bin.
        assert close(tg, tc, rtol=1e-9, atol=0.0)
    else:
        assert close(tg, tc, atol=0.0)


def test_power_iteration_matches():
    b = decks.config0(nparticles=2000)
    eng, ora, _ = pair(b, nthreads=oracle.cores())
    sg, kg, hg = eng.run_power_iteration(6, 2)
    sc, kc, hc = ora.run_power_iteration(6, 2)
    assert np.allclose(kg, kc, rtol=1e-11, atol=0)
    assert np.allclose(hg, hc, rtol=1e-11, atol=0)
    assert sg["collisions"] == sc["collisions"] and sg["histories"] == sc["histories"]
    assert abs(sg["kcol_avg"] - sc["kcol_avg"]) <= 1e-11 * sc["kcol_avg"]
    tg, tc = eng.tally(0), ora.tally(0)
    assert tg["generations"] == tc["generations"] == 4
    assert np.allclose(tg["avg"], tc["avg"], rtol=1e-10, atol=0)


def _pcg_start(seed, stride, hid):
    """pcg32 state of history `hid`: seeded on the default stream, then
    advanced stride * hid steps (the LCG jump-ahead by squaring)."""
    M, INC, MASK = 6364136223846793005, 1442695040888963407, (1 << 64) - 1
    state = ((seed + INC) * M + INC) & MASK
    delta, am, ap, cm, cp = (stride * hid) & MASK, 1, 0, M, INC
    while delta:
        if delta & 1:
            am, ap = (am * cm) & MASK, (ap * cm + cp) & MASK
        cp, cm = ((cm + 1) * cp) & MASK, (cm * cm) & MASK
        delta >>= 1
    return (am * state + ap) & MASK


def test_source_bank_after_power_iteration():
    """The bank the next generation would run (PowerIterator's `bank` after
    its loop): consecutive history ids after every history already run,
    weights normalised to N in total, each stream re-seeded at its history id,
    the last k_col; a transport of it matches the oracle's transport of the
    same bank, and that transport replaces it."""
    b = decks.config0(nparticles=2000)
    eng, ora, _ = pair(b, nthreads=oracle.cores())
    st, kc, _ = eng.run_power_iteration(4, 1)
    bank, kcol = eng.read_source_bank()
    assert kcol == kc[-1]
    n = len(bank)
    assert n > 0
    ids = bank["history_id"]
    assert ids[0] == st["histories"] and np.array_equal(ids, np.arange(ids[0], ids[0] + n))
    assert abs(bank["wgt"].sum() - 2000.0) <= 1e-9 * 2000.0
    for i in (0, 1, n - 1):  # pcg32 seeded, then advanced stride * history id (particle.hpp:188-193)
        assert int(bank["rng_state"][i]) == _pcg_start(b.seed, b.stride, int(ids[i]))
    sg, cg = eng.transport(bank, kcol, True)
    sc, cc = ora.transport(bank, kcol, True)
    assert np.array_equal(sg["parent_history_id"], sc["parent_history_id"])
    assert np.array_equal(sg["parent_daughter_id"], sc["parent_daughter_id"])
    assert close(sg["r"], sc["r"], atol=1e-9)
    for k in ("collisions", "flights", "lost"):
        assert cg[k] == cc[k], k
    with pytest.raises(AbxError):
        eng.read_source_bank()


def test_restart_from_a_source_bank_matches():
    """PowerIterator::load_source_from_file: rows x y z ux uy uz E wgt wgt2
    become histories 0..n-1 seeded at their ids, nparticles becomes the
    rounded total weight; the restarted power iteration matches the oracle's
    generation by generation."""
    b = decks.config0(nparticles=2000)
    eng, ora, _ = pair(b, nthreads=oracle.cores())
    eng.run_power_iteration(4, 1)
    bank, _ = eng.read_source_bank()
    rows = Engine.source_rows(bank)
    rows[:, 7] *= 1.25  # total weight 2500: the restarted run normalises to it
    eng.set_source_bank(rows)
    ora.set_source_bank(rows)
    sg, kg, hg = eng.run_power_iteration(5, 1)
    sc, kc, hc = ora.run_power_iteration(5, 1)
    assert np.allclose(kg, kc, rtol=1e-11, atol=0) and np.allclose(hg, hc, rtol=1e-11, atol=0)
    assert sg["collisions"] == sc["collisions"] and sg["histories"] == sc["histories"]
    nxt, _ = eng.read_source_bank()
    assert abs(nxt["wgt"].sum() - 2500.0) <= 1e-9 * 2500.0
    eng.set_source_bank(None)  # back to sampling the problem's sources
    eng.run_power_iteration(2, 1)


def test_fixed_source_matches():
    b = decks.fixed_source_problem(0, nparticles=3000, precision="fp64")
    eng, ora, _ = pair(b, nthreads=oracle.cores())
    sg = eng.run_fixed_source(2, 3000)
    sc = ora.run_fixed_source(2, 3000)
    assert sg["collisions"] == sc["collisions"]
    assert abs(sg["leak_avg"] - sc["leak_avg"]) <= 1e-11 * abs(sc["leak_avg"])
    assert np.allclose(eng.tally(0)["avg"], ora.tally(0)["avg"], rtol=1e-10, atol=0)


def reference_deck(name):
    """A reference deck from the fixtures; c5g7's 1224x1224x10 track-length
    tally is cut to 51x51x10 bins over the same extent (parity tests need the
    estimator, not the resolution)."""
    d = dict(DECKS[name])
    if name == "c5g7":
        d["tallies"] = [dict(t, shape=[51, 51, 10]) for t in d["tallies"]]
    return d


@pytest.mark.parametrize("name,tracking", [("PUa-1-0-IN", None), ("PUb-1-0-SL", None), ("Ua-1-1-CY", None),
                                           ("PUa-1-1-SL", None), ("PUa-1-2-SL", None), ("Ua-1-1-IN", None),
                                           ("PUa-1-2-SL", "delta-tracking"), ("c5g7", "delta-tracking"),
                                           ("c5g7", "surface-tracking")])
def test_reference_decks_trace_parity(name, tracking):
    b = decks.from_reference_deck(reference_deck(name), nparticles=256, tracking=tracking)
    eng, ora, _ = pair(b)
    bank = ora.sample_sources(0, 256)
    eng.set_trace(128, 1 << 20)
    ora.set_trace(128, 1 << 20)
    eng.transport(bank, 1.0, True)
    ora.transport(bank, 1.0, True)
    compare_traces(eng.get_trace(), ora.get_trace())


@pytest.mark.parametrize("name,tracking", [("PUa-1-0-SL", "implicit-leakage-delta-tracking"),
                                           ("UD2O-2-1-SL", "implicit-leakage-delta-tracking"),
                                           ("Ua-1-1-CY", "implicit-leakage-delta-tracking")])
def test_implicit_leakage_traces_match(name, tracking):
    b = decks.from_reference_deck(DECKS[name], nparticles=256, tracking=tracking)
    eng, ora, _ = pair(b)
    bank = ora.sample_sources(0, 256)
    eng.set_trace(128, 1 << 20)
    ora.set_trace(128, 1 << 20)
    sg, cg = eng.transport(bank, 1.0, True)
    sc, cc = ora.transport(bank, 1.0, True)
    compare_traces(eng.get_trace(), ora.get_trace())
    assert abs(cg["leakage"] - cc["leakage"]) <= RTOL * abs(cc["leakage"]) + 1e-300


@pytest.mark.parametrize("name,precision,tracking", [("PUa-1-0-IN", "fp64", None), ("PUa-1-0-IN", "mixed", None),
                                                     ("PUb-1-0-SL", "mixed", None),
                                                     ("PUa-1-0-SL", "fp64", "implicit-leakage-delta-tracking"),
                                                     ("PUb-1-0-SL", "mixed", "implicit-leakage-delta-tracking")])
def test_reference_known_answers_on_gpu(name, precision, tracking):
    deck = DECKS[name]
    eng = Engine(decks.from_reference_deck(deck, nparticles=100000, tracking=tracking).build(precision=precision), 0)
    st, _, _ = eng.run_power_iteration(40, 10)
    assert abs(st["kcol_avg"] - deck["_expected_k"]) < 4 * st["kcol_std"] + 2e-4, st


def _replicas(builder_fn, prec, seed0, R, ngen, nign):
    ks, avgs = [], []
    for rep in range(R):
        b = builder_fn()
        b.seed = seed0 + rep
        eng = Engine(b.build(precision=prec), 0)
        st, _, _ = eng.run_power_iteration(ngen, nign)
        ks.append(st["kcol_avg"])
        avgs.append(eng.tally(0)["avg"])
        eng.close()
    return np.array(ks), np.array(avgs)


def _agreement(x, y, keep=None):
    """k difference in sigma, fraction of bins with |z| < 2 and mean z between
    two replica sets (sigma of each mean from its replica spread)."""
    (kx, ax), (ky, ay) = x, y
    dk = (kx.mean() - ky.mean()) / np.sqrt(kx.var(ddof=1) / len(kx) + ky.var(ddof=1) / len(ky))
    z = (ax.mean(0) - ay.mean(0)) / np.sqrt(ax.var(0, ddof=1) / len(ax) + ay.var(0, ddof=1) / len(ay))
    if keep is not None:
        z = z[keep]
    return dk, np.mean(np.abs(z) < 2), z.mean()


def test_mixed_precision_statistics_config0():
    """FP32 tracking / FP64 tallies against the FP64 path on config 0: k within
    2 sigma, and flux bins with |z| < 2 at the rate two independent FP64
    replica sets reach between themselves.

    The standard deviations come from independent replicas (different seeds):
    generation-to-generation statistics of one power iteration underestimate
    the error because successive generations are correlated.  The 289 bins
    share one fission source, so the fraction of bins with |z| < 2 moves by
    several percent from one replica set to another (FP64 against FP64 gives
    0.89 to 0.97); the bar is therefore set against an FP64/FP64 control
    computed in the same test, and the mean z must stay near 0."""
    R = 24
    fp64_a = _replicas(lambda: decks.config0(nparticles=5000), "fp64", 1000, R, 40, 10)
    fp64_b = _replicas(lambda: decks.config0(nparticles=5000), "fp64", 5000, R, 40, 10)
    mixed = _replicas(lambda: decks.config0(nparticles=5000), "mixed", 9000, R, 40, 10)
    dk, frac, mz = _agreement(mixed, fp64_a)
    dk_c, frac_c, mz_c = _agreement(fp64_b, fp64_a)
    print(f"mixed vs fp64: dk = {dk:.2f} sigma, {frac:.3f} of bins |z| < 2, mean z {mz:+.3f}; "
          f"fp64 vs fp64 control: dk = {dk_c:.2f}, {frac_c:.3f}, mean z {mz_c:+.3f}")
    assert abs(dk) < 2, dk
    assert frac >= 0.85 and frac >= frac_c - 0.08, (frac, frac_c)
    assert abs(mz) < 0.3, mz


def test_errors_leave_the_context_usable():
    b = decks.config0(nparticles=64)
    eng, ora, _ = pair(b)
    bank = ora.sample_sources(0, 64)
    bad = bank.copy()
    bad["E"][5] = 99.0  # outside the group structure
    with pytest.raises(AbxError) as e:
        eng.transport(bad, 1.0, True)
    assert e.value.code == 1
    sg, _ = eng.transport(bank, 1.0, True)
    sc, _ = ora.transport(bank, 1.0, True)
    assert np.array_equal(sg["parent_daughter_id"], sc["parent_daughter_id"])
    with pytest.raises(AbxError):
        eng.transport(bank, 1.0, True, site_capacity=1)


def _t_frac(dof):
    """P(|t| < 2) for Student's t with `dof` degrees of freedom: the expected
    fraction of bins with |z| < 2 when both sides sample one distribution."""
    from scipy import stats
    return float(stats.t.cdf(2, dof) - stats.t.cdf(-2, dof))


def test_mixed_precision_statistics_config1():
    """The acceptance check of the FP32-tracking / FP64-tally mode on config 1
    (51x51 pins, 10 axial zones, 51x51x20 flux tally): k within 2 sigma and
    flux bins with |z| < 2, mixed against FP64, over independent replicas.

    Two sets of 32 replicas per precision (5e4 histories, 10 inactive + 40
    active generations each) give four mixed/FP64 pairs of sets (62 degrees
    of freedom per pair) and one pooled comparison (64 against 64 replicas,
    126 degrees of freedom).  For two samples of one distribution the
    fraction of bins with |z| < 2 is the t-distribution's P(|t| < 2): 0.950
    per pair, 0.952 pooled -- the acceptance bar of 95 % sits at that
    expectation.  All bins share one fission source, so the fraction of one
    comparison scatters around it by about 0.8 % (one standard deviation)
    even between two sets of the same precision: measured over 18 FP64/FP64
    and mixed/mixed pairs of 40-replica sets in two studies, 0.940-0.968.
    Every build re-draws the mixed trajectories (any change of FP32 rounding
    sends the histories elsewhere), so a bar one percent under the
    expectation would fail about one correct build in ten; it did once, on a
    build whose own 9-pair study then gave a 0.9544 mean, the same as the
    build before it.  The test therefore asserts each figure at three standard
    deviations of that measured spread: the pooled fraction and the mean
    over pairs within 2.5 % and 2 % of the expectation, the mean over pairs
    within 3 % of an FP64/FP64 control drawn in the same test, and the mean z
    (a bias would move it; every comparison measured stays within 0.025)
    within 0.06.  The 95 % bar itself is read from `bench.py --zscore`,
    which compares many more replicas."""
    R, n = 32, 50000
    mk = lambda: decks.config1(nparticles=n)  # noqa: E731
    sets = {}
    for si in range(2):
        sets[f"fp64{si}"] = _replicas(mk, "fp64", 30000 + 1000 * si, R, 50, 10)
        sets[f"mixed{si}"] = _replicas(mk, "mixed", 40000 + 1000 * si, R, 50, 10)
    keep = np.all([v[1].mean(0) > 0 for v in sets.values()], axis=0)
    pairs = [_agreement(sets[f"mixed{a}"], sets[f"fp64{b}"], keep) for a in range(2) for b in range(2)]
    pool = lambda p: (np.concatenate([sets[f"{p}{i}"][0] for i in range(2)]),  # noqa: E731
                      np.concatenate([sets[f"{p}{i}"][1] for i in range(2)]))
    dk, frac, mz = _agreement(pool("mixed"), pool("fp64"), keep)
    _, frac_c, _ = _agreement(sets["fp641"], sets["fp640"], keep)
    mean_pairs = float(np.mean([p[1] for p in pairs]))
    print(f"config 1 mixed vs fp64 pooled: dk = {dk:.2f} sigma, {frac:.4f} of {keep.sum()} bins |z| < 2 "
          f"(expected {_t_frac(4 * R - 2):.4f}), mean z {mz:+.3f}; pairs: "
          f"{[round(p[1], 4) for p in pairs]} mean {mean_pairs:.4f} (expected {_t_frac(2 * R - 2):.4f}); "
          f"fp64/fp64 control {frac_c:.4f}")
    assert abs(dk) < 2, dk
    assert all(abs(p[0]) < 2 for p in pairs), pairs
    assert frac >= _t_frac(4 * R - 2) - 0.025, frac
    assert mean_pairs >= _t_frac(2 * R - 2) - 0.02, mean_pairs
    assert mean_pairs >= frac_c - 0.03, (mean_pairs, frac_c)
    assert abs(mz) < 0.06, mz


@pytest.mark.parametrize("tracking", ["surface-tracking", "delta-tracking"])
def test_mixed_config2_tracks_like_fp64(tracking):
    """Config 2 (nested cylinders r = 0.41/0.42/0.475 in every pin, 70 groups,
    P1) in the mixed mode: no particle may bounce between the surfaces of the
    thin gap ring; almost none is lost, and flights and collisions per history
    stay within 2 % of the FP64 path's (statistical quantities, different
    rounding)."""
    out = {}
    for prec in ("fp64", "mixed"):
        b = decks.config2(nparticles=20000, tracking=tracking)
        eng = Engine(b.build(precision=prec), 0)
        st, recs = eng.run_power_iteration_records(4, 0)
        out[prec] = (sum(r["flights"] for r in recs), sum(r["collisions"] for r in recs),
                     sum(r["histories"] for r in recs), sum(r["lost"] for r in recs))
        eng.close()
    f64, c64, h64, l64 = out["fp64"]
    f32, c32, h32, l32 = out["mixed"]
    assert l64 == 0
    assert l32 <= 1e-4 * h32, out
    assert abs(f32 / h32 - f64 / h64) <= 0.02 * f64 / h64, out
    assert abs(c32 / h32 - c64 / h64) <= 0.02 * c64 / h64, out


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_captured_generation_step_matches_direct_launches(precision):
    """Power iteration with each generation as one CUDA-graph launch against the
    same kernels launched one by one: collision counts identical, k, entropy and
    tallies within 1e-11 relative (FP64 atomic additions in another order)."""
    out = {}
    for graphs in (False, True):
        eng = Engine(decks.config0(nparticles=3000).build(precision=precision), 0)
        eng.set_graphs(graphs)
        st, recs = eng.run_power_iteration_records(12, 4)
        out[graphs] = (st, recs, eng.tally(0))
        eng.close()
    (s0, r0, t0), (s1, r1, t1) = out[False], out[True]
    assert [r["collisions"] for r in r0] == [r["collisions"] for r in r1]
    assert [r["sites"] for r in r0] == [r["sites"] for r in r1]
    assert np.allclose([r["kcol"] for r in r0], [r["kcol"] for r in r1], rtol=1e-11, atol=0)
    assert np.allclose([r["entropy"] for r in r0], [r["entropy"] for r in r1], rtol=1e-11, atol=0)
    assert t0["generations"] == t1["generations"] == 8
    assert np.allclose(t0["avg"], t1["avg"], rtol=1e-10, atol=0)
    assert abs(s0["kcol_avg"] - s1["kcol_avg"]) <= 1e-11 * s0["kcol_avg"]


def test_autotuned_launch_shape_gives_the_same_results():
    b = decks.config0(nparticles=4096)
    eng, ora, _ = pair(b)
    bank = ora.sample_sources(0, 4096)
    s0, c0 = eng.transport(bank, 1.1, True)
    block, grid, ms = eng.autotune(20000)
    assert block in (128, 256) and grid % 152 == 0 or grid > 0
    assert ms > 0
    s1, c1 = eng.transport(bank, 1.1, True)
    assert np.array_equal(s0["parent_history_id"], s1["parent_history_id"])
    assert np.array_equal(s0["parent_daughter_id"], s1["parent_daughter_id"])
    assert close(s0["r"], s1["r"], atol=0) and c0["collisions"] == c1["collisions"]
    assert abs(c0["k_col"] - c1["k_col"]) <= RTOL * abs(c0["k_col"])
    eng.close()


@pytest.mark.parametrize("case", ["keig-1.3", "fixed-0.9"])
def test_carter_tracking_matches(case):
    """CarterTracker against the oracle, FP64: per-event traces, scores and
    collision counts; `fixed-0.9` samples 10 % below the total cross section
    (signed weights, splitting onto the secondary stack)."""
    if case == "keig-1.3":
        b = decks.config0(nparticles=512, tracking="carter-tracking")
        b.sampling_xs_ratio = [1.3] * b.G
    else:
        b = decks.fixed_source_problem(3, precision="fp64", nparticles=512, tracking="carter-tracking")
        b.sampling_xs_ratio = [0.9] * b.G
    eng, ora, _ = pair(b)
    bank = ora.sample_sources(0, 512)
    eng.set_trace(128, 1 << 21)
    ora.set_trace(128, 1 << 21)
    sg, cg = eng.transport(bank, 1.0, True)
    sc, cc = ora.transport(bank, 1.0, True)
    compare_traces(eng.get_trace(), ora.get_trace())
    assert cg["collisions"] == cc["collisions"] and cg["flights"] == cc["flights"]
    for k in ("k_col", "leakage", "mig_area"):
        assert abs(cg[k] - cc[k]) <= 1e-11 * abs(cc[k]) + 1e-300, (k, cg[k], cc[k])
    if case == "fixed-0.9":
        st_g = eng.run_fixed_source(3, 512)
        st_c = ora.run_fixed_source(3, 512)
        assert st_g["collisions"] == st_c["collisions"]
        assert abs(st_g["leak_avg"] - st_c["leak_avg"]) <= 1e-11 * abs(st_c["leak_avg"])
    eng.close()
