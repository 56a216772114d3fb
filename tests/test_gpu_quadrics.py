"""Spheres, general planes and x/y-cylinders on the GPU against the oracle.

The lattice configurations use only axis planes and z-cylinders.  The
`quadrics` deck puts every other surface kind of the multigroup path in one
problem (src/sphere.cpp:33-80, src/plane.cpp:33-60, src/xcylinder.cpp,
src/ycylinder.cpp): a fuel sphere, a fuel x-cylinder rod, a water y-cylinder
rod, a moderator split by a general plane, a vacuum sphere as the outer
boundary and a reflective general plane cutting it.

FP64 mode: per-event traces (kind, group, cell, rng state bit-exact;
positions and directions within 1e-12 relative), fission banks, scores and
both tallies as in the lattice parity tests.  FP32-tracking mode: rays aimed
within 1e-7..1e-3 of tangent at the sphere and at the x-cylinder (where the
quadric roots cancel) are tracked without losing a particle, and flights and
collisions per history stay within a few percent of the FP64 path's.
"""
import numpy as np
import pytest

import oracle
from abeille_gb300 import Engine, decks

from test_gpu_parity import RTOL, close, compare_traces, pair

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("tracking", ["delta-tracking", "surface-tracking"])
@pytest.mark.parametrize("legendre", [False, True])
def test_quadric_traces_match_per_history(tracking, legendre):
    b = decks.quadrics(nparticles=256, tracking=tracking, legendre=legendre)
    eng, ora, _ = pair(b)
    bank = ora.sample_sources(0, 256)
    eng.set_trace(96, 1 << 21)
    ora.set_trace(96, 1 << 21)
    eng.transport(bank, 1.0, True)
    ora.transport(bank, 1.0, True)
    compare_traces(eng.get_trace(), ora.get_trace())
    eng.close()


@pytest.mark.parametrize("tracking", ["delta-tracking", "surface-tracking"])
def test_quadric_transport_step_matches(tracking):
    n = 2048
    b = decks.quadrics(nparticles=n, tracking=tracking, legendre=True)
    eng, ora, _ = pair(b, nthreads=oracle.cores())
    bank = ora.sample_sources(0, n)
    sg, cg = eng.transport(bank, 0.64, True)
    sc, cc = ora.transport(bank, 0.64, True)
    assert len(sg) == len(sc) > 0
    assert np.array_equal(sg["parent_history_id"], sc["parent_history_id"])
    assert np.array_equal(sg["parent_daughter_id"], sc["parent_daughter_id"])
    assert np.array_equal(sg["wgt"], sc["wgt"]) and np.array_equal(sg["E"], sc["E"])
    assert close(sg["r"], sc["r"], atol=1e-9) and close(sg["u"], sc["u"], atol=1e-9)
    for k in ("collisions", "flights", "lost"):
        assert cg[k] == cc[k], k
    for k in ("k_col", "k_abs", "k_trk", "leakage", "mig_area"):
        assert abs(cg[k] - cc[k]) <= RTOL * abs(cc[k]) + 1e-300, (k, cg[k], cc[k])
    # collision estimator: order of FP64 additions only
    tg, tc = eng.tally(0)["gen"], ora.tally(0)["gen"]
    assert np.array_equal(tg != 0, tc != 0) and close(tg, tc, atol=0.0)
    # track-length estimator: segments are differences of positions
    tg, tc = eng.tally(1)["gen"], ora.tally(1)["gen"]
    assert np.array_equal(tg != 0, tc != 0)
    assert abs(tg.sum() - tc.sum()) <= RTOL * tc.sum()
    assert close(tg, tc, rtol=1e-9, atol=0.0)
    eng.close()


def test_quadric_power_iteration_matches():
    b = decks.quadrics(nparticles=2000, tracking="surface-tracking")
    eng, ora, _ = pair(b, nthreads=oracle.cores())
    sg, kg, hg = eng.run_power_iteration(5, 2)
    sc, kc, hc = ora.run_power_iteration(5, 2)
    assert sg["collisions"] == sc["collisions"] and sg["histories"] == sc["histories"]
    assert np.allclose(kg, kc, rtol=1e-11, atol=0) and np.allclose(hg, hc, rtol=1e-11, atol=0)
    for t in (0, 1):
        assert np.allclose(eng.tally(t)["avg"], ora.tally(t)["avg"], rtol=1e-9, atol=0)
    eng.close()


def _grazing_bank(eng, n):
    """Rays tangent to within a relative offset of 1e-7..1e-3 (inside and
    outside) to the sphere r = 3 at the origin (flying along x) and to the
    x-cylinder y0 = 6, z0 = 3, r = 1.5 (flying along y), each starting 0.3 cm
    before its tangent point."""
    bank = eng.sample_sources(0, n)
    rng = np.random.default_rng(7)
    off = 10.0 ** rng.uniform(-7, -3, n) * rng.choice([-1.0, 1.0], n)
    half = n // 2
    r = np.zeros((n, 3))
    u = np.zeros((n, 3))
    phi = rng.uniform(0, 2 * np.pi, half)  # the impact point goes round the sphere
    bimp = 3.0 * (1.0 + off[:half])
    r[:half, 0] = -0.3
    r[:half, 1] = bimp * np.cos(phi)
    r[:half, 2] = bimp * np.sin(phi)
    u[:half, 0] = 1.0
    r[half:, 0] = rng.uniform(-5.0, 5.0, n - half)
    r[half:, 1] = 5.7
    r[half:, 2] = 3.0 + 1.5 * (1.0 + off[half:])
    u[half:, 1] = 1.0
    bank["r"] = r
    bank["u"] = u
    bank["E"] = 0.5
    return bank


@pytest.mark.parametrize("tracking", ["surface-tracking", "delta-tracking"])
def test_mixed_grazing_rays_track_like_fp64(tracking):
    n = 8192
    out = {}
    for prec in ("fp64", "mixed"):
        eng = Engine(decks.quadrics(nparticles=n, tracking=tracking).build(precision=prec), 0)
        bank = _grazing_bank(eng, n)
        _, sc = eng.transport(bank, 0.64, True, site_capacity=8 * n)
        out[prec] = sc
        eng.close()
    f64, f32 = out["fp64"], out["mixed"]
    assert f64["lost"] == 0 and f32["lost"] == 0, (f64, f32)
    for k in ("flights", "collisions"):
        assert abs(f32[k] - f64[k]) <= 0.03 * f64[k], (k, f32[k], f64[k])
    assert abs(f32["leakage"] - f64["leakage"]) <= 0.03 * f64["leakage"] + 5.0, (f32["leakage"], f64["leakage"])


@pytest.mark.parametrize("tracking", ["surface-tracking", "delta-tracking"])
def test_mixed_quadrics_tracks_like_fp64(tracking):
    """Power iterations of the quadrics deck in both precisions: no particle
    lost, flights and collisions per history within 2 %.  The plane that caps
    the sphere is a vacuum boundary here: 80,000 FP64 histories against a
    reflective general plane meet, now and then, a grazing reflection the
    reference's own plane distance loses (see decks.quadrics)."""
    out = {}
    for prec in ("fp64", "mixed"):
        eng = Engine(decks.quadrics(nparticles=20000, tracking=tracking, legendre=True,
                                    cap="vacuum").build(precision=prec), 0)
        st, recs = eng.run_power_iteration_records(4, 0)
        out[prec] = (sum(r["flights"] for r in recs), sum(r["collisions"] for r in recs),
                     sum(r["histories"] for r in recs), sum(r["lost"] for r in recs))
        eng.close()
    f64, c64, h64, l64 = out["fp64"]
    f32, c32, h32, l32 = out["mixed"]
    assert l64 == 0 and l32 <= 1e-4 * h32, out
    assert abs(f32 / h32 - f64 / h64) <= 0.02 * f64 / h64, out
    assert abs(c32 / h32 - c64 / h64) <= 0.02 * c64 / h64, out
