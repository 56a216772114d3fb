"""The oracle pinned to the reference itself.

oracle/refshim/build_ref.py compiles the reference's unmodified multigroup
sources (src/delta_tracker.cpp, surface_tracker.cpp, transporter.cpp,
cell.cpp, rect_lattice.cpp, the surfaces, mg_nuclide.cpp,
legendre_distribution.cpp, the tallies, source.cpp, parser.cpp, ...) against
stand-ins for its absent third-party headers into oracle/_ref/abeille_ref.
Its own parser builds each deck (the dictionary ProblemBuilder.to_deck
writes) and its own Simulation::sample_sources and Transporter::transport
run it.  The oracle must give:

* source banks bit for bit (positions, directions, energies, weights, ids,
  pcg32 states);
* the fission bank of a transport step with the same length, parent history
  and daughter ids, energies and weights bit for bit, positions and
  directions within 1e-12 (the same last-bit differences as between the GPU
  and the oracle: both builds call glibc's libm, but a few sites differ in
  the last bits);
* the generation's score sums within 1e-12 relative, collision-estimator
  tallies within 1e-12 and track-length ones within 1e-9 per bin (sums of
  position differences).

Runs where the reference tree and pyarrow's vendored pcg-cpp are present
(the build container); skipped elsewhere.
"""
import json
import os

import numpy as np
import pytest

import oracle
from abeille_gb300 import decks

HERE = os.path.dirname(os.path.abspath(__file__))
DECKS = json.load(open(os.path.join(HERE, "golden", "reference_decks.json")))


@pytest.fixture(scope="module")
def exe():
    from oracle import reference
    path = reference.driver()
    if not path:
        pytest.skip("the reference cannot be built here (no reference tree or pcg-cpp)")
    return path


def _ref_deck(name):
    d = dict(DECKS[name])
    if name == "c5g7":
        d["tallies"] = [dict(t, shape=[51, 51, 10]) for t in d["tallies"]]
    return decks.from_reference_deck(d, nparticles=512)


def _builder(case):
    kind, arg = case
    if kind == "deck":
        return _ref_deck(arg)
    b = getattr(decks, kind)(nparticles=512)
    if arg:
        for k, v in arg.items():
            setattr(b, k, v)
    return b


CASES = [("config0", None), ("config0", {"tracking": "surface-tracking"}),
         ("config0", {"tracking": "implicit-leakage-delta-tracking"}),
         ("config0", {"tracking": "carter-tracking", "sampling_xs_ratio": [1.3] * 7}),
         ("config0", {"mode": "branchless-k-eigenvalue"}),
         ("config0", {"mode": "branchless-k-eigenvalue", "branchless_material": False}),
         ("config1", None),
         ("config2", {"nparticles": 256}), ("config2", {"nparticles": 256, "tracking": "delta-tracking"}),
         ("quadrics", {"tracking": "delta-tracking"}), ("quadrics", {"tracking": "surface-tracking"}),
         ("deck", "PUa-1-0-IN"), ("deck", "PUb-1-0-SL"), ("deck", "Ua-1-1-CY"), ("deck", "UD2O-2-1-SL"),
         ("deck", "PUa-1-1-SL"), ("deck", "PUa-1-2-SL"), ("deck", "Ua-1-1-IN"), ("deck", "c5g7")]
IDS = [f"{k}-{a if isinstance(a, str) else '-'.join(f'{x}' for x in (a or {}).values())}" for k, a in CASES]


@pytest.mark.parametrize("case", CASES, ids=IDS)
def test_oracle_is_the_reference(exe, case):
    from oracle import reference
    b = _builder(case)
    if case[0] == "quadrics":
        b = decks.quadrics(nparticles=512, tracking=case[1]["tracking"], legendre=True)
    n = b.nparticles
    ref = reference.ReferenceRun(b.to_deck(ngenerations=10, nignored=2), exe)
    ora = oracle.Oracle(b.build(precision="fp64"), nthreads=1)

    rb = ref.sample_sources(n)
    ob = ora.sample_sources(0, n)
    for f in ("rng_state", "r", "u", "E", "wgt", "history_id"):
        assert np.array_equal(rb[f], ob[f]), f

    rs, rsc, rt = ref.transport(ob, 1.1, True)
    os_, osc = ora.transport(ob, 1.1, True)
    assert len(rs) == len(os_)
    for f in ("parent_history_id", "parent_daughter_id", "E", "wgt"):
        assert np.array_equal(rs[f], os_[f]), f
    assert np.allclose(rs["r"], os_["r"], rtol=1e-12, atol=1e-12)
    assert np.allclose(rs["u"], os_["u"], rtol=1e-12, atol=1e-12)
    exact = np.mean(np.all(rs["r"] == os_["r"], axis=1) & np.all(rs["u"] == os_["u"], axis=1)) if len(rs) else 1.0
    for k, v in rsc.items():
        assert abs(v - osc[k]) <= 1e-12 * abs(v) + 1e-300, (k, v, osc[k])
    # the reference lists collision estimators first, then track-length ones
    order = [i for i, t in enumerate(b.tallies) if t["est"] == 0] + [i for i, t in enumerate(b.tallies) if t["est"] != 0]
    for rtally, i in zip(rt, order):
        otally = ora.tally(i)["gen"]
        rtol = 1e-12 if b.tallies[i]["est"] == 0 else 1e-9
        assert np.array_equal(rtally != 0, otally != 0)
        assert np.allclose(rtally, otally, rtol=rtol, atol=0.0)
    print(f"{len(rs)} sites, {exact:.4f} bit-identical in position and direction")
