"""Reference-format decks: the YAML reader, the writer, and running a deck.

The reader is checked against the reference's own decks as they were parsed
into tests/golden/reference_decks.json (written back out as YAML by our
writer, since the reference tree is not available where tests run) and
against hand-written snippets in the reference's layout: multi-line flow
lists, flow maps as sequence items, quoted regions, comments.  A synthetic
problem written as a deck and read back must flatten to the same arrays.
"""
import ctypes as C
import json
import os

import numpy as np
import pytest

from abeille_gb300 import deck, decks

HERE = os.path.dirname(os.path.abspath(__file__))
DECKS = json.load(open(os.path.join(HERE, "golden", "reference_decks.json")))

SNIPPET = """
materials:
  # a two-group material, lists spread over lines
  - total:      [1.0E-01,
                 2.5E-01]
    absorption: [0.05, .1]
    scatter:   [[0.04, 0.01],
                [0.,   0.15]]
    id: 7
    name: "mat # seven"

surfaces:
  - {type: xplane, x0: -5., boundary: reflective, id: 1}
  - type: zcylinder
    x0: 0.
    y0: 0.
    r: 0.54
    id: 2

cells:
  - region: "-2 & +1"   # a comment after a value
    material: 7
    id: 1

universes:
  - cells: [1]
    id: 1
root-universe: 1
settings:
  nparticles: 1000
  energy-bounds: [0, 1, 2]
  cancellation: false
"""


def test_reader_on_a_snippet():
    d = deck.parse_yaml(SNIPPET)
    m = d["materials"][0]
    assert m["total"] == [0.1, 0.25] and m["absorption"] == [0.05, 0.1]
    assert m["scatter"] == [[0.04, 0.01], [0.0, 0.15]] and m["name"] == "mat # seven"
    assert d["surfaces"][0] == {"type": "xplane", "x0": -5.0, "boundary": "reflective", "id": 1}
    assert d["surfaces"][1]["r"] == 0.54
    assert d["cells"][0]["region"] == "-2 & +1"
    assert d["root-universe"] == 1 and d["settings"]["cancellation"] is False


@pytest.mark.parametrize("name", sorted(DECKS))
def test_reference_decks_round_trip(name):
    ref = {k: v for k, v in DECKS[name].items() if not k.startswith("_")}
    text = deck.dump_yaml(ref)
    assert deck.parse_yaml(text) == ref


def _flat(built):
    p = built.struct
    out = {"n": [p.n_surfaces, p.n_cells, p.n_rpn, p.n_universes, p.n_cell_lists, p.n_lattice_elems,
                 p.n_materials, p.n_mg_data, p.n_tallies, p.n_sources, p.root_universe]}
    for name, n, ty in [("surfaces", p.n_surfaces, None), ("cells", p.n_cells, None), ("rpn", p.n_rpn, None),
                        ("universes", p.n_universes, None), ("cell_lists", p.n_cell_lists, None),
                        ("lattice_elems", p.n_lattice_elems, None), ("materials", p.n_materials, None),
                        ("mg_data", p.n_mg_data, None), ("tallies", p.n_tallies, None),
                        ("sources", p.n_sources, None)]:
        arr = getattr(p, name)
        size = C.sizeof(arr._type_) * n
        out[name] = bytes(C.string_at(arr, size)) if n else b""
    return out


@pytest.mark.parametrize("cfg", [0, 1, 2])
def test_synthetic_deck_written_and_read_back_builds_the_same_problem(cfg):
    b = decks.CONFIGS[cfg](nparticles=1234)
    text = deck.dump_yaml(b.to_deck(ngenerations=5, nignored=1))
    b2, d = deck.deck_from_text(text)
    assert d["settings"]["ngenerations"] == 5
    f1, f2 = _flat(b.build(precision="fp64")), _flat(b2.build(precision="fp64"))
    for k in f1:
        assert f1[k] == f2[k], k


@pytest.mark.gpu
def test_run_a_reference_deck_from_yaml():
    import io
    from abeille_gb300.__main__ import run_deck
    ref = DECKS["PUa-1-0-IN"]
    text = deck.dump_yaml({k: v for k, v in ref.items() if not k.startswith("_")})
    buf = io.StringIO()
    st = run_deck(text, precision="mixed", particles=100000, generations=40, ignored=10, is_text=True, out=buf)
    assert abs(st["kcol_avg"] - ref["_expected_k"]) < 4 * st["kcol_std"] + 2e-4, buf.getvalue()
    assert "k_col" in buf.getvalue()


def test_branchless_settings_round_trip():
    """A branchless-k-eigenvalue deck keeps its collision flags through the
    writer and the reader, and the global stream's skip counts the deck's
    cells and materials (6 outputs each for their plot colours)."""
    b = decks.config0(nparticles=100)
    b.mode = "branchless-k-eigenvalue"
    b.branchless_material, b.branchless_splitting, b.branchless_combing = False, True, True
    text = deck.dump_yaml(b.to_deck(ngenerations=5, nignored=1))
    b2, d = deck.deck_from_text(text)
    assert d["settings"]["simulation"] == "branchless-k-eigenvalue"
    assert (b2.branchless_material, b2.branchless_splitting, b2.branchless_combing) == (False, True, True)
    s1, s2 = b.build(precision="fp64").struct.settings, b2.build(precision="fp64").struct.settings
    assert s1.branchless == s2.branchless == 1 | 4 | 8
    assert s2.global_rng_skip == 6 * (len(d["cells"]) + len(d["materials"])) == s1.global_rng_skip
    d["settings"]["cancellation"] = True
    with pytest.raises(ValueError):
        deck.deck_from_text(deck.dump_yaml(d))
