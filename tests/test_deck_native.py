"""The library's native deck reader (abx_deck_read, abeille_gb300/csrc/deck.cpp)
against the package's Python deck reader: the same reference-format YAML
gives the same flattened abx_problem, byte for byte -- settings, surfaces,
cells and their RPN regions, universes in the reference parser's order,
lattice elements, material data, tallies, entropy mesh, sources and the
sampling-xs ratio.  The decks are the reference's own (the fixtures) and the
synthetic configurations written out as decks.  Also: decks outside the
multigroup path are refused with a reason.  No GPU needed.
"""
import ctypes as C
import json
import os

import pytest

from abeille_gb300 import abi, deck, decks

HERE = os.path.dirname(os.path.abspath(__file__))
DECKS = json.load(open(os.path.join(HERE, "golden", "reference_decks.json")))

ARRAYS = [("surfaces", "n_surfaces", abi.Surface), ("cells", "n_cells", abi.Cell), ("rpn", "n_rpn", C.c_int32),
          ("universes", "n_universes", abi.Universe), ("cell_lists", "n_cell_lists", C.c_int32),
          ("lattice_elems", "n_lattice_elems", C.c_int32), ("materials", "n_materials", abi.Material),
          ("mg_data", "n_mg_data", C.c_double), ("tallies", "n_tallies", abi.MeshTally),
          ("tally_ebounds", "n_tally_ebounds", C.c_double), ("sources", "n_sources", abi.Source)]


def _bytes(ptr, n, ty):
    if n == 0:
        return b""
    return C.string_at(C.cast(ptr, C.c_void_p), n * C.sizeof(ty))


def _same_problem(a, b, G):
    assert bytes(a.settings) == bytes(b.settings)
    assert _bytes(a.energy_bounds, G + 1, C.c_double) == _bytes(b.energy_bounds, G + 1, C.c_double)
    for f, nf, ty in ARRAYS:
        assert getattr(a, nf) == getattr(b, nf), nf
        assert _bytes(getattr(a, f), getattr(a, nf), ty) == _bytes(getattr(b, f), getattr(b, nf), ty), f
    assert a.root_universe == b.root_universe
    assert bytes(a.entropy) == bytes(b.entropy)
    assert bool(a.sampling_xs_ratio) == bool(b.sampling_xs_ratio)
    if a.sampling_xs_ratio:
        assert _bytes(a.sampling_xs_ratio, G, C.c_double) == _bytes(b.sampling_xs_ratio, G, C.c_double)


def _native(text, precision):
    lib = abi.load()
    h, p = C.c_void_p(), C.POINTER(abi.Problem)()
    rc = lib.abx_deck_read(text.encode(), abi.PRECISION[precision], C.byref(h), C.byref(p))
    return lib, rc, h, p


def _compare(text, precision="fp64"):
    b, d = deck.deck_from_text(text)
    built = b.build(precision=precision)
    lib, rc, h, p = _native(text, precision)
    abi.check(rc, lib)
    try:
        _same_problem(built.struct, p.contents, b.G)
    finally:
        lib.abx_deck_free(h)


def _reference_deck_text(name):
    d = {k: v for k, v in DECKS[name].items() if not k.startswith("_")}
    return deck.dump_yaml(d)


@pytest.mark.parametrize("name", sorted(DECKS))
def test_reference_decks_read_alike(name):
    _compare(_reference_deck_text(name))


@pytest.mark.parametrize("case", ["config0", "config1", "config2", "quadrics", "carter", "branchless", "fixed"])
def test_synthetic_decks_read_alike(case):
    if case == "carter":
        b = decks.config0(nparticles=500, tracking="carter-tracking")
        b.sampling_xs_ratio = [1.1 + 0.01 * g for g in range(b.G)]
    elif case == "branchless":
        b = decks.config0(nparticles=500)
        b.mode = "branchless-k-eigenvalue"
        b.branchless_material, b.branchless_splitting = False, True
    elif case == "fixed":
        b = decks.fixed_source_problem(5, precision="mixed")
    elif case == "quadrics":
        b = decks.quadrics(nparticles=500, tracking="surface-tracking", legendre=True)
    else:
        b = getattr(decks, case)(nparticles=500)
    text = deck.dump_yaml(b.to_deck(ngenerations=10, nignored=2))
    _compare(text, "mixed")
    _compare(text, "fp64")


def test_reference_c5g7_yaml_as_written_by_the_reference():
    """The fixture of input_files/c5g7.yaml is stored parsed; its YAML as
    written back (flow and block forms) reads alike in both readers."""
    _compare(_reference_deck_text("c5g7"), "mixed")


@pytest.mark.parametrize("edit,reason", [
    (lambda d: d["settings"].update({"energy-mode": "continuous-energy"}), "multigroup"),
    (lambda d: d["settings"].update({"simulation": "noise"}), "outside"),
    (lambda d: d["surfaces"].append({"type": "cone", "id": 999, "x0": 0, "y0": 0, "z0": 0, "t2": 1}), "cone"),
    (lambda d: d["cells"][0].update({"region": "+1 & -9999"}), "9999"),
])
def test_decks_outside_the_path_are_refused(edit, reason):
    d = json.loads(json.dumps({k: v for k, v in DECKS["PUa-1-0-SL"].items() if not k.startswith("_")}))
    edit(d)
    lib, rc, h, p = _native(deck.dump_yaml(d), "fp64")
    assert rc == 1  # ABX_ERR_INVALID
    assert reason in lib.abx_last_error_string().decode()
