"""Host-side flattening of reference decks."""
import numpy as np
import pytest

from abeille_gb300 import abi, decks, infix_to_rpn, tokenize_region
from abeille_gb300.problem import ProblemBuilder

I, U, Cm, L, R = abi.OP_INTR, abi.OP_UNIN, abi.OP_COMP, abi.OP_LPAR, abi.OP_RPAR


def test_region_tokens_use_surface_index_plus_one():
    idx = {11: 0, 12: 1, 13: 2}
    assert tokenize_region("+11 & -12", idx) == [1, I, -2]
    assert tokenize_region("-13", idx) == [-3]
    with pytest.raises(ValueError):
        tokenize_region("+99", idx)


def test_infix_to_rpn_precedence():
    # intersection binds tighter than union, complement tightest, parentheses group
    assert infix_to_rpn([1, I, 2, U, 3]) == [1, 2, I, 3, U]
    assert infix_to_rpn([1, U, 2, I, 3]) == [1, 2, 3, I, U]
    assert infix_to_rpn([L, 1, U, 2, R, I, 3]) == [1, 2, U, 3, I]
    assert infix_to_rpn([Cm, L, 1, I, 2, R]) == [1, 2, I, Cm]
    with pytest.raises(ValueError):
        infix_to_rpn([L, 1, I, 2])


def test_universe_creation_order_matches_reference_parser():
    b = decks.config0(nparticles=10)
    # universes in deck order; a lattice comes after its tiles and outer universe
    assert b.universe_order() == [100, 1, 10]
    b = ProblemBuilder(1, [0, 1])
    b.material(1, total=[1], absorption=[0.5], scatter=[[0.5]])
    b.surface("zcylinder", 1, r=0.5)
    b.cell(1, "-1", material=1)
    b.cell(2, "+1", material=1)
    b.rect_lattice(10, [2, 2, 1], [1, 1, 1], [0, 0, 0], [1, 2, 2, 1], outer=3)
    b.cell_universe(1, [1, 2])
    b.cell_universe(2, [2, 1])
    b.cell_universe(3, [2])
    assert b.universe_order() == [1, 2, 3, 10]
    b.cell(5, "-1", universe=10)
    assert b.universe_order() == [1, 2, 3, 10]


def test_built_struct_counts():
    built = decks.config1(nparticles=10).build()
    p = built.struct
    assert p.n_universes == 13 and p.n_cells == 13 and p.n_materials == 3
    assert p.settings.ngroups == 7 and p.n_tallies == 1


def test_chi_row_is_repeated():
    b = ProblemBuilder(2, [0, 1, 2])
    b.material(1, total=[1, 1], absorption=[0.5, 0.5], scatter=[[0.5, 0], [0, 0.5]], fission=[0.1, 0.1],
               nu=[2, 2], chi=[0.7, 0.3])
    d = b.materials[0]["data"]
    chi = d[5 * 2: 5 * 2 + 4].reshape(2, 2)
    assert np.array_equal(chi, [[0.7, 0.3], [0.7, 0.3]])
