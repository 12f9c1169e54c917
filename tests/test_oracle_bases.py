"""The converted basis data: every reference basis set and element builds CGFs
with the expected function counts, and the oracle SCF converges for the small
test molecules."""
import pytest

import oracle as O
from gbhf import basis as B, molecules as M

COUNTS = {  # functions per element: H, He, Li..Ne
    "sto-3g": (1, 1, 5), "3-21g": (2, 2, 9), "6-31g": (2, 2, 9), "6-31g*": (2, 2, 15),
    "6-31g**": (5, 5, 15), "6-31++g*": (3, 2, 19),
}


@pytest.mark.parametrize("basis", sorted(COUNTS))
def test_function_counts(basis):
    h, he, heavy = COUNTS[basis]
    assert len(B.basis_for("H", basis)) == h and len(B.basis_for("He", basis)) == he
    for e in ("Li", "Be", "B", "C", "N", "O", "F", "Ne"):
        assert len(B.basis_for(e, basis)) == heavy, (basis, e)
        assert len(B.basis_for(e, basis, "shipped")) == heavy


def test_small_molecules_converge():
    for name in M.SMALL_MOLECULES:
        atoms, q = M.small_molecule(name, "3-21g")
        r = O.scf(B.flatten(atoms), O.SCFOptions.baseline(charge=q))
        assert r.iterations < 30, name
    # CH4/6-31G* near its known RHF energy at this geometry
    atoms, _ = M.small_molecule("CH4", "6-31g*")
    assert abs(O.scf(B.flatten(atoms), O.SCFOptions.baseline()).energy + 40.1951583) < 1e-6
