"""The oracle's unrestricted HF (the reference has no open-shell SCF): known
values and limits."""
import oracle as O
from gbhf import basis as B, molecules as M


def test_hydrogen_atom_sto3g():
    atoms, q, mult = M.open_shell_molecule("H", "sto-3g")
    r = O.uhf(B.flatten(atoms), mult, q)
    # one electron: E is the STO-3G 1s expectation value, <S^2> = 3/4 exactly
    assert abs(r.energy + 0.466581850) < 1e-8
    assert abs(r.s2 - 0.75) < 1e-12 and (r.n_alpha, r.n_beta) == (1, 0)


def test_closed_shell_uhf_is_rhf():
    fb = B.flatten(M.water_atoms("6-31g", "text"))
    r = O.uhf(fb, 1)
    assert abs(r.energy - O.scf(fb, O.SCFOptions.baseline()).energy) < 1e-9 and abs(r.s2) < 1e-9


def test_triplet_spin_contamination_small():
    atoms, q, mult = M.open_shell_molecule("CH2", "sto-3g")
    r = O.uhf(B.flatten(atoms), mult, q)
    assert (r.n_alpha, r.n_beta) == (5, 3) and 2.0 < r.s2 < 2.05
