"""Every basis set and element of the reference's basis data (STO-3G, 3-21G,
6-31G, 6-31G*, 6-31G**, 6-31++G*; H-Ne) through the device SCF, against the
oracle: small molecules, neutral and charged."""
import numpy as np
import pytest

import oracle as O
from gbhf import _lib, basis as B, molecules as M

pytestmark = pytest.mark.gpu

BASES = ["sto-3g", "3-21g", "6-31g*", "6-31g**", "6-31++g*"]


@pytest.mark.parametrize("name", M.SMALL_MOLECULES)
def test_small_molecules_every_basis(ctx, name):
    for b in BASES:
        atoms, q = M.small_molecule(name, b)
        fb = B.flatten(atoms)
        ctx.set_basis(fb)
        r = ctx.scf(_lib.baseline_opts(charge=q), want_matrices=False)
        o = O.scf(fb, O.SCFOptions.baseline(charge=q))
        assert abs(r["energy"] - o.energy) < 1e-8, (name, b, r["energy"], o.energy)


def test_reference_numerics_co_shipped(ctx):
    """CO/STO-3G with the reference's numerics on its shipped basis blobs (SP
    exponents 1.0): the oracle's reference-mode energy to 1e-8 (core guess; the
    Harris guess of the reference also runs for this basis)."""
    atoms, q = M.small_molecule("CO", "sto-3g", "shipped")
    fb = B.flatten(atoms)
    ctx.set_basis(fb)
    ctx.set_boys_grid(O.boys_ref_grid())
    r = ctx.scf(_lib.reference_opts())
    o = O.scf(fb, O.SCFOptions())
    assert abs(r["energy"] - o.energy) < 1e-8 and r["iterations"] == o.iterations


def test_gradient_nh3_polarised_hydrogens(ctx):
    """NH3/6-31G** (d on N, p on H): analytic gradient against central
    differences on a few coordinates; mixed precision within 1e-6 Eh/bohr."""
    atoms, q = M.small_molecule("NH3", "6-31g**")
    fb = B.flatten(atoms)
    xyz = fb.xyz.copy()
    xyz[1, 0] += 0.04
    labels = fb.labels
    tight = dict(conv_energy=1e-12, conv_density=1e-10, max_iter=200)

    def energy(p):
        ctx.set_basis(B.flatten(B.make_atoms(labels, p, "6-31g**", "text")))
        return ctx.scf(_lib.baseline_opts(**tight), want_matrices=False)["energy"]

    ctx.set_basis(B.flatten(B.make_atoms(labels, xyz, "6-31g**", "text")))
    ctx.scf(_lib.baseline_opts(**tight), want_matrices=False)
    g = ctx.gradient()
    assert np.max(np.abs(g.sum(axis=0))) < 1e-9
    h = 1e-4
    for (a, x) in [(0, 2), (1, 0), (2, 1), (3, 2)]:
        xp, xm = xyz.copy(), xyz.copy()
        xp[a, x] += h
        xm[a, x] -= h
        fd = (energy(xp) - energy(xm)) / (2 * h)
        assert abs(g[a, x] - fd) < 1e-6, ((a, x), g[a, x], fd)
    ctx.set_basis(B.flatten(B.make_atoms(labels, xyz, "6-31g**", "text")))
    ctx.scf(_lib.baseline_opts(precision=_lib.PREC_MIXED, incremental=1, **tight), want_matrices=False)
    assert np.max(np.abs(ctx.gradient(precision=_lib.PREC_MIXED) - g)) < 1e-6
