"""Open-shell (unrestricted) SCF on the device against the oracle's UHF:
radicals, triplets, a cation, atoms; closed shells reduce to RHF."""
import numpy as np
import pytest

import oracle as O
from gbhf import _lib, basis as B, molecules as M

pytestmark = pytest.mark.gpu

TIGHT = dict(conv_energy=1e-12, conv_density=1e-10, max_iter=200)


@pytest.mark.parametrize("name", M.OPEN_SHELL)
def test_uhf_energies(ctx, name):
    for b in ("sto-3g", "6-31g*"):
        atoms, q, mult = M.open_shell_molecule(name, b)
        fb = B.flatten(atoms)
        ctx.set_basis(fb)
        r = ctx.scf_uhf(mult, _lib.baseline_opts(charge=q, guess=_lib.GUESS_CORE, **TIGHT))
        o = O.uhf(fb, mult, q)
        assert (r["n_alpha"], r["n_beta"]) == (o.n_alpha, o.n_beta)
        assert abs(r["energy"] - o.energy) < 1e-8, (name, b, r["energy"], o.energy)
        assert abs(r["s2"] - o.s2) < 1e-6
        da = O.tri_to_square(r["density_alpha"])
        assert abs(np.trace(da @ O.tri_to_square(O.OracleBasis(fb).overlap(False))) - o.n_alpha) < 1e-8


def test_uhf_closed_shell_equals_rhf_and_mixed(ctx):
    fb = B.flatten(M.cluster_atoms("batch256", "6-31g*", index=7))
    ctx.set_basis(fb)
    e_rhf = ctx.scf(_lib.baseline_opts(**TIGHT), want_matrices=False)["energy"]
    r = ctx.scf_uhf(1, _lib.baseline_opts(guess=_lib.GUESS_SAD, **TIGHT), want_matrices=False)
    assert abs(r["energy"] - e_rhf) < 1e-9 and abs(r["s2"]) < 1e-8
    # an open-shell cation of the same dimer: mixed precision within 1e-6 Eh of FP64
    e64 = ctx.scf_uhf(2, _lib.baseline_opts(charge=1.0, **TIGHT), want_matrices=False)["energy"]
    emx = ctx.scf_uhf(2, _lib.baseline_opts(charge=1.0, precision=_lib.PREC_MIXED, **TIGHT),
                      want_matrices=False)["energy"]
    assert abs(emx - e64) < 1e-6


def test_uhf_bad_multiplicity(ctx):
    ctx.set_basis(B.flatten(M.water_atoms("sto-3g", "text")))
    for mult in (0, 2):   # 10 electrons: even multiplicities impossible
        with pytest.raises(_lib.GBHFError) as e:
            ctx.scf_uhf(mult)
        assert e.value.name == "GBHF_ERR_BAD_INPUT"
