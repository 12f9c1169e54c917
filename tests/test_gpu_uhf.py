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


H = 1e-4


def _uhf_energy(ctx, labels, xyz, basis, q, mult):
    ctx.set_basis(B.flatten(B.make_atoms(labels, xyz, basis, "text")))
    return ctx.scf_uhf(mult, _lib.baseline_opts(charge=q, guess=_lib.GUESS_CORE, **TIGHT),
                       want_matrices=False)["energy"]


@pytest.mark.parametrize("name,basis", [("OH", "6-31g"), ("CH2", "sto-3g"), ("H2O+", "6-31g*"), ("NH2", "6-31g")])
def test_uhf_gradient_vs_finite_differences(ctx, name, basis):
    """Open-shell analytic gradient against central differences (1e-4 bohr) of
    the GPU UHF energy on every coordinate, and of the oracle's UHF energy on
    two; translational invariance."""
    atoms, q, mult = M.open_shell_molecule(name, basis)
    labels = [a.label for a in atoms]
    xyz = np.array([a.coord for a in atoms], dtype=np.float64)
    if len(atoms) > 1:
        xyz[1] += (0.03, -0.02, 0.01)   # off any symmetry point
    e0 = _uhf_energy(ctx, labels, xyz, basis, q, mult)
    g = ctx.gradient_uhf()
    assert np.max(np.abs(g.sum(axis=0))) < 1e-9
    for a in range(len(atoms)):
        for x in range(3):
            e = [_uhf_energy(ctx, labels, xyz + s * H * np.eye(len(atoms) * 3)[3 * a + x].reshape(-1, 3), basis, q,
                             mult) for s in (1, -1)]
            fd = (e[0] - e[1]) / (2 * H)
            assert abs(fd - g[a, x]) < 1e-6, (name, a, x, g[a, x], fd)
    for (a, x) in ((0, 2), (len(atoms) - 1, 0)):
        e = []
        for s in (1, -1):
            p = xyz.copy()
            p[a, x] += s * H
            e.append(O.uhf(B.flatten(B.make_atoms(labels, p, basis, "text")), mult, q).energy)
        assert abs((e[0] - e[1]) / (2 * H) - g[a, x]) < 1e-6
    assert np.isfinite(e0)


def test_uhf_gradient_explicit_densities_and_mixed(ctx):
    """gbhf_gradient_uhf with the caller's D_alpha, D_beta and W equals the
    last-SCF path; the mixed-precision gradient stays within 1e-5 Eh/bohr."""
    atoms, q, mult = M.open_shell_molecule("O2", "6-31g")
    fb = B.flatten(atoms)
    ctx.set_basis(fb)
    r = ctx.scf_uhf(mult, _lib.baseline_opts(charge=q, **TIGHT))
    g_last = ctx.gradient_uhf()
    ob = O.OracleBasis(fb)
    h = O.tri_to_square(ob.hcore(False))
    da, db = O.tri_to_square(r["density_alpha"]), O.tri_to_square(r["density_beta"])
    # W = D_a F_a D_a + D_b F_b D_b from the oracle's Fock matrices of these densities
    eri = O.eri_tensor(ob, fb.n_cgf)
    j = np.einsum("abcd,cd->ab", eri, da + db)
    fa = h + j - np.einsum("acbd,cd->ab", eri, da)
    fbm = h + j - np.einsum("acbd,cd->ab", eri, db)
    w = da @ fa @ da + db @ fbm @ db
    g_dw = ctx.gradient_uhf(O.square_to_tri(da), O.square_to_tri(db), O.square_to_tri(w))
    np.testing.assert_allclose(g_dw, g_last, rtol=0, atol=1e-8)
    g_mx = ctx.gradient_uhf(precision=_lib.PREC_MIXED)
    assert np.max(np.abs(g_mx - g_last)) < 1e-5
    # a closed-shell UHF gradient is the RHF gradient
    ctx.set_basis(B.flatten(M.water_atoms("6-31g", "text")))
    ctx.scf(_lib.baseline_opts(**TIGHT), want_matrices=False)
    g_rhf = ctx.gradient()
    ctx.scf_uhf(1, _lib.baseline_opts(**TIGHT), want_matrices=False)
    np.testing.assert_allclose(ctx.gradient_uhf(), g_rhf, rtol=0, atol=1e-8)
