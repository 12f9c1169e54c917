"""Basis sets with d shells (6-31G*): the warp-per-quartet J/K and gradient
kernels, d-shell Schwarz bounds, SAD guess, mixed precision, stored canonical
ERIs with reference numerics and the batched driver, against the oracle."""
import numpy as np
import pytest

import oracle as O
from gbhf import _lib, basis as B, molecules as M

pytestmark = pytest.mark.gpu

H = 1e-4
TIGHT = dict(conv_energy=1e-12, conv_density=1e-10, max_iter=200)


def _rand_density(n, seed, scale=0.2):
    rng = np.random.default_rng(seed)
    d = rng.standard_normal((n, n)) * scale
    return O.square_to_tri(d + d.T)


SYSTEMS = [
    ("water 6-31g*", lambda: M.water_atoms("6-31g*", "text")),
    ("(H2O)2 6-31g*", lambda: M.cluster_atoms("batch256", "6-31g*", index=7)),
]


@pytest.mark.parametrize("name,make", SYSTEMS, ids=[s[0] for s in SYSTEMS])
def test_fock_d_unscreened_matches_stored_eri_fock(ctx, name, make):
    """Every (d..|..) class of the direct build, FP64, no screening: equal to the
    oracle's Fock matrix from its stored canonical ERIs to 1e-11."""
    fb = B.flatten(make())
    ob = O.OracleBasis(fb)
    ctx.set_basis(fb)
    h = ob.hcore(False)
    d = _rand_density(fb.n_cgf, 11)
    ref = O.fock_canonical(h, d, ob.eri_canonical(False))
    got = ctx.fock(h, d, _lib.MODE_EXACT, _lib.PREC_FP64, 0.0, 0.0)
    np.testing.assert_allclose(got, ref, rtol=0, atol=1e-11)


def test_fock_d_screened_and_mixed(ctx):
    """(H2O)4/6-31G*: Schwarz-screened FP64 build against the oracle's direct
    build (same 1e-12 screening on the scaled d components), and the mixed
    build (FP32 below bound 1e-4) within 1e-6 of FP64."""
    fb = B.flatten(M.cluster_atoms("batch256", "6-31g*", index=20))
    ob = O.OracleBasis(fb)
    ctx.set_basis(fb)
    h = ob.hcore(False)
    d = _rand_density(fb.n_cgf, 12, 0.05)
    ref, _ = ob.fock_direct(h, d, 1e-12)
    f64 = ctx.fock(h, d, _lib.MODE_EXACT, _lib.PREC_FP64, 1e-12, 0.0)
    np.testing.assert_allclose(f64, ref, rtol=0, atol=1e-10)
    fmx = ctx.fock(h, d, _lib.MODE_EXACT, _lib.PREC_MIXED, 1e-12, 1e-4)
    err = np.max(np.abs(fmx - f64))
    assert 0 < err < 1e-6


@pytest.mark.parametrize("name,make", SYSTEMS, ids=[s[0] for s in SYSTEMS])
def test_scf_d_fp64_energy(ctx, name, make):
    fb = B.flatten(make())
    ctx.set_basis(fb)
    r = ctx.scf(_lib.baseline_opts())
    o = O.scf(fb, O.SCFOptions.baseline())
    assert abs(r["energy"] - o.energy) < 1e-8
    np.testing.assert_allclose(r["density"], o.density, rtol=0, atol=1e-6)


def test_scf_d_sad_and_mixed(ctx):
    """(H2O)4/6-31G*: the SAD guess reaches the core-guess energy; the mixed
    incremental SCF lands within 1e-6 Eh of FP64."""
    fb = B.flatten(M.cluster_atoms("batch256", "6-31g*", index=20))
    ctx.set_basis(fb)
    e64 = ctx.scf(_lib.baseline_opts(), want_matrices=False)["energy"]
    es = ctx.scf(_lib.baseline_opts(guess=_lib.GUESS_SAD), want_matrices=False)["energy"]
    em = ctx.scf(_lib.baseline_opts(precision=_lib.PREC_MIXED, incremental=1, guess=_lib.GUESS_SAD),
                 want_matrices=False)["energy"]
    o = O.scf(fb, O.SCFOptions.baseline())
    assert abs(e64 - o.energy) < 1e-8
    assert abs(es - e64) < 1e-8
    assert abs(em - e64) < 1e-6


def test_reference_numerics_d_stored_eris(ctx):
    """Water/6-31G* with the reference's numerics (Boys grid, primitive
    screening, S_ii = 1, stored canonical ERIs up to L = 8) from the core
    guess: the oracle's energy to 1e-8.  The reference's own Harris guess reads
    outside its ERI array for this basis (as for 6-31G water) and fails with
    the index status."""
    fb = B.flatten(M.water_atoms("6-31g*", "text"))
    ctx.set_basis(fb)
    ctx.set_boys_grid(O.boys_ref_grid())
    r = ctx.scf(_lib.reference_opts(guess=_lib.GUESS_CORE))
    o = O.scf(fb, O.SCFOptions(guess="core"))
    assert abs(r["energy"] - o.energy) < 1e-8
    assert r["iterations"] == o.iterations
    with pytest.raises(_lib.GBHFError) as ei:
        ctx.scf(_lib.reference_opts())
    assert ei.value.name == "GBHF_ERR_INDEX"


def _energy(ctx, labels, xyz, basis):
    ctx.set_basis(B.flatten(B.make_atoms(labels, xyz, basis, "text")))
    return ctx.scf(_lib.baseline_opts(**TIGHT), want_matrices=False)["energy"]


def test_gradient_d_vs_finite_differences(ctx):
    """Water/6-31G*, distorted: analytic gradient (d-class two-electron and
    nuclear-attraction derivative kernels) against central differences."""
    labels, xyz = ["O", "H", "H"], M.WATER_BOHR.copy()
    xyz[1, 0] += 0.05
    xyz[2, 2] -= 0.03
    ctx.set_basis(B.flatten(B.make_atoms(labels, xyz, "6-31g*", "text")))
    ctx.scf(_lib.baseline_opts(**TIGHT), want_matrices=False)
    g = ctx.gradient()
    assert np.max(np.abs(g.sum(axis=0))) < 1e-9
    for a in range(3):
        for x in range(3):
            xp, xm = xyz.copy(), xyz.copy()
            xp[a, x] += H
            xm[a, x] -= H
            fd = (_energy(ctx, labels, xp, "6-31g*") - _energy(ctx, labels, xm, "6-31g*")) / (2 * H)
            assert abs(g[a, x] - fd) < 1e-6, ((a, x), g[a, x], fd)


def test_gradient_d_dimer_mixed(ctx):
    """(H2O)2/6-31G*: translational invariance, a few finite differences, and
    the mixed-precision gradient within 1e-5 Eh/bohr of FP64."""
    xyz = M.cluster_coords("batch256", 7)
    labels = M.water_labels(len(xyz) // 3)
    ctx.set_basis(B.flatten(B.make_atoms(labels, xyz, "6-31g*", "text")))
    ctx.scf(_lib.baseline_opts(**TIGHT), want_matrices=False)
    g = ctx.gradient()
    assert np.max(np.abs(g.sum(axis=0))) < 1e-9
    for (a, x) in [(0, 0), (1, 1), (3, 2), (5, 0)]:
        xp, xm = xyz.copy(), xyz.copy()
        xp[a, x] += H
        xm[a, x] -= H
        fd = (_energy(ctx, labels, xp, "6-31g*") - _energy(ctx, labels, xm, "6-31g*")) / (2 * H)
        assert abs(g[a, x] - fd) < 1e-6, ((a, x), g[a, x], fd)
    ctx.set_basis(B.flatten(B.make_atoms(labels, xyz, "6-31g*", "text")))
    ctx.scf(_lib.baseline_opts(precision=_lib.PREC_MIXED, incremental=1, **TIGHT), want_matrices=False)
    gm = ctx.gradient(precision=_lib.PREC_MIXED)
    assert np.max(np.abs(gm - g)) < 1e-5


def test_batch_d_matches_single_runs(ctx):
    """A batch mixing 6-31G* and 6-31G molecules: energies and gradients equal
    the one-at-a-time runs."""
    picks = [(1, "6-31g*"), (2, "6-31g"), (3, "6-31g*"), (4, "6-31g*"), (5, "sto-3g")]
    flats = [B.flatten(M.cluster_atoms("batch256", b, index=i)) for i, b in picks]
    opts = _lib.baseline_opts(precision=_lib.PREC_MIXED, incremental=1)
    e, it, cv, grads = ctx.scf_batch(flats, opts, gradients=True)
    assert cv.all()
    for k in (0, 2, 3):
        ctx.set_basis(flats[k])
        r = ctx.scf(_lib.baseline_opts(precision=_lib.PREC_MIXED, incremental=1), want_matrices=False)
        assert abs(r["energy"] - e[k]) < 1e-8
        np.testing.assert_allclose(grads[k], ctx.gradient(), rtol=0, atol=1e-7)
