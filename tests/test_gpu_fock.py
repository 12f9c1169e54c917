"""Direct J/K Fock build on the device versus the oracle."""
import numpy as np
import pytest

import oracle as O
from gbhf import _lib, basis as B, molecules as M

pytestmark = pytest.mark.gpu


def _rand_density(n, seed, scale=0.2):
    rng = np.random.default_rng(seed)
    d = rng.standard_normal((n, n)) * scale
    return O.square_to_tri(d + d.T)


SYSTEMS = [
    ("water sto-3g", lambda: M.water_atoms("sto-3g", "text")),
    ("water sto-3g shipped", lambda: M.water_atoms("sto-3g", "shipped")),
    ("water 6-31g", lambda: M.water_atoms("6-31g", "text")),
    ("(H2O)2 6-31g", lambda: M.cluster_atoms("batch256", "6-31g", index=7)),
    ("(H2O)4 sto-3g", lambda: M.cluster_atoms("batch256", "sto-3g", index=20)),
]


@pytest.mark.parametrize("name,make", SYSTEMS, ids=[s[0] for s in SYSTEMS])
def test_fock_fp64_unscreened_matches_stored_eri_fock(ctx, name, make):
    fb = B.flatten(make())
    ob = O.OracleBasis(fb)
    ctx.set_basis(fb)
    h = ob.hcore(False)
    d = _rand_density(fb.n_cgf, 1)
    ref = O.fock_canonical(h, d, ob.eri_canonical(False))
    got = ctx.fock(h, d, _lib.MODE_EXACT, _lib.PREC_FP64, 0.0, 0.0)
    np.testing.assert_allclose(got, ref, rtol=0, atol=1e-11)


def test_fock_reference_mode(ctx):
    fb = B.flatten(M.water_atoms("sto-3g", "shipped"))
    ob = O.OracleBasis(fb)
    ctx.set_basis(fb)
    ctx.set_boys_grid(O.boys_ref_grid())
    h = ob.hcore(True)
    d = _rand_density(fb.n_cgf, 2)
    ref = O.fock_canonical(h, d, ob.eri_canonical(True))
    np.testing.assert_allclose(ctx.fock(h, d, _lib.MODE_REFERENCE), ref, rtol=0, atol=1e-13)


def test_fock_fp64_screened_matches_oracle_direct(ctx):
    fb = B.flatten(M.cluster_atoms("w8", "6-31g"))
    ob = O.OracleBasis(fb)
    ctx.set_basis(fb)
    h = ob.hcore(False)
    d = _rand_density(fb.n_cgf, 3, 0.05)
    ref, _ = ob.fock_direct(h, d, 1e-12)
    got = ctx.fock(h, d, _lib.MODE_EXACT, _lib.PREC_FP64, 1e-12, 0.0)
    np.testing.assert_allclose(got, ref, rtol=0, atol=1e-11)


def test_fock_mixed_precision_error(ctx):
    """FP32 for quartets with Schwarz bound < 1e-4: Fock error stays below 1e-6."""
    fb = B.flatten(M.cluster_atoms("w8", "6-31g"))
    ctx.set_basis(fb)
    ob = O.OracleBasis(fb)
    h = ob.hcore(False)
    d = _rand_density(fb.n_cgf, 4, 0.05)
    f64 = ctx.fock(h, d, _lib.MODE_EXACT, _lib.PREC_FP64, 1e-12, 0.0)
    fmx = ctx.fock(h, d, _lib.MODE_EXACT, _lib.PREC_MIXED, 1e-12, 1e-4)
    err = np.max(np.abs(fmx - f64))
    assert 0 < err < 1e-6


def test_fock_zero_density_is_core(ctx):
    fb = B.flatten(M.water_atoms("6-31g", "text"))
    ctx.set_basis(fb)
    h = np.arange(fb.n_cgf * (fb.n_cgf + 1) // 2, dtype=float)
    got = ctx.fock(h, np.zeros_like(h), _lib.MODE_EXACT, _lib.PREC_FP64, 1e-12, 0.0)
    np.testing.assert_array_equal(got, h)


def test_fock_single_atom_and_linearity(ctx):
    fb = B.flatten(B.make_atoms(["O"], [[0.1, -0.2, 0.3]], "6-31g"))
    ob = O.OracleBasis(fb)
    ctx.set_basis(fb)
    h = np.zeros(fb.n_cgf * (fb.n_cgf + 1) // 2)
    d1, d2 = _rand_density(fb.n_cgf, 5), _rand_density(fb.n_cgf, 6)
    f1 = ctx.fock(h, d1, _lib.MODE_EXACT, _lib.PREC_FP64, 0.0, 0.0)
    f2 = ctx.fock(h, d2, _lib.MODE_EXACT, _lib.PREC_FP64, 0.0, 0.0)
    f12 = ctx.fock(h, d1 + 2 * d2, _lib.MODE_EXACT, _lib.PREC_FP64, 0.0, 0.0)
    np.testing.assert_allclose(f12, f1 + 2 * f2, rtol=0, atol=1e-12)
    np.testing.assert_allclose(f1, O.fock_canonical(h, d1, ob.eri_canonical(False)), rtol=0, atol=1e-12)
