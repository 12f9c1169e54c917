"""Parity of the device Boys function, one-electron matrices and canonical ERIs
with the oracle (FP64; tolerances are absolute unless stated)."""
import numpy as np
import pytest

import oracle as O
from conftest import golden
from gbhf import _lib, basis as B, molecules as M

pytestmark = pytest.mark.gpu


def test_reference_boys_grid_generated_on_device(ctx):
    g = ctx.generate_boys_grid()
    o = O.boys_ref_grid()
    rel = np.abs(g - o) / np.maximum(np.abs(o), 1e-300)
    assert np.max(rel) < 1e-13


def test_boys_exact_table(ctx):
    x = np.concatenate([np.linspace(0, 40, 1601), np.linspace(37.9, 38.1, 41), np.linspace(40, 200, 161),
                        [1e-12, 1e-6, 0.025, 0.075]])
    got = ctx.boys(_lib.MODE_EXACT, 9, x)
    ref = np.array([[O.boys_exact(m, v) for m in range(10)] for v in x])
    # integrals need absolute accuracy: |dF| < 2e-15 everywhere; relative 5e-14
    # wherever F_m > 1e-4 (beyond T = 38 the asymptotic form drops exp(-T) terms,
    # which only matters relative to values far below that)
    assert np.max(np.abs(got - ref)) < 2e-15
    big = ref > 1e-4
    assert np.max(np.abs(got - ref)[big] / ref[big]) < 5e-14


def test_boys_reference_taylor(ctx):
    ctx.set_boys_grid(O.boys_ref_grid())
    x = np.concatenate([np.linspace(0, 130, 2601), [0.3, 99.95, 100.0, 100.05, 100.1, 100.15]])
    got = ctx.boys(_lib.MODE_REFERENCE, 4, x)
    ref = np.array([[O.boys_taylor(m, v) for m in range(5)] for v in x])
    assert np.max(np.abs(got - ref)) < 1e-15


@pytest.mark.parametrize("basis,variant", [("sto-3g", "shipped"), ("sto-3g", "text"), ("6-31g", "text"),
                                           ("6-31g*", "text")])
def test_one_electron_matrices(ctx, basis, variant):
    fb = B.flatten(M.water_atoms(basis, variant))
    ob = O.OracleBasis(fb)
    ctx.set_basis(fb)
    ctx.set_boys_grid(O.boys_ref_grid())
    for mode, ref in ((_lib.MODE_REFERENCE, True), (_lib.MODE_EXACT, False)):
        np.testing.assert_allclose(ctx.overlap(mode), ob.overlap(ref), rtol=0, atol=1e-14)
        np.testing.assert_allclose(ctx.hcore(mode), ob.hcore(ref), rtol=0, atol=2e-13)


@pytest.mark.parametrize("variant", ["shipped", "text"])
def test_canonical_eris_match_golden(ctx, variant):
    g = golden("water_sto3g.json")[variant]
    ctx.set_basis(B.flatten(M.water_atoms("sto-3g", variant)))
    ctx.set_boys_grid(O.boys_ref_grid())
    for mode, key in ((_lib.MODE_REFERENCE, "reference"), (_lib.MODE_EXACT, "exact")):
        eri = ctx.eri_canonical(mode)
        assert eri.size == 406
        np.testing.assert_allclose(eri, g[key]["eri"], rtol=0, atol=1e-14)


def test_canonical_eris_dimer(ctx):
    fb = B.flatten(M.cluster_atoms("batch256", "6-31g", index=7))   # (H2O)2, N = 26
    ob = O.OracleBasis(fb)
    ctx.set_basis(fb)
    ctx.set_boys_grid(O.boys_ref_grid())
    for mode, ref in ((_lib.MODE_REFERENCE, True), (_lib.MODE_EXACT, False)):
        np.testing.assert_allclose(ctx.eri_canonical(mode), ob.eri_canonical(ref), rtol=0, atol=1e-13)


def _drop_cgf(fb, i):
    """The flat basis without CGF i (its primitives removed too)."""
    off = np.concatenate([[0], np.cumsum(fb.cgf_nprim)])
    keep = np.ones(len(fb.prim_exp), bool)
    keep[off[i]:off[i + 1]] = False
    fb.prim_exp, fb.prim_coef = fb.prim_exp[keep], fb.prim_coef[keep]
    for k in ("cgf_atom", "cgf_lxyz", "cgf_nprim"):
        setattr(fb, k, np.delete(getattr(fb, k), i, axis=0))
    fb.n_cgf -= 1
    return fb


def test_canonical_eris_with_d_shells(ctx):
    fb = B.flatten(M.water_atoms("6-31g*", "text"))
    ctx.set_basis(fb)
    got = ctx.eri_canonical(_lib.MODE_EXACT)
    np.testing.assert_allclose(got, O.OracleBasis(fb).eri_canonical(False), rtol=0, atol=1e-12)


def test_unsupported_and_bad_input(ctx):
    # O 2p without its y component: fine for per-function integrals, not for the
    # shell-based direct J/K build
    fb = _drop_cgf(B.flatten(M.water_atoms("sto-3g", "text")), 3)
    ctx.set_basis(fb)
    d = np.zeros(fb.n_cgf * (fb.n_cgf + 1) // 2)
    with pytest.raises(_lib.GBHFError) as e:
        ctx.fock(d, d, _lib.MODE_EXACT)
    assert e.value.name == "GBHF_ERR_UNSUPPORTED"
    with pytest.raises(_lib.GBHFError) as e:
        ctx.boys(_lib.MODE_EXACT, 3, [-1.0])
    assert e.value.name == "GBHF_ERR_BAD_INPUT"
    bad = B.flatten(M.water_atoms("sto-3g", "text"))
    bad.prim_exp = bad.prim_exp.copy()
    bad.prim_exp[0] = -1.0
    with pytest.raises(_lib.GBHFError) as e:
        ctx.set_basis(bad)
    assert e.value.name == "GBHF_ERR_BAD_INPUT"
