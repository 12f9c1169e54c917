"""Dense FP64 steps on the device: eigen-solve, symmOrtho, diagonalHF, DIIS."""
import numpy as np
import pytest

import oracle as O
from gbhf import _lib, basis as B, molecules as M

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [1, 2, 3, 5, 64, 207, 208, 333])
def test_eigen_solve_random(ctx, n):
    rng = np.random.default_rng(n)
    a = rng.standard_normal((n, n))
    a = a + a.T
    w, v = ctx.eigen_solve(a)
    wr = np.linalg.eigvalsh(a)
    assert np.all(np.diff(w) >= 0)
    np.testing.assert_allclose(w, wr, rtol=0, atol=1e-12 * max(1.0, np.abs(wr).max()))
    assert np.max(np.abs(a @ v - v * w)) < 1e-11 * max(1.0, np.abs(wr).max())
    assert np.max(np.abs(v.T @ v - np.eye(n))) < 1e-12


def test_eigen_solve_degenerate_and_diagonal(ctx):
    a = np.diag([3.0, 1.0, 2.0, 1.0, 3.0])
    w, v = ctx.eigen_solve(a)
    np.testing.assert_allclose(w, [1, 1, 2, 3, 3], atol=0)
    assert np.max(np.abs(v.T @ v - np.eye(5))) < 1e-15
    b = np.kron(np.eye(4), [[2.0, 1.0], [1.0, 2.0]])
    w, v = ctx.eigen_solve(b)
    np.testing.assert_allclose(w, [1] * 4 + [3] * 4, atol=1e-14)
    assert np.max(np.abs(b @ v - v * w)) < 1e-14


def test_symm_ortho_and_diagonal_hf(ctx):
    fb = B.flatten(M.cluster_atoms("batch256", "6-31g", index=7))
    ob = O.OracleBasis(fb)
    s = O.tri_to_square(ob.overlap(False))
    x = ctx.symm_ortho(s)
    np.testing.assert_allclose(x, O.symm_ortho(s), rtol=0, atol=1e-11)
    np.testing.assert_allclose(x @ s @ x, np.eye(fb.n_cgf), rtol=0, atol=1e-11)
    h = ob.hcore(False)
    c, d, e = ctx.diagonal_hf(h, x, fb.n_occupied)
    co, do, eo = O.diagonal_hf(h, x, fb.n_occupied)
    np.testing.assert_allclose(e, eo, rtol=0, atol=1e-10)
    np.testing.assert_allclose(d, do, rtol=0, atol=1e-10)
    # eigenvector signs are arbitrary: compare |C|
    np.testing.assert_allclose(np.abs(c), np.abs(co), rtol=0, atol=1e-8)


def test_diis_error_matrix(ctx):
    fb = B.flatten(M.water_atoms("6-31g", "text"))
    ob = O.OracleBasis(fb)
    s = ob.overlap(False)
    x = O.symm_ortho(O.tri_to_square(s))
    rng = np.random.default_rng(7)
    n = fb.n_cgf
    f = O.square_to_tri(rng.standard_normal((n, n)))
    d = O.square_to_tri(rng.standard_normal((n, n)))
    np.testing.assert_allclose(ctx.diis_error(f, s, d, x), O.calc_error_mtx(f, s, d, x), rtol=0, atol=1e-11)


def test_gauss_elim_known_answer_and_singular(ctx):
    np.testing.assert_allclose(ctx.gauss_elem([[4, -2, 1], [-2, 4, -2], [1, -2, 4]], [11, -16, 17]), [1, -2, 3],
                               atol=1e-14)
    with pytest.raises(_lib.GBHFError) as e:
        ctx.gauss_elem([[1.0, 2.0], [2.0, 4.0]], [1.0, 2.0])
    assert e.value.name == "GBHF_ERR_SINGULAR"


def test_diis_extrapolation_matches_oracle(ctx):
    rng = np.random.default_rng(8)
    n = 9
    es = [rng.standard_normal((n, n)) * 10.0 ** -k for k in range(4)]
    fs = [rng.standard_normal(n * (n + 1) // 2) for _ in range(4)]
    got, used = ctx.diis_extrapolate(es, fs)
    ref, dat = O.diis(es[0], fs[0], O.DataDIIS(es[1:], fs[1:], 5))
    assert used == len(dat.errors) == 3
    np.testing.assert_allclose(got, ref, rtol=0, atol=1e-10)
    # linearly dependent history: the oldest pairs are dropped, as the reference does
    es2 = [es[0], es[0], es[0]]
    got2, used2 = ctx.diis_extrapolate(es2, fs[:3])
    ref2, dat2 = O.diis(es2[0], fs[0], O.DataDIIS(es2[1:], fs[1:3], 5))
    assert used2 == len(dat2.errors)
    np.testing.assert_allclose(got2, ref2, rtol=0, atol=1e-10)
